"""Generate the Gauss-Kronrod 21- and 15-point tables of the device QAGS
(fj_kronrod.h, host arrays plus __constant__ device copies):
    python gen_kronrod.py fj_kronrod.h fj_

The nodes are the zeros of P_n (Gauss) and of the
Stieltjes polynomial E_{n+1} (Kronrod extension); the Kronrod weights make the
(2n+1)-point rule exact for polynomials of degree <= 3n+1.  Everything is
computed from these definitions with mpmath at 60 digits and printed with 17
significant digits, so no published table is transcribed.
"""
import sys
import mpmath as mp

mp.mp.dps = 60


def legendre_coeffs(n):
    # ascending coefficients of P_n
    p0, p1 = [mp.mpf(1)], [mp.mpf(0), mp.mpf(1)]
    if n == 0:
        return p0
    for k in range(1, n):
        nxt = [mp.mpf(0)] * (k + 2)
        for i, c in enumerate(p1):
            nxt[i + 1] += (2 * k + 1) * c / (k + 1)
        for i, c in enumerate(p0):
            nxt[i] -= k * c / (k + 1)
        p0, p1 = p1, nxt
    return p1


def moment(k):
    # int_{-1}^{1} x^k dx
    return mp.mpf(0) if k % 2 else mp.mpf(2) / (k + 1)


def poly_eval(c, x):
    return sum(ci * x ** i for i, ci in enumerate(c))


def kronrod(n):
    pn = legendre_coeffs(n)
    m = n + 1
    # E_{n+1}(x) = x^{m} + sum_{j<m} e_j x^j, orthogonal to x^k P_n for k < m
    A = mp.matrix(m, m)
    rhs = mp.matrix(m, 1)
    for k in range(m):
        for j in range(m):
            A[k, j] = sum(pn[i] * moment(i + j + k) for i in range(len(pn)))
        rhs[k] = -sum(pn[i] * moment(i + m + k) for i in range(len(pn)))
    e = mp.lu_solve(A, rhs)
    ecoef = [e[j] for j in range(m)] + [mp.mpf(1)]
    knodes = sorted(mp.polyroots(list(reversed(ecoef)), maxsteps=500, extraprec=400), key=lambda z: mp.re(z))
    knodes = [mp.re(z) for z in knodes]
    gnodes = sorted(mp.polyroots(list(reversed(pn)), maxsteps=500, extraprec=400), key=lambda z: mp.re(z))
    gnodes = [mp.re(z) for z in gnodes]
    nodes = sorted(knodes + gnodes)
    N = len(nodes)
    V = mp.matrix(N, N)
    b = mp.matrix(N, 1)
    for k in range(N):
        for j in range(N):
            V[k, j] = nodes[j] ** k
        b[k] = moment(k)
    w = mp.lu_solve(V, b)
    # Gauss weights
    dp = [i * pn[i] for i in range(1, len(pn))]
    gw = {float(x): 2 / ((1 - x * x) * poly_eval(dp, x) ** 2) for x in gnodes}
    # QUADPACK ordering: non-negative nodes from the largest down to 0
    half = [(nodes[j], w[j]) for j in range(N) if nodes[j] >= -mp.mpf(10) ** -40]
    half.sort(key=lambda t: -t[0])
    xgk = [x if abs(x) > mp.mpf(10) ** -40 else mp.mpf(0) for x, _ in half]
    wgk = [wt for _, wt in half]
    # Gauss weights for the Gauss nodes among xgk (odd positions), plus centre if n odd
    wg = [gw[float(x)] for x in xgk if any(abs(x - g) < mp.mpf(10) ** -30 for g in gnodes) and x > 0]
    if n % 2 == 1:
        wg.append(gw[0.0] if 0.0 in gw else [v for k, v in gw.items() if abs(k) < 1e-30][0])
    return xgk, wgk, wg


def emit(name, vals, device=False):
    body = ",\n    ".join(mp.nstr(v, 17, min_fixed=-1, max_fixed=1) if v != 0 else "0.0" for v in vals)
    txt = f"static const double {name}[{len(vals)}] = {{\n    {body}\n}};\n"
    if device:
        txt += f"__constant__ double {name}_d[{len(vals)}] = {{\n    {body}\n}};\n"
    return txt


def main(out, prefix):
    x21, w21, g21 = kronrod(10)
    x15, w15, g15 = kronrod(7)
    txt = ["/* Generated by gen_kronrod.py: Gauss-Kronrod nodes/weights from their definitions. */",
           f"#ifndef {prefix.upper()}KRONROD_H", f"#define {prefix.upper()}KRONROD_H"]
    dev = prefix == "fj_"
    txt.append(emit(prefix + "xgk21", x21, dev))
    txt.append(emit(prefix + "wgk21", w21, dev))
    txt.append(emit(prefix + "wg10", g21, dev))
    txt.append(emit(prefix + "xgk15", x15, dev))
    txt.append(emit(prefix + "wgk15", w15, dev))
    txt.append(emit(prefix + "wg7", g15, dev))
    txt.append("#endif")
    open(out, "w").write("\n".join(txt) + "\n")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "orc_kronrod.h", sys.argv[2] if len(sys.argv) > 2 else "orc_")
