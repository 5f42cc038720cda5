"""Generate the golden fixtures from the reference's own sources.

Builds oracle/_ref (the reference's unmodified C++ compiled against the GSL
stand-in in oracle/ref_build) for small grids, runs it on seeded inputs and
stores every dumped intermediate in tests/golden/<scenario>.npz, plus the
coefficient file the reference's writeOut produced.  Needs the reference
checkout, named by the REF_DIR environment variable; the fixtures it writes
are committed so the tests never need the reference at run time.

    REF_DIR=<reference checkout> python tests/golden/make_golden.py [scenario ...]
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
BUILD = os.path.join(ROOT, "oracle", "ref_build")
REFBIN = os.path.join(ROOT, "oracle", "_ref")
REF_DIR = os.environ.get("REF_DIR")

PARAM = """itermax {itermax}
model {model}
h(J):dphi {dphi_h}
h(J):dz {dz_h}
g(J):dphi {dphi_g}
g(J):dz {dz_g}
chi {chi}
mass {mass}
r0 {r0}
q 1.
"""

SCENARIOS = {
    # name: grid, DF variant, parameters
    "hern_dpl": dict(nr=12, ng=4, np=3, df="dpl", k=1.0, rmin=0.01, rmax=100.0,
                     p=dict(itermax=2, model="Hernquist", dphi_h=0.55, dz_h=0.55, dphi_g=1.0, dz_g=1.0,
                            chi=0.0, mass=1.0, r0=1.0)),
    "nfw_dpl_rot": dict(nr=12, ng=4, np=3, df="dpl", k=0.5, rmin=0.01, rmax=300.0,
                        p=dict(itermax=1, model="NFW", dphi_h=0.55, dz_h=0.55, dphi_g=1.0, dz_g=1.0,
                               chi=1.0, mass=1.0, r0=1.0)),
    "hern_qiso": dict(nr=12, ng=4, np=3, df="qiso", k=1.0, rmin=0.01, rmax=100.0,
                      p=dict(itermax=1, model="Hernquist", dphi_h=0.55, dz_h=0.55, dphi_g=1.0, dz_g=1.0,
                             chi=0.0, mass=1.0, r0=1.0)),
    # the full 40 x 20, l <= 8 Hernquist configuration, five iterations from the guess
    "c1_hern": dict(nr=40, ng=20, np=5, df="dpl", k=0.5, rmin=0.01, rmax=100.0,
                    p=dict(itermax=5, model="Hernquist", dphi_h=0.55, dz_h=0.55, dphi_g=1.0, dz_g=1.0,
                           chi=0.0, mass=1.0, r0=1.0)),
    # the reference's two-component loop (twoComp, its own component order): a Hernquist bulge
    # and a rotating NFW halo, two iterations
    "twocomp_ref": dict(nr=12, ng=4, np=3, df="dpl", k=0.5, rmin=0.01, rmax=300.0,
                        p=dict(itermax=2, model="Hernquist", dphi_h=0.7, dz_h=0.5, dphi_g=0.9, dz_g=0.6,
                               chi=0.0, mass=0.1, r0=1.0),
                        p2=dict(model="NFW", dphi_h=0.45, dz_h=0.8, dphi_g=0.55, dz_g=0.95, chi=1.0, mass=1.0,
                                r0=10.0)),
}

PARAM2 = """2:model {model}
2:h(J):dphi {dphi_h}
2:h(J):dz {dz_h}
2:g(J):dphi {dphi_g}
2:g(J):dz {dz_g}
2:chi {chi}
2:mass {mass}
2:r0 {r0}
2:q 1.
"""


def points(seed):
    rng = np.random.default_rng(seed)
    lines = []
    for _ in range(16):
        r = 10 ** rng.uniform(-2.3, 2.6)
        c = rng.uniform(0.0, 1.0)
        lines.append(f"P {r * np.sqrt(1 - c * c):.17g} {r * c:.17g}")
    for _ in range(48):
        r = 10 ** rng.uniform(-1.5, 1.5)
        c = rng.uniform(0.02, 0.98)
        v = rng.uniform(-1, 1, 3) * rng.uniform(0.05, 1.0) / np.sqrt(1 + r)
        lines.append(f"A {r * np.sqrt(1 - c * c):.17g} {r * c:.17g} {v[0]:.17g} {v[1]:.17g} {v[2]:.17g}")
    for R, z in ((0.8, 0.3), (2.0, 1.5)):
        lines.append(f"M {R:.17g} {z:.17g}")
    # projected density, line profiles and velocity distributions (Integ.cpp:168-220)
    for R, z in ((0.5, 0.2), (3.0, 0.05)):
        lines.append(f"S {R:.17g} {z:.17g}")
    for R, z, v in ((0.5, 0.2, 0.3), (0.5, 0.2, -0.05), (3.0, 0.05, 0.6)):
        lines.append(f"L {R:.17g} {z:.17g} {v:.17g}")
    for kind in "FZX":
        for R, z, v in ((0.5, 0.2, 0.2), (3.0, 0.05, -0.1)):
            lines.append(f"{kind} {R:.17g} {z:.17g} {v:.17g}")
    return "\n".join(lines) + "\n"


def parse_dump(path):
    out, name, vals, n = {}, None, [], 0
    for line in open(path):
        parts = line.split()
        if len(parts) == 2 and not parts[0][0].isdigit() and parts[0][0] != '-':
            if name is not None:
                out[name] = np.array(vals)
            name, n, vals = parts[0], int(parts[1]), []
        else:
            vals.append(float(parts[0]))
    if name is not None:
        out[name] = np.array(vals)
    return out


def parse_vir2(text):
    rows = []
    for line in text.splitlines():
        if line.startswith("Mass("):
            cur = [float(x) for x in line.split(":")[1].split()]
        elif line.startswith("KE, PE, W/K"):
            cur += [float(x) for x in line.split("=")[1].split()]
        elif line.startswith("Kxx, Wxx"):
            cur += [float(x) for x in line.split("=")[1].split()]
        elif line.startswith("Kzz, Wzz"):
            cur += [float(x) for x in line.split("=")[1].split()]
            rows.append(cur)
    return np.array(rows)


def run(name, sc):
    tag = f"{sc['nr']}_{sc['ng']}_{sc['np']}"
    subprocess.run(["make", "-s", "-C", BUILD, f"NR={sc['nr']}", f"NG={sc['ng']}", f"NP={sc['np']}",
                    f"REF={REF_DIR}"], check=True)
    exe = os.path.join(REFBIN, f"fjref_{sc['df']}_{tag}")
    with tempfile.TemporaryDirectory() as td:
        os.makedirs(os.path.join(td, "models"))
        param = PARAM.format(**sc["p"]) + (PARAM2.format(**sc["p2"]) if "p2" in sc else "")
        open(os.path.join(td, "param.txt"), "w").write(param)
        pts = points(abs(hash(name)) % 2**31 if False else sum(map(ord, name)))
        open(os.path.join(td, "points.txt"), "w").write(pts)
        env = dict(os.environ, FJREF_K=str(sc["k"]), OMP_NUM_THREADS=str(os.cpu_count()))
        res = subprocess.run([exe, "param.txt", str(sc["rmin"]), str(sc["rmax"]), "points.txt", "dump.txt"],
                             cwd=td, env=env, capture_output=True, text=True, check=True)
        d = parse_dump(os.path.join(td, "dump.txt"))
        d["vir2"] = parse_vir2(res.stdout)
        d["points"] = np.array(pts.encode())
        outs = sorted(os.listdir(os.path.join(td, "models")))
        for f in outs:
            data = open(os.path.join(td, "models", f), "rb").read()
            d["outfile_" + f.replace(".", "_")] = np.frombuffer(data, dtype=np.uint8)
        d["meta"] = np.array(repr(sc).encode())
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print(name, sorted(d.keys()))


if __name__ == "__main__":
    if not REF_DIR or not os.path.isdir(REF_DIR):
        sys.exit("make_golden.py: set REF_DIR to the reference checkout")
    names = sys.argv[1:] or list(SCENARIOS)
    for n in names:
        run(n, SCENARIOS[n])
