"""Shared test helpers: oracle models built from golden fixtures, comparisons."""
import numpy as np

from oracle import oracle as O

SLOPES = {"Hernquist": (1.667, 5.0), "NFW": (1.667, 3.0), "Isochrone": (0.0, 5.0)}


def oracle_model(g, meta, phil, Pr, Pr2, Egrid=None, Dgrid=None, jquad=0, xq=O.XPT11, wq=O.XW11):
    p = meta["p"]
    a, b = SLOPES[p["model"]]
    kind = O.DF_QUASIISO if meta["df"] == "qiso" else O.DF_DPL
    return O.Model(g["ar"], phil, Pr, Pr2, g["Egrid"] if Egrid is None else Egrid,
                   g["Dgrid"] if Dgrid is None else Dgrid, meta["ng"], df_kind=kind, alpha=a, beta=b,
                   mass=p["mass"], r0=p["r0"], dphi_h=p["dphi_h"], dz_h=p["dz_h"], dphi_g=p["dphi_g"],
                   dz_g=p["dz_g"], chi=p["chi"], k=meta["k"], jquad=jquad, xq=xq, wq=wq)


def _nan_diff(a, ref):
    """|a-ref| with NaN==NaN counted as equal (empty outer shells give 0/0 sigmas in both)."""
    d = np.abs(a - ref)
    both = np.isnan(a) & np.isnan(ref)
    d[both] = 0.0
    d[np.isnan(d)] = np.inf
    return d


def rel_rows(a, ref):
    """max |a-ref| scaled by the |monopole| of the same radius (rows of [nr][npoly])."""
    a = np.asarray(a, dtype=float).reshape(ref.shape)
    scale = np.abs(ref[:, :1]) + 1e-300
    scale[np.isnan(scale)] = 1.0
    return float(np.max(_nan_diff(a, ref) / scale))


def rel(a, ref, floor=1e-300):
    a, ref = np.asarray(a, dtype=float), np.asarray(ref, dtype=float)
    s = np.maximum(np.abs(ref), floor)
    s[np.isnan(s)] = 1.0
    return float(np.max(_nan_diff(a, ref) / s))
