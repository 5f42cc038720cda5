"""CPU-side checks of the product library: it loads, exports every entry point
include/fjgpu.h declares, and its host-side setup and I/O match the reference
(grid, Gauss-Legendre nodes, guess density, focal-distance table, coefficient
file bytes, parameter-file parsing).  No GPU compute is called here."""
import os
import re

import numpy as np
import pytest

import fjmodels_gb300 as F
from fjmodels_gb300 import _abi
from oracle import oracle as O
from tests.conftest import ROOT, load_golden
from tests.helpers import rel, rel_rows


def declared_functions():
    src = open(os.path.join(ROOT, "include", "fjgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char \*|void \*)\s*(fj_\w+)\s*\(", src, flags=re.M)))


def test_library_exports_every_declared_symbol():
    lib = F.load_library()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) <= set(_abi.SIGNATURES), "ctypes table misses a declared entry point"
    assert lib.fj_version().startswith(b"fjmodels-gb300")


def test_no_device_reports_error_code():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import ctypes as C
    h = C.c_void_p()
    assert F.load_library().fj_ctx_create(0, C.byref(h)) != 0


def test_host_grid_and_nodes_match_oracle():
    assert rel(F.log_grid(1e-3, 300.0, 80), O.log_grid(1e-3, 300.0, 80)) == 0.0
    for n in (4, 20, 40):
        x, w = F.gauleg(0, 1, n)
        xo, wo = O.gauleg(0, 1, n)
        assert np.array_equal(x, xo) and np.array_equal(w, wo)


@pytest.mark.parametrize("name", ["hern_dpl", "nfw_dpl_rot", "hern_qiso"])
def test_guess_and_delta_table_match_reference(name):
    g, meta, _ = load_golden(name)
    nr, ng, npl = meta["nr"], meta["ng"], meta["np"]
    p = meta["p"]
    rhl = F.guess_rhl(g["ar"], ng, npl, p["model"], p["mass"], p["r0"])
    assert rel_rows(rhl, g["guess_rhl"].reshape(nr, npl)) < 1e-14
    E, D, _ = F.tabulate_delta(g["ar"], g["guess_phil"], g["guess_Pr"], g["guess_Pr2"])
    assert rel(E, g["Egrid"]) < 1e-12 and rel(D, g["Dgrid"]) < 1e-9


@pytest.mark.parametrize("name", ["hern_dpl", "nfw_dpl_rot"])
def test_write_out_is_byte_identical(name, tmp_path):
    g, meta, _ = load_golden(name)
    nr, ng, npl = meta["nr"], meta["ng"], meta["np"]
    p = meta["p"]
    a, b = {"Hernquist": (1.667, 5.0), "NFW": (1.667, 3.0)}[p["model"]]
    mats = np.stack([g["it0_" + k].reshape(nr, npl) for k in
                     ("rhl", "vrotl", "sigRl", "sigpl", "sigzl", "sigRzl", "phil", "Pr", "Pr2")])
    name_ref = F.composeName(p["model"], p["dphi_h"], p["dz_h"], p["dphi_g"], p["dz_g"], 0)
    key = "outfile_" + os.path.basename(name_ref).replace(".", "_")
    assert key in g.files, (key, g.files)
    out = tmp_path / "x.out"
    F.writeOut(str(out), g["ar"], mats, ng, (p["dphi_h"], p["dz_h"], p["dphi_g"], p["dz_g"], p["chi"], p["mass"],
                                             p["r0"], a, b))
    assert out.read_bytes() == g[key].tobytes()


def test_read_param_two_component_quirk(tmp_path):
    """'2:model' commented out but 2:A/2:B set still makes two components (io/readParam.cpp:124-131)."""
    f = tmp_path / "param.txt"
    f.write_text("#\n# c\n#\n\nitermax\t\t4\n\t\nmodel\t\tHernquist\noutfile\t\t2comp_test\nh(J):dphi\t0.55\n"
                 "h(J):dz\t\t0.55\ng(J):dphi\t1.\ng(J):dz\t\t1.\nchi\t\t0.\nmass\t\t1.\nr0\t\t1.\nq\t\t1.\n"
                 "#2:model \t  NFW\n2:outfile\t  x2\n2:A\t\t  0.\n2:B\t\t  2.\n2:h(J):dphi       0.55\n"
                 "2:h(J):dz         2.\n2:g(J):dphi       1.\n2:g(J):dz         4.\n2:chi\t\t  10.\n"
                 "2:mass            2.\n2:r0              2.\n2:q               .6\n")
    p, comps = F.readParam(str(f))
    assert comps == 2 and p["itermax"] == 4 and p["modName"] == "Hernquist" and p["alpha_2"] == 0.0
    assert p["beta_2"] == 2.0 and p["q_2"] == 0.6 and p["outName"] == "2comp_test"
    f.write_text("model Hernquist\nchi 0\n")
    with pytest.raises(F.FJError):
        F.readParam(str(f))


def test_compose_name():
    assert F.composeName("Hernquist", 0.55, 0.55, 1, 1, 3) == os.path.join("models", "Hernq_0.55_0.55_1.00_1.00_3.out")
    assert F.composeName("NFW", 0.5, 2, 1, 4, 0, comp=2).endswith("NFW_0.50_2.00_1.00_4.00_0.out2c")


@pytest.mark.parametrize("name", ["hern_dpl", "nfw_dpl_rot"])
def test_read_out_of_the_reference_file(name, tmp_path):
    """The reference's own coefficient file (6 significant digits) read back: sizes, header
    and every table within the rounding of the printed digits; a full-precision copy
    (17 digits) reads back exactly; a truncated or missing file is an error."""
    g, meta, _ = load_golden(name)
    nr, ng, npl = meta["nr"], meta["ng"], meta["np"]
    p = meta["p"]
    name_ref = F.composeName(p["model"], p["dphi_h"], p["dz_h"], p["dphi_g"], p["dz_g"], 0)
    f = tmp_path / "ref.out"
    f.write_bytes(g["outfile_" + os.path.basename(name_ref).replace(".", "_")].tobytes())
    r = F.readOut(str(f))
    assert (r["nr"], r["npoly"], r["ngauss"]) == (nr, npl, ng)
    assert np.allclose(r["header"][:7], [p["dphi_h"], p["dz_h"], p["dphi_g"], p["dz_g"], p["chi"], p["mass"], p["r0"]])
    assert np.all(np.abs(r["ar"] - g["ar"]) <= 5e-6 * np.abs(g["ar"]))
    keys = ("rhl", "vrotl", "sigRl", "sigpl", "sigzl", "sigRzl", "phil", "Pr", "Pr2")
    for k in keys:
        ref = g["it0_" + k].reshape(nr, npl)
        assert np.all(np.abs(r[k] - ref) <= 5e-6 * np.abs(ref) + 1e-300), k
    mats = np.stack([g["it0_" + k].reshape(nr, npl) for k in keys])
    full = tmp_path / "full.out"
    F.writeOut(str(full), g["ar"], mats, ng, r["header"], digits=17)
    r17 = F.readOut(str(full))
    assert np.array_equal(r17["ar"], g["ar"]) and np.array_equal(r17["header"], r["header"])
    for i, k in enumerate(keys):
        assert np.array_equal(r17[k], mats[i]), k
    cut = tmp_path / "cut.out"
    cut.write_bytes(full.read_bytes()[:-200])
    with pytest.raises(F.FJError):
        F.readOut(str(cut))
    with pytest.raises(F.FJError):
        F.readOut(str(tmp_path / "missing.out"))
