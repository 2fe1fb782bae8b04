"""Pins the C restatement of the lmgc path (oracle/lmgc_oracle.c) to the UG
reference: every kernel's known-answer vector and every ls + lmgc solve in
tests/golden/ was produced by UG 3.12.1 itself (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden

NAMES = golden_names()


def rel(a, b):
    a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("name", NAMES)
def test_kernels_match_ug(name, oracle_mod):
    fx = load_golden(name)
    H = oracle_mod.Hierarchy.from_ugfx(fx)
    top = int(fx["nlevels"][0]) - 1
    assert rel(H.matmul_minus(top, fx["kat_x"], fx["kat_y"]), fx["kat_matmul"]) <= 1e-14
    assert rel(H.jac(top, fx["kat_d"]), fx["kat_jac"]) <= 1e-14
    assert rel(H.lgs(top, fx["kat_d"]), fx["kat_gs"]) <= 1e-14
    lu = H.ilu_decomp(top)
    assert rel(lu, fx["kat_ilu_factors"]) <= 1e-14
    assert rel(H.luiter(top, lu, fx["kat_d"]), fx["kat_ilu"]) <= 1e-14
    assert rel(H.nrm2x(top, fx["kat_d"]), fx["kat_nrm"]) <= 1e-14
    assert rel(H.restrict(top, fx["kat_restrict_pre"], fx["kat_d"]), fx["kat_restrict"]) <= 1e-14
    assert rel(H.interpolate(top, fx["kat_interp_coarse"]), fx["kat_interp"]) <= 1e-14


@pytest.mark.parametrize("name", NAMES)
def test_solve_matches_ug(name, oracle_mod):
    fx = load_golden(name)
    H = oracle_mod.Hierarchy.from_ugfx(fx)
    sm = fx["smoother"]
    x, it, conv, hist = H.ls_solve(fx["rhs"], smoother=sm, baselevel=int(fx["baselevel"][0]),
                                   damp=0.8 if sm == "jac" else 1.0, red=1e-10, abslimit=1e-50)
    assert conv and it == int(fx["ls_iters"][0])
    assert rel(x, fx["ls_x"]) <= 1e-12
    assert rel(hist.ravel(), fx["ls_hist"]) <= 1e-12
    # UG's own replay of the ls loop reproduces its solve exactly
    assert rel(fx["ls_x_replay"], fx["ls_x"]) == 0.0


@pytest.mark.parametrize("name", NAMES)
def test_cg_matches_ug(name, oracle_mod):
    """UG's cg (np/procs/ls.cc:901-1064) preconditioned by the same lmgc:
    the oracle takes UG's iteration count and reaches UG's solution."""
    fx = load_golden(name)
    H = oracle_mod.Hierarchy.from_ugfx(fx)
    sm = fx["smoother"]
    x, it, conv, hist = H.cg_solve(fx["rhs"], smoother=sm, baselevel=int(fx["baselevel"][0]),
                                   damp=0.8 if sm == "jac" else 1.0, red=1e-10, abslimit=1e-50)
    assert conv == bool(fx["cg_converged"][0]) and it == int(fx["cg_iters"][0])
    assert rel(x, fx["cg_x"]) <= 1e-12
    assert rel(hist[-1], fx["cg_last"]) <= 1e-10


@pytest.mark.parametrize("name", NAMES)
def test_bcgs_matches_ug(name, oracle_mod):
    """UG's bcgs (np/procs/ls.cc:1711-2062) preconditioned by the same lmgc:
    the oracle takes UG's (half-step) iteration count and reaches UG's
    solution."""
    fx = load_golden(name)
    H = oracle_mod.Hierarchy.from_ugfx(fx)
    sm = fx["smoother"]
    x, it, conv, hist = H.bcgs_solve(fx["rhs"], smoother=sm, baselevel=int(fx["baselevel"][0]),
                                     damp=0.8 if sm == "jac" else 1.0, red=1e-10, abslimit=1e-50)
    assert conv == bool(fx["bcgs_converged"][0]) and it == int(fx["bcgs_iters"][0])
    assert rel(x, fx["bcgs_x"]) <= 1e-12
    assert rel(hist[-1], fx["bcgs_last"]) <= 1e-10
