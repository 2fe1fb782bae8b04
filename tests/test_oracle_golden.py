"""Pins the C restatement of the lmgc path (oracle/lmgc_oracle.c) to the UG
reference: every kernel's known-answer vector and every ls + lmgc solve in
tests/golden/ was produced by UG 3.12.1 itself (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden

NAMES = golden_names()
LOCAL = golden_names("local")


def rel(a, b):
    a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("name", NAMES + LOCAL)
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
    if name in LOCAL:
        # dnrm2x over ALL_VECTORS; the top level of a local hierarchy also holds
        # copies outside the NEW_DEFECT set, which orc_nrm2x leaves out
        d = np.asarray(fx["kat_d"]).reshape(int(fx[f"L{top}_n"][0]), -1)
        assert rel(np.sqrt((d * d).sum(axis=0)), fx["kat_nrm"]) <= 1e-14
        nd = fx[f"L{top}_new_defect"].astype(bool)
        assert rel(H.nrm2x(top, fx["kat_d"]), np.sqrt((d[nd] * d[nd]).sum(axis=0))) <= 1e-14
    else:
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
    # the last defect sits near the rounding level of the first one (~1e-12 of
    # it); its summation order differs, so it is compared on that scale
    assert np.all(np.abs(np.asarray(hist[-1]) - fx["cg_last"]) <= 1e-12 * fx["cg_first"])


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
    # the last defect sits near the rounding level of the first one (~1e-12 of
    # it); its summation order differs, so it is compared on that scale
    assert np.all(np.abs(np.asarray(hist[-1]) - fx["bcgs_last"]) <= 1e-12 * fx["bcgs_first"])


def _split(fx, flat):
    n = int(fx["nlevels"][0]); s = int(fx["blocksize"][0])
    offs = np.cumsum([0] + [int(fx[f"L{l}_n"][0]) * s for l in range(n)])
    return [np.asarray(flat)[offs[l]:offs[l + 1]] for l in range(n)]


@pytest.mark.parametrize("name", LOCAL)
def test_surface_flags_match_ug(name, oracle_mod):
    """UG's surface of a locally refined hierarchy follows from the vector
    classes alone (gm/algebra.cc:2917-2921): FINE_GRID_DOF = VCLASS >= 2 and
    VNCLASS <= 1, NEW_DEFECT = VCLASS >= 2, FULLREFINELEVEL = the lowest level
    with a FINE_GRID_DOF vector; the rhs lives on exactly those rows."""
    fx = load_golden(name)
    H = oracle_mod.Hierarchy.from_ugfx(fx)
    n = int(fx["nlevels"][0]); s = int(fx["blocksize"][0])
    assert H.fullrefinelevel() == int(fx["fullrefinelevel"][0]) < n - 1
    rhs = _split(fx, fx["rhs_all"])
    nsurf = 0
    for l in range(n):
        vc, vn = fx[f"L{l}_vclass"], fx[f"L{l}_vnclass"]
        assert np.array_equal(fx[f"L{l}_fine_grid_dof"], ((vc >= 2) & (vn <= 1)).astype(np.int32))
        assert np.array_equal(fx[f"L{l}_new_defect"], (vc >= 2).astype(np.int32))
        surf = (vc >= 2) if l == n - 1 else ((vc >= 2) & (vn <= 1))
        if l < int(fx["fullrefinelevel"][0]):
            surf = np.zeros_like(surf)
        assert not np.any(rhs[l].reshape(-1, s)[~surf]), l
        nsurf += int(surf.sum())
    assert nsurf > int(fx[f"L{n - 1}_n"][0])  # the surface spans several levels


@pytest.mark.parametrize("name", LOCAL)
def test_surface_solve_matches_ug(name, oracle_mod):
    """ls + lmgc on the locally refined L-shaped elasticity problem: the
    oracle repeats UG's defect history and solution on every level."""
    fx = load_golden(name)
    H = oracle_mod.Hierarchy.from_ugfx(fx)
    sm = fx["smoother"]
    x, it, conv, hist = H.ls_solve_surface(fx["rhs_all"], smoother=sm, baselevel=int(fx["baselevel"][0]),
                                           damp=0.8 if sm == "jac" else 1.0, red=1e-10, abslimit=1e-50)
    assert conv and it == int(fx["ls_iters"][0])
    assert rel(hist.ravel(), fx["ls_hist"]) <= 1e-12
    assert rel(x, fx["ls_x_all"]) <= 1e-12
    assert rel(_split(fx, x)[-1], fx["ls_x"]) <= 1e-12
    assert rel(fx["ls_x_replay"], fx["ls_x"]) == 0.0


@pytest.mark.parametrize("name", ["q1_gs", "el_ilu", "p1k_jac"])
def test_surface_solve_is_ls_on_uniform(name, oracle_mod):
    """On a uniformly refined hierarchy the surface is the top level, so the
    all-level solve gives the top-level solve exactly."""
    fx = load_golden(name)
    H = oracle_mod.Hierarchy.from_ugfx(fx)
    sm = fx["smoother"]
    kw = dict(smoother=sm, baselevel=int(fx["baselevel"][0]), damp=0.8 if sm == "jac" else 1.0)
    x1, it1, _, h1 = H.ls_solve(fx["rhs"], **kw)
    x2, it2, _, h2 = H.ls_solve_surface(fx["rhs_all"], **kw)
    assert it1 == it2 and np.array_equal(h1, h2)
    assert np.array_equal(_split(fx, x2)[-1], x1)


@pytest.mark.parametrize("name", NAMES + LOCAL)
def test_solution_transfer_matches_ug(name, oracle_mod):
    """StandardIntNewNodeVector / StandardProject (transgrid.cc:354, 655) as
    UG's transfer numproc runs them over every level (transfer.cc:775, 794):
    the oracle repeats UG's results bit for bit."""
    fx = load_golden(name)
    H = oracle_mod.Hierarchy.from_ugfx(fx)
    n = int(fx["nlevels"][0])
    vnew = [fx[f"L{l}_vnew"] for l in range(n)]
    x = H.interpolate_new_vectors(0, n - 1, fx["kat_newvec_pre"], vnew)
    assert np.array_equal(x, fx["kat_newvec"])
    x = H.project_solution(0, n - 1, fx["kat_project_pre"])
    assert np.array_equal(x, fx["kat_project"])


@pytest.mark.parametrize("solver", ["cg", "bcgs"])
@pytest.mark.parametrize("name", LOCAL)
def test_surface_krylov_matches_ug(name, solver, oracle_mod):
    """UG's cg and bcgs with the lmgc preconditioner on the locally refined
    problem: vector operations on every level, dot products (and bcgs's
    matrix products) ON_SURFACE.  The oracle takes UG's iteration count and
    reaches UG's solution on every level."""
    fx = load_golden(name)
    H = oracle_mod.Hierarchy.from_ugfx(fx)
    sm = fx["smoother"]
    f = H.cg_solve_surface if solver == "cg" else H.bcgs_solve_surface
    x, it, conv, hist = f(fx["rhs_all"], smoother=sm, baselevel=int(fx["baselevel"][0]),
                          damp=0.8 if sm == "jac" else 1.0, red=1e-10, abslimit=1e-50)
    assert conv == bool(fx[f"{solver}_converged"][0]) and it == int(fx[f"{solver}_iters"][0])
    assert rel(x, fx[f"{solver}_x_all"]) <= 1e-12
    assert rel(hist[-1], fx[f"{solver}_last"]) <= 1e-10


IMAT = golden_names("imat")


@pytest.mark.parametrize("name", IMAT)
def test_oracle_matrix_transfer_matches_ug(oracle_mod, name):
    """The transfer's matrix mode (`npinit transfer $M`): RestrictByMatrix and
    InterpolateCorrectionByMatrix on UG's interpolation matrices, plain and
    damped, bit for bit, InterpolateNewVectorsByMatrix over every level as
    the `$M` transfer numproc runs it (transfer.cc:775 through its intnew,
    transgrid.cc:1425), and UG's solves in that mode (iterations, defect
    history, solution), on uniform and locally refined hierarchies."""
    fx = load_golden(name)
    H = oracle_mod.Hierarchy.from_ugfx(fx)
    top = len(H.levels) - 1
    vnew = [fx[f"L{l}_vnew"] for l in range(top + 1)]
    assert np.array_equal(H.interpolate_new_vectors(0, top, fx["kat_newvec_pre"], vnew), fx["kat_newvec"])
    dm = [0.7 - 0.1 * i for i in range(8)]
    assert np.array_equal(H.restrict_imat(top, fx["kat_mrestrict_pre"], fx["kat_d"]), fx["kat_mrestrict"])
    assert np.array_equal(H.restrict_imat(top, fx["kat_mrestrict_damp_pre"], fx["kat_d"], dm),
                          fx["kat_mrestrict_damp"])
    assert np.array_equal(H.interpolate_imat(top, fx["kat_minterp_coarse"]), fx["kat_minterp"])
    assert np.array_equal(H.interpolate_imat(top, fx["kat_minterp_coarse"], dm), fx["kat_minterp_damp"])
    sm = str(fx["smoother"])
    kw = dict(smoother=sm, baselevel=int(fx["baselevel"][0]), damp=0.8 if sm == "jac" else 1.0, red=1e-10,
              matrix_transfer=True)
    if name.startswith("im_ls"):
        x, it, conv, hist = H.ls_solve_surface(fx["rhs_all"], **kw)
        assert rel(x, fx["ls_x_all"]) <= 1e-14
    else:
        x, it, conv, hist = H.ls_solve(fx["rhs"], **kw)
        assert rel(x, fx["ls_x"]) <= 1e-14
    assert it == int(fx["ls_iters"][0]) and conv == bool(fx["ls_converged"][0])
    assert rel(hist.ravel(), fx["ls_hist"]) <= 1e-14
