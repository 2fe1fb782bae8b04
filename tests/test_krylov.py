"""Krylov solvers preconditioned by lmgc on the device: `gcg` (UG's cg,
np/procs/ls.cc:901-1064) and `gbcgs` (UG's bcgs, ls.cc:1711-2062) against
UG's own solves (tests/golden: cg_* / bcgs_*) in UG's vector order, against
the oracle's cg / bcgs on the reordered hierarchy in multicolour order, and
their FP32-preconditioner variants against the FP64 stopping test.  Tolerances: iterations equal (+-1 allowed by the contract),
solution 1e-10 relative (jac) / 1e-8 (gs, ilu; order-dependent smoothers)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, permuted_levels, rel

pytestmark = pytest.mark.gpu
NAMES = golden_names()


@pytest.fixture(scope="module")
def G():
    import ug_gb300
    ug_gb300.lib()
    return ug_gb300


def _setup_cg(G, mg, sm, bl, red=1e-10, mixed=False, name="cgs", dloop=True):
    G.setup_lmgc(mg, sm, baselevel=bl, damp=0.8 if sm == "jac" else 1.0, red=red, abslimit=1e-50)
    mg.npcreate(name, "linear_solver.gcg")
    st = mg.npinit(name, f"$A MAT $x sol $b rhs $red {red} $abslimit 1e-50 $m 100 $I lmgc $mixed {int(mixed)}"
                         f" $dloop {int(dloop)}")
    assert st == G.NP_EXECUTABLE
    return name


@pytest.mark.parametrize("name", NAMES)
def test_cg_matches_ug(G, name):
    fx = load_golden(name)
    levels = G.levels_from_ugfx(fx)
    mg = G.MultiGrid(levels, order=G.ORDER_LIST, fp32=True)
    sm, bl = fx["smoother"], int(fx["baselevel"][0])
    _setup_cg(G, mg, sm, bl)
    x, lr = mg.solve_host("cgs", fx["rhs"])
    assert lr.converged and abs(lr.iters - int(fx["cg_iters"][0])) <= 1
    assert rel(x, fx["cg_x"]) <= (1e-10 if sm == "jac" else 1e-8)
    # the FP32 preconditioner inside the FP64 cg meets the same stopping test
    mg.npcreate("cgs32", "linear_solver.gcg")
    mg.npinit("cgs32", "$A MAT $x sol $b rhs $red 1e-10 $abslimit 1e-50 $m 100 $I lmgc $mixed 1")
    x32, lr32 = mg.solve_host("cgs32", fx["rhs"])
    assert lr32.converged and lr32.iters <= int(fx["cg_iters"][0]) + 3
    assert rel(x32, fx["cg_x"]) <= 1e-6
    mg.close()


@pytest.mark.parametrize("sm", ["jac", "ilu"])
@pytest.mark.parametrize("order", [0, 1])
def test_cg_vs_oracle_midsize(G, oracle_mod, order, sm):
    """3D P1 diffusion 17^3, k = exp(g): device cg vs the oracle's cg on the
    same (possibly reordered) hierarchy.  (With forward Gauss-Seidel as pre-
    and post-smoother the V-cycle is not symmetric and UG's cg stagnates near
    1e-8 on this problem; the oracle reproduces that, so gs is not used here.)"""
    gen = G.Generator(1, 4, seed=5, corr=0.1, var=1.0)
    levels = gen.levels()
    mg = G.MultiGrid(levels, order=order, fp32=True)
    _setup_cg(G, mg, sm, 0)
    x, lr = mg.solve_host("cgs", gen.rhs)
    H = oracle_mod.Hierarchy(permuted_levels(levels, mg))
    perm = mg.order(mg.top)
    xo, ito, conv, _ = H.cg_solve(gen.rhs[perm], smoother=sm, baselevel=0, damp=0.8 if sm == "jac" else 1.0,
                                  red=1e-10, abslimit=1e-50)
    xr = np.empty_like(xo); xr[perm] = xo
    assert conv and lr.converged and abs(lr.iters - ito) <= 1
    assert rel(x, xr) <= (1e-10 if sm == "jac" else 1e-8)
    mg.close()


def _setup_bcgs(G, mg, sm, bl, red=1e-10, mixed=False, name="bcgs"):
    G.setup_lmgc(mg, sm, baselevel=bl, damp=0.8 if sm == "jac" else 1.0, red=red, abslimit=1e-50)
    mg.npcreate(name, "linear_solver.gbcgs")
    st = mg.npinit(name, f"$A MAT $x sol $b rhs $red {red} $abslimit 1e-50 $m 100 $I lmgc $mixed {int(mixed)}")
    assert st == G.NP_EXECUTABLE
    return name


@pytest.mark.parametrize("name", NAMES)
def test_bcgs_matches_ug(G, name):
    """bcgs (ls.cc:1711-2062) with the lmgc preconditioner against UG's own
    bcgs solves: half-step iteration counts +-1, UG's solution."""
    fx = load_golden(name)
    levels = G.levels_from_ugfx(fx)
    mg = G.MultiGrid(levels, order=G.ORDER_LIST, fp32=True)
    sm, bl = fx["smoother"], int(fx["baselevel"][0])
    _setup_bcgs(G, mg, sm, bl)
    x, lr = mg.solve_host("bcgs", fx["rhs"])
    assert lr.converged and abs(lr.iters - int(fx["bcgs_iters"][0])) <= 1
    assert rel(x, fx["bcgs_x"]) <= (1e-10 if sm == "jac" else 1e-8)
    mg.npcreate("bcgs32", "linear_solver.gbcgs")
    mg.npinit("bcgs32", "$A MAT $x sol $b rhs $red 1e-10 $abslimit 1e-50 $m 100 $I lmgc $mixed 1")
    x32, lr32 = mg.solve_host("bcgs32", fx["rhs"])
    assert lr32.converged and lr32.iters <= int(fx["bcgs_iters"][0]) + 4
    assert rel(x32, fx["bcgs_x"]) <= 1e-6
    mg.close()


@pytest.mark.parametrize("order", [0, 1])
def test_bcgs_gs_vs_oracle_midsize(G, oracle_mod, order):
    """3D P1 diffusion 17^3, k = exp(g), with the (nonsymmetric) Gauss-Seidel
    V-cycle, where cg stagnates: device bcgs vs the oracle's bcgs on the same
    (possibly reordered) hierarchy."""
    gen = G.Generator(1, 4, seed=5, corr=0.1, var=1.0)
    levels = gen.levels()
    mg = G.MultiGrid(levels, order=order, fp32=True)
    _setup_bcgs(G, mg, "gs", 0)
    x, lr = mg.solve_host("bcgs", gen.rhs)
    H = oracle_mod.Hierarchy(permuted_levels(levels, mg))
    perm = mg.order(mg.top)
    xo, ito, conv, _ = H.bcgs_solve(gen.rhs[perm], smoother="gs", baselevel=0, red=1e-10, abslimit=1e-50)
    xr = np.empty_like(xo); xr[perm] = xo
    assert conv and lr.converged and abs(lr.iters - ito) <= 1
    assert rel(x, xr) <= 1e-8
    mg.close()


@pytest.mark.parametrize("name,order,mixed", [("p1k_gs", 1, False), ("el_ilu", 0, True), ("ls_gs", 0, False)])
def test_cg_device_loop_matches_host_loop(G, name, order, mixed):
    """cg's iterations after the first run as one conditional graph (the loop
    test also watches CGUpdate's (A p, p) = 0 flag); the host loop ($dloop 0)
    takes the same iterations to the same x, bit for bit."""
    fx = load_golden(name)
    levels = G.levels_from_ugfx(fx)
    sm, bl = fx["smoother"], int(fx["baselevel"][0])
    out = {}
    for dloop in (True, False):
        mg = G.MultiGrid(levels, order=order, fp32=True)
        _setup_cg(G, mg, sm, bl, mixed=mixed, dloop=dloop)
        x, lr = mg.solve_host("cgs", fx["rhs_all"] if mg.local else fx["rhs"])
        out[dloop] = (x, lr, mg.npdisplay("cgs"))
        mg.close()
    (xd, ld, dd), (xh, lh, dh) = out[True], out[False]
    assert "loop = device (built)" in dd and "loop = host" in dh
    assert ld.converged and ld.iters == lh.iters
    assert list(ld.last_defect) == list(lh.last_defect)
    assert np.array_equal(xd, xh)
