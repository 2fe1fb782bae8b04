"""Locally refined hierarchies on the GPU: the L-shaped plane-strain problem
refined toward its re-entrant corner by UG itself (tests/golden/ls_*.npz).
The surface spans several levels (FINE_GRID_DOF rows below the top level),
so ls's defect and norms run over UG's ON_SURFACE rows of every level and
LSUpdate adds the correction on every level (np/procs/ls.cc:562, 577, 869).

* list order: UG's iteration count and UG's solution on EVERY level (jac
  1e-10 relative, gs / ilu 1e-8 and iterations +-1, the contract's bounds);
* multicolour order: the oracle's surface solve on the reordered hierarchy;
* mixed precision (FP32 V-cycle in FP64 refinement of the surface defect):
  converges to the FP64 stopping test, error against a tightly converged
  FP64 oracle solution at most 1e-6 relative.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden, permuted_levels, rel

pytestmark = pytest.mark.gpu
LOCAL = golden_names("local")


@pytest.fixture(scope="module")
def G():
    import ug_gb300
    ug_gb300.lib()
    return ug_gb300


def _damp(sm):
    return 0.8 if sm == "jac" else 1.0


def _split(mg, flat):
    return mg.split_levels(np.asarray(flat))


@pytest.mark.parametrize("graph", [True, False])
@pytest.mark.parametrize("fuse", [0, None])
@pytest.mark.parametrize("name", LOCAL)
def test_local_solve_matches_ug(G, name, fuse, graph):
    fx = load_golden(name)
    mg = G.MultiGrid(G.levels_from_ugfx(fx), order=0)
    assert mg.local and mg.frl == int(fx["fullrefinelevel"][0])
    sm = fx["smoother"]
    G.setup_lmgc(mg, sm, baselevel=int(fx["baselevel"][0]), damp=_damp(sm), red=1e-10, abslimit=1e-50, fuse=fuse,
                 graph=graph)
    x, lr = mg.solve_host("mgs", fx["rhs_all"])
    it_ug = int(fx["ls_iters"][0])
    assert lr.converged
    assert abs(lr.first_defect[0] - fx["ls_hist"][0]) <= 1e-12 * fx["ls_hist"][0]
    if sm == "jac":
        assert lr.iters == it_ug
        assert rel(x, fx["ls_x_all"]) <= 1e-10
    else:
        assert abs(lr.iters - it_ug) <= 1
        assert rel(x, fx["ls_x_all"]) <= 1e-8
    x2, lr2 = mg.solve_host("mgs", fx["rhs_all"])
    assert lr2.iters == lr.iters and np.array_equal(x, x2)
    mg.close()


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("name", LOCAL + ["el_ilu", "q1_gs", "p1k_ilu"])
def test_local_multicolour_matches_oracle(G, oracle_mod, name, order):
    """Multicolour (1) and subdomain (2) processing orders: the device solve
    is the oracle's on the reordered hierarchy (uniform fixtures included:
    their surface is the top level)."""
    fx = load_golden(name)
    levels = G.levels_from_ugfx(fx)
    mg = G.MultiGrid(levels, order=order)
    if "rhs_all" not in fx:
        fx = dict(fx)
        fx["rhs_all"] = np.concatenate([np.zeros(d["n"] * d["s"]) for d in levels[:-1]] + [fx["rhs"]])
    sm = fx["smoother"]
    bl = int(fx["baselevel"][0])
    G.setup_lmgc(mg, sm, baselevel=bl, damp=_damp(sm), red=1e-10, abslimit=1e-50)
    b_in = fx["rhs_all"] if mg.local else fx["rhs"]
    x, lr = mg.solve_host("mgs", b_in)
    H = oracle_mod.Hierarchy(permuted_levels(levels, mg))
    s = levels[0]["s"]
    perms = [mg.order(l) for l in range(mg.nlevels)]
    lens = [d["n"] * s for d in levels]
    offs = np.cumsum([0] + lens)
    b_all = np.asarray(fx["rhs_all"])
    b_p = np.concatenate([b_all[offs[l]:offs[l + 1]].reshape(-1, s)[p].ravel() for l, p in enumerate(perms)])
    xo, ito, conv, _ = H.ls_solve_surface(b_p, smoother=sm, baselevel=bl, damp=_damp(sm), red=1e-10, abslimit=1e-50)
    xr = []
    for l, p in enumerate(perms):
        o = np.empty((len(p), s)); o[p] = xo[offs[l]:offs[l + 1]].reshape(-1, s); xr.append(o.ravel())
    xr = np.concatenate(xr) if mg.local else xr[-1]
    assert conv and lr.converged and lr.iters == ito
    assert rel(x, xr) <= 1e-10
    mg.close()


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("name", LOCAL)
def test_local_mixed_precision(G, oracle_mod, name, order):
    fx = load_golden(name)
    levels = G.levels_from_ugfx(fx)
    mg = G.MultiGrid(levels, order=order, fp32=True)
    sm = fx["smoother"]
    bl = int(fx["baselevel"][0])
    G.setup_lmgc(mg, sm, baselevel=bl, damp=_damp(sm), red=1e-8, abslimit=1e-50, mixed=True)
    x, lr = mg.solve_host("mgs", fx["rhs_all"])
    assert lr.converged and lr.last_defect[0] <= 1e-8 * lr.first_defect[0]
    # the FP64 iteration in the same order (multicolour ILU / GS is another
    # preconditioner than UG's list order) to the same reduction
    m64 = G.MultiGrid(levels, order=order)
    G.setup_lmgc(m64, sm, baselevel=bl, damp=_damp(sm), red=1e-8, abslimit=1e-50)
    _, lr64 = m64.solve_host("mgs", fx["rhs_all"])
    m64.close()
    assert lr64.converged and lr.iters <= lr64.iters + 2
    H = oracle_mod.Hierarchy.from_ugfx(fx)
    xo, _, conv, _ = H.ls_solve_surface(fx["rhs_all"], smoother=sm, baselevel=bl, damp=_damp(sm), red=1e-14,
                                        abslimit=1e-50)
    assert conv
    # the surface solution: FINE_GRID_DOF rows below the top, NEW_DEFECT rows on it
    frl, top = mg.frl, mg.top
    s = levels[0]["s"]
    xs, xos = [], []
    for l, (a, b) in enumerate(zip(_split(mg, x), _split(mg, xo))):
        if l < frl:
            continue
        vc, vn = fx[f"L{l}_vclass"], fx[f"L{l}_vnclass"]
        m = (vc >= 2) if l == top else ((vc >= 2) & (vn <= 1))
        xs.append(a.reshape(-1, s)[m].ravel()); xos.append(b.reshape(-1, s)[m].ravel())
    assert rel(np.concatenate(xs), np.concatenate(xos)) <= 1e-6
    mg.close()


@pytest.mark.parametrize("sm,order", [("ilu", 2), ("gs", 2), ("gs", 0), ("jac", 1)])
def test_generated_local_vs_oracle(G, oracle_mod, sm, order):
    """The generated L-shape hierarchy (UG's local refinement rebuilt on the
    host, 5 uniform + 9 local steps, 43k surface unknowns): the device solve
    and the oracle's surface solve on the same (reordered) hierarchy agree."""
    gen = G.LocalGenerator(5, 9, seed=2026)
    levels = gen.levels()
    mg = G.MultiGrid(levels, order=order)
    assert mg.local and mg.nlevels == 15
    G.setup_lmgc(mg, sm, baselevel=0, damp=_damp(sm), red=1e-8, abslimit=1e-50)
    x, lr = mg.solve_host("mgs", gen.rhs)
    H = oracle_mod.Hierarchy(permuted_levels(levels, mg))
    s = 2
    perms = [mg.order(l) for l in range(mg.nlevels)]
    b_p = np.concatenate([b.reshape(-1, s)[p].ravel() for b, p in zip(_split(mg, gen.rhs), perms)])
    xo, ito, conv, _ = H.ls_solve_surface(b_p, smoother=sm, baselevel=0, damp=_damp(sm), red=1e-8, abslimit=1e-50)
    xr = []
    for xl, p in zip(_split(mg, xo), perms):
        o = np.empty((len(p), s)); o[p] = xl.reshape(-1, s); xr.append(o.ravel())
    assert conv and lr.converged and abs(lr.iters - ito) <= 1
    assert rel(x, np.concatenate(xr)) <= 1e-8
    mg.close()


@pytest.mark.parametrize("graph", [True, False])
def test_iface_one_launch_is_bit_identical(G, graph):
    """The interface ILU sweeps of the subdomain order in one cooperative
    launch per direction (rows waiting on their neighbours' completion
    flags) against one launch per interface colour: the generated L-shape
    hierarchy's FP64 and mixed solves agree bit for bit."""
    gen = G.LocalGenerator(5, 9, seed=2026)
    levels = gen.levels()
    out = []
    for mode in (0, 2):
        mg = G.MultiGrid(levels, order=G.ORDER_DOMAIN, fp32=True)
        mg.set_iface_sweep(mode)
        assert mg.domain_info(mg.top)["interface_colours"] >= 2
        G.setup_lmgc(mg, "ilu", baselevel=0, red=1e-8, abslimit=1e-50, graph=graph, dloop=graph)
        mg.npcreate("mgs32", "linear_solver.gls")
        mg.npinit("mgs32", f"$A MAT $x sol $b rhs $red 1e-8 $abslimit 1e-50 $m 100 $I lmgc $mixed 1"
                           f" $graph {int(graph)} $dloop {int(graph)}")
        x64, lr64 = mg.solve_host("mgs", gen.rhs)
        x32, lr32 = mg.solve_host("mgs32", gen.rhs)
        x32b, _ = mg.solve_host("mgs32", gen.rhs)  # again: the flags' epochs have moved on
        out.append((x64, lr64.iters, x32, lr32.iters, x32b))
        assert lr64.converged and lr32.converged
        mg.close()
    (a64, ai64, a32, ai32, _), (b64, bi64, b32, bi32, b32b) = out
    assert ai64 == bi64 and ai32 == bi32
    assert np.array_equal(a64, b64) and np.array_equal(a32, b32) and np.array_equal(b32, b32b)


def test_update_values_scales_local_solution(G):
    """gmg_mg_update_values on the generated L-shape hierarchy in subdomain
    order (ILU factors rebuilt in place): doubling every level's matrix
    halves the converged solution on every level."""
    gen = G.LocalGenerator(5, 9, seed=2026)
    levels = gen.levels()
    mg = G.MultiGrid(levels, order=2)
    G.setup_lmgc(mg, "ilu", baselevel=0, red=1e-12, abslimit=1e-50)
    x1, lr1 = mg.solve_host("mgs", gen.rhs)
    for l, d in enumerate(levels):
        v = np.array(d["val"], np.float64).reshape(-1, 4)
        # Dirichlet rows keep their unit diagonal (UG's assembly sets them so)
        rp = d["rowptr"]
        for i in np.nonzero(d["skip"])[0]:
            v[rp[i]:rp[i + 1]] /= 2.0
        mg.update_values(l, 2.0 * v)
    x2, lr2 = mg.solve_host("mgs", gen.rhs)
    assert lr1.converged and lr2.converged and abs(lr1.iters - lr2.iters) <= 1
    assert rel(2.0 * x2, x1) <= 1e-8
    mg.close()


def _setup_krylov(G, mg, cls, sm, name, red=1e-10, mixed=False):
    mg.npcreate(name, f"linear_solver.{cls}")
    st = mg.npinit(name, f"$A MAT $x sol $b rhs $red {red} $abslimit 1e-50 $m 100 $I lmgc $mixed {int(mixed)}")
    assert st == G.NP_EXECUTABLE


@pytest.mark.parametrize("solver", ["cg", "bcgs"])
@pytest.mark.parametrize("name", LOCAL)
def test_local_krylov_matches_ug(G, name, solver):
    """UG's cg / bcgs preconditioned by lmgc on the locally refined problem
    (vector operations on every level, products ON_SURFACE): UG's iteration
    count and UG's solution on every level; the FP32 preconditioner meets the
    same stopping test within 1e-6."""
    fx = load_golden(name)
    mg = G.MultiGrid(G.levels_from_ugfx(fx), order=0, fp32=True)
    sm, bl = fx["smoother"], int(fx["baselevel"][0])
    G.setup_lmgc(mg, sm, baselevel=bl, damp=_damp(sm), red=1e-10, abslimit=1e-50)
    _setup_krylov(G, mg, "g" + solver, sm, "ks")
    x, lr = mg.solve_host("ks", fx["rhs_all"])
    it_ug = int(fx[f"{solver}_iters"][0])
    assert lr.converged and abs(lr.iters - it_ug) <= 1
    assert rel(x, fx[f"{solver}_x_all"]) <= (1e-10 if sm == "jac" else 1e-8)
    _setup_krylov(G, mg, "g" + solver, sm, "ks32", mixed=True)
    x32, lr32 = mg.solve_host("ks32", fx["rhs_all"])
    assert lr32.converged and lr32.iters <= it_ug + 3
    top, frl = mg.top, mg.frl
    s = 2
    parts = []
    for l, (a, b) in enumerate(zip(_split(mg, x32), _split(mg, fx[f"{solver}_x_all"]))):
        if l < frl:
            continue
        vc, vn = fx[f"L{l}_vclass"], fx[f"L{l}_vnclass"]
        m = (vc >= 2) if l == top else ((vc >= 2) & (vn <= 1))
        parts.append((a.reshape(-1, s)[m].ravel(), b.reshape(-1, s)[m].ravel()))
    assert rel(np.concatenate([p[0] for p in parts]), np.concatenate([p[1] for p in parts])) <= 1e-6
    mg.close()


@pytest.mark.parametrize("solver", ["cg", "bcgs"])
def test_generated_local_krylov_vs_oracle(G, oracle_mod, solver):
    """cg / bcgs with ILU in subdomain order on the generated L-shape
    hierarchy (5 uniform + 9 local steps): the device matches the oracle on
    the reordered hierarchy."""
    gen = G.LocalGenerator(5, 9, seed=2026)
    levels = gen.levels()
    mg = G.MultiGrid(levels, order=2)
    G.setup_lmgc(mg, "ilu", baselevel=0, red=1e-8, abslimit=1e-50)
    _setup_krylov(G, mg, "g" + solver, "ilu", "ks", red=1e-8)
    x, lr = mg.solve_host("ks", gen.rhs)
    H = oracle_mod.Hierarchy(permuted_levels(levels, mg))
    s = 2
    perms = [mg.order(l) for l in range(mg.nlevels)]
    b_p = np.concatenate([b.reshape(-1, s)[p].ravel() for b, p in zip(_split(mg, gen.rhs), perms)])
    f = H.cg_solve_surface if solver == "cg" else H.bcgs_solve_surface
    xo, ito, conv, _ = f(b_p, smoother="ilu", baselevel=0, red=1e-8, abslimit=1e-50)
    xr = []
    for xl, p in zip(_split(mg, xo), perms):
        o = np.empty((len(p), s)); o[p] = xl.reshape(-1, s); xr.append(o.ravel())
    assert conv and lr.converged and abs(lr.iters - ito) <= 1
    assert rel(x, np.concatenate(xr)) <= 1e-8
    mg.close()


def _same_level(a, b):
    for k in ("n", "rowptr", "col", "val", "vclass", "vnclass", "skip", "prowptr", "pcol", "pw"):
        x, y = a.get(k), b.get(k)
        if (x is None) != (y is None) or (x is not None and not np.array_equal(np.asarray(x), np.asarray(y))):
            return False
    return True


@pytest.mark.parametrize("order,sm", [(0, "gs"), (1, "gs"), (2, "ilu"), (0, "ilu")])
@pytest.mark.parametrize("nuni,nloc", [(3, 3), (2, 6)])
def test_replace_levels_after_adaptation(G, nuni, nloc, order, sm):
    """Incremental re-flattening: one more local refinement step toward the
    corner changes the old top level (its VNCLASS) and adds a level above it;
    gmg_mg_replace_levels swaps in exactly those levels on a hierarchy that
    has already solved (ILU factors, fused images, captured loop built).  The
    next solve of the refined problem equals, bit for bit, the solve on a
    hierarchy created from scratch for it, and the kept levels' arrays are
    untouched."""
    a = G.LocalGenerator(nuni, nloc, seed=5)
    b = G.LocalGenerator(nuni, nloc + 1, seed=5)
    la = [a.level(l) for l in range(a.nlevels)]
    lb = [b.level(l) for l in range(b.nlevels)]
    first = next(l for l in range(len(la)) if not _same_level(la[l], lb[l]))
    assert 1 <= first < len(la)

    def solver(mg):
        G.setup_lmgc(mg, sm, baselevel=0, damp=_damp(sm), red=1e-10, abslimit=1e-50)

    fresh = G.MultiGrid(lb, order=order)
    solver(fresh)
    x_ref, lr_ref = fresh.solve_host("mgs", b.rhs)
    fresh.close()

    mg = G.MultiGrid(la, order=order)
    solver(mg)
    mg.solve_host("mgs", a.rhs)
    kept = [mg.matrix(l) for l in range(first)]
    mg.replace_levels(first, lb[first:])
    assert mg.nlevels == len(lb) and mg.local
    for l in range(first):
        assert all(np.array_equal(u, v) for u, v in zip(mg.matrix(l), kept[l]))
    x, lr = mg.solve_host("mgs", b.rhs)
    assert lr.converged and lr.iters == lr_ref.iters
    assert np.array_equal(x, x_ref)
    # replacing the top with itself changes nothing
    mg.replace_levels(mg.top, lb[-1:])
    x2, lr2 = mg.solve_host("mgs", b.rhs)
    assert lr2.iters == lr_ref.iters and np.array_equal(x2, x_ref)
    mg.close()


def test_replace_levels_errors(G):
    gen = G.LocalGenerator(2, 2, seed=5)
    levels = [gen.level(l) for l in range(gen.nlevels)]
    mg = G.MultiGrid(levels)
    with pytest.raises(G.GmgError, match="first level"):
        mg.replace_levels(0, levels)
    with pytest.raises(G.GmgError, match="first level"):
        mg.replace_levels(len(levels) + 1, levels[-1:])
    bad = dict(levels[-1])
    bad["pcol"] = np.asarray(bad["pcol"]) + 10 ** 6
    with pytest.raises(G.GmgError, match="coarse index"):
        mg.replace_levels(mg.top, [bad])
    assert mg.nlevels == len(levels)  # a failed replacement keeps the hierarchy
    mg.close()
