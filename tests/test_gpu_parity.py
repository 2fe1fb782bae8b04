"""GPU parity of the lmgc path against the UG reference and its C restatement.

* Kernels: every level kernel called through the C ABI on UG's own hierarchies
  (tests/golden) reproduces UG's known-answer vectors; tolerance 1e-12
  relative (FP64; only the summation order inside a row differs).
* Solves: ls + lmgc with jac / gs / ilu in UG's VECTOR-list order takes UG's
  iteration count and reaches UG's solution (jac 1e-10, gs / ilu 1e-8
  relative, iterations +-1 allowed by the contract, equal in practice);
  in multicolour order it matches the oracle run on the same (reordered)
  hierarchy.
* Mixed precision: an FP32 V-cycle inside FP64 iterative refinement meets
  the FP64 stopping test; its error against a tightly converged FP64 oracle
  solution is bounded by 1e-6 relative.
* Full-size workloads: the 2D Q1 257x257 and 3D P1 65^3 hierarchies.
"""
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


def _setup(G, fx, order=0, fp32=False):
    levels = G.levels_from_ugfx(fx)
    mg = G.MultiGrid(levels, order=order, fp32=fp32)
    return mg, levels


def _damp(sm):
    return 0.8 if sm == "jac" else 1.0


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("name", NAMES)
def test_kernels_match_ug(G, oracle_mod, name, order):
    fx = load_golden(name)
    mg, levels = _setup(G, fx, order)
    top = mg.top
    mg.createvector("x", "y", "d", "v", "c", "t")
    mg.upload("x", top, fx["kat_x"]); mg.upload("y", top, fx["kat_y"])
    mg.dmatmul_minus(top, "x", "y")
    assert rel(mg.download("x", top), fx["kat_matmul"]) <= 1e-12
    mg.upload("d", top, fx["kat_d"])
    mg.l_jac(top, "v", "d")
    assert rel(mg.download("v", top), fx["kat_jac"]) <= 1e-12
    assert rel(mg.dnrm2x(top, "d"), fx["kat_nrm"]) <= 1e-12
    mg.upload("c", top - 1, fx["kat_restrict_pre"])
    mg.standard_restrict(top, "c", "d")
    assert rel(mg.download("c", top - 1), fx["kat_restrict"]) <= 1e-12
    mg.upload("c", top - 1, fx["kat_interp_coarse"])
    mg.upload("t", top, np.full(fx["kat_d"].size, 7.0))
    mg.standard_interpolate_correction(top, "t", "c")
    assert rel(mg.download("t", top), fx["kat_interp"]) <= 1e-12
    mg.l_lgs(top, "v", "d")
    gs = mg.download("v", top)
    mg.l_ilu_decomp(top)
    mg.l_luiter(top, "v", "d")
    ilu = mg.download("v", top)
    if order == 0:  # UG's own list order: UG's numbers
        assert rel(gs, fx["kat_gs"]) <= 1e-12
        assert rel(ilu, fx["kat_ilu"]) <= 1e-12
    else:  # multicolour order: the reference algorithm on the reordered grid
        H = oracle_mod.Hierarchy(permuted_levels(levels, mg))
        perm = mg.order(top)
        s = levels[top]["s"]
        d_p = fx["kat_d"].reshape(-1, s)[perm].ravel()
        ref_gs = np.empty((len(perm), s)); ref_gs[perm] = H.lgs(top, d_p).reshape(-1, s)
        assert rel(gs, ref_gs.ravel()) <= 1e-12
        lu = H.ilu_decomp(top)
        ref_ilu = np.empty((len(perm), s)); ref_ilu[perm] = H.luiter(top, lu, d_p).reshape(-1, s)
        assert rel(ilu, ref_ilu.ravel()) <= 1e-12
    mg.close()


@pytest.mark.parametrize("fuse", [0, None])
@pytest.mark.parametrize("name", NAMES)
def test_solve_matches_ug(G, name, fuse):
    """fuse=0: one kernel per level operation; None: the small levels run as
    one fused single-CTA kernel (here the whole hierarchy)."""
    fx = load_golden(name)
    mg, _ = _setup(G, fx, 0)
    sm = fx["smoother"]
    G.setup_lmgc(mg, sm, baselevel=int(fx["baselevel"][0]), damp=_damp(sm), red=1e-10, abslimit=1e-50, fuse=fuse)
    x, lr = mg.solve_host("mgs", fx["rhs"])
    it_ug = int(fx["ls_iters"][0])
    assert lr.converged
    assert abs(lr.first_defect[0] - fx["ls_hist"][0]) <= 1e-12 * fx["ls_hist"][0]
    if sm == "jac":
        assert lr.iters == it_ug
        assert rel(x, fx["ls_x"]) <= 1e-10
    else:
        assert abs(lr.iters - it_ug) <= 1
        assert rel(x, fx["ls_x"]) <= 1e-8
    # a second solve on the same device state is bitwise reproducible
    x2, lr2 = mg.solve_host("mgs", fx["rhs"])
    assert lr2.iters == lr.iters and np.array_equal(x, x2)
    mg.close()


@pytest.mark.parametrize("fuse", [0, None])
@pytest.mark.parametrize("name", NAMES)
def test_solve_multicolour_matches_oracle(G, oracle_mod, name, fuse):
    fx = load_golden(name)
    mg, levels = _setup(G, fx, 1)
    sm = fx["smoother"]
    bl = int(fx["baselevel"][0])
    G.setup_lmgc(mg, sm, baselevel=bl, damp=_damp(sm), red=1e-10, abslimit=1e-50, fuse=fuse)
    x, lr = mg.solve_host("mgs", fx["rhs"])
    H = oracle_mod.Hierarchy(permuted_levels(levels, mg))
    top = mg.top
    perm = mg.order(top)
    s = levels[top]["s"]
    xo, ito, conv, _ = H.ls_solve(fx["rhs"].reshape(-1, s)[perm].ravel(), smoother=sm, baselevel=bl,
                                  damp=_damp(sm), red=1e-10, abslimit=1e-50)
    xr = np.empty((len(perm), s)); xr[perm] = xo.reshape(-1, s)
    assert conv and lr.converged and lr.iters == ito
    assert rel(x, xr.ravel()) <= 1e-10
    mg.close()


@pytest.mark.parametrize("name", ["q1_jac", "p1k_gs", "el_ilu", "q1_ilu"])
def test_mixed_precision_refinement(G, oracle_mod, name):
    fx = load_golden(name)
    mg, levels = _setup(G, fx, 0, fp32=True)
    sm = fx["smoother"]
    bl = int(fx["baselevel"][0])
    G.setup_lmgc(mg, sm, baselevel=bl, damp=_damp(sm), red=1e-8, abslimit=1e-50, mixed=True)
    x, lr = mg.solve_host("mgs", fx["rhs"])
    assert lr.converged
    H = oracle_mod.Hierarchy(levels)
    top = mg.top
    # the FP64 defect of the mixed solution meets the stopping test
    d = H.matmul_minus(top, fx["rhs"], x)
    d0 = H.nrm2x(top, fx["rhs"])
    assert np.all(H.nrm2x(top, d) <= 1.01e-8 * d0)
    xo, ito, _, _ = H.ls_solve(fx["rhs"], smoother=sm, baselevel=bl, damp=_damp(sm), red=1e-13, abslimit=1e-50)
    assert rel(x, xo) <= 1e-6
    mg.close()


def test_numproc_status_and_errors(G):
    fx = load_golden("q1_jac")
    mg, _ = _setup(G, fx, 0)
    mg.createvector("sol", "rhs")
    mg.npcreate("lmgc", "iter.glmgc")
    assert mg.npinit("lmgc", "$n1 2") == G.NP_NOT_ACTIVE          # no $S / $T
    mg.npcreate("ls", "linear_solver.gls")
    assert mg.npinit("ls", "$m 5") == G.NP_NOT_ACTIVE             # no $I
    with pytest.raises(G.GmgError):
        mg.npcreate("bad", "iter.nosuchclass")
    with pytest.raises(G.GmgError):
        mg.npexecute("lmgc", "$s")                                  # not executable
    # the function-table entries refuse a numproc whose init failed or that
    # was never initialised (its $I / $S / $T partners are missing)
    with pytest.raises(G.GmgError, match="not initialised"):
        mg.ls_preprocess("ls", mg.top, "sol", "rhs")
    with pytest.raises(G.GmgError, match="not initialised"):
        mg.solve_host("ls", fx["rhs"])
    mg.npcreate("j", "iter.gjac")
    with pytest.raises(G.GmgError, match="not initialised"):
        mg.iter_iter("j", mg.top, "sol", "rhs")
    G.setup_lmgc(mg, "jac", baselevel=2)
    assert "n1 = 2" in mg.npdisplay("lmgc") and "baselevel = 2" in mg.npdisplay("lmgc")
    mg.upload("rhs", mg.top, fx["rhs"])
    mg.npexecute("mgs", "$i $d $r $s $p")
    assert rel(mg.download("sol", mg.top), fx["ls_x"]) <= 1e-10
    mg.close()


def test_vectors_of_another_multigrid_are_refused(G):
    """The BLAS entries and the numproc function-table entries refuse a
    missing vector and a vector of another hierarchy (whose levels and
    lengths differ) instead of handing its pointers to a kernel."""
    fx = load_golden("q1_jac")
    mg, _ = _setup(G, fx, 0)
    other, _ = _setup(G, fx, 0)
    mg.createvector("sol", "rhs")
    other.createvector("sol")
    L = G.lib()
    assert L.gmg_dset(mg._h, mg.top, other.vec("sol"), 1.0) != 0
    assert b"another multigrid" in L.gmg_last_error()
    assert L.gmg_dset(mg._h, mg.top, None, 1.0) != 0
    assert b"vector missing" in L.gmg_last_error()
    assert L.gmg_dcopy(mg._h, mg.top, mg.vec("sol"), other.vec("sol")) != 0
    assert L.gmg_dnrm2x(mg._h, mg.top, other.vec("sol"), None) != 0
    G.setup_lmgc(mg, "jac", baselevel=2)
    assert L.gmg_iter_iter(mg.np("lmgc"), mg.top, other.vec("sol"), mg.vec("rhs"), mg.mat(), None) != 0
    assert b"another multigrid" in L.gmg_last_error()
    assert L.gmg_ls_defect(mg.np("mgs"), mg.top, mg.vec("sol"), None, mg.mat(), None) != 0
    assert b"vector missing" in L.gmg_last_error()
    # the hierarchy still solves afterwards
    mg.upload("rhs", mg.top, fx["rhs"])
    mg.npexecute("mgs", "$i $d $r $s $p")
    assert rel(mg.download("sol", mg.top), fx["ls_x"]) <= 1e-10
    mg.close()
    other.close()


def test_full_size_q1_jacobi(G, oracle_mod):
    """2D Q1 Poisson 257x257 (66,049 unknowns), V(2,2) jac 0.8, base 4x4, red 1e-10."""
    gen = G.Generator(0, 8, seed=1)
    levels = gen.levels()
    mg = G.MultiGrid(levels)
    G.setup_lmgc(mg, "jac", baselevel=2, red=1e-10)
    x, lr = mg.solve_host("mgs", gen.rhs)
    H = oracle_mod.Hierarchy(levels)
    xo, ito, conv, _ = H.ls_solve(gen.rhs, smoother="jac", baselevel=2, damp=0.8, red=1e-10)
    assert lr.converged and conv and lr.iters == ito
    assert rel(x, xo) <= 1e-10
    mg.close()


def test_full_size_p1_diffusion_gs(G, oracle_mod):
    """3D P1 diffusion 65^3 (274,625 unknowns), k = exp(g), multicolour GS V(2,2), red 1e-8."""
    gen = G.Generator(1, 6, seed=2, corr=0.1, var=1.0)
    levels = gen.levels()
    mg = G.MultiGrid(levels, order=G.ORDER_COLOR)
    G.setup_lmgc(mg, "gs", baselevel=0, red=1e-8)
    x, lr = mg.solve_host("mgs", gen.rhs)
    H = oracle_mod.Hierarchy(permuted_levels(levels, mg))
    perm = mg.order(mg.top)
    xo, ito, conv, _ = H.ls_solve(gen.rhs[perm], smoother="gs", baselevel=0, red=1e-8)
    xr = np.empty_like(xo); xr[perm] = xo
    assert lr.converged and conv and lr.iters == ito
    assert rel(x, xr) <= 1e-10
    mg.close()


@pytest.mark.parametrize("kind", [1, 3], ids=["freudenthal", "ug_red_rules"])
def test_full_size_p1_diffusion_mixed(G, oracle_mod, kind):
    """The benchmarked solve itself: 3D P1 diffusion 65^3 (274,625 unknowns,
    k = exp(g), seed 2026), multicolour GS V(2,2), the FP32 V-cycle inside FP64
    iterative refinement to 1e-8, autotuned kernels, as bench.py runs it, on
    both tetrahedral meshes of the cube (UG's red rules, Freudenthal).
    Checked in FP64 by the oracle on the same (reordered) hierarchy: the
    solution meets the stopping test (FP64 defect <= 1e-8 of the first), takes
    the FP64 solve's iteration count +-1, and is within 1e-6 (relative,
    max-norm) of the FP64 solution converged to 1e-12."""
    gen = G.Generator(kind, 6, seed=2026, corr=0.1, var=1.0)
    levels = gen.levels()
    mg = G.MultiGrid(levels, order=G.ORDER_COLOR, fp32=True, autotune=True)
    G.setup_lmgc(mg, "gs", baselevel=0, red=1e-8, abslimit=1e-50)
    mg.npcreate("mgs32", "linear_solver.gls")
    mg.npinit("mgs32", "$A MAT $x sol $b rhs $red 1e-8 $abslimit 1e-50 $m 100 $I lmgc $mixed 1")
    x32, lr32 = mg.solve_host("mgs32", gen.rhs)
    x32b, _ = mg.solve_host("mgs32", gen.rhs)  # a second solve on the warm hierarchy (graph replay)
    H = oracle_mod.Hierarchy(permuted_levels(levels, mg))
    perm = mg.order(mg.top)
    b = gen.rhs[perm]
    _, it8, conv8, _ = H.ls_solve(b, smoother="gs", baselevel=0, red=1e-8, abslimit=1e-50)
    xt, _, convt, _ = H.ls_solve(b, smoother="gs", baselevel=0, red=1e-12, abslimit=1e-50, base_abslimit=1e-30)
    mg.close()
    xtl = np.empty_like(xt); xtl[perm] = xt
    assert lr32.converged and conv8 and convt and abs(lr32.iters - it8) <= 1
    assert np.array_equal(x32, x32b)
    d = H.matmul_minus(6, b, x32[perm])
    assert H.nrm2x(6, d)[0] <= 1.0000001e-8 * H.nrm2x(6, b)[0]
    assert rel(x32, xtl) <= 1e-6


MID = [  # generator kind, nref, smoother, baselevel, var
    (0, 6, "jac", 2, 0.0), (0, 6, "gs", 2, 0.0), (0, 6, "ilu", 2, 0.0),
    (1, 4, "gs", 0, 1.0), (1, 4, "ilu", 0, 1.0), (1, 4, "jac", 0, 1.0),
    (3, 4, "gs", 0, 1.0), (3, 4, "ilu", 0, 1.0), (3, 5, "gs", 0, 1.0),
    (2, 6, "gs", 1, 0.0), (2, 6, "ilu", 1, 0.0), (2, 6, "jac", 1, 0.0),
]


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("kind,nref,sm,bl,var", MID)
def test_midsize_vs_oracle(G, oracle_mod, kind, nref, sm, bl, var, order):
    """Levels above 2048 VECTORs use the sliced-ELLPACK kernels (and, in
    multicolour order, colour-range Gauss-Seidel waves); small levels the
    shared-memory fused cycle.  Same iterations and solution as the oracle."""
    gen = G.Generator(kind, nref, seed=5, corr=0.1, var=var)
    levels = gen.levels()
    mg = G.MultiGrid(levels, order=order, fp32=True)
    G.setup_lmgc(mg, sm, baselevel=bl, damp=_damp(sm), red=1e-10, abslimit=1e-50)
    x, lr = mg.solve_host("mgs", gen.rhs)
    H = oracle_mod.Hierarchy(permuted_levels(levels, mg))
    perm = mg.order(mg.top)
    s = levels[-1]["s"]
    xo, ito, conv, _ = H.ls_solve(gen.rhs.reshape(-1, s)[perm].ravel(), smoother=sm, baselevel=bl,
                                  damp=_damp(sm), red=1e-10, abslimit=1e-50)
    xr = np.empty((len(perm), s)); xr[perm] = xo.reshape(-1, s)
    assert conv and lr.converged and lr.iters == ito
    assert rel(x, xr.ravel()) <= 1e-10
    # the mixed-precision solver on the same device hierarchy
    mg.npcreate("mgs32", "linear_solver.gls")
    mg.npinit("mgs32", "$A MAT $x sol $b rhs $red 1e-8 $abslimit 1e-50 $m 100 $I lmgc $mixed 1")
    x32, lr32 = mg.solve_host("mgs32", gen.rhs)
    _, it8, _, _ = H.ls_solve(gen.rhs.reshape(-1, s)[perm].ravel(), smoother=sm, baselevel=bl,
                              damp=_damp(sm), red=1e-8, abslimit=1e-50)
    assert lr32.converged and abs(lr32.iters - it8) <= 1
    d = H.matmul_minus(mg.top, gen.rhs.reshape(-1, s)[perm].ravel(), x32.reshape(-1, s)[perm].ravel())
    assert np.all(H.nrm2x(mg.top, d) <= 1.01e-8 * H.nrm2x(mg.top, gen.rhs.reshape(-1, s)[perm].ravel()))
    mg.close()


@pytest.mark.parametrize("order", [0, 1, 2])
@pytest.mark.parametrize("name", golden_names("all"))
def test_solution_transfer_matches_ug(G, name, order):
    """NP_TRANSFER's InterpolateNewVectors and ProjectSolution (transfer.cc:775,
    794) on every level of UG's hierarchies: the new vectors of the last
    refinement take UG's interpolated values, the projection copies son to
    father as UG's StandardProject does, bit for bit."""
    fx = load_golden(name)
    mg = G.MultiGrid(G.levels_from_ugfx(fx), order=order)
    mg.createvector("x")
    mg.npcreate("tr", "transfer.gtransfer"); mg.npinit("tr", "")
    n = mg.nlevels
    offs = np.cumsum([0] + mg.level_len)
    for l in range(n):
        mg.set_new_vectors(l, fx[f"L{l}_vnew"])
    for pre, post, op in (("kat_newvec_pre", "kat_newvec", mg.transfer_interpolate_new_vectors),
                          ("kat_project_pre", "kat_project", mg.transfer_project_solution)):
        for l in range(n):
            mg.upload("x", l, fx[pre][offs[l]:offs[l + 1]])
        op("tr", 0, n - 1, "x")
        got = np.concatenate([mg.download("x", l) for l in range(n)])
        assert np.array_equal(got, fx[post]), (name, post)
    mg.close()


@pytest.mark.parametrize("fuse", [0, None])
@pytest.mark.parametrize("sm", ["jac", "gs", "ilu"])
def test_update_values_matches_ug(G, sm, fuse):
    """New matrix values on a resident hierarchy (gmg_mg_update_values): the
    3D Poisson hierarchy, solved once (ILU factors, base inverse, fused coarse
    images and the captured iteration built), gets the k = exp(g) diffusion
    values of every level (the same mesh); its next solve is UG's diffusion
    solve (iterations and solution)."""
    src, dst = load_golden("p1_gs"), load_golden(f"p1k_{sm}")
    n = int(src["nlevels"][0])
    for l in range(n):
        assert np.array_equal(src[f"L{l}_rowptr"], dst[f"L{l}_rowptr"])
        assert np.array_equal(src[f"L{l}_col"], dst[f"L{l}_col"])
    mg = G.MultiGrid(G.levels_from_ugfx(src), order=0)
    bl = int(dst["baselevel"][0])
    G.setup_lmgc(mg, sm, baselevel=bl, damp=0.8 if sm == "jac" else 1.0, red=1e-10, abslimit=1e-50, fuse=fuse)
    for _ in range(2):
        _, lr0 = mg.solve_host("mgs", src["rhs"])
        assert lr0.converged
    for l in range(n):
        mg.update_values(l, dst[f"L{l}_val"])
    x, lr = mg.solve_host("mgs", dst["rhs"])
    it_ug = int(dst["ls_iters"][0])
    assert lr.converged
    if sm == "jac":
        assert lr.iters == it_ug and rel(x, dst["ls_x"]) <= 1e-10
    else:
        assert abs(lr.iters - it_ug) <= 1 and rel(x, dst["ls_x"]) <= 1e-8
    x2, lr2 = mg.solve_host("mgs", dst["rhs"])  # replayed graph after the update
    assert lr2.iters == lr.iters and np.array_equal(x, x2)
    mg.close()


@pytest.mark.parametrize("maxit", [100, 3])
@pytest.mark.parametrize("name,order,mixed", [("p1_gs", 0, False), ("q1_jac", 1, False), ("el_ilu", 0, False),
                                              ("q1_gs", 1, True), ("ls_ilu", 0, False), ("ls_gs", 0, True)])
def test_device_loop_matches_host_loop(G, name, order, mixed, maxit):
    """ls's loop after the first iteration runs on the device as one
    conditional graph (a WHILE node over the iteration and the stopping test,
    ls.cc:680-730); the host loop ($dloop 0) is the same loop tested on the
    host.  Both stop at the same iteration (converged, or at $m unconverged)
    with the same last defect and the same x, bit for bit; the second solve
    replays the built loop graph."""
    fx = load_golden(name)
    levels = G.levels_from_ugfx(fx)
    sm = fx["smoother"]
    out = {}
    for dloop in (True, False):
        mg = G.MultiGrid(levels, order=order, fp32=mixed)
        G.setup_lmgc(mg, sm, baselevel=int(fx["baselevel"][0]), damp=_damp(sm), red=1e-10, abslimit=1e-50,
                     maxit=maxit, mixed=mixed, dloop=dloop)
        rhs = fx["rhs_all"] if mg.local else fx["rhs"]
        runs = [mg.solve_host("mgs", rhs) for _ in range(2)]
        out[dloop] = (runs, mg.npdisplay("mgs"))
        mg.close()
    (dev, dev_disp), (host, host_disp) = out[True], out[False]
    assert "loop = device (built)" in dev_disp, dev_disp
    assert "loop = host" in host_disp
    for (xd, ld), (xh, lh) in zip(dev, host):
        assert ld.iters == lh.iters and ld.converged == lh.converged
        assert ld.converged == (maxit == 100)
        assert ld.iters == (lh.iters if maxit == 100 else 3)
        assert list(ld.last_defect) == list(lh.last_defect)
        assert np.array_equal(xd, xh)


@pytest.mark.parametrize("name,order", [("p1k_gs", 1), ("p1k_ilu", 0), ("q1_jac", 0), ("el_ilu", 0), ("el_gs", 1),
                                        ("ls_gs", 0)])
def test_coarse_narrow_team_is_bit_identical(G, name, order):
    """The fused coarse cycle runs its smallest levels (at most ~4 rows per
    lane group) with a team of 128 threads on a named barrier while the other
    warps wait once ($narrow 1, the default).  Rows, lanes per row and the
    summation order are those of the whole block, so the solve is identical
    bit for bit to $narrow 0."""
    fx = load_golden(name)
    levels = G.levels_from_ugfx(fx)
    sm = fx["smoother"]
    out = []
    for narrow in (True, False):
        mg = G.MultiGrid(levels, order=order)
        G.setup_lmgc(mg, sm, baselevel=int(fx["baselevel"][0]), damp=_damp(sm), red=1e-10, abslimit=1e-50,
                     narrow=narrow)
        out.append(mg.solve_host("mgs", fx["rhs_all"] if mg.local else fx["rhs"]))
        mg.close()
    (x1, l1), (x0, l0) = out
    assert l1.converged and l1.iters == l0.iters
    assert np.array_equal(x1, x0)


def _bsr_apply(d, y):
    s = int(d["s"]); rp, col = np.asarray(d["rowptr"]), np.asarray(d["col"])
    val = np.asarray(d["val"]).reshape(-1, s, s)
    yb = np.asarray(y).reshape(-1, s)
    out = np.zeros_like(yb)
    for i in range(int(d["n"])):
        for k in range(rp[i], rp[i + 1]):
            out[i] += val[k] @ yb[col[k]]
    return out.ravel()


@pytest.mark.parametrize("name", ["q1_jac", "el_ilu", "p1k_gs"])
def test_blas_level_operations(G, name):
    """dmatmul, dmatmul_add, dscalx, daxpy, ddot (ugblas.cc:3782, 3889, 2510,
    2875, 3104) on one level against numpy, 1e-12 relative."""
    fx = load_golden(name)
    levels = G.levels_from_ugfx(fx)
    mg = G.MultiGrid(levels, order=1)
    top = mg.top
    d = levels[top]
    s = int(d["s"])
    rng = np.random.default_rng(3)
    x0, y = rng.uniform(-1, 1, d["n"] * s), rng.uniform(-1, 1, d["n"] * s)
    mg.createvector("x", "y")
    mg.upload("y", top, y)
    ay = _bsr_apply(d, y)
    mg.upload("x", top, x0); mg.dmatmul(top, "x", "y")
    assert rel(mg.download("x", top), ay) <= 1e-12
    mg.upload("x", top, x0); mg.dmatmul_add(top, "x", "y")
    assert rel(mg.download("x", top), x0 + ay) <= 1e-12
    a = np.array([0.5, -2.0, 3.0])[:s]
    mg.upload("x", top, x0); mg.dscalx(top, "x", a)
    assert rel(mg.download("x", top), (x0.reshape(-1, s) * a).ravel()) <= 1e-15
    mg.upload("x", top, x0); mg.daxpy(top, "x", a, "y")
    assert rel(mg.download("x", top), (x0.reshape(-1, s) + a * y.reshape(-1, s)).ravel()) <= 1e-15
    mg.upload("x", top, x0)
    assert abs(mg.ddot(top, "x", "y") - float(x0 @ y)) <= 1e-12 * np.sum(np.abs(x0 * y))
    mg.close()


def test_host_copy_paths_agree(G):
    """Host vectors through pinned staging (the path of hosts whose GPU cannot
    read pageable memory) and, where the device reads host page tables,
    straight from / to pageable memory: the same solution and iterations,
    bit for bit, through gmg_solve_host and the per-level upload / download."""
    fx = load_golden("p1k_jac")
    levels = G.levels_from_ugfx(fx)
    out = []
    for direct in (False, True):
        mg = G.MultiGrid(levels, order=1)
        try:
            mg.set_direct_host(direct)
        except G.GmgError:
            mg.close()
            assert direct  # only the direct path can be unavailable
            continue
        G.setup_lmgc(mg, "jac", baselevel=0, damp=0.8, red=1e-10)
        x, lr = mg.solve_host("mgs", fx["rhs"])
        mg.createvector("v")
        mg.upload("v", mg.top, fx["rhs"])
        back = mg.download("v", mg.top)
        out.append((x, lr.iters, back))
        mg.close()
    assert np.array_equal(out[0][2], fx["rhs"])
    if len(out) == 2:
        assert out[0][1] == out[1][1] and np.array_equal(out[0][0], out[1][0])
        assert np.array_equal(out[1][2], fx["rhs"])
