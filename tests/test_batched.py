"""Batched hierarchies (gmg_mg_create_batched): independent instances of
different depths stored block-diagonally, advanced by one union V-cycle per
ls iteration with per-instance convergence tests.

Each instance's result is the one it gets alone:
* against the oracle (UG's algorithm, list order): iterations equal (+-1 by
  the contract) and the solution within 1e-10 relative (FP64 jac / gs / ilu);
* against its own single-instance device solve in multicolour order (the
  batch keeps every instance's own colouring): same iterations, 1e-10;
* mixed precision: the FP64 stopping test holds per instance (defect
  <= 1.01e-8 x initial, checked with the oracle's FP64 matmul) and the
  iteration count is the solo one +-1.
The host-side checks of the batched layout run without a GPU."""
import numpy as np
import pytest

from conftest import permuted_levels, rel


@pytest.fixture(scope="module")
def G():
    import ug_gb300
    ug_gb300.lib()
    return ug_gb300


def _damp(sm):
    return 0.8 if sm == "jac" else 1.0


def _instances(G, kind, nrefs, var=0.5, seed0=100):
    return [G.Generator(kind, n, seed=seed0 + k, corr=0.1, var=var) for k, n in enumerate(nrefs)]


def test_batched_rejects_non_surface_top(G):
    """An instance's top level must be its surface (VNCLASS < 2, UG's top
    level); the check runs on the host before any device work."""
    gen = G.Generator(0, 2, seed=1)
    levels = gen.levels()
    bad = [dict(d) for d in levels]
    bad[-1]["vnclass"] = np.full(bad[-1]["n"], 3, np.int32)
    with pytest.raises(G.GmgError, match="VNCLASS"):
        G.MultiGrid([levels, bad], batched=True)


def test_batched_rejects_mixed_block_sizes(G):
    a = G.Generator(0, 2, seed=1).levels()
    b = G.Generator(2, 2, seed=1).levels()
    with pytest.raises(G.GmgError, match="block size"):
        G.MultiGrid([a, b], batched=True)


BATCHES = [  # kind, nrefs of the instances, smoother, order, baselevel
    (0, [2, 5, 3, 4, 2, 3], "jac", 0, 0),
    (0, [2, 5, 3, 4, 2, 3], "gs", 0, 0),
    (0, [3, 4, 2, 5], "ilu", 0, 0),
    (0, [2, 5, 3, 4, 2, 3], "jac", 1, 0),
    (0, [2, 5, 3, 4, 2, 3], "gs", 1, 1),
    (1, [1, 3, 2], "gs", 1, 0),
    (2, [2, 4, 3], "ilu", 1, 1),
    (2, [2, 4, 3], "jac", 0, 1),
]


@pytest.mark.gpu
@pytest.mark.parametrize("bsmem", [None, 0, 200000])
@pytest.mark.parametrize("kind,nrefs,sm,order,bl", BATCHES)
def test_batched_equals_alone(G, oracle_mod, kind, nrefs, sm, order, bl, bsmem):
    """bsmem: the per-instance shared-memory budget of the batched fused
    coarse cycle (None: default; 0: every level as separate launches;
    200000: deep fusion, shallow instances run their whole cycle there)."""
    gens = _instances(G, kind, nrefs, var=0.5 if kind != 2 else 0.0)
    insts = [g.levels() for g in gens]
    mg = G.MultiGrid(insts, batched=True, order=order, fp32=True)
    assert mg.ninst == len(nrefs) and mg.inst_top == [len(l) - 1 for l in insts]
    G.setup_lmgc(mg, sm, baselevel=bl, damp=_damp(sm), red=1e-10, abslimit=1e-50, bsmem=bsmem)
    b = mg.pack([g.rhs for g in gens])
    x, lr = mg.solve_host("mgs", b)
    assert lr.converged
    xs = mg.split(x)
    s = insts[0][0]["s"]
    for k, (g, levels) in enumerate(zip(gens, insts)):
        r = mg.instance_result("mgs", k)
        solo = G.MultiGrid(levels, order=order, fp32=True)
        G.setup_lmgc(solo, sm, baselevel=bl, damp=_damp(sm), red=1e-10, abslimit=1e-50)
        x1, lr1 = solo.solve_host("mgs", g.rhs)
        assert r.converged and abs(r.iters - lr1.iters) <= 1, (k, r.iters, lr1.iters)
        assert rel(xs[k], x1) <= 1e-10, k
        assert np.allclose(r.first_defect[:s], lr1.first_defect[:s], rtol=1e-12, atol=0)
        if order == 0:
            H = oracle_mod.Hierarchy(levels)
            xo, ito, conv, _ = H.ls_solve(g.rhs, smoother=sm, baselevel=bl, damp=_damp(sm), red=1e-10,
                                          abslimit=1e-50)
            assert conv and abs(r.iters - ito) <= 1
            assert rel(xs[k], xo) <= 1e-10
        solo.close()
    # the mixed-precision solver on the same batched hierarchy
    mg.npcreate("mgs32", "linear_solver.gls")
    mg.npinit("mgs32", "$A MAT $x sol $b rhs $red 1e-8 $abslimit 1e-50 $m 100 $I lmgc $mixed 1")
    x32, lr32 = mg.solve_host("mgs32", b)
    assert lr32.converged
    for k, (g, levels) in enumerate(zip(gens, insts)):
        r = mg.instance_result("mgs32", k)
        solo = G.MultiGrid(levels, order=order, fp32=True)
        H = oracle_mod.Hierarchy(permuted_levels(levels, solo))
        perm = solo.order(len(levels) - 1)
        G.setup_lmgc(solo, sm, baselevel=bl, damp=_damp(sm), red=1e-8, abslimit=1e-50, mixed=True)
        _, lr1 = solo.solve_host("mgs", g.rhs)
        assert r.converged and abs(r.iters - lr1.iters) <= 1, (k, r.iters, lr1.iters)
        bp = g.rhs.reshape(-1, s)[perm].ravel()
        d = H.matmul_minus(len(levels) - 1, bp, mg.split(x32)[k].reshape(-1, s)[perm].ravel())
        top = len(levels) - 1
        assert np.all(H.nrm2x(top, d) <= 1.01e-8 * H.nrm2x(top, bp)), k
        solo.close()
    mg.close()


@pytest.mark.gpu
def test_batched_converged_instances_stay(G):
    """An instance that starts converged (zero right-hand side) keeps x = 0
    and reports 0 iterations while the others iterate; graph replay and
    eager launches give bitwise the same batch."""
    gens = _instances(G, 0, [3, 4, 2])
    insts = [g.levels() for g in gens]
    rhs = [g.rhs.copy() for g in gens]
    rhs[1][:] = 0.0
    out = []
    for graph in (True, False):
        mg = G.MultiGrid(insts, batched=True, fp32=True)
        G.setup_lmgc(mg, "jac", red=1e-8, abslimit=1e-50, mixed=True, graph=graph)
        x, lr = mg.solve_host("mgs", mg.pack(rhs))
        r = [mg.instance_result("mgs", k) for k in range(3)]
        assert r[1].converged and r[1].iters == 0 and np.all(mg.split(x)[1] == 0.0)
        assert r[0].iters > 1 and r[2].iters > 1 and lr.iters == max(q.iters for q in r)
        out.append(x)
        mg.close()
    assert np.array_equal(out[0], out[1])


@pytest.mark.gpu
@pytest.mark.parametrize("mixed,maxit", [(True, 100), (False, 100), (True, 3)])
def test_batched_device_loop_matches_host_loop(G, mixed, maxit):
    """The batched ls loop after the first iteration (every later solve: all
    of it) runs as one conditional graph whose test keeps every instance's
    convergence, iteration count and last defect on the device; the host loop
    ($dloop 0) gives the same per-instance results and the same x, bit for
    bit, including an instance converged from the start and, with $m 3,
    instances stopped unconverged."""
    gens = _instances(G, 0, [3, 5, 2, 4, 6])
    insts = [g.levels() for g in gens]
    rhs = [g.rhs.copy() for g in gens]
    rhs[2][:] = 0.0
    out = {}
    for dloop in (True, False):
        mg = G.MultiGrid(insts, batched=True, fp32=True)
        G.setup_lmgc(mg, "jac", red=1e-8, abslimit=1e-50, mixed=mixed, maxit=maxit, dloop=dloop)
        runs = []
        for _ in range(2):
            x, lr = mg.solve_host("mgs", mg.pack(rhs))
            r = [mg.instance_result("mgs", k) for k in range(len(gens))]
            runs.append((x, lr.iters, lr.converged,
                         [(q.iters, q.converged, list(q.last_defect)) for q in r]))
        out[dloop] = (runs, mg.npdisplay("mgs"))
        mg.close()
    (dev, dev_disp), (host, host_disp) = out[True], out[False]
    assert "loop = device (built)" in dev_disp and "loop = host" in host_disp
    for (xd, itd, cd, rd), (xh, ith, ch, rh) in zip(dev, host):
        assert itd == ith and cd == ch and rd == rh
        assert np.array_equal(xd, xh)
        assert rd[2][0] == 0 and rd[2][1]
        assert cd == (maxit == 100)


@pytest.mark.gpu
def test_batched_many_small_instances(G, oracle_mod):
    """64 instances of levels 3..7 (the batched workload's size range, fewer
    instances): every instance meets its own stopping test."""
    rng = np.random.default_rng(7)
    nrefs = [int(v) for v in rng.integers(3, 8, size=64)]
    gens = _instances(G, 0, nrefs, var=0.5, seed0=1000)
    insts = [g.levels() for g in gens]
    mg = G.MultiGrid(insts, batched=True, order=G.ORDER_COLOR, fp32=True)
    G.setup_lmgc(mg, "jac", red=1e-8, abslimit=1e-50, mixed=True)
    x, lr = mg.solve_host("mgs", mg.pack([g.rhs for g in gens]))
    assert lr.converged
    xs = mg.split(x)
    for k in rng.choice(64, size=8, replace=False):
        levels = insts[k]
        top = len(levels) - 1
        H = oracle_mod.Hierarchy(levels)
        d = H.matmul_minus(top, gens[k].rhs, xs[k])
        assert np.all(H.nrm2x(top, d) <= 1.01e-8 * H.nrm2x(top, gens[k].rhs)), k
    mg.close()
