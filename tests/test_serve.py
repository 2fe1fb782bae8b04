"""Serving pools and the continuous-batching loop (ug_gb300/serve.py,
ug_gb300/csrc/gmg_serve.cpp, gmg_assemble.cu).

* On-device assembly reproduces the host generator's matrices, on both
  cube meshes (UG's red rules, the pools' default, and the Freudenthal
  triangulation): exactly up to
  rounding (1e-13 relative) for k = 1, and to 1e-12 relative with the
  log-normal field evaluated in FP64 (the pools' default), so a slot holds
  the FP64 problem; with the optional FP32 field (phases in 32-bit fixed
  point, FP32 cosines, ~1e-6 relative in k) to 2e-5.  The right-hand side is
  the same position-keyed load (1e-15).
* Alone == in the mix: a request's solution and iteration count are bitwise
  the same whether it runs alone in a pool or joins it between iterations
  while other requests come and go (same pool shape; every kernel is
  row-local per slot and the norms reduce each slot's rows in a fixed order).
* In the mix vs the host-assembled problem solved alone (MultiGrid on the
  generator's hierarchy, the same mixed-precision solver): the same
  iterations and solution to 1e-10; and against the FP64 oracle's solution
  of the host-assembled problem converged to 1e-12: within 1e-6 (the stopping
  test at 1e-8).
"""
import numpy as np
import pytest

from conftest import rel


@pytest.fixture(scope="module")
def G():
    import ug_gb300
    ug_gb300.lib()
    return ug_gb300


def test_stream_is_seeded(G):
    from ug_gb300.serve import poisson_stream, slot_bytes
    a, b = poisson_stream(50, 200.0), poisson_stream(50, 200.0)
    assert [(r.arrival, r.nref, r.seed) for r in a] == [(r.arrival, r.nref, r.seed) for r in b]
    assert all(2 <= r.nref <= 7 for r in a) and all(x.arrival < y.arrival for x, y in zip(a, a[1:]))
    assert abs(np.mean(np.diff([r.arrival for r in poisson_stream(4000, 200.0)])) - 1 / 200) < 3e-4
    assert slot_bytes(7) > 7 * slot_bytes(6) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("mesh", [3, 1], ids=["ug_red_rules", "freudenthal"])
@pytest.mark.parametrize("var,fp64,tol", [(0.0, True, 1e-13), (1.0, True, 1e-12), (1.0, False, 2e-5)])
@pytest.mark.parametrize("nref", [3, 5])
def test_device_assembly_matches_generator(G, var, fp64, tol, nref, mesh):
    from ug_gb300.serve import Pool
    seed = 77
    pool = Pool(nref, 2, field_fp64=fp64, mesh=mesh)
    pool.free.remove(1)
    pool.admit(1, seed, 0.1, var)
    gen = G.Generator(mesh, nref, seed=seed, corr=0.1, var=var)
    for l in range(nref + 1):
        ref = gen.level(l)["val"]
        got = pool.slot_matrix(1, l, ref.size)
        assert rel(got, ref) <= tol, l
    # the slot's right-hand side is the generator's (packed: slot after slot)
    mg = G.lib().gmg_pool_multigrid(pool._h)
    b = np.empty(pool.n_top * 2)
    assert G.lib().gmg_vec_download_packed(G.lib().gmg_vec_by_name(mg, b"rhs"), b.ctypes.data) == 0
    assert rel(b[pool.n_top:], gen.rhs) <= 1e-15
    pool.close()


def _mixed_solo(G, nref, seed, var, mesh=3):
    gen = G.Generator(mesh, nref, seed=seed, corr=0.1, var=var)
    mg = G.MultiGrid(gen, order=G.ORDER_COLOR, fp32=True)
    G.setup_lmgc(mg, "gs", red=1e-8, abslimit=1e-50, mixed=True)
    x, lr = mg.solve_host("mgs", gen.rhs)
    mg.close()
    return x, lr


@pytest.mark.gpu
def test_alone_equals_in_the_mix(G):
    from ug_gb300.serve import Pool
    nref, seed = 4, 4242
    alone = Pool(nref, 3)
    xa, lra = alone.solve(seed, slot=0)
    alone.close()
    # the same request joins a pool at its third iteration, in another slot,
    # while two others run and one more arrives later
    mix = Pool(nref, 3)
    got = {}
    others = [11, 12, 13]
    mix.free = []
    mix.admit(0, others[0], 0.1, 1.0)
    mix.active = {0: others[0]}
    it = 0
    pending = [(2, 1, seed), (4, 2, others[1])]  # (iteration, slot, seed)
    while mix.active or pending:
        while pending and pending[0][0] <= it:
            _, k, s = pending.pop(0)
            mix.admit(k, s, 0.1, 1.0)
            mix.active[k] = s
        mix.launch()
        while (done := mix.poll()) is None:
            pass
        it += 1
        for k in done:
            s = mix.active.pop(k)
            x, lr = mix.fetch(k)
            got[s] = (x, lr)
            if s == others[0] and others[2] not in got and 0 not in mix.active:
                mix.admit(0, others[2], 0.1, 1.0)  # a new request reuses the freed slot
                mix.active[0] = others[2]
    mix.close()
    xm, lrm = got[seed]
    assert lrm.converged and lra.converged and lrm.iters == lra.iters
    assert np.array_equal(xm, xa)
    assert all(got[s][1].converged for s in others)
    # the host-assembled problem solved alone: the same FP64 problem
    xs, lrs = _mixed_solo(G, nref, seed, 1.0)
    assert lrs.iters == lrm.iters and rel(xm, xs) <= 1e-10
    # ... and its FP64 oracle solution
    import oracle
    oracle.build()
    gen = G.Generator(G.Generator.DIFFUSION3D_UG, nref, seed=seed, corr=0.1, var=1.0)
    H = oracle.Hierarchy(gen.levels())
    xo, _, conv, _ = H.ls_solve(gen.rhs, smoother="gs", baselevel=0, red=1e-12, abslimit=1e-50, base_abslimit=1e-30)
    assert conv and rel(xm, xo) <= 1e-6


@pytest.mark.gpu
def test_server_stream(G):
    """A short Poisson stream through the server: every request converges and
    equals its alone solution; latencies are measured."""
    from ug_gb300.serve import Pool, Server, poisson_stream
    reqs = poisson_stream(18, 3000.0, levels=(1, 3), seed=9)
    srv = Server(depths=range(1, 4), slots={1: 2, 2: 3, 3: 2})
    st = srv.run(reqs, keep_x=True)
    srv.close()
    assert st.completed == 18 and st.all_converged and st.p99_ms >= st.p50_ms > 0
    for L, n in ((1, 2), (2, 3), (3, 2)):
        p = Pool(L, n, field_fp64=srv.field_fp64)
        for r in [q for q in reqs if q.nref == L][:3]:
            xa, lra = p.solve(r.seed, slot=0)
            assert lra.iters == r.iters and np.array_equal(xa, r.x), (L, r.rid)
        p.close()


@pytest.mark.gpu
def test_mixed_pool_batches_depths(G):
    """A mixed pool (slots of depths 2, 2, 3, 3, 4 in one batched hierarchy,
    every iteration one V-cycle over all of them, level by level): a depth-3
    request gives bitwise the same result alone in such a pool and joining it
    while depth-2 and depth-4 requests come and go; and the same iterations
    and solution to 1e-10 as in a pool of depth-3 slots only."""
    from ug_gb300.serve import Pool
    dep = [2, 2, 3, 3, 4]
    seed = 515
    alone = Pool(0, 0, depths=dep)
    xa, lra = alone.solve(seed, slot=3)
    alone.close()
    mix = Pool(0, 0, depths=dep)
    mix.free = []
    mix.admit(0, 21, 0.1, 1.0)
    mix.admit(4, 22, 0.1, 1.0)
    mix.active = {0: 21, 4: 22}
    got, it, joined = {}, 0, False
    while mix.active:
        if it == 2 and not joined:
            mix.admit(3, seed, 0.1, 1.0)
            mix.active[3] = seed
            joined = True
        mix.launch()
        while (done := mix.poll()) is None:
            pass
        it += 1
        for k in done:
            s = mix.active.pop(k)
            got[s] = mix.fetch(k)
            if s == 21:
                mix.admit(1, 23, 0.1, 1.0)  # another depth-2 request in the other depth-2 slot
                mix.active[1] = 23
    mix.close()
    xm, lrm = got[seed]
    assert lrm.converged and lrm.iters == lra.iters and np.array_equal(xm, xa)
    assert all(got[q][1].converged for q in (21, 22, 23))
    assert len(got[22][0]) == 17 ** 3 and len(got[21][0]) == 5 ** 3
    uni = Pool(3, 2)
    xu, lru = uni.solve(seed)
    uni.close()
    assert lru.iters == lrm.iters and rel(xm, xu) <= 1e-10


@pytest.mark.gpu
def test_server_stream_mixed_pools(G):
    """The server with depths 1..3 sharing mixed pools: every request converges
    and matches its solution in a pool of its own depth to 1e-10."""
    from ug_gb300.serve import Pool, Server, poisson_stream
    reqs = poisson_stream(18, 3000.0, levels=(1, 3), seed=10)
    srv = Server(depths=range(1, 4), slots={1: 2, 2: 3, 3: 2}, mixed=[(1, 2, 3)])
    assert len(srv.all_pools) == 1 and sorted(srv.all_pools[0].depths) == [1, 1, 2, 2, 2, 3, 3]
    st = srv.run(reqs, keep_x=True)
    srv.close()
    assert st.completed == 18 and st.all_converged
    for L, n in ((1, 2), (2, 3), (3, 2)):
        p = Pool(L, n, field_fp64=srv.field_fp64)
        for r in [q for q in reqs if q.nref == L][:3]:
            xa, lra = p.solve(r.seed, slot=0)
            assert lra.iters == r.iters and rel(r.x, xa) <= 1e-10, (L, r.rid)
        p.close()


@pytest.mark.gpu
def test_server_grows_pools_by_free_memory(G):
    """Demand-driven growth: one one-slot pool of depth 3 and a burst of
    requests; once requests have waited, the server creates (on a helper
    thread, the loop serving on) another pool of that shape because the
    device's free memory allows it, and the burst finishes with every
    request converged and equal to its alone solution."""
    from ug_gb300.serve import Pool, Server, poisson_stream
    reqs = [r for r in poisson_stream(400, 3000.0, levels=(3, 3), seed=12)][:120]
    srv = Server(depths=[3], layout={3: (1, 1)}, grow_after_ms=5.0)
    assert srv._may_grow(3)
    st = srv.run(reqs, keep_x=True)
    grown = list(srv.grown)
    npools = len(srv.pools[3])
    srv.close()
    assert st.completed == len(reqs) and st.all_converged
    assert grown and npools == 1 + len(grown) and all(L == 3 for _, L in grown)
    p = Pool(3, 1, field_fp64=srv.field_fp64)
    for r in reqs[:3]:
        xa, lra = p.solve(r.seed)
        assert lra.iters == r.iters and np.array_equal(xa, r.x)
    p.close()
