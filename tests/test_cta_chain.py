"""Chained Gauss-Seidel steps of a multicolour level in one thread block
(sell_gs_chain_cta_kernel) or one thread-block cluster of 2-16 blocks
(sell_gs_chain_cluster_kernel), set by gmg_mg_set_level_cta_chain, against
the same steps as one launch per colour wave: every row does the same
arithmetic in the same order, so whole lmgc solves (FP64 and the FP32
V-cycle in FP64 refinement) agree bit for bit, on both tetrahedral meshes of
the cube and on 2x2-block elasticity."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import ug_gb300
    ug_gb300.lib()
    return ug_gb300

CASES = [  # generator kind, nref, base level, {level: blocks}
    (3, 5, 0, {4: 1}),          # UG's mesh: level 4 = 4913 rows, 7 colours
    (1, 5, 0, {4: 1}),          # Freudenthal: 4 colours
    (2, 6, 1, {6: 1}),          # plane-strain elasticity, 4225 rows of 2x2 blocks
    (3, 5, 0, {4: 2, 5: 8}),    # clusters: level 4 rows streamed (2 blocks) or staged
    #                             in shared memory (4+); level 5 = 35,937 rows, 8 colours
    (3, 5, 0, {4: 8, 5: 16}),
    (3, 5, 0, {5: 8}),
    (1, 5, 0, {4: 4, 5: 8}),
    (2, 6, 1, {6: 2}),          # 2x2 blocks in a cluster
    (2, 6, 1, {6: 16}),
]


def _solve(G, gen, bl, cta_levels, fp32):
    mg = G.MultiGrid(gen.levels(), order=G.ORDER_COLOR, fp32=fp32)
    for l, nb in cta_levels.items():
        mg.set_cta_chain(l, nb)
        assert mg.level_variant(l)["cta_chain"] == nb
    G.setup_lmgc(mg, "gs", baselevel=bl, red=1e-10, abslimit=1e-50)
    out = {}
    x, lr = mg.solve_host("mgs", gen.rhs)
    out["fp64"] = (x, lr.iters)
    if fp32:
        mg.npcreate("mgs32", "linear_solver.gls")
        mg.npinit("mgs32", "$A MAT $x sol $b rhs $red 1e-8 $abslimit 1e-50 $m 100 $I lmgc $mixed 1")
        x32, lr32 = mg.solve_host("mgs32", gen.rhs)
        out["mixed"] = (x32, lr32.iters)
    mg.close()
    return out


@pytest.mark.parametrize("kind,nref,bl,levels", CASES)
def test_cta_chain_bit_identical(G, kind, nref, bl, levels):
    gen = G.Generator(kind, nref, seed=9, corr=0.1, var=1.0 if kind != 2 else 0.0)
    ref = _solve(G, gen, bl, {}, fp32=True)
    cta = _solve(G, gen, bl, levels, fp32=True)
    for key in ("fp64", "mixed"):
        assert cta[key][1] == ref[key][1], key
        assert np.array_equal(cta[key][0], ref[key][0]), key


def test_cta_chain_refuses_large_levels(G):
    gen = G.Generator(1, 6, seed=9, corr=0.1, var=1.0)
    mg = G.MultiGrid(gen.levels(), order=G.ORDER_COLOR, fp32=True)
    with pytest.raises(G.GmgError, match="one thread block"):
        mg.set_cta_chain(6, True)  # 274,625 rows: t and c need 2.2 MB
    with pytest.raises(G.GmgError, match="cluster of 16"):
        mg.set_cta_chain(6, 16)  # t alone needs 1.1 MB in every block
    with pytest.raises(G.GmgError, match="bad arguments"):
        mg.set_cta_chain(5, 3)
    with pytest.raises(G.GmgError):
        mg.set_cta_chain(1, True)  # 27 rows: a CSR level, no sliced-ELLPACK copy
    mg.close()
    # level 5 (35,937 rows): its FP64 t (287 KB) fits no block; with the FP32
    # t (144 KB) each block's slots (c, inverse diagonal, row start and width
    # of its rows) fit for 8 or 16 blocks, not for 2 (18k rows a block)
    gen = G.Generator(3, 5, seed=9, corr=0.1, var=1.0)
    mg = G.MultiGrid(gen.levels(), order=G.ORDER_COLOR, fp32=False)
    with pytest.raises(G.GmgError, match="cluster of 8"):
        mg.set_cta_chain(5, 8)
    mg.close()
    mg = G.MultiGrid(gen.levels(), order=G.ORDER_COLOR, fp32=True)
    with pytest.raises(G.GmgError, match="cluster of 2"):
        mg.set_cta_chain(5, 2)
    mg.set_cta_chain(5, 8)
    mg.close()


def test_autotuner_choice_is_reported(G):
    gen = G.Generator(3, 5, seed=9, corr=0.1, var=1.0)
    mg = G.MultiGrid(gen.levels(), order=G.ORDER_COLOR, fp32=True, autotune=True)
    v = [mg.level_variant(l)["cta_chain"] for l in range(mg.nlevels)]
    mg.close()
    assert all(x in (0, 1, 2, 4, 8, 16) for x in v)
    assert all(x == 0 for x in v[:3])  # CSR levels
