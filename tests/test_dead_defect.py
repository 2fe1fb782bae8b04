"""lmgc leaves out the final defect of a post-smoothing where nothing reads
it: a coarse level of a V-cycle whose defect the next restriction
overwrites, and the top of a mixed ls iteration, whose FP32 defect is
rebuilt from the FP64 one.  The solutions must be bit for bit those of
`$defect 1`, which computes every final defect as UG does.  Checked on
uniform hierarchies (chained Gauss-Seidel on both cube meshes and on 2x2
blocks, Jacobi) and batched ones of mixed depths (the serving pools'
case), FP64 and mixed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import ug_gb300
    ug_gb300.lib()
    return ug_gb300


def _solves(G, levels, rhs, sm, order, bl, defect, batched=False):
    mg = G.MultiGrid(levels, batched=batched, order=order, fp32=True)
    G.setup_lmgc(mg, sm, baselevel=bl, red=1e-10, abslimit=1e-50, defect=defect)
    assert ("every level" if defect else "where read") in mg.npdisplay("lmgc")
    mg.npcreate("mgs32", "linear_solver.gls")
    mg.npinit("mgs32", "$A MAT $x sol $b rhs $red 1e-8 $abslimit 1e-50 $m 100 $I lmgc $mixed 1")
    b = mg.pack(rhs) if batched else rhs
    x64, l64 = mg.solve_host("mgs", b)
    x32, l32 = mg.solve_host("mgs32", b)
    assert l64.converged and l32.converged
    mg.close()
    return x64, l64.iters, x32, l32.iters


def _same(a, b):
    assert a[1] == b[1] and a[3] == b[3]
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[2], b[2])


@pytest.mark.parametrize("kind,nref,sm,order,bl", [
    (3, 5, "gs", 1, 0),   # UG's mesh of the cube, chained GS on every level above the fused cycle
    (1, 5, "gs", 1, 0),   # Freudenthal triangulation
    (2, 6, "gs", 1, 1),   # plane-strain elasticity, 2x2 blocks
    (0, 7, "jac", 0, 2),  # 2D Q1 Poisson, Jacobi (its last step only adds its correction)
])
def test_uniform_solutions_unchanged(G, kind, nref, sm, order, bl):
    gen = G.Generator(kind, nref, seed=5, corr=0.1, var=1.0 if kind in (1, 3) else 0.0)
    levels = gen.levels()
    _same(_solves(G, levels, gen.rhs, sm, order, bl, defect=False),
          _solves(G, levels, gen.rhs, sm, order, bl, defect=True))


@pytest.mark.parametrize("kind,nrefs,sm,order", [
    (3, [2, 4, 3, 4], "gs", 1),   # the pools' mesh and smoother
    (0, [2, 5, 3, 4], "jac", 0),  # the batched Jacobi workload's kind
])
def test_batched_solutions_unchanged(G, kind, nrefs, sm, order):
    gens = [G.Generator(kind, n, seed=40 + k, corr=0.1, var=0.5) for k, n in enumerate(nrefs)]
    insts = [g.levels() for g in gens]
    rhs = [g.rhs for g in gens]
    _same(_solves(G, insts, rhs, sm, order, 0, defect=False, batched=True),
          _solves(G, insts, rhs, sm, order, 0, defect=True, batched=True))
