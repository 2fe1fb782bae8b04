"""The colouring of the multicolour order (gmg_colour_graph, ug_gb300/csrc/
gmg_mg.cpp: DSATUR, then a bounded tabu search for fewer colours), on the
host: every colour class is an independent set of the symmetrised matrix
graph, the result does not depend on the call (fixed seed), and the colour
counts of the cube meshes are the ones the multicolour Gauss-Seidel waves
are built from: 4 on every level of the Freudenthal triangulation (its
clique number, so no search runs), and 4, 5, 6, 6, 7, 8 on levels 0..5 of
UG's red refinement (8 on the 65^3 level, where DSATUR alone needs 9)."""
import numpy as np
import pytest


def _proper(rowptr, col, colour):
    rows = np.repeat(np.arange(len(rowptr) - 1), np.diff(rowptr))
    off = rows != col
    return not np.any(colour[rows[off]] == colour[col[off]])


@pytest.mark.parametrize("kind,expect", [(1, [4, 4, 4, 4, 4, 4]), (3, [4, 5, 6, 6, 7, 8])])
def test_cube_colourings(kind, expect):
    import ug_gb300 as G
    gen = G.Generator(kind, 5, seed=3, corr=0.1, var=1.0)
    got = []
    for l in range(gen.nlevels):
        d = gen.level(l)
        colour, nc = G.colour_graph(d["rowptr"], d["col"])
        assert colour.min() == 0 and colour.max() == nc - 1
        assert len(np.unique(colour)) == nc
        assert _proper(d["rowptr"], d["col"], colour)
        got.append(nc)
    assert got == expect


def test_colouring_is_deterministic():
    import ug_gb300 as G
    d = G.Generator(3, 4, seed=3).level(4)
    a, na = G.colour_graph(d["rowptr"], d["col"])
    b, nb = G.colour_graph(d["rowptr"], d["col"])
    assert na == nb and np.array_equal(a, b)


def test_colouring_rejects_bad_columns():
    import ug_gb300 as G
    with pytest.raises(G.GmgError, match="out of range"):
        G.colour_graph(np.array([0, 1, 2]), np.array([0, 5]))
