"""UG's ordering numprocs (np/procs/order.cc: order.bw, order.lex) on a
flattened hierarchy, host side.

The ``*bw*`` / ``*lex*`` fixtures are UG's own hierarchies after UG ran the
order numproc on every level (tests/golden/make_golden.py).  gmg_order_bw /
gmg_order_lex on the unordered fixture of the same case, applied with
permute_levels, give exactly UG's reordered hierarchy: rows, columns and
values of every level's matrix, the transfer weights, the vector classes,
the positions and the right-hand side.  The solves on the reordered fixtures
(UG's iteration counts in the new Gauss-Seidel / ILU order) are covered by
the generic oracle and device parity tests over every fixture.
"""
import numpy as np
import pytest

from conftest import load_golden

# ordered fixture: (unordered fixture of the same case, domain radius of the
# UG domain: unit square / cube 0.5, L-shape 1.0)
ORDERED = {"q1bw_gs": ("q1_gs", 0.5), "q1lex_ilu": ("q1_ilu", 0.5), "p1lex_gs": ("p1_gs", 0.5),
           "elbw_ilu": ("el_ilu", 0.5), "ls_bw_gs": ("ls_gs", 1.0)}
KEYS = ("rowptr", "col", "val", "vclass", "vnclass", "skip", "prowptr", "pcol", "pw")


@pytest.fixture(scope="module")
def G():
    import ug_gb300
    ug_gb300.lib()
    return ug_gb300


def _xyz(fx, l):
    return np.asarray(fx[f"L{l}_xyz"]).reshape(-1, 3)


def _perms(G, fx, order, radius):
    levels = G.levels_from_ugfx(fx)
    dim = int(fx["dim"][0])
    perms = []
    for l, lev in enumerate(levels):
        if order == "bw":
            p, bw = G.order_bw(lev)
            assert bw >= 0
        else:
            p = G.order_lex(lev, _xyz(fx, l)[:, :dim], order[4:], G.lex_inv_mesh_size(l, levels[0]["n"], dim, radius))
        assert np.array_equal(np.sort(p), np.arange(lev["n"]))
        perms.append(p)
    return levels, perms


@pytest.mark.parametrize("name", sorted(ORDERED))
def test_order_reproduces_ug(G, name):
    base_name, radius = ORDERED[name]
    fx, base = load_golden(name), load_golden(base_name)
    order = str(fx["order"])
    assert order != "none" and str(base.get("order", "none")) == "none"
    levels, perms = _perms(G, base, order, radius)
    got = G.permute_levels(levels, perms)
    want = G.levels_from_ugfx(fx)
    s = int(fx["blocksize"][0])
    for l, (a, b) in enumerate(zip(got, want)):
        for k in KEYS:
            if b.get(k) is not None:
                assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), (name, l, k)
        assert np.array_equal(_xyz(base, l)[perms[l]], _xyz(fx, l)), (name, l)
        for k in ("fine_grid_dof", "new_defect"):
            assert np.array_equal(np.asarray(base[f"L{l}_{k}"])[perms[l]], fx[f"L{l}_{k}"])
    assert np.array_equal(G.permute_vector(base["rhs"], perms[-1], s), fx["rhs"])
    offs = np.cumsum([0] + [lev["n"] * s for lev in levels])
    rhs_all = np.concatenate([G.permute_vector(base["rhs_all"][offs[l]:offs[l + 1]], perms[l], s)
                              for l in range(len(levels))])
    assert np.array_equal(rhs_all, fx["rhs_all"])


def test_order_bw_bandwidth(G):
    """The bandwidth order.bw reports (order.cc:400-411) on UG's reordered
    finest level: max |i - j| over its entries."""
    fx = load_golden("q1bw_gs")
    top = G.levels_from_ugfx(fx)[-1]
    rp, col = np.asarray(top["rowptr"]), np.asarray(top["col"])
    rows = np.repeat(np.arange(top["n"]), np.diff(rp))
    levels, perms = _perms(G, load_golden("q1_gs"), "bw", 0.5)
    _, bw = G.order_bw(levels[-1])
    assert bw == int(np.max(np.abs(rows - col)))


def test_order_errors(G):
    """order.bw on a matrix graph that is not connected fails (UG asserts);
    order.lex rejects configs that OrderLexInit rejects."""
    lev = {"n": 4, "s": 1, "rowptr": np.array([0, 2, 4, 6, 8]), "col": np.array([0, 1, 1, 0, 2, 3, 3, 2]),
           "val": np.ones(8), "vclass": np.full(4, 3), "vnclass": np.full(4, 3), "skip": np.zeros(4)}
    with pytest.raises(G.GmgError, match="not connected"):
        G.order_bw(lev)
    xyz = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0]])
    for bad in ("rx", "r", "ruf"):
        with pytest.raises(G.GmgError):
            G.order_lex(lev, xyz, bad, 1.0, dim=2)
    # 'ru': x ascending within rows of equal y (the last letter is the major key)
    assert G.order_lex(lev, xyz, "ru", 1.0).tolist() == [0, 1, 2, 3]
    assert G.order_lex(lev, xyz, "ur", 1.0).tolist() == [0, 2, 1, 3]
    assert G.order_lex(lev, xyz, "ld", 1.0).tolist() == [3, 2, 1, 0]


@pytest.mark.parametrize("name", ["q1_gs", "el_ilu", "ls_gs"])
def test_permute_levels_round_trip(G, name):
    """permute_levels by random permutations and then by their inverses gives
    the hierarchy back; the permuted level matrix is P A P^T and the permuted
    transfer is P_f T P_c^T (dense check on the small levels)."""
    levels = G.levels_from_ugfx(load_golden(name))
    rng = np.random.default_rng(3)
    perms = [rng.permutation(lev["n"]) for lev in levels]
    inv = [np.argsort(p) for p in perms]
    there = G.permute_levels(levels, perms)
    back = G.permute_levels(there, inv)
    for a, b in zip(back, levels):
        for k in KEYS:
            if b.get(k) is not None:
                assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k
    s = int(levels[0]["s"])

    def dense(rp, col, val, nr, nc, w):
        m = np.zeros((nr * w, nc * w))
        v = np.asarray(val).reshape(-1, w, w)
        for i in range(nr):
            for e in range(rp[i], rp[i + 1]):
                m[i * w:(i + 1) * w, col[e] * w:(col[e] + 1) * w] += v[e]
        return m

    def blockperm(p, w):
        return (np.asarray(p)[:, None] * w + np.arange(w)[None, :]).ravel()

    for l in range(min(3, len(levels))):
        a, t = levels[l], there[l]
        A = dense(a["rowptr"], a["col"], a["val"], a["n"], a["n"], s)
        At = dense(t["rowptr"], t["col"], t["val"], t["n"], t["n"], s)
        q = blockperm(perms[l], s)
        assert np.array_equal(At, A[np.ix_(q, q)])
        if l > 0:
            nc = levels[l - 1]["n"]
            T = dense(a["prowptr"], a["pcol"], a["pw"], a["n"], nc, 1)
            Tt = dense(t["prowptr"], t["pcol"], t["pw"], t["n"], nc, 1)
            assert np.array_equal(Tt, T[np.ix_(perms[l], perms[l - 1])])


@pytest.mark.parametrize("config", ["ru", "ur", "ld", "dl", "ruf", "bdl", "fru", "lub"])
def test_order_lex_is_a_lexicographic_sort(G, config):
    """On a lattice (distinct positions, spacing far above the 1e-3 tolerance)
    order.lex is numpy's lexicographic sort with the last config letter as
    the major key and each letter's direction."""
    dim = len(config)
    rng = np.random.default_rng(len(config) + ord(config[0]))
    side = 5
    pts = np.stack(np.meshgrid(*[np.arange(side)] * dim, indexing="ij"), -1).reshape(-1, dim).astype(float)
    pts = pts[rng.permutation(len(pts))] * 0.25
    n = len(pts)
    lev = {"n": n, "s": 1, "rowptr": np.arange(n + 1), "col": np.arange(n), "val": np.ones(n),
           "vclass": np.full(n, 3), "vnclass": np.full(n, 3), "skip": np.zeros(n)}
    axis = {"r": (0, 1), "l": (0, -1), "u": (1, 1), "d": (1, -1), "f": (2, 1), "b": (2, -1)}
    keys = [axis[c][1] * pts[:, axis[c][0]] for c in config]  # np.lexsort: last key is the primary one
    want = np.lexsort(keys)
    got = G.order_lex(lev, pts, config, 1.0)
    assert got.tolist() == want.tolist()


@pytest.mark.parametrize("name", ["q1_gs", "p1_gs", "el_ilu"])
def test_order_bw_is_breadth_first(G, name):
    """order.bw's order is a breadth-first order of the matrix graph: graph
    distances from its first vector never decrease along it, and its first
    vector is the one a breadth-first sweep from the level's first vector
    reaches last."""
    for lev in G.levels_from_ugfx(load_golden(name)):
        n = lev["n"]
        rp, col = np.asarray(lev["rowptr"]), np.asarray(lev["col"])
        perm, _ = G.order_bw(lev)

        def bfs(src):
            dist = np.full(n, -1)
            dist[src] = 0
            q, h = [src], 0
            while h < len(q):
                v = q[h]; h += 1
                for w in col[rp[v]:rp[v + 1]]:
                    if dist[w] < 0:
                        dist[w] = dist[v] + 1
                        q.append(w)
            return dist, q

        _, first_sweep = bfs(0)
        assert perm[0] == first_sweep[-1]
        dist, _ = bfs(perm[0])
        assert np.all(np.diff(dist[perm]) >= 0)


@pytest.mark.parametrize("name", sorted(ORDERED))
def test_order_levels_reproduces_ug(G, name):
    """order_levels (UG's `npexecute ord $a`) with the default radius (half
    the extent of level 0) gives UG's reordered hierarchy."""
    base_name, _ = ORDERED[name]
    fx, base = load_golden(name), load_golden(base_name)
    levels = G.levels_from_ugfx(base)
    xyz = [_xyz(base, l) for l in range(len(levels))]
    got, perms = G.order_levels(levels, str(fx["order"]), xyz=xyz)
    for a, b in zip(got, G.levels_from_ugfx(fx)):
        for k in KEYS:
            if b.get(k) is not None:
                assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), (name, k)
    with pytest.raises(G.GmgError):
        G.order_levels(levels, "so")
