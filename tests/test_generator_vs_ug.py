"""The structured hierarchy generator (ug_gb300/csrc/meshgen.cpp) builds, without
UG, the same hierarchies UG's grid manager builds for the workloads: every
level's matrix, VECSKIP mask, standard-transfer weights and the right-hand
side agree with the UG-exported golden fixtures once vectors are matched by
their coordinates (UG numbers them in refinement order, the generator
lexicographically).  Runs on the CPU: the generator needs no GPU.

In 3D, kind 3 is UG's own hierarchy and matches on every level: UG's red
rule for tetrahedra picks the octahedron's shortest interior diagonal and
breaks the tie between the two equally short ones of a Kuhn tetrahedron by
its local edge numbering (ShortestInteriorEdge, gm/rm.cc:1567), which kind 3
follows through the sons' corner orders of UG's rule table.  Kind 1 always
takes the diagonal that keeps the Freudenthal triangulation: it matches on
the coarse grid and in the level sizes (unknowns, nonzeros) of every level
(both are red refinements with the same vertices and edge counts)."""
import numpy as np
import pytest

from conftest import load_golden

CASES = [  # fixture, generator kind, nref, seed, corr, var
    ("q1_jac", 0, 5, 11, 0.1, 0.0),
    ("p1_gs", 1, 3, 12, 0.1, 0.0),
    ("p1k_jac", 1, 3, 13, 0.1, 1.0),
    ("p1_gs", 3, 3, 12, 0.1, 0.0),
    ("p1k_jac", 3, 3, 13, 0.1, 1.0),
    ("el_jac", 2, 4, 14, 0.1, 0.0),
]


def _keys(xyz, scale):
    return [tuple(int(round(c * scale)) for c in p) for p in np.asarray(xyz).reshape(-1, 3)]


class _OracleCube:
    """The oracle's generator (oracle/cube_gen.c) behind the Generator
    interface the checks below read."""

    def __init__(self, oracle_mod, nref, seed, corr, var):
        self._lv, self.rhs, xyz = oracle_mod.cube_levels(nref, seed, corr, var, threads=2, ug_rules=True)
        for d, x in zip(self._lv, xyz):
            d["xyz"] = x
        self.nlevels = len(self._lv)

    def level(self, l):
        return self._lv[l]


@pytest.mark.parametrize("name,kind,nref,seed,corr,var", CASES)
def test_generator_matches_ug(name, kind, nref, seed, corr, var):
    import ug_gb300 as G
    _check_against_ug(name, G.Generator(kind, nref, seed=seed, corr=corr, var=var), kind, nref)


@pytest.mark.parametrize("name,nref,seed,corr,var", [c[:1] + c[2:] for c in CASES if c[1] == 3])
def test_oracle_ug_rules_match_ug(oracle_mod, name, nref, seed, corr, var):
    """The oracle's restatement of UG's red refinement, pinned on its own
    against UG's exported 3D hierarchies (every level, pattern, values,
    transfer, right-hand side)."""
    _check_against_ug(name, _OracleCube(oracle_mod, nref, seed, corr, var), 3, nref)


def _check_against_ug(name, gen, kind, nref):
    fx = load_golden(name)
    assert gen.nlevels == int(fx["nlevels"][0])
    s = int(fx["blocksize"][0])
    scale = 1 << nref
    maps = []
    for l in range(gen.nlevels):
        g = gen.level(l)
        n = int(fx[f"L{l}_n"][0])
        assert g["n"] == n
        assert g["rowptr"][-1] == fx[f"L{l}_rowptr"][-1]
        assert np.array_equal(np.unique(g["vnclass"]), np.unique(fx[f"L{l}_vnclass"]))
        if kind == 1 and l > 0:
            maps.append(None)
            continue
        ug_keys = _keys(fx[f"L{l}_xyz"], scale)
        gk = {k: i for i, k in enumerate(_keys(g["xyz"], scale))}
        m = np.array([gk[k] for k in ug_keys])  # ug index -> generator index
        maps.append(m)
        assert np.array_equal(g["skip"][m], fx[f"L{l}_skip"])
        assert np.array_equal(g["vclass"][m], fx[f"L{l}_vclass"])
        # matrices, entry by entry
        rp, col, val = fx[f"L{l}_rowptr"], fx[f"L{l}_col"], fx[f"L{l}_val"].reshape(-1, s * s)
        gval = g["val"].reshape(-1, s * s)
        vmax = np.abs(val).max()
        for i in range(n):
            gi = m[i]
            gents = {int(g["col"][k]): gval[k] for k in range(g["rowptr"][gi], g["rowptr"][gi + 1])}
            assert g["col"][g["rowptr"][gi]] == gi  # diagonal first
            uents = {int(m[col[k]]): val[k] for k in range(rp[i], rp[i + 1])}
            assert set(gents) == set(uents), f"level {l} row {i}: pattern differs"
            for c, v in uents.items():
                assert np.allclose(gents[c], v, rtol=0, atol=1e-13 * vmax), f"level {l} row {i}"
        if l == 0:
            continue
        prp, pcol, pw = fx[f"P{l}_rowptr"], fx[f"P{l}_col"], fx[f"P{l}_w"]
        mc = maps[l - 1]
        for i in range(n):
            gi = m[i]
            ge = {int(g["pcol"][k]): g["pw"][k] for k in range(g["prowptr"][gi], g["prowptr"][gi + 1])}
            ue = {int(mc[pcol[k]]): pw[k] for k in range(prp[i], prp[i + 1])}
            assert ge.keys() == ue.keys() and all(abs(ge[k] - ue[k]) < 1e-15 for k in ue)
    top = gen.nlevels - 1
    if maps[top] is None:
        gk = {k: i for i, k in enumerate(_keys(gen.level(top)["xyz"], scale))}
        maps[top] = np.array([gk[k] for k in _keys(fx[f"L{top}_xyz"], scale)])
    rhs_g = gen.rhs.reshape(-1, s)[maps[top]].ravel()
    assert np.allclose(rhs_g, fx["rhs"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("name,nuni,nloc,seed", [("ls_gs", 2, 6, 22)])
def test_local_generator_matches_ug(name, nuni, nloc, seed):
    """The locally refined L-shape hierarchy (meshgen_local.cpp) is UG's:
    after matching vectors by coordinates, every level has UG's vectors,
    matrix (pattern and values), VCLASS / VNCLASS / VECSKIP, transfer weights
    and right-hand side."""
    import ug_gb300 as G
    fx = load_golden(name)
    gen = G.LocalGenerator(nuni, nloc, seed=seed)
    assert gen.nlevels == int(fx["nlevels"][0])
    s = int(fx["blocksize"][0])
    scale = 1 << (gen.nlevels - 1)
    offs_g = np.cumsum([0] + [gen.level(l)["n"] * s for l in range(gen.nlevels)])
    offs_u = np.cumsum([0] + [int(fx[f"L{l}_n"][0]) * s for l in range(gen.nlevels)])
    maps = []
    for l in range(gen.nlevels):
        g = gen.level(l)
        n = int(fx[f"L{l}_n"][0])
        assert g["n"] == n and g["rowptr"][-1] == fx[f"L{l}_rowptr"][-1]
        gk = {k: i for i, k in enumerate(_keys(g["xyz"], scale))}
        m = np.array([gk[k] for k in _keys(fx[f"L{l}_xyz"], scale)])
        maps.append(m)
        for f in ("skip", "vclass", "vnclass"):
            assert np.array_equal(g[f][m], fx[f"L{l}_{f}"]), (l, f)
        rp, col, val = fx[f"L{l}_rowptr"], fx[f"L{l}_col"], fx[f"L{l}_val"].reshape(-1, s * s)
        gval = g["val"].reshape(-1, s * s)
        vmax = np.abs(val).max()
        for i in range(n):
            gi = m[i]
            gents = {int(g["col"][k]): gval[k] for k in range(g["rowptr"][gi], g["rowptr"][gi + 1])}
            uents = {int(m[col[k]]): val[k] for k in range(rp[i], rp[i + 1])}
            assert set(gents) == set(uents), f"level {l} row {i}: pattern differs"
            for c, v in uents.items():
                assert np.allclose(gents[c], v, rtol=0, atol=1e-13 * vmax), f"level {l} row {i}"
        rg = gen.rhs[offs_g[l]:offs_g[l + 1]].reshape(-1, s)[m].ravel()
        assert np.allclose(rg, fx["rhs_all"][offs_u[l]:offs_u[l + 1]], rtol=0, atol=1e-15), l
        if l == 0:
            continue
        prp, pcol, pw = fx[f"P{l}_rowptr"], fx[f"P{l}_col"], fx[f"P{l}_w"]
        mc = maps[l - 1]
        for i in range(n):
            gi = m[i]
            ge = {int(g["pcol"][k]): g["pw"][k] for k in range(g["prowptr"][gi], g["prowptr"][gi + 1])}
            ue = {int(mc[pcol[k]]): pw[k] for k in range(prp[i], prp[i + 1])}
            assert ge.keys() == ue.keys() and all(abs(ge[k] - ue[k]) < 1e-15 for k in ue)
