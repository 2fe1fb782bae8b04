"""ILU(0) decomposition on the device (ug_gb300/csrc/gmg_ilu.cu) against UG's
l_ilubthdecomp (np/algebra/ugiter.cc:2252-2625): the factors UG left in its
copy of the finest-level matrix (golden `kat_ilu_factors`, UG's list order)
and the oracle's restatement on the reordered hierarchies (multicolour and
subdomain orders), entry by entry to 1e-14 of the largest factor entry; the
beta modification against the oracle; and new values on a resident
hierarchy (gmg_mg_update_values) re-factored on the device give the factors
of a hierarchy created with those values, bit for bit."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, permuted_levels

pytestmark = pytest.mark.gpu

NAMES = golden_names("all")


@pytest.fixture(scope="module")
def G():
    import ug_gb300
    ug_gb300.lib()
    return ug_gb300


def _blocks(rowptr, col, val, s, perm=None):
    """{(row, col): block} of a block-CSR matrix, rows / columns mapped through perm."""
    v = np.asarray(val).reshape(-1, s * s)
    out = {}
    for i in range(len(rowptr) - 1):
        r = i if perm is None else int(perm[i])
        for k in range(rowptr[i], rowptr[i + 1]):
            c = int(col[k]) if perm is None else int(perm[col[k]])
            out[(r, c)] = v[k]
    return out


def _close(a, b, tol=1e-14):
    assert a.keys() == b.keys()
    scale = max(np.abs(x).max() for x in b.values())
    worst = max(np.abs(a[k] - b[k]).max() for k in b)
    assert worst <= tol * scale, worst / scale


@pytest.mark.parametrize("name", NAMES)
def test_factors_match_ug(G, name):
    fx = load_golden(name)
    mg = G.MultiGrid(G.levels_from_ugfx(fx), order=G.ORDER_LIST)
    top = mg.top
    s = int(fx["blocksize"][0])
    mg.l_ilu_decomp(top)
    rp, col, _ = mg.matrix(top)
    got = _blocks(rp, col, mg.l_ilu_factors(top), s, mg.order(top))
    ref = _blocks(fx[f"L{top}_rowptr"], fx[f"L{top}_col"], fx["kat_ilu_factors"], s)
    _close(got, ref)
    mg.close()


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("name", NAMES)
def test_factors_match_oracle_reordered(G, oracle_mod, name, order):
    fx = load_golden(name)
    levels = G.levels_from_ugfx(fx)
    mg = G.MultiGrid(levels, order=order)
    H = oracle_mod.Hierarchy(permuted_levels(levels, mg))
    s = int(fx["blocksize"][0])
    for l in range(mg.nlevels):
        if mg.size(l)[0] < 2:
            continue
        mg.l_ilu_decomp(l)
        rp, col, _ = mg.matrix(l)
        _close(_blocks(rp, col, mg.l_ilu_factors(l), s), _blocks(rp, col, H.ilu_decomp(l), s))
    mg.close()


@pytest.mark.parametrize("name", ["q1_ilu", "el_ilu", "p1k_ilu"])
def test_beta_modification(G, oracle_mod, name):
    fx = load_golden(name)
    levels = G.levels_from_ugfx(fx)
    mg = G.MultiGrid(levels, order=G.ORDER_COLOR)
    H = oracle_mod.Hierarchy(permuted_levels(levels, mg))
    s = int(fx["blocksize"][0])
    top = mg.top
    beta = [0.5, 0.25][:s] if s > 1 else [0.5]
    mg.l_ilu_decomp(top, beta=beta)
    rp, col, _ = mg.matrix(top)
    _close(_blocks(rp, col, mg.l_ilu_factors(top), s), _blocks(rp, col, H.ilu_decomp(top, beta=beta), s))
    mg.close()


def test_update_values_refactors_on_device(G):
    """A Poisson hierarchy whose values are replaced by the diffusion problem's
    has, after the device re-factorisation, exactly the factors of a hierarchy
    created from the diffusion problem (subdomain order, every level)."""
    poisson = G.Generator(1, 4, seed=3, corr=0.1, var=0.0)
    diff = G.Generator(1, 4, seed=3, corr=0.1, var=1.0)
    a = G.MultiGrid(poisson.levels(), order=G.ORDER_DOMAIN)
    b = G.MultiGrid(diff.levels(), order=G.ORDER_DOMAIN)
    for mg in (a, b):
        G.setup_lmgc(mg, "ilu", baselevel=0, red=1e-8)
        mg.createvector("x0", "b0")
        mg.ls_preprocess("mgs", mg.top, "sol", "rhs")
    for l in range(a.nlevels):
        a.update_values(l, diff.level(l)["val"])
    for l in range(1, a.nlevels):
        assert np.array_equal(a.l_ilu_factors(l), b.l_ilu_factors(l)), l
    xa, la = a.solve_host("mgs", diff.rhs)
    xb, lb = b.solve_host("mgs", diff.rhs)
    assert la.iters == lb.iters and np.array_equal(xa, xb)
    a.close()
    b.close()
