"""UG's transfer in its matrix mode (`npinit transfer $M`, transfer.cc:564):
RestrictByMatrix and InterpolateCorrectionByMatrix (np/algebra/transgrid.cc:
1113, 1292) with the interpolation matrices (IMATRIX) UG stored on every fine
level (tests/golden/im_*.npz: the standard weights times seeded blocks near
the identity, uniform and locally refined hierarchies).

* kernels: UG's known-answer vectors, plain and damped, in every processing
  order, to 1e-12;
* solves: list order takes UG's iterations and reaches UG's solution (jac
  1e-10; gs / ilu 1e-8 and iterations +-1, the contract's bounds; the local
  case, which UG runs to its 100-iteration limit without converging, the
  same iterations and solution to 1e-8);
* the FP32 V-cycle in FP64 refinement with the matrix-mode transfer meets the
  FP64 stopping test;
* InterpolateNewVectors in the matrix mode (InterpolateNewVectorsByMatrix,
  transgrid.cc:1425) over every level: UG's values bit for bit;
* errors: the matrix mode without interpolation matrices, and $R (not
  implemented) leaving the numproc not active."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, rel

pytestmark = pytest.mark.gpu
IMAT = golden_names("imat")


@pytest.fixture(scope="module")
def G():
    import ug_gb300
    ug_gb300.lib()
    return ug_gb300


def _mg(G, fx, order=0, fp32=False):
    mg = G.MultiGrid(G.levels_from_ugfx(fx), order=order, fp32=fp32)
    for l, m in enumerate(G.imatrices_from_ugfx(fx)):
        if m is not None:
            mg.set_imatrix(l, *m)
    return mg


@pytest.mark.parametrize("order", [0, 1, 2])
@pytest.mark.parametrize("name", IMAT)
def test_matrix_transfer_kernels_match_ug(G, name, order):
    fx = load_golden(name)
    mg = _mg(G, fx, order)
    top = mg.top
    dm = [0.7 - 0.1 * i for i in range(8)]
    mg.createvector("c", "d", "t")
    mg.upload("d", top, fx["kat_d"])
    for pre, out, damp in (("kat_mrestrict_pre", "kat_mrestrict", None),
                           ("kat_mrestrict_damp_pre", "kat_mrestrict_damp", dm)):
        mg.upload("c", top - 1, fx[pre])
        mg.restrict_by_matrix(top, "c", "d", damp)
        assert rel(mg.download("c", top - 1), fx[out]) <= 1e-12, out
    mg.upload("c", top - 1, fx["kat_minterp_coarse"])
    for out, damp in (("kat_minterp", None), ("kat_minterp_damp", dm)):
        mg.upload("t", top, np.full(fx["kat_d"].size, 7.0))
        mg.interpolate_correction_by_matrix(top, "t", "c", damp)
        assert rel(mg.download("t", top), fx[out]) <= 1e-12, out
    mg.close()


@pytest.mark.parametrize("fuse", [0, None])
@pytest.mark.parametrize("name", IMAT)
def test_matrix_transfer_solve_matches_ug(G, name, fuse):
    fx = load_golden(name)
    mg = _mg(G, fx)
    sm = str(fx["smoother"])
    G.setup_lmgc(mg, sm, baselevel=int(fx["baselevel"][0]), damp=0.8 if sm == "jac" else 1.0, red=1e-10,
                 abslimit=1e-50, fuse=fuse, transfer="$M")
    assert "RestrictByMatrix" in mg.npdisplay("transfer")
    local = mg.local
    x, lr = mg.solve_host("mgs", fx["rhs_all"] if local else fx["rhs"])
    xu = fx["ls_x_all"] if local else fx["ls_x"]
    it_ug, conv_ug = int(fx["ls_iters"][0]), bool(fx["ls_converged"][0])
    assert lr.converged == conv_ug
    assert abs(lr.first_defect[0] - fx["ls_hist"][0]) <= 1e-12 * fx["ls_hist"][0]
    if sm == "jac" or not conv_ug:
        assert lr.iters == it_ug
        assert rel(x, xu) <= (1e-10 if sm == "jac" else 1e-8)
    else:
        assert abs(lr.iters - it_ug) <= 1
        assert rel(x, xu) <= 1e-8
    mg.close()


@pytest.mark.parametrize("name", ["im_q1_gs", "im_el_ilu", "im_p1k_jac"])
def test_matrix_transfer_mixed_precision(G, oracle_mod, name):
    fx = load_golden(name)
    mg = _mg(G, fx, order=1, fp32=True)
    sm = str(fx["smoother"])
    G.setup_lmgc(mg, sm, baselevel=int(fx["baselevel"][0]), damp=0.8 if sm == "jac" else 1.0, red=1e-8,
                 abslimit=1e-50, mixed=True, transfer="$M")
    x, lr = mg.solve_host("mgs", fx["rhs"])
    assert lr.converged
    H = oracle_mod.Hierarchy.from_ugfx(fx)
    top = len(H.levels) - 1
    d = H.matmul_minus(top, fx["rhs"], x)
    assert np.all(H.nrm2x(top, d) <= 1.0000001e-8 * H.nrm2x(top, fx["rhs"]))
    mg.close()


@pytest.mark.parametrize("order", [0, 1, 2])
@pytest.mark.parametrize("name", IMAT)
def test_matrix_mode_new_vectors_match_ug(G, name, order):
    fx = load_golden(name)
    mg = _mg(G, fx, order=order)
    mg.createvector("x")
    mg.npcreate("tr", "transfer.gtransfer")
    mg.npinit("tr", "$M")
    n = mg.nlevels
    offs = np.cumsum([0] + mg.level_len)
    for l in range(n):
        mg.set_new_vectors(l, fx[f"L{l}_vnew"])
        mg.upload("x", l, fx["kat_newvec_pre"][offs[l]:offs[l + 1]])
    mg.transfer_interpolate_new_vectors("tr", 0, n - 1, "x")
    got = np.concatenate([mg.download("x", l) for l in range(n)])
    assert np.array_equal(got, fx["kat_newvec"])
    mg.close()


def test_matrix_transfer_errors(G):
    fx = load_golden("im_q1_gs")
    mg = G.MultiGrid(G.levels_from_ugfx(fx))  # no interpolation matrices set
    mg.createvector("c", "d")
    with pytest.raises(G.GmgError, match="interpolation matrix"):
        mg.restrict_by_matrix(mg.top, "c", "d")
    mg.npcreate("tr", "transfer.gtransfer")
    assert mg.npinit("tr", "$M $R") == G.NP_NOT_ACTIVE  # Init rejects $R (RestrictByMatrix_s)
    assert b"$R" in G.lib().gmg_last_error()
    mg.close()
