import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_names(kind="uniform"):
    """Fixture names: "uniform" (uniformly refined hierarchies, the surface is
    the top level), "local" (the ls_* cases, locally refined), "all" (both),
    or "imat" (the im_* cases: interpolation matrices on every fine level and
    UG's transfer in its matrix mode, uniform and local)."""
    names = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
    if kind == "imat":
        return [n for n in names if n.startswith("im_")]
    names = [n for n in names if not n.startswith("im_")]
    if kind == "all":
        return names
    return [n for n in names if n.startswith("ls_") == (kind == "local")]


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: (str(z[k]) if z[k].dtype.kind == "U" else z[k]) for k in z.files}


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


def permuted_levels(levels, mg):
    """The hierarchy as the device processes it (processing order of every
    level), as plain arrays for the oracle: rows, columns, transfer rows and
    transfer columns renumbered by mg.order(level)."""
    out = []
    inv_prev = None
    for l, d in enumerate(levels):
        perm = mg.order(l)
        inv = np.empty_like(perm)
        inv[perm] = np.arange(len(perm), dtype=perm.dtype)
        rp, col, val = mg.matrix(l)
        e = {"n": d["n"], "s": d["s"], "rowptr": rp, "col": col, "val": val,
             "vclass": np.asarray(d["vclass"])[perm], "vnclass": np.asarray(d["vnclass"])[perm],
             "skip": np.asarray(d["skip"])[perm]}
        if l > 0:
            prp, pcol, pw = np.asarray(d["prowptr"]), np.asarray(d["pcol"]), np.asarray(d["pw"])
            rows = [np.arange(prp[o], prp[o + 1]) for o in perm]
            newrp = np.concatenate([[0], np.cumsum([len(r) for r in rows])]).astype(np.int32)
            idx = np.concatenate(rows) if rows else np.zeros(0, int)
            e.update(prowptr=newrp, pcol=inv_prev[pcol[idx]].astype(np.int32), pw=pw[idx])
        out.append(e)
        inv_prev = inv
    return out


def rel(a, b):
    a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
