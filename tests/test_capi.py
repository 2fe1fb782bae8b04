"""The C ABI library builds, loads without a GPU and exports every entry point
include/ug_gb300.h declares; the numproc argument conventions and error
reporting work without touching the device."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    with open(os.path.join(ROOT, "include", "ug_gb300.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gmg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    import ug_gb300
    lib = ug_gb300.lib()
    names = declared_functions()
    assert len(names) >= 50
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_no_device_reports_error_instead_of_aborting():
    import ug_gb300
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    gen = ug_gb300.Generator(0, 2)
    with pytest.raises(ug_gb300.GmgError):
        ug_gb300.MultiGrid(gen)


def test_generator_sizes():
    import ug_gb300
    g = ug_gb300.Generator(1, 2, seed=3, var=1.0)
    sizes = [g.level(l)["n"] for l in range(g.nlevels)]
    assert sizes == [8, 27, 125]
    top = g.level(2)
    assert top["rowptr"][0] == 0 and all(top["col"][top["rowptr"][i]] == i for i in range(top["n"]))
    # boundary rows are unit rows
    for i in range(top["n"]):
        if top["skip"][i]:
            k0, k1 = top["rowptr"][i], top["rowptr"][i + 1]
            assert top["val"][k0] == 1.0 and not top["val"][k0 + 1:k1].any()


def test_python_binding_declares_every_entry_point():
    """The ctypes front end (ug_gb300/__init__.py) gives every entry point of
    include/ug_gb300.h its argument and result types (a missing declaration
    makes ctypes pass doubles as ints); gmg_nrm2x_static, which takes raw
    device pointers, is declared by its caller."""
    import re
    hdr = open(os.path.join(ROOT, "include", "ug_gb300.h")).read()
    src = open(os.path.join(ROOT, "ug_gb300", "__init__.py")).read()
    names = set(re.findall(r"\b(gmg_\w+)\s*\(", hdr)) - {"gmg_nrm2x_static"}
    assert sorted(n for n in names if f'"{n}"' not in src) == []
