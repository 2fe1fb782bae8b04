"""The UG-side binding (ug_gb300/ug_glue/gpu_numprocs.cc) compiled into UG
3.12.1 itself: oracle/Makefile builds it against UG's headers, links it with
UG's library and libug_gb300 (oracle/_ref/ug_glue_test2d, part of the
reference build), and that program runs UG's own script commands on a 2D
hierarchy.  Checked here, on a host without a GPU: the classes register
with CreateClass, `npcreate mgs $c gls` / `npinit ...` resolve to the
forwarding classes (the objects are UG numprocs of those classes, status
EXECUTABLE), the flattener walks UG's VECTOR / MATRIX lists and transfer
weights as the device expects them, and a solve without a CUDA device fails
through UG's numproc error path (NP_RETURN, `npexecute` reports the failing
PreProcess) with the library's message instead of aborting."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "oracle", "_ref", "ug_glue_test2d")


@pytest.mark.skipif(not os.path.exists(EXE), reason="the UG reference build (make -C oracle ref REF=...) is absent")
def test_glue_in_ug_without_device():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([EXE], capture_output=True, text=True, timeout=300, env=env)
    out = r.stdout + r.stderr
    checks = [l for l in out.splitlines() if l.startswith(("ok ", "FAIL "))]
    assert r.returncode == 0 and len(checks) == 8 and all(c.startswith("ok ") for c in checks), out[-3000:]
    assert "class linear_solver.gls (GB300)" in out
    assert "gpu numprocs: gmg_mg_create:" in out and "PreProcess failed" in out
