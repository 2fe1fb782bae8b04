"""gmg_nrm2x_static, the allocation-free variant of the defect-norm kernel.

Some callers of this library cannot let it call cudaMalloc: a host framework
whose memory manager owns all device memory (UG keeps all of its data on its
own heap) hands the solver device buffers and nothing else, and a process
that has spent its device-memory budget cannot grow it.  For them the norm
kernel's scratch lives in a fixed device array inside the library.  This test
calls that entry point through the C ABI on buffers the caller owns and
compares it with the library's ordinary entry point (gmg_dnrm2x, which uses
the multigrid's allocated scratch) on two calls in a row, for one and two
components per row, and with numpy for three and eight; it also checks that
a size beyond the fixed scratch is rejected with an error instead of being
run.

Collected last (file name) so that a run stopping at the first failure has
already run every other test; it passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_static_scratch_norms_match_dnrm2x():
    import torch

    import ug_gb300 as G

    lib = G.lib()
    f = lib.gmg_nrm2x_static
    f.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    rng = np.random.default_rng(11)
    for kind, nref in [(G.Generator.POISSON2D, 6), (G.Generator.ELASTICITY2D, 5)]:
        gen = G.Generator(kind, nref, seed=7)
        mg = G.MultiGrid(gen)
        n, s, _ = mg.size(mg.top)
        mg.createvector("v")
        for _call in range(2):  # two calls in a row share the static scratch
            x = rng.uniform(-1.0, 1.0, n * s)
            mg.upload("v", mg.top, x)
            ref = mg.dnrm2x(mg.top, "v")
            xd = torch.tensor(x, dtype=torch.float64, device="cuda")
            out = torch.full((s,), -1.0, dtype=torch.float64, device="cuda")
            stream = torch.cuda.current_stream().cuda_stream
            rc = f(xd.data_ptr(), n, s, out.data_ptr(), C.c_void_p(stream))
            assert rc == 0, lib.gmg_last_error()
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert np.allclose(got, ref, rtol=1e-12, atol=0.0), (got, ref)
            assert np.allclose(got, np.sqrt((x.reshape(-1, s) ** 2).sum(axis=0)), rtol=1e-12, atol=0.0)
        mg.close()
    # three and eight components per row (the largest the scratch holds) on
    # synthetic device data, two calls in a row each
    for s in (3, 8):
        n = 40_000 + s
        for _call in range(2):
            x = rng.uniform(-1.0, 1.0, n * s)
            xd = torch.tensor(x, dtype=torch.float64, device="cuda")
            out = torch.full((s,), -1.0, dtype=torch.float64, device="cuda")
            rc = f(xd.data_ptr(), n, s, out.data_ptr(), C.c_void_p(torch.cuda.current_stream().cuda_stream))
            assert rc == 0, lib.gmg_last_error()
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert np.allclose(got, np.sqrt((x.reshape(-1, s) ** 2).sum(axis=0)), rtol=1e-12, atol=0.0), (s, got)
    # more components than the fixed scratch holds: rejected, nothing launched
    out = torch.zeros(16, dtype=torch.float64, device="cuda")
    xd = torch.zeros(16 * 9, dtype=torch.float64, device="cuda")
    rc = f(xd.data_ptr(), 16, G.MAX_S + 1, out.data_ptr(), None)
    assert rc != 0
    assert b"at most" in lib.gmg_last_error()
