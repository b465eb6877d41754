"""The allocation-free dense operator, edfmm_dense_matvec_noalloc.

It exists for callers that cannot allocate device memory while applying the
operator (an application whose framework allocator already holds the GPU's
free memory, or a binding without a CUDA allocator).  Its partial sums live
in a fixed 8 MiB device array shared by all calls, so this test calls it
twice in a row through the C ABI and compares both results with the
allocating entry point, edfmm_dense_matvec, at the tolerance the dense tests
use (FP64 1e-12, FP32 2e-6 relative L2).  It is collected last so that a run
that stops at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

K_E = 1.0 / (4.0 * np.pi * 8.854187817e-12)


def _call(lib, fn, c, s, a, si, out, dtype_code):
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    vp = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    return getattr(lib, fn)(vp(c), vp(s), vp(a), vp(si), s.shape[0], dtype_code, K_E, vp(out), stream)


@pytest.mark.parametrize("dt,tol,sizes", [(torch.float64, 1e-12, (5120, 40000, 262144)),
                                           (torch.float32, 2e-6, (5120, 40000))])
def test_noalloc_matches_allocating_entry_point_twice(cuda_lib, dt, tol, sizes):
    # 262144 is the entry point's limit, where its FP64 partial sums take the
    # largest share of the fixed array
    from electrodrive_gb300 import _lib

    code = _lib.dtype_code(dt)
    for n, seed in zip(sizes, (1, 2, 3)):
        g = torch.Generator().manual_seed(seed)
        c = torch.rand(n, 3, generator=g, dtype=torch.float64).to("cuda", dt)
        a = (0.5 + torch.rand(n, generator=g, dtype=torch.float64)).to("cuda", dt) / n
        si = torch.rand(n, generator=g, dtype=torch.float64).to("cuda", dt) * 1e3
        ref = torch.empty(n, dtype=dt, device="cuda")
        got = [torch.empty(n, dtype=dt, device="cuda") for _ in range(2)]
        sig = [(2 * torch.rand(n, generator=g, dtype=torch.float64) - 1).to("cuda", dt) for _ in range(2)]
        for k in range(2):
            assert _call(cuda_lib, "edfmm_dense_matvec_noalloc", c, sig[k], a, si, got[k], code) == 0
        torch.cuda.synchronize()
        for k in range(2):
            assert _call(cuda_lib, "edfmm_dense_matvec", c, sig[k], a, si, ref, code) == 0
            torch.cuda.synchronize()
            r = ref.double().cpu().numpy()
            err = np.linalg.norm(got[k].double().cpu().numpy() - r) / np.linalg.norm(r)
            assert err < tol, (n, k, err)


def test_noalloc_rejects_sizes_above_its_limit(cuda_lib):
    from electrodrive_gb300 import _lib

    n = 262145
    x = torch.zeros(1, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = ctypes.c_void_p(x.data_ptr())
    rc = cuda_lib.edfmm_dense_matvec_noalloc(p, p, p, None, n, _lib.EDFMM_F32, 1.0, p, stream)
    assert rc == _lib.EDFMM_ERR_ARG
    assert b"262144" in cuda_lib.edfmm_last_error()
