"""Dense single-layer operator (edfmm_dense_matvec) against the oracle's
restatement of bem_kernel.py:157-230 and the reference's own outputs.
Tolerances: FP64 1e-12 relative L2, FP32 2e-6."""
import glob
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

K_E = 1.0 / (4.0 * np.pi * 8.854187817e-12)


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n", [1, 7, 256, 257, 5120, 20000, 70001])
@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_dense_matches_oracle(cuda_lib, oracle, n, dt):
    from electrodrive_gb300 import _lib

    rng = np.random.default_rng(n)
    c = rng.random((n, 3))
    s = rng.uniform(-1, 1, n)
    a = rng.uniform(0.5, 1.5, n) / n
    si = rng.uniform(0, 1e3, n)
    ref = oracle.dense_matvec(c.astype(np.float64 if dt == torch.float64 else np.float32), s, a, si)
    T = lambda x: torch.as_tensor(x, dtype=dt, device="cuda").contiguous()
    v = _lib.dense_matvec(T(c), T(s), T(a), T(si), k_e=K_E).cpu().numpy()
    tol = 1e-12 if dt == torch.float64 else 2e-6
    if n == 1:
        assert abs(v[0] - si[0] * s[0] * a[0]) <= tol * abs(si[0] * s[0] * a[0])
    else:
        assert rel(v, ref) < tol


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "fmm_*.npz"))),
                         ids=lambda p: os.path.basename(p)[4:-4])
def test_public_dense_matches_reference_fixture(cuda_lib, path):
    from electrodrive_gb300.core.bem_kernel import bem_matvec_gpu

    z = np.load(path)
    c, s, a, si = (torch.as_tensor(z[k]) for k in ("points", "sigma", "areas", "self_integrals"))
    ref = z["v_dense_reference"].astype(np.float64)
    for dev in ("cpu", "cuda"):
        v = bem_matvec_gpu(s.to(dev), c.to(dev), a.to(dev), self_integrals=si.to(dev), backend="torch_tiled")
        assert v.device.type == dev
        assert rel(v.cpu().numpy(), ref) < 2e-6


def test_external_backend_calls_matvec_impl(cuda_lib):
    from electrodrive_gb300.core.bem_kernel import bem_matvec_gpu
    from electrodrive_gb300.fmm3d import make_laplace_fmm_backend

    rng = np.random.default_rng(2)
    n = 3000
    c = torch.as_tensor(rng.random((n, 3)), dtype=torch.float64)
    a = torch.full((n,), 1.0 / n, dtype=torch.float64)
    s = torch.as_tensor(rng.uniform(-1, 1, n))
    fmm = make_laplace_fmm_backend(c, a, max_leaf_size=32)
    v_fmm = bem_matvec_gpu(s, c, a, backend="external", matvec_impl=fmm.matvec)
    v_dense = bem_matvec_gpu(s, c, a, backend="auto")
    assert rel(v_fmm.numpy(), v_dense.numpy()) < 1e-6
    with pytest.raises(ValueError):
        bem_matvec_gpu(s, c, a, backend="external")
    with pytest.raises(ValueError):
        bem_matvec_gpu(s, c, a, backend="nope")


def test_dense_nonfinite_clamped_and_empty(cuda_lib):
    from electrodrive_gb300 import _lib

    n = 500
    c = torch.rand(n, 3, device="cuda")
    s = torch.ones(n, device="cuda")
    a = torch.ones(n, device="cuda")
    si = torch.zeros(n, device="cuda")
    si[3] = float("nan")
    v = _lib.dense_matvec(c, s, a, si)
    assert v[3].item() == 0.0 and torch.isfinite(v).all()
    e = torch.empty(0, device="cuda")
    assert _lib.dense_matvec(torch.empty(0, 3, device="cuda"), e, e).numel() == 0
