"""This library's on-the-fly near-field module (edfmm_near_quadrature_matvec
through core.bem_near.apply_near_quadrature_matvec_cuda) against the
reference's own CUDA module (electrodrive/core/bem_near_cuda_kernel.cu and
bem_near_cuda.cpp, built unmodified from the reference's sources by
oracle/ref_near.py) on the same inputs, FP64, orders 1 and 2: equal within
1e-10 of the size of the terms each correction is a difference of.  Skipped
where the reference sources are not available to build."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
NEAR = np.load(os.path.join(GOLDEN, "near_cases.npz"))


@pytest.fixture(scope="module")
def ref_module():
    from oracle import ref_near

    if not ref_near.copy_sources():
        pytest.skip("the reference's near-field sources are not present on this machine")
    return ref_near.load()


@pytest.mark.parametrize("order", [1, 2])
def test_on_the_fly_module_equals_the_reference_module(cuda_lib, ref_module, order):
    from electrodrive_gb300.core.bem_near import apply_near_quadrature_matvec_cuda
    from electrodrive_gb300.utils.config import K_E

    C, A, PV = (NEAR[f"torus__{k}"] for k in ("centroids", "areas", "panel_vertices"))
    pairs = NEAR["torus__near_pairs"]
    sig = NEAR["torus__sigma"]
    T = lambda x: torch.as_tensor(np.ascontiguousarray(x), device="cuda")
    rng = np.random.default_rng(3)
    pp = T(pairs[rng.permutation(pairs.shape[0])].astype(np.int64))  # unsorted, as callers pass them
    vfar = T(rng.uniform(-1, 1, C.shape[0]) * 1e9)
    ref = ref_module.near_quadrature_matvec(vfar, T(sig), T(C), T(A), T(PV), pp, float(K_E), order)
    ours = apply_near_quadrature_matvec_cuda(vfar, T(sig), centroids=T(C), areas=T(A), panel_vertices=T(PV),
                                             near_pairs=pp, quad_order=order)
    i, j = pairs[:, 0], pairs[:, 1]
    r = np.linalg.norm(C[i] - C[j], axis=1)
    scale = np.zeros(C.shape[0])
    np.add.at(scale, i, K_E * A[j] * np.abs(sig[j]) / r)
    diff = np.abs(ref.cpu().numpy() - ours.cpu().numpy())
    assert np.all(diff <= 1e-10 * (scale + np.abs(vfar.cpu().numpy())) + 1e-300)
