"""C ABI checks that need no GPU: the library loads and exports every
function include/edfmm.h declares, and the ctypes mirror of
edfmm_plan_info has the C layout (checked with gcc against the header)."""
import ctypes
import os
import subprocess
import tempfile

import pytest


def test_library_exports_every_header_symbol(edlib):
    from electrodrive_gb300 import _lib

    names = _lib.header_symbols()
    assert "edfmm_plan_create" in names and "edfmm_plan_matvec" in names
    missing = [n for n in names if not hasattr(edlib, n)]
    assert not missing, missing


def test_version_and_error_strings(edlib):
    assert edlib.edfmm_version().decode().startswith("edfmm")
    assert isinstance(edlib.edfmm_last_error(), bytes)


def test_null_plan_is_an_argument_error(edlib):
    from electrodrive_gb300 import _lib

    info = _lib.PlanInfo()
    assert edlib.edfmm_plan_get_info(None, ctypes.byref(info)) == _lib.EDFMM_ERR_ARG
    assert b"NULL" in edlib.edfmm_last_error()
    assert edlib.edfmm_plan_matvec(None, None, None, None, 1.0, None, 0, None) == _lib.EDFMM_ERR_ARG


def test_plan_create_rejects_bad_arguments_before_touching_the_gpu(edlib):
    from electrodrive_gb300 import _lib

    h = ctypes.c_void_p()
    assert edlib.edfmm_plan_create(None, 10, 0, 64, 32, 0.5, 8, None, ctypes.byref(h)) == _lib.EDFMM_ERR_ARG
    assert edlib.edfmm_plan_create(None, 0, 7, 64, 32, 0.5, 8, None, ctypes.byref(h)) == _lib.EDFMM_ERR_ARG
    assert edlib.edfmm_plan_create(None, 0, 0, 0, 32, 0.5, 8, None, ctypes.byref(h)) == _lib.EDFMM_ERR_ARG
    assert edlib.edfmm_plan_create(None, 0, 0, 64, 32, 1.5, 8, None, ctypes.byref(h)) == _lib.EDFMM_ERR_ARG
    assert edlib.edfmm_plan_create(None, 0, 0, 64, 32, 0.5, 11, None, ctypes.byref(h)) == _lib.EDFMM_ERR_UNSUPPORTED
    assert not h.value


def test_plan_info_layout_matches_header():
    from electrodrive_gb300 import _lib

    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "edfmm.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(edfmm_plan_info), offsetof(edfmm_plan_info, max_level),
         offsetof(edfmm_plan_info, max_depth), offsetof(edfmm_plan_info, mac_theta));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        with open(c, "w") as f:
            f.write(src)
        r = subprocess.run(["gcc", "-I", os.path.dirname(_lib.HEADER_PATH), c, "-o", exe], capture_output=True, text=True)
        if r.returncode != 0:
            pytest.skip("gcc unavailable: " + r.stderr)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    P = _lib.PlanInfo
    assert [int(x) for x in out] == [ctypes.sizeof(P), P.max_level.offset, P.max_depth.offset, P.mac_theta.offset]


def test_product_fails_loudly_without_cuda(monkeypatch):
    import torch

    from electrodrive_gb300 import _lib

    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    with pytest.raises(RuntimeError, match="CUDA"):
        _lib.load_library(require_cuda=True)
    from electrodrive_gb300.fmm3d import make_laplace_fmm_backend

    c = torch.rand(10, 3)
    a = torch.ones(10)
    with pytest.raises(RuntimeError):
        make_laplace_fmm_backend(c, a)


def test_fmm_config_validation_matches_reference():
    import torch

    from electrodrive_gb300.fmm3d import FmmConfig

    assert FmmConfig().dtype == torch.float32
    assert FmmConfig(precision="double").dtype == torch.float64
    for bad in (dict(expansion_order=0), dict(mac_theta=0.95), dict(leaf_size=0), dict(expansion_order=17),
                dict(p2p_batch_size=0)):
        with pytest.raises(ValueError):
            FmmConfig(**bad)


def test_new_entry_points_reject_bad_arguments_before_touching_the_gpu(edlib):
    """Field, evaluation-side near quadrature and batched GMRES check their
    arguments on the host and return EDFMM_ERR_ARG without a CUDA call."""
    from electrodrive_gb300 import _lib

    E = _lib.EDFMM_ERR_ARG
    # field at targets: negative sizes, bad dtype, NULL arrays
    assert edlib.edfmm_dense_field_targets(None, -1, None, None, None, 4, 0, 1.0, None, None) == E
    assert edlib.edfmm_dense_field_targets(None, 4, None, None, None, 4, 9, 1.0, None, None) == E
    assert edlib.edfmm_dense_field_targets(None, 4, None, None, None, 4, 0, 1.0, None, None) == E
    # m = 0 is a no-op
    assert edlib.edfmm_dense_field_targets(None, 0, None, None, None, 4, 0, 1.0, None, None) == _lib.EDFMM_OK
    # evaluation-side near quadrature: depth beyond the rule's limit, NULL arrays
    assert edlib.edfmm_near_targets_correct(None, 3, None, None, None, None, 3, 1.5, 2, 9, 1.0, None, None) == E
    assert edlib.edfmm_near_targets_correct(None, 3, None, None, None, None, 3, 1.5, 2, 3, 1.0, None, None) == E
    assert edlib.edfmm_near_targets_correct(None, 0, None, None, None, None, 3, 1.5, 2, 3, 1.0, None, None) == \
        _lib.EDFMM_OK
    # batched GMRES: restart out of range, max_seg beyond n, NULL arrays, bad step index
    assert edlib.edfmm_bgmres_start(10, 0, 2, None, 5, 0, None, None, None, None, None, 1, None, None, None) == E
    assert edlib.edfmm_bgmres_start(10, 0, 2, None, 11, 8, None, None, None, None, None, 1, None, None, None) == E
    assert edlib.edfmm_bgmres_start(10, 0, 2, None, 5, 8, None, None, None, None, None, 1, None, None, None) == E
    assert edlib.edfmm_bgmres_arnoldi(10, 0, 2, None, 5, 8, 8, None, None, None, None, None, None, None) == E
    assert edlib.edfmm_bgmres_update(10, 0, 2, None, 5, 8, 9, None, None, None, None, None) == E
    assert int(edlib.edfmm_bgmres_state_cols(40)) == 50
    # near-set conversion: NULL handle or output, bad dtype
    import ctypes
    h = ctypes.c_void_p()
    assert edlib.edfmm_near_convert(None, 0, None, ctypes.byref(h)) == E
    assert edlib.edfmm_near_convert(None, 0, None, None) == E
    assert edlib.edfmm_near_convert(ctypes.c_void_p(1), 7, None, ctypes.byref(h)) == E and not h.value
    # plan conversion: NULL plan or output, bad dtype, order out of range
    assert edlib.edfmm_plan_convert(None, 0, 8, None, ctypes.byref(h)) == E and not h.value
    assert edlib.edfmm_plan_convert(ctypes.c_void_p(1), 0, 8, None, None) == E
    assert edlib.edfmm_plan_convert(ctypes.c_void_p(1), 5, 8, None, ctypes.byref(h)) == E
    assert edlib.edfmm_plan_convert(ctypes.c_void_p(1), 0, 11, None, ctypes.byref(h)) == _lib.EDFMM_ERR_UNSUPPORTED
    assert int(edlib.edfmm_bgmres_work_bytes(3, 2000, 40)) > 0


def test_gmres_batched_validates_segments():
    import torch

    from electrodrive_gb300.core.bem_solver import gmres_batched

    b = torch.ones(6, dtype=torch.float64)
    with pytest.raises(ValueError):
        gmres_batched(lambda v: v, b, [0, 3, 5])  # does not end at len(b)
    with pytest.raises(ValueError):
        gmres_batched(lambda v: v, b, [0, 4, 3, 6])  # decreasing
    with pytest.raises(ValueError):
        gmres_batched(lambda v: v, b, [0, 6], restart=0)
    with pytest.raises(RuntimeError):
        gmres_batched(lambda v: v, b, [0, 2, 6])  # CPU tensors: the solver runs on CUDA only


def test_bem_E_field_targets_validates_like_the_reference():
    import torch

    from electrodrive_gb300.core.bem_kernel import bem_E_field_targets

    t = torch.zeros(3, 3, dtype=torch.float64)
    c = torch.zeros(4, 3, dtype=torch.float64)
    a = torch.ones(4, dtype=torch.float64)
    with pytest.raises(ValueError):
        bem_E_field_targets(t, c, a, a, backend="bogus")
    with pytest.raises(ValueError):
        bem_E_field_targets(t[:, :2], c, a, a)
    # no panels: a zero field without touching the GPU
    z = bem_E_field_targets(t, c[:0], a[:0], a[:0])
    assert z.shape == (3, 3) and not z.any()
