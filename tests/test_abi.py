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
