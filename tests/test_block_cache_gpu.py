"""Build-time block cache of the plan builders (plan.cu): inside one cache
scope, released temporaries are reused by later reserves that fit, a
reserve larger than every held block still gets memory, and a buffer that
outlives the build and took an oversized cached block is moved to a block
of its own size."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_block_cache_reuse_fallback_and_exact_shrink(cuda_lib):
    res = (ctypes.c_int64 * 4)()
    assert cuda_lib.edfmm_block_cache_selfcheck(res) == 0, cuda_lib.edfmm_last_error()
    assert list(res) == [1, 1, 1, 1]
