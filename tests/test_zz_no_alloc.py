"""lina_gpu_dot_noalloc: the dot product for callers that cannot allocate device memory.

Such callers (an application that reserves the GPU's memory for its own pool at
start-up, a job under a hard device-memory quota) cannot have the library call
cudaMalloc in the middle of their computation.  They get the same result as
lina_gpu_dot, whose partial sums live in memory the library allocates; this
entry point keeps them in a fixed device array instead.  The
test allocates its own input vectors (the caller still provides inputs and
outputs) and compares the two entry points through the C-ABI on two calls in a
row, since every call reuses the shared array.
"""
import ctypes as C

import numpy as np
import pytest

from fem_gb300 import lina
from tests.conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA device")]

MAX_N = 33_554_432


def _dot(fn, a, b):
    r = C.c_double()
    rc = fn(a.ptr, b.ptr, a.n, C.byref(r))
    assert rc == 0, lina.last_error()
    return r.value


@pytest.mark.parametrize("n", [1, 2047, 2048, 1_000_003, 5 * (1 << 20)])
def test_noalloc_dot_matches_dot_on_two_calls(n):
    L = lina.lib()
    rng = np.random.default_rng(100 + n)
    tol = 1e-13
    for call in range(2):
        a = rng.standard_normal(n)
        b = rng.standard_normal(n)
        da, db = lina.DeviceArray.from_host(a), lina.DeviceArray.from_host(b)
        want = _dot(L.lina_gpu_dot, da, db)
        got = _dot(L.lina_gpu_dot_noalloc, da, db)
        scale = max(1.0, float(np.abs(a) @ np.abs(b)))
        assert abs(got - want) <= tol * scale, (call, got, want)
        assert abs(got - float(a @ b)) <= tol * scale


def test_noalloc_dot_zero_length_and_limit():
    L = lina.lib()
    da = lina.DeviceArray(1)
    r = C.c_double(5.0)
    assert L.lina_gpu_dot_noalloc(da.ptr, da.ptr, 0, C.byref(r)) == 0 and r.value == 0.0
    # beyond the fixed scratch capacity the call is refused before touching the GPU
    assert L.lina_gpu_dot_noalloc(da.ptr, da.ptr, MAX_N + 1, C.byref(r)) == lina.EINVAL
    assert "33554432" in lina.last_error()
