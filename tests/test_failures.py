"""Failure paths of the library, made to happen on the host: no GPU fault, trap or hang is involved.

Each case returns its documented code (or the drop-in API its documented value), and the device is
still usable afterwards: a normal solve on the same device follows every failure.
  - a NaN or infinite right-hand side: lina_gpu_pcg returns LINA_GPU_EBREAKDOWN; the drop-in pcg prints
    the reference's message and returns -1 where the reference exits (LinA/PCGS.c:220-223)
  - a zero diagonal in AMG_setup: LINA_GPU_ESETUP with the reference's message (the reference prints it
    and exits, LinA/Multigrid.c:999-1002); the drop-in AMG_setup returns NULL
  - an allocation that fails (a device-memory limit per handle, lina_gpu_set_device_memory_limit):
    LINA_GPU_ECUDA from the set-up, nothing left allocated
The bounded device waits of the ILU kernels are exercised in tests/test_ilu.py (a flag nothing sets).
"""
import ctypes as C

import numpy as np
import pytest

from fem_gb300 import lina, problems

def _zero_diagonal_system():
    s = problems.poisson_p1(17, seed=0)
    data = s.data.copy()
    i = 8 * 17 + 8  # an interior row, strongly connected to its neighbours
    for p in range(s.indptr[i], s.indptr[i + 1]):
        if s.indices[p] == i:
            data[p] = 0.0
    return s, data


def test_zero_diagonal_rejected_by_setup():
    """The host set-up stops where the reference aborts: no device is touched."""
    s, data = _zero_diagonal_system()
    with pytest.raises(lina.LinaError) as e:
        lina.AMG(s.n, s.indptr, s.indices, data, host_only=True, depth=3)
    assert "diagonal zero" in str(e.value) + lina.last_error()
    assert "(-3)" in str(e.value) or "ESETUP" in str(e.value) or "-3" in str(e.value)


def _solve_ok(amg, s):
    x, info = amg.pcg(s.b, tol=1e-8, max_iter=500)
    assert info.status == 0 and info.true_rel_residual <= 1e-8
    return x


@pytest.mark.gpu
@pytest.mark.parametrize("bad", [np.nan, np.inf])
@pytest.mark.parametrize("precision", [lina.PREC_FP64, lina.PREC_MIXED])
def test_nonfinite_rhs_is_a_breakdown(bad, precision):
    from tests.conftest import gpu_available
    if not gpu_available():
        pytest.skip("no CUDA device")
    s = problems.poisson_p1(33, seed=0)
    amg = lina.AMG.from_system(s, depth=4, precision=precision)
    b = s.b.copy()
    b[100] = bad
    x = np.zeros(s.n)
    info = lina.SolveInfo()
    rc = lina.lib().lina_gpu_pcg(amg.h, lina._dp(b), lina._dp(x), 1e-8, 200, lina.STOP_RELATIVE, 0,
                                 C.byref(info))
    assert rc == lina.EBREAKDOWN
    _solve_ok(amg, s)


@pytest.mark.gpu
def test_dropin_pcg_nan_returns_minus_one(capfd):
    from tests.conftest import gpu_available
    if not gpu_available():
        pytest.skip("no CUDA device")
    s = problems.poisson_p1(33, seed=0)
    L = lina.dropin()
    A = lina.RowListView(s.indptr, s.indices, s.data)
    L.AMG_print_info(0)
    data = L.AMG_setup(A.ref, 1, 4, 2, 2, 2, 0, 1, None, None)
    assert data
    L.PCG_default(A.ref, None, None)
    L.PCG_set_AMG_data(data)
    L.PCG_set_precon(C.cast(L.PCG_AMG_vcycle_precon, C.c_void_p))
    dp = C.POINTER(C.c_double)
    b = s.b.copy()
    b[7] = np.nan
    x = np.zeros(s.n)
    assert L.pcg(x.ctypes.data_as(dp), b.ctypes.data_as(dp), s.n, 1e-8, 200) == -1
    C.CDLL(None).fflush(None)  # the library prints through C stdio
    assert "nan" in capfd.readouterr().out
    b = s.b.copy()
    x = np.zeros(s.n)
    assert L.pcg(x.ctypes.data_as(dp), b.ctypes.data_as(dp), s.n, 1e-8, 200) > 0
    L.AMG_free_data(data)


@pytest.mark.gpu
def test_dropin_setup_with_zero_diagonal_returns_null():
    from tests.conftest import gpu_available
    if not gpu_available():
        pytest.skip("no CUDA device")
    s, data = _zero_diagonal_system()
    L = lina.dropin()
    A = lina.RowListView(s.indptr, s.indices, data)
    L.AMG_print_info(0)
    assert not L.AMG_setup(A.ref, 1, 3, 2, 2, 2, 0, 1, None, None)
    B = lina.RowListView(s.indptr, s.indices, s.data)
    ok = L.AMG_setup(B.ref, 1, 3, 2, 2, 2, 0, 1, None, None)
    assert ok
    L.AMG_free_data(ok)


@pytest.mark.gpu
def test_allocation_failure_is_reported_and_recoverable():
    from tests.conftest import gpu_available
    if not gpu_available():
        pytest.skip("no CUDA device")
    s = problems.elasticity_p1(65)
    try:
        lina.set_device_memory_limit(1 << 20)  # 1 MB: the hierarchy needs more
        with pytest.raises(lina.LinaError) as e:
            lina.AMG.from_system(s, depth=5)
        assert "device-memory limit" in str(e.value) or "device-memory limit" in lina.last_error()
    finally:
        lina.set_device_memory_limit(0)
    amg = lina.AMG.from_system(s, depth=5)
    _solve_ok(amg, s)
