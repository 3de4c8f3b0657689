"""The coarsest AMG block inverted on the GPU (gpu_coarse.cu, lina_gpu_dense_inverse).

Blocked Gauss-Jordan elimination without pivoting, with the rank-32 updates on the FP64 CUDA cores
(SIMT) or on the FP64 tensor cores (DMMA, mma.sync m8n8k4): both must give the inverse to rounding
(checked against numpy's LU-based inverse), detect a zero pivot as the reference's LU would meet it, and,
inside a hierarchy, give the same V-cycles and solves as the host inversion.  The reference's own
coarse solves on a two-level hierarchy with a 2,000-row block are checked by the golden-file tests
(tests/golden/poisson65_d2.npz, e.g. tests/test_gpu_solve.py).
"""
import numpy as np
import pytest

from fem_gb300 import lina, problems
from tests.conftest import gpu_available, load_golden, system_for

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA device")]


def _matrix(m, seed):
    rng = np.random.default_rng(seed)
    a = rng.uniform(-1, 1, (m, m))
    a += np.diag(np.abs(a).sum(axis=1) + 1.0)  # diagonally dominant: no pivoting needed
    return a


@pytest.mark.parametrize("m", [1, 2, 31, 32, 33, 64, 100, 257, 1000])
@pytest.mark.parametrize("method", [lina.DENSE_SIMT, lina.DENSE_DMMA])
def test_inverse_matches_numpy(m, method):
    a = _matrix(m, m)
    d = lina.DeviceArray.from_host(a.ravel())
    lina.dense_inverse_device(d, m, method)
    inv = d.to_host().reshape(m, m)
    ref = np.linalg.inv(a)
    assert np.linalg.norm(inv - ref) <= 1e-13 * np.linalg.norm(ref) * max(1, m) ** 0.5
    assert np.linalg.norm(inv @ a - np.eye(m)) <= 1e-12 * max(1, m) ** 0.5


def test_simt_and_dmma_agree():
    m = 700
    a = _matrix(m, 7)
    out = []
    for method in (lina.DENSE_SIMT, lina.DENSE_DMMA):
        d = lina.DeviceArray.from_host(a.ravel())
        lina.dense_inverse_device(d, m, method)
        out.append(d.to_host())
    assert np.linalg.norm(out[0] - out[1]) <= 1e-13 * np.linalg.norm(out[0])


@pytest.mark.parametrize("method", [lina.DENSE_SIMT, lina.DENSE_DMMA])
def test_zero_pivot_is_reported(method):
    a = _matrix(40, 3)
    a[0, 0] = 0.0  # the first pivot of the elimination without pivoting
    d = lina.DeviceArray.from_host(a.ravel())
    with pytest.raises(lina.LinaError):
        lina.dense_inverse_device(d, 40, method)
    # the device stays usable
    b = lina.DeviceArray.from_host(_matrix(40, 4).ravel())
    lina.dense_inverse_device(b, 40, method)


@pytest.mark.parametrize("method", [lina.DENSE_SIMT, lina.DENSE_DMMA])
def test_hierarchy_device_inverse_equals_host_inverse(method):
    """The two-level Poisson hierarchy (coarsest block about 2,000 rows): V-cycle and solve with the block
    inverted on the GPU equal those with the host inverse to rounding, iterations exactly."""
    g = load_golden("poisson65_d2")
    s = system_for("poisson65_d2")
    out = []
    try:
        for rows in (256, 0):
            lina.set_coarse_inverse(rows, method)
            a = lina.AMG.from_system(s, depth=2, coarsening=lina.STANDARD, smoother=lina.SMOOTHER_JACOBI, omega=0.6)
            assert a.coarse_block > 1000
            z = a.vcycle(g["vcycle_r"])
            x, info = a.pcg(s.b, tol=1e-8, max_iter=100, stop=lina.STOP_REFERENCE,
                            flags=lina.PCG_NORMALIZE | lina.PCG_FINAL_PRECON)
            out.append((z, x, info.iterations))
    finally:
        lina.set_coarse_inverse(256, lina.DENSE_SIMT)
    assert np.linalg.norm(out[0][0] - out[1][0]) <= 1e-12 * np.linalg.norm(out[1][0])
    assert np.linalg.norm(out[0][1] - out[1][1]) <= 1e-12 * np.linalg.norm(out[1][1])
    assert out[0][2] == out[1][2]
    # and the reference's own solve (its dense LU on the same block)
    assert abs(out[0][2] - int(g["pcg_jacobi_it"])) <= 1
    assert np.linalg.norm(out[0][1] - g["pcg_jacobi_x"]) <= 1e-9 * np.linalg.norm(g["pcg_jacobi_x"])
