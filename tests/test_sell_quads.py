"""The quad layout of SELL-32 (lina_gpu_set_sell_quads): each lane holds four consecutive entries of
its row, loaded as one float4 of values and one uint2 of four 16-bit column offsets.

FP32 passes over natural-order SELL-32 matrices read it; it changes only how entries are fetched, never
the arithmetic of a row (entries are summed in stored order), so SpMV, Jacobi sweeps, prolongations,
residuals, V-cycles and whole PCG solves must equal those of the one-entry layout bit for bit, also after
new values are written into the matrix on the device.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from fem_gb300 import lina, problems
from tests.conftest import golden_cases, gpu_available, load_golden, system_for

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA device")]


@pytest.fixture
def layouts():
    yield
    lina.set_sell_quads(1)
    lina.set_sell_index_bits(16)
    lina.set_layout(lina.LAYOUT_AUTO)


def _pair(n, ptr, col, val, ncols=None):
    """(quad layout, one-entry layout) device matrices of the same CSR matrix."""
    lina.set_layout(lina.LAYOUT_SELL)
    out = []
    for q in (1, 0):
        lina.set_sell_quads(q)
        out.append(lina.Matrix(n, ptr, col, val, ncols=ncols))
    lina.set_sell_quads(1)
    return out


def _jacobi(M, n, prec, sweeps, seed=5):
    dt = np.float32 if prec == lina.PREC_MIXED else np.float64
    rng = np.random.default_rng(seed)
    b = lina.DeviceArray.from_host(rng.uniform(-1, 1, n).astype(dt))
    x = lina.DeviceArray.from_host(np.zeros(n, dt))
    t = lina.DeviceArray(n, dt)
    M.jacobi_device(b, x, t, 0.6, sweeps, prec)
    return (t if sweeps % 2 else x).to_host()


def _ragged(n, hi, seed, spread=2000):
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, hi, n)
    ptr = np.zeros(n + 1, np.int64)
    cols, vals = [], []
    for i in range(n):
        if lens[i] == 0:
            c, v = np.array([i]), np.array([0.0])  # the (i, 0.0) placeholder of an empty row
        else:
            c = np.unique(np.clip(i + rng.integers(-spread, spread, lens[i]), 0, n - 1))
            c = np.union1d(c, [i])
            v = rng.uniform(-1, 1, len(c))
            v[c == i] = 60.0
        cols.append(c)
        vals.append(v)
        ptr[i + 1] = ptr[i] + len(c)
    return ptr.astype(np.int32), np.concatenate(cols).astype(np.int32), np.concatenate(vals)


@pytest.mark.parametrize("n,hi", [(100_003, 61), (50_017, 13), (31, 9), (1_000_001, 5)])
def test_spmv_and_jacobi_identical(n, hi, layouts):
    """Row lengths 0..hi-1 (lengths not multiples of four, empty rows, a partial last slice)."""
    ptr, col, val = _ragged(n, hi, seed=n)
    Q, S = _pair(n, ptr, col, val)
    assert Q.index_bits() == 16
    x = np.random.default_rng(3).uniform(-1, 1, n)
    assert np.array_equal(Q.spmv(x, lina.PREC_MIXED), S.spmv(x, lina.PREC_MIXED))
    assert np.array_equal(Q.spmv(x, lina.PREC_FP64), S.spmv(x, lina.PREC_FP64))
    for sweeps in (1, 2, 3):
        assert np.array_equal(_jacobi(Q, n, lina.PREC_MIXED, sweeps), _jacobi(S, n, lina.PREC_MIXED, sweeps))
    A = sp.csr_matrix((val, col, ptr), shape=(n, n))
    y = Q.spmv(x, lina.PREC_MIXED)
    assert np.linalg.norm(y - A @ x) <= 1e-5 * np.linalg.norm(A @ x)


def test_rectangular_with_placeholder_columns(layouts):
    """A prolongation-like matrix (n x nc) whose empty rows hold (i, 0.0) with i >= nc: the
    placeholder is stored as padding inside the operand."""
    n, nc = 120_000, 30_000
    rng = np.random.default_rng(9)
    ptr = [0]
    cols, vals = [], []
    for i in range(n):
        if i % 7 == 3:
            c, v = [i], [0.0]
        else:
            c = sorted(set(rng.integers(max(0, i // 4 - 40), min(nc, i // 4 + 40), 4).tolist()))
            v = rng.uniform(0, 1, len(c)).tolist()
        cols += c
        vals += v
        ptr.append(len(cols))
    ptr, col, val = np.array(ptr, np.int32), np.array(cols, np.int32), np.array(vals)
    Q, S = _pair(n, ptr, col, val, ncols=nc)
    x = rng.uniform(-1, 1, nc)
    assert np.array_equal(Q.spmv(x, lina.PREC_MIXED), S.spmv(x, lina.PREC_MIXED))


def test_value_updates_reach_the_quad_layout(layouts):
    n = 40_000
    ptr, col, val = _ragged(n, 40, seed=11)
    Q, S = _pair(n, ptr, col, val)
    new = val * np.random.default_rng(12).uniform(0.5, 2.0, len(val))
    Q.update_values(new)
    S.update_values(new)
    x = np.random.default_rng(13).uniform(-1, 1, n)
    assert np.array_equal(Q.spmv(x, lina.PREC_MIXED), S.spmv(x, lina.PREC_MIXED))
    assert np.array_equal(_jacobi(Q, n, lina.PREC_MIXED, 2), _jacobi(S, n, lina.PREC_MIXED, 2))


@pytest.mark.parametrize("name", golden_cases("hierarchy"))
@pytest.mark.parametrize("smoother", [lina.SMOOTHER_JACOBI, lina.SMOOTHER_MC_SOR])
def test_mixed_solves_identical(name, smoother, layouts):
    """Every level in SELL-32: mixed-precision V-cycles and PCG solves with the quad layout equal those
    with the one-entry layout bit for bit."""
    g = load_golden(name)
    s = system_for(name)
    omega = 0.6 if smoother == lina.SMOOTHER_JACOBI else 1.0
    lina.set_layout(lina.LAYOUT_SELL)
    out = []
    for q in (1, 0):
        lina.set_sell_quads(q)
        a = lina.AMG.from_system(s, depth=int(g["depth"]), coarsening=int(g["coarsening"]), smoother=smoother,
                                 omega=omega, precision=lina.PREC_MIXED)
        z = a.vcycle(g["vcycle_r"])
        x, info = a.pcg(s.b, tol=1e-8, max_iter=500)
        assert info.status == 0
        out.append((z, x, info.iterations))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1]) and out[0][2] == out[1][2]


def test_update_values_of_hierarchy(layouts):
    """lina_gpu_amg_update_values writes the finest matrix's new values into the quad layout too."""
    s = problems.elasticity_p1(129)
    new = s.data * 1.25  # same pattern, symmetric
    out = []
    for q in (1, 0):
        lina.set_sell_quads(q)
        lina.set_layout(lina.LAYOUT_SELL)
        a = lina.AMG.from_system(s, depth=6, coarsening=lina.STANDARD, smoother=lina.SMOOTHER_JACOBI, omega=0.6,
                                 precision=lina.PREC_MIXED)
        a.update_values(new)
        x, info = a.pcg(s.b, tol=1e-8, max_iter=500)
        out.append((x, info.iterations))
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1] == out[1][1]
