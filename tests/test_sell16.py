"""16-bit column offsets in the SELL-32 layout (lina_gpu_set_sell_index_bits).

A SELL-32 matrix with long rows (at least 24 entries per row on average) also stores, per slice of
32 rows, two bases and for every entry a 15-bit offset from one of them, which its FP32 passes read;
a matrix with a slice whose columns do not fit two windows of 32,768, or with short rows, keeps int
columns only.  The layout changes only the bytes moved, never the arithmetic of a row: SpMV, Jacobi
sweeps, V-cycles and whole PCG solves must be bit-identical to the int layout.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from fem_gb300 import lina, problems
from tests.conftest import golden_cases, gpu_available, load_golden, system_for

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA device")]


@pytest.fixture
def bits():
    """The one-entry SELL-32 layout (quads off; tests/test_sell_quads.py covers the quad layout)."""
    def set_bits(b):
        lina.set_sell_index_bits(b)
    lina.set_sell_quads(0)
    yield set_bits
    lina.set_sell_index_bits(16)
    lina.set_sell_quads(1)
    lina.set_layout(lina.LAYOUT_AUTO)


def test_rejects_other_widths():
    with pytest.raises(lina.LinaError):
        lina.set_sell_index_bits(8)


def _matrix(n, ptr, col, val, b):
    lina.set_sell_index_bits(b)
    return lina.Matrix(n, ptr, col, val)


def test_two_windows_elasticity(bits):
    """The square of the 2x257^2 = 132,098-row elasticity matrix (about 50 entries per row; the
    components blocked, so the coupling to the other component lies half the matrix away and
    slices use both windows): SpMV equals the int layout exactly; the short-row matrix itself keeps
    int columns."""
    s = problems.elasticity_p1(257)
    A = sp.csr_matrix((s.data, s.indices, s.indptr), shape=(s.n, s.n))
    assert _matrix(s.n, s.indptr, s.indices, s.data, 16).index_bits() == 32
    A2 = (A @ A).tocsr()
    A2.sort_indices()
    ip, ix = A2.indptr.astype(np.int32), A2.indices.astype(np.int32)
    M16 = _matrix(s.n, ip, ix, A2.data, 16)
    M32 = _matrix(s.n, ip, ix, A2.data, 32)
    assert M16.index_bits() == 16 and M32.index_bits() == 32
    x = np.random.default_rng(0).uniform(-1, 1, s.n)
    for prec in (lina.PREC_FP64, lina.PREC_MIXED):
        y16, y32 = M16.spmv(x, prec), M32.spmv(x, prec)
        assert np.array_equal(y16, y32)
    assert np.linalg.norm(M16.spmv(x, lina.PREC_FP64) - A2 @ x) <= 1e-14 * np.linalg.norm(A2 @ x)


def test_scattered_columns_keep_int_columns(bits):
    """Long rows whose columns spread over the whole range: no slice fits two windows, the matrix
    keeps int columns and stays exact.  n is not a multiple of 32 (the last slice is partial)."""
    n = 100_003
    rng = np.random.default_rng(1)
    rows = np.repeat(np.arange(n), 31)
    cols = np.concatenate([np.arange(n)[:, None], rng.integers(0, n, (n, 30))], axis=1).ravel()
    vals = rng.uniform(-1, 1, len(cols))
    vals[::31] = 40.0
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    A.sum_duplicates()
    A.sort_indices()
    M = _matrix(n, A.indptr, A.indices, A.data, 16)
    assert M.index_bits() == 32
    x = rng.uniform(-1, 1, n)
    assert np.linalg.norm(M.spmv(x, lina.PREC_FP64) - A @ x) <= 1e-14 * np.linalg.norm(A @ x)


def test_ragged_rows_and_partial_slice(bits):
    """Long rows of very different lengths (empty ones hold the (i, 0.0) placeholder), n = 100,001."""
    n = 100_001
    rng = np.random.default_rng(2)
    lens = rng.integers(0, 60, n)
    lens[rng.integers(0, n, 500)] = 0
    ptr = np.zeros(n + 1, np.int64)
    cols, vals = [], []
    for i in range(n):
        if lens[i] == 0:
            c = np.array([i])
            v = np.array([0.0])
        else:
            c = np.unique(np.clip(i + rng.integers(-3000, 3000, lens[i]), 0, n - 1))
            v = rng.uniform(-1, 1, len(c))
        cols.append(c)
        vals.append(v)
        ptr[i + 1] = ptr[i] + len(c)
    col = np.concatenate(cols).astype(np.int32)
    val = np.concatenate(vals)
    lina.set_layout(lina.LAYOUT_SELL)
    M16 = _matrix(n, ptr.astype(np.int32), col, val, 16)
    M32 = _matrix(n, ptr.astype(np.int32), col, val, 32)
    assert M16.index_bits() == 16
    x = rng.uniform(-1, 1, n)
    A = sp.csr_matrix((val, col, ptr), shape=(n, n))
    for prec in (lina.PREC_FP64, lina.PREC_MIXED):
        assert np.array_equal(M16.spmv(x, prec), M32.spmv(x, prec))
    assert np.linalg.norm(M16.spmv(x, lina.PREC_FP64) - A @ x) <= 1e-14 * np.linalg.norm(A @ x)


@pytest.mark.parametrize("name", golden_cases("hierarchy"))
@pytest.mark.parametrize("smoother", [lina.SMOOTHER_JACOBI, lina.SMOOTHER_MC_SOR])
@pytest.mark.parametrize("precision", [lina.PREC_FP64, lina.PREC_MIXED])
def test_solves_identical_to_int_columns(name, smoother, precision, bits):
    """Every level in SELL-32: V-cycles and PCG solves with 16-bit columns equal those with int
    columns bit for bit."""
    g = load_golden(name)
    s = system_for(name)
    omega = 0.6 if smoother == lina.SMOOTHER_JACOBI else 1.0
    lina.set_layout(lina.LAYOUT_SELL)
    out = []
    for b in (16, 32):
        lina.set_sell_index_bits(b)
        a = lina.AMG.from_system(s, depth=int(g["depth"]), coarsening=int(g["coarsening"]), smoother=smoother,
                                 omega=omega, precision=precision)
        widths = {w for l in range(a.depth) for w in a.index_bits(l)}
        assert widths <= ({0, 16, 32} if b == 16 else {0, 32})
        z = a.vcycle(g["vcycle_r"])
        x, info = a.pcg(s.b, tol=1e-8, max_iter=500)
        assert info.status == 0
        out.append((z, x, info.iterations))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1]) and out[0][2] == out[1][2]


def _jacobi(M, n, dt, prec, sweeps=3):
    rng = np.random.default_rng(5)
    b = lina.DeviceArray.from_host(rng.uniform(-1, 1, n).astype(dt))
    x = lina.DeviceArray.from_host(np.zeros(n, dt))
    t = lina.DeviceArray(n, dt)
    M.jacobi_device(b, x, t, 0.6, sweeps, prec)
    return (t if sweeps % 2 else x).to_host()


def test_jacobi_identical_long_rows(bits):
    """Rows of 0 to 60 entries (the software-pipelined variant for long rows and the short-row
    variant): Jacobi sweeps in both precisions equal those of the 32-bit layout bit for bit."""
    n = 50_017
    rng = np.random.default_rng(4)
    res = []
    for lens_hi in (61, 12):
        lens = rng.integers(0, lens_hi, n)
        rows = np.repeat(np.arange(n), lens)
        cols = np.clip(rows + rng.integers(-2000, 2000, len(rows)), 0, n - 1)
        R = (sp.csr_matrix((rng.uniform(-1, 1, len(rows)), (rows, cols)), shape=(n, n)) + sp.identity(n) * 50.0).tocsr()
        R.sum_duplicates()
        R.sort_indices()
        lina.set_layout(lina.LAYOUT_SELL)
        out = []
        for b in (16, 32):
            M = _matrix(n, R.indptr.astype(np.int32), R.indices.astype(np.int32), R.data, b)
            assert M.index_bits() == (b if lens_hi > 48 else 32)
            out.append([_jacobi(M, n, np.float64, lina.PREC_FP64), _jacobi(M, n, np.float32, lina.PREC_MIXED)])
            M.close()
        for a, c in zip(*out):
            assert np.array_equal(a, c)
