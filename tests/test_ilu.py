"""ILU(0) factorisation and application (lina_gpu_ilu_*).

Oracle: the reference's incomplete_LU_factorization on model, nonsymmetric, ragged and
zero-pivot matrices (tests/golden/ilu.npz, made by tests/golden/make_golden.py); the two CPU
restatements (oracle/ilu.py, oracle/lina_port.c) are pinned to it bit for bit and check the
device factors at full size.  The bar for the factors is bit-identity.
"""
import ctypes as C
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from fem_gb300 import lina, problems
from oracle import ilu as oilu
from oracle import port
from tests.conftest import ROOT, gpu_available

GOLDEN = os.path.join(ROOT, "tests", "golden", "ilu.npz")
CASES = ["poisson33", "elast17", "damage65", "nonsym400"]


def load():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


def matrix(g, name):
    return g[f"{name}_ptr"], g[f"{name}_col"], g[f"{name}_val"]


def factors(n, ptr, col, f):
    """(L with its diagonal, U with a unit diagonal) as scipy matrices from values on A's pattern."""
    A = sp.csr_matrix((f, col, ptr), shape=(n, n))
    return sp.tril(A, format="csr"), (sp.triu(A, k=1) + sp.identity(n)).tocsr()


@pytest.mark.parametrize("name", CASES)
def test_restatements_match_reference_factors(name):
    """Pins both CPU restatements against the reference's factors."""
    g = load()
    assert int(g[f"{name}_ok"]) == 1
    f = g[f"{name}_f"]
    assert not np.isnan(f).any()
    assert np.array_equal(oilu.ilu0(*matrix(g, name)), f)
    assert np.array_equal(port.ilu0(*matrix(g, name)), f)


def test_zero_pivot_fails_like_reference():
    g = load()
    assert int(g["zeropivot3_ok"]) == 0
    with pytest.raises(oilu.ZeroPivot):
        oilu.ilu0(*matrix(g, "zeropivot3"))
    with pytest.raises(ArithmeticError):
        port.ilu0(*matrix(g, "zeropivot3"))


@pytest.mark.parametrize("name", ["poisson33", "elast17"])
def test_golden_inputs_regenerate(name):
    """The generator reproduces the stored inputs: the pattern exactly, the values to the last bits (the
    stored elasticity values came from a library exponential, the generator's is portable_exp)."""
    g = load()
    s = problems.poisson_p1(33, seed=0) if name == "poisson33" else problems.elasticity_p1(17)
    ptr, col, val = matrix(g, name)
    assert np.array_equal(s.indptr, ptr) and np.array_equal(s.indices, col)
    np.testing.assert_allclose(s.data, val, rtol=1e-14, atol=1e-300)


def test_factors_solve_the_pattern_equations():
    """(L U)_ij = a_ij on A's pattern (the defining property of ILU(0)), on the stored factors."""
    g = load()
    for name in CASES:
        ptr, col, val = matrix(g, name)
        n = len(ptr) - 1
        L, U = factors(n, ptr, col, g[f"{name}_f"])
        LU = (L @ U).tocsr()
        rows = np.repeat(np.arange(n), np.diff(ptr))
        lu = np.asarray(LU[rows, col]).ravel()
        assert np.abs(lu - val).max() <= 1e-12 * np.abs(val).max(), name


def test_invalid_pattern_is_rejected():
    """Unsorted or repeated columns are refused before any device work."""
    ptr = np.array([0, 2, 4], dtype=np.int32)
    for col in (np.array([1, 0, 0, 1]), np.array([0, 0, 0, 1]), np.array([0, 2, 0, 1])):
        with pytest.raises(lina.LinaError):
            lina.ILU(2, ptr, col, np.ones(4))


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
@pytest.mark.parametrize("name", CASES)
def test_gpu_factors_are_bit_identical_to_reference(name):
    g = load()
    ptr, col, val = matrix(g, name)
    ilu = lina.ILU(len(ptr) - 1, ptr, col, val)
    assert np.array_equal(ilu.factor_values(), g[f"{name}_f"])


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
def test_gpu_zero_pivot_is_a_setup_error():
    g = load()
    ptr, col, val = matrix(g, "zeropivot3")
    with pytest.raises(lina.LinaError, match=f"\\({lina.ESETUP}\\)"):
        lina.ILU(3, ptr, col, val)
    # the library stays usable after the failure
    ptr, col, val = matrix(g, "nonsym400")
    assert np.array_equal(lina.ILU(400, ptr, col, val).factor_values(), g["nonsym400_f"])


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("prec", [lina.PREC_FP64, lina.PREC_MIXED])
def test_gpu_apply_matches_triangular_solves(name, prec):
    """z = U^-1 L^-1 r against scipy's triangular solves with the reference's factors; repeated
    applications give the same bits."""
    g = load()
    ptr, col, val = matrix(g, name)
    n = len(ptr) - 1
    L, U = factors(n, ptr, col, g[f"{name}_f"])
    r = np.random.default_rng(3).standard_normal(n)
    z_ref = spla.spsolve_triangular(U, spla.spsolve_triangular(L, r, lower=True), lower=False)
    ilu = lina.ILU(n, ptr, col, val)
    z = ilu.apply(r, prec)
    tol = 1e-12 if prec == lina.PREC_FP64 else 1e-4
    assert np.linalg.norm(z - z_ref) / np.linalg.norm(z_ref) <= tol
    for _ in range(5):
        assert np.array_equal(ilu.apply(r, prec), z)


def _full_size_systems():
    yield "damage1025", problems.damage_qp(1025)
    yield "elast257", problems.elasticity_p1(257)


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
def test_gpu_factors_full_size_match_restatement():
    """The damage Hessian at 1025 x 1025 nodes (1,050,625 rows) and plane elasticity at 257 x 257
    nodes: device factors bit-identical to the C restatement."""
    for name, s in _full_size_systems():
        ilu = lina.ILU(s.n, s.indptr, s.indices, s.data)
        assert np.array_equal(ilu.factor_values(), port.ilu0(s.indptr, s.indices, s.data)), name


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
def test_gpu_factors_wide_levels_match_restatement():
    """Two levels of 1,000 and 99,000 rows (every row past the first thousand couples to three of
    them, symmetrically): 99,000 rows factorised concurrently by the row pool, bit-identical to the
    C restatement."""
    n, k = 100_000, 1_000
    rng = np.random.default_rng(12)
    rows = np.repeat(np.arange(k, n), 3)
    cols = rng.integers(0, k, len(rows))
    v = rng.uniform(-1, 1, len(rows))
    A = sp.coo_matrix((v, (rows, cols)), shape=(n, n))
    A = (A + A.T + sp.diags(10.0 + rng.random(n))).tocsr()
    A.sum_duplicates()
    A.sort_indices()
    ilu = lina.ILU(n, A.indptr, A.indices, A.data)
    assert ilu.levels()[0] == 2
    assert np.array_equal(ilu.factor_values(), port.ilu0(A.indptr, A.indices, A.data))


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
def test_gpu_apply_inverts_a_tridiagonal_matrix():
    """On a tridiagonal matrix ILU(0) is the exact LU factorisation, so the application solves
    A z = r: 1,000,000 rows (more than the GPU holds threads at once), nonsymmetric, one level per
    row in the factorisation and both solves."""
    n = 1_000_000
    rng = np.random.default_rng(9)
    lo, up = rng.uniform(-1, 0, n - 1), rng.uniform(-1, 0, n - 1)
    d = 2.5 + rng.random(n)
    A = sp.diags([lo, d, up], [-1, 0, 1], format="csr")
    A.sort_indices()
    r = rng.standard_normal(n)
    ilu = lina.ILU(n, A.indptr, A.indices, A.data)
    assert ilu.levels() == (n, n)
    z = ilu.apply(r)
    assert np.linalg.norm(A @ z - r) / np.linalg.norm(r) <= 1e-13
    z32 = ilu.apply(r, lina.PREC_MIXED)
    assert np.linalg.norm(A @ z32 - r) / np.linalg.norm(r) <= 1e-5


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
@pytest.mark.parametrize("name", ["nonsym400", "damage65"])
def test_gpu_refactor_equals_new_factorisation(name):
    """New values on the same pattern: the refactorised handle gives the factors and the
    application of a handle created from the new values, bit for bit."""
    g = load()
    ptr, col, val = matrix(g, name)
    n = len(ptr) - 1
    rng = np.random.default_rng(12)
    val2 = val * (1.0 + 0.1 * rng.standard_normal(len(val)))
    ilu = lina.ILU(n, ptr, col, val)
    ilu.refactor(val2)
    fresh = lina.ILU(n, ptr, col, val2)
    assert np.array_equal(ilu.factor_values(), fresh.factor_values())
    assert np.array_equal(ilu.factor_values(), port.ilu0(ptr, col, val2))
    r = rng.standard_normal(n)
    for prec in (lina.PREC_FP64, lina.PREC_MIXED):
        assert np.array_equal(ilu.apply(r, prec), fresh.apply(r, prec))


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
def test_gpu_refactor_zero_pivot_keeps_handle_usable():
    g = load()
    ptr, col, val = matrix(g, "nonsym400")
    ilu = lina.ILU(400, ptr, col, val)
    # a row with no entries left of the diagonal and some right of it: a zero diagonal there is a
    # zero pivot L_rr = a_rr = 0
    rows = [r for r in range(400) if not (col[ptr[r]:ptr[r + 1]] < r).any() and (col[ptr[r]:ptr[r + 1]] > r).any()]
    assert rows
    r = rows[0]
    bad = val.copy()
    bad[ptr[r] + int(np.nonzero(col[ptr[r]:ptr[r + 1]] == r)[0][0])] = 0.0
    with pytest.raises(lina.LinaError, match=f"\\({lina.ESETUP}\\)"):
        ilu.refactor(bad)
    ilu.refactor(val)
    assert np.array_equal(ilu.factor_values(), g["nonsym400_f"])


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
def test_gpu_wait_runs_out_and_device_stays_usable():
    """A device wait on a flag nothing sets ends after its limit with the error a timed-out solve
    reports; the next solve works."""
    waited = C.c_double()
    rc = lina.lib().lina_gpu_wait_probe(200000, C.byref(waited))
    assert rc == lina.ECUDA and "ran out" in lina.last_error()
    assert 200e3 <= waited.value < 5e6
    g = load()
    ptr, col, val = matrix(g, "nonsym400")
    assert np.array_equal(lina.ILU(400, ptr, col, val).factor_values(), g["nonsym400_f"])
    assert lina.lib().lina_gpu_wait_probe(0, None) == lina.EINVAL


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
@pytest.mark.parametrize("prec", [lina.PREC_FP64, lina.PREC_MIXED])
def test_gpu_timed_application_runs_the_solves(prec):
    """lina_gpu_ilu_time_apply: positive device time, and the handle applies correctly afterwards."""
    q = problems.at2_damage(65)
    ilu = lina.ILU(q.n, q.indptr, q.indices, q.data)
    ms = ilu.time_apply(5, prec)
    assert 0.0 < ms < 1e3
    assert ilu.apply_bytes(prec) > 8 * q.n
    r = np.random.default_rng(0).standard_normal(q.n)
    f = port.ilu0(q.indptr, q.indices, q.data)
    A = sp.csr_matrix((f, q.indices, q.indptr), shape=(q.n, q.n))
    L = sp.tril(A, format="csr")
    U = sp.triu(A, 1, format="csr") + sp.identity(q.n, format="csr")
    z_ref = spla.spsolve_triangular(U, spla.spsolve_triangular(L, r, lower=True), lower=False)
    z = ilu.apply(r, prec)
    assert np.linalg.norm(z - z_ref) / np.linalg.norm(z_ref) < (1e-12 if prec == lina.PREC_FP64 else 1e-5)
