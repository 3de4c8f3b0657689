"""Synthetic systems: determinism, symmetry and the stored digests of the golden inputs."""
import numpy as np
import pytest
import scipy.sparse as sp

from fem_gb300 import problems
from tests.conftest import golden_cases, regenerate, system_for


@pytest.mark.parametrize("name", golden_cases("hierarchy") + golden_cases("solve"))
def test_golden_inputs_regenerate(name):
    """The generator reproduces the stored inputs: pattern exactly, values to the last bits
    (bit for bit on the host that wrote the files; exp may differ in the last ulp elsewhere)."""
    g, s = system_for(name), regenerate(name)
    assert np.array_equal(g.indptr, s.indptr) and np.array_equal(g.indices, s.indices)
    np.testing.assert_allclose(s.data, g.data, rtol=1e-14, atol=1e-300)
    np.testing.assert_allclose(s.b, g.b, rtol=1e-14, atol=1e-300)


@pytest.mark.parametrize("maker", [lambda: problems.poisson_p1(33), lambda: problems.elasticity_p1(17)])
def test_symmetric_and_sorted(maker):
    s = maker()
    A = sp.csr_matrix((s.data, s.indices, s.indptr), shape=(s.n, s.n))
    assert abs(A - A.T).max() == 0.0
    for i in range(s.n):
        c = s.indices[s.indptr[i]:s.indptr[i + 1]]
        assert np.all(np.diff(c) > 0)


def test_poisson_stencil_and_zeros():
    s = problems.poisson_p1(5)
    # interior node 6 of a 5x5 grid: diagonal 4, interior axis neighbours -1, the diagonal
    # (NE) neighbour kept as an explicit 0; boundary columns (1, 5, 0) are eliminated
    row = dict(zip(s.indices[s.indptr[6]:s.indptr[7]], s.data[s.indptr[6]:s.indptr[7]]))
    assert row[6] == 4.0 and row[7] == -1.0 and row[11] == -1.0
    assert 12 in row and row[12] == 0.0
    assert 0 not in row and 1 not in row and 5 not in row


def test_elasticity_sizes_full_config():
    # the 1025 x 1025 configuration: 2,101,250 unknowns; checked on a small grid by formula
    m = 65
    s = problems.elasticity_p1(m)
    assert s.n == 2 * m * m and s.dof == 2
    interior = s.indptr[1:] - s.indptr[:-1]
    assert interior.max() == 14
