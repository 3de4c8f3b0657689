"""PMIS coarsening on the GPU (coarsening LINA_PMIS, opt-in; not the reference's algorithm).

The labels of the finest level are compared with a restatement in numpy of the same rules
(strong connections as the reference defines them, measure |T_i| + hash fraction, independent-set
rounds, the final fix-up); hierarchies built on them must solve.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from fem_gb300 import lina, problems
from tests.conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA device")]

UNDECIDED, COARSE, FINE, ISOLATED = 0, 1, 2, 3


def strong_sets(ptr, col, val, em=0.3, ep=0.5):
    """S_i: the points row i depends on strongly (scalar problem: one unknown)."""
    n = len(ptr) - 1
    S = []
    for i in range(n):
        c, v = col[ptr[i]:ptr[i + 1]], val[ptr[i]:ptr[i + 1]]
        off = c != i
        neg = v[off & (v < 0)]
        if len(neg) == 0:
            S.append(np.zeros(0, np.int64))
            continue
        mn = neg.min()
        lo, hi = -em * abs(mn), ep * abs(mn)
        S.append(c[off & ((v < lo) | (v > hi))])
    return S


def mix32(h):
    h = h.astype(np.uint32)
    h ^= h >> np.uint32(16)
    h = h * np.uint32(0x85EBCA6B)
    h ^= h >> np.uint32(13)
    h = h * np.uint32(0xC2B2AE35)
    h ^= h >> np.uint32(16)
    return h


def pmis_labels(ptr, col, val):
    n = len(ptr) - 1
    S = strong_sets(ptr, col, val)
    T = [[] for _ in range(n)]
    for i in range(n):
        for j in S[i]:
            T[j].append(i)
    tlen = np.array([len(t) for t in T], np.float64)
    m = tlen + (mix32(np.arange(n)) >> np.uint32(8)).astype(np.float64) * (1.0 / 16777216.0)
    label = np.full(n, UNDECIDED)
    for i in range(n):
        if len(S[i]) == 0:
            nz = np.count_nonzero(val[ptr[i]:ptr[i + 1]])
            label[i] = ISOLATED if nz == 1 else COARSE
    label[(label == UNDECIDED) & (tlen == 0)] = FINE

    def above(a, b):
        return m[a] > m[b] or (m[a] == m[b] and a > b)

    while (label == UNDECIDED).any():
        new = label.copy()
        for i in np.flatnonzero(label == UNDECIDED):
            nb = list(S[i]) + T[i]
            if all(label[j] != UNDECIDED or above(i, j) for j in nb):
                new[i] = COARSE
        label = new
        new = label.copy()
        for i in np.flatnonzero(label == UNDECIDED):
            if any(label[j] == COARSE for j in S[i]):
                new[i] = FINE
        label = new
    new = label.copy()
    for i in np.flatnonzero(label == FINE):
        if len(S[i]) and not any(label[j] == COARSE for j in S[i]):
            new[i] = COARSE
    return new, S


@pytest.mark.parametrize("maker", [lambda: problems.poisson_p1(65, seed=0), lambda: problems.damage_qp(65)],
                         ids=["poisson65", "damage65"])
def test_finest_labels_match_restatement(maker):
    s = maker()
    a = lina.AMG.from_system(s, depth=4, coarsening=lina.PMIS)
    got = np.asarray(a.level(a.depth - 1).labels)
    want, S = pmis_labels(s.indptr, s.indices, s.data)
    assert np.array_equal(got, want)
    # every fine point depends strongly on a coarse point
    for i in np.flatnonzero(got == FINE):
        assert len(S[i]) == 0 or (got[S[i]] == COARSE).any()


@pytest.mark.parametrize("precision", [lina.PREC_FP64, lina.PREC_MIXED])
def test_pmis_hierarchy_solves(precision):
    """Elasticity at 129 x 129 nodes: a PMIS hierarchy is built (labels on every level from the GPU)
    and the preconditioned CG solve reaches the tolerance; building it twice gives the same
    hierarchy."""
    s = problems.elasticity_p1(129)
    opts = dict(depth=6, coarsening=lina.PMIS, smoother=lina.SMOOTHER_JACOBI, omega=0.6, precision=precision)
    a = lina.AMG.from_system(s, **opts)
    b = lina.AMG.from_system(s, **opts)
    assert a.sizes() == b.sizes()
    for l in range(1, a.depth):
        assert np.array_equal(a.level(l).labels, b.level(l).labels)
    x, info = a.pcg(s.b, tol=1e-8, max_iter=400)
    assert info.status == 0
    A = sp.csr_matrix((s.data, s.indices, s.indptr), shape=(s.n, s.n))
    assert np.linalg.norm(s.b - A @ x) <= 1e-7 * np.linalg.norm(s.b)


def test_pmis_hierarchy_files_round_trip(tmp_path):
    """A PMIS hierarchy saved and loaded keeps its coarsening and solves exactly as before."""
    s = problems.poisson_p1(65, seed=3)
    opts = dict(smoother=lina.SMOOTHER_JACOBI, omega=0.6, precision=lina.PREC_MIXED)
    a = lina.AMG.from_system(s, depth=4, coarsening=lina.PMIS, **opts)
    a.save(tmp_path / "h")
    b = lina.AMG.load(tmp_path / "h", **opts)
    assert a.sizes() == b.sizes()
    x1, i1 = a.pcg(s.b, tol=1e-8, max_iter=300)
    x2, i2 = b.pcg(s.b, tol=1e-8, max_iter=300)
    assert i1.status == 0 and i1.iterations == i2.iterations
    assert np.array_equal(x1, x2)
