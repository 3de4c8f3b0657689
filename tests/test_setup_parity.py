"""AMG setup of the GB300 library (host phase) against the reference hierarchy.

C/F labels and the sparsity patterns of A, P and R on every level are integer
work and must be identical; the values are also required to be bit-identical
because the library reproduces the reference's operation order.
"""
import numpy as np
import pytest

from fem_gb300 import lina, problems
from oracle import ref
from tests.conftest import golden_cases, load_golden, system_for


def _same(a, b):
    return (len(a[0]) == len(b[0]) and np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
            and np.array_equal(np.asarray(a[2]).view(np.int64), np.asarray(b[2]).view(np.int64)))


@pytest.mark.parametrize("name", golden_cases("hierarchy"))
def test_hierarchy_matches_golden(name):
    g = load_golden(name)
    s = system_for(name)
    amg = lina.AMG.from_system(s, host_only=True, depth=int(g["depth"]), coarsening=int(g["coarsening"]))
    assert amg.sizes() == [int(v) for v in g["sizes"]]
    for l in range(int(g["depth"])):
        L = amg.level(l)
        assert _same(L.A, (g[f"L{l}_A_ptr"], g[f"L{l}_A_col"], g[f"L{l}_A_val"])), f"A level {l}"
        if l > 0:
            assert np.array_equal(L.labels, g[f"L{l}_labels"]), f"labels level {l}"
            assert _same(L.P, (g[f"L{l}_P_ptr"], g[f"L{l}_P_col"], g[f"L{l}_P_val"])), f"P level {l}"
            assert _same(L.R, (g[f"L{l}_R_ptr"], g[f"L{l}_R_col"], g[f"L{l}_R_val"])), f"R level {l}"
            assert np.array_equal(amg.colours(l), g[f"L{l}_colour"]), f"colouring level {l}"


LIVE = [
    ("poisson65_aggr", lambda: problems.poisson_p1(65), 5, lina.AGGRESSIVE),
    ("poisson65_std", lambda: problems.poisson_p1(65), 5, lina.STANDARD),
    ("elast33_std", lambda: problems.elasticity_p1(33), 4, lina.STANDARD),
    ("elast33_aggr", lambda: problems.elasticity_p1(33), 4, lina.AGGRESSIVE),
    ("elast33_young", lambda: problems.elasticity_p1(
        33, young=210.0 * np.exp(0.5 * np.random.default_rng(3).standard_normal((2, 32 * 32)))), 4, lina.STANDARD),
    # larger cases: many ties in the coarsening queue, and an unstructured high-contrast system
    ("elast129_std", lambda: problems.elasticity_p1(129), 6, lina.STANDARD),
    ("elast129_aggr", lambda: problems.elasticity_p1(129), 6, lina.AGGRESSIVE),
    ("batch_elast20k", lambda: problems.batch_system("elasticity", 20000, 7), 5, lina.STANDARD),
]


@pytest.mark.skipif(not ref.available(), reason="reference library not built here (needs the reference tree)")
@pytest.mark.parametrize("case", LIVE, ids=[c[0] for c in LIVE])
def test_hierarchy_matches_live_reference(case):
    _, factory, depth, coarsening = case
    s = factory()
    R = ref.hierarchy(s, depth, 2, 2, coarsening)
    G = lina.AMG.from_system(s, host_only=True, depth=depth, coarsening=coarsening)
    assert G.sizes() == R.sizes()
    for l in range(depth):
        a, b = R.level(l), G.level(l)
        assert _same(a.A, b.A), f"A level {l}"
        if l > 0:
            assert np.array_equal(a.labels, b.labels)
            assert _same(a.P, b.P) and _same(a.R, b.R)
            nc, col = ref.greedy_colouring(len(a.A[0]) - 1, *a.A)
            assert np.array_equal(G.colours(l), col)


@pytest.mark.skipif(not ref.available(), reason="reference library not built here")
def test_recompute_matches_reference():
    s = problems.elasticity_p1(17)
    s2 = problems.elasticity_p1(17, young=210.0 * np.exp(0.3 * np.random.default_rng(5).standard_normal((2, 256))))
    R = ref.RefAMG(s, 3, 2, 2, ref.STANDARD)
    M = ref.RefMatrix.from_csr(s2.n, s2.indptr, s2.indices, s2.data)
    ref.lib().rs_amg_recompute(R.ptr, M.ptr)
    G = lina.AMG.from_system(s, host_only=True, depth=3, coarsening=lina.STANDARD)
    # host-only handles support recompute of the host hierarchy as well
    G.recompute(s2.indptr, s2.indices, s2.data)
    for l in range(3):
        assert _same(R.level(l).A, G.level(l).A), f"A level {l}"


def test_setup_rejects_bad_csr():
    with pytest.raises(lina.LinaError):
        lina.AMG(3, np.array([0, 1, 2, 5]), np.array([0, 1, 2, 1, 0]), np.ones(5), host_only=True)
