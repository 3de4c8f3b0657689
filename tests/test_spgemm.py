"""Sparse matrix product with the reference's sparse_product semantics (L4).

Oracle: the reference's own sparse_product on seeded rectangular factors with explicit zeros,
empty rows and an exactly cancelling row (tests/golden/spgemm.npz), and the reference's Galerkin
coarse matrices of the golden hierarchies.  The bar is bit-identity (patterns and values).
"""
import os

import numpy as np
import pytest

from fem_gb300 import lina
from oracle import spgemm as ospgemm
from tests.conftest import ROOT, golden_cases, load_golden, system_for

GOLDEN = os.path.join(ROOT, "tests", "golden", "spgemm.npz")


def load():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


def same(x, y):
    return all(np.array_equal(np.asarray(p), np.asarray(q)) for p, q in zip(x, y))


def level_csr(g, l, name):
    return (g[f"L{l}_{name}_ptr"], g[f"L{l}_{name}_col"], g[f"L{l}_{name}_val"])


def test_restatement_matches_reference_product():
    """Pins the oracle restatement against the reference's sparse_product."""
    g = load()
    c = ospgemm.sparse_product((g["a_ptr"], g["a_col"], g["a_val"]), (g["b_ptr"], g["b_col"], g["b_val"]))
    assert same(c, (g["c_ptr"], g["c_col"], g["c_val"]))
    # the cancelling row and the empty rows end as (i, 0.0)
    for i in (5, 7, 17, 123):
        assert list(c[1][c[0][i]:c[0][i + 1]]) == [i] and c[2][c[0][i]] == 0.0


@pytest.mark.parametrize("name", golden_cases())
def test_restatement_gives_reference_coarse_matrices(name):
    """R (A P) with square_matrix_clean from the oracle equals the reference's coarse matrices."""
    g = load_golden(name)
    depth = int(g["depth"])
    for l in range(depth - 1, 0, -1):
        if f"L{l}_P_ptr" not in g.files:
            continue
        A, P, R = level_csr(g, l, "A"), level_csr(g, l, "P"), level_csr(g, l, "R")
        nc = len(R[0]) - 1
        rap = ospgemm.square_clean(ospgemm.sparse_product(R, ospgemm.sparse_product(A, P)), nc)
        assert same(rap, level_csr(g, l - 1, "A")), f"level {l - 1}"


@pytest.mark.gpu
def test_gpu_product_is_bit_identical_to_reference():
    g = load()
    c = lina.spgemm((g["a_ptr"], g["a_col"], g["a_val"]), (g["b_ptr"], g["b_col"], g["b_val"]), 150)
    assert same(c, (g["c_ptr"], g["c_col"], g["c_val"]))


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_cases())
def test_gpu_galerkin_products_match_reference(name):
    g = load_golden(name)
    depth = int(g["depth"])
    for l in range(depth - 1, 0, -1):
        A, P, R = level_csr(g, l, "A"), level_csr(g, l, "P"), level_csr(g, l, "R")
        nc = len(R[0]) - 1
        ap = lina.spgemm(A, P, nc)
        assert same(ap, ospgemm.sparse_product(A, P))
        rap = lina.spgemm(R, ap, nc)
        assert same(ospgemm.square_clean(rap, nc), level_csr(g, l - 1, "A")), f"level {l - 1}"


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_cases())
def test_device_hierarchy_setup_and_recompute_match_host(name, capfd):
    """A device hierarchy forms its Galerkin products on the GPU; every level equals the reference's
    (golden) and, after a recompute with a new matrix, the host-only hierarchy's."""
    g = load_golden(name)
    s = system_for(name)
    depth, coarsening = int(g["depth"]), int(g["coarsening"])
    dev = lina.AMG.from_system(s, depth=depth, coarsening=coarsening)
    for l in range(depth):
        assert same(dev.level(l).A, level_csr(g, l, "A")), f"level {l}"
    # a new matrix on the same pattern, kept symmetric: entries (i, j) and (j, i) scaled alike
    rows = np.repeat(np.arange(s.n), np.diff(s.indptr))
    key = np.minimum(rows, s.indices) * s.n + np.maximum(rows, s.indices)
    _, inv = np.unique(key, return_inverse=True)
    scale = 1.0 + 0.2 * np.random.default_rng(4).random(inv.max() + 1)[inv]
    data2 = s.data * scale
    host = lina.AMG.from_system(s, depth=depth, coarsening=coarsening, host_only=True)
    dev.recompute(s.indptr, s.indices, data2)
    host.recompute(s.indptr, s.indices, data2)
    for l in range(depth):
        assert same(dev.level(l).A, host.level(l).A), f"level {l} after recompute"
    # the products ran on the GPU (the library says so on stderr when it falls back to the host)
    assert "Galerkin product on the host" not in capfd.readouterr().err


def _symmetric_scale(s, seed, amount):
    rows = np.repeat(np.arange(s.n), np.diff(s.indptr))
    key = np.minimum(rows, s.indices) * s.n + np.maximum(rows, s.indices)
    _, inv = np.unique(key, return_inverse=True)
    return s.data * (1.0 + amount * np.random.default_rng(seed).random(inv.max() + 1)[inv])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["poisson33_std", "elast17_std"])
@pytest.mark.parametrize("precision", [lina.PREC_FP64, lina.PREC_MIXED])
def test_repeated_recompute_updates_values_in_place(name, precision):
    """The first recompute rebuilds the device hierarchy and keeps where every entry sits in its layouts;
    later recomputes on the same patterns only move values.  A hierarchy recomputed twice (the second time
    in place) solves exactly as one recomputed once, with a rebuild, to the same matrix; and the captured
    solve graph of the first keeps working."""
    g = load_golden(name)
    s = system_for(name)
    depth, coarsening = int(g["depth"]), int(g["coarsening"])
    opts = dict(depth=depth, coarsening=coarsening, precision=precision)
    v2, v3 = _symmetric_scale(s, 4, 0.2), _symmetric_scale(s, 5, 0.3)
    twice = lina.AMG.from_system(s, **opts)
    twice.pcg(s.b, tol=1e-8, max_iter=500)  # a captured graph before the recomputes
    twice.recompute(s.indptr, s.indices, v2)
    twice.pcg(s.b, tol=1e-8, max_iter=500)
    twice.recompute(s.indptr, s.indices, v3)
    once = lina.AMG.from_system(s, **opts)
    once.recompute(s.indptr, s.indices, v3)
    for l in range(depth):
        assert same(twice.level(l).A, once.level(l).A), f"level {l}"
    r = np.random.default_rng(6).uniform(-1, 1, s.n)
    assert np.array_equal(twice.vcycle(r), once.vcycle(r))
    x1, i1 = twice.pcg(s.b, tol=1e-8, max_iter=500)
    x2, i2 = once.pcg(s.b, tol=1e-8, max_iter=500)
    assert i1.status == 0 and i1.iterations == i2.iterations
    assert np.array_equal(x1, x2)
