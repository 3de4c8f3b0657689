"""Cluster-fused V-cycle steps: multicolour SOR (lina_gpu_set_fused_rows) and damped Jacobi
(lina_gpu_set_fused_jacobi_entries).

The fused launch computes every row as the per-colour launches do, so V-cycles, FMG passes and
whole PCG solves must agree bit for bit with the fusion on and off; the reference parity of the
multicolour-SOR V-cycle itself is checked in test_gpu_solve.
"""
import os

import numpy as np
import pytest

from fem_gb300 import lina, problems
from tests.conftest import ROOT, golden_cases, gpu_available, load_golden, system_for

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA device")]

BATCH = os.path.join(ROOT, "tests", "golden", "batch_small.npz")


def systems():
    out = []
    for name in golden_cases("hierarchy"):
        g = load_golden(name)
        out.append((name, system_for(name), int(g["depth"]), int(g["coarsening"])))
    with np.load(BATCH) as z:
        for name in ("belast4k", "bpoisson12k"):
            s = problems.CSRSystem(len(z[f"{name}_ptr"]) - 1, z[f"{name}_ptr"], z[f"{name}_col"], z[f"{name}_val"],
                                   z[f"{name}_b"], dof=int(z[f"{name}_dof"]))
            out.append((name, s, int(z[f"{name}_depth"]), lina.STANDARD))
    return out


CASES = systems()


def build(s, depth, coarsening, precision, fused_rows):
    lina.set_fused_rows(fused_rows)
    try:
        return lina.AMG.from_system(s, depth=depth, coarsening=coarsening, smoother=lina.SMOOTHER_MC_SOR, omega=1.0,
                                    precision=precision)
    finally:
        lina.set_fused_rows(lina.FUSED_ROWS_DEFAULT)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_vcycle_and_fmg_identical(case):
    name, s, depth, coarsening = case
    on = build(s, depth, coarsening, lina.PREC_FP64, lina.FUSED_ROWS_DEFAULT)
    off = build(s, depth, coarsening, lina.PREC_FP64, 0)
    r = np.random.default_rng(1).uniform(-1, 1, s.n)
    lina.set_fused_rows(lina.FUSED_ROWS_DEFAULT)
    z_on = on.vcycle(r)
    x_on, _ = on.fmg(s.b)
    lina.set_fused_rows(0)
    try:
        z_off = off.vcycle(r)
        x_off, _ = off.fmg(s.b)
    finally:
        lina.set_fused_rows(lina.FUSED_ROWS_DEFAULT)
    assert np.array_equal(z_on, z_off)
    assert np.array_equal(x_on, x_off)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("precision", [lina.PREC_FP64, lina.PREC_MIXED])
def test_pcg_identical(case, precision):
    name, s, depth, coarsening = case
    res = []
    for rows in (lina.FUSED_ROWS_DEFAULT, 0):
        amg = build(s, depth, coarsening, precision, rows)
        lina.set_fused_rows(rows)
        try:
            res.append(amg.pcg(s.b, tol=1e-8, max_iter=500, stop=lina.STOP_RELATIVE))
        finally:
            lina.set_fused_rows(lina.FUSED_ROWS_DEFAULT)
    (x1, i1), (x2, i2) = res
    assert i1.status == 0 and i1.iterations == i2.iterations
    assert np.array_equal(x1, x2)


def test_fused_rows_validation():
    with pytest.raises(lina.LinaError):
        lina.set_fused_rows(-1)


# ---------------------------------------------------------------- damped Jacobi (two copies of x)
def build_jacobi(s, depth, coarsening, precision, entries):
    lina.set_fused_jacobi_entries(entries)
    try:
        return lina.AMG.from_system(s, depth=depth, coarsening=coarsening, smoother=lina.SMOOTHER_JACOBI,
                                    omega=0.6, precision=precision)
    finally:
        lina.set_fused_jacobi_entries(lina.FUSED_JACOBI_ENTRIES_DEFAULT)


def _with_entries(entries, f):
    lina.set_fused_jacobi_entries(entries)
    try:
        return f()
    finally:
        lina.set_fused_jacobi_entries(lina.FUSED_JACOBI_ENTRIES_DEFAULT)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("precision", [lina.PREC_FP64, lina.PREC_MIXED])
def test_jacobi_vcycle_and_pcg_identical(case, precision):
    """Every level of these hierarchies fits the fused step (entries cap raised): V-cycles and whole
    solves with the fused damped-Jacobi steps equal the separate launches bit for bit."""
    name, s, depth, coarsening = case
    big = 1 << 40
    on = build_jacobi(s, depth, coarsening, precision, big)
    off = build_jacobi(s, depth, coarsening, precision, 0)
    r = np.random.default_rng(2).uniform(-1, 1, s.n)
    z_on = _with_entries(big, lambda: on.vcycle(r))
    z_off = _with_entries(0, lambda: off.vcycle(r))
    assert np.array_equal(z_on, z_off)
    x1, i1 = _with_entries(big, lambda: on.pcg(s.b, tol=1e-8, max_iter=500, stop=lina.STOP_RELATIVE))
    x2, i2 = _with_entries(0, lambda: off.pcg(s.b, tol=1e-8, max_iter=500, stop=lina.STOP_RELATIVE))
    assert i1.status == 0 and i1.iterations == i2.iterations
    assert np.array_equal(x1, x2)


def test_jacobi_fused_levels_of_an_elasticity_hierarchy():
    """A 257 x 257 elasticity hierarchy with the levels of up to 400,000 entries fused: a mixed solve
    equals the unfused one bit for bit."""
    s = problems.elasticity_p1(257)
    res = []
    for entries in (400000, 0):
        amg = build_jacobi(s, 7, lina.STANDARD, lina.PREC_MIXED, entries)
        res.append(_with_entries(entries, lambda: amg.pcg(s.b, tol=1e-8, max_iter=500)))
    (x1, i1), (x2, i2) = res
    assert i1.status == 0 and i1.iterations == i2.iterations
    assert np.array_equal(x1, x2)


def _symmetric_scale(s, seed, amount):
    rows = np.repeat(np.arange(s.n), np.diff(s.indptr))
    key = np.minimum(rows, s.indices) * s.n + np.maximum(rows, s.indices)
    _, inv = np.unique(key, return_inverse=True)
    return s.data * (1.0 + amount * np.random.default_rng(seed).random(inv.max() + 1)[inv])


@pytest.mark.parametrize("name", ["poisson33_aggr", "elast17_std"])
@pytest.mark.parametrize("precision", [lina.PREC_FP64, lina.PREC_MIXED])
def test_staged_images_follow_value_changes(name, precision):
    """The staged fused steps sweep from copies of the levels' entries and of omega / a_ii.  After a
    recompute that rebuilds the hierarchy, one that only moves values, an update of the finest values
    and a new omega, V-cycles with the fusion on still equal those with it off."""
    g = load_golden(name)
    s = system_for(name)
    depth, coarsening = int(g["depth"]), int(g["coarsening"])
    on = build(s, depth, coarsening, precision, lina.FUSED_ROWS_DEFAULT)
    off = build(s, depth, coarsening, precision, 0)
    r = np.random.default_rng(2).uniform(-1, 1, s.n)
    changes = [
        lambda a: a.recompute(s.indptr, s.indices, _symmetric_scale(s, 4, 0.2)),
        lambda a: a.recompute(s.indptr, s.indices, _symmetric_scale(s, 5, 0.3)),
        lambda a: a.update_values(_symmetric_scale(s, 6, 0.1)),
        lambda a: a.set_smoother(lina.SMOOTHER_MC_SOR, 1.3, precision),
    ]
    for k, change in enumerate(changes):
        change(on)
        change(off)
        z_on = on.vcycle(r)
        lina.set_fused_rows(0)
        try:
            z_off = off.vcycle(r)
        finally:
            lina.set_fused_rows(lina.FUSED_ROWS_DEFAULT)
        assert np.array_equal(z_on, z_off), f"after change {k}"
    # and the new values took effect: a hierarchy built on them from the start gives the same V-cycle
    fresh = build(s, depth, coarsening, precision, lina.FUSED_ROWS_DEFAULT)
    fresh.recompute(s.indptr, s.indices, _symmetric_scale(s, 5, 0.3))
    fresh.update_values(_symmetric_scale(s, 6, 0.1))
    fresh.set_smoother(lina.SMOOTHER_MC_SOR, 1.3, precision)
    assert np.array_equal(fresh.vcycle(r), on.vcycle(r))
