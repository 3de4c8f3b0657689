"""Segmented batched AMG-PCG (lina_gpu_segbatch_*): independent systems solved as one block-diagonal
system, every level the concatenation of the systems' levels, each system with its own FCG scalars and
stopping test.

Oracle: the reference's pcg and accurate solutions of small systems of the batched workload
(tests/golden/batch_small.npz), and the library's single-system solves of every system.  Bars: each
system meets the relative rule on its true residual; its solution is within 1e-7 of the accurate one
(or 10x the single-system solve's own error); its iteration count is within max(2, 10 %) of the
single-system solve's (the segmented reductions add the same products in another order, and a
shallower system's padded levels return its coarse solution to rounding).
"""
import ctypes as C

import numpy as np
import pytest

from fem_gb300 import lina, problems
from tests.conftest import gpu_available
from tests.test_batch import NAMES, _hierarchies, load, rel, stored_system

gpu = pytest.mark.skipif(not gpu_available(), reason="no CUDA device")


def test_segbatch_rejects_invalid_arguments():
    h = C.c_void_p()
    assert lina.lib().lina_gpu_segbatch_create(0, None, C.byref(h)) == lina.EINVAL
    assert lina.lib().lina_gpu_segbatch_solve(None, None, None, 1e-8, 10, 0, None) == lina.EINVAL


def _close_iterations(a, b):
    return abs(a - b) <= max(2, int(np.ceil(0.1 * max(a, b))))


@pytest.mark.gpu
@gpu
@pytest.mark.parametrize("precision", [lina.PREC_FP64, lina.PREC_MIXED])
def test_segbatch_matches_single_solves_and_reference(precision):
    g = load()
    systems = [stored_system(g, n) for n in NAMES]
    amgs = _hierarchies(systems, precision, [int(g[f"{n}_depth"]) for n in NAMES])
    singles = [a.pcg(s.b, tol=1e-8, max_iter=500) for a, s in zip(amgs, systems)]
    seg = lina.SegmentedBatch(amgs)
    xs, infos = seg.solve([s.b for s in systems], tol=1e-8, max_iter=500)
    for name, s, (x1, i1), x, info in zip(NAMES, systems, singles, xs, infos):
        assert info.status == 0 and info.true_rel_residual <= 1e-8, (name, info.status, info.true_rel_residual)
        assert _close_iterations(info.iterations, i1.iterations), (name, info.iterations, i1.iterations)
        xt = g[f"{name}_x_tight"]
        assert rel(x, xt) <= max(1e-7, 10 * rel(x1, xt)), name


@pytest.mark.gpu
@gpu
def test_segbatch_generated_systems_of_different_depths():
    """Twelve systems of the workload's generator (10k-80k dofs, both kinds, hierarchies of different
    depths: the shallower ones are padded) with the workload's settings (multicolour SOR, matrix_tol
    0.3, mixed precision)."""
    plan = problems.batch_plan(count=12, seed=3, lo=10_000, hi=80_000)
    systems = [problems.batch_system(*p) for p in plan]
    amgs = _hierarchies(systems, lina.PREC_MIXED, smoother=lina.SMOOTHER_MC_SOR, omega=1.0, matrix_tol=0.3)
    depths = {a.depth for a in amgs}
    seg = lina.SegmentedBatch(amgs)
    rows, _ = seg.levels()
    assert len(rows) == max(depths) and rows[-1] == sum(s.n for s in systems)
    xs, infos = seg.solve([s.b for s in systems], tol=1e-8, max_iter=1000)
    for a, s, x, info in zip(amgs, systems, xs, infos):
        assert info.status == 0 and info.true_rel_residual <= 1e-8
        A = s.matvec(x)
        assert np.linalg.norm(s.b - A) / np.linalg.norm(s.b) <= 1e-8
        _, i1 = a.pcg(s.b, tol=1e-8, max_iter=1000)
        assert _close_iterations(info.iterations, i1.iterations), (info.iterations, i1.iterations)


@pytest.mark.gpu
@gpu
def test_segbatch_zero_rhs_repeat_and_device_pointers():
    g = load()
    systems = [stored_system(g, n) for n in NAMES]
    amgs = _hierarchies(systems, lina.PREC_MIXED, [int(g[f"{n}_depth"]) for n in NAMES])
    seg = lina.SegmentedBatch(amgs)
    bs = [s.b for s in systems]
    bs[1] = np.zeros(systems[1].n)
    xs, infos = seg.solve(bs)
    assert infos[1].iterations == 0 and infos[1].status == 0 and not xs[1].any()
    for i in (0, 2):
        assert infos[i].status == 0 and infos[i].true_rel_residual <= 1e-8
    rng = np.random.default_rng(5)
    bs2 = [rng.uniform(-1, 1, s.n) for s in systems]
    xs2, infos2 = seg.solve(bs2)
    assert all(i.status == 0 and i.true_rel_residual <= 1e-8 for i in infos2)
    bd = [lina.DeviceArray.from_host(b) for b in bs2]
    xd, _ = seg.solve(bd, device=True)
    for x, xh in zip(xd, xs2):
        assert np.array_equal(x.to_host(), xh)


@pytest.mark.gpu
@gpu
def test_segbatch_rejects_mixed_settings():
    g = load()
    s = [stored_system(g, n) for n in NAMES[:2]]
    a = _hierarchies(s[:1], lina.PREC_MIXED, [int(g[f"{NAMES[0]}_depth"])])
    b = _hierarchies(s[1:], lina.PREC_FP64, [int(g[f"{NAMES[1]}_depth"])])
    with pytest.raises(lina.LinaError):
        lina.SegmentedBatch(a + b)


@pytest.mark.gpu
@gpu
def test_segbatch_grouped_fused_steps_match_colour_launches():
    """The concatenated small levels run the cluster-fused multicolour-SOR step, one cluster per group of
    whole systems.  Its sweeps compute every row as the colour launches do; its residual and transfers
    sum each row in lane-group order, where the separate FP32 launches on levels of 20,000 rows or more
    read the quad layout (stored order), so the solves agree to rounding: the same iteration counts, both
    meeting the rule, solutions within 1e-6 of each other."""
    plan = problems.batch_plan(count=12, seed=3, lo=10_000, hi=80_000)
    systems = [problems.batch_system(*p) for p in plan]
    amgs = _hierarchies(systems, lina.PREC_MIXED, smoother=lina.SMOOTHER_MC_SOR, omega=1.0, matrix_tol=0.3)
    lina.set_fused_groups(True)
    try:
        on = lina.SegmentedBatch(amgs)
    finally:
        lina.set_fused_groups(False)
    lina.set_fused_rows(0)
    try:
        off = lina.SegmentedBatch(amgs)
    finally:
        lina.set_fused_rows(lina.FUSED_ROWS_DEFAULT)
    bs = [s.b for s in systems]
    x1, i1 = on.solve(bs, tol=1e-8, max_iter=1000)
    lina.set_fused_rows(0)
    try:
        x2, i2 = off.solve(bs, tol=1e-8, max_iter=1000)
    finally:
        lina.set_fused_rows(lina.FUSED_ROWS_DEFAULT)
    for a, b, p, q in zip(x1, x2, i1, i2):
        assert p.status == 0 and q.status == 0 and p.true_rel_residual <= 1e-8 and q.true_rel_residual <= 1e-8
        assert p.iterations == q.iterations
        assert rel(a, b) <= 1e-6


@pytest.mark.gpu
@gpu
@pytest.mark.parametrize("smoother,omega", [(lina.SMOOTHER_JACOBI, 0.6), (lina.SMOOTHER_MC_SOR, 1.0)])
def test_autotuned_hierarchy_solves(smoother, omega):
    """A hierarchy whose level layouts were measured at upload (lina_gpu_set_autotune) solves to the
    rule, with the iteration count of the rule-chosen layouts within 1."""
    s = problems.elasticity_p1(129)
    res = []
    for tune in (True, False):
        lina.set_autotune(tune)
        try:
            a = lina.AMG.from_system(s, depth=6, coarsening=lina.STANDARD, smoother=smoother, omega=omega,
                                     precision=lina.PREC_MIXED)
        finally:
            lina.set_autotune(False)
        res.append(a.pcg(s.b, tol=1e-8, max_iter=500))
    (x1, i1), (x2, i2) = res
    assert i1.status == 0 and i1.true_rel_residual <= 1e-8
    assert abs(i1.iterations - i2.iterations) <= 1
    assert rel(x1, x2) <= 1e-6
