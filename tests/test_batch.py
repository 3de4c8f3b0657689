"""Batched AMG-PCG over independent unstructured systems (lina_gpu_batch_*).

Oracle: the reference's pcg (damped-Jacobi V-cycle, its own stopping rule) and accurate solutions
on small systems of the batched workload (tests/golden/batch_small.npz, made by
tests/golden/make_golden.py); and, for every system of a batch, the library's own single-system
solve, which the batch must reproduce bit for bit (same kernels, one branch per system).
"""
import ctypes as C
import os

import numpy as np
import pytest
import scipy.sparse as sp

from fem_gb300 import lina, problems
from tests.conftest import ROOT, gpu_available

GOLDEN = os.path.join(ROOT, "tests", "golden", "batch_small.npz")
NAMES = ["bpoisson3k", "belast4k", "bpoisson12k"]
CASES = {"bpoisson3k": ("poisson", 3000, 11), "belast4k": ("elasticity", 4000, 12),
         "bpoisson12k": ("poisson", 12000, 13)}


def load():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


def stored_system(g, name):
    return problems.CSRSystem(len(g[f"{name}_ptr"]) - 1, g[f"{name}_ptr"], g[f"{name}_col"], g[f"{name}_val"],
                              g[f"{name}_b"], dof=int(g[f"{name}_dof"]))


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("name", NAMES)
def test_golden_inputs_regenerate(name):
    g = load()
    s = problems.batch_system(*CASES[name])
    assert np.array_equal(s.indptr, g[f"{name}_ptr"]) and np.array_equal(s.indices, g[f"{name}_col"])
    np.testing.assert_allclose(s.data, g[f"{name}_val"], rtol=1e-12, atol=0)
    np.testing.assert_allclose(s.b, g[f"{name}_b"], rtol=1e-12, atol=1e-300)
    assert int(g[f"{name}_depth"]) == problems.batch_depth(s.n)


@pytest.mark.parametrize("name", NAMES)
def test_reference_solutions_solve_the_systems(name):
    """Pins the oracle: the accurate reference solution meets 1e-11, and the reference's 1e-8 run
    is within 1e-6 of it."""
    g = load()
    s = stored_system(g, name)
    A = sp.csr_matrix((s.data, s.indices, s.indptr), shape=(s.n, s.n))
    assert abs(A - A.T).max() == 0.0
    xt = g[f"{name}_x_tight"]
    assert np.linalg.norm(s.b - A @ xt) / np.linalg.norm(s.b) <= 1e-11
    assert rel(g[f"{name}_x"], xt) <= 1e-6


def test_batch_plan():
    plan = problems.batch_plan()
    assert len(plan) == 96 and plan == problems.batch_plan()
    assert [k for k, _, _ in plan].count("poisson") == 48
    d = np.array([n for _, n, _ in plan])
    assert d.min() >= 10_000 and d.max() <= 500_000
    assert 8e6 <= d.sum() <= 20e6  # log-uniform on [10k, 500k]: mean about 125k


@pytest.mark.parametrize("nodes", [162 ** 2, 55 ** 2, 100 ** 2])
def test_batch_system_boundary_conditions(nodes):
    """Every edge node is found (k x k lattices whose spacing does not divide 1 exactly included):
    elasticity fixes both components on the bottom edge and u_y on the top edge, Poisson the whole
    boundary; the right-hand sides are not zero."""
    k = int(round(np.sqrt(nodes)))
    e = problems.batch_system("elasticity", 2 * nodes, seed=4)
    ident = np.diff(e.indptr) == 1
    assert ident.sum() == 3 * k and np.linalg.norm(e.b) > 0
    assert np.allclose(e.b[k * k:][ident[k * k:]], np.r_[np.zeros(k), np.full(k, 1e-3)])
    p = problems.batch_system("poisson", nodes, seed=4)
    assert (np.diff(p.indptr) == 1).sum() == 4 * (k - 1) and np.linalg.norm(p.b) > 0


def test_batch_create_rejects_empty():
    h = C.c_void_p()
    assert lina.lib().lina_gpu_batch_create(0, None, lina.STOP_RELATIVE, C.byref(h)) == lina.EINVAL
    assert lina.lib().lina_gpu_batch_solve(None, None, None, 1e-8, 10, 0, None) == lina.EINVAL


gpu = pytest.mark.skipif(not gpu_available(), reason="no CUDA device")


def _hierarchies(systems, precision, depths=None, smoother=lina.SMOOTHER_JACOBI, omega=0.6, matrix_tol=0.1):
    return [lina.AMG.from_system(s, depth=depths[i] if depths else problems.batch_depth(s.n),
                                 coarsening=lina.STANDARD, smoother=smoother, omega=omega, precision=precision,
                                 matrix_tol=matrix_tol) for i, s in enumerate(systems)]


@pytest.mark.gpu
@gpu
def test_batch_fp64_matches_reference():
    """FP64 batch with the reference's stopping rule: iterations within 10 % of the reference's pcg
    (at least one), solutions within 1e-7 of its."""
    g = load()
    systems = [stored_system(g, n) for n in NAMES]
    amgs = _hierarchies(systems, lina.PREC_FP64, [int(g[f"{n}_depth"]) for n in NAMES])
    batch = lina.Batch(amgs, stop=lina.STOP_REFERENCE)
    xs, infos = batch.solve([s.b for s in systems], tol=1e-8, max_iter=500)
    for name, x, info in zip(NAMES, xs, infos):
        assert info.status == 0, name
        it_ref = int(g[f"{name}_it"])
        assert abs(info.iterations - it_ref) <= max(1, int(np.ceil(0.1 * it_ref))), (name, info.iterations, it_ref)
        assert rel(x, g[f"{name}_x"]) <= 1e-7, name


@pytest.mark.gpu
@gpu
@pytest.mark.parametrize("precision", [lina.PREC_FP64, lina.PREC_MIXED])
@pytest.mark.parametrize("stop", [lina.STOP_REFERENCE, lina.STOP_RELATIVE])
def test_batch_reproduces_single_solves(precision, stop):
    """Every branch of the batch gives the bits and the iteration count of the single-system solve."""
    g = load()
    systems = [stored_system(g, n) for n in NAMES]
    amgs = _hierarchies(systems, precision, [int(g[f"{n}_depth"]) for n in NAMES])
    singles = [a.pcg(s.b, tol=1e-8, max_iter=500, stop=stop) for a, s in zip(amgs, systems)]
    batch = lina.Batch(amgs, stop=stop)
    xs, infos = batch.solve([s.b for s in systems], tol=1e-8, max_iter=500)
    for (xs1, is1), x, info in zip(singles, xs, infos):
        assert info.status == 0 and info.iterations == is1.iterations
        assert np.array_equal(x, xs1)
        assert info.true_rel_residual == pytest.approx(is1.true_rel_residual, rel=1e-12)


@pytest.mark.gpu
@gpu
def test_batch_mixed_precision_accuracy():
    """Mixed precision to 1e-8 (relative rule): the true residual meets it and the solution error
    against the accurate reference solution is at most 1e-7, or 10x the FP64 path's."""
    g = load()
    systems = [stored_system(g, n) for n in NAMES]
    depths = [int(g[f"{n}_depth"]) for n in NAMES]
    x64, _ = lina.Batch(_hierarchies(systems, lina.PREC_FP64, depths)).solve([s.b for s in systems])
    xs, infos = lina.Batch(_hierarchies(systems, lina.PREC_MIXED, depths)).solve([s.b for s in systems])
    for name, x, xd, info in zip(NAMES, xs, x64, infos):
        assert info.status == 0 and info.true_rel_residual <= 1e-8
        xt = g[f"{name}_x_tight"]
        assert rel(x, xt) <= max(1e-7, 10 * rel(xd, xt)), name


@pytest.mark.gpu
@gpu
def test_batch_zero_rhs_repeat_and_device_pointers():
    g = load()
    systems = [stored_system(g, n) for n in NAMES]
    amgs = _hierarchies(systems, lina.PREC_MIXED, [int(g[f"{n}_depth"]) for n in NAMES])
    batch = lina.Batch(amgs)
    bs = [s.b for s in systems]
    bs[1] = np.zeros(systems[1].n)
    xs, infos = batch.solve(bs)
    assert infos[1].iterations == 0 and infos[1].status == 0 and not xs[1].any()
    # a second launch of the same graph with other right-hand sides
    rng = np.random.default_rng(5)
    bs2 = [rng.uniform(-1, 1, s.n) for s in systems]
    xs2, infos2 = batch.solve(bs2)
    for a, b, x, info in zip(amgs, bs2, xs2, infos2):
        x1, i1 = a.pcg(b, tol=1e-8, max_iter=1000)
        assert info.status == 0 and info.iterations == i1.iterations and np.array_equal(x, x1)
    # device pointers
    bd = [lina.DeviceArray.from_host(b) for b in bs2]
    xd, infod = batch.solve(bd, device=True)
    for x, xh in zip(xd, xs2):
        assert np.array_equal(x.to_host(), xh)


@pytest.mark.gpu
@gpu
def test_batch_rejects_duplicates():
    g = load()
    s = stored_system(g, NAMES[0])
    a = _hierarchies([s], lina.PREC_MIXED, [int(g[f"{NAMES[0]}_depth"])])[0]
    with pytest.raises(lina.LinaError):
        lina.Batch([a, a])


@pytest.mark.gpu
@gpu
def test_batch_of_generated_systems():
    """Twelve systems of the workload's generator (10k-80k dofs, both kinds) with the workload's
    hierarchy settings (multicolour SOR, matrix_tol 0.3: the cluster-fused level steps run inside
    the batch graph): each branch equals its single-system solve and reaches 1e-8."""
    plan = problems.batch_plan(count=12, seed=3, lo=10_000, hi=80_000)
    systems = [problems.batch_system(*p) for p in plan]
    amgs = _hierarchies(systems, lina.PREC_MIXED, smoother=lina.SMOOTHER_MC_SOR, omega=1.0, matrix_tol=0.3)
    batch = lina.Batch(amgs)
    xs, infos = batch.solve([s.b for s in systems], tol=1e-8, max_iter=1000)
    for a, s, x, info in zip(amgs, systems, xs, infos):
        assert info.status == 0 and info.true_rel_residual <= 1e-8
        x1, i1 = a.pcg(s.b, tol=1e-8, max_iter=1000)
        assert info.iterations == i1.iterations and np.array_equal(x, x1)
