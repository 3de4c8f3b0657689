"""P1 assembly on the GPU (lina_gpu_p1_*): the scalar Laplacian and plane-strain elasticity with
per-element coefficients, straight into CSR.

Oracle: the reference's own assembly, FEM2D/FEM2D.c set_matrix_Aij_11_2D with its element integrals
(tests/golden/p1_fem2d.npz, made by tests/golden/make_golden.py from the reference built by
`make -C oracle fem2d`, and live where that library is built): the same pattern, values to rounding
(bit for bit for the Laplacian on structured grids); the numpy element assembly of
fem_gb300.problems; and the library's host assembly bit for bit on the device.
"""
import os

import numpy as np
import pytest
import scipy.sparse as sp

from fem_gb300 import lina, problems
from oracle import ref
from tests.conftest import ROOT, gpu_available

P1_GOLDEN = os.path.join(ROOT, "tests", "golden", "p1_fem2d.npz")
# max |difference| / max |entry| against the reference's assembly: the entries of a node's fan of
# triangles are summed in another order on irregular meshes (observed up to 5e-15)
P1_TOL = 1e-13
P1_KINDS = {"laplace": lina.P1_LAPLACE, "elastic": lina.P1_ELASTIC}


def _p1_golden():
    with np.load(P1_GOLDEN) as z:
        return {k: z[k] for k in z.files}


def _coef(kind, n_elems):
    """coefficient 1 (Laplacian), Young's modulus 210 (elasticity, nu 0.3), as in the fixture"""
    return np.ones(n_elems) if kind == "laplace" else np.full(n_elems, 210.0)


def _check_against(got, want, bitwise=False):
    ptr, col, val = got
    wp, wc, wv = want
    assert np.array_equal(ptr, wp) and np.array_equal(col, wc), "pattern differs from the reference's"
    err = np.abs(val - wv).max() / np.abs(wv).max()
    assert err <= P1_TOL, err
    if bitwise:
        assert np.array_equal(val, wv)


@pytest.mark.parametrize("mesh", ["grid17", "delaunay600"])
@pytest.mark.parametrize("kind", ["laplace", "elastic"])
def test_host_assembly_matches_reference_fem2d(mesh, kind):
    g = _p1_golden()
    xy, tri = g[f"{mesh}_xy"], g[f"{mesh}_tri"]
    ptr, col, val, _ = lina.p1_assemble_host(P1_KINDS[kind], xy, tri, _coef(kind, len(tri)), nu=0.3)
    _check_against((ptr, col, val), (g[f"{mesh}_{kind}_ptr"], g[f"{mesh}_{kind}_col"], g[f"{mesh}_{kind}_val"]),
                   bitwise=(mesh == "grid17" and kind == "laplace"))


@pytest.mark.skipif(not ref.fem2d_available(), reason="reference FEM2D not built here (needs the reference tree)")
@pytest.mark.parametrize("mesh", ["grid65", "delaunay5000"])
@pytest.mark.parametrize("kind", ["laplace", "elastic"])
def test_host_assembly_matches_live_reference_fem2d(mesh, kind):
    xy, tri = problems.elastic_mesh(65)[:2] if mesh == "grid65" else problems.delaunay_mesh(5000, 21)
    ptr, col, val, _ = lina.p1_assemble_host(P1_KINDS[kind], xy, tri, _coef(kind, len(tri)), nu=0.3)
    _check_against((ptr, col, val), ref.p1_assemble(xy, tri, kind, 210.0, 0.3),
                   bitwise=(mesh == "grid65" and kind == "laplace"))


def csr(ptr, col, val, n):
    return sp.csr_matrix((val, col, ptr), shape=(n, n))


def poisson_case(dofs, seed):
    """the inputs of problems.batch_system('poisson', dofs, seed)"""
    xy, tri = problems.delaunay_mesh(dofs, seed)
    kappa = np.exp(1.5 * np.random.default_rng(seed).standard_normal(len(tri)))
    on_edge = (xy[:, 0] == 0.0) | (xy[:, 0] == 1.0) | (xy[:, 1] == 0.0) | (xy[:, 1] == 1.0)
    fixed = np.nonzero(on_edge)[0]
    return xy, tri, kappa, fixed, np.zeros(len(fixed))


def elastic_case(dofs, seed):
    """the inputs of problems.batch_system('elasticity', dofs, seed)"""
    xy, tri = problems.delaunay_mesh(max(dofs // 2, 9), seed)
    E = 210.0 * np.exp(1.5 * np.random.default_rng(seed).standard_normal(len(tri)))
    nn = len(xy)
    bottom = np.nonzero(xy[:, 1] == 0.0)[0]
    top = np.nonzero(xy[:, 1] == 1.0)[0]
    fixed = np.concatenate([bottom, nn + bottom, nn + top])
    val = np.concatenate([np.zeros(2 * len(bottom)), np.full(len(top), 1e-3)])
    o = np.argsort(fixed)
    return xy, tri, E, fixed[o], val[o]


@pytest.mark.parametrize("dofs,seed", [(3000, 11), (12000, 13)])
def test_laplace_matches_numpy_assembly(dofs, seed):
    xy, tri, kappa, fd, fv = poisson_case(dofs, seed)
    ptr, col, val, b = lina.p1_assemble_host(lina.P1_LAPLACE, xy, tri, kappa, 0.0, fd, fv)
    s = problems.batch_system("poisson", dofs, seed)
    A, R = csr(ptr, col, val, s.n), csr(s.indptr, s.indices, s.data, s.n)
    assert abs(A - A.T).max() == 0.0
    assert abs(A - R).max() <= 1e-12 * abs(R).max()
    assert not b.any()  # homogeneous conditions: nothing lifted


@pytest.mark.parametrize("dofs,seed", [(4000, 12), (20000, 7)])
def test_elasticity_matches_numpy_assembly(dofs, seed):
    xy, tri, E, fd, fv = elastic_case(dofs, seed)
    ptr, col, val, b = lina.p1_assemble_host(lina.P1_ELASTIC, xy, tri, E, 0.3, fd, fv)
    s = problems.batch_system("elasticity", dofs, seed)
    A, R = csr(ptr, col, val, s.n), csr(s.indptr, s.indices, s.data, s.n)
    assert abs(A - R).max() <= 1e-12 * abs(R).max()
    assert np.abs(b - s.b).max() <= 1e-12 * np.abs(s.b).max()


def test_structured_laplace_pattern_and_values():
    """On the structured grid the pattern is poisson_p1's 7-point stencil, explicit zeros included."""
    m = 33
    xy, tri, _, _ = problems.elastic_mesh(m)
    r = np.arange(m * m) // m
    c = np.arange(m * m) % m
    fixed = np.nonzero((r == 0) | (r == m - 1) | (c == 0) | (c == m - 1))[0]
    ptr, col, val, _ = lina.p1_assemble_host(lina.P1_LAPLACE, xy, tri, np.ones(len(tri)), 0.0, fixed,
                                             np.zeros(len(fixed)))
    s = problems.poisson_p1(m, seed=0)
    assert np.array_equal(ptr, s.indptr) and np.array_equal(col, s.indices)
    assert np.abs(val - s.data).max() <= 1e-13 * np.abs(s.data).max()


def test_invalid_problems_are_rejected():
    xy, tri, kappa, fd, fv = poisson_case(3000, 11)
    with pytest.raises(lina.LinaError):
        lina.p1_assemble_host(3, xy, tri, kappa)
    with pytest.raises(lina.LinaError):
        lina.p1_assemble_host(lina.P1_ELASTIC, xy, tri, kappa, nu=0.5)
    bad = tri.copy()
    bad[0, 0] = len(xy)
    with pytest.raises(lina.LinaError):
        lina.p1_assemble_host(lina.P1_LAPLACE, xy, bad, kappa)
    with pytest.raises(lina.LinaError):
        lina.p1_assemble_host(lina.P1_LAPLACE, xy, tri, kappa, 0.0, np.r_[fd, fd[:1]], np.zeros(len(fd) + 1))


gpu = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="no CUDA device")]


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
@pytest.mark.parametrize("kind", [lina.P1_LAPLACE, lina.P1_ELASTIC])
def test_device_assembly_is_bit_identical_to_host(kind):
    xy, tri, coef, fd, fv = (poisson_case(12000, 13) if kind == lina.P1_LAPLACE else elastic_case(20000, 7))
    asm = lina.P1Assembly(kind, xy, tri, 0.3, fd, fv)
    for scale in (1.0, 1.7):
        asm.assemble(coef * scale)
        ptr, col, val, b = asm.system()
        hp, hc, hv, hb = lina.p1_assemble_host(kind, xy, tri, coef * scale, 0.3, fd, fv)
        assert np.array_equal(ptr, hp) and np.array_equal(col, hc)
        assert np.array_equal(val, hv) and np.array_equal(b, hb)


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
def test_device_assembly_feeds_the_solver():
    """Assemble on the GPU, build a hierarchy, then new coefficients: the device values go straight
    into the hierarchy (no host copy) and the solve meets the tolerance on the new matrix."""
    xy, tri, E, fd, fv = elastic_case(20000, 7)
    asm = lina.P1Assembly(lina.P1_ELASTIC, xy, tri, 0.3, fd, fv)
    asm.assemble(E)
    ptr, col, val, b = asm.system()
    amg = lina.AMG(len(b), ptr, col, val, dof=2, depth=problems.batch_depth(len(b)), smoother=lina.SMOOTHER_MC_SOR,
                   omega=1.0, matrix_tol=0.3, precision=lina.PREC_MIXED)
    E2 = E * np.exp(0.2 * np.random.default_rng(1).standard_normal(len(E)))
    asm.assemble(E2)
    vdev, _ = asm.device_values()
    amg.update_values(device_ptr=vdev)
    _, _, val2, b2 = asm.system()
    x, info = amg.pcg(b2, tol=1e-8, max_iter=1000)
    A2 = csr(ptr, col, val2, len(b2))
    assert info.status == 0
    assert np.linalg.norm(b2 - A2 @ x) / np.linalg.norm(b2) <= 1e-8


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="no CUDA device")
@pytest.mark.parametrize("mesh", ["grid17", "delaunay600"])
@pytest.mark.parametrize("kind", ["laplace", "elastic"])
def test_device_assembly_matches_reference_fem2d(mesh, kind):
    g = _p1_golden()
    xy, tri = g[f"{mesh}_xy"], g[f"{mesh}_tri"]
    asm = lina.P1Assembly(P1_KINDS[kind], xy, tri, 0.3)
    asm.assemble(_coef(kind, len(tri)))
    ptr, col, val, _ = asm.system()
    _check_against((ptr, col, val), (g[f"{mesh}_{kind}_ptr"], g[f"{mesh}_{kind}_col"], g[f"{mesh}_{kind}_val"]),
                   bitwise=(mesh == "grid17" and kind == "laplace"))
