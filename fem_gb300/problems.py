"""Seeded synthetic linear systems for the LinA solve path.

The reference assembles P1 (linear triangle) stiffness matrices in FEM2D
(``FEM2D/FEM2D.c:2783-2888`` for the element integrals, ``:5949-5968`` for the
row loop, ``insert_A_bbV_a`` at ``:4728`` for the scalar Laplacian) and feeds
them to LinA as row-list ``sparse_matrix`` objects.  This module restates that
element arithmetic on a structured grid so that the same CSR matrix and
right-hand side can be handed to the GPU library, to the CPU oracle and to the
reference itself.  It is harness code, not part of the solve path.

Grid: ``m x m`` nodes on the unit square, node ``k = r*m + c`` at
``(x, y) = (c*h, r*h)``, ``h = 1/(m-1)``.  Every cell is split along the
diagonal from ``(r, c)`` to ``(r+1, c+1)`` into a lower triangle
``[(r,c), (r,c+1), (r+1,c+1)]`` and an upper triangle
``[(r,c), (r+1,c+1), (r+1,c)]``.  Each node therefore couples to 7 nodes
(itself, the 4 axis neighbours and the two diagonal neighbours); the stored
pattern keeps all 7 even where the coupling is an exact zero (the Laplacian's
hypotenuse couplings), as the reference's assembly does.

Dirichlet conditions are imposed by symmetric elimination: known values are
lifted into the right-hand side, the constrained columns are removed from the
free rows and each constrained row becomes an identity row.  This keeps the
matrix symmetric so that CG applies (the reference's ``Set_dirichlet_BC`` in
``Crack/crack.c:6445-6459`` resets rows only, which would make it
nonsymmetric).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# stencil slots sorted by column offset: SW, S, W, C, E, N, NE  as (dr, dc)
_SLOTS = [(-1, -1), (-1, 0), (0, -1), (0, 0), (0, 1), (1, 0), (1, 1)]
_SLOT_OF = {o: s for s, o in enumerate(_SLOTS)}
# local (dr, dc) of the three vertices of the two triangles of a cell
_TRI_LOWER = [(0, 0), (0, 1), (1, 1)]
_TRI_UPPER = [(0, 0), (1, 1), (1, 0)]


@dataclass
class CSRSystem:
    """A square CSR matrix with int32 indices and FP64 values plus a RHS."""

    n: int
    indptr: np.ndarray
    indices: np.ndarray
    data: np.ndarray
    b: np.ndarray
    dof: int = 1          # number of unknowns per node, block ordering [u0..., u1...]
    meta: dict = field(default_factory=dict)

    @property
    def nnz(self) -> int:
        return int(self.indptr[-1])

    def matvec(self, x: np.ndarray) -> np.ndarray:
        """y = A x in FP64 (row-wise, columns in stored order)."""
        prod = self.data * x[self.indices]
        return np.add.reduceat(prod, self.indptr[:-1]) if self.nnz else np.zeros(self.n)


def _tri_geometry(tri, h):
    """b, c coefficient vectors and |area| of a triangle given local offsets."""
    xs = np.array([dc * h for (dr, dc) in tri])
    ys = np.array([dr * h for (dr, dc) in tri])
    b = np.array([ys[1] - ys[2], ys[2] - ys[0], ys[0] - ys[1]])
    c = np.array([xs[2] - xs[1], xs[0] - xs[2], xs[1] - xs[0]])
    area2 = xs[0] * (ys[1] - ys[2]) + xs[1] * (ys[2] - ys[0]) + xs[2] * (ys[0] - ys[1])
    return b, c, abs(area2) / 2.0


def _laplace_element(tri, h):
    """3x3 P1 stiffness  K_ab = (b_a b_b + c_a c_b) / (4|T|)."""
    b, c, area = _tri_geometry(tri, h)
    return (np.outer(b, b) + np.outer(c, c)) / (4.0 * area)


def _elastic_element(tri, h, E, nu):
    """6x6 plane-strain P1 stiffness, dofs ordered (ux0, uy0, ux1, uy1, ux2, uy2)."""
    b, c, area = _tri_geometry(tri, h)
    B = np.zeros((3, 6))
    B[0, 0::2] = b
    B[1, 1::2] = c
    B[2, 0::2] = c
    B[2, 1::2] = b
    B /= 2.0 * area
    f = E / ((1.0 + nu) * (1.0 - 2.0 * nu))
    D = f * np.array([[1.0 - nu, nu, 0.0], [nu, 1.0 - nu, 0.0], [0.0, 0.0, (1.0 - 2.0 * nu) / 2.0]])
    return area * (B.T @ D @ B)


def _assemble(m, dof, elem_mats, cell_factor):
    """Stencil-slot assembly. Returns vals[dof, m*m, dof*7] (zeros where absent) and a mask."""
    nn = m * m
    nc = m - 1
    vals = np.zeros((dof, nn, dof * 7))
    rr, cc = np.meshgrid(np.arange(nc), np.arange(nc), indexing="ij")
    rr = rr.ravel()
    cc = cc.ravel()
    for t, (tri, ke) in enumerate(elem_mats):
        g = cell_factor[t] if cell_factor is not None else None
        for a, (ar, ac) in enumerate(tri):
            node_a = (rr + ar) * m + (cc + ac)
            for bb, (br, bc) in enumerate(tri):
                slot = _SLOT_OF[(br - ar, bc - ac)]
                for p in range(dof):
                    for q in range(dof):
                        k = ke[a * dof + p, bb * dof + q]
                        contrib = k if g is None else g * k
                        vals[p, node_a, q * 7 + slot] += contrib
    # valid slots: neighbour inside the grid
    r = np.arange(nn) // m
    c = np.arange(nn) % m
    valid = np.zeros((nn, 7), dtype=bool)
    for s, (dr, dc) in enumerate(_SLOTS):
        valid[:, s] = (r + dr >= 0) & (r + dr < m) & (c + dc >= 0) & (c + dc < m)
    return vals, valid


def _to_csr(m, dof, vals, valid, fixed, fixed_val):
    """Eliminate fixed dofs symmetrically and compress to CSR (columns sorted)."""
    nn = m * m
    n = dof * nn
    offs = np.array([dr * m + dc for (dr, dc) in _SLOTS], dtype=np.int64)
    node = np.arange(nn, dtype=np.int64)
    cols = np.empty((dof, nn, dof * 7), dtype=np.int64)
    mask = np.empty((dof, nn, dof * 7), dtype=bool)
    for p in range(dof):
        for q in range(dof):
            cols[p, :, q * 7:(q + 1) * 7] = q * nn + node[:, None] + offs[None, :]
            mask[p, :, q * 7:(q + 1) * 7] = valid
    cols = cols.reshape(n, dof * 7)
    vals = vals.reshape(n, dof * 7)
    mask = mask.reshape(n, dof * 7)
    safe_cols = np.where(mask, cols, 0)
    # lift known values: b = -A u_D on free rows
    u_d = np.zeros(n)
    u_d[fixed] = fixed_val
    b = -np.sum(np.where(mask, vals * u_d[safe_cols], 0.0), axis=1)
    is_fixed = np.zeros(n, dtype=bool)
    is_fixed[fixed] = True
    keep = mask & ~is_fixed[safe_cols]
    keep[is_fixed, :] = False
    rows_fixed = np.nonzero(is_fixed)[0]
    # identity rows for the constrained dofs: keep only the diagonal slot
    diag_slot = (np.arange(n) // nn) * 7 + 3
    keep[rows_fixed, diag_slot[rows_fixed]] = True
    vals = vals.copy()
    vals[rows_fixed, diag_slot[rows_fixed]] = 1.0
    b[rows_fixed] = u_d[rows_fixed]
    counts = keep.sum(axis=1)
    indptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=indptr[1:])
    indices = cols[keep].astype(np.int32)
    data = vals[keep].astype(np.float64)
    return indptr.astype(np.int32), indices, data, b


def poisson_p1(m: int, seed: int = 0) -> CSRSystem:
    """Scalar P1 Laplacian on an m x m grid, homogeneous Dirichlet on all edges.

    RHS i.i.d. uniform in [-1, 1] from ``numpy.random.default_rng(seed)``,
    zero on the boundary rows.
    """
    h = 1.0 / (m - 1)
    elems = [(_TRI_LOWER, _laplace_element(_TRI_LOWER, h)), (_TRI_UPPER, _laplace_element(_TRI_UPPER, h))]
    vals, valid = _assemble(m, 1, elems, None)
    r = np.arange(m * m) // m
    c = np.arange(m * m) % m
    bnd = np.nonzero((r == 0) | (r == m - 1) | (c == 0) | (c == m - 1))[0]
    indptr, indices, data, _ = _to_csr(m, 1, vals, valid, bnd, 0.0)
    rng = np.random.default_rng(seed)
    b = rng.uniform(-1.0, 1.0, m * m)
    b[bnd] = 0.0
    return CSRSystem(m * m, indptr, indices, data, b, dof=1,
                     meta={"kind": "poisson_p1", "m": m, "seed": seed, "n_boundary": len(bnd)})


_LN2_HI = 6.93147180369123816490e-01  # ln 2 split so that k * _LN2_HI is exact for |k| < 2^20
_LN2_LO = 1.90821492927058770002e-10
_INV_LN2 = 1.44269504088896338700e+00


def portable_exp(x: np.ndarray) -> np.ndarray:
    """exp(x) for |x| < 700 from IEEE basic operations only, so that every host computes the same bits.

    Library exponentials (numpy's vectorised loops, libm) may round the last bit differently on x86 and
    Arm hosts; the benchmark's systems are generated on both, and their AMG hierarchies are compared
    bit for bit.  Cody-Waite reduction x = k ln2 + r (|r| <= ln2 / 2, ln 2 in two parts), the Taylor
    series of exp(r) to degree 14 (truncation below 1e-18 relative) by Horner's rule, then 2^k.
    Accurate to about 2 ulp.
    """
    x = np.asarray(x, dtype=np.float64)
    k = np.rint(x * _INV_LN2)
    r = (x - k * _LN2_HI) - k * _LN2_LO
    p = np.full_like(r, 1.0)
    for j in range(14, 0, -1):
        p = p * (r / j) + 1.0
    return np.ldexp(p, k.astype(np.int64))


def notch_damage(m: int, ell: float | None = None) -> np.ndarray:
    """Per-element damage d = exp(-dist/ell) to the notch (0,0.5)-(0.5,0.5).

    Returned as [2, (m-1)^2] (lower, upper triangle of each cell) evaluated at
    the triangle centroids; ``ell`` defaults to 2h.  The exponential is
    ``portable_exp``: the same bits on every host.
    """
    h = 1.0 / (m - 1)
    if ell is None:
        ell = 2.0 * h
    nc = m - 1
    rr, cc = np.meshgrid(np.arange(nc), np.arange(nc), indexing="ij")
    out = []
    for tri in (_TRI_LOWER, _TRI_UPPER):
        cx = (cc.ravel() + np.mean([dc for (dr, dc) in tri])) * h
        cy = (rr.ravel() + np.mean([dr for (dr, dc) in tri])) * h
        dx = np.where(cx > 0.5, cx - 0.5, 0.0)
        dist = np.sqrt(dx * dx + (cy - 0.5) ** 2)
        out.append(portable_exp(-dist / ell))
    return np.stack(out)


def elasticity_p1(m: int, E: float = 210.0, nu: float = 0.3, degraded: bool = True,
                  top_uy: float = 1e-3, residual_stiffness: float = 1e-6,
                  young: np.ndarray | None = None) -> CSRSystem:
    """Plane-strain P1 elasticity, block dof ordering [u_x(all nodes), u_y(all nodes)].

    Stiffness of each element scaled by ``(1-d)^2 + residual_stiffness`` with
    ``d`` the notch damage field (``degraded=True``), or by ``young/E`` when a
    per-element Young's modulus array ``young[2, (m-1)^2]`` is given.  Bottom
    edge clamped (u_x = u_y = 0); top edge u_y = ``top_uy`` with u_x free.
    """
    h = 1.0 / (m - 1)
    elems = [(_TRI_LOWER, _elastic_element(_TRI_LOWER, h, E, nu)),
             (_TRI_UPPER, _elastic_element(_TRI_UPPER, h, E, nu))]
    if young is not None:
        factor = np.asarray(young, dtype=np.float64) / E
    elif degraded:
        d = notch_damage(m)
        factor = (1.0 - d) ** 2 + residual_stiffness
    else:
        factor = None
    vals, valid = _assemble(m, 2, elems, factor)
    nn = m * m
    r = np.arange(nn) // m
    bottom = np.nonzero(r == 0)[0]
    top = np.nonzero(r == m - 1)[0]
    fixed = np.concatenate([bottom, nn + bottom, nn + top])
    fixed_val = np.concatenate([np.zeros(2 * len(bottom)), np.full(len(top), top_uy)])
    order = np.argsort(fixed)
    indptr, indices, data, b = _to_csr(m, 2, vals, valid, fixed[order], fixed_val[order])
    return CSRSystem(2 * nn, indptr, indices, data, b, dof=2,
                     meta={"kind": "elasticity_p1", "m": m, "E": E, "nu": nu,
                           "degraded": degraded, "top_uy": top_uy, "n_fixed": len(fixed)})


def _mass_element(tri, h):
    """3x3 lumped P1 mass: |T|/3 on the diagonal."""
    _, _, area = _tri_geometry(tri, h)
    return np.eye(3) * (area / 3.0)


def damage_qp(m: int, gc: float = 1.0, ell: float = 0.03, drive: float = 100.0,
              lower_scale: float = 0.5) -> CSRSystem:
    """Bound-constrained quadratic of phase-field (AT2) damage type on an m x m grid.

    Minimise ``q(d) = d.H.d/2 + d.b`` subject to ``lower <= d <= upper`` with
    ``H = gc*ell*K + (gc/ell)*M + 2*psi*M`` and ``b = -(2*psi + drive*psi)*M*1``:
    K the P1 Laplacian (natural boundary), M the lumped mass and ``psi`` a
    per-element driving energy peaked at the notch tip (0.5, 0.5).  The extra
    ``drive`` term pushes the unconstrained minimiser above 1 around the tip, so
    both bounds are active somewhere: ``upper = 1`` and ``lower`` = the nodal
    notch damage times ``lower_scale`` (irreversibility against a previous
    state).  The start ``x0`` is the midpoint of the box.  This is the subproblem
    Crack/crack.c hands to LinA's reflective_newton.
    """
    h = 1.0 / (m - 1)
    nc = m - 1
    rr, cc = np.meshgrid(np.arange(nc), np.arange(nc), indexing="ij")
    psi = []
    for tri in (_TRI_LOWER, _TRI_UPPER):
        cx = (cc.ravel() + np.mean([dc for (dr, dc) in tri])) * h
        cy = (rr.ravel() + np.mean([dr for (dr, dc) in tri])) * h
        dist = np.sqrt((cx - 0.5) ** 2 + (cy - 0.5) ** 2)
        psi.append(np.exp(-dist / 0.08))
    psi = np.stack(psi)
    kl = [(_TRI_LOWER, gc * ell * _laplace_element(_TRI_LOWER, h)),
          (_TRI_UPPER, gc * ell * _laplace_element(_TRI_UPPER, h))]
    ml = [(_TRI_LOWER, _mass_element(_TRI_LOWER, h)), (_TRI_UPPER, _mass_element(_TRI_UPPER, h))]
    vk, valid = _assemble(m, 1, kl, None)
    vm, _ = _assemble(m, 1, ml, gc / ell + 2.0 * psi)
    vf, _ = _assemble(m, 1, ml, (2.0 + drive) * psi)
    indptr, indices, data, _ = _to_csr(m, 1, vk + vm, valid, np.zeros(0, dtype=np.int64), 0.0)
    b = -vf[0, :, 3].copy()
    nn = m * m
    r = np.arange(nn) // m
    c = np.arange(nn) % m
    x, y = c * h, r * h
    dx = np.where(x > 0.5, x - 0.5, 0.0)
    lower = lower_scale * np.exp(-np.sqrt(dx * dx + (y - 0.5) ** 2) / ell)
    upper = np.ones(nn)
    x0 = 0.5 * (lower + upper)
    return CSRSystem(nn, indptr, indices, data, b, dof=1,
                     meta={"kind": "damage_qp", "m": m, "gc": gc, "ell": ell, "drive": drive,
                           "lower": lower, "upper": upper, "x0": x0})


def elastic_mesh(m: int, top_uy: float = 1e-3):
    """The m x m grid of ``elasticity_p1`` as an unstructured triangle mesh.

    Returns ``(xy[n_nodes, 2], tri[n_elems, 3], fixed_dof, fixed_val)``.  Triangle
    ``e = t*(m-1)^2 + r*(m-1) + c`` is the lower (t = 0) or upper (t = 1) triangle
    of cell (r, c), the element order of ``notch_damage`` and of the ``young``
    argument of ``elasticity_p1``; vertices counter-clockwise.  Dirichlet dofs as
    in ``elasticity_p1``: bottom edge clamped, top edge u_y = ``top_uy``.
    """
    h = 1.0 / (m - 1)
    nn = m * m
    r = np.arange(nn) // m
    c = np.arange(nn) % m
    xy = np.stack([c * h, r * h], axis=1).astype(np.float64)
    nc = m - 1
    rr, cc = np.meshgrid(np.arange(nc), np.arange(nc), indexing="ij")
    rr = rr.ravel()
    cc = cc.ravel()
    tris = []
    for tri in (_TRI_LOWER, _TRI_UPPER):
        tris.append(np.stack([(rr + dr) * m + (cc + dc) for (dr, dc) in tri], axis=1))
    tri = np.concatenate(tris).astype(np.int32)
    bottom = np.nonzero(r == 0)[0]
    top = np.nonzero(r == m - 1)[0]
    fixed = np.concatenate([bottom, nn + bottom, nn + top])
    fixed_val = np.concatenate([np.zeros(2 * len(bottom)), np.full(len(top), top_uy)])
    order = np.argsort(fixed)
    return xy, tri, fixed[order].astype(np.int32), fixed_val[order]


def adjoint_case(m: int, seed: int = 0, sigma: float = 0.5, n_sensors: int = 256, median: float = 210.0):
    """Material identification on the ``elastic_mesh(m)``: moduli, target moduli and sensors.

    ``young`` and ``young_target`` are per-element lognormal fields
    ``median * exp(sigma * z)`` with z standard normal from
    ``numpy.random.default_rng(seed)`` and ``(seed + 1)``; ``n_sensors`` sensor
    nodes are drawn without replacement from ``default_rng(seed + 2)`` among the
    nodes off the top and bottom edges (so neither component is a Dirichlet dof),
    and observe both displacement components: ``sensor_dof = [nodes, n_nodes + nodes]``.
    The targets are the forward solution for ``young_target`` at those dofs; they
    are computed by the caller's solver.
    """
    ne = 2 * (m - 1) ** 2
    young = median * np.exp(sigma * np.random.default_rng(seed).standard_normal(ne))
    young_t = median * np.exp(sigma * np.random.default_rng(seed + 1).standard_normal(ne))
    nn = m * m
    r = np.arange(nn) // m
    candidates = np.nonzero((r > 0) & (r < m - 1))[0]
    nodes = np.sort(np.random.default_rng(seed + 2).choice(candidates, size=n_sensors, replace=False))
    sensor_dof = np.concatenate([nodes, nn + nodes]).astype(np.int32)
    return {"m": m, "young": young, "young_target": young_t, "sensor_dof": sensor_dof}


def element_gradient(m: int, u: np.ndarray, lam: np.ndarray, nu: float = 0.3) -> np.ndarray:
    """dL/dE_e = -lambda_e^T Khat_e u_e for the ``elastic_mesh(m)`` (numpy, FP64).

    ``lam`` must vanish on Dirichlet dofs; ``u`` holds the known values there.
    Khat_e is the unit-modulus plane-strain element stiffness of ``_elastic_element``.
    """
    h = 1.0 / (m - 1)
    nn = m * m
    nc = m - 1
    rr, cc = np.meshgrid(np.arange(nc), np.arange(nc), indexing="ij")
    rr = rr.ravel()
    cc = cc.ravel()
    out = []
    for tri in (_TRI_LOWER, _TRI_UPPER):
        ke = _elastic_element(tri, h, 1.0, nu)
        nodes = [(rr + dr) * m + (cc + dc) for (dr, dc) in tri]
        ue = np.stack([v for k in nodes for v in (u[k], u[nn + k])], axis=1)
        le = np.stack([v for k in nodes for v in (lam[k], lam[nn + k])], axis=1)
        out.append(-np.einsum("ea,ab,eb->e", le, ke, ue))
    return np.concatenate(out)


def _smooth_field(m, seed, modes=4):
    """A seeded smooth displacement field on the m x m grid: sums of sine modes, [2, m*m]."""
    rng = np.random.default_rng(seed)
    h = 1.0 / (m - 1)
    r = np.arange(m * m) // m
    c = np.arange(m * m) % m
    x, y = c * h, r * h
    u = np.zeros((2, m * m))
    for comp in range(2):
        for _ in range(modes):
            kx, ky = rng.integers(1, 4, size=2)
            amp = 1e-3 * rng.standard_normal()
            ph = rng.uniform(0, 2 * np.pi)
            u[comp] += amp * np.sin(np.pi * kx * x + ph) * np.sin(np.pi * ky * y)
    return u


def indefinite_qp(m: int, shift: float = 0.5, seed: int = 0) -> CSRSystem:
    """A bound-constrained quadratic with an indefinite Hessian on an m x m grid (one unknown per node).

    ``H = K - shift I`` with K the graph Laplacian of the 5-point grid (diagonal = number of neighbours,
    -1 per neighbour; eigenvalues in [0, 8]), so the smooth modes below ``shift`` have negative
    curvature; ``b`` i.i.d. uniform in [-1/2, 1/2] from ``default_rng(seed)``; bounds 0 <= x <= 1, start at
    the midpoint 1/2.  Reflective Newton meets an indefinite scaled matrix here and takes the
    direction of negative curvature (get_neg_curvature_direction).  meta: lower, upper, x0.
    """
    n = m * m
    r = np.arange(n) // m
    c = np.arange(n) % m
    rows, cols, vals = [], [], []
    deg = np.zeros(n)
    for dr, dc in ((-1, 0), (1, 0), (0, -1), (0, 1)):
        ok = (r + dr >= 0) & (r + dr < m) & (c + dc >= 0) & (c + dc < m)
        i = np.nonzero(ok)[0]
        j = (r[i] + dr) * m + (c[i] + dc)
        rows.append(i)
        cols.append(j)
        vals.append(-np.ones(len(i)))
        deg[i] += 1.0
    rows.append(np.arange(n))
    cols.append(np.arange(n))
    vals.append(deg - shift)
    rows, cols, vals = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    indptr = np.zeros(n + 1, dtype=np.int32)
    np.add.at(indptr, rows + 1, 1)
    indptr = np.cumsum(indptr).astype(np.int32)
    b = np.random.default_rng(seed).uniform(-0.5, 0.5, n)
    return CSRSystem(n, indptr, cols.astype(np.int32), vals.astype(np.float64), b, dof=1,
                     meta={"lower": np.zeros(n), "upper": np.ones(n), "x0": np.full(n, 0.5)})


def at2_damage(m: int, seed: int = 0, gc: float = 2.7e-3, sigma: float = 1.0, E: float = 210.0,
               nu: float = 0.3) -> CSRSystem:
    """Phase-field damage step of AT2 type on the m x m grid (scalar P1, one unknown per node).

    Minimise ``sum_e [ (1-d)^2 H_e + gc (d^2/(2 ell) + (ell/2)|grad d|^2) ]`` over the elements,
    ``ell = 2h``, subject to ``d_prev <= d <= 1``: the quadratic ``d.A.d/2 + d.b`` with
    ``A = gc*ell*K + (gc/ell)*M + 2*M_H`` and ``b = -2*M_H*1`` (K the P1 Laplacian with natural
    boundary, M the lumped mass, M_H the lumped mass weighted by H_e).  The history field H_e is
    lognormal(sigma) from ``default_rng(seed)`` per element times the plane-strain strain energy
    density of a seeded smooth displacement field; ``d_prev`` is 0.9 times the nodal notch field
    (exp(-dist/ell) to the notch (0, 0.5)-(0.5, 0.5), the field of ``notch_damage``; the factor
    keeps the box open where the notch field reaches 1); the start is the midpoint of the box.
    Returned with meta lower/upper/x0 like ``damage_qp``.
    """
    h = 1.0 / (m - 1)
    ell = 2.0 * h
    nc = m - 1
    u = _smooth_field(m, seed + 1)
    rr, cc = np.meshgrid(np.arange(nc), np.arange(nc), indexing="ij")
    rr = rr.ravel()
    cc = cc.ravel()
    rng = np.random.default_rng(seed)
    psi = []
    f = E / ((1.0 + nu) * (1.0 - 2.0 * nu))
    D = f * np.array([[1.0 - nu, nu, 0.0], [nu, 1.0 - nu, 0.0], [0.0, 0.0, (1.0 - 2.0 * nu) / 2.0]])
    for tri in (_TRI_LOWER, _TRI_UPPER):
        b, cvec, area = _tri_geometry(tri, h)
        nodes = [(rr + dr) * m + (cc + dc) for (dr, dc) in tri]
        exx = sum(b[k] * u[0][nodes[k]] for k in range(3)) / (2 * area)
        eyy = sum(cvec[k] * u[1][nodes[k]] for k in range(3)) / (2 * area)
        gxy = sum(cvec[k] * u[0][nodes[k]] + b[k] * u[1][nodes[k]] for k in range(3)) / (2 * area)
        eps = np.stack([exx, eyy, gxy])
        psi.append(0.5 * np.einsum("ie,ij,je->e", eps, D, eps))
    H = np.stack(psi) * np.exp(sigma * rng.standard_normal((2, nc * nc)))
    kl = [(_TRI_LOWER, gc * ell * _laplace_element(_TRI_LOWER, h)),
          (_TRI_UPPER, gc * ell * _laplace_element(_TRI_UPPER, h))]
    ml = [(_TRI_LOWER, _mass_element(_TRI_LOWER, h)), (_TRI_UPPER, _mass_element(_TRI_UPPER, h))]
    vk, valid = _assemble(m, 1, kl, None)
    vm, _ = _assemble(m, 1, ml, gc / ell + 2.0 * H)
    vf, _ = _assemble(m, 1, ml, 2.0 * H)
    indptr, indices, data, _ = _to_csr(m, 1, vk + vm, valid, np.zeros(0, dtype=np.int64), 0.0)
    b = -vf[0, :, 3].copy()
    nn = m * m
    r = np.arange(nn) // m
    c = np.arange(nn) % m
    x, y = c * h, r * h
    dx = np.where(x > 0.5, x - 0.5, 0.0)
    lower = 0.9 * np.exp(-np.sqrt(dx * dx + (y - 0.5) ** 2) / ell)
    upper = np.ones(nn)
    x0 = 0.5 * (lower + upper)
    return CSRSystem(nn, indptr, indices, data, b, dof=1,
                     meta={"kind": "at2_damage", "m": m, "gc": gc, "ell": ell, "lower": lower, "upper": upper,
                           "x0": x0})


# ----------------------------------------------------------------------------- unstructured batches
def delaunay_mesh(n_nodes: int, seed: int = 0, jitter: float = 0.35):
    """Seeded unstructured triangle mesh of the unit square with about ``n_nodes`` nodes.

    The nodes are a k x k lattice (k = round(sqrt(n_nodes))) whose interior points are moved by a
    seeded uniform offset of up to ``jitter`` spacings in each direction; boundary nodes stay on
    the edges.  The triangles are their Delaunay triangulation (scipy.spatial.Delaunay), ordered
    counter-clockwise.  Returns ``(xy[n, 2], tri[n_elems, 3])``.
    """
    from scipy.spatial import Delaunay

    k = max(3, int(round(np.sqrt(n_nodes))))
    h = 1.0 / (k - 1)
    r, c = np.divmod(np.arange(k * k), k)
    xy = np.stack([c / (k - 1), r / (k - 1)], axis=1)  # edges exactly at 0 and 1
    rng = np.random.default_rng(seed)
    inner = (r > 0) & (r < k - 1) & (c > 0) & (c < k - 1)
    xy[inner] += rng.uniform(-jitter * h, jitter * h, size=(int(inner.sum()), 2))
    tri = Delaunay(xy).simplices.astype(np.int64)
    p = xy[tri]
    area2 = (p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])
    tri = tri[np.abs(area2) > 1e-9 * h * h]
    flip = area2[np.abs(area2) > 1e-9 * h * h] < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    return xy, tri.astype(np.int32)


def _p1_gradients(xy, tri):
    """b, c (shape [n_elems, 3]) and areas of P1 triangles: grad phi_a = (b_a, c_a) / (2 area)."""
    x = xy[tri, 0]
    y = xy[tri, 1]
    b = np.stack([y[:, 1] - y[:, 2], y[:, 2] - y[:, 0], y[:, 0] - y[:, 1]], axis=1)
    c = np.stack([x[:, 2] - x[:, 1], x[:, 0] - x[:, 2], x[:, 1] - x[:, 0]], axis=1)
    area = 0.5 * np.abs(x[:, 0] * b[:, 0] + x[:, 1] * b[:, 1] + x[:, 2] * b[:, 2])
    return b, c, area


def _csr_eliminate(n, rows, cols, vals, fixed, fixed_val, b):
    """Sum duplicates to a symmetric CSR matrix (sorted columns), then eliminate the fixed dofs
    symmetrically."""
    import scipy.sparse as sp

    A = sp.coo_matrix((vals, (rows, cols)), shape=(n, n)).tocsr()
    A.sum_duplicates()
    A = ((A + A.T) * 0.5).tocsr()  # exactly symmetric: the sums of duplicates ran in different orders
    A.sort_indices()
    is_fixed = np.zeros(n, dtype=bool)
    is_fixed[fixed] = True
    u_d = np.zeros(n)
    u_d[fixed] = fixed_val
    b = b - A @ u_d
    r = np.repeat(np.arange(n), np.diff(A.indptr))
    keep = ~is_fixed[r] & ~is_fixed[A.indices]
    diag = (r == A.indices) & is_fixed[r]
    data = A.data.copy()
    data[diag] = 1.0
    keep |= diag
    counts = np.bincount(r[keep], minlength=n)
    indptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=indptr[1:])
    b[is_fixed] = u_d[is_fixed]
    return indptr.astype(np.int32), A.indices[keep].astype(np.int32), data[keep], b


def batch_system(kind: str, dofs: int, seed: int = 0, sigma: float = 1.5, nu: float = 0.3,
                 top_uy: float = 1e-3) -> CSRSystem:
    """One system of the batched workload on ``delaunay_mesh``: a per-element lognormal coefficient
    (sigma 1.5, seeded) times the P1 stiffness.

    ``kind`` "poisson": scalar Laplacian, homogeneous Dirichlet on the whole boundary, right-hand
    side uniform in [-1, 1] on the free rows (``dofs`` nodes).  ``kind`` "elasticity": plane
    strain, E_e = 210 * lognormal, nu 0.3, block dof ordering [u_x of all nodes, u_y of all nodes]
    (dof 2), bottom edge clamped, top edge u_y = ``top_uy`` (``dofs / 2`` nodes).  Dirichlet
    conditions by symmetric elimination, as in ``elasticity_p1``.
    """
    rng = np.random.default_rng(seed)
    if kind == "poisson":
        xy, tri = delaunay_mesh(dofs, seed)
        nn = len(xy)
        b_, c_, area = _p1_gradients(xy, tri)
        kappa = np.exp(sigma * rng.standard_normal(len(tri)))
        ke = (b_[:, :, None] * b_[:, None, :] + c_[:, :, None] * c_[:, None, :]) / (4.0 * area)[:, None, None]
        ke *= kappa[:, None, None]
        rows = np.repeat(tri, 3, axis=1).ravel()
        cols = np.tile(tri, (1, 3)).ravel()
        on_edge = (xy[:, 0] == 0.0) | (xy[:, 0] == 1.0) | (xy[:, 1] == 0.0) | (xy[:, 1] == 1.0)
        fixed = np.nonzero(on_edge)[0]
        rhs = rng.uniform(-1.0, 1.0, nn)
        ptr, col, val, b = _csr_eliminate(nn, rows, cols, ke.ravel(), fixed, np.zeros(len(fixed)), rhs)
        return CSRSystem(nn, ptr, col, val, b, dof=1, meta={"kind": kind, "seed": seed, "elements": len(tri)})
    if kind == "elasticity":
        xy, tri = delaunay_mesh(max(dofs // 2, 9), seed)
        nn = len(xy)
        b_, c_, area = _p1_gradients(xy, tri)
        E = 210.0 * np.exp(sigma * rng.standard_normal(len(tri)))
        ne = len(tri)
        B = np.zeros((ne, 3, 6))
        B[:, 0, 0::2] = b_
        B[:, 1, 1::2] = c_
        B[:, 2, 0::2] = c_
        B[:, 2, 1::2] = b_
        B /= (2.0 * area)[:, None, None]
        D = np.array([[1.0 - nu, nu, 0.0], [nu, 1.0 - nu, 0.0], [0.0, 0.0, (1.0 - 2.0 * nu) / 2.0]])
        D = D / ((1.0 + nu) * (1.0 - 2.0 * nu))
        ke = np.einsum("eia,ij,ejb->eab", B, D, B) * (area * E)[:, None, None]
        ke = 0.5 * (ke + ke.transpose(0, 2, 1))  # exactly symmetric
        # element dof (a, p) -> global p * nn + node
        gd = np.stack([tri, tri + nn], axis=2).reshape(ne, 6)
        rows = np.repeat(gd, 6, axis=1).ravel()
        cols = np.tile(gd, (1, 6)).ravel()
        bottom = np.nonzero(xy[:, 1] == 0.0)[0]
        top = np.nonzero(xy[:, 1] == 1.0)[0]
        fixed = np.concatenate([bottom, nn + bottom, nn + top])
        fval = np.concatenate([np.zeros(2 * len(bottom)), np.full(len(top), top_uy)])
        order = np.argsort(fixed)
        ptr, col, val, b = _csr_eliminate(2 * nn, rows, cols, ke.ravel(), fixed[order], fval[order],
                                          np.zeros(2 * nn))
        return CSRSystem(2 * nn, ptr, col, val, b, dof=2, meta={"kind": kind, "seed": seed, "elements": ne})
    raise ValueError(f"unknown system kind {kind!r}")


def batch_plan(count: int = 96, seed: int = 0, lo: int = 10_000, hi: int = 500_000):
    """(kind, dofs, seed) of the batched workload: kinds alternate Poisson / elasticity, dof counts
    log-uniform on [lo, hi] (seeded)."""
    rng = np.random.default_rng(seed)
    dofs = np.exp(rng.uniform(np.log(lo), np.log(hi), count)).astype(np.int64)
    return [("poisson" if i % 2 == 0 else "elasticity", int(dofs[i]), seed * 1000 + i + 1) for i in range(count)]


def batch_depth(n: int) -> int:
    """AMG depth for a batched system: coarsest level of roughly a thousand rows (standard
    coarsening shrinks a 2D P1 level by about 2.3x)."""
    return int(min(10, max(2, 1 + np.ceil(np.log(max(n, 1000) / 1000.0) / np.log(2.3)))))


def batch_shard(plan, rank: int, world: int):
    """The systems of ``plan`` that rank ``rank`` of ``world`` solves: a greedy dof-balanced split
    (largest system first, to the least-loaded rank; ties to the lower rank), every system on exactly
    one rank, in plan order within a rank.  Independent systems need no exchange between ranks."""
    load = [0] * world
    owner = [0] * len(plan)
    for k in sorted(range(len(plan)), key=lambda k: (-plan[k][1], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        owner[k] = r
        load[r] += plan[k][1]
    return [p for p, o in zip(plan, owner) if o == rank]
