"""ctypes front end to oracle/_ref/libLinA_ref.so (the reference LinA built from its sources).

Test infrastructure only: tests and the CPU-baseline leg of bench.py use this
to obtain the reference's own answers.  The library exists only where the
reference tree was available to build it (``make -C oracle ref``); callers
check :func:`available` first.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libLinA_ref.so")

# labels of LinA/Multigrid.h:23-27
UNDECIDED, COARSE, FINE, ISOLATED = 0, 1, 2, 3
STANDARD, AGGRESSIVE = 2, 1
SMOOTHER_REF_SOR, SMOOTHER_REF_JACOBI, SMOOTHER_DAMPED_JACOBI, SMOOTHER_MC_SOR = 0, 1, 2, 3

_lib = None


def available() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    try:
        lib()
    except OSError:
        return False
    return True


def lib():
    global _lib
    if _lib is not None:
        return _lib
    L = C.CDLL(LIB_PATH)
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    sig = {
        "rs_silence": (None, [C.c_int]),
        "rs_malloc_zero": (None, []),
        "rs_from_csr": (vp, [C.c_int, ip, ip, dp]),
        "rs_free": (None, [vp]),
        "rs_size": (C.c_int, [vp]),
        "rs_nnz": (C.c_long, [vp]),
        "rs_to_csr": (None, [vp, ip, ip, dp]),
        "rs_amg_setup": (vp, [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
        "rs_amg_depth": (C.c_int, [vp]),
        "rs_amg_fine_size": (C.c_int, [vp, C.c_int]),
        "rs_amg_coarse_size": (C.c_int, [vp, C.c_int]),
        "rs_amg_A": (vp, [vp, C.c_int]),
        "rs_amg_P": (vp, [vp, C.c_int]),
        "rs_amg_R": (vp, [vp, C.c_int]),
        "rs_amg_L": (vp, [vp, C.c_int]),
        "rs_amg_U": (vp, [vp, C.c_int]),
        "rs_amg_signs": (vp, [vp]),
        "rs_amg_labels": (ip, [vp, C.c_int]),
        "rs_amg_free": (None, [vp]),
        "rs_amg_recompute": (None, [vp, vp]),
        "rs_greedy_colouring": (C.c_int, [vp, ip]),
        "rs_forget_colouring": (None, []),
        "rs_set_smoother": (None, [C.c_int, C.c_double]),
        "rs_pcg_amg": (C.c_int, [vp, vp, dp, dp, C.c_double, C.c_int, dp]),
        "rs_amg_solve": (C.c_int, [vp, dp, dp, C.c_double, C.c_int]),
        "rs_vcycle_zero": (None, [vp, dp, dp]),
        "rs_spmv": (None, [vp, dp, dp]),
        "rs_product": (vp, [vp, vp]),
        "rs_transpose": (vp, [vp, C.c_int]),
        "rs_ilu": (C.c_int, [vp, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
        "rs_ilu_apply": (None, [vp, vp, dp]),
        "rs_pcg_stock_amg": (C.c_int, [vp, C.c_int, C.c_int, C.c_double, dp, dp, C.c_double, C.c_int, dp]),
        "rs_amg_solve_fresh": (C.c_int, [vp, dp, dp, C.c_double, C.c_int]),
        "rs_bicgstab_ilu": (C.c_int, [vp, dp, dp, C.c_double, C.c_int, C.c_int]),
        "rs_amg_fmg": (C.c_int, [vp, dp, dp]),
        "rs_gmres": (C.c_int, [vp, dp, dp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, ip, dp]),
        "rs_newton": (C.c_int, [vp, C.c_double, dp, dp, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_double]),
        "rs_active_set": (C.c_int, [vp, dp, dp, dp, dp, C.c_int, ip]),
        "rs_reflective_newton_qp": (C.c_int, [vp, dp, dp, dp, dp, C.c_int, C.c_int, C.c_double, C.c_double]),
        "rs_rn_neg_curv": (C.c_int, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    L.rs_malloc_zero()
    _lib = L
    return L


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class RefMatrix:
    """Owning handle to a reference row-list sparse_matrix."""

    def __init__(self, ptr, owned=True):
        self.ptr = ptr
        self.owned = owned

    @classmethod
    def from_csr(cls, n, indptr, indices, data):
        ip_ = np.ascontiguousarray(indptr, dtype=np.int32)
        ix_ = np.ascontiguousarray(indices, dtype=np.int32)
        dt_ = np.ascontiguousarray(data, dtype=np.float64)
        return cls(lib().rs_from_csr(n, _ip(ip_), _ip(ix_), _dp(dt_)))

    @property
    def size(self):
        return lib().rs_size(self.ptr)

    def to_csr(self):
        n = self.size
        nnz = lib().rs_nnz(self.ptr)
        indptr = np.zeros(n + 1, dtype=np.int32)
        indices = np.zeros(max(nnz, 1), dtype=np.int32)
        data = np.zeros(max(nnz, 1), dtype=np.float64)
        lib().rs_to_csr(self.ptr, _ip(indptr), _ip(indices), _dp(data))
        return indptr, indices[:nnz], data[:nnz]

    def transpose(self):
        """get_transpose (LinA/linear_algebra.c:1290)."""
        return RefMatrix(lib().rs_transpose(self.ptr, self.size))

    def __del__(self):
        if self.owned and self.ptr and _lib is not None:
            _lib.rs_free(self.ptr)
            self.ptr = None


@dataclass
class RefLevel:
    A: tuple            # (indptr, indices, data)
    labels: np.ndarray | None
    P: tuple | None
    R: tuple | None


class RefAMG:
    """AMG_setup (LinA/Multigrid.c:1613) on a CSR matrix, hierarchy read back as CSR."""

    def __init__(self, sysm, depth, sm=2, aggr_sm=2, coarsening=AGGRESSIVE, quiet=True):
        self.A = RefMatrix.from_csr(sysm.n, sysm.indptr, sysm.indices, sysm.data)
        if quiet:
            lib().rs_silence(1)
        try:
            self.ptr = lib().rs_amg_setup(self.A.ptr, int(sysm.dof), depth, sm, aggr_sm, coarsening)
        finally:
            if quiet:
                lib().rs_silence(0)
        self.depth = depth
        self.n = sysm.n

    def level(self, lv) -> RefLevel:
        L = lib()
        A = RefMatrix(L.rs_amg_A(self.ptr, lv), owned=False).to_csr()
        if lv == 0:
            return RefLevel(A, None, None, None)
        n = L.rs_amg_fine_size(self.ptr, lv)
        labels = np.ctypeslib.as_array(L.rs_amg_labels(self.ptr, lv), shape=(n,)).copy()
        P = RefMatrix(L.rs_amg_P(self.ptr, lv), owned=False).to_csr()
        R = RefMatrix(L.rs_amg_R(self.ptr, lv), owned=False).to_csr()
        return RefLevel(A, labels, P, R)

    def sizes(self):
        return [lib().rs_amg_fine_size(self.ptr, lv) for lv in range(self.depth)]

    def pcg(self, b, tol=1e-8, max_iter=1000, smoother=SMOOTHER_REF_SOR, omega=1.0, x0=None):
        """pcg with a one-V-cycle zero-guess preconditioner; returns (x, iterations, pcg_residuum)."""
        x = np.zeros(self.n) if x0 is None else np.array(x0, dtype=np.float64)
        bb = np.array(b, dtype=np.float64)
        res = C.c_double(0.0)
        lib().rs_set_smoother(smoother, omega)
        lib().rs_forget_colouring()
        lib().rs_silence(1)
        try:
            it = lib().rs_pcg_amg(self.ptr, self.A.ptr, _dp(x), _dp(bb), tol, max_iter, C.byref(res))
        finally:
            lib().rs_silence(0)
        return x, it, res.value

    def amg_solve(self, F, eps=1e-8, max_iter=200, smoother=SMOOTHER_REF_SOR, omega=1.0):
        """AMG_solve from a zero guess; returns (x, V-cycles)."""
        x = np.zeros(self.n)
        f = np.array(F, dtype=np.float64)
        lib().rs_set_smoother(smoother, omega)
        lib().rs_forget_colouring()
        lib().rs_silence(1)
        try:
            it = lib().rs_amg_solve_fresh(self.ptr, _dp(f), _dp(x), eps, max_iter)
        finally:
            lib().rs_silence(0)
        return x, it

    def fmg(self, F, x0=None, smoother=SMOOTHER_REF_SOR, omega=1.0):
        """AMG_solve with the FULL_AMG cycle structure (one full-multigrid pass); returns x."""
        x = np.zeros(self.n) if x0 is None else np.array(x0, dtype=np.float64)
        f = np.array(F, dtype=np.float64)
        lib().rs_set_smoother(smoother, omega)
        lib().rs_forget_colouring()
        lib().rs_silence(1)
        try:
            lib().rs_amg_fmg(self.ptr, _dp(f), _dp(x))
        finally:
            lib().rs_silence(0)
        return x

    def vcycle(self, r, smoother=SMOOTHER_REF_SOR, omega=1.0):
        z = np.zeros(self.n)
        rr = np.array(r, dtype=np.float64)
        lib().rs_set_smoother(smoother, omega)
        lib().rs_forget_colouring()
        lib().rs_silence(1)
        try:
            lib().rs_vcycle_zero(self.ptr, _dp(rr), _dp(z))
        finally:
            lib().rs_silence(0)
        return z

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.rs_amg_free(self.ptr)
            self.ptr = None


class RefHierarchy:
    """A reference hierarchy read back as arrays (sizes and per-level A, labels, P, R), detached from the
    library: the result of :func:`hierarchy`."""

    def __init__(self, sizes, levels):
        self._sizes = list(sizes)
        self._levels = list(levels)
        self.depth = len(self._levels)

    def sizes(self):
        return list(self._sizes)

    def level(self, lv) -> RefLevel:
        return self._levels[lv]


def _hierarchy_child(n, indptr, indices, data, dof, depth, sm, aggr_sm, coarsening):
    from types import SimpleNamespace
    sysm = SimpleNamespace(n=n, indptr=indptr, indices=indices, data=data, dof=dof)
    R = RefAMG(sysm, depth, sm, aggr_sm, coarsening)
    return R.sizes(), [R.level(lv) for lv in range(depth)]


_HIERARCHIES: dict = {}


def hierarchy(sysm, depth, sm=2, aggr_sm=2, coarsening=AGGRESSIVE) -> RefHierarchy:
    """AMG_setup of the reference on a CSR system, run in a child process of its own (spawned) and
    remembered for the rest of the session by the system's bytes and the settings.

    After one large set-up the reference's later set-ups in the same process run many times slower
    (a 33k-dof elasticity hierarchy: 5 s the first time, 90-110 s the next; the allocator's state
    after the reference frees its row lists, which malloc_trim does not undo).  A child process per
    set-up keeps every run at its first-run speed and the test process's heap clean."""
    import hashlib
    import multiprocessing as mp

    ip_ = np.ascontiguousarray(sysm.indptr, dtype=np.int32)
    ix_ = np.ascontiguousarray(sysm.indices, dtype=np.int32)
    dt_ = np.ascontiguousarray(sysm.data, dtype=np.float64)
    h = hashlib.sha256()
    for a in (ip_, ix_, dt_):
        h.update(a.tobytes())
    key = (h.hexdigest(), int(sysm.dof), depth, sm, aggr_sm, coarsening)
    if key not in _HIERARCHIES:
        with mp.get_context("spawn").Pool(1) as pool:
            sizes, levels = pool.apply(_hierarchy_child, (int(sysm.n), ip_, ix_, dt_, int(sysm.dof), depth, sm,
                                                          aggr_sm, coarsening))
        _HIERARCHIES[key] = RefHierarchy(sizes, levels)
    return _HIERARCHIES[key]


def pcg_stock(sysm, depth, smoother=SMOOTHER_MC_SOR, omega=1.6, tol=1e-8, max_iter=500):
    """PCG_default + PCG_set_AMG_preconditioner + pcg on the reference; returns (x, iterations, residuum)."""
    A = RefMatrix.from_csr(sysm.n, sysm.indptr, sysm.indices, sysm.data)
    x = np.zeros(sysm.n)
    b = np.array(sysm.b, dtype=np.float64)
    res = C.c_double(0.0)
    lib().rs_set_smoother(smoother, omega)
    lib().rs_forget_colouring()
    lib().rs_silence(1)
    try:
        it = lib().rs_pcg_stock_amg(A.ptr, int(sysm.dof), depth, omega, _dp(x), _dp(b), tol, max_iter, C.byref(res))
    finally:
        lib().rs_silence(0)
    return x, it, res.value


def ilu_apply(sysm, r):
    """z = U^-1 L^-1 r with the reference's ILU(0) of the system matrix."""
    A = RefMatrix.from_csr(sysm.n, sysm.indptr, sysm.indices, sysm.data)
    Lp, Up = C.c_void_p(), C.c_void_p()
    if lib().rs_ilu(A.ptr, C.byref(Lp), C.byref(Up)) != 1:
        raise RuntimeError("reference ILU(0) hit a zero pivot")
    Lm, Um = RefMatrix(Lp.value), RefMatrix(Up.value)
    z = np.array(r, dtype=np.float64)
    lib().rs_ilu_apply(Lm.ptr, Um.ptr, _dp(z))
    return z


def ilu_factors(n, indptr, indices, data):
    """incomplete_LU_factorization of the reference; returns (ok, f) with f the factors on A's
    pattern (L_ij where j <= i, U_ij where j > i), or (False, None) when it fails."""
    A = RefMatrix.from_csr(n, indptr, indices, data)
    Lp, Up = C.c_void_p(), C.c_void_p()
    ok = lib().rs_ilu(A.ptr, C.byref(Lp), C.byref(Up)) == 1
    Lm, Um = RefMatrix(Lp.value), RefMatrix(Up.value)
    if not ok:
        return False, None
    ptr = np.asarray(indptr, dtype=np.int64)
    col = np.asarray(indices, dtype=np.int64)
    f = np.full(len(col), np.nan)
    where = {}
    for i in range(n):
        for p in range(ptr[i], ptr[i + 1]):
            where[(i, int(col[p]))] = p
    for M, lower in ((Lm, True), (Um, False)):
        mp, mc, mv = M.to_csr()
        for i in range(n):
            for q in range(mp[i], mp[i + 1]):
                j = int(mc[q])
                if (lower and j <= i) or (not lower and j > i):
                    f[where[(i, j)]] = mv[q]
    return True, f


def bicgstab_ilu(sysm, eps=1e-8, max_iter=1000):
    """BiCGStab_solve with the ILU(0) preconditioner; returns (x, iterations)."""
    A = RefMatrix.from_csr(sysm.n, sysm.indptr, sysm.indices, sysm.data)
    x = np.zeros(sysm.n)
    b = np.array(sysm.b, dtype=np.float64)
    lib().rs_silence(1)
    try:
        it = lib().rs_bicgstab_ilu(A.ptr, _dp(x), _dp(b), eps, max_iter, 1)
    finally:
        lib().rs_silence(0)
    return x, it


def rn_neg_curv():
    """Negative-curvature events of the last reflective_newton run (its statistics)."""
    return lib().rs_rn_neg_curv()


def reflective_newton_qp(qp, solver=5, max_iter=50, eps=1e-8, bi_eps=1e-8):
    """reflective_newton on min x.H.x/2 + x.b, lower <= x <= upper; returns (x, iterations)."""
    H = RefMatrix.from_csr(qp.n, qp.indptr, qp.indices, qp.data)
    b = np.array(qp.b, dtype=np.float64)
    lo = np.array(qp.meta["lower"], dtype=np.float64)
    up = np.array(qp.meta["upper"], dtype=np.float64)
    x = np.array(qp.meta["x0"], dtype=np.float64)
    lib().rs_silence(1)
    try:
        it = lib().rs_reflective_newton_qp(H.ptr, _dp(b), _dp(lo), _dp(up), _dp(x), solver, max_iter, eps, bi_eps)
    finally:
        lib().rs_silence(0)
    return x, it


def gmres(s, y0=None, tol=1e-8, i_max=30, maxiter=1000, check_each=False, use_ilu=True):
    """The reference gmres on s's matrix with its ILU(0) as right preconditioner; returns
    (y, iterations, rcode, nomatvec, precision) with y the preconditioned iterate."""
    A = RefMatrix.from_csr(s.n, s.indptr, s.indices, s.data)
    y = np.zeros(s.n) if y0 is None else np.array(y0, dtype=np.float64)
    b = np.array(s.b, dtype=np.float64)
    out = np.zeros(3, dtype=np.int32)
    prec = C.c_double()
    lib().rs_silence(1)
    try:
        lib().rs_gmres(A.ptr, _dp(y), _dp(b), tol, i_max, maxiter, int(check_each), int(use_ilu), _ip(out),
                       C.byref(prec))
    finally:
        lib().rs_silence(0)
    return y, int(out[0]), int(out[1]), int(out[2]), prec.value


def newton(s, c, B, X0, maxiter=50, eps=1e-10, mode=1, i_max=30, gmres_maxiter=1000, gmres_tol=1e-10):
    """Newton_solver for A X + c X^3 = B (A = s's matrix); returns (X, Newton steps)."""
    A = RefMatrix.from_csr(s.n, s.indptr, s.indices, s.data)
    X = np.array(X0, dtype=np.float64)
    BB = np.array(B, dtype=np.float64)
    lib().rs_silence(1)
    try:
        it = lib().rs_newton(A.ptr, c, _dp(BB), _dp(X), maxiter, eps, mode, i_max, gmres_maxiter, gmres_tol)
    finally:
        lib().rs_silence(0)
    return X, it


def active_set(s, lower, upper, x0=None, max_iter=100):
    """active_set_solver with identity constraints lower <= x <= upper and a dense-LU KKT solver;
    returns (x, iterations, final active count)."""
    A = RefMatrix.from_csr(s.n, s.indptr, s.indices, s.data)
    x = np.zeros(s.n) if x0 is None else np.array(x0, dtype=np.float64)
    b = np.array(s.b, dtype=np.float64)
    lo = np.array(lower, dtype=np.float64)
    up = np.array(upper, dtype=np.float64)
    na = C.c_int()
    lib().rs_silence(1)
    try:
        it = lib().rs_active_set(A.ptr, _dp(x), _dp(b), _dp(lo), _dp(up), max_iter, C.byref(na))
    finally:
        lib().rs_silence(0)
    return x, it, na.value


def greedy_colouring(n, indptr, indices, data):
    M = RefMatrix.from_csr(n, indptr, indices, data)
    col = np.zeros(n, dtype=np.int32)
    nc = lib().rs_greedy_colouring(M.ptr, _ip(col))
    return nc, col


# ------------------------------------------------------------------ FEM2D P1 assembly (oracle/fem2d_shim.c)
FEM2D_PATH = os.path.join(HERE, "_ref", "libFEM2D_ref.so")
_fem2d = None


def fem2d_available() -> bool:
    if not os.path.exists(FEM2D_PATH):
        return False
    try:
        fem2d_lib()
    except OSError:
        return False
    return True


def fem2d_lib():
    global _fem2d
    if _fem2d is None:
        L = C.CDLL(FEM2D_PATH)
        ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
        L.fs_p1_assemble.restype = C.c_long
        L.fs_p1_assemble.argtypes = [C.c_int, C.c_int, dp, ip, ip, C.c_double, C.c_double, ip, ip, dp, C.c_long]
        _fem2d = L
    return _fem2d


def mesh_neighbours(n_nodes, tri):
    """Neighbour lists of a triangle mesh (each node's adjacent nodes, ascending) as (ptr, nb)."""
    tri = np.asarray(tri, dtype=np.int64)
    e = np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]])
    e = np.concatenate([e, e[:, ::-1]])
    e = np.unique(e, axis=0)
    ptr = np.zeros(n_nodes + 1, np.int32)
    np.add.at(ptr, e[:, 0] + 1, 1)
    return np.cumsum(ptr).astype(np.int32), np.ascontiguousarray(e[:, 1], dtype=np.int32)


def p1_assemble(xy, tri, kind="laplace", E=210.0, nu=0.3):
    """The reference's P1 assembly on the mesh (FEM2D set_matrix_Aij_11_2D): kind "laplace" the Laplacian
    with coefficient 1 (insert_A_bbV), n x n; kind "elastic" plane-strain elasticity with Young's modulus
    E and Poisson ratio nu, combined as crack.c does, 2n x 2n with the components blocked.  Returns
    (indptr, indices, data) with ascending columns."""
    L = fem2d_lib()
    xy = np.ascontiguousarray(xy, dtype=np.float64)
    n = len(xy)
    nptr, nb = mesh_neighbours(n, tri)
    k = 1 if kind == "laplace" else 2
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    mu = E / (2.0 * (1.0 + nu))
    rows = n * k
    nnz = L.fs_p1_assemble(k, n, _dp(xy), _ip(nptr), _ip(nb), lam, mu, None, None, None, 0)
    if nnz < 0:
        raise MemoryError("FEM2D assembly: out of memory")
    ptr = np.zeros(rows + 1, np.int32)
    col = np.zeros(max(nnz, 1), np.int32)
    val = np.zeros(max(nnz, 1))
    L.fs_p1_assemble(k, n, _dp(xy), _ip(nptr), _ip(nb), lam, mu, _ip(ptr), _ip(col), _dp(val), nnz)
    return ptr, col[:nnz], val[:nnz]
