"""Python binding of the GB300 LinA library's C-ABI (include/lina_gpu.h).

The product is the shared library ``fem_gb300/_build/libLinA_gb300.so``: host
C/C++ plus sm_103a kernels.  This module is a thin ctypes layer over its
exported ``lina_gpu_*`` functions for tests and benchmarks; it contains no
numerical code and has no fallback: if the library is missing it raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libLinA_gb300.so")

AGGRESSIVE, STANDARD, PMIS = 1, 2, 3  # PMIS: labels computed on the GPU (opt-in, not the reference's)
SMOOTHER_JACOBI, SMOOTHER_MC_SOR = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
STOP_REFERENCE, STOP_RELATIVE = 0, 1
PCG_DEVICE_PTRS, PCG_USE_X0, PCG_FINAL_PRECON, PCG_TIME_KERNELS, PCG_NORMALIZE, PCG_HOST_LOOP = 1, 2, 4, 8, 16, 32
PCG_BETA_FLEXIBLE, PCG_BETA_STANDARD = 256, 512
UNDECIDED, COARSE, FINE, ISOLATED = 0, 1, 2, 3
OK, EINVAL, ECUDA, ESETUP, EBREAKDOWN, ENOCONV = 0, -1, -2, -3, -4, -5
ELASTIC_RECOMPUTE = 64
GMRES_APPLY_PRECON = 128


class AmgOptions(C.Structure):
    _fields_ = [
        ("dof", C.c_int),
        ("depth", C.c_int),
        ("smoothing_iterations", C.c_int),
        ("aggr_smoothing_iterations", C.c_int),
        ("coarsening", C.c_int),
        ("eps_minus", C.c_double),
        ("eps_plus", C.c_double),
        ("matrix_tol", C.c_double),
        ("smoother", C.c_int),
        ("omega", C.c_double),
        ("precision", C.c_int),
    ]


class P1Problem(C.Structure):
    _fields_ = [("kind", C.c_int), ("n_nodes", C.c_int), ("n_elems", C.c_int), ("xy", C.c_void_p), ("tri", C.c_void_p),
                ("nu", C.c_double), ("n_fixed", C.c_int), ("fixed_dof", C.c_void_p), ("fixed_val", C.c_void_p)]


P1_LAPLACE, P1_ELASTIC = 1, 2


class SolveInfo(C.Structure):
    _fields_ = [
        ("iterations", C.c_int),
        ("status", C.c_int),
        ("rel_residual", C.c_double),
        ("true_rel_residual", C.c_double),
        ("pcg_residuum", C.c_double),
        ("smoother_ms", C.c_double),
        ("smoother_launches", C.c_int),
        ("smoother_bytes", C.c_double),
        ("timed_level", C.c_int),
        ("timed_rows", C.c_int),
        ("timed_entries", C.c_long),
        ("restarts", C.c_int),
    ]


class ElasticProblem(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("n_elems", C.c_int), ("xy", C.c_void_p), ("tri", C.c_void_p),
                ("nu", C.c_double), ("n_fixed", C.c_int), ("fixed_dof", C.c_void_p), ("fixed_val", C.c_void_p),
                ("n_sensors", C.c_int), ("sensor_dof", C.c_void_p), ("target", C.c_void_p)]


class LinaError(RuntimeError):
    pass


_lib = None


def lib():
    """Load the product library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise LinaError(f"GB300 LinA library not built: {LIB_PATH} missing (run __graft_entry__.build())")
    L = C.CDLL(LIB_PATH)
    vp, ip, dp, lp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_long)
    sig = {
        "lina_gpu_default_options": (None, [C.POINTER(AmgOptions)]),
        "lina_gpu_amg_create": (C.c_int, [C.c_int, ip, ip, dp, C.POINTER(AmgOptions), C.POINTER(vp)]),
        "lina_gpu_amg_create_host_only": (C.c_int, [C.c_int, ip, ip, dp, C.POINTER(AmgOptions), C.POINTER(vp)]),
        "lina_gpu_amg_recompute": (C.c_int, [vp, C.c_int, ip, ip, dp]),
        "lina_gpu_amg_destroy": (C.c_int, [vp]),
        "lina_gpu_p1_create": (C.c_int, [C.POINTER(P1Problem), C.POINTER(vp)]),
        "lina_gpu_p1_assemble": (C.c_int, [vp, vp, C.c_int]),
        "lina_gpu_p1_sizes": (C.c_int, [vp, ip, C.POINTER(C.c_long)]),
        "lina_gpu_p1_download": (C.c_int, [vp, ip, ip, dp, dp]),
        "lina_gpu_p1_device": (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp)]),
        "lina_gpu_p1_destroy": (C.c_int, [vp]),
        "lina_gpu_p1_assemble_host": (C.c_int, [C.POINTER(P1Problem), dp, ip, ip, dp, dp, C.POINTER(C.c_long)]),
        "lina_gpu_amg_save": (C.c_int, [vp, C.c_char_p]),
        "lina_gpu_amg_load": (C.c_int, [C.c_char_p, C.POINTER(AmgOptions), C.c_int, C.POINTER(vp)]),
        "lina_gpu_amg_set_smoother": (C.c_int, [vp, C.c_int, C.c_double, C.c_int]),
        "lina_gpu_amg_set_fcg_history": (C.c_int, [vp, C.c_int]),
        "lina_gpu_pcg": (C.c_int, [vp, vp, vp, C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(SolveInfo)]),
        "lina_gpu_batch_create": (C.c_int, [C.c_int, C.POINTER(vp), C.c_int, C.POINTER(vp)]),
        "lina_gpu_batch_solve": (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp), C.c_double, C.c_int, C.c_int,
                                           C.POINTER(SolveInfo)]),
        "lina_gpu_batch_size": (C.c_int, [vp]),
        "lina_gpu_batch_destroy": (C.c_int, [vp]),
        "lina_gpu_segbatch_create": (C.c_int, [C.c_int, C.POINTER(vp), C.POINTER(vp)]),
        "lina_gpu_segbatch_solve": (C.c_int, [vp, C.POINTER(vp), C.POINTER(vp), C.c_double, C.c_int, C.c_int,
                                              C.POINTER(SolveInfo)]),
        "lina_gpu_segbatch_levels": (C.c_int, [vp, ip, C.POINTER(C.c_long), C.POINTER(C.c_long)]),
        "lina_gpu_segbatch_hierarchy": (C.c_int, [vp, C.POINTER(vp)]),
        "lina_gpu_segbatch_destroy": (C.c_int, [vp]),
        "lina_gpu_vcycle": (C.c_int, [vp, vp, vp]),
        "lina_gpu_spmv": (C.c_int, [vp, C.c_int, vp, vp]),
        "lina_gpu_amg_depth": (C.c_int, [vp]),
        "lina_gpu_level_sizes": (C.c_int, [vp, C.c_int, ip, lp, lp, lp, ip]),
        "lina_gpu_level_export": (C.c_int, [vp, C.c_int, ip, ip, ip, dp, ip, ip, dp, ip, ip, dp]),
        "lina_gpu_level_colours": (C.c_int, [vp, C.c_int, ip]),
        "lina_gpu_coarse_block_size": (C.c_int, [vp]),
        "lina_gpu_amg_device_bytes": (C.c_long, [vp]),
        "lina_gpu_malloc": (vp, [C.c_size_t]),
        "lina_gpu_free": (C.c_int, [vp]),
        "lina_gpu_memcpy_h2d": (C.c_int, [vp, vp, C.c_size_t]),
        "lina_gpu_memcpy_d2h": (C.c_int, [vp, vp, C.c_size_t]),
        "lina_gpu_synchronize": (C.c_int, []),
        "lina_gpu_device_count": (C.c_int, []),
        "lina_gpu_set_device": (C.c_int, [C.c_int]),
        "lina_gpu_set_layout": (C.c_int, [C.c_int]),
        "lina_gpu_set_fused_rows": (C.c_int, [C.c_int]),
        "lina_gpu_set_fused_jacobi_entries": (C.c_int, [C.c_long]),
        "lina_gpu_set_fused_groups": (C.c_int, [C.c_int]),
        "lina_gpu_set_autotune": (C.c_int, [C.c_int]),
        "lina_gpu_set_sell_index_bits": (C.c_int, [C.c_int]),
        "lina_gpu_set_sell_quads": (C.c_int, [C.c_int]),
        "lina_gpu_set_pdl": (C.c_int, [C.c_int]),
        "lina_gpu_set_device_memory_limit": (C.c_int, [C.c_long]),
        "lina_gpu_dense_inverse": (C.c_int, [C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
        "lina_gpu_set_coarse_inverse": (C.c_int, [C.c_int, C.c_int]),
        "lina_gpu_matrix_index_bits": (C.c_int, [vp]),
        "lina_gpu_level_index_bits": (C.c_int, [vp, C.c_int, ip, ip, ip]),
        "lina_gpu_last_error": (C.c_char_p, []),
        "lina_gpu_timer_begin": (C.c_int, [vp]),
        "lina_gpu_timer_end": (C.c_int, [vp, dp]),
        "lina_gpu_launches": (C.c_ulonglong, []),
        "lina_gpu_malloc_host": (vp, [C.c_size_t]),
        "lina_gpu_matrix_create": (C.c_int, [C.c_int, C.c_int, ip, ip, dp, C.POINTER(vp)]),
        "lina_gpu_matrix_destroy": (C.c_int, [vp]),
        "lina_gpu_matrix_spmv": (C.c_int, [vp, C.c_int, vp, vp]),
        "lina_gpu_matrix_jacobi": (C.c_int, [vp, C.c_int, C.c_double, C.c_int, vp, vp, vp]),
        "lina_gpu_matrix_padded_entries": (C.c_long, [vp]),
        "lina_gpu_matrix_rows": (C.c_int, [vp]),
        "lina_gpu_ilu_create_from_matrix": (C.c_int, [C.c_int, ip, ip, dp, C.POINTER(vp)]),
        "lina_gpu_ilu_destroy": (C.c_int, [vp]),
        "lina_gpu_ilu_levels": (C.c_int, [vp, ip, ip]),
        "lina_gpu_ilu_factor_values": (C.c_int, [vp, dp]),
        "lina_gpu_ilu_refactor": (C.c_int, [vp, dp, C.c_int]),
        "lina_gpu_wait_probe": (C.c_int, [C.c_int, dp]),
        "lina_gpu_matrix_update_values": (C.c_int, [vp, dp, C.c_int]),
        "lina_gpu_ilu_apply": (C.c_int, [vp, C.c_int, vp, vp]),
        "lina_gpu_ilu_time_apply": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]),
        "lina_gpu_dot": (C.c_int, [vp, vp, C.c_long, dp]),
        "lina_gpu_dot_noalloc": (C.c_int, [vp, vp, C.c_long, dp]),
        "lina_gpu_bicgstab": (C.c_int, [vp, vp, C.c_int, vp, vp, C.c_double, C.c_int, C.c_int, C.POINTER(SolveInfo)]),
        "lina_gpu_free_host": (C.c_int, [vp]),
        "lina_gpu_amg_update_values": (C.c_int, [vp, vp, C.c_int]),
        "lina_gpu_reflective_newton_csr": (C.c_int, [C.c_int, ip, ip, dp, dp, dp, dp, dp, C.c_int, C.c_int,
                                                     C.c_double, C.c_double]),
        "lina_gpu_spgemm": (C.c_int, [C.c_int, C.c_int, ip, ip, dp, C.c_int, ip, ip, dp, C.c_long, ip, ip, dp, lp]),
        "lina_gpu_amg_fmg": (C.c_int, [vp, vp, vp, C.c_int, dp]),
        "lina_gpu_gmres": (C.c_int, [vp, vp, vp, C.c_int, vp, vp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                     C.POINTER(SolveInfo)]),
        "lina_gpu_elastic_create": (C.c_int, [C.POINTER(ElasticProblem), dp, C.POINTER(AmgOptions), C.POINTER(vp)]),
        "lina_gpu_elastic_forward": (C.c_int, [vp, vp, C.c_double, C.c_int, C.c_int, vp, dp, C.POINTER(SolveInfo)]),
        "lina_gpu_elastic_backward": (C.c_int, [vp, C.c_double, C.c_int, C.c_int, vp, vp, C.POINTER(SolveInfo)]),
        "lina_gpu_elastic_sizes": (C.c_int, [vp, ip, lp]),
        "lina_gpu_elastic_system": (C.c_int, [vp, ip, ip, dp, dp]),
        "lina_gpu_elastic_amg": (vp, [vp]),
        "lina_gpu_elastic_destroy": (C.c_int, [vp]),
        "lina_gpu_elastic_assemble_host": (C.c_int, [C.POINTER(ElasticProblem), dp, ip, ip, dp, dp, lp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    return lib().lina_gpu_last_error().decode()


def _check(rc, what):
    if rc != 0:
        raise LinaError(f"{what} failed ({rc}): {last_error()}")


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def options(**kw) -> AmgOptions:
    o = AmgOptions()
    lib().lina_gpu_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


@dataclass
class Level:
    n: int
    A: tuple
    labels: np.ndarray | None
    P: tuple | None
    R: tuple | None
    n_colours: int


class DeviceArray:
    """A device buffer owned through the library's allocator (FP64 or int32)."""

    def __init__(self, n, dtype=np.float64):
        self.n = int(n)
        self.dtype = np.dtype(dtype)
        self.nbytes = self.n * self.dtype.itemsize
        self.ptr = lib().lina_gpu_malloc(max(self.nbytes, 1))
        if not self.ptr:
            raise LinaError(f"device allocation of {self.nbytes} bytes failed: {last_error()}")

    @classmethod
    def from_host(cls, a):
        a = np.ascontiguousarray(a)
        d = cls(a.size, a.dtype)
        _check(lib().lina_gpu_memcpy_h2d(d.ptr, a.ctypes.data, d.nbytes), "h2d copy")
        return d

    def to_host(self):
        out = np.empty(self.n, dtype=self.dtype)
        _check(lib().lina_gpu_memcpy_d2h(out.ctypes.data, self.ptr, self.nbytes), "d2h copy")
        return out

    def free(self):
        if self.ptr:
            lib().lina_gpu_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class PinnedArray:
    """Page-locked host memory (cudaMallocHost) viewed as a numpy array."""

    def __init__(self, n, dtype=np.float64):
        self.dtype = np.dtype(dtype)
        self.nbytes = int(n) * self.dtype.itemsize
        self.ptr = lib().lina_gpu_malloc_host(max(self.nbytes, 1))
        if not self.ptr:
            raise LinaError(f"pinned allocation failed: {last_error()}")
        buf = (C.c_char * max(self.nbytes, 1)).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=self.dtype, count=int(n))

    def free(self):
        if self.ptr:
            self.array = None
            lib().lina_gpu_free_host(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


LAYOUT_AUTO, LAYOUT_SELL, LAYOUT_CSRV = 0, 1, 2


def set_layout(layout: int):
    _check(lib().lina_gpu_set_layout(int(layout)), "set layout")


FUSED_ROWS_DEFAULT = 24576
FUSED_JACOBI_ENTRIES_DEFAULT = 0


def set_fused_rows(max_rows: int):
    """Levels of at most max_rows rows run a multicolour-SOR V-cycle step as one cluster launch
    (0: one launch per colour)."""
    _check(lib().lina_gpu_set_fused_rows(int(max_rows)), "set fused rows")


def set_autotune(on: bool):
    """Hierarchies created afterwards measure each level's candidate layouts at upload and keep the fastest."""
    _check(lib().lina_gpu_set_autotune(int(bool(on))), "set autotune")


def set_fused_groups(on: bool):
    """Segmented batches created afterwards run the multicolour-SOR step of concatenated levels as one
    cluster per group of whole systems (off by default)."""
    _check(lib().lina_gpu_set_fused_groups(int(bool(on))), "set fused groups")


def set_fused_jacobi_entries(max_entries: int):
    """Damped Jacobi: levels of at most max_entries stored entries run a V-cycle step as one cluster
    launch (0: never)."""
    _check(lib().lina_gpu_set_fused_jacobi_entries(int(max_entries)), "set fused Jacobi entries")


def set_sell_index_bits(bits: int):
    """16 (the default): SELL-32 matrices with long rows uploaded afterwards also get 16-bit column
    offsets (two bases per slice, where the columns fit), read by FP32 passes; 32: int columns only."""
    _check(lib().lina_gpu_set_sell_index_bits(int(bits)), "set SELL index bits")


DENSE_SIMT, DENSE_DMMA = 0, 1


def dense_inverse_device(a: "DeviceArray", m, method=DENSE_SIMT):
    """In-place inverse of the m x m row-major matrix in a (device) by blocked Gauss-Jordan without
    pivoting; returns the device time in ms."""
    ms = C.c_double()
    _check(lib().lina_gpu_dense_inverse(C.c_int(m), C.c_void_p(a.ptr), method, C.byref(ms)), "dense inverse")
    return ms.value


def set_coarse_inverse(min_rows, method=DENSE_SIMT):
    """Coarsest blocks of min_rows rows or more inverted on the GPU (0: host) with method."""
    _check(lib().lina_gpu_set_coarse_inverse(int(min_rows), int(method)), "set coarse inverse")


def set_device_memory_limit(nbytes):
    """Device bytes one handle may allocate (0: no limit); beyond it allocations fail with ECUDA."""
    _check(lib().lina_gpu_set_device_memory_limit(int(nbytes)), "set memory limit")


def set_pdl(on):
    """Programmatic dependent launch of the solve kernels (1, default) or plain stream order (0)."""
    _check(lib().lina_gpu_set_pdl(int(on)), "set PDL")


def set_sell_quads(on):
    """FP32 passes over natural-order SELL-32 matrices uploaded afterwards read the quad layout (1) or
    the one-entry layout (0); identical results."""
    _check(lib().lina_gpu_set_sell_quads(int(on)), "set quads")


def dot(a: "DeviceArray", b: "DeviceArray") -> float:
    r = C.c_double()
    _check(lib().lina_gpu_dot(a.ptr, b.ptr, a.n, C.byref(r)), "dot")
    return r.value


def set_device(device: int):
    _check(lib().lina_gpu_set_device(int(device)), "set device")


def launches() -> int:
    return int(lib().lina_gpu_launches())


class Matrix:
    """A single device matrix (SELL-32) with the library's SpMV and Jacobi kernels."""

    def __init__(self, n, indptr, indices, data, ncols=None):
        self.n = int(n)
        self.ncols = int(ncols or n)
        ip_ = np.ascontiguousarray(indptr, dtype=np.int32)
        ix_ = np.ascontiguousarray(indices, dtype=np.int32)
        dv_ = np.ascontiguousarray(data, dtype=np.float64)
        h = C.c_void_p()
        _check(lib().lina_gpu_matrix_create(self.n, self.ncols, _ip(ip_), _ip(ix_), _dp(dv_), C.byref(h)),
               "matrix create")
        self.h = h

    @property
    def padded_entries(self):
        return lib().lina_gpu_matrix_padded_entries(self.h)

    def index_bits(self):
        """Column-index width of the FP32 passes: 16 or 32 (SELL-32), 0 for the lane-group CSR layout."""
        return lib().lina_gpu_matrix_index_bits(self.h)

    def update_values(self, data):
        """New values on the pattern given at creation (CSR order)."""
        dv_ = np.ascontiguousarray(data, dtype=np.float64)
        _check(lib().lina_gpu_matrix_update_values(self.h, _dp(dv_), 0), "matrix update values")

    def spmv_device(self, x: DeviceArray, y: DeviceArray, precision=PREC_FP64):
        _check(lib().lina_gpu_matrix_spmv(self.h, precision, x.ptr, y.ptr), "matrix spmv")

    def spmv(self, x, precision=PREC_FP64):
        dt = np.float32 if precision == PREC_MIXED else np.float64
        xd = DeviceArray.from_host(np.asarray(x, dtype=dt))
        yd = DeviceArray(self.n, dt)
        self.spmv_device(xd, yd, precision)
        return yd.to_host()

    def jacobi_device(self, b: DeviceArray, x: DeviceArray, tmp: DeviceArray, omega, sweeps, precision=PREC_FP64):
        _check(lib().lina_gpu_matrix_jacobi(self.h, precision, omega, sweeps, b.ptr, x.ptr, tmp.ptr), "jacobi")

    def jacobi(self, b, x0, omega, sweeps, precision=PREC_FP64):
        dt = np.float32 if precision == PREC_MIXED else np.float64
        bd = DeviceArray.from_host(np.asarray(b, dtype=dt))
        xd = DeviceArray.from_host(np.asarray(x0, dtype=dt))
        td = DeviceArray(self.n, dt)
        self.jacobi_device(bd, xd, td, omega, sweeps, precision)
        return (td if sweeps % 2 else xd).to_host()

    def close(self):
        if getattr(self, "h", None):
            lib().lina_gpu_matrix_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ILU:
    """ILU(0) of a CSR matrix (the reference's factorisation) applied on the GPU."""

    def __init__(self, n, indptr, indices, data):
        self.n = int(n)
        ip_ = np.ascontiguousarray(indptr, dtype=np.int32)
        ix_ = np.ascontiguousarray(indices, dtype=np.int32)
        dv_ = np.ascontiguousarray(data, dtype=np.float64)
        h = C.c_void_p()
        self.h = None
        self.nnz = len(ix_)
        _check(lib().lina_gpu_ilu_create_from_matrix(self.n, _ip(ip_), _ip(ix_), _dp(dv_), C.byref(h)), "ILU")
        self.h = h

    def refactor(self, data):
        """New values of A on the same pattern; the factors are recomputed on the GPU."""
        dv_ = np.ascontiguousarray(data, dtype=np.float64)
        _check(lib().lina_gpu_ilu_refactor(self.h, _dp(dv_), 0), "ILU refactor")

    def factor_values(self):
        """The factors on A's pattern: L_ij where j <= i, U_ij where j > i."""
        f = np.zeros(max(self.nnz, 1))
        _check(lib().lina_gpu_ilu_factor_values(self.h, _dp(f)), "ILU factor values")
        return f[:self.nnz]

    def levels(self):
        a, b = C.c_int(), C.c_int()
        _check(lib().lina_gpu_ilu_levels(self.h, C.byref(a), C.byref(b)), "ILU levels")
        return a.value, b.value

    def apply(self, r, precision=PREC_FP64):
        rd = DeviceArray.from_host(np.asarray(r, dtype=np.float64))
        zd = DeviceArray(self.n)
        _check(lib().lina_gpu_ilu_apply(self.h, precision, rd.ptr, zd.ptr), "ILU apply")
        return zd.to_host()

    def time_apply(self, reps=20, precision=PREC_MIXED):
        """Device milliseconds of one application (forward + backward triangular solve), CUDA events on
        the handle's stream around reps applications."""
        ms = C.c_double()
        _check(lib().lina_gpu_ilu_time_apply(self.h, precision, reps, C.byref(ms)), "ILU timing")
        return ms.value

    def apply_bytes(self, precision=PREC_MIXED):
        """Algorithmic bytes of one application: every off-diagonal factor entry's value and column
        once, and per row and triangular solve its row bounds, 1/diagonal, right-hand side and result."""
        w = 4 if precision == PREC_MIXED else 8
        return (w + 4) * (self.nnz - self.n) + 2 * self.n * (8 + 3 * w)

    def close(self):
        if getattr(self, "h", None):
            lib().lina_gpu_ilu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def bicgstab(M: "Matrix", b, ilu: "ILU | None" = None, ilu_precision=PREC_FP64, tol=1e-8, max_iter=1000, x0=None):
    """BiCGStab_solve on the GPU; returns (x, SolveInfo)."""
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(M.n) if x0 is None else np.array(x0, dtype=np.float64)
    info = SolveInfo()
    flags = PCG_USE_X0 if x0 is not None else 0
    rc = lib().lina_gpu_bicgstab(M.h, ilu.h if ilu else None, ilu_precision, bb.ctypes.data, x.ctypes.data, tol,
                                 max_iter, flags, C.byref(info))
    if rc not in (0, ENOCONV):
        raise LinaError(f"bicgstab failed ({rc}): {last_error()}")
    return x, info


RN_GPU_BICGSTAB_ILU, RN_PCG = 6, 3


def reflective_newton(s, lower, upper, x0, solver=RN_GPU_BICGSTAB_ILU, max_iter=50, eps=1e-8, bi_eps=1e-8):
    """min x.A.x/2 + x.b over lower <= x <= upper (A, b from the CSRSystem s); returns (x, steps)."""
    x = np.array(x0, dtype=np.float64)
    ip_ = np.ascontiguousarray(s.indptr, np.int32)
    ix_ = np.ascontiguousarray(s.indices, np.int32)
    dv_ = np.ascontiguousarray(s.data, np.float64)
    b = np.ascontiguousarray(s.b, np.float64)
    lo = np.ascontiguousarray(lower, np.float64)
    up = np.ascontiguousarray(upper, np.float64)
    it = lib().lina_gpu_reflective_newton_csr(s.n, _ip(ip_), _ip(ix_), _dp(dv_), _dp(b), _dp(lo), _dp(up), _dp(x),
                                              solver, max_iter, eps, bi_eps)
    if it < 0:
        raise LinaError(f"reflective_newton failed ({it}): {last_error()}")
    return x, it


def spgemm(a, b, ncols_b):
    """C = A B on the GPU with the reference's sparse_product semantics; a and b are
    (indptr, indices, data) triples; returns C's triple."""
    ap, ac, av = (np.ascontiguousarray(a[0], np.int32), np.ascontiguousarray(a[1], np.int32),
                  np.ascontiguousarray(a[2], np.float64))
    bp, bc, bv = (np.ascontiguousarray(b[0], np.int32), np.ascontiguousarray(b[1], np.int32),
                  np.ascontiguousarray(b[2], np.float64))
    n, nb = len(ap) - 1, len(bp) - 1
    nnz = C.c_long()
    _check(lib().lina_gpu_spgemm(n, ncols_b, _ip(ap), _ip(ac), _dp(av), nb, _ip(bp), _ip(bc), _dp(bv), 0, None, None,
                                 None, C.byref(nnz)), "spgemm")
    cp, cc, cv = np.zeros(n + 1, np.int32), np.zeros(max(nnz.value, 1), np.int32), np.zeros(max(nnz.value, 1))
    _check(lib().lina_gpu_spgemm(n, ncols_b, _ip(ap), _ip(ac), _dp(av), nb, _ip(bp), _ip(bc), _dp(bv),
                                 max(nnz.value, 1), _ip(cp), _ip(cc), _dp(cv), C.byref(nnz)), "spgemm")
    return cp, cc[:nnz.value], cv[:nnz.value]


def _p1_problem(kind, xy, tri, nu, fixed_dof, fixed_val):
    keep = (np.ascontiguousarray(xy, dtype=np.float64).reshape(-1, 2), np.ascontiguousarray(tri, dtype=np.int32).reshape(-1, 3),
            np.ascontiguousarray(fixed_dof, dtype=np.int32), np.ascontiguousarray(fixed_val, dtype=np.float64))
    p = P1Problem(kind, len(keep[0]), len(keep[1]), keep[0].ctypes.data, keep[1].ctypes.data, float(nu), len(keep[2]),
                  keep[2].ctypes.data if len(keep[2]) else None, keep[3].ctypes.data if len(keep[3]) else None)
    return p, keep


def p1_assemble_host(kind, xy, tri, coef, nu=0.3, fixed_dof=(), fixed_val=()):
    """Host P1 assembly (lina_gpu_p1_assemble_host); returns (indptr, indices, data, b)."""
    p, keep = _p1_problem(kind, xy, tri, nu, fixed_dof, fixed_val)
    nnz = C.c_long()
    _check(lib().lina_gpu_p1_assemble_host(C.byref(p), None, None, None, None, None, C.byref(nnz)), "P1 assembly")
    n = p.n_nodes * (2 if kind == P1_ELASTIC else 1)
    ptr, col = np.zeros(n + 1, np.int32), np.zeros(max(nnz.value, 1), np.int32)
    val, b = np.zeros(max(nnz.value, 1)), np.zeros(n)
    cf = np.ascontiguousarray(coef, dtype=np.float64)
    _check(lib().lina_gpu_p1_assemble_host(C.byref(p), _dp(cf), _ip(ptr), _ip(col), _dp(val), _dp(b), None),
           "P1 assembly")
    return ptr, col[:nnz.value], val[:nnz.value], b


class P1Assembly:
    """P1 Laplacian or plane-strain elasticity assembled on the GPU into a fixed CSR pattern."""

    def __init__(self, kind, xy, tri, nu=0.3, fixed_dof=(), fixed_val=()):
        p, self._keep = _p1_problem(kind, xy, tri, nu, fixed_dof, fixed_val)
        h = C.c_void_p()
        self.h = None
        _check(lib().lina_gpu_p1_create(C.byref(p), C.byref(h)), "P1 create")
        self.h = h
        n, nnz = C.c_int(), C.c_long()
        _check(lib().lina_gpu_p1_sizes(self.h, C.byref(n), C.byref(nnz)), "P1 sizes")
        self.n, self.nnz = n.value, nnz.value

    def assemble(self, coef):
        cf = np.ascontiguousarray(coef, dtype=np.float64)
        _check(lib().lina_gpu_p1_assemble(self.h, cf.ctypes.data, 0), "P1 assemble")

    def system(self):
        """(indptr, indices, data, b) of the last assembly, copied to the host."""
        ptr, col = np.zeros(self.n + 1, np.int32), np.zeros(max(self.nnz, 1), np.int32)
        val, b = np.zeros(max(self.nnz, 1)), np.zeros(self.n)
        _check(lib().lina_gpu_p1_download(self.h, _ip(ptr), _ip(col), _dp(val), _dp(b)), "P1 download")
        return ptr, col[:self.nnz], val[:self.nnz], b

    def device_values(self):
        """Device pointers (values, b) of the last assembly."""
        v, b = C.c_void_p(), C.c_void_p()
        _check(lib().lina_gpu_p1_device(self.h, C.byref(v), C.byref(b)), "P1 device")
        return v.value, b.value

    def close(self):
        if getattr(self, "h", None):
            lib().lina_gpu_p1_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Independent AMG-PCG solves in one CUDA graph launch (lina_gpu_batch_*)."""

    def __init__(self, systems, stop=STOP_RELATIVE):
        self.systems = list(systems)
        self.sizes = [a.n for a in self.systems]
        arr = (C.c_void_p * len(self.systems))(*[a.h.value if isinstance(a.h, C.c_void_p) else a.h
                                                  for a in self.systems])
        h = C.c_void_p()
        self.h = None
        _check(lib().lina_gpu_batch_create(len(self.systems), arr, stop, C.byref(h)), "batch create")
        self.h = h

    def solve(self, bs, tol=1e-8, max_iter=1000, device=False):
        """bs: host arrays (or DeviceArray with device=True); returns (xs, [SolveInfo])."""
        k = len(self.systems)
        if device:
            xs = [DeviceArray(n) for n in self.sizes]
            bp = (C.c_void_p * k)(*[b.ptr for b in bs])
            xp = (C.c_void_p * k)(*[x.ptr for x in xs])
        else:
            bb = [np.ascontiguousarray(b, dtype=np.float64) for b in bs]
            xs = [np.zeros(n) for n in self.sizes]
            bp = (C.c_void_p * k)(*[b.ctypes.data for b in bb])
            xp = (C.c_void_p * k)(*[x.ctypes.data for x in xs])
        infos = (SolveInfo * k)()
        rc = lib().lina_gpu_batch_solve(self.h, bp, xp, tol, max_iter, PCG_DEVICE_PTRS if device else 0, infos)
        if rc not in (0, ENOCONV):
            raise LinaError(f"batch solve failed ({rc}): {last_error()}")
        return xs, list(infos)

    def close(self):
        if getattr(self, "h", None):
            lib().lina_gpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SegmentedBatch(Batch):
    """Independent systems solved as one segmented system (lina_gpu_segbatch_*): block-diagonal combined
    hierarchy, per-system FCG scalars and stopping, one graph launch."""

    def __init__(self, systems):
        self.systems = list(systems)
        self.sizes = [a.n for a in self.systems]
        arr = (C.c_void_p * len(self.systems))(*[a.h.value if isinstance(a.h, C.c_void_p) else a.h
                                                  for a in self.systems])
        h = C.c_void_p()
        self.h = None
        _check(lib().lina_gpu_segbatch_create(len(self.systems), arr, C.byref(h)), "segmented batch create")
        self.h = h

    def solve(self, bs, tol=1e-8, max_iter=1000, device=False, host_loop=False):
        """bs: host arrays (or DeviceArray with device=True); returns (xs, [SolveInfo]).  host_loop: the
        iterations launched from the host (for profiling)."""
        k = len(self.systems)
        if device:
            xs = [DeviceArray(n) for n in self.sizes]
            bp = (C.c_void_p * k)(*[b.ptr for b in bs])
            xp = (C.c_void_p * k)(*[x.ptr for x in xs])
        else:
            bb = [np.ascontiguousarray(b, dtype=np.float64) for b in bs]
            xs = [np.zeros(n) for n in self.sizes]
            bp = (C.c_void_p * k)(*[b.ctypes.data for b in bb])
            xp = (C.c_void_p * k)(*[x.ctypes.data for x in xs])
        infos = (SolveInfo * k)()
        rc = lib().lina_gpu_segbatch_solve(self.h, bp, xp, tol, max_iter,
                                           (PCG_DEVICE_PTRS if device else 0) | (PCG_HOST_LOOP if host_loop else 0),
                                           infos)
        if rc not in (0, ENOCONV):
            raise LinaError(f"segmented batch solve failed ({rc}): {last_error()}")
        return xs, list(infos)

    def hierarchy(self):
        """The combined hierarchy as an AMG object that does not own it (valid while the batch lives)."""
        h = C.c_void_p()
        _check(lib().lina_gpu_segbatch_hierarchy(self.h, C.byref(h)), "segmented batch hierarchy")
        a = AMG.__new__(AMG)
        a.h = h
        a.borrowed = True
        a.depth = lib().lina_gpu_amg_depth(h)
        a.n = a.level_size(a.depth - 1)
        return a

    def levels(self):
        """(rows, entries) per level of the combined hierarchy, coarsest first."""
        d = C.c_int()
        _check(lib().lina_gpu_segbatch_levels(self.h, C.byref(d), None, None), "segmented batch levels")
        rows = (C.c_long * d.value)()
        ent = (C.c_long * d.value)()
        _check(lib().lina_gpu_segbatch_levels(self.h, C.byref(d), rows, ent), "segmented batch levels")
        return list(rows), list(ent)

    def close(self):
        if getattr(self, "h", None):
            lib().lina_gpu_segbatch_destroy(self.h)
            self.h = None


def gmres(M: "Matrix", b, ilu: "ILU | None" = None, amg: "AMG | None" = None, precon_precision=PREC_FP64, tol=1e-8,
          i_max=30, max_iter=1000, check_each=False, y0=None, apply_precon=False):
    """Restarted GMRES on the GPU with a right preconditioner; returns (y, SolveInfo), y the
    preconditioned iterate (or x = B_r y with apply_precon)."""
    bb = np.ascontiguousarray(b, dtype=np.float64)
    y = np.zeros(M.n) if y0 is None else np.array(y0, dtype=np.float64)
    info = SolveInfo()
    flags = GMRES_APPLY_PRECON if apply_precon else 0
    rc = lib().lina_gpu_gmres(M.h, ilu.h if ilu else None, amg.h if amg else None, precon_precision, bb.ctypes.data,
                              y.ctypes.data, tol, i_max, max_iter, int(check_each), flags, C.byref(info))
    if rc not in (0, ENOCONV):
        raise LinaError(f"gmres failed ({rc}): {last_error()}")
    return y, info


class AMG:
    """A hierarchy built by the library (AMG_setup) and held on the GPU."""

    def __init__(self, n, indptr, indices, data, host_only=False, **opts):
        self.n = int(n)
        self._ip = np.ascontiguousarray(indptr, dtype=np.int32)
        self._ix = np.ascontiguousarray(indices, dtype=np.int32)
        self._dv = np.ascontiguousarray(data, dtype=np.float64)
        self.opts = options(**opts)
        h = C.c_void_p()
        fn = lib().lina_gpu_amg_create_host_only if host_only else lib().lina_gpu_amg_create
        _check(fn(self.n, _ip(self._ip), _ip(self._ix), _dp(self._dv), C.byref(self.opts), C.byref(h)), "AMG setup")
        self.h = h
        self.depth = lib().lina_gpu_amg_depth(self.h)

    def save(self, directory):
        """Write the hierarchy to a directory (lina_gpu_amg_save)."""
        _check(lib().lina_gpu_amg_save(self.h, os.fsencode(directory)), "AMG save")

    @classmethod
    def load(cls, directory, host_only=False, **opts):
        """A hierarchy saved by save(): its structure from the files, the solve options from opts."""
        self = cls.__new__(cls)
        self.opts = options(**opts)
        h = C.c_void_p()
        self.h = None
        _check(lib().lina_gpu_amg_load(os.fsencode(directory), C.byref(self.opts), int(host_only), C.byref(h)),
               "AMG load")
        self.h = h
        self.depth = lib().lina_gpu_amg_depth(self.h)
        self.n = self.level_size(self.depth - 1)
        return self

    @classmethod
    def from_system(cls, s, host_only=False, **opts):
        opts.setdefault("dof", s.dof)
        return cls(s.n, s.indptr, s.indices, s.data, host_only=host_only, **opts)

    def index_bits(self, lv):
        """(A, P, R) column-index widths of the FP32 passes over level lv: 16 or 32 for SELL-32, 0 for
        the lane-group CSR layout or a missing matrix."""
        a, p, r = C.c_int(), C.c_int(), C.c_int()
        _check(lib().lina_gpu_level_index_bits(self.h, lv, C.byref(a), C.byref(p), C.byref(r)), "index bits")
        return a.value, p.value, r.value

    def level(self, lv) -> Level:
        L = lib()
        n, na, np_, nr, nc = C.c_int(), C.c_long(), C.c_long(), C.c_long(), C.c_int()
        _check(L.lina_gpu_level_sizes(self.h, lv, C.byref(n), C.byref(na), C.byref(np_), C.byref(nr), C.byref(nc)),
               "level sizes")
        n = n.value
        A = (np.zeros(n + 1, np.int32), np.zeros(max(na.value, 1), np.int32), np.zeros(max(na.value, 1)))
        labels = np.zeros(n, np.int32)
        if lv > 0:
            P = (np.zeros(n + 1, np.int32), np.zeros(max(np_.value, 1), np.int32), np.zeros(max(np_.value, 1)))
            nrr = P and None
            # R has one row per coarse point
            R = None
        _Pp = _Pc = _Pv = _Rp = _Rc = _Rv = None
        if lv > 0:
            ncoarse = self.level_size(lv - 1)
            R = (np.zeros(ncoarse + 1, np.int32), np.zeros(max(nr.value, 1), np.int32), np.zeros(max(nr.value, 1)))
            _Pp, _Pc, _Pv = (_ip(P[0]), _ip(P[1]), _dp(P[2]))
            _Rp, _Rc, _Rv = (_ip(R[0]), _ip(R[1]), _dp(R[2]))
        _check(L.lina_gpu_level_export(self.h, lv, _ip(labels), _ip(A[0]), _ip(A[1]), _dp(A[2]),
                                       _Pp, _Pc, _Pv, _Rp, _Rc, _Rv), "level export")
        A = (A[0], A[1][:na.value], A[2][:na.value])
        if lv == 0:
            return Level(n, A, None, None, None, nc.value)
        P = (P[0], P[1][:np_.value], P[2][:np_.value])
        R = (R[0], R[1][:nr.value], R[2][:nr.value])
        return Level(n, A, labels, P, R, nc.value)

    def level_size(self, lv):
        n = C.c_int()
        _check(lib().lina_gpu_level_sizes(self.h, lv, C.byref(n), None, None, None, None), "level sizes")
        return n.value

    def sizes(self):
        return [self.level_size(lv) for lv in range(self.depth)]

    def colours(self, lv):
        c = np.zeros(self.level_size(lv), np.int32)
        _check(lib().lina_gpu_level_colours(self.h, lv, _ip(c)), "colours")
        return c

    def set_smoother(self, smoother, omega, precision):
        _check(lib().lina_gpu_amg_set_smoother(self.h, smoother, omega, precision), "set smoother")

    def set_fcg_history(self, m):
        """Directions kept by the flexible CG (0 default: FCG(6) mixed, CG FP64; 1 two-term; 2..8 FCG(m))."""
        _check(lib().lina_gpu_amg_set_fcg_history(self.h, m), "set FCG history")

    def update_values(self, data=None, device_ptr=None):
        """New finest values on the creation pattern (lina_gpu_amg_update_values): a host array, or a
        device pointer (e.g. P1Assembly.device_values())."""
        if device_ptr is not None:
            _check(lib().lina_gpu_amg_update_values(self.h, device_ptr, PCG_DEVICE_PTRS), "AMG update values")
        else:
            dv_ = np.ascontiguousarray(data, dtype=np.float64)
            _check(lib().lina_gpu_amg_update_values(self.h, dv_.ctypes.data, 0), "AMG update values")

    def recompute(self, indptr, indices, data):
        ip_ = np.ascontiguousarray(indptr, dtype=np.int32)
        ix_ = np.ascontiguousarray(indices, dtype=np.int32)
        dv_ = np.ascontiguousarray(data, dtype=np.float64)
        _check(lib().lina_gpu_amg_recompute(self.h, self.n, _ip(ip_), _ip(ix_), _dp(dv_)), "AMG recompute")

    def pcg(self, b, x0=None, tol=1e-8, max_iter=1000, stop=STOP_RELATIVE, flags=0):
        """Solve on host arrays (copies inside); returns (x, SolveInfo)."""
        bb = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.n) if x0 is None else np.array(x0, dtype=np.float64)
        if x0 is not None:
            flags |= PCG_USE_X0
        info = SolveInfo()
        rc = lib().lina_gpu_pcg(self.h, bb.ctypes.data, x.ctypes.data, tol, max_iter, stop, flags, C.byref(info))
        if rc not in (0, -5):
            raise LinaError(f"pcg failed ({rc}): {last_error()}")
        return x, info

    def pcg_device(self, b_dev: DeviceArray, x_dev: DeviceArray, tol=1e-8, max_iter=1000, stop=STOP_RELATIVE,
                   flags=0):
        info = SolveInfo()
        rc = lib().lina_gpu_pcg(self.h, b_dev.ptr, x_dev.ptr, tol, max_iter, stop, flags | PCG_DEVICE_PTRS,
                                C.byref(info))
        if rc not in (0, -5):
            raise LinaError(f"pcg failed ({rc}): {last_error()}")
        return info

    def fmg(self, F):
        """One full-multigrid pass (AMG_solve with FULL_AMG); returns (x, ||F - A x|| / ||F||)."""
        f = np.ascontiguousarray(F, dtype=np.float64)
        x = np.zeros(self.n)
        rel = C.c_double()
        _check(lib().lina_gpu_amg_fmg(self.h, f.ctypes.data, x.ctypes.data, 0, C.byref(rel)), "FMG")
        return x, rel.value

    def vcycle(self, r):
        rd = DeviceArray.from_host(np.asarray(r, dtype=np.float64))
        zd = DeviceArray(self.n)
        _check(lib().lina_gpu_vcycle(self.h, rd.ptr, zd.ptr), "vcycle")
        return zd.to_host()

    def spmv(self, x, level=None):
        lv = self.depth - 1 if level is None else level
        n = self.level_size(lv)
        xd = DeviceArray.from_host(np.asarray(x, dtype=np.float64))
        yd = DeviceArray(n)
        _check(lib().lina_gpu_spmv(self.h, lv, xd.ptr, yd.ptr), "spmv")
        return yd.to_host()

    def timer_begin(self):
        _check(lib().lina_gpu_timer_begin(self.h), "timer begin")

    def timer_end(self) -> float:
        ms = C.c_double()
        _check(lib().lina_gpu_timer_end(self.h, C.byref(ms)), "timer end")
        return ms.value

    @property
    def device_bytes(self):
        return lib().lina_gpu_amg_device_bytes(self.h)

    @property
    def coarse_block(self):
        return lib().lina_gpu_coarse_block_size(self.h)

    def close(self):
        if getattr(self, "h", None) and not getattr(self, "borrowed", False):
            lib().lina_gpu_amg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _ProblemArrays:
    """Keeps the arrays an ElasticProblem points to alive."""

    def __init__(self, xy, tri, nu, fixed_dof, fixed_val, sensor_dof, target):
        self.xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1)
        self.tri = np.ascontiguousarray(tri, dtype=np.int32).reshape(-1)
        self.fd = np.ascontiguousarray(fixed_dof, dtype=np.int32)
        self.fv = np.ascontiguousarray(fixed_val, dtype=np.float64)
        self.sd = np.ascontiguousarray(sensor_dof if sensor_dof is not None else np.zeros(0), dtype=np.int32)
        self.tg = np.ascontiguousarray(target if target is not None else np.zeros(len(self.sd)), dtype=np.float64)
        self.p = ElasticProblem(len(self.xy) // 2, len(self.tri) // 3, self.xy.ctypes.data, self.tri.ctypes.data, nu,
                                len(self.fd), self.fd.ctypes.data, self.fv.ctypes.data, len(self.sd),
                                self.sd.ctypes.data, self.tg.ctypes.data)


def elastic_assemble_host(xy, tri, nu, fixed_dof, fixed_val, young):
    """The library's host assembly of A(young) and b; returns (indptr, indices, data, b)."""
    pa = _ProblemArrays(xy, tri, nu, fixed_dof, fixed_val, None, None)
    E = np.ascontiguousarray(young, dtype=np.float64)
    nnz = C.c_long()
    _check(lib().lina_gpu_elastic_assemble_host(C.byref(pa.p), _dp(E), None, None, None, None, C.byref(nnz)),
           "elastic assembly")
    n = 2 * pa.p.n_nodes
    ptr, col = np.zeros(n + 1, np.int32), np.zeros(nnz.value, np.int32)
    val, b = np.zeros(nnz.value), np.zeros(n)
    _check(lib().lina_gpu_elastic_assemble_host(C.byref(pa.p), _dp(E), _ip(ptr), _ip(col), _dp(val), _dp(b),
                                                C.byref(nnz)), "elastic assembly")
    return ptr, col, val, b


class ElasticAdjoint:
    """Forward/backward pair of the P1 plane-strain adjoint (lina_gpu_elastic_*)."""

    def __init__(self, xy, tri, nu, fixed_dof, fixed_val, sensor_dof, target, young, **opts):
        self._pa = _ProblemArrays(xy, tri, nu, fixed_dof, fixed_val, sensor_dof, target)
        self.n_elems = self._pa.p.n_elems
        self.n = 2 * self._pa.p.n_nodes
        opts.setdefault("dof", 2)
        self.opts = options(**opts)
        E = np.ascontiguousarray(young, dtype=np.float64)
        h = C.c_void_p()
        _check(lib().lina_gpu_elastic_create(C.byref(self._pa.p), _dp(E), C.byref(self.opts), C.byref(h)),
               "elastic create")
        self.h = h

    def forward(self, young, tol=1e-12, max_iter=2000, warm=False, recompute=False):
        """Returns (u, loss, SolveInfo)."""
        E = np.ascontiguousarray(young, dtype=np.float64)
        u = np.zeros(self.n)
        loss = C.c_double()
        info = SolveInfo()
        flags = (PCG_USE_X0 if warm else 0) | (ELASTIC_RECOMPUTE if recompute else 0)
        rc = lib().lina_gpu_elastic_forward(self.h, E.ctypes.data, tol, max_iter, flags, u.ctypes.data,
                                            C.byref(loss), C.byref(info))
        if rc not in (0, ENOCONV):
            raise LinaError(f"elastic forward failed ({rc}): {last_error()}")
        return u, loss.value, info

    def backward(self, tol=1e-12, max_iter=2000):
        """Returns (grad, lambda, SolveInfo) at the last forward solution."""
        g = np.zeros(self.n_elems)
        lam = np.zeros(self.n)
        info = SolveInfo()
        rc = lib().lina_gpu_elastic_backward(self.h, tol, max_iter, 0, g.ctypes.data, lam.ctypes.data,
                                             C.byref(info))
        if rc not in (0, ENOCONV):
            raise LinaError(f"elastic backward failed ({rc}): {last_error()}")
        return g, lam, info

    def system(self):
        n, nnz = C.c_int(), C.c_long()
        _check(lib().lina_gpu_elastic_sizes(self.h, C.byref(n), C.byref(nnz)), "elastic sizes")
        ptr, col = np.zeros(n.value + 1, np.int32), np.zeros(nnz.value, np.int32)
        val, b = np.zeros(nnz.value), np.zeros(n.value)
        _check(lib().lina_gpu_elastic_system(self.h, _ip(ptr), _ip(col), _dp(val), _dp(b)), "elastic system")
        return ptr, col, val, b

    def close(self):
        if getattr(self, "h", None):
            lib().lina_gpu_elastic_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- the drop-in LinA API (include/*.h)
class SparseMatrix(C.Structure):
    """The reference's row-list sparse_matrix (LinA/linear_algebra.h:29-34)."""
    _fields_ = [("Values", C.POINTER(C.POINTER(C.c_double))), ("Indices", C.POINTER(C.POINTER(C.c_int))),
                ("Len", C.POINTER(C.c_int)), ("size", C.c_int)]


class RowListView:
    """A sparse_matrix whose rows point into the arrays of a CSR matrix (no copy): what a caller of the
    drop-in API hands to AMG_setup, PCG_default and friends.  Read-only use: the library functions that
    would grow or free rows must not be called on it."""

    def __init__(self, indptr, indices, data):
        self.ptr = np.ascontiguousarray(indptr, dtype=np.int64)
        self.col = np.ascontiguousarray(indices, dtype=np.int32)
        self.val = np.ascontiguousarray(data, dtype=np.float64)
        n = len(self.ptr) - 1
        self.len = np.ascontiguousarray(np.diff(self.ptr), dtype=np.int32)
        self.vrows = (self.val.ctypes.data + 8 * self.ptr[:-1]).astype(np.uint64)
        self.crows = (self.col.ctypes.data + 4 * self.ptr[:-1]).astype(np.uint64)
        self.m = SparseMatrix(C.cast(self.vrows.ctypes.data, C.POINTER(C.POINTER(C.c_double))),
                              C.cast(self.crows.ctypes.data, C.POINTER(C.POINTER(C.c_int))),
                              C.cast(self.len.ctypes.data, C.POINTER(C.c_int)), n)

    @property
    def ref(self):
        return C.byref(self.m)


def dropin():
    """The library with the signatures of the drop-in functions used from Python (AMG, PCG)."""
    L = lib()
    if getattr(L, "_dropin_ready", False):
        return L
    vp, dp = C.c_void_p, C.POINTER(C.c_double)
    sig = {
        "AMG_setup": (vp, [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp]),
        "AMG_free_data": (None, [vp]),
        "AMG_set_smoother": (None, [vp]),
        "AMG_set_SOR_relaxation_coeff": (None, [C.c_double]),
        "AMG_set_matrix_tolerance": (None, [C.c_double]),
        "AMG_gpu_set_precision": (None, [C.c_int]),
        "AMG_print_info": (None, [C.c_int]),
        "PCG_default": (None, [vp, vp, vp]),
        "PCG_set_AMG_data": (None, [vp]),
        "PCG_set_precon": (None, [vp]),
        "pcg": (C.c_int, [dp, dp, C.c_int, C.c_double, C.c_int]),
        "get_pcg_residuum": (C.c_double, []),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    L._dropin_ready = True
    return L
