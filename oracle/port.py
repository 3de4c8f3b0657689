"""ctypes front end to the CPU restatement oracle/_build/liblina_port.so (ORACLE).

Test infrastructure and CPU baseline only.  ``make -C oracle port`` builds the
library (plain gcc, no reference tree needed).
"""
from __future__ import annotations

import ctypes as C
import os
from types import SimpleNamespace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblina_port.so")

REF_SOR, JACOBI, MC_SOR = 0, 2, 3
_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is not None:
        return _lib
    L = C.CDLL(LIB_PATH)
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    sig = {
        "port_amg_new": (vp, [C.c_int, C.c_int, C.c_double, C.c_int, C.c_int]),
        "port_amg_set_level": (C.c_int, [vp, C.c_int, C.c_int, ip, ip, dp, ip, ip, ip, dp, ip, ip, dp, C.c_int]),
        "port_amg_finalize": (C.c_int, [vp]),
        "port_amg_free": (None, [vp]),
        "port_amg_colouring": (C.c_int, [vp, C.c_int, ip]),
        "port_vcycle": (None, [vp, dp, dp]),
        "port_pcg": (C.c_int, [vp, dp, dp, C.c_double, C.c_int, C.c_int, C.c_double, dp]),
        "port_spmv": (None, [vp, C.c_int, dp, dp]),
        "port_ilu0": (C.c_int, [C.c_int, ip, ip, dp, dp]),
        "port_bicgstab_ilu": (C.c_int, [C.c_int, ip, ip, dp, dp, dp, dp, C.c_double, C.c_int, C.c_int, dp]),
        "port_amg_setup": (C.c_int, [vp, C.c_int, ip, ip, dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                     C.c_double]),
        "port_amg_level_info": (C.c_int, [vp, C.c_int, ip, C.POINTER(C.c_long), C.POINTER(C.c_long),
                                          C.POINTER(C.c_long)]),
        "port_amg_level_export": (C.c_int, [vp, C.c_int, ip, ip, ip, dp, ip, ip, dp, ip, ip, dp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _ip(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def ilu0(indptr, indices, data):
    """ILU(0) factors on A's pattern (the C restatement); raises ArithmeticError on a zero pivot."""
    ptr = np.ascontiguousarray(indptr, dtype=np.int32)
    col = np.ascontiguousarray(indices, dtype=np.int32)
    val = np.ascontiguousarray(data, dtype=np.float64)
    f = np.zeros(max(len(col), 1))
    rc = lib().port_ilu0(len(ptr) - 1, _ip(ptr), _ip(col), _dp(val), _dp(f))
    if rc != 1:
        raise ArithmeticError("ILU(0): zero pivot" if rc == 0 else "ILU(0): out of memory")
    return f[:len(col)]


def bicgstab_ilu(indptr, indices, data, b, eps=1e-8, max_iter=1000, factors=None, x0=None):
    """BiCGStab_solve with the ILU(0) preconditioner (the C restatement); returns (x, iterations,
    ||R|| / ||R0||).  ``factors`` from ilu0() may be passed to skip the factorisation."""
    ptr = np.ascontiguousarray(indptr, dtype=np.int32)
    col = np.ascontiguousarray(indices, dtype=np.int32)
    val = np.ascontiguousarray(data, dtype=np.float64)
    f = ilu0(ptr, col, val) if factors is None else np.ascontiguousarray(factors, dtype=np.float64)
    n = len(ptr) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    rel = C.c_double()
    it = lib().port_bicgstab_ilu(n, _ip(ptr), _ip(col), _dp(val), _dp(f), _dp(bb), _dp(x), eps, max_iter, 1,
                                 C.byref(rel))
    if it < 0:
        raise MemoryError("BiCGStab: out of memory")
    return x, it, rel.value


class PortAMG:
    """Solve-phase restatement on a given hierarchy.

    ``levels`` is a list indexed like the reference (0 = coarsest) of dicts with
    keys A=(ptr, col, val) and, for levels > 0, labels, P, R.
    """

    def __init__(self, levels, smoother=MC_SOR, omega=1.0, nu=2, nu_finest=2):
        self.depth = len(levels)
        self.h = lib().port_amg_new(self.depth, smoother, omega, nu, nu_finest)
        self._keep = []
        for l, lv in enumerate(levels):
            A = [np.ascontiguousarray(a) for a in (lv["A"][0].astype(np.int32), lv["A"][1].astype(np.int32),
                                                    lv["A"][2].astype(np.float64))]
            n = len(A[0]) - 1
            if l > 0:
                lab = np.ascontiguousarray(lv["labels"], dtype=np.int32)
                P = [np.ascontiguousarray(lv["P"][0], dtype=np.int32), np.ascontiguousarray(lv["P"][1], dtype=np.int32),
                     np.ascontiguousarray(lv["P"][2], dtype=np.float64)]
                R = [np.ascontiguousarray(lv["R"][0], dtype=np.int32), np.ascontiguousarray(lv["R"][1], dtype=np.int32),
                     np.ascontiguousarray(lv["R"][2], dtype=np.float64)]
                nc = len(R[0]) - 1
            else:
                lab, P, R, nc = None, [None] * 3, [None] * 3, 0
            rc = lib().port_amg_set_level(self.h, l, n, _ip(A[0]), _ip(A[1]), _dp(A[2]), _ip(lab), _ip(P[0]),
                                          _ip(P[1]), _dp(P[2]), _ip(R[0]), _ip(R[1]), _dp(R[2]), nc)
            if rc:
                raise RuntimeError("port_amg_set_level failed")
        rc = lib().port_amg_finalize(self.h)
        if rc:
            raise RuntimeError(f"port_amg_finalize failed ({rc})")
        self.n = len(levels[-1]["A"][0]) - 1

    @classmethod
    def setup(cls, system, depth, coarsening=2, matrix_tol=0.1, smoother=MC_SOR, omega=1.0, nu=2, nu_finest=2,
              eps_minus=0.3, eps_plus=0.5):
        """AMG_setup restated in C (amg_setup_port.c) on a CSR system (indptr, indices, data, dof):
        the hierarchy is built by the oracle itself, without the GPU library."""
        self = cls.__new__(cls)
        self.depth = depth
        self._keep = []
        self.h = lib().port_amg_new(depth, smoother, omega, nu, nu_finest)
        ptr = np.ascontiguousarray(system.indptr, dtype=np.int32)
        col = np.ascontiguousarray(system.indices, dtype=np.int32)
        val = np.ascontiguousarray(system.data, dtype=np.float64)
        rc = lib().port_amg_setup(self.h, len(ptr) - 1, _ip(ptr), _ip(col), _dp(val), int(system.dof), depth,
                                  coarsening, eps_minus, eps_plus, matrix_tol)
        if rc:
            raise RuntimeError(f"port_amg_setup failed ({rc})")
        self.n = len(ptr) - 1
        return self

    def level_sizes(self, l):
        n, a, p, r = C.c_int(), C.c_long(), C.c_long(), C.c_long()
        if lib().port_amg_level_info(self.h, l, C.byref(n), C.byref(a), C.byref(p), C.byref(r)):
            raise IndexError(l)
        return n.value, a.value, p.value, r.value

    def sizes(self):
        return [self.level_sizes(l)[0] for l in range(self.depth)]

    def level(self, l):
        """Host copy of level l: an object with A, P, R (CSR triples) and labels (None on level 0)."""
        n, na, np_, nr = self.level_sizes(l)
        A = (np.zeros(n + 1, np.int32), np.zeros(max(na, 1), np.int32), np.zeros(max(na, 1)))
        lab = P = R = None
        if l > 0:
            nc = self.level_sizes(l - 1)[0]
            lab = np.zeros(n, np.int32)
            P = (np.zeros(n + 1, np.int32), np.zeros(max(np_, 1), np.int32), np.zeros(max(np_, 1)))
            R = (np.zeros(nc + 1, np.int32), np.zeros(max(nr, 1), np.int32), np.zeros(max(nr, 1)))
        Pp = (_ip(P[0]), _ip(P[1]), _dp(P[2])) if P else (None, None, None)
        Rp = (_ip(R[0]), _ip(R[1]), _dp(R[2])) if R else (None, None, None)
        if lib().port_amg_level_export(self.h, l, _ip(lab), _ip(A[0]), _ip(A[1]), _dp(A[2]), *Pp, *Rp):
            raise IndexError(l)
        return SimpleNamespace(n=n, A=(A[0], A[1][:na], A[2][:na]), labels=lab,
                               P=(P[0], P[1][:np_], P[2][:np_]) if P else None,
                               R=(R[0], R[1][:nr], R[2][:nr]) if R else None)

    def vcycle(self, r):
        rr = np.ascontiguousarray(r, dtype=np.float64)
        z = np.zeros(self.n)
        lib().port_vcycle(self.h, _dp(rr), _dp(z))
        return z

    def pcg(self, b, tol=1e-8, max_iter=1000, stop_rule=0, max_seconds=0.0, x0=None):
        bb = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.n) if x0 is None else np.array(x0, dtype=np.float64)
        res = C.c_double(0.0)
        it = lib().port_pcg(self.h, _dp(bb), _dp(x), tol, max_iter, stop_rule, max_seconds, C.byref(res))
        return x, it, res.value

    def colouring(self, l):
        n = None
        # the level size is the length of its row pointer minus one; callers pass the level's n
        raise NotImplementedError

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.port_amg_free(self.h)
            self.h = None


def levels_from_golden(g):
    """Hierarchy dict list from a golden npz (tests/golden/*.npz)."""
    depth = int(g["depth"])
    out = []
    for l in range(depth):
        d = {"A": (g[f"L{l}_A_ptr"], g[f"L{l}_A_col"], g[f"L{l}_A_val"])}
        if l > 0:
            d["labels"] = g[f"L{l}_labels"]
            d["P"] = (g[f"L{l}_P_ptr"], g[f"L{l}_P_col"], g[f"L{l}_P_val"])
            d["R"] = (g[f"L{l}_R_ptr"], g[f"L{l}_R_col"], g[f"L{l}_R_val"])
        out.append(d)
    return out


def levels_from_amg(amg):
    """Hierarchy dict list from a fem_gb300.lina.AMG handle (host copy of the setup)."""
    out = []
    for l in range(amg.depth):
        L = amg.level(l)
        d = {"A": L.A}
        if l > 0:
            d["labels"], d["P"], d["R"] = L.labels, L.P, L.R
        out.append(d)
    return out
