"""CPU restatement of the reference's ILU(0) factorisation on CSR.

Test infrastructure only (the oracle): pure-Python loops, for small matrices.  It follows
incomplete_LU_factorization (LinA/linear_algebra.c:1952-1982) with row_times_row (:1795-1818):
row by row, for the entries a_ij of row i in column order,

    L_ij = a_ij - sum_{k<j} L_ik U_kj                     (j <= i)
    U_ij = (a_ij - sum_{k<i} L_ik U_kj) / L_ii            (j > i; a zero or absent L_ii fails)

where a product term exists when (i, k) and (k, j) are both in A's pattern, the terms are added
in ascending k to a sum that starts at 0, and every product and sum is rounded on its own (IEEE
doubles, no fused multiply-add).  The factors are returned on A's pattern: L_ij where j <= i,
U_ij where j > i (U's unit diagonal is not stored).
"""
from __future__ import annotations

import numpy as np


class ZeroPivot(ArithmeticError):
    """incomplete_LU_factorization returned 0: L_ii was zero for a row with entries right of the diagonal."""


def ilu0(indptr, indices, data):
    ptr = [int(v) for v in indptr]
    col = [int(v) for v in indices]
    a = [float(v) for v in data]
    n = len(ptr) - 1
    f = [0.0] * len(a)
    upper = [dict() for _ in range(n)]  # row k: column j > k -> position of U_kj
    for i in range(n):
        r0, r1 = ptr[i], ptr[i + 1]
        diag = None
        for p in range(r0, r1):
            j = col[p]
            jmax = j - 1 if j <= i else i - 1
            s = 0.0
            for q in range(r0, r1):
                k = col[q]
                if k > jmax:
                    break
                pos = upper[k].get(j)
                if pos is not None:
                    s += f[q] * f[pos]
            v = a[p] - s
            if j <= i:
                f[p] = v
                if j == i:
                    diag = v
            else:
                if not diag:
                    raise ZeroPivot(f"zero pivot in row {i}")
                f[p] = v / diag
                upper[i][j] = p
    return np.array(f, dtype=np.float64)
