"""CPU restatement of the reference's sparse_product (LinA/linear_algebra.c:186-222) on CSR.

Test infrastructure only (the oracle): pure-Python loops, for small matrices.  Row i of
C = A B starts as the entry (i, 0.0); for every nonzero a_ik in A's stored order and every
nonzero b_kj in B's stored order, a_ik * b_kj starts column j or is added to it (rounded one
operation at a time, as IEEE doubles); the row is sorted by column; delete_zeros
(linear_algebra.c:793, with remove_element_at :1161-1178) then drops exact zeros from rows of
more than one entry and leaves an emptied row as (i, 0.0).
"""
from __future__ import annotations

import numpy as np


def sparse_product(a, b):
    """a, b: (indptr, indices, data) triples; returns C's triple."""
    ap, ac, av = a
    bp, bc, bv = b
    n = len(ap) - 1
    ptr = [0]
    cols, vals = [], []
    for i in range(n):
        acc = {i: 0.0}
        for p in range(ap[i], ap[i + 1]):
            x = float(av[p])
            if x == 0.0:
                continue
            k = int(ac[p])
            for r in range(bp[k], bp[k + 1]):
                y = float(bv[r])
                if y == 0.0:
                    continue
                j = int(bc[r])
                acc[j] = acc[j] + x * y if j in acc else x * y
        row = sorted(acc.items())
        if len(row) > 1:
            row = [(j, v) for j, v in row if v != 0.0] or [(i, 0.0)]
        for j, v in row:
            cols.append(j)
            vals.append(v)
        ptr.append(len(cols))
    return np.array(ptr, np.int32), np.array(cols, np.int32), np.array(vals, np.float64)


def square_clean(c, n):
    """square_matrix_clean (linear_algebra.c:3100) as applied to a Galerkin product: entries in
    columns >= n must be zero and are dropped, zeros off the diagonal are dropped, an emptied row
    becomes (i, 0.0)."""
    cp, cc, cv = c
    ptr, cols, vals = [0], [], []
    for i in range(n):
        row = []
        for p in range(cp[i], cp[i + 1]):
            j, v = int(cc[p]), float(cv[p])
            if j >= n:
                assert v == 0.0
                continue
            if v == 0.0 and j != i:
                continue
            row.append((j, v))
        if not row:
            row = [(i, 0.0)]
        for j, v in row:
            cols.append(j)
            vals.append(v)
        ptr.append(len(cols))
    return np.array(ptr, np.int32), np.array(cols, np.int32), np.array(vals, np.float64)
