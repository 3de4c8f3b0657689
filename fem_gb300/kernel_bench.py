"""Single-kernel runs on one matrix of the benchmark workload (for profiling).

    python -m fem_gb300.kernel_bench --m 1025 --reps 3              # finest matrix
    python -m fem_gb300.kernel_bench --m 1025 --level 8 --reps 3    # a level of the AMG hierarchy

Builds the degraded plane-strain elasticity matrix (m x m nodes, 2 m^2 unknowns) or, with
--level, the AMG hierarchy of the benchmark (standard coarsening, depth 10, matrix tolerance
0.1) on the host, uploads that one matrix as a device matrix in the library's layout, and runs
`reps` FP32 and `reps` FP64 damped-Jacobi sweeps and SpMVs, so that a profiler can capture them
in isolation with little device memory in use.
"""
from __future__ import annotations

import argparse
import time

import numpy as np

from fem_gb300 import lina, problems


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--m", type=int, default=1025)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--level", type=int, default=-1, help="AMG level (default: the finest matrix itself)")
    ap.add_argument("--depth", type=int, default=10)
    ap.add_argument("--matrix-tol", type=float, default=0.1)
    ap.add_argument("--sell-bits", type=int, default=16, choices=[16, 32], help="SELL-32 column-index width")
    args = ap.parse_args()
    lina.set_sell_index_bits(args.sell_bits)
    s = problems.elasticity_p1(args.m)
    if args.level >= 0:
        amg = lina.AMG.from_system(s, depth=args.depth, coarsening=lina.STANDARD, matrix_tol=args.matrix_tol,
                                   host_only=True)
        L = amg.level(args.level)
        n, (ip, ix, dv) = L.n, L.A
        amg.close()
    else:
        n, ip, ix, dv = s.n, s.indptr, s.indices, s.data
    M = lina.Matrix(n, ip, ix, dv)
    out = {}
    for prec, dt in ((lina.PREC_MIXED, np.float32), (lina.PREC_FP64, np.float64)):
        b = lina.DeviceArray.from_host(np.ones(n, dt))
        x = lina.DeviceArray.from_host(np.zeros(n, dt))
        t = lina.DeviceArray(n, dt)
        t0 = time.perf_counter()
        M.jacobi_device(b, x, t, 0.6, args.reps, prec)
        out[f"jacobi_{dt.__name__}_ms"] = (time.perf_counter() - t0) * 1e3 / max(args.reps, 1)
        t0 = time.perf_counter()
        for _ in range(args.reps):
            M.spmv_device(b, t, prec)
        out[f"spmv_{dt.__name__}_ms"] = (time.perf_counter() - t0) * 1e3 / max(args.reps, 1)
    out.update(level=args.level, n=n, nnz=int(ip[-1]), padded=int(M.padded_entries),
               index_bits=M.index_bits())
    print(out)


if __name__ == "__main__":
    main()
