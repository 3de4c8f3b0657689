"""Single-kernel runs on the finest matrix of the benchmark workload (for profiling).

    python -m fem_gb300.kernel_bench --m 1025 --reps 3

Builds the degraded plane-strain elasticity matrix (m x m nodes, 2 m^2
unknowns), uploads it as one device matrix (SELL-32, ~0.5 GB for m = 1025)
and runs `reps` FP32 and `reps` FP64 damped-Jacobi sweeps and SpMVs, so that a
profiler can capture them in isolation with little device memory in use.
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
    args = ap.parse_args()
    s = problems.elasticity_p1(args.m)
    M = lina.Matrix(s.n, s.indptr, s.indices, s.data)
    out = {}
    for prec, dt in ((lina.PREC_MIXED, np.float32), (lina.PREC_FP64, np.float64)):
        b = lina.DeviceArray.from_host(s.b.astype(dt))
        x = lina.DeviceArray.from_host(np.zeros(s.n, dt))
        t = lina.DeviceArray(s.n, dt)
        t0 = time.perf_counter()
        M.jacobi_device(b, x, t, 0.6, args.reps, prec)
        out[f"jacobi_{dt.__name__}_ms"] = (time.perf_counter() - t0) * 1e3 / max(args.reps, 1)
        t0 = time.perf_counter()
        for _ in range(args.reps):
            M.spmv_device(b, t, prec)
        out[f"spmv_{dt.__name__}_ms"] = (time.perf_counter() - t0) * 1e3 / max(args.reps, 1)
    out.update(n=s.n, nnz=int(s.nnz), padded=int(M.padded_entries))
    print(out)


if __name__ == "__main__":
    main()
