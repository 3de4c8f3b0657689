"""Single-kernel runs on one matrix of the benchmark workload (for profiling).

    python -m fem_gb300.kernel_bench --m 1025 --reps 3              # finest matrix
    python -m fem_gb300.kernel_bench --m 1025 --level 8 --reps 3    # a level of the AMG hierarchy
    python -m fem_gb300.kernel_bench --m 1025 --solve --reps 2      # whole mixed-precision solves
    python -m fem_gb300.kernel_bench --solve --poisson --reps 3     # whole FP64 solves of P1 Poisson 257 x 257
    python -m fem_gb300.kernel_bench --segbatch 24 --reps 2         # a segmented batch, host-launched

Builds the degraded plane-strain elasticity matrix (m x m nodes, 2 m^2 unknowns) or, with
--level, the AMG hierarchy of the benchmark (standard coarsening, depth 10, matrix tolerance
0.1) on the host, uploads that one matrix as a device matrix in the library's layout, and runs
`reps` FP32 and `reps` FP64 damped-Jacobi sweeps and SpMVs, so that a profiler can capture them
in isolation with little device memory in use.

--solve instead builds the benchmark's device hierarchy (damped Jacobi, omega 0.6, mixed precision) and
runs `reps` AMG-PCG solves to the relative residual 1e-8, each iteration launched from the host rather
than from the captured graph (a profiler cannot see the kernels of a graph with conditional nodes).
With --poisson the solves are those of the P1 Poisson workload (257 x 257 nodes, aggressive coarsening,
depth 6, 2 + 2 multicolour-SOR sweeps with omega 1, FP64, stopping rule ||r|| / ||M^-1 r0|| <= 1e-8);
--mixed runs its V-cycle in FP32 instead (for comparison: the workload itself is FP64).

--segbatch K builds the first K systems of the batched workload (seeded Delaunay meshes, the workload's
hierarchy settings: standard coarsening, matrix_tol 0.3, multicolour SOR, mixed precision), their
segmented batch, and runs `reps` of its iterations launched from the host.
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
    ap.add_argument("--dense-inverse", type=str, default="",
                    help="comma-separated sizes m: time the device inverse of a dense m x m block with FP64 CUDA "
                         "cores and with FP64 tensor cores instead")
    ap.add_argument("--solve", action="store_true", help="whole solves, launched iteration by iteration")
    ap.add_argument("--poisson", action="store_true", help="with --solve: the P1 Poisson 257 x 257 workload")
    ap.add_argument("--mixed", action="store_true", help="with --solve --poisson: the FP32 V-cycle instead of FP64")
    ap.add_argument("--segbatch", type=int, default=0, help="a segmented batch of this many workload systems")
    args = ap.parse_args()
    if args.solve:
        solve(args)
        return
    if args.segbatch:
        segbatch(args.segbatch, args.reps)
        return
    if args.dense_inverse:
        dense_inverse(int(v) for v in args.dense_inverse.split(","))
        return
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


def solve(args):
    lina.set_sell_index_bits(args.sell_bits)
    if args.poisson:
        s = problems.poisson_p1(257, seed=0)
        amg = lina.AMG.from_system(s, depth=6, coarsening=lina.AGGRESSIVE, smoother=lina.SMOOTHER_MC_SOR,
                                   omega=1.0, precision=lina.PREC_MIXED if args.mixed else lina.PREC_FP64)
        stop, flags = lina.STOP_REFERENCE, lina.PCG_NORMALIZE | lina.PCG_FINAL_PRECON
    else:
        s = problems.elasticity_p1(args.m)
        amg = lina.AMG.from_system(s, depth=args.depth, coarsening=lina.STANDARD, smoother=lina.SMOOTHER_JACOBI,
                                   omega=0.6, precision=lina.PREC_MIXED, matrix_tol=args.matrix_tol)
        stop, flags = lina.STOP_RELATIVE, 0
    if args.poisson:
        print({"level_sizes": amg.sizes(),
               "colours": [int(amg.colours(l).max()) + 1 for l in range(1, amg.depth)]}, flush=True)
    b = lina.DeviceArray.from_host(s.b)
    x = lina.DeviceArray(s.n)
    for _ in range(args.reps):
        t0 = time.perf_counter()
        info = amg.pcg_device(b, x, tol=1e-8, max_iter=2000, stop=stop, flags=flags | lina.PCG_HOST_LOOP)
        print({"iterations": info.iterations, "status": info.status, "ms": (time.perf_counter() - t0) * 1e3,
               "launches": lina.launches()}, flush=True)
    amg.close()


def segbatch(count, iterations):
    plan = problems.batch_plan(96, seed=0)[:count]
    systems = [problems.batch_system(*p) for p in plan]
    amgs = [lina.AMG.from_system(s, depth=problems.batch_depth(s.n), coarsening=lina.STANDARD,
                                 smoother=lina.SMOOTHER_MC_SOR, omega=1.0, precision=lina.PREC_MIXED, matrix_tol=0.3)
            for s in systems]
    bd = [lina.DeviceArray.from_host(s.b) for s in systems]
    seg = lina.SegmentedBatch(amgs)
    rows, ents = seg.levels()
    t0 = time.perf_counter()
    seg.solve(bd, tol=1e-8, max_iter=iterations, device=True, host_loop=True)
    print({"systems": count, "depths": [a.depth for a in amgs], "level_rows": rows, "level_entries": ents,
           "iterations": iterations, "ms": (time.perf_counter() - t0) * 1e3}, flush=True)


def dense_inverse(sizes, reps=3):
    """Blocked Gauss-Jordan inverse of diagonally dominant m x m blocks: device time per inverse with the
    rank-32 updates on FP64 CUDA cores (SIMT) and on FP64 tensor cores (DMMA); 2 m^3 flops each."""
    for m in sizes:
        rng = np.random.default_rng(m)
        a = rng.uniform(-1, 1, (m, m))
        a += np.diag(np.abs(a).sum(axis=1) + 1.0)
        row = {"m": m}
        for name, method in (("simt", lina.DENSE_SIMT), ("dmma", lina.DENSE_DMMA)):
            ts = []
            for _ in range(reps):
                d = lina.DeviceArray.from_host(a.ravel())
                ts.append(lina.dense_inverse_device(d, m, method))
            ms = min(ts)
            row[f"{name}_ms"] = ms
            row[f"{name}_tflops"] = 2.0 * m ** 3 / (ms * 1e-3) / 1e12
        print(row, flush=True)


if __name__ == "__main__":
    main()
