"""Benchmark of the LinA sparse solve path on one GB300.

Workload (the configuration the headline metric is quoted on): plane-strain
P1 elasticity on a 1025 x 1025 node grid of the unit square, 2,101,250
unknowns (block ordering [u_x, u_y]), ~29.3M stored nonzeros, E = 210,
nu = 0.3, stiffness degraded by (1-d)^2 + 1e-6 around a notch from (0, 0.5)
to (0.5, 0.5) with d = exp(-dist / 2h); bottom edge clamped, top edge
u_y = 1e-3.  AMG setup as the reference's AMG_setup with standard coarsening
and dof = 2; one V-cycle per iteration (2 pre + 2 post sweeps) inside CG.

A step is one complete solve to the true relative residual 1e-8 with the
mixed-precision preconditioner (FP32 V-cycle, FP64 coarse solve, FP64
flexible CG).  ``value`` is solves/s with the matrix hierarchy and the
right-hand side already in HBM; ``e2e`` is the same solve through the C-ABI
with host buffers (pinned), so the H2D copy of b and the D2H copy of x are in
the timed region.  The same GPU's plain FP64 path and the CPU baseline are
measured in the same run.  The finest-level matrix (~235 MB FP32 values and
indices, ~352 MB FP64) exceeds the 129 MB L2, so no L2 flush is needed
between steps.

``--impl reference`` times the CPU implementation of the reference's solve
(the CPU restatement in oracle/, bit-exact to the reference on its golden
vectors, or the reference itself where it was built here) on the same
workload and prints the same metric.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "AMG-PCG solves/s at 2.1M dofs to rel-res 1e-8: mixed vs FP64 GPU; HBM GB/s"
DEFAULT_DEPTH = {65: 5, 129: 6, 257: 8, 513: 9, 1025: 10}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=None,
                   help="timed steps (default 20; 5 for --impl reference, whose steps are CPU solves)")
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--m", type=int, default=1025, help="grid nodes per side")
    p.add_argument("--depth", type=int, default=0)
    p.add_argument("--smoother", default="jacobi", choices=["jacobi", "mcsor"])
    p.add_argument("--omega", type=float, default=0.0)
    p.add_argument("--tol", type=float, default=1e-8)
    p.add_argument("--matrix-tol", type=float, default=0.1,
                   help="interpolation truncation (AMG_set_matrix_tolerance); 0.1 is the reference default")
    p.add_argument("--cpu-seconds", type=float, default=20.0, help="bound of the CPU baseline sample")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--ref-sor", type=int, default=1,
                   help="reference arm: also time one solve with the reference's lexicographic SOR (1) or not (0)")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--workload", default="elasticity", choices=["elasticity", "poisson", "damage", "adjoint", "batch"],
                   help="elasticity: the headline AMG-PCG solve (default); poisson: the 257 x 257 P1 Poisson "
                        "system in FP64 (66,049 unknowns); damage: the reflective-Newton "
                        "damage step on the same mesh; adjoint: the material-identification gradient; "
                        "batch: independent unstructured systems solved in one graph launch")
    p.add_argument("--coarsening", default="standard", choices=["standard", "pmis"],
                   help="standard: the reference's sequential coarsening (default); pmis: labels computed on "
                        "the GPU (opt-in, other hierarchies)")
    p.add_argument("--sell-bits", type=int, default=16, choices=[16, 32],
                   help="column-index width of the SELL-32 matrices (16: offsets from two bases per slice)")
    p.add_argument("--batch-count", type=int, default=96, help="systems of the batch workload")
    p.add_argument("--batch-matrix-tol", type=float, default=0.3,
                   help="interpolation truncation of the batch workload's hierarchies (with 0.1 the "
                        "high-contrast elasticity systems need far more iterations)")
    a = p.parse_args()
    if a.steps is None:
        a.steps = 5 if a.impl == "reference" else 20
    return a


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples every 200 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "", 1).isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "", 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if line.startswith("dram_bytes_per_launch_full_size:"):
                return float(line.split(":", 1)[1])
    return None


def build_system(m):
    from fem_gb300 import problems
    return problems.elasticity_p1(m)


def cpu_baseline(args, s, depth, omega):
    """The CPU baseline: the reference's set-up and FP64 pcg restated in C (oracle/), OpenMP over the host
    cores, on the same system and settings; whole solves, as many as fit the time bound (at least one).
    Returns the cpu_baseline record and the last solution (the FP64 oracle solution of this system)."""
    from oracle import port
    kind = port.JACOBI if args.smoother == "jacobi" else port.MC_SOR
    t0 = time.perf_counter()
    P = port.PortAMG.setup(s, depth, 2, args.matrix_tol, kind, omega, 2, 2)
    setup_s = time.perf_counter() - t0
    times, its, x = [], [], None
    while not times or (sum(times) < args.cpu_seconds and len(times) < 20):
        t0 = time.perf_counter()
        x, it, _ = P.pcg(s.b, args.tol, 2000, 1)
        times.append(time.perf_counter() - t0)
        its.append(it)
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    rec = {"value": len(times) / sum(times), "unit": "solves/s", "cores": cores, "kind": "port",
           "sample": f"{len(times)} whole FP64 solves ({its[0]} PCG iterations each, {sum(times):.1f} s) on the "
                     f"hierarchy of the restated AMG_setup ({setup_s:.1f} s, not timed)",
           "iterations": its[0], "setup_s": setup_s}
    return rec, x


def reference_api_e2e(args, s, depth, omega, world):
    """Solves through the drop-in LinA API on host arrays: AMG_setup on the row-list matrix, PCG_default,
    PCG_set_AMG_data, PCG_set_precon(PCG_AMG_vcycle_precon) and pcg (which then runs on the device), mixed
    precision, the reference's stopping rule ||r|| / ||M^-1 r0|| <= tol.  Each step is one pcg call from
    X = 0 with host B and X (their copies to and from the device inside the call)."""
    from fem_gb300 import lina
    L = lina.dropin()
    A = lina.RowListView(s.indptr, s.indices, s.data)
    L.AMG_print_info(0)
    L.AMG_set_matrix_tolerance(args.matrix_tol)
    L.AMG_set_SOR_relaxation_coeff(omega)
    sm = L.AMG_damped_Jacobi_smoother if args.smoother == "jacobi" else L.AMG_SOR_smoother
    L.AMG_set_smoother(ctypes.cast(sm, ctypes.c_void_p))
    L.AMG_gpu_set_precision(1)
    coarsening = 2  # STANDARD
    t0 = time.perf_counter()
    data = L.AMG_setup(A.ref, int(s.dof), depth, 2, 2, coarsening, 0, 1, None, None)
    setup_s = time.perf_counter() - t0
    if not data:
        raise RuntimeError("AMG_setup through the drop-in API failed")
    L.PCG_default(A.ref, None, None)
    L.PCG_set_AMG_data(data)
    L.PCG_set_precon(ctypes.cast(L.PCG_AMG_vcycle_precon, ctypes.c_void_p))
    b = np.ascontiguousarray(s.b, dtype=np.float64)
    x = np.zeros(s.n)
    dp = ctypes.POINTER(ctypes.c_double)
    bp, xp = b.ctypes.data_as(dp), x.ctypes.data_as(dp)
    times, its = [], []
    for k in range(args.warmup + args.steps):
        x[:] = 0.0
        t0 = time.perf_counter()
        it = L.pcg(xp, bp, s.n, args.tol, 2000)
        dt = time.perf_counter() - t0
        if it < 0:
            raise RuntimeError("pcg through the drop-in API failed")
        if k >= args.warmup:
            times.append(dt)
            its.append(it)
    trr = float(np.linalg.norm(s.b - _csr_matvec(s)(x)) / np.linalg.norm(s.b))
    L.AMG_free_data(data)
    value = world * len(times) / max_over_ranks(sum(times), world)
    return {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 16 * s.n, "d2h_bytes_per_step": 8 * s.n,
            "api": "AMG_setup + PCG_default + PCG_set_AMG_data + PCG_set_precon(PCG_AMG_vcycle_precon) + pcg on host "
                   "arrays (drop-in LinA API), mixed precision",
            "stop_rule": f"reference: ||r|| / ||M^-1 r0|| <= {args.tol:g}", "iterations": its,
            "true_rel_residual": trr, "pcg_residuum": float(L.get_pcg_residuum()), "setup_s": setup_s}


def reference_digest(m):
    """The reference's own results for the benchmark system, if committed (tests/golden)."""
    path = os.path.join(ROOT, "tests", "golden", f"elast{m}_digest.npz")
    if not os.path.exists(path):
        return None
    return np.load(path)


def run_gb300(args, rank, world, local):
    from fem_gb300 import lina
    m = args.m
    depth = args.depth or DEFAULT_DEPTH.get(m, 8)
    smoother = lina.SMOOTHER_JACOBI if args.smoother == "jacobi" else lina.SMOOTHER_MC_SOR
    omega = args.omega or (0.6 if args.smoother == "jacobi" else 1.0)
    if lina.lib().lina_gpu_device_count() < 1:
        raise SystemExit("no CUDA device")
    s = build_system(m)
    t0 = time.perf_counter()
    coarsening = lina.PMIS if args.coarsening == "pmis" else lina.STANDARD
    amg = lina.AMG.from_system(s, depth=depth, coarsening=coarsening, smoother=smoother, omega=omega,
                               precision=lina.PREC_MIXED, matrix_tol=args.matrix_tol)
    setup_s = time.perf_counter() - t0
    n = s.n
    b_dev = lina.DeviceArray.from_host(s.b)
    x_dev = lina.DeviceArray(n)

    def solve_dev(flags=0):
        return amg.pcg_device(b_dev, x_dev, tol=args.tol, max_iter=2000, stop=lina.STOP_RELATIVE, flags=flags)

    for _ in range(args.warmup):
        solve_dev()
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    lina.lib().lina_gpu_synchronize()
    launches0 = lina.launches()
    amg.timer_begin()
    infos = [solve_dev() for _ in range(args.steps)]
    ms = amg.timer_end()
    launches = lina.launches() - launches0
    clocks.stop()
    ms = max_over_ranks(ms, world)
    value = world * args.steps / (ms / 1e3)
    it_mixed = [i.iterations for i in infos]
    trr = max(i.true_rel_residual for i in infos)
    # kernel timing: the same solves again, driven iteration by iteration from the host with
    # CUDA events (on the library's stream) around every smoother sweep of the level with the most
    # stored entries, whose sweeps are the largest share of an iteration
    x_mixed = x_dev.to_host()
    kinfos = [solve_dev(lina.PCG_TIME_KERNELS) for _ in range(args.steps)]
    sm_ms = sum(i.smoother_ms for i in kinfos)
    sm_n = sum(i.smoother_launches for i in kinfos)
    sm_bytes = kinfos[0].smoother_bytes
    peak, peak_kind = measured_peaks()
    achieved = sm_bytes / (sm_ms / sm_n / 1e3) / 1e9 if sm_n else None

    # end to end through the C-ABI with pinned host buffers
    hb = lina.PinnedArray(n)
    hx = lina.PinnedArray(n)
    hb.array[:] = s.b
    e2e_ms = []
    for k in range(args.warmup + args.steps):
        info = lina.SolveInfo()
        amg.timer_begin()
        rc = lina.lib().lina_gpu_pcg(amg.h, hb.ptr, hx.ptr, args.tol, 2000, lina.STOP_RELATIVE, 0,
                                     ctypes.byref(info))
        t = amg.timer_end()
        if rc not in (0, -5):
            raise RuntimeError(lina.last_error())
        if k >= args.warmup:
            e2e_ms.append(t)
    e2e_value = world * len(e2e_ms) / (max_over_ranks(sum(e2e_ms), world) / 1e3)
    # end to end through the reference-facing drop-in API, as crack.c / FEM2D would call it
    api = reference_api_e2e(args, s, depth, omega, world)

    # the same GPU's plain FP64 path on the same hierarchy
    fp64 = None
    if not args.no_fp64:
        amg.set_smoother(smoother, omega, lina.PREC_FP64)
        for _ in range(max(1, args.warmup)):
            solve_dev()
        amg.timer_begin()
        i64 = [solve_dev() for _ in range(args.steps)]
        ms64 = max_over_ranks(amg.timer_end(), world)
        k64 = [solve_dev(lina.PCG_TIME_KERNELS) for _ in range(2)]
        sm64 = sum(i.smoother_ms for i in k64) / max(1, sum(i.smoother_launches for i in k64))
        x64 = x_dev.to_host()
        fp64 = {"value": world * args.steps / (ms64 / 1e3), "unit": "solves/s",
                "iterations": [i.iterations for i in i64],
                "true_rel_residual": max(i.true_rel_residual for i in i64),
                "smoother_gbs": k64[0].smoother_bytes / (sm64 / 1e3) / 1e9 if sm64 else None}
        amg.set_smoother(smoother, omega, lina.PREC_MIXED)

    # parity at this size: the reference's own FP64 pcg (its stopping rule ||r|| / ||M^-1 r0||) on the same
    # system, from the committed digest, against both GPU paths under the same rule; solution errors
    # against the FP64 oracle solution (the restated reference solve, whole vector) and against the
    # reference's tight solve (tolerance 1e-13, its committed subsample)
    parity = {}
    g = reference_digest(m) if (depth == 10 and args.matrix_tol == 0.1 and args.smoother == "jacobi"
                                and args.coarsening == "standard" and omega == 0.6) else None
    if g is not None:
        idx = g["sample_index"]
        xt = g["tight_xs"]
        ref_rule = {}
        for prec, name in ((lina.PREC_MIXED, "mixed"), (lina.PREC_FP64, "fp64")):
            amg.set_smoother(smoother, omega, prec)
            xr, ir = amg.pcg(s.b, tol=args.tol, max_iter=2000, stop=lina.STOP_REFERENCE,
                             flags=lina.PCG_NORMALIZE | lina.PCG_FINAL_PRECON)
            ref_rule[name] = {"iterations": ir.iterations,
                              "err_vs_ref_tight": float(np.linalg.norm(xr[idx] - xt) / np.linalg.norm(xt))}
        amg.set_smoother(smoother, omega, lina.PREC_MIXED)
        it_ref = int(g["pcg_jacobi_it"])
        # the device hierarchy (set-up with Galerkin products on the GPU) against the reference's,
        # SHA-256 of every level's labels, A, P and R
        from tests.golden import digest as D
        got = D.level_digest(amg.level, depth)
        mism = sorted(k for k, v in got.items() if v != str(g[f"sha_{k}"]))
        parity = {"hierarchy_sha256_equal_reference": not mism, "hierarchy_mismatches": mism[:5],
                  "reference_iterations": it_ref, "reference_rule": ref_rule,
                  "mixed_iterations_vs_reference": ref_rule["mixed"]["iterations"] / it_ref,
                  "err_vs_ref_tight": float(np.linalg.norm(x_mixed[idx] - xt) / np.linalg.norm(xt)),
                  "reference_sor_iterations": int(g["pcg_refsor_it"]) if "pcg_refsor_it" in g else None}
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu, x_port = cpu_baseline(args, s, depth, omega)
        parity["err_vs_fp64_oracle"] = float(np.linalg.norm(x_mixed - x_port) / np.linalg.norm(x_port))

    if cpu is not None and fp64 is not None:
        parity["fp64_err_vs_fp64_oracle"] = float(np.linalg.norm(x64 - x_port) / np.linalg.norm(x_port))
    traffic = profiled_traffic()
    sizes = amg.sizes()
    out = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 preconditioner / f64 Krylov",
        "data": "synthetic (seeded structured P1 mesh, notch damage field)",
        "config": workload_config(args, s, depth, omega, sizes),
        "parallelism": "replicas" if world > 1 else "single GPU", "sell_index_bits": args.sell_bits,
        "iterations": it_mixed, "restarts": max(i.restarts for i in infos), "true_rel_residual": trr,
        "dofs_per_s": value * n, "setup_s": setup_s, "parity": parity,
        "e2e": api,
        "e2e_c_abi": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n,
                      "api": "lina_gpu_pcg with pinned host buffers, relative rule"},
        "gpu_launches": int(launches),
        "fp64_gpu": fp64,
        "mixed_vs_fp64": (value / fp64["value"]) if fp64 else None,
        "roofline": {"bound": "hbm",
                     "kernel": f"level {kinfos[0].timed_level} FP32 damped-Jacobi sweep "
                               f"({kinfos[0].timed_rows} rows, {kinfos[0].timed_entries} stored entries; "
                               f"the level with the most entries)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "peak_kind": peak_kind,
                     "traffic": traffic, "bytes_per_launch": sm_bytes,
                     "avg_launch_us": (sm_ms / sm_n * 1e3) if sm_n else None},
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
    }
    if rank == 0:
        print(json.dumps(out))


def common_line(metric, value, unit, world, steps, warmup, ms, dtype, data, config, e2e, launches, clocks,
                higher=True):
    return {"metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": steps, "warmup": warmup,
            "ms_per_step": ms / steps, "higher_is_better": higher, "scaling": "weak", "vs_baseline": None,
            "dtype": dtype, "data": data, "config": config, "e2e": e2e, "gpu_launches": int(launches),
            "clocks": clocks.summary()}


def port_threads():
    """Host threads the OpenMP restatement uses."""
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def sweep_roofline(amg, b_dev, x_dev, tol, stop, flags, reps, what):
    """The smoother sweeps of a hierarchy's level with the most stored entries, timed live: the same solve
    driven iteration by iteration with CUDA events on the library's stream around every sweep of that
    level (every colour launch for multicolour SOR), reps solves.  Algorithmic bytes per launch as the
    library counts them (matrix entries with their column indices, x, b, 1/a_ii and the result; a colour
    launch carries its share of the sweep).  No ncu capture stands behind these: traffic is null."""
    from fem_gb300 import lina
    kinfos = [amg.pcg_device(b_dev, x_dev, tol=tol, max_iter=2000, stop=stop, flags=flags | lina.PCG_TIME_KERNELS)
              for _ in range(reps)]
    n = sum(i.smoother_launches for i in kinfos)
    ms = sum(i.smoother_ms for i in kinfos)
    if not n or ms <= 0:
        return None
    k = kinfos[0]
    peak, peak_kind = measured_peaks()
    achieved = k.smoother_bytes / (ms / n / 1e3) / 1e9
    return {"bound": "hbm", "kernel": f"{what}: smoother launches of level {k.timed_level} ({k.timed_rows} rows, "
                                      f"{k.timed_entries} stored entries; the level with the most entries)",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
            "traffic": None, "bytes_per_launch": k.smoother_bytes, "avg_launch_us": ms / n * 1e3, "launches": n}


def run_poisson(args, rank, world, local):
    """Plain FP64 AMG-PCG on the P1 Poisson system of a 257 x 257 grid (66,049 unknowns, homogeneous
    Dirichlet rows, right-hand side uniform in [-1, 1] from seed 0): aggressive coarsening, depth 6, one
    V-cycle of 2 + 2 multicolour-SOR sweeps (omega 1) per iteration, the reference's stopping rule
    ||r|| / ||M^-1 r0|| <= 1e-8.  value: device-resident solves; e2e: the drop-in pcg on host arrays; the
    CPU baseline: the restated reference set-up and pcg with its own lexicographic SOR."""
    from fem_gb300 import lina, problems
    from oracle import port
    m = 257
    s = problems.poisson_p1(m, seed=0)
    depth = 6
    amg = lina.AMG.from_system(s, depth=depth, coarsening=lina.AGGRESSIVE, smoother=lina.SMOOTHER_MC_SOR, omega=1.0,
                               precision=lina.PREC_FP64)
    b_dev = lina.DeviceArray.from_host(s.b)
    x_dev = lina.DeviceArray(s.n)
    flags = lina.PCG_NORMALIZE | lina.PCG_FINAL_PRECON

    def solve():
        return amg.pcg_device(b_dev, x_dev, tol=args.tol, max_iter=500, stop=lina.STOP_REFERENCE, flags=flags)

    for _ in range(args.warmup):
        solve()
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = lina.launches()
    amg.timer_begin()
    infos = [solve() for _ in range(args.steps)]
    ms = max_over_ranks(amg.timer_end(), world)
    launches = lina.launches() - launches0
    clocks.stop()
    x = x_dev.to_host()
    value = world * args.steps / (ms / 1e3)
    # the drop-in API on host arrays (FP64, the same smoother)
    L = lina.dropin()
    A = lina.RowListView(s.indptr, s.indices, s.data)
    L.AMG_print_info(0)
    L.AMG_set_matrix_tolerance(0.1)
    L.AMG_set_SOR_relaxation_coeff(1.0)
    L.AMG_set_smoother(ctypes.cast(L.AMG_SOR_smoother, ctypes.c_void_p))
    L.AMG_gpu_set_precision(0)
    data = L.AMG_setup(A.ref, 1, depth, 2, 2, 1, 0, 1, None, None)
    L.PCG_default(A.ref, None, None)
    L.PCG_set_AMG_data(data)
    L.PCG_set_precon(ctypes.cast(L.PCG_AMG_vcycle_precon, ctypes.c_void_p))
    bh = np.ascontiguousarray(s.b)
    xh = np.zeros(s.n)
    dp = ctypes.POINTER(ctypes.c_double)
    times, e2e_its = [], []
    for k in range(args.warmup + args.steps):
        xh[:] = 0.0
        t0 = time.perf_counter()
        e2e_its.append(L.pcg(xh.ctypes.data_as(dp), bh.ctypes.data_as(dp), s.n, args.tol, 500))
        if k >= args.warmup:
            times.append(time.perf_counter() - t0)
    L.AMG_free_data(data)
    e2e_value = world * len(times) / max_over_ranks(sum(times), world)
    # parity against the reference's own digest of this system
    parity = {}
    gpath = os.path.join(ROOT, "tests", "golden", "poisson257_digest.npz")
    if os.path.exists(gpath):
        g = np.load(gpath)
        idx = g["sample_index"]
        xt = g["tight_xs"]
        parity = {"reference_iterations_mcsor": int(g["pcg_mcsor_it"]),
                  "reference_iterations_lexicographic_sor": int(g["pcg_refsor_it"]),
                  "err_vs_ref_tight": float(np.linalg.norm(x[idx] - xt) / np.linalg.norm(xt)),
                  "err_vs_ref_same_tol": float(np.linalg.norm(x[idx] - g["pcg_mcsor_xs"]) /
                                               np.linalg.norm(g["pcg_mcsor_xs"]))}
    cpu = None
    if rank == 0 and not args.no_cpu:
        t0 = time.perf_counter()
        P = port.PortAMG.setup(s, depth, 1, 0.1, port.REF_SOR, 1.0, 2, 2)
        setup_s = time.perf_counter() - t0
        ts, its = [], []
        while not ts or (sum(ts) < args.cpu_seconds and len(ts) < 20):
            t0 = time.perf_counter()
            _, it, _ = P.pcg(s.b, args.tol, 500, 0)
            ts.append(time.perf_counter() - t0)
            its.append(it)
        cpu = {"value": len(ts) / sum(ts), "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": f"{len(ts)} whole solves with the reference's lexicographic SOR (serial, as the reference), "
                         f"{its[0]} PCG iterations each; restated set-up {setup_s:.1f} s (not timed)",
               "iterations": its[0]}
    out = common_line("AMG-PCG solves/s at 66k dofs (P1 Poisson 257 x 257, FP64) to the reference's rel-res 1e-8",
                      value, "solves/s", world, args.steps, args.warmup, ms, "f64",
                      "synthetic (seeded uniform right-hand side)",
                      {"workload": f"P1 Poisson {m}x{m} nodes, {s.n} dofs, aggressive coarsening, depth {depth}, "
                                   "one V-cycle of 2+2 multicolour-SOR sweeps (omega 1) per iteration, stopping "
                                   f"rule ||r||/||M^-1 r0|| <= {args.tol:g}; inputs resident (fit L2)",
                       "dofs": s.n, "nnz": int(s.nnz), "amg_depth": depth, "level_sizes": amg.sizes()},
                      {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": 16 * s.n,
                       "d2h_bytes_per_step": 8 * s.n, "api": "drop-in AMG_setup + PCG_set_AMG_data + "
                       "PCG_AMG_vcycle_precon + pcg on host arrays", "iterations": e2e_its[args.warmup:][:3]},
                      launches, clocks)
    out["iterations"] = [i.iterations for i in infos]
    out["parity"] = parity
    out["roofline"] = sweep_roofline(amg, b_dev, x_dev, args.tol, lina.STOP_REFERENCE, flags, 3,
                                     "FP64 multicolour-SOR colour sweeps (the level fits L2)")
    out["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(out))


def run_damage(args, rank, world, local):
    """Phase-field damage step (AT2 quadratic, 1025 x 1025 nodes, 1.05M unknowns, bounds
    d_prev <= d <= 1) by reflective Newton with the device BiCGStab + mixed-precision ILU(0) local
    solver, through the C-ABI with host arrays: a step is one full minimisation from the same start.
    gpu_launches counts the library's SpMV-family launches only."""
    from fem_gb300 import lina, problems
    q = problems.at2_damage(args.m)
    lo, up, x0 = q.meta["lower"], q.meta["upper"], q.meta["x0"]
    for _ in range(args.warmup):
        lina.reflective_newton(q, lo, up, x0)
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = lina.launches()
    t0 = time.perf_counter()
    its = [lina.reflective_newton(q, lo, up, x0)[1] for _ in range(args.steps)]
    ms = max_over_ranks((time.perf_counter() - t0) * 1e3, world)
    launches = lina.launches() - launches0
    clocks.stop()
    value = world * args.steps / (ms / 1e3)
    out = common_line("reflective-Newton damage minimisations/s at 1.05M dofs to rel. decrease 1e-8", value,
                      "solves/s", world, args.steps, args.warmup, ms, "f64 Newton / f32 ILU in f64 BiCGStab",
                      "synthetic (seeded AT2 history field, notch lower bound)",
                      {"workload": f"AT2 damage {args.m}x{args.m} nodes, {q.n} dofs, bounds d_prev <= d <= 1, "
                                   "reflective Newton with device BiCGStab + ILU(0)", "dofs": q.n,
                       "nnz": int(q.nnz)},
                      {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 8 * 3 * q.n,
                       "d2h_bytes_per_step": 8 * q.n}, launches, clocks)
    out["newton_steps"] = its
    # dominant kernel: the ILU(0) application (forward + backward triangular solve, FP32) inside every
    # BiCGStab iteration; timed with CUDA events on the handle's stream, on the ILU(0) of the Hessian
    # (the Newton systems D H D + diag(|g| J) keep its pattern and level schedule)
    ilu = lina.ILU(q.n, q.indptr, q.indices, q.data)
    ms_apply = ilu.time_apply(20, lina.PREC_MIXED)
    nlev = ilu.levels()[0]
    by = ilu.apply_bytes(lina.PREC_MIXED)
    ilu.close()
    peak, peak_kind = measured_peaks()
    achieved = by / (ms_apply / 1e3) / 1e9
    out["roofline"] = {"bound": "hbm", "kernel": f"FP32 ILU(0) application (forward + backward triangular solve, "
                                                 f"{nlev} levels each way; latency-bound: one block barrier per level)",
                       "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                       "peak_kind": peak_kind, "traffic": None, "bytes_per_launch": by,
                       "avg_launch_us": ms_apply * 1e3}
    out["cpu_baseline"] = None
    if rank == 0 and not args.no_cpu:
        from oracle import port
        # one Newton step's local solve as the reference runs it (incomplete_LU_factorization, then
        # BiCGStab_solve with the ILU(0) preconditioner to 1e-8), restated, serial as the reference
        t0 = time.perf_counter()
        f = port.ilu0(q.indptr, q.indices, q.data)
        t_ilu = time.perf_counter() - t0
        t0 = time.perf_counter()
        _, bit, _ = port.bicgstab_ilu(q.indptr, q.indices, q.data, q.b, 1e-8, 1000, factors=f)
        t_bi = time.perf_counter() - t0
        steps = int(np.mean(its)) if its else 1
        t_min = steps * (t_ilu + t_bi)
        out["cpu_baseline"] = {"value": 1.0 / t_min, "unit": "solves/s", "cores": 1, "kind": "port",
                               "sample": f"one Newton step's local solve on the AT2 Hessian ({q.n} rows): ILU(0) "
                                         f"{t_ilu:.2f} s + BiCGStab to 1e-8 ({bit} iterations) {t_bi:.2f} s, the "
                                         f"reference's algorithm restated and serial as the reference; times "
                                         f"{steps} Newton steps.  The reflective-Newton host work (assembly of "
                                         f"D H D + diag(|g| J), line search) is not counted, so the CPU figure "
                                         f"is an upper bound on the reference's rate"}
    if rank == 0:
        print(json.dumps(out))


def run_adjoint(args, rank, world, local):
    """Material identification on the 513 x 513 elasticity mesh (526,338 dofs, 524,288 elements,
    256 sensor nodes): a step is one forward solve and one backward (adjoint) solve with the
    per-element gradient, through the C-ABI with host arrays, tolerance 1e-10."""
    from fem_gb300 import lina, problems
    m = 513 if args.m == 1025 else args.m
    case = problems.adjoint_case(m, seed=0)
    xy, tri, fd, fv = problems.elastic_mesh(m)
    opts = dict(depth=DEFAULT_DEPTH.get(m, 8) - 1, precision=lina.PREC_MIXED,
                coarsening=lina.PMIS if args.coarsening == "pmis" else lina.STANDARD)
    probe = lina.ElasticAdjoint(xy, tri, 0.3, fd, fv, case["sensor_dof"], np.zeros(len(case["sensor_dof"])),
                                case["young_target"], **opts)
    ut, _, _ = probe.forward(case["young_target"], tol=1e-10)
    probe.close()
    adj = lina.ElasticAdjoint(xy, tri, 0.3, fd, fv, case["sensor_dof"], ut[case["sensor_dof"]], case["young"],
                              **opts)
    E = case["young"]

    def step():
        adj.forward(E, tol=1e-10)
        return adj.backward(tol=1e-10)

    for _ in range(args.warmup):
        step()
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = lina.launches()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    ms = max_over_ranks((time.perf_counter() - t0) * 1e3, world)
    launches = lina.launches() - launches0
    clocks.stop()
    value = world * args.steps / (ms / 1e3)
    n = 2 * m * m
    out = common_line("adjoint gradients/s (forward + adjoint solve + per-element dL/dE) at 526k dofs", value,
                      "gradients/s", world, args.steps, args.warmup, ms, "f32 preconditioner / f64 Krylov",
                      "synthetic (seeded lognormal moduli, seeded sensors)",
                      {"workload": f"P1 plane-strain elasticity {m}x{m} nodes, {n} dofs, {len(E)} elements, "
                                   f"{len(case['sensor_dof']) // 2} sensor nodes, tol 1e-10", "dofs": n},
                      {"value": value, "unit": "gradients/s", "h2d_bytes_per_step": 8 * len(E),
                       "d2h_bytes_per_step": 8 * (2 * n + len(E))}, launches, clocks)
    # the assembled system of the timed moduli: the forward and the adjoint solve both run on it (A is
    # symmetric, so get_transpose(A) = A); the dominant kernel is timed on a hierarchy with the same
    # options, and the CPU baseline solves it with the restated reference
    ptr, col, val, b = adj.system()
    sysm = problems.CSRSystem(n, ptr, col, val, b, dof=2)
    amg = lina.AMG(n, ptr, col, val, dof=2, **opts)
    b_dev = lina.DeviceArray.from_host(b)
    x_dev = lina.DeviceArray(n)
    out["roofline"] = sweep_roofline(amg, b_dev, x_dev, 1e-10, lina.STOP_RELATIVE, 0, 2,
                                     "FP32 damped-Jacobi sweeps of the adjoint's hierarchy")
    amg.close()
    out["cpu_baseline"] = None
    if rank == 0 and not args.no_cpu:
        from oracle import port
        P = port.PortAMG.setup(sysm, opts["depth"], 2, 0.1, port.JACOBI, 0.6, 2, 2)
        t0 = time.perf_counter()
        _, it_c, _ = P.pcg(b, 1e-10, 2000, 1)
        t1 = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1.0 / (2 * t1), "unit": "gradients/s", "cores": port_threads(),
                               "kind": "port", "sample": f"one FP64 solve of the system to 1e-10 ({it_c} iterations, "
                                                         f"{t1:.2f} s) on the restated reference hierarchy, times two "
                                                         "(forward and adjoint); assembly and gradient not counted"}
    if rank == 0:
        print(json.dumps(out))


def run_batch(args, rank, world, local):
    """Independent SPD systems on seeded unstructured Delaunay meshes (half Poisson, half plane-strain
    elasticity, dof counts log-uniform on [10k, 500k], per-element lognormal coefficients with sigma
    1.5): a step solves all of them to a relative residual of 1e-8 in mixed precision as one segmented
    system (lina_gpu_segbatch: every level the block-diagonal concatenation of the systems' levels,
    per-system FCG scalars and stopping, one graph launch).  Beside it, the same systems in one graph with
    a branch per system, and solved one after another by the single-system FP64 and mixed paths, on the
    same hierarchies."""
    from fem_gb300 import lina, problems
    # with several ranks each solves its dof-balanced share of the systems (no exchange)
    plan = problems.batch_shard(problems.batch_plan(args.batch_count, seed=0), rank, world)
    t0 = time.perf_counter()
    systems = [problems.batch_system(*p) for p in plan]
    t_mesh = time.perf_counter() - t0
    t0 = time.perf_counter()
    # multicolour SOR: with damped Jacobi the large high-contrast elasticity systems stall
    coarsening = lina.PMIS if args.coarsening == "pmis" else lina.STANDARD
    amgs = [lina.AMG.from_system(s, depth=problems.batch_depth(s.n), coarsening=coarsening,
                                 smoother=lina.SMOOTHER_MC_SOR, omega=1.0, precision=lina.PREC_MIXED,
                                 matrix_tol=args.batch_matrix_tol) for s in systems]
    t_setup = time.perf_counter() - t0
    dofs = int(sum(s.n for s in systems))
    nnz = int(sum(s.nnz for s in systems))
    t0 = time.perf_counter()
    seg = lina.SegmentedBatch(amgs)
    t_seg = time.perf_counter() - t0
    batch = lina.Batch(amgs, stop=lina.STOP_RELATIVE)
    bs = [s.b for s in systems]
    bd = [lina.DeviceArray.from_host(b) for b in bs]
    for _ in range(args.warmup):
        seg.solve(bd, tol=args.tol, device=True)
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = lina.launches()
    # device-resident inputs and outputs
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, infos = seg.solve(bd, tol=args.tol, device=True)
    ms = max_over_ranks((time.perf_counter() - t0) * 1e3, world)
    launches = lina.launches() - launches0
    # end to end: host arrays in and out
    t0 = time.perf_counter()
    for _ in range(args.steps):
        xs, infos = seg.solve(bs, tol=args.tol)
    ms_e2e = max_over_ranks((time.perf_counter() - t0) * 1e3, world)
    clocks.stop()
    worst = max(i.true_rel_residual for i in infos)
    its = [i.iterations for i in infos]
    assert all(i.status == 0 for i in infos), [i.status for i in infos]
    # the same systems as one graph with a branch per system (each system's own hierarchy and kernels)
    batch.solve(bd, tol=args.tol, device=True)
    t0 = time.perf_counter()
    _, infos_b = batch.solve(bd, tol=args.tol, device=True)
    t_branches = max_over_ranks(time.perf_counter() - t0, world)
    # the single-system paths, one system after another
    t0 = time.perf_counter()
    loop_mixed_its = [a.pcg(b, tol=args.tol, max_iter=1000)[1].iterations for a, b in zip(amgs, bs)]
    t_loop_mixed = time.perf_counter() - t0
    for a in amgs:
        a.set_smoother(lina.SMOOTHER_MC_SOR, 1.0, lina.PREC_FP64)
    for a, b in zip(amgs[:2], bs[:2]):
        a.pcg(b, tol=args.tol, max_iter=1000)  # graph capture of the FP64 iteration
    t0 = time.perf_counter()
    loop64 = [a.pcg(b, tol=args.tol, max_iter=1000)[1] for a, b in zip(amgs, bs)]
    t_loop64 = time.perf_counter() - t0
    # whole job: all ranks' systems; every rank loops over its own share at the same time
    n_sys = args.batch_count
    dofs = int(sum_over_ranks(dofs, world))
    nnz = int(sum_over_ranks(nnz, world))
    t_loop64 = max_over_ranks(t_loop64, world)
    t_loop_mixed = max_over_ranks(t_loop_mixed, world)
    worst = max_over_ranks(worst, world)
    value = n_sys * args.steps / (ms / 1e3)
    e2e = n_sys * args.steps / (ms_e2e / 1e3)
    out = common_line(f"batched AMG-PCG: systems/s over {n_sys} unstructured systems ({dofs} dofs) to rel. res. "
                      f"{args.tol:g}, segmented hierarchy, one graph launch", value, "systems/s", world, args.steps,
                      args.warmup, ms,
                      "f32 preconditioner / f64 Krylov", "synthetic (seeded Delaunay meshes, lognormal coefficients)",
                      {"workload": f"{n_sys} systems, half P1 Poisson and half P1 plane-strain elasticity on seeded "
                                   "Delaunay meshes, dofs log-uniform on [10k, 500k], sigma 1.5; "
                                   f"{args.coarsening} coarsening, "
                                   f"matrix_tol {args.batch_matrix_tol:g}, multicolour SOR 2+2; inputs larger than "
                                   "L2 (no flush)", "systems": n_sys, "dofs": dofs, "nnz": nnz},
                      {"value": e2e, "unit": "systems/s", "h2d_bytes_per_step": 8 * dofs,
                       "d2h_bytes_per_step": 8 * dofs}, launches, clocks)
    out["dofs_per_s"] = value * dofs / n_sys
    out["branch_graph_systems_per_s"] = n_sys / t_branches
    out["loop_fp64_systems_per_s"] = n_sys / t_loop64
    out["loop_mixed_systems_per_s"] = n_sys / t_loop_mixed
    out["batch_over_loop_fp64"] = value / (n_sys / t_loop64)
    out["iterations"] = {"batch_min": min(its), "batch_max": max(its), "batch_sum": int(sum(its)),
                         "branch_graph_sum": int(sum(i.iterations for i in infos_b)),
                         "loop_fp64_sum": int(sum(i.iterations for i in loop64)),
                         "loop_mixed_sum": int(sum(loop_mixed_its))}
    out["worst_true_rel_residual"] = worst
    out["setup_s"] = {"meshes_and_assembly": t_mesh, "amg_setup": t_setup, "segmented_hierarchy": t_seg}
    rows, ents = seg.levels()
    out["segmented_levels"] = {"rows": rows, "entries": ents}
    # the dominant kernel: the colour sweeps of the combined hierarchy's finest level (all systems' rows),
    # timed in solves of the whole block-diagonal system on the combined hierarchy
    comb = seg.hierarchy()
    bcat = lina.DeviceArray.from_host(np.concatenate(bs))
    out["roofline"] = sweep_roofline(comb, bcat, lina.DeviceArray(comb.n), args.tol, lina.STOP_RELATIVE, 0, 1,
                                     "FP32 multicolour-SOR colour launches of the segmented hierarchy")
    out["cpu_baseline"] = None
    if rank == 0 and not args.no_cpu:
        from oracle import port
        # the restated reference on systems taken in plan order until the time bound; the whole batch's
        # CPU time estimated in proportion to the stored entries
        t_sum, nnz_done, done, its_c = 0.0, 0, 0, 0
        for sy in systems:
            if t_sum >= args.cpu_seconds:
                break
            P = port.PortAMG.setup(sy, problems.batch_depth(sy.n), 2, args.batch_matrix_tol, port.MC_SOR, 1.0, 2, 2)
            t0 = time.perf_counter()
            _, it_c, _ = P.pcg(sy.b, args.tol, 2000, 1)
            t_sum += time.perf_counter() - t0
            nnz_done += sy.nnz
            done += 1
            its_c += it_c
            del P
        t_all = t_sum * (sum(sy.nnz for sy in systems) / nnz_done)
        out["cpu_baseline"] = {"value": len(systems) / t_all, "unit": "systems/s", "cores": port_threads(),
                               "kind": "port", "sample": f"{done} of {len(systems)} systems solved to {args.tol:g} in "
                                                         f"FP64 ({its_c} PCG iterations, {t_sum:.1f} s) on restated "
                                                         "reference hierarchies (multicolour SOR, as the batch); "
                                                         "scaled to the batch by stored entries"}
    if rank == 0:
        print(json.dumps(out))


def run_reference(args, rank, world):
    """The reference's CPU solve path on the same workload (rank 0 only): its AMG_setup and pcg restated
    in C under oracle/ (amg_setup_port.c, lina_port.c; hierarchies, V-cycles and whole pcg solves
    bit-identical to the reference compiled from its sources, tests/test_oracle_port.py), OpenMP over all
    host cores where the reference's loops allow it.  The GPU library is not loaded.  Every timed step is
    one whole solve; a second leg times the reference's default lexicographic SOR smoother."""
    if rank != 0:
        return
    from fem_gb300 import problems  # numpy only: the seeded system
    from oracle import port
    m = args.m
    depth = args.depth or DEFAULT_DEPTH.get(m, 8)
    omega = args.omega or (0.6 if args.smoother == "jacobi" else 1.0)
    s = build_system(m)
    kind = port.JACOBI if args.smoother == "jacobi" else port.MC_SOR
    t0 = time.perf_counter()
    P = port.PortAMG.setup(s, depth, 2, args.matrix_tol, kind, omega, 2, 2)
    setup_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        P.pcg(s.b, args.tol, 2000, 1)
    times, its = [], []
    x = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        x, it, _ = P.pcg(s.b, args.tol, 2000, 1)
        times.append(time.perf_counter() - t0)
        its.append(it)
    total = sum(times)
    value = args.steps / total
    A = _csr_matvec(s)
    trr = float(np.linalg.norm(s.b - A(x)) / np.linalg.norm(s.b))
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    # the reference's default smoother: lexicographic SOR (AMG_SOR_smoother, LinA/Multigrid.c:1345), omega 1,
    # serial as in the reference; one whole solve
    sor = None
    if args.ref_sor:
        Q = port.PortAMG.setup(s, depth, 2, args.matrix_tol, port.REF_SOR, 1.0, 2, 2)
        t0 = time.perf_counter()
        xs, it_s, _ = Q.pcg(s.b, args.tol, 2000, 1)
        dt = time.perf_counter() - t0
        sor = {"value": 1.0 / dt, "unit": "solves/s", "iterations": it_s, "seconds": dt,
               "true_rel_residual": float(np.linalg.norm(s.b - A(xs)) / np.linalg.norm(s.b))}
    sample = (f"{args.steps} whole FP64 solves ({sum(its)} PCG iterations, {total:.1f} s) after {args.warmup} "
              f"untimed ones; hierarchy built by the restated AMG_setup in {setup_s:.1f} s (not timed)")
    out = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded structured P1 mesh, notch damage field)", "impl": "reference",
           "config": workload_config(args, s, depth, omega, P.sizes()),
           "iterations": its, "true_rel_residual": trr, "setup_s": setup_s, "dofs_per_s": value * s.n,
           "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "reference_sor": sor}
    print(json.dumps(out))


def _csr_matvec(s):
    """y = A x for a CSR system with numpy only (residual checks outside the timed regions)."""
    rows = np.repeat(np.arange(s.n), np.diff(s.indptr))

    def mv(x):
        return np.bincount(rows, weights=s.data * x[s.indices], minlength=s.n)
    return mv


def workload_config(args, s, depth, omega, sizes):
    """The workload both arms run, described identically by both."""
    m = args.m
    return {"workload": f"degraded plane-strain P1 elasticity {m}x{m} nodes, {s.n} dofs, AMG-PCG "
                        f"(one V-cycle per iteration) to true rel-res {args.tol:g}",
            "dofs": s.n, "nnz": int(s.nnz), "amg_depth": depth, "level_sizes": [int(v) for v in sizes],
            "coarsening": args.coarsening, "matrix_tol": args.matrix_tol, "smoother": args.smoother,
            "omega": omega, "sweeps": "2+2", "tol": args.tol,
            "l2": "inputs exceed L2 (finest matrix > 129 MB), no flush"}


_pg = None


def init_dist(world):
    global _pg
    if world > 1 and _pg is None:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        _pg = dist


def barrier(world):
    if world > 1:
        _pg.barrier()


def sum_over_ranks(v, world):
    if world <= 1:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    _pg.all_reduce(t, op=_pg.ReduceOp.SUM)
    return float(t.item())


def max_over_ranks(v, world):
    if world <= 1:
        return v
    import torch
    t = torch.tensor([float(v)])
    _pg.all_reduce(t, op=_pg.ReduceOp.MAX)
    return float(t.item())


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    init_dist(world)
    from fem_gb300 import lina
    if world > 1:
        lina.set_device(local)
    lina.set_sell_index_bits(args.sell_bits)
    if args.workload == "damage":
        run_damage(args, rank, world, local)
    elif args.workload == "poisson":
        run_poisson(args, rank, world, local)
    elif args.workload == "adjoint":
        run_adjoint(args, rank, world, local)
    elif args.workload == "batch":
        run_batch(args, rank, world, local)
    else:
        run_gb300(args, rank, world, local)


if __name__ == "__main__":
    main()
