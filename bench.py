"""Benchmark of the spectral Rayleigh-Benard time step on GB300.

Workload (one "step" = one Integrate::update of the whole case):
  Navier2D::new_periodic(nx=512, ny=257, Ra=1e7, Pr=1, dt=1e-3, aspect=2), FP64,
  seeded initial fields (set_velocity(0.2,1,1) + 1e-3 interior temperature noise).
Metric: grid-point-steps per second (nx*ny*steps / s), higher is better.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Timing: W untimed warm-up steps, then K steps, each bracketed by CUDA events
on the case stream; L2 is flushed (256 MiB memset) between timed steps, outside
the events.  `e2e` repeats the measurement through the public API with the
step's state copied host->device from pinned memory and back every step.
`--impl reference` times the CPU restatement of the reference algorithm
(oracle/, the reference itself is Rust and cannot be built here) on all host
cores.  With N > 1 (torchrun) every rank advances its own replica of the case;
there is no collective on the data path (replicas only).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NX, NY, RA, PR, DT, ASPECT = 512, 257, 1e7, 1.0, 1e-3, 2.0
GP = NX * NY
METRIC = "grid-pt-steps/s"
WORKLOAD = "Navier2D::new_periodic 512x257 Ra=1e7 Pr=1 dt=1e-3 aspect=2 (FourierR2c x ChebDirichlet), plain FP64"


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return

        def reader():
            for line in self.proc.stdout:
                self.rows.append([x.strip() for x in line.split(",")])

        self.thread = threading.Thread(target=reader, daemon=True)
        self.thread.start()

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                smax = float(r[1])
            except (ValueError, IndexError):
                continue
            for k, n in enumerate(names):
                if len(r) > 3 + k and r[3 + k].lower().startswith("active"):
                    reasons.add(n)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def fp64_peak_tflops():
    """Measured FP64 throughput of this GPU: cuBLAS DGEMM 4096^3 (best of 5)."""
    try:
        import torch
        a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
        b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
        for _ in range(2):
            torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 0.0
        for _ in range(5):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            torch.matmul(a, b)
            e.record()
            e.synchronize()
            best = max(best, 2 * 4096 ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
        del a, b
        torch.cuda.empty_cache()
        return best, "torch.matmul float64 4096^3 (cuBLAS DGEMM), best of 5"
    except Exception as exc:  # pragma: no cover - torch missing on the box
        return 1.19, f"probe value 1.19 TFLOP/s (DFMA loop); torch unavailable: {exc}"


def stage_model(name):
    """Algorithmic HBM bytes and FP64 flops of one launch of a stage of the
    periodic step.  Bytes: every array the stage must read or write, once.
    Flops: conventional 5 N log2 N per complex FFT of length N plus the
    element-wise work of the pass (stencils, derivatives, banded solves)."""
    import math
    mx, ny, nx, myc, kx = NX // 2 + 1, NY, NX, NY - 2, (NX // 2 + 1) * 2 // 3
    c16 = 16
    N = NY - 1  # DCT-I through a complex FFT of length ny-1
    M = NX // 2  # r2c/c2r through a complex FFT of length nx/2
    fft = lambda n: 5.0 * n * math.log2(n)  # noqa: E731
    dct = fft(N) + 24.0 * N  # pre-twiddle, C_1, even/odd outputs (complex lane)
    if name == "y1_complex":
        b = 3 * mx * myc * c16 + 6 * mx * ny * c16
        f = mx * 3 * (2 * dct + 30 * ny)
    elif name == "periodic_x":
        b = 6 * mx * ny * c16 + 2 * nx * ny * 8 + 3 * kx * ny * c16
        f = ny * (11 * (fft(M) + 12 * M) + 3 * nx * 4)
    elif name == "periodic_y2":
        # q (3 fields) in; ux, uy, temp read and written; p1, p0 written;
        # the boundary-field constants read; per-row solver factors read
        b = (3 * kx * ny * c16 + 2 * 3 * mx * myc * c16 + mx * myc * c16 + mx * ny * c16
             + 2 * mx * ny * c16 + 3 * 4 * mx * myc * 8)
        f = kx * 3 * dct + mx * ny * 180
    elif name == "periodic_y2a":
        b = 3 * kx * ny * c16 + 2 * 3 * mx * myc * c16 + 4 * mx * ny * c16 + 3 * 4 * mx * myc * 8
        f = kx * 3 * dct + mx * 3 * ny * 60
    elif name == "periodic_y2b":
        b = 2 * 2 * mx * myc * c16 + mx * myc * c16 + 2 * mx * ny * c16 + 4 * mx * myc * 8
        f = mx * ny * 120
    else:
        b, f = 0, 0
    return b, f


def run_ours(args, rank, world, local):
    import numpy as np

    import rustpde_gb300 as R
    from rustpde_gb300 import build
    build.build()

    nav = R.Navier2D(NX, NY, RA, PR, DT, ASPECT, R.PERIODIC, seed=None)
    R.standard_ic(nav, seed=1 + rank)
    flush = R.DeviceArray((256 * 1024 * 1024 // 8,))
    lib = R.lib()
    stream = nav.stream()

    import ctypes
    cudart = ctypes.CDLL("libcudart.so.13") if os.path.exists("/usr/local/cuda/lib64/libcudart.so.13") else None
    if cudart is None:
        cudart = ctypes.CDLL("libcudart.so")
    cudart.cudaEventCreate.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
    cudart.cudaEventRecord.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    cudart.cudaEventSynchronize.argtypes = [ctypes.c_void_p]
    cudart.cudaEventElapsedTime.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_void_p, ctypes.c_void_p]
    cudart.cudaMemsetAsync.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p]

    def ev():
        e = ctypes.c_void_p()
        assert cudart.cudaEventCreate(ctypes.byref(e)) == 0
        return e

    # warm-up
    nav.update(args.warmup)
    nav.synchronize()
    if args.quick:
        t0 = time.perf_counter()
        nav.update(args.steps)
        nav.synchronize()
        dt = time.perf_counter() - t0
        return {"metric": METRIC, "value": GP * args.steps / dt, "unit": "grid-pt-steps/s", "steps": args.steps,
                "warmup": args.warmup, "mode": "quick (host wall clock, no L2 flush)", "status": nav.status()}

    barrier = None
    if world > 1:
        import torch.distributed as dist
        barrier = dist.barrier
        barrier()

    K = args.steps
    starts = [ev() for _ in range(K)]
    ends = [ev() for _ in range(K)]
    clocks = ClockSampler(local)
    clocks.start()
    t_wall0 = time.perf_counter()
    for k in range(K):
        cudart.cudaMemsetAsync(flush.ptr, k & 0xFF, flush.nbytes, ctypes.c_void_p(stream))
        cudart.cudaEventRecord(starts[k], ctypes.c_void_p(stream))
        nav.update(1)
        cudart.cudaEventRecord(ends[k], ctypes.c_void_p(stream))
    nav.synchronize()
    t_wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    total_ms = 0.0
    f = ctypes.c_float()
    for k in range(K):
        cudart.cudaEventElapsedTime(ctypes.byref(f), starts[k], ends[k])
        total_ms += f.value
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([total_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    status = nav.status()

    # per-stage timing of the step kernels (dominant kernel roofline)
    stages = nav.profile_step(20)
    dom = max(stages, key=stages.get)
    b_alg, f_alg = stage_model(dom)
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    dom_s = stages[dom] * 1e-3
    fp64_peak, fp64_how = fp64_peak_tflops()

    # end-to-end through the public API: state host->device, step, state device->host
    fields = (R.TEMP, R.UX, R.UY, R.PRES, R.PSEUDO_PRES)
    pinned = {fid: R.PinnedArray(nav.shape(fid)[0], np.complex128) for fid in fields}
    for fid in fields:
        pinned[fid].array[...] = nav.get(fid)
    h2d = sum(p.array.nbytes for p in pinned.values())
    Ke = min(K, 50)
    t0 = time.perf_counter()
    for _ in range(Ke):
        for fid in fields:
            nav.set(fid, pinned[fid].array)
        nav.update(1)
        for fid in fields:
            lib.rbc_get_state(nav._h, fid, pinned[fid].array.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                              pinned[fid].array.size * 2)
    nav.synchronize()
    e2e_s = time.perf_counter() - t0

    value = GP * K / (total_ms * 1e-3) * world
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "grid-pt-steps/s",
        "n_gpus": world,
        "steps": K,
        "warmup": args.warmup,
        "ms_per_step": total_ms / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic seeded fields (set_velocity(0.2,1,1) + splitmix64 temperature noise 1e-3)",
        "config": {"workload": WORKLOAD, "nx": NX, "ny": NY, "ra": RA, "pr": PR, "dt": DT, "aspect": ASPECT,
                   "precision": "fp64", "parallelism": f"replicas{world}",
                   "l2": "flushed between timed steps (256 MiB memset outside the events)",
                   "wall_s_timed_region": t_wall},
        "e2e": {"value": GP * Ke / e2e_s * world, "unit": "grid-pt-steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": h2d, "steps": Ke,
                "how": "per step: rbc_set_state x5 from pinned host memory, rbc_step(1), rbc_get_state x5"},
        "gpu_launches": K * len(stages),
        "stages_ms": stages,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": b_alg / dom_s / 1e9, "peak": hbm_peak,
                     "unit": "GB/s", "frac": b_alg / dom_s / 1e9 / hbm_peak, "traffic": None,
                     "algorithmic_bytes_per_launch": b_alg,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
        "fp64_roofline": {"kernel": dom, "achieved_tflops": f_alg / dom_s / 1e12, "peak_tflops": fp64_peak,
                          "frac": f_alg / dom_s / 1e12 / fp64_peak, "algorithmic_flops_per_launch": f_alg,
                          "peak_source": fp64_how},
        "clocks": clk,
        "status": status,
    }
    if rank == 0 and world == 1:
        line["cpu_baseline"] = cpu_baseline(budget_s=args.cpu_budget)
    return line


def cpu_baseline(budget_s=15.0):
    """The oracle (CPU restatement of the reference algorithm, OpenMP over
    lanes) on a bounded sample of the same workload."""
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    o = O.Navier2D(NX, NY, RA, PR, DT, ASPECT, O.PERIODIC)
    O.standard_ic(o, 1)
    o.update(1)  # warm-up (plans, first touch)
    n = 0
    t0 = time.perf_counter()
    while n < 3 or time.perf_counter() - t0 < budget_s:
        o.update(1)
        n += 1
        if n >= 400:
            break
    dt = time.perf_counter() - t0
    return {"value": GP * n / dt, "unit": "grid-pt-steps/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"{n} steps of the same 512x257 periodic case after 1 warm-up step ({dt:.1f} s)"}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    from oracle import oracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1)
    o = O.Navier2D(NX, NY, RA, PR, DT, ASPECT, O.PERIODIC)
    O.standard_ic(o, 1)
    t0 = time.perf_counter()
    o.update(1)
    per_step = time.perf_counter() - t0
    warm = max(0, min(args.warmup, int(20.0 / max(per_step, 1e-6))))
    o.update(warm)
    K = max(1, min(args.steps, int(90.0 / max(per_step, 1e-6))))
    t0 = time.perf_counter()
    o.update(K)
    dt = time.perf_counter() - t0
    v = GP * K / dt
    return {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "grid-pt-steps/s", "n_gpus": world, "steps": K,
        "warmup": warm, "ms_per_step": dt / K * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic seeded fields",
        "config": {"workload": WORKLOAD, "nx": NX, "ny": NY, "ra": RA, "pr": PR, "dt": DT, "aspect": ASPECT},
        "cpu_baseline": {"value": v, "unit": "grid-pt-steps/s", "cores": O.num_threads(), "kind": "port",
                         "sample": f"{K} steps of the workload (bounded to ~90 s)"},
        "e2e": {"value": v, "unit": "grid-pt-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference is Rust (no toolchain here or on the box); timed: the C++ restatement in oracle/",
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--quick", action="store_true",
                    help="only warm-up + timed steps (profiling target); prints a reduced line")
    args = ap.parse_args()
    rank, world, local = dist_info()
    if world > 1 and args.impl == "ours":
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("gloo")
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    else:
        args.warmup = max(args.warmup, 3)
        line = run_ours(args, rank, world, local)
    if rank == 0 and line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
