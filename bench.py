"""Benchmark of the spectral Rayleigh-Benard time step on GB300.

Metric: grid-point-steps per second (sum over cases of nx*ny*steps / s),
higher is better.

Workloads (--workload):
  ensemble (default)  256 independent cases of uneven size (rustpde_gb300.ensemble,
                      seed 2024): (nx, ny) in {64,128,256}^2, box or periodic
                      50/50, Ra log-uniform [1e4, 1e8], Pr in {0.7,1,7}, aspect
                      U[1,2], dt = min(0.02, 2/sqrt(Ra)).  `value` is the batched
                      mixed-precision form (one CUDA graph per ensemble step,
                      tensor-core 3xTF32 transforms, FP32 products, FP64 solves);
                      `plain_fp64` times the plain FP64 path run case by case on
                      the same ensemble, and `mixed_error` gives the Nu / KE
                      deviation of every mixed case from its FP64 run.
  periodic512         Navier2D::new_periodic(512, 257, Ra=1e7, Pr=1, dt=1e-3,
                      aspect=2), plain FP64, one case.
  serving             the serving loop alone (see run_serving).
  precision           batched 1-D stages, FP64 vs mixed (see run_precision).
  extras              per-update device time of the solid-mask step, Diffusion2D
                      and Navier2DAdjoint beside the oracle on the host cores
                      (see run_extras).
  profile-step        one batched ensemble step between cudaProfilerStart/Stop,
                      for `ncu --profile-from-start off` (see run_profile_step).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload ...]

Timing: W untimed warm-up steps, then K steps bracketed by CUDA events on the
stream that runs them, L2 flushed (256 MiB memset, outside the events) first.
The ensemble runs its K steps in one call (its state alone exceeds L2) and
reports the same K steps with one call and one flush per step beside it; the
single-case workloads flush between timed steps.  `e2e` is the same metric through the public API with the
whole state copied host->device from pinned memory before, and device->host
after, every step.  `--impl reference` times the CPU restatement of the
reference algorithm (oracle/, the reference is Rust and cannot be built here)
on all host cores over a bounded sample of the workload.  With N > 1
(torchrun) every rank advances its own replica; there is no collective on the
data path (replicas only).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid-pt-steps/s"
NX, NY, RA, PR, DT, ASPECT = 512, 257, 1e7, 1.0, 1e-3, 2.0
WORKLOAD_512 = "Navier2D::new_periodic 512x257 Ra=1e7 Pr=1 dt=1e-3 aspect=2 (FourierR2c x ChebDirichlet), plain FP64"
ENSEMBLE_N, ENSEMBLE_SEED = 256, 2024
WORKLOAD_ENS = ("256-case RBC ensemble of uneven size (nx,ny in {64,128,256}^2, box/periodic 50/50, "
                "Ra log-U[1e4,1e8], Pr {0.7,1,7}, aspect U[1,2], dt=min(0.02,2/sqrt(Ra)), seed 2024), "
                "batched mixed precision")


def dist_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


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


class Cudart:
    """CUDA events and memset through the runtime the library links."""

    def __init__(self):
        try:
            self.lib = ctypes.CDLL("libcudart.so.13")
        except OSError:
            self.lib = ctypes.CDLL("libcudart.so")
        L = self.lib
        L.cudaEventCreate.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
        L.cudaEventRecord.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.cudaEventSynchronize.argtypes = [ctypes.c_void_p]
        L.cudaEventElapsedTime.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_void_p, ctypes.c_void_p]
        L.cudaMemsetAsync.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p]
        L.cudaEventDestroy.argtypes = [ctypes.c_void_p]

    def event(self):
        e = ctypes.c_void_p()
        assert self.lib.cudaEventCreate(ctypes.byref(e)) == 0
        return e

    def record(self, e, stream):
        self.lib.cudaEventRecord(e, ctypes.c_void_p(stream))

    def elapsed(self, a, b):
        f = ctypes.c_float()
        self.lib.cudaEventSynchronize(b)
        self.lib.cudaEventElapsedTime(ctypes.byref(f), a, b)
        return f.value

    def memset(self, ptr, v, n, stream):
        self.lib.cudaMemsetAsync(ptr, v, n, ctypes.c_void_p(stream))

    def destroy(self, *evs):
        for e in evs:
            self.lib.cudaEventDestroy(e)


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per ensemble step of
# each kernel of the batched mixed step, from one ncu capture of the 256-case
# ensemble (the launch list in profiles/launches_ensemble256_mixed.md); the
# roofline's `traffic` for the dominant kernel, per step like its `achieved`
NCU_DRAM_BYTES_PER_STEP = {
    "state_f32": 144e6, "lane_gemm": 738e6, "periodic_x_mixed_t128": 93e6, "lanes_periodic_y2a": 404e6,
    "lanes_periodic_y2b": 108e6, "lanes_periodic_y2c": 260e6, "box_prod_mixed": 128e6, "lanes_box_gpx": 23e6,
    "box_y2_pre": 237e6, "lanes_box_x2": 112e6, "lanes_box_y3": 179e6, "box_x3_mix_t128": 50e6,
    "lanes_box_y4": 131e6, "lanes_box_x4": 45e6, "lanes_box_y5": 263e6,
}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "MEASURED_PEAKS.json hbm_gbs (measured)"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback 6.8 TB/s"


def timed_steps(cu, stream, K, step, flush):
    """K steps, each between CUDA events on `stream`, L2 flushed in between."""
    starts = [cu.event() for _ in range(K)]
    ends = [cu.event() for _ in range(K)]
    for k in range(K):
        cu.memset(flush.ptr, k & 0xFF, flush.nbytes, stream)
        cu.record(starts[k], stream)
        step()
        cu.record(ends[k], stream)
    total = sum(cu.elapsed(starts[k], ends[k]) for k in range(K))
    cu.destroy(*starts, *ends)
    return total


def max_over_ranks(v, world):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------------------
# ensemble workload (default)
# ---------------------------------------------------------------------------
def run_ensemble(args, rank, world, local):
    import numpy as np

    import rustpde_gb300 as R
    from rustpde_gb300 import build
    from rustpde_gb300.ensemble import draw_ensemble
    build.build()
    cu = Cudart()
    params = draw_ensemble(args.cases, ENSEMBLE_SEED)
    gp = sum(p[0] * p[1] for p in params)
    flush = R.DeviceArray((256 * 1024 * 1024 // 8,))
    W, K = args.warmup, args.steps

    # ---- batched mixed precision
    t_setup = time.perf_counter()
    B = R.Batch(params, precision=R.PREC_MIXED)
    t_setup = time.perf_counter() - t_setup
    for i, c in enumerate(B.cases):
        R.standard_ic(c, seed=1000 + i)
    stream = B.stream()
    B.update(W)
    B.synchronize()
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    # K steps in one rbc_batch_step call, as a user advances the ensemble, L2
    # flushed once before (as for the plain FP64 arm below); the groups' graph
    # branches run their steps independently within the call
    t_wall = time.perf_counter()
    e0, e1 = cu.event(), cu.event()
    cu.memset(flush.ptr, 0x5A, flush.nbytes, stream)
    cu.record(e0, stream)
    B.update(K)
    cu.record(e1, stream)
    total_ms = cu.elapsed(e0, e1)
    cu.destroy(e0, e1)
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    barrier(world)
    total_ms = max_over_ranks(total_ms, world)
    nb, launches = B.layout()
    tuning = B.tuning()
    tuning_forms = B.tuning_forms()
    status = [c.status() for c in B.cases]
    mixed_nu = [c.eval(R.NU) for c in B.cases]
    mixed_ke = [c.eval(R.KE) for c in B.cases]
    mixed_temp = [c.get(R.TEMP) for c in B.cases]
    # K more steps, one call each, L2 flushed before every step (reported beside)
    flushed_ms = max_over_ranks(timed_steps(cu, stream, K, lambda: B.update(1), flush), world)
    value = gp * K / (total_ms * 1e-3) * world

    # ---- per-kernel profile of the batched step (each launch alone) and roofline
    prof = B.profile_step(3)
    per_launch = [{"bucket": b_, "pass": p_, "kernel": k_, "ms": round(m_, 4), "bytes": b2_}
                  for b_, p_, k_, m_, b2_ in B.profile_launches(3)]
    dom = max(prof, key=lambda k: prof[k][0])
    dom_ms, dom_bytes = prof[dom]
    pk, pk_src = peaks()
    hbm = pk.get("hbm_gbs", 6800.0)
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9

    # ---- end to end through the public API (whole ensemble state in and out every step)
    nbytes = B.state_bytes()
    host = R.PinnedArray((nbytes,), np.uint8)
    B.get_state_all(host.array)
    Ke = min(K, 20)
    t0 = time.perf_counter()
    for _ in range(Ke):
        B.set_state_all(host.array)
        B.update(1)
        B.get_state_all(host.array)
    e2e_s = time.perf_counter() - t0
    del B

    if args.skip_plain:  # profiling runs: the batched mixed step only
        return {"metric": METRIC, "value": value, "unit": "grid-pt-steps/s", "steps": K, "warmup": W,
                "cases": len(params), "mode": "batched mixed only", "autotuner_forms": tuning_forms,
                "kernels_ms_per_step": {k: v[0] for k, v in prof.items()},
                "launches": per_launch}

    # ---- plain FP64, case by case, same ensemble and initial fields
    plain_ms = 0.0
    err_nu, err_ke, err_t, ke_ref = [], [], [], []
    t_plain = time.perf_counter()
    for i, p in enumerate(params):
        nav = R.Navier2D(*p, precision=R.PREC_FP64, seed=None)
        R.standard_ic(nav, seed=1000 + i)
        nav.update(W)
        st = nav.stream()
        e0, e1 = cu.event(), cu.event()
        cu.memset(flush.ptr, i & 0xFF, flush.nbytes, st)
        cu.record(e0, st)
        nav.update(K)
        cu.record(e1, st)
        plain_ms += cu.elapsed(e0, e1)
        cu.destroy(e0, e1)
        for lst, what, ref in ((err_nu, R.NU, mixed_nu[i]), (err_ke, R.KE, mixed_ke[i])):
            v = nav.eval(what)
            lst.append(abs(ref - v) / max(abs(v), 1e-300))
        ke_ref.append(nav.eval(R.KE))
        t64 = nav.get(R.TEMP)
        err_t.append(float(np.linalg.norm(mixed_temp[i] - t64) / max(np.linalg.norm(t64), 1e-300)))
        del nav
    t_plain = time.perf_counter() - t_plain
    plain_value = gp * K / (plain_ms * 1e-3) * world
    err_nu, err_ke, err_t = np.array(err_nu), np.array(err_ke), np.array(err_t)

    line = {
        "metric": METRIC,
        "value": value,
        "unit": "grid-pt-steps/s",
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": total_ms / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 state and solves, tf32x3 tensor-core transforms, f32 products",
        "data": "synthetic: seeded ensemble draw; set_velocity(0.2,1,1) + splitmix64 temperature noise 1e-3 per case",
        "config": {"workload": WORKLOAD_ENS, "cases": len(params), "grid_points": gp, "precision": "mixed",
                   "buckets": nb, "launches_per_step": launches, "parallelism": f"replicas{world}",
                   "l2": "flushed once before the K timed steps (256 MiB memset outside the events); the "
                         "ensemble state (221 MB) and each step's scratch exceed L2",
                   "one_call_per_step_l2_flushed": {"value": gp * K / (flushed_ms * 1e-3) * world,
                                                    "ms_per_step": flushed_ms / K},
                   "setup_s": t_setup, "wall_s_timed_region": t_wall},
        "plain_fp64": {"value": plain_value, "unit": "grid-pt-steps/s", "ms_per_ensemble_step": plain_ms / K,
                       "how": "each case alone through rbc_step (its own CUDA graph), K steps between CUDA events, "
                              "cases one after another; L2 flushed before each case", "wall_s": t_plain},
        "speedup_vs_plain_fp64": value / plain_value,
        "mixed_error": {"steps": W + K, "nu_max_rel": float(err_nu.max()), "nu_median_rel": float(np.median(err_nu)),
                        "ke_max_rel": float(err_ke.max()), "ke_median_rel": float(np.median(err_ke)),
                        "temp_l2_max_rel": float(err_t.max()), "temp_l2_median_rel": float(np.median(err_t)),
                        "cases_nu_ke_within_1e-6": int(np.sum((err_nu <= 1e-6) & (err_ke <= 1e-6))),
                        "worst_ke_cases": [{"case": int(i), "params": list(params[i]), "ke_rel": float(err_ke[i]),
                                            "nu_rel": float(err_nu[i]), "ke": float(ke_ref[i]),
                                            "temp_l2_rel": float(err_t[i])}
                                           for i in np.argsort(err_ke)[::-1][:5]],
                        "against": "the plain FP64 GPU path (parity with the FP64 oracle <= 1e-9)"},
        "e2e": {"value": gp * Ke / e2e_s * world, "unit": "grid-pt-steps/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes, "steps": Ke,
                "how": "per step: rbc_batch_set_state_all (pinned h2d), rbc_batch_step(1), rbc_batch_get_state_all"},
        "gpu_launches": K * launches,
        "kernels_ms_per_step": {k: v[0] for k, v in prof.items()},
        "launches_ms": per_launch,
        "autotuner": [{"pass": t[0], "ms_cta_per_lane": t[1], "ms_thread_per_lane": t[2], "chosen": t[3]}
                      for t in tuning],
        "autotuner_forms": tuning_forms,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": NCU_DRAM_BYTES_PER_STEP.get(dom),
                     "traffic_source": "ncu dram bytes per step, profiles/launches_ensemble256_mixed.md",
                     "algorithmic_bytes_per_step": dom_bytes,
                     "peak_source": pk_src},
        "clocks": clk,
        "status_nonzero_cases": int(sum(1 for s in status if s)),
    }
    if rank == 0 and world == 1:
        line["serving"] = run_serving(args, args.requests, args.horizon_scale)
        line["cpu_baseline"] = cpu_baseline_ensemble(params, budget_s=args.cpu_budget)
    return line


def cpu_baseline_ensemble(params, budget_s=15.0, steps_per_case=2):
    """The oracle (CPU restatement of the reference algorithm, OpenMP over
    lanes, all host threads) on the leading cases of the same ensemble."""
    from oracle import oracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1)
    done_gp, t_acc, ncase = 0, 0.0, 0
    for p in params:
        nx, ny, ra, pr, dt, asp, kind = p
        o = O.Navier2D(nx, ny, ra, pr, dt, asp, kind)
        O.standard_ic(o, 1)
        o.update(1)
        t0 = time.perf_counter()
        o.update(steps_per_case)
        t_acc += time.perf_counter() - t0
        done_gp += nx * ny * steps_per_case
        ncase += 1
        if t_acc > budget_s:
            break
    return {"value": done_gp / t_acc, "unit": "grid-pt-steps/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"first {ncase} ensemble cases x {steps_per_case} steps after 1 warm-up step each "
                      f"({t_acc:.1f} s timed)"}


# ---------------------------------------------------------------------------
# serving: Poisson arrivals of solve requests, continuous batching
# ---------------------------------------------------------------------------
def run_serving(args, n_requests, horizon_scale, n_check=12):
    """Requests of rustpde_gb300.ensemble.draw_requests (50/s, seed 7, 5 %
    512x257) with horizons scaled by `horizon_scale`, submitted at their
    arrival times to the serving loop (mixed precision, 150 GB budget).
    Returns p50/p99 completion latency, aggregate throughput, and the Nu/KE
    deviation of the first `n_check` results from the same cases run alone in
    FP64."""
    import numpy as np

    import rustpde_gb300 as R
    from rustpde_gb300.ensemble import draw_requests
    reqs = draw_requests(n_requests, rate=50.0, seed=7)
    srv = R.Server(hbm_budget_bytes=150 * 10**9, max_active=256, chunk_steps=8,
                   setup_threads=max(1, min(8, (os.cpu_count() or 2) // 2)))
    t0 = time.perf_counter()
    ids = {}
    for rq in reqs:
        wait = rq.arrival - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        rid = srv.submit(rq.params + (R.PREC_MIXED,), rq.horizon * horizon_scale, rq.seed)
        ids[rid] = rq
    ok = srv.wait_idle(1800.0)
    res = srv.poll(len(reqs) + 8)
    st = srv.stats()
    srv.close()
    lat = np.array([r["t_done"] - r["t_submit"] for r in res])
    setup = np.array([r["t_admit"] - r["t_submit"] for r in res])
    gp_steps = sum(r["grid_points"] * r["steps"] for r in res)
    span = max(r["t_done"] for r in res) - min(r["t_submit"] for r in res)
    errs_nu, errs_ke = [], []
    for r in sorted(res, key=lambda r: r["id"])[:n_check]:
        rq = ids[r["id"]]
        c = R.Navier2D(*rq.params, precision=R.PREC_FP64, seed=None)
        c.set_velocity(0.2, 1.0, 1.0)
        c.set_temperature_noise(1e-3, rq.seed)
        c.update(r["steps"])
        for lst, what, v in ((errs_nu, R.NU, r["nu"]), (errs_ke, R.KE, r["ke"])):
            ref = c.eval(what)
            lst.append(abs(v - ref) / max(abs(ref), 1e-300))
        del c
    return {
        "requests": len(reqs), "completed": len(res), "idle": ok,
        "failed": int(sum(1 for r in res if r["status"] != 0)),
        "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
        "p50_queue_and_setup_s": float(np.percentile(setup, 50)),
        "aggregate_grid_pt_steps_per_s": gp_steps / span, "span_s": span,
        "steps_launched": st["steps_launched"], "graph_rebuilds": st["rebuilds"],
        "nu_max_rel_vs_fp64": float(max(errs_nu)), "ke_max_rel_vs_fp64": float(max(errs_ke)),
        "checked": len(errs_nu),
        "workload": (f"{n_requests} requests, Poisson 50/s (seed 7), sizes as the ensemble + 512x257 at 5 %, "
                     f"horizon U[1,20] time units x {horizon_scale} (scaled so the run fits in minutes), "
                     "mixed precision, 150 GB budget, max 256 active, 8 steps per round"),
    }


# ---------------------------------------------------------------------------
# precision microbenchmark: batched 1-D stages, FP64 vs mixed
# ---------------------------------------------------------------------------
def run_precision(args):
    """4096 lanes of length N in {128, 256, 512}, Chebyshev-Dirichlet basis:
    forward, backward, to_ortho, from_ortho and the 1-D Helmholtz solve
    (c = dt/2, dt = 1e-3), each in FP64 and in the mixed form (tensor-core
    3xTF32 products, FP64 banded sweep).  Inputs: spectral coefficients
    g_k exp(-k/20), g ~ N(0, 1) (seed 11).  Per stage: relative L2 error of
    the mixed result against FP64, and the device time of both forms."""
    import numpy as np

    import rustpde_gb300 as R
    from rustpde_gb300 import build
    build.build()
    cu = Cudart()
    lanes = 4096
    names = {R.OP_FORWARD: "forward", R.OP_BACKWARD: "backward", R.OP_TO_ORTHO: "to_ortho",
             R.OP_FROM_ORTHO: "from_ortho", R.OP_HHOLTZ: "hholtz"}
    rng = np.random.default_rng(11)
    out = {}
    for n in (128, 256, 512):
        f64 = R.Lanes(R.Base(1, n), R.PREC_FP64, hholtz_c=5e-4)
        mix = R.Lanes(R.Base(1, n), R.PREC_MIXED, hholtz_c=5e-4)
        spec = rng.standard_normal((lanes, f64.m)) * np.exp(-np.arange(f64.m) / 20.0)
        phys = f64.apply(R.OP_BACKWARD, spec)
        ortho = f64.apply(R.OP_TO_ORTHO, spec)
        inputs = {R.OP_FORWARD: phys, R.OP_BACKWARD: spec, R.OP_TO_ORTHO: spec, R.OP_FROM_ORTHO: ortho,
                  R.OP_HHOLTZ: ortho}
        row = {}
        for op, x in inputs.items():
            il, ol = f64.lengths(op)
            d_in = R.DeviceArray.from_host(x)
            d_a, d_b = R.DeviceArray((lanes, ol)), R.DeviceArray((lanes, ol))
            times = {}
            for tag, L, d_out in (("fp64", f64, d_a), ("mixed", mix, d_b)):
                for _ in range(3):
                    L.apply_dev(op, d_in, d_out, lanes)
                e0, e1 = cu.event(), cu.event()
                cu.record(e0, 0)
                for _ in range(20):
                    L.apply_dev(op, d_in, d_out, lanes)
                cu.record(e1, 0)
                times[tag] = cu.elapsed(e0, e1) / 20
                cu.destroy(e0, e1)
            a, b = d_a.to_host(), d_b.to_host()
            row[names[op]] = {"rel_l2_mixed_vs_fp64": float(np.linalg.norm(b - a) / np.linalg.norm(a)),
                              "ms_fp64": times["fp64"], "ms_mixed": times["mixed"]}
        out[f"N={n}"] = row
    return {"metric": "relative L2 error of the mixed form per stage", "workload": "precision microbenchmark",
            "config": {"lanes": lanes, "basis": "ChebDirichlet", "N": [128, 256, 512], "hholtz_c": 5e-4,
                       "inputs": "g_k exp(-k/20), g ~ N(0,1), seed 11"},
            "stages": out}


# ---------------------------------------------------------------------------
# solid masks, Diffusion2D, Navier2DAdjoint: device time per update
# ---------------------------------------------------------------------------
def run_extras(args):
    """Each solver on a fixed seeded case: K updates, each between CUDA events
    on the solver's stream with L2 flushed in between, against the oracle on
    all host cores (a bounded sample of updates of the same case)."""
    import numpy as np

    import rustpde_gb300 as R
    from oracle import oracle as O
    from rustpde_gb300 import build
    from rustpde_gb300 import solid_masks as S
    build.build()
    O.build()
    O.set_threads(os.cpu_count() or 1)
    cu = Cudart()
    flush = R.DeviceArray((256 * 1024 * 1024 // 8,))
    K = min(args.steps, 50)

    def device_ms(obj, stream):
        obj.update(3)
        return timed_steps(cu, stream, K, lambda: obj.update(1), flush) / K

    def oracle_ms(obj, budget=3.0):
        obj.update(1)
        n, t0 = 0, time.perf_counter()
        while n < 2 or (time.perf_counter() - t0 < budget and n < 200):
            obj.update(1)
            n += 1
        return (time.perf_counter() - t0) / n * 1e3

    out = {}
    for name, (nx, ny, ra, dt, kind) in {"solid_box128": (128, 128, 1e6, 2e-3, R.BOX_ADIABATIC),
                                         "solid_periodic256x129": (256, 129, 1e6, 2e-3, R.PERIODIC)}.items():
        plain = R.Navier2D(nx, ny, ra, 1.0, dt, 1.0, kind, seed=None)
        R.standard_ic(plain, 1)
        g = R.Navier2D(nx, ny, ra, 1.0, dt, 1.0, kind, seed=None)
        R.standard_ic(g, 1)
        x, y = g.coords(R.TEMP)
        g.solid = S.solid_cylinder_inner(x, y, 0.5 * (x[0] + x[-1]), 0.0, 0.3)
        o = O.Navier2D(nx, ny, ra, 1.0, dt, 1.0, kind)
        O.standard_ic(o, 1)
        o.set_solid(*g.solid)
        ms_plain, ms_solid = device_ms(plain, plain.stream()), device_ms(g, g.stream())
        out[name] = {"ms_per_step_plain": ms_plain, "ms_per_step_solid": ms_solid,
                     "solid_overhead": ms_solid / ms_plain - 1.0, "oracle_ms_per_step": oracle_ms(o),
                     "grid_pt_steps_per_s": nx * ny / (ms_solid * 1e-3)}
    for name, (k0, n0, k1, n1) in {"diffusion_cd256xcd256": (R.CHEB_DIRICHLET, 256, R.CHEB_DIRICHLET, 256),
                                   "diffusion_f512xcd257": (R.FOURIER_R2C, 512, R.CHEB_DIRICHLET, 257)}.items():
        f = R.Field2(R.Space2(R.Base(k0, n0), R.Base(k1, n1)))
        g = R.Diffusion2D(f, 1.0, 1e-3)
        g.impulse()
        o = O.Diffusion2D(k0, n0, k1, n1, 1.0, 1e-3)
        o.impulse()
        ms = device_ms(g, g.stream())
        out[name] = {"ms_per_update": ms, "oracle_ms_per_update": oracle_ms(o),
                     "grid_pt_steps_per_s": n0 * n1 / (ms * 1e-3)}
    for name, (nx, ny, kind) in {"adjoint_box64": (64, 64, R.BOX_ADIABATIC),
                                 "adjoint_periodic128x65": (128, 65, R.PERIODIC)}.items():
        g = R.Navier2DAdjoint(nx, ny, 1e5, 1.0, 0.02, 1.0, kind)
        o = O.Navier2DAdjoint(nx, ny, 1e5, 1.0, 0.02, 1.0, kind)
        for a in (g, o):
            a.set_temperature(0.5, 1.0, 1.0)
            a.set_velocity(0.5, 1.0, 1.0)
        ms = device_ms(g, g.stream())
        out[name] = {"ms_per_update": ms, "oracle_ms_per_update": oracle_ms(o),
                     "grid_pt_steps_per_s": nx * ny / (ms * 1e-3)}
    return {"metric": "ms per update", "workload": "extras", "steps": K, "unit": "ms", "higher_is_better": False,
            "dtype": "f64", "data": "synthetic seeded fields",
            "config": {"l2": "flushed between timed updates (256 MiB memset outside the events)",
                       "oracle_cores": O.num_threads()},
            "cases": out}


# ---------------------------------------------------------------------------
# single periodic 512x257 case, plain FP64
# ---------------------------------------------------------------------------
def run_periodic512(args, rank, world, local):
    import numpy as np

    import rustpde_gb300 as R
    from rustpde_gb300 import build
    build.build()
    cu = Cudart()
    gp = NX * NY
    nav = R.Navier2D(NX, NY, RA, PR, DT, ASPECT, R.PERIODIC, seed=None)
    R.standard_ic(nav, seed=1 + rank)
    flush = R.DeviceArray((256 * 1024 * 1024 // 8,))
    stream = nav.stream()
    nav.update(args.warmup)
    nav.synchronize()
    barrier(world)
    K = args.steps
    clocks = ClockSampler(local)
    clocks.start()
    t_wall = time.perf_counter()
    total_ms = timed_steps(cu, stream, K, lambda: nav.update(1), flush)
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    barrier(world)
    total_ms = max_over_ranks(total_ms, world)
    stages = nav.profile_step(20, with_bytes=True)
    dom = max(stages, key=lambda k: stages[k][0])
    dom_ms, dom_bytes = stages[dom]
    pk, pk_src = peaks()
    hbm = pk.get("hbm_gbs", 6800.0)
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    fields = (R.TEMP, R.UX, R.UY, R.PRES, R.PSEUDO_PRES)
    pinned = {fid: R.PinnedArray(nav.shape(fid)[0], np.complex128) for fid in fields}
    for fid in fields:
        pinned[fid].array[...] = nav.get(fid)
    h2d = sum(p.array.nbytes for p in pinned.values())
    Ke = min(K, 50)
    lib = R.lib()
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
    line = {
        "metric": METRIC, "value": gp * K / (total_ms * 1e-3) * world, "unit": "grid-pt-steps/s", "n_gpus": world,
        "steps": K, "warmup": args.warmup, "ms_per_step": total_ms / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic seeded fields (set_velocity(0.2,1,1) + splitmix64 temperature noise 1e-3)",
        "config": {"workload": WORKLOAD_512, "nx": NX, "ny": NY, "ra": RA, "pr": PR, "dt": DT, "aspect": ASPECT,
                   "precision": "fp64", "parallelism": f"replicas{world}",
                   "l2": "flushed between timed steps (256 MiB memset outside the events)",
                   "wall_s_timed_region": t_wall},
        "e2e": {"value": gp * Ke / e2e_s * world, "unit": "grid-pt-steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": h2d, "steps": Ke,
                "how": "per step: rbc_set_state x5 from pinned host memory, rbc_step(1), rbc_get_state x5"},
        "gpu_launches": K * len(stages),
        "stages_ms": {k: v[0] for k, v in stages.items()},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": None, "algorithmic_bytes_per_launch": dom_bytes,
                     "peak_source": pk_src},
        "clocks": clk, "status": nav.status(),
    }
    if rank == 0 and world == 1:
        line["cpu_baseline"] = cpu_baseline_512(budget_s=args.cpu_budget)
    return line


def cpu_baseline_512(budget_s=15.0):
    from oracle import oracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1)
    o = O.Navier2D(NX, NY, RA, PR, DT, ASPECT, O.PERIODIC)
    O.standard_ic(o, 1)
    o.update(1)
    n = 0
    t0 = time.perf_counter()
    while n < 3 or (time.perf_counter() - t0 < budget_s and n < 400):
        o.update(1)
        n += 1
    dt = time.perf_counter() - t0
    return {"value": NX * NY * n / dt, "unit": "grid-pt-steps/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"{n} steps of the same 512x257 periodic case after 1 warm-up step ({dt:.1f} s)"}


# ---------------------------------------------------------------------------
# reference arm: the oracle on the host cores
# ---------------------------------------------------------------------------
def run_reference(args, rank, world):
    if rank != 0:
        return None
    from oracle import oracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1)
    budget = 90.0
    if args.workload == "periodic512":
        cases = [(NX, NY, RA, PR, DT, ASPECT, O.PERIODIC)]
        config = {"workload": WORKLOAD_512, "nx": NX, "ny": NY}
    else:
        from rustpde_gb300.ensemble import draw_ensemble
        cases = draw_ensemble(args.cases, ENSEMBLE_SEED)
        config = {"workload": WORKLOAD_ENS.replace("batched mixed precision", "case by case, FP64"),
                  "cases": len(cases)}
    # one timed "step" advances every sampled case once; the sample is the
    # leading cases of the workload that fit the time budget
    objs, per_case = [], []
    for p in cases:
        nx, ny, ra, pr, dt, asp, kind = p
        o = O.Navier2D(nx, ny, ra, pr, dt, asp, kind)
        O.standard_ic(o, 1)
        t0 = time.perf_counter()
        o.update(1)
        per_case.append(time.perf_counter() - t0)
        objs.append((o, nx * ny))
        if sum(per_case) * max(args.steps, 1) > budget:
            break
    warm = min(args.warmup, 2)
    for o, _ in objs:
        o.update(warm)
    K = max(1, args.steps)
    t0 = time.perf_counter()
    done = 0
    for _ in range(K):
        for o, _g in objs:
            o.update(1)
        done += 1
        if time.perf_counter() - t0 > budget:
            break
    dt_s = time.perf_counter() - t0
    gp = sum(g for _, g in objs)
    v = gp * done / dt_s
    return {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "grid-pt-steps/s", "n_gpus": world,
        "steps": done, "warmup": warm, "ms_per_step": dt_s / done * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic seeded fields", "config": config,
        "cpu_baseline": {"value": v, "unit": "grid-pt-steps/s", "cores": O.num_threads(), "kind": "port",
                         "sample": f"{len(objs)} of {len(cases)} cases, {done} steps each (bounded to ~{budget:.0f} s)"},
        "e2e": {"value": v, "unit": "grid-pt-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference is Rust (no toolchain here or on the box); timed: the C++ restatement in oracle/",
    }


def run_profile_step(args):
    """The ensemble's batched mixed step for a profiler: the batch (forms from
    the autotuner, or pinned by RBC_BATCH_FORM), W warm-up steps, then ONE step
    between cudaProfilerStart and cudaProfilerStop, so that
    `ncu --profile-from-start off` captures exactly the launches of one step."""
    import rustpde_gb300 as R
    from rustpde_gb300 import build
    from rustpde_gb300.ensemble import draw_ensemble
    build.build()
    cu = Cudart()
    cu.lib.cudaProfilerStart.argtypes = []
    cu.lib.cudaProfilerStop.argtypes = []
    params = draw_ensemble(args.cases, ENSEMBLE_SEED)
    B = R.Batch(params, precision=R.PREC_MIXED)
    for i, c in enumerate(B.cases):
        R.standard_ic(c, seed=1000 + i)
    B.update(args.warmup)
    B.synchronize()
    cu.lib.cudaProfilerStart()
    B.update(1)
    B.synchronize()
    cu.lib.cudaProfilerStop()
    nb, launches = B.layout()
    return {"workload": "profile-step", "cases": len(params), "warmup": args.warmup, "launches_in_step": launches,
            "autotuner_forms": B.tuning_forms(), "status_max": max(c.status() for c in B.cases)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ensemble",
                    choices=["ensemble", "periodic512", "serving", "precision", "extras", "profile-step"])
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--cases", type=int, default=ENSEMBLE_N, help="ensemble size (default 256)")
    ap.add_argument("--skip-plain", action="store_true",
                    help="time the batched mixed step only (profiling runs; prints a reduced line)")
    ap.add_argument("--requests", type=int, default=300, help="serving: number of requests")
    ap.add_argument("--horizon-scale", type=float, default=0.01, help="serving: horizon multiplier")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 500 if args.workload == "ensemble" else 200
    rank, world, local = dist_info()
    if world > 1 and args.impl == "ours":
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("gloo")
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    elif args.workload == "precision":
        line = run_precision(args)
    elif args.workload == "extras":
        line = run_extras(args)
    elif args.workload == "profile-step":
        line = run_profile_step(args)
    elif args.workload == "serving":
        from rustpde_gb300 import build
        build.build()
        line = {"metric": METRIC, "workload": "serving", **run_serving(args, args.requests, args.horizon_scale)}
    else:
        args.warmup = max(args.warmup, 3)
        line = (run_ensemble if args.workload == "ensemble" else run_periodic512)(args, rank, world, local)
    if rank == 0 and line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
