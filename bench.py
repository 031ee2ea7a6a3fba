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
  cpu-table           the CPU restatement of the reference algorithm on the host
                      cores for configurations 0-3, all threads and one thread
                      (see run_cpu_table); no GPU work.

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
WORKLOAD_ENS = ("{n}-case RBC ensemble of uneven size (nx,ny in {64,128,256}^2, box/periodic 50/50, "
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
def ensemble_config(params):
    """The workload's `config`, shared by both arms (what is run, not how)."""
    return {"workload": WORKLOAD_ENS.replace("{n}", str(len(params))), "cases": len(params),
            "grid_points": sum(p[0] * p[1] for p in params),
            "seeds": "ensemble 2024, initial fields 1000 + case index",
            "l2": "GPU: flushed before the timed call (256 MiB memset outside the events); the state "
                  "(221 MB for 256 cases) exceeds L2"}


def transform_flops(params):
    """Useful flops per ensemble step of the dense transforms (the tensor-core
    work): per grid-point-step 26 (nx + ny) + 4 nx for a box and 26 ny for a
    periodic case (13 transforms of 2N flops per point, plus the two box
    eigenbasis products)."""
    f = 0.0
    for nx, ny, _ra, _pr, _dt, _asp, kind in params:
        per = 26 * ny if kind == 2 else 26 * (nx + ny) + 4 * nx
        f += float(per) * nx * ny
    return f


def step_state_bytes(params):
    """Compulsory HBM bytes per ensemble step: read and write of the spectral
    state {ux, uy, temp, pres[1]} (composite) and pres[0] (ortho), complex for
    periodic cases."""
    b = 0.0
    for nx, ny, _ra, _pr, _dt, _asp, kind in params:
        if kind == 2:
            sc, so, w = (nx // 2 + 1) * (ny - 2), (nx // 2 + 1) * ny, 2
        else:
            sc, so, w = (nx - 2) * (ny - 2), nx * ny, 1
        b += 2 * 8 * w * (4 * sc + so)
    return b


DETAIL_DIR = None  # --detail-dir: where per-launch detail files go (none written without it)


def side_file(name, obj):
    """Per-launch detail that would crowd the JSON line, into --detail-dir."""
    if DETAIL_DIR is None:
        return
    os.makedirs(DETAIL_DIR, exist_ok=True)
    with open(os.path.join(DETAIL_DIR, name), "w") as f:
        json.dump(obj, f, indent=1)


def ensemble_accuracy(R, params, steps):
    """Nu, KE and temperature of the batched mixed form against an FP64 batch
    (each FP64 batch case is bit-identical to the case stepped alone) after
    `steps` steps from the benchmark's initial fields."""
    import numpy as np
    out = {}
    for prec in (R.PREC_MIXED, R.PREC_FP64):
        b = R.Batch(params, precision=prec)
        for i, c in enumerate(b.cases):
            R.standard_ic(c, seed=1000 + i)
        b.update(steps)
        b.synchronize()
        out[prec] = ([c.eval(R.NU) for c in b.cases], [c.eval(R.KE) for c in b.cases],
                     [c.get(R.TEMP) for c in b.cases], [c.status() for c in b.cases])
        del b
    m, d = out[R.PREC_MIXED], out[R.PREC_FP64]
    nu = np.array([abs(a - r) / abs(r) for a, r in zip(m[0], d[0])])
    ke = np.array([abs(a - r) / abs(r) for a, r in zip(m[1], d[1])])
    tl = np.array([np.linalg.norm(a - r) / np.linalg.norm(r) for a, r in zip(m[2], d[2])])
    w = int(np.argmax(np.maximum(nu, ke)))
    return {"steps": steps, "against": "FP64 batch (= each case alone in FP64, <= 1e-9 of the oracle)",
            "nu_max_rel": float(nu.max()), "ke_max_rel": float(ke.max()), "temp_l2_max_rel": float(tl.max()),
            "nu_median_rel": float(np.median(nu)), "ke_median_rel": float(np.median(ke)),
            "status_nonzero": int(sum(1 for s in m[3] + d[3] if s)),
            "worst_case": {"case": w, "params": [round(x, 6) if isinstance(x, float) else x for x in params[w]],
                           "nu_rel": float(nu[w]), "ke_rel": float(ke[w])},
            "cases_nu_ke_within_1e-6": int(np.sum((nu <= 1e-6) & (ke <= 1e-6)))}


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
    # flushed once before (the state, 221 MB, and each step's scratch exceed L2)
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
    status_bad = int(sum(1 for c in B.cases if c.status()))
    # the same K steps, one call each with L2 flushed before every step
    flushed_ms = max_over_ranks(timed_steps(cu, stream, K, lambda: B.update(1), flush), world)
    value = gp * K / (total_ms * 1e-3) * world

    # ---- every launch of the step timed alone: the dominant kernel's roofline
    prof = B.profile_step(3)
    per_launch = [{"bucket": b_, "pass": p_, "kernel": k_, "ms": round(m_, 4), "bytes": b2_}
                  for b_, p_, k_, m_, b2_ in B.profile_launches(3)]
    tuning = [{"pass": t[0], "ms_cta_per_lane": t[1], "ms_thread_per_lane": t[2], "chosen": t[3]}
              for t in B.tuning()]
    forms = B.tuning_forms()
    dom = max(prof, key=lambda k: prof[k][0])
    dom_ms, dom_bytes = prof[dom]
    pk, pk_src = peaks()
    hbm = pk.get("hbm_gbs", 6800.0)
    step_bytes = step_state_bytes(params)
    if dom == "lane_gemm":
        # the tensor-core kernel: useful transform flops over its time, against
        # the TF32 dense rate (half the measured bf16 rate)
        tf32 = pk.get("bf16_tflops", 1900.0) / 2.0
        flops = transform_flops(params)
        achieved = flops / (dom_ms * 1e-3) / 1e12
        roof = {"bound": "tensor", "kernel": dom, "achieved": achieved, "peak": tf32, "unit": "TFLOP/s",
                "frac": achieved / tf32, "traffic": None, "flops_per_step": flops,
                "ms_per_step": dom_ms, "launches_per_step": sum(1 for x in per_launch if x["kernel"] == dom),
                "peak_source": "MEASURED_PEAKS.json bf16_tflops / 2 (TF32 dense rate), " + pk_src,
                "hbm_view": {"algorithmic_bytes": dom_bytes, "gbs": dom_bytes / (dom_ms * 1e-3) / 1e9}}
    else:
        achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": None, "algorithmic_bytes_per_step": dom_bytes,
                "ms_per_step": dom_ms, "peak_source": pk_src}
    roof["traffic_note"] = "not measured in this run (no profiler in the timed process); ncu DRAM bytes in profiles/"
    roof["step_hbm"] = {"bytes": step_bytes, "gbs": step_bytes / (total_ms / K * 1e-3) / 1e9,
                        "frac": step_bytes / (total_ms / K * 1e-3) / 1e9 / hbm}

    # ---- end to end through the public API (whole ensemble state in and out every step):
    # rbc_batch_step_io, whose per-group copies overlap the other group's step,
    # and, for comparison, the same copies and step as three calls in sequence
    # (three repetitions of each loop, median reported: the host link is
    # shared with the machine's other GPUs)
    nbytes = B.state_bytes()
    host = R.PinnedArray((nbytes,), np.uint8)
    B.get_state_all(host.array)
    Ke = min(K, 20)

    def e2e_median(one_step):
        runs = []
        for _rep in range(3):
            t0 = time.perf_counter()
            for _ in range(Ke):
                one_step()
            runs.append(time.perf_counter() - t0)
        return sorted(runs)[1], runs

    def sequential():
        B.set_state_all(host.array)
        B.update(1)
        B.get_state_all(host.array)

    e2e_s, e2e_runs = e2e_median(lambda: B.step_io(host.array, host.array, 1))
    e2e_seq_s, _ = e2e_median(sequential)
    del B
    side_file("bench_ensemble_detail.json", {"launches_ms": per_launch, "autotuner": tuning, "forms": forms,
                                              "kernels_ms_per_step": {k: v[0] for k, v in prof.items()}})

    line = {
        "metric": METRIC, "value": value, "unit": "grid-pt-steps/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 state/solves, tf32x3 tensor-core transforms, f32 products",
        "data": "synthetic seeded ensemble and fields",
        "config": ensemble_config(params),
    }
    if args.skip_plain:  # profiling runs: the batched mixed step only
        line.update({"autotuner_forms": forms, "kernels_ms_per_step": {k: v[0] for k, v in prof.items()}})
        return line

    # ---- plain FP64, case by case, same ensemble and initial fields
    plain_ms = 0.0
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
        del nav
    plain_value = gp * K / (plain_ms * 1e-3) * world

    line.update({
        "gpu_launches": K * launches,
        "e2e": {"value": gp * Ke / e2e_s * world, "unit": "grid-pt-steps/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes, "steps": Ke,
                "runs_s": [round(x, 4) for x in e2e_runs],
                "how": "per step: rbc_batch_step_io(pinned in, pinned out, 1): each group's state range copied in, "
                       "stepped, copied back on its own branch; median of 3 runs",
                "sequential_value": gp * Ke / e2e_seq_s * world,
                "sequential_how": "rbc_batch_set_state_all, rbc_batch_step(1), rbc_batch_get_state_all in sequence"},
        "roofline": roof,
        "clocks": clk,
        "timing": {"one_call_per_step_l2_flushed": gp * K / (flushed_ms * 1e-3) * world,
                   "setup_s": round(t_setup, 3), "wall_s_timed_region": round(t_wall, 4), "buckets": nb,
                   "launches_per_step": launches, "status_nonzero_cases": status_bad},
    })
    if rank == 0 and world == 1:
        line["serving"] = run_serving(args, args.requests, args.horizon_scale, args.serving_check)
        line["cpu_baseline"] = cpu_baseline_ensemble(params, steps=args.cpu_steps)
    line["plain_fp64"] = {"value": plain_value, "ms_per_ensemble_step": plain_ms / K,
                          "how": "each case alone through rbc_step, cases one after another"}
    line["speedup_vs_plain_fp64"] = value / plain_value
    line["mixed_error"] = ensemble_accuracy(R, params, args.accuracy_steps)
    return line


def cpu_ensemble_sample(O, params, steps, warmup):
    """The oracle on every case of the ensemble: `warmup` untimed steps, then
    `steps` timed ensemble steps (each advances every case once).  The cases
    run in parallel on the host threads, one case per thread at a time,
    largest first.  The one CPU sample of the ensemble, used by cpu_baseline
    and by the reference arm."""
    objs = []
    for i, p in enumerate(params):
        nx, ny, ra, pr, dt, asp, kind = p
        o = O.Navier2D(nx, ny, ra, pr, dt, asp, kind)
        O.standard_ic(o, 1000 + i)
        objs.append((o, nx * ny))
    objs.sort(key=lambda x: -x[1])
    navs = [o for o, _ in objs]
    if warmup > 0:
        O.update_many(navs, warmup)
    t0 = time.perf_counter()
    for _ in range(steps):
        O.update_many(navs, 1)
    secs = time.perf_counter() - t0
    gp = sum(g for _, g in objs)
    return gp * steps / secs, secs


def cpu_baseline_ensemble(params, steps=60):
    from oracle import oracle as O
    O.build()
    O.set_threads(os.cpu_count() or 1)
    v, secs = cpu_ensemble_sample(O, params, steps, 1)
    return {"value": v, "unit": "grid-pt-steps/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"all {len(params)} cases x {steps} ensemble steps after 1 warm-up step ({secs:.1f} s)"}


# ---------------------------------------------------------------------------
# serving: Poisson arrivals of solve requests, continuous batching
# ---------------------------------------------------------------------------
def run_serving(args, n_requests, horizon_scale, n_check=8):
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
    if DETAIL_DIR is not None:  # one JSON line per request
        os.makedirs(DETAIL_DIR, exist_ok=True)
        path = os.path.join(DETAIL_DIR, "serving_requests.jsonl")
        if os.path.exists(path):
            os.remove(path)
        srv.write_records(path, res)
    srv.close()
    lat = np.array([r["t_done"] - r["t_submit"] for r in res])
    setup = np.array([r["t_admit"] - r["t_submit"] for r in res])
    gp_steps = sum(r["grid_points"] * r["steps"] for r in res)
    span = max(r["t_done"] for r in res) - min(r["t_submit"] for r in res)
    errs_nu, errs_ke = [], []
    # the n_check cheapest results (steps x grid points) are re-run alone in FP64
    for r in sorted(res, key=lambda r: (r["steps"] * r["grid_points"], r["id"]))[:n_check]:
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
        "aggregate_grid_pt_steps_per_s": gp_steps / span, "span_s": round(span, 2),
        "graph_rebuilds": st["rebuilds"], "peak_device_gb": round(st["peak_bytes_in_use"] / 1e9, 2),
        "nu_max_rel_vs_fp64": float(max(errs_nu)), "ke_max_rel_vs_fp64": float(max(errs_ke)),
        "checked": len(errs_nu), "checked_how": "the cheapest results re-run alone in FP64",
        "horizon_scale": horizon_scale,
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
    if args.workload == "periodic512":
        o = O.Navier2D(NX, NY, RA, PR, DT, ASPECT, O.PERIODIC)
        O.standard_ic(o, 1)
        o.update(args.warmup)
        K = max(1, args.steps)
        t0 = time.perf_counter()
        o.update(K)
        secs = time.perf_counter() - t0
        v = NX * NY * K / secs
        config = {"workload": WORKLOAD_512, "nx": NX, "ny": NY}
        sample = f"{K} steps after {args.warmup} warm-up steps"
    else:
        from rustpde_gb300.ensemble import draw_ensemble
        params = draw_ensemble(args.cases, ENSEMBLE_SEED)
        K = max(1, args.steps)
        v, secs = cpu_ensemble_sample(O, params, K, args.warmup)
        config = ensemble_config(params)
        sample = f"all {len(params)} cases x {K} ensemble steps after {args.warmup} warm-up steps"
    return {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "grid-pt-steps/s", "n_gpus": world,
        "steps": K, "warmup": args.warmup, "ms_per_step": secs / K * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic seeded ensemble and fields",
        "config": config,
        "cpu_baseline": {"value": v, "unit": "grid-pt-steps/s", "cores": O.num_threads(), "kind": "port",
                         "sample": sample},
        "e2e": {"value": v, "unit": "grid-pt-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is Rust (no toolchain here or on the box): the C++ restatement in oracle/, "
                "FP64, the ensemble's cases in parallel on all host threads (one case per thread at a time)",
    }


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return "unknown"


def run_cpu_table(args):
    """The reference algorithm (the oracle, OpenMP over lanes) on the host
    cores for configurations 0-3, with all threads and with one, each on a
    bounded sample: per-step latency percentiles for the single cases, per
    stage times for the 1-D lanes, and the ensemble with its cases in parallel
    (one case per thread at a time)."""
    import numpy as np

    from oracle import oracle as O
    from rustpde_gb300.ensemble import draw_ensemble
    O.build()
    allc = os.cpu_count() or 1
    rows = []

    def single(name, p, steps):
        nx, ny = p[0], p[1]
        o = O.Navier2D(*p)
        O.standard_ic(o, 1)
        o.update(1)
        ts = []
        for _ in range(steps):
            t0 = time.perf_counter()
            o.update(1)
            ts.append(time.perf_counter() - t0)
        ts = np.array(ts)
        return {"config": name, "threads": O.num_threads(), "gp_steps_per_s": nx * ny * steps / ts.sum(),
                "p50_step_ms": float(np.percentile(ts, 50) * 1e3), "p99_step_ms": float(np.percentile(ts, 99) * 1e3),
                "sample": f"{steps} steps after 1 warm-up step"}

    for threads in (allc, 1):
        O.set_threads(threads)
        rows.append(single("0: box 64^2 Ra 1e5 dt 0.02", (64, 64, 1e5, 1.0, 0.02, 1.0, O.BOX_ADIABATIC),
                           100))
        rows.append(single("1: periodic 512x257 Ra 1e7 dt 1e-3", (NX, NY, RA, PR, DT, ASPECT, O.PERIODIC),
                           20 if threads > 1 else 5))
        rng = np.random.default_rng(11)
        for n in (128, 256, 512):
            m = n - 2
            spec = rng.standard_normal((4096, m)) * np.exp(-np.arange(m) / 20.0)
            phys = O.lanes_apply(O.CD, n, 1, spec)
            ortho = O.lanes_apply(O.CD, n, 2, spec)
            stage = {}
            for op, name, x in ((0, "forward", phys), (1, "backward", spec), (2, "to_ortho", spec),
                                (3, "from_ortho", ortho), (4, "hholtz", ortho)):
                O.lanes_apply(O.CD, n, op, x, 5e-4)
                reps = 3
                t0 = time.perf_counter()
                for _ in range(reps):
                    O.lanes_apply(O.CD, n, op, x, 5e-4)
                stage[name] = (time.perf_counter() - t0) / reps * 1e3
            rows.append({"config": f"2: 4096 lanes x N={n}, ChebDirichlet", "threads": O.num_threads(),
                         "ms_per_stage": stage})
        params = draw_ensemble(args.cases, ENSEMBLE_SEED)
        steps = 10 if threads > 1 else 2
        v, secs = cpu_ensemble_sample(O, params, steps, 1)
        rows.append({"config": "3: 256-case ensemble, cases in parallel (one per thread)", "threads": O.num_threads(),
                     "gp_steps_per_s": v, "sample": f"all {len(params)} cases x {steps} ensemble steps "
                                                       f"({secs:.1f} s)"})
    return {"workload": "cpu-table", "cpu_model": cpu_model(), "host_threads": allc,
            "what": "oracle/ (C++ restatement of the reference algorithm, FP64, -O3; OpenMP over lanes in "
                    "a single case, over cases in the ensemble)",
            "rows": rows}


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
    if args.periodic_only:  # the ensemble's periodic cases alone: a batch of one group
        params = [p for p in params if p[6] == R.PERIODIC]
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
    return {"workload": "profile-step" + (" (periodic cases)" if args.periodic_only else ""), "cases": len(params),
            "warmup": args.warmup, "launches_in_step": launches,
            "autotuner_forms": B.tuning_forms(), "status_max": max(c.status() for c in B.cases)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ensemble",
                    choices=["ensemble", "periodic512", "serving", "precision", "extras", "profile-step",
                             "cpu-table"])
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="periodic512: oracle seconds")
    ap.add_argument("--cpu-steps", type=int, default=60, help="ensemble: oracle ensemble steps in cpu_baseline")
    ap.add_argument("--accuracy-steps", type=int, default=505,
                    help="ensemble: steps of the mixed-vs-FP64 comparison (the configuration's horizon)")
    ap.add_argument("--cases", type=int, default=ENSEMBLE_N, help="ensemble size (default 256)")
    ap.add_argument("--detail-dir", default=None,
                    help="directory for the ensemble's per-launch detail file (bench_ensemble_detail.json)")
    ap.add_argument("--periodic-only", action="store_true",
                    help="profile-step: the ensemble's periodic cases alone (one group)")
    ap.add_argument("--skip-plain", action="store_true",
                    help="time the batched mixed step only (profiling runs; prints a reduced line)")
    ap.add_argument("--requests", type=int, default=100, help="serving: number of requests")
    ap.add_argument("--horizon-scale", type=float, default=0.1, help="serving: horizon multiplier")
    ap.add_argument("--serving-check", type=int, default=8,
                    help="serving: results re-run alone in FP64 for the Nu/KE error")
    args = ap.parse_args()
    global DETAIL_DIR
    DETAIL_DIR = args.detail_dir
    if args.steps is None:
        # the reference arm's ensemble step is every case on the CPU (about 1.5 s)
        if args.workload == "ensemble":
            args.steps = 20 if args.impl == "reference" else 500
        else:
            args.steps = 200
    rank, world, local = dist_info()
    if world > 1 and args.impl == "ours":
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("gloo")
    if args.impl == "ours" and args.workload != "cpu-table":
        # the library links its own CUDA runtime: select the rank's GPU there too
        import rustpde_gb300 as R
        from rustpde_gb300 import build
        build.build()
        R.set_device(local)
        assert R.get_device() == local
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    elif args.workload == "precision":
        line = run_precision(args)
    elif args.workload == "extras":
        line = run_extras(args)
    elif args.workload == "profile-step":
        line = run_profile_step(args)
    elif args.workload == "cpu-table":
        line = run_cpu_table(args)
    elif args.workload == "serving":
        from rustpde_gb300 import build
        build.build()
        line = {"metric": METRIC, "workload": "serving",
                **run_serving(args, args.requests, args.horizon_scale, args.serving_check)}
    else:
        args.warmup = max(args.warmup, 3)
        line = (run_ensemble if args.workload == "ensemble" else run_periodic512)(args, rank, world, local)
    if rank == 0 and line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
