"""Benchmark of the raytracer_3D time-stepping path on GB300.

Workload (N=1): the 32^3 x 32^3 wave field with a mean flow
U = 0.1 sin(2 pi y/Ly) exp(z/500), log-normal spectrum, CFL 0.4, plain
binary64 form (1,073,741,824 cells per step).  A step is one forward-Euler
time step of the whole field with the schedule the autotuner picks (the
division-free two-pass step: flux pass and update pass, two launches).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  `value` = cell-updates/s with the state resident in
HBM, timed with CUDA events on the library's own stream; `e2e` = the same
metric through the host-array drop-in call rt_integrate_host (upload,
step, download each step).  The state (8.6 GB) is far larger than L2, so no
L2 flush is needed between steps.  N>1 runs N independent replicas, one per
GPU (the path does not shard), with a barrier and max-over-ranks timing.
`--impl reference` times the CPU restatement of the reference path on the
host cores instead (the Fortran reference cannot be built on this machine).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "6D cell-updates/s"
UNIT = "cell-updates/s"
B_ALG = {"fp64": 72, "fp32": 36}   # algorithmic bytes per cell-update (E r/w + 6 velocities + 1 rate)
WORKLOAD = dict(n=(32, 32, 32, 32, 32, 32))
# CPU sample grids: the oracle holds the reference's 20 padded binary64 fields
# (+2 cells on every axis), 348 GB at 32^6, so it runs on the largest cube
# the host's memory holds; per-cell rates are compared, and the padded /
# interior ratio of the sample is stated beside the rate (2.03 at 32^6)
CPU_SAMPLES = ((24,) * 6, (16,) * 6)


def host_ram_bytes():
    try:
        return os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES")
    except (ValueError, OSError, AttributeError):
        return 0


def cpu_sample_grid(override=None):
    """the sample cube: `override` (cube size) or the largest of CPU_SAMPLES
    whose 20 padded binary64 fields fit in half the host memory"""
    if override:
        return (int(override),) * 6
    ram = host_ram_bytes()
    for n in CPU_SAMPLES:
        padded = 1
        for k in n:
            padded *= k + 4
        if 20 * 8 * padded <= ram / 2:
            return n
    return CPU_SAMPLES[-1]


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(kernel_key, with_source=False):
    """per-cell DRAM bytes of a kernel from the committed ncu summary (and
    the summary it comes from)"""
    p = os.path.join(ROOT, "profiles", "dram_traffic.json")
    e = None
    if os.path.exists(p):
        with open(p) as f:
            e = json.load(f).get(kernel_key)
    b = None if e is None else float(e["bytes_per_cell"])
    return (b, None if e is None else e.get("source")) if with_source else b


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region"""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# distributed plumbing (replicas only)
# ---------------------------------------------------------------------------
def dist_init(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world <= 1:
        return 0, 1, 0, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    torch.cuda.set_device(local)
    dist.init_process_group("gloo")
    return rank, world, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (restatement of the reference path) with OpenMP
# ---------------------------------------------------------------------------
def cpu_baseline(steps, warmup=1, n=None):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle import build_oracle as bo
    bo.build()
    from harness import build_oracle
    from raytracer_3d_gb300 import configs
    n = n or cpu_sample_grid()
    exp = configs.jet_large(n=n)
    o = build_oracle(exp, threads=True)
    o.integrate(warmup)
    t0 = time.perf_counter()
    o.integrate(steps)
    dt = time.perf_counter() - t0
    cells = exp.cells
    value = cells * steps / dt
    ratio = 1.0
    for k in n:
        ratio *= (k + 4) / k
    sample = ("jet_large physics (U=0.1 sin(2 pi y/Ly) exp(z/500), CFL 0.4) on a %s grid, %d steps after %d "
              "warm-up, padded reference layout (padded/interior cells %.2f; 2.03 at 32^6, whose 348 GB of "
              "fields exceed this host's %.0f GB), OpenMP over the outer m loop"
              % ("x".join(map(str, n)), steps, warmup, ratio, host_ram_bytes() / 1e9))
    return {"value": value, "unit": UNIT, "cores": o.threads(), "kind": "port", "sample": sample,
            "seconds": dt}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def time_steps(model, steps):
    import torch
    stream = torch.cuda.ExternalStream(model.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    l0 = model.launch_count()
    e0.record(stream)
    model.integrate(steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3, model.launch_count() - l0


FP32_CANDIDATES = ([(v, b, t, s) for v in ("w2z", "w2q", "w3", "w6") for t in (128, 256, 512) for b in (4, 8)
                    for s in (0, 1)]
                   + [("tma", b, t, s) for t in (256, 512, 1024) for b in (4, 8) for s in (0, 1)])


# binary64: the fused plane kernel, the two-pass step that evaluates every
# face flux once (both bit-identical to the reference's arithmetic), or the
# two-pass step without divisions (within 1e-12 relative per step); all are
# bound by the binary64 pipe, and dry steps pick the fastest
FP64_CANDIDATES = [("tma", 8, 256, 0), ("split", 8, 256, 0), ("fast", 8, 256, 0)]


def fp64_ops_per_cell(schedule, n, lower_reflection=True):
    """binary64 pipe instructions (add, multiply, fma; each counted once) per
    cell-update of the fast schedule, from its source: per axis with n > 1,
    4 per right-face flux (Rj, the upwind difference, v*E_up, the fma with
    h; 3 along x when nx divides 32, where the lanes of a row share their
    differences) and 2 in the update (F_l - F_r, the fma with dt/d); the
    face-0 flux of an axis, once per n cells, costs 1 (v*E(0), the edge
    copied into the ghosts) or 4 (z with the lower reflection); plus the
    final fma with mu.  None for the bit-exact schedules, whose divisions
    and comparisons are compiler sequences (their counts come from ncu,
    profiles/)."""
    if schedule != "fast":
        return None
    ops = 1.0
    for a, k in enumerate(n):
        if k > 1:
            face0 = 4.0 if (a == 2 and lower_reflection) else 1.0
            flux = 3.0 if (a == 0 and 32 % k == 0) else 4.0
            ops += flux + 2.0 + face0 / k
    return ops


def fp64_peak():
    """binary64 fma instructions per second of this GPU (rt_fp64_rate, best
    of three), with the clocks seen while it ran"""
    import ctypes
    import torch
    from raytracer_3d_gb300 import _lib
    lib = _lib.load()
    best = 0.0
    with ClockSampler(torch.cuda.current_device()) as cs:
        for _ in range(3):
            r = ctypes.c_double()
            if lib.rt_fp64_rate(ctypes.byref(r)) == 0:
                best = max(best, r.value)
    return {"fma_per_s": best, "clocks": cs.summary(),
            "how": "rt_fp64_rate: 8 or 16 independent fma chains per thread, 4 or 8 CTAs of 256 threads per SM, "
                   "CUDA events on the second launch of each shape; best of 3 calls"}


# committed per-cell DRAM traffic (profiles/dram_traffic.json) of each timed binary32 kernel
FP32_TRAFFIC = {"w2z": "step_fp32_w2z", "w2q": "step_fp32_w2q", "w3": "step_fp32_w3"}

SCHEDULE_NOTES = {
    "fast": "two passes without divisions (rt_fast.cu): within 1e-12 relative L-inf of the reference per step, "
            "not bit-identical",
    "split": "two passes, the reference's arithmetic bit for bit (rt_split.cu)",
    "tma": "fused plane kernel, the reference's arithmetic bit for bit (rt_step3.cuh)",
}


def run_form(precision, n, steps, warmup, dist, e2e_steps, sched=None, tune=False, candidates=None,
             final_step=0):
    """time one form on the jet workload; with final_step > 0 the model is
    then restarted from the initial state rounded to binary32 (the input
    both precisions can hold exactly), stepped final_step times, and its
    interior is returned (out["final"]) for the error against the other
    precision"""
    import numpy as np
    import torch
    from raytracer_3d_gb300 import configs
    exp = configs.jet_large(n=n)
    m = configs.build_model(exp, precision)
    tuned = None
    table = None
    if tune:
        from raytracer_3d_gb300.autotune import tune_model
        tuned, table = tune_model(m, candidates=candidates or FP32_CANDIDATES, reps=2, use_cache=False)
    elif sched:
        m.set_tuning(*sched)
    cells = exp.cells
    m.integrate(warmup)
    torch.cuda.synchronize()
    barrier(dist)
    with ClockSampler(torch.cuda.current_device()) as cs:
        secs, launches = time_steps(m, steps)
    secs = max_over_ranks(dist, secs)
    out = {"cells": cells, "seconds": secs, "launches": launches, "clocks": cs.summary(), "dt": m.dt,
           "schedule": tuned or sched,
           "tuning_table_ms": None if table is None else [["%s b%d t%d s%d" % c, round(1e3 * t, 3)]
                                                           for c, t in table]}
    # end to end through the host-array drop-in (rt_integrate_host)
    if e2e_steps > 0:
        m.get_state()
        m.integrate_host()  # warm-up of the host path
        torch.cuda.synchronize()
        barrier(dist)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            m.integrate_host()
        t1 = time.perf_counter()
        e2e_secs = max_over_ranks(dist, t1 - t0)
        out["e2e"] = {"seconds": e2e_secs, "steps": e2e_steps,
                      "bytes": cells * 8, "host_access": "direct" if m.host_direct() else "staged"}
        out["finite"] = bool(np.isfinite(m.E).all())
    if final_step > 0:
        E0 = initial_interior(exp, m).astype(np.float32).astype(np.float64)
        out["energy0"] = energy_sum(E0, vol_weights(m))
        sl = tuple(slice(2, 2 + k) for k in m.n)
        m.E[sl] = E0
        m.set_state()
        m.integrate(final_step)
        out["final"] = np.array(m.get_state()[sl], dtype=np.float64, order="F")
        out["widths"] = vol_weights(m)
    m.close()
    return out


def vol_weights(model):
    return [model.grid["xyzklm"[a]]["dt"][2:2 + model.n[a]] for a in range(6)]


def initial_interior(exp, model):
    """the experiment's initial state (interior, binary64), rebuilt from its
    seed on a stand-in that carries only what the initial conditions read"""
    import numpy as np

    class Shell:
        pass
    shell = Shell()
    shell.n, shell.padded, shell.grid = model.n, False, model.grid
    shell.E = np.zeros(model.n, order="F")
    exp.initial(shell, np.random.Generator(np.random.PCG64(exp.seed)))
    return shell.E


def energy_sum(E, widths):
    """sum(E*vol) of an interior 6D array, one m plane at a time"""
    import numpy as np
    v5 = np.ones([len(w) for w in widths[:5]])
    for a in range(5):
        shp = [1] * 5
        shp[a] = len(widths[a])
        v5 = v5 * widths[a].reshape(shp)
    return sum(float(np.sum(np.asarray(E[..., m], dtype=np.float64) * v5)) * float(widths[5][m])
               for m in range(E.shape[5]))


def error_against(got, ref, widths, energy0=None):
    """relative L2 and L-inf (to max |ref|) of got - ref and the relative
    total-energy difference, one m plane at a time"""
    import numpy as np
    num2 = den2 = dmax = rmax = 0.0
    for m in range(ref.shape[5]):
        r = np.asarray(ref[..., m], dtype=np.float64)
        d = np.asarray(got[..., m], dtype=np.float64) - r
        num2 += float(np.sum(d * d))
        den2 += float(np.sum(r * r))
        dmax = max(dmax, float(np.max(np.abs(d))))
        rmax = max(rmax, float(np.max(np.abs(r))))
    e_ref, e_got = energy_sum(ref, widths), energy_sum(got, widths)
    out = {"l2": (num2 / den2) ** 0.5, "linf": dmax / rmax, "energy": abs(e_got - e_ref) / abs(e_ref)}
    if energy0:
        out["reference_energy_change"] = abs(e_ref - energy0) / abs(energy0)
    return out


def bench_batched(steps, warmup, members=48, seed=2024, fixed=None, spatial=None, error_steps=0):
    """48 independent fp32 instances (dims per axis from {8,16,24,32} spatial
    and {8,12,16,24} spectral, own N0, f, mean-flow amplitude, packet init)
    advanced by one persistent, graph-captured launch per step, with the
    schedule chosen by the autotuner."""
    import numpy as np
    import torch
    from raytracer_3d_gb300 import configs
    from raytracer_3d_gb300.autotune import tune_batch
    from raytracer_3d_gb300.batch import Batch
    rng = np.random.default_rng(seed)
    kw = {"spatial": spatial} if spatial else {}
    exps = [configs.ensemble_member(rng, steps=500, **kw) for _ in range(members)]
    t0 = time.perf_counter()
    models = []
    for e in exps:
        models.append(configs.build_model(e, "fp32", padded=False))   # no padded host array
    setup_s = time.perf_counter() - t0
    b = Batch(models)
    if fixed:   # band, threads, sweep, persistent threads[, slice threads[, fused]] (profiling runs)
        fixed = tuple(fixed) + (-1, 0)[len(fixed) - 4:]
        b.set_tuning(fixed[0], fixed[1], fixed[2], 16)
        b.set_persistent(fixed[3])
        b.set_slices(fixed[4])
        b.set_fused(fixed[5])
        best = fixed
    else:
        best, table = tune_batch(b, reps=2, use_cache=False)
    b.integrate(warmup)
    b.sync()
    stream = torch.cuda.ExternalStream(b.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    l0 = b.launch_count()
    with ClockSampler(torch.cuda.current_device()) as cs:
        e0.record(stream)
        b.integrate(steps)
        e1.record(stream)
        e1.synchronize()
    secs = e0.elapsed_time(e1) / 1e3
    b.sync()
    launches = b.launch_count() - l0
    cells = b.cells
    # the fastest schedule that steps both warp-specialised classes in ONE
    # launch, timed the same way when the tuner preferred another
    one_launch = None
    if not fixed:
        fused = [c for c, _ in table if len(c) > 5 and c[5] == 1 and c[3] == c[4] and c[3] > 0]
        if fused and tuple(fused[0]) != tuple(best):
            c = fused[0]
            b.set_tuning(c[0], c[1], c[2], 16)
            b.set_persistent(c[3])
            b.set_slices(c[4])
            b.set_fused(1)
            b.integrate(warmup)
            b.sync()
            f0 = torch.cuda.Event(enable_timing=True)
            f1 = torch.cuda.Event(enable_timing=True)
            k0 = b.launch_count()
            f0.record(stream)
            b.integrate(steps)
            f1.record(stream)
            f1.synchronize()
            fsecs = f0.elapsed_time(f1) / 1e3
            one_launch = {"value": cells * steps / fsecs, "ms_per_step": 1e3 * fsecs / steps,
                          "launches_per_step": (b.launch_count() - k0) / steps,
                          "tuning": {"band": c[0], "threads": c[1], "sweep": c[2], "persistent_threads": c[3],
                                     "slice_threads": c[4], "fused": True}}
            b.set_tuning(best[0], best[1], best[2], 16)   # back to the timed schedule for the error run
            b.set_persistent(best[3])
            b.set_slices(best[4])
            b.set_fused(best[5] if len(best) > 5 else 0)
        elif fused:
            one_launch = "the timed schedule"
    error = None
    if error_steps > 0:
        # every member on to error_steps in the batch, then each alone in
        # binary64 (the fast schedule) from the same initial state
        taken = (warmup + steps) * (2 if isinstance(one_launch, dict) else 1)
        if error_steps > taken:
            b.integrate(error_steps - taken)
        b.sync()
        worst = {"l2": 0.0, "linf": 0.0, "energy": 0.0}
        tot32 = tot64 = 0.0
        for e, m in zip(exps, models):
            got = m.get_state()
            r = configs.build_model(e, "fp64", padded=False)
            r.E = np.asfortranarray(r.E.astype(np.float32).astype(np.float64))   # the binary32 member's input
            r.set_state()
            r.set_tuning("fast", 8, 256)
            r.integrate(max(error_steps, taken))
            ref = r.get_state()
            w = vol_weights(r)
            err = error_against(got, ref, w)
            tot32 += energy_sum(got, w)
            tot64 += energy_sum(ref, w)
            r.close()
            for k in worst:
                worst[k] = max(worst[k], err[k])
        error = {"steps": max(error_steps, taken), "worst_member": worst,
                 "ensemble_energy": abs(tot32 - tot64) / abs(tot64),
                 "reference": "each member alone in binary64 (fast schedule, within 1e-12 per step of the "
                              "reference's arithmetic) from the member's binary32 initial state"}
    out = {"value": cells * steps / secs, "unit": UNIT, "members": members, "cells_per_step": cells,
           "steps": steps, "ms_per_step": 1e3 * secs / steps, "launches": launches,
           "graph_steps": b.tuning[3],
           "tuning": {"band": best[0], "threads": best[1], "sweep": best[2], "persistent_threads": best[3],
                      "slice_threads": best[4], "fused": bool(best[5]) if len(best) > 5 else False,
                      "staged_members": b.persistent_members()},
           "launches_per_step": launches / steps,
           "roofline": roofline("fp32", cells, secs / steps, "batch_fp32"), "clocks": cs.summary(),
           "setup_s": round(setup_s, 2), "error": error, "one_launch_per_step": one_launch}
    b.close()
    for m in models:
        m.close()
    return out


def bench_serving(nreq=60, rate=20.0, seed=77, budget=120e9, baseline_req=12, stable_rate=1.5, stable_req=30,
                  fp64_schedule=("fast", 8, 256, 0)):
    """Poisson arrivals (mean 20/s), step counts uniform in [50,1000], dims
    as the batched form, 120 GB HBM budget, fp32 continuous batching; the
    same at an arrival rate the GPU keeps up with; and the fp64
    one-at-a-time baseline on the first requests of the same trace."""
    from raytracer_3d_gb300.serve import GpuExecutor, SequentialExecutor, Server, poisson_requests

    def serve(reqs):
        ex = GpuExecutor("fp32", batch_tuning=(8, 512, 1, 16), persistent=512)
        rep = Server(ex, budget_bytes=budget, chunk_max=50, setup_workers=8).run(reqs)
        ex.close()
        breakdown = {k: round(v, 2) for k, v in ex.times.items()}
        breakdown["batch_rebuilds"] = ex.rebuilds
        for r in reqs:
            r.result = None
        return rep.summary(), breakdown

    s, breakdown = serve(poisson_requests(nreq, rate=rate, seed=seed))
    st, _ = serve(poisson_requests(stable_req, rate=stable_rate, seed=seed + 1))
    base = poisson_requests(nreq, rate=rate, seed=seed)[:baseline_req]
    exb = SequentialExecutor("fp64", schedule=fp64_schedule)
    repb = Server(exb, budget_bytes=budget, chunk_max=10 ** 9, max_members=1).run(base)
    sb = repb.summary()
    return {"requests": nreq, "arrival_rate_per_s": rate, "budget_bytes": budget,
            "p50_s": s["p50_s"], "p99_s": s["p99_s"], "value": s["cell_updates_per_s"], "unit": UNIT,
            "makespan_s": s["makespan_s"], "chunks": s["chunks"], "backlog_max": s["backlog_max"],
            "peak_bytes": s["peak_bytes"], "seconds_by_activity": breakdown,
            "spectral_dims": "each of k, l, m from {8, 12, 16, 24}",
            "stable_load": {"requests": stable_req, "arrival_rate_per_s": stable_rate, "p50_s": st["p50_s"],
                            "p99_s": st["p99_s"], "value": st["cell_updates_per_s"],
                            "makespan_s": st["makespan_s"], "backlog_max": st["backlog_max"]},
            "fp64_one_at_a_time": {"requests": baseline_req, "trace": "the first requests of the 20/s trace",
                                   "schedule": fp64_schedule[0], "value": sb["cell_updates_per_s"],
                                   "p50_s": sb["p50_s"], "p99_s": sb["p99_s"]}}


def roofline(precision, cells, seconds_per_launch, traffic_key=None, fp64=None):
    """HBM roofline of one step (algorithmic bytes per cell x cells / step
    time against the measured copy bandwidth); for the binary64 form, given
    fp64 = (ops per cell, measured fma/s), the binary64-pipe roofline that
    bounds it, with the HBM figures beside it"""
    peak, src = peaks()
    achieved = B_ALG[precision] * cells / seconds_per_launch / 1e9
    tb, tsrc = profile_traffic(traffic_key or "step_%s" % precision, with_source=True)
    hbm = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
           "frac": round(achieved / peak, 4), "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % src
           if src == "measured" else "fallback 6.8 TB/s",
           "traffic": None if tb is None else tb * cells, "traffic_source": tsrc,
           "alg_bytes_per_cell": B_ALG[precision]}
    if fp64 is None or fp64[0] is None or not fp64[1]:
        return hbm
    ops, rate = fp64
    got = ops * cells / seconds_per_launch / 1e9
    return {"bound": "fp64", "achieved": round(got, 2), "peak": round(rate / 1e9, 2),
            "unit": "G binary64 ops/s", "frac": round(got / (rate / 1e9), 4),
            "peak_source": "measured in this run (rt_fp64_rate: binary64 fma instructions/s)",
            "ops_per_cell": round(ops, 4), "traffic": hbm["traffic"], "traffic_source": tsrc,
            "hbm": {k: hbm[k] for k in ("achieved", "peak", "unit", "frac", "peak_source", "alg_bytes_per_cell")}}


def gpu_arm(args):
    rank, world, local, dist = dist_init(args.gpus)
    n = tuple(int(v) for v in args.dims.split(",")) if args.dims else (args.n,) * 6
    sched = (args.variant, args.band, args.threads, args.sweep)
    if args.only == "serve":   # the serving form alone
        out = bench_serving(nreq=args.serve_requests)
        if rank == 0:
            print(json.dumps({"profile_only": "serving", **out}), flush=True)
        return
    if args.only == "batch":   # profiling runs of the batched form only
        out = bench_batched(args.batch_steps, args.warmup, members=args.batch_members,
                            fixed=tuple(int(v) for v in args.batch_tuning.split(",")) if args.batch_tuning else None,
                            spatial=tuple(int(v) for v in args.batch_spatial.split(",")) if args.batch_spatial else None)
        if rank == 0:
            print(json.dumps({"profile_only": "fp32_batched", **out}), flush=True)
        return
    if args.no_fp64:  # profiling runs of the fp32 form only
        f32 = run_form("fp32", n, args.steps, args.warmup, dist, 0, sched, tune=args.tune)
        if rank == 0:
            ms = 1e3 * f32["seconds"] / args.steps
            print(json.dumps({"profile_only": "fp32", "dims": n, "cells": f32["cells"], "ms_per_step": ms,
                              "cells_per_s": f32["cells"] / (ms / 1e3),
                              "schedule": f32["schedule"], "tuning_table_ms": f32["tuning_table_ms"],
                              "roofline": roofline("fp32", f32["cells"], ms / 1e3)}), flush=True)
        return
    # the binary64 form is bound by the FP64 pipe; 256-thread CTAs keep its
    # registers unspilled (the flags set the fp32 schedule when --tune 0)
    peak64 = fp64_peak()
    err_steps = 0 if args.no_fp32 else args.error_steps
    if args.fp64_variant:
        main = run_form("fp64", n, args.steps, args.warmup, dist, args.e2e_steps, (args.fp64_variant, 8, 256, 0),
                        final_step=err_steps)
    else:
        main = run_form("fp64", n, args.steps, args.warmup, dist, args.e2e_steps, FP64_CANDIDATES[-1],
                        tune=args.tune, candidates=FP64_CANDIDATES, final_step=err_steps)
    f64_sched = tuple(main["schedule"])
    f64_key = {"split": "step_fp64_split", "fast": "step_fp64_fast"}.get(f64_sched[0], "step_fp64")
    forms = {}
    if not args.no_fp32:
        f32 = run_form("fp32", n, args.steps, args.warmup, dist, 0, sched, tune=args.tune, final_step=err_steps)
        error = None
        if err_steps:
            error = error_against(f32.pop("final"), main["final"], main["widths"], main.get("energy0"))
            error.update({"steps": err_steps, "reference": "the binary64 run of this bench line (schedule %s) "
                          "from the same initial state (rounded to binary32 for both)" % f64_sched[0]})
        forms["fp32"] = {"value": f32["cells"] * args.steps * world / f32["seconds"], "error": error,
                         "ms_per_step": 1e3 * f32["seconds"] / args.steps,
                         "schedule": "%s band %d threads %d sweep %d" % tuple(f32["schedule"]),
                         "tuning_table_ms": f32["tuning_table_ms"],
                         "roofline": roofline("fp32", f32["cells"], f32["seconds"] / args.steps,
                                              FP32_TRAFFIC.get(f32["schedule"][0], "none")),
                         "clocks": f32["clocks"]}
    if not args.no_batch:
        forms["fp32_batched"] = bench_batched(
            args.batch_steps, args.warmup, members=args.batch_members, error_steps=args.batch_error_steps,
            fixed=tuple(int(v) for v in args.batch_tuning.split(",")) if args.batch_tuning else None)
    if not args.no_serve:
        forms["serving"] = bench_serving(nreq=args.serve_requests)
    cells = main["cells"]
    value = cells * args.steps * world / main["seconds"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * main["seconds"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded log-normal spectrum, analytic N(z), U(y,z))",
        "config": {"workload": "jet_large %d^3x%d^3 plain fp64, CFL 0.4 (dt=%%.6g s)" % (n[0], n[0]) % main["dt"],
                   "cells": cells, "form": "fp64", "schedule": "%s band %d threads %d sweep %d" % f64_sched,
                   "schedule_note": SCHEDULE_NOTES.get(f64_sched[0], ""),
                   "tuning_table_ms": main["tuning_table_ms"], "l2": "state 8.6 GB per field >> L2; no flush needed",
                   "parallelism": "replicas x%d" % world},
        "roofline": roofline("fp64", cells, main["seconds"] / args.steps, f64_key,
                             fp64=(fp64_ops_per_cell(f64_sched[0], n), peak64["fma_per_s"])),
        "fp64_peak": peak64,
        "clocks": main["clocks"],
        "gpu_launches": main["launches"],
    }
    if "e2e" in main:
        e = main["e2e"]
        line["e2e"] = {"value": cells * e["steps"] * world / e["seconds"], "unit": UNIT,
                       "h2d_bytes_per_step": e["bytes"], "d2h_bytes_per_step": e["bytes"],
                       "api": "rt_integrate_host (padded host array in, stepped array out)",
                       "host_access": e["host_access"]}
    line["forms"] = forms
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args.cpu_steps, n=cpu_sample_grid(args.cpu_sample))
        line["cpu_baseline"].pop("seconds", None)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    n = cpu_sample_grid(args.cpu_sample)
    cb = cpu_baseline(args.steps, warmup=args.warmup, n=n)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * cb["seconds"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": "jet_large 32^3x32^3 plain fp64, CFL 0.4",
                                             "cells": 32 ** 6, "form": "fp64",
                                             "sample_grid": "x".join(map(str, n)),
                                             "sample": "each step is a bounded sample: the same physics "
                                                       "on the sample grid (the rate is per cell)"},
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-steps", type=int, default=10)
    ap.add_argument("--cpu-sample", type=int, default=None,
                    help="cube size of the CPU sample (default: the largest that fits the host memory)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp32", action="store_true")
    ap.add_argument("--n", type=int, default=32, help="cube size of the workload (profiling of small cases)")
    ap.add_argument("--dims", default=None, help="nx,ny,nz,nk,nl,nm of a profiling case (with --no-fp64)")
    ap.add_argument("--variant", default="tma", choices=("w2z", "w2q", "w6", "w3", "tma", "group", "plane", "cell"))
    ap.add_argument("--fp64-variant", default=None, choices=("tma", "split", "fast"),
                    help="binary64 schedule (default: the fastest of the candidates by dry steps)")
    ap.add_argument("--band", type=int, default=8)
    ap.add_argument("--threads", type=int, default=1024)
    ap.add_argument("--sweep", type=int, default=0)
    ap.add_argument("--tune", type=int, default=1, help="autotune the fp32 schedule (1) or use the flags (0)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the fp64 form (profiling only)")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--batch-steps", type=int, default=50)
    ap.add_argument("--batch-members", type=int, default=48)
    ap.add_argument("--batch-spatial", default=None, help="spatial extents of the members, e.g. 8,16 (profiling)")
    ap.add_argument("--batch-tuning", default=None,
                    help="band,threads,sweep,persistent[,slices[,fused]]: a fixed batch schedule instead of the batch tuner")
    ap.add_argument("--only", default="all", choices=("all", "batch", "serve"),
                    help="batch / serve: that form alone (profiling)")
    ap.add_argument("--serve-requests", type=int, default=60)
    ap.add_argument("--error-steps", type=int, default=1000,
                    help="binary32 error against binary64 after this many steps (0: skip)")
    ap.add_argument("--batch-error-steps", type=int, default=500,
                    help="ensemble error against binary64 members after this many steps (0: skip)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        reference_arm(args)
    else:
        import __graft_entry__ as g
        g.build()
        gpu_arm(args)


if __name__ == "__main__":
    main()
