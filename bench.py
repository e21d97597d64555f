#!/usr/bin/env python
"""Throughput of the SPH particle step on GB300.

Workload: the 3D throughput configuration at 1,000,000 particles -- a
jittered 100^3 lattice filling the unit cube (+-0.1 dx uniform jitter,
seeded), h = 1.2 dx, velocities N(0, 0.01^2), rho0 = 1, Tait c0 = 1,
Monaghan alpha = 0.1; one step = NNPS + SPHRho + Tait + pressure gradient
+ artificial viscosity + RK2 (two evaluations).  Inputs are synthetic.

Metric: pair interactions per second = 4 * K * N / step time (K = mean
neighbour count including self; 2 pair passes x 2 evaluations per RK2 step),
summed over all GPUs (independent replicas, weak scaling).

``value`` is timed on the device with CUDA events around each step (inputs
resident in HBM; L2 flushed between steps outside the timed events).
``e2e`` is the same metric through the public API with host buffers: every
step uploads the particle state from pinned host memory, integrates, and
reads the new state back -- with staged transfers (``ParticleArray.upload`` /
``set_staged`` / ``download``: the link runs on copy streams beside the
neighbouring steps' computation), and, under ``e2e.serial``, with
``ParticleArray.set`` -> integrate -> ``get``.

``--impl reference`` times the reference PySPH's own Cython path (built by
``oracle/build_ref.py`` into ``oracle/_ref``) on the host cores instead: one
single-threaded process per core, each stepping a bounded sample of the same
workload (a 32^3 lattice with the same spacing ratio).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "pair interactions/s (3D SPH RK2 step, NNPS+SPHRho+Tait+PGrad+AV)"
UNIT = "pair-interactions/s"
DT = 1e-4

# Algorithmic bytes per particle per launch (FP32 snapshot reads + FP64
# outputs the interface requires; neighbour re-reads excluded):
#   rates:   pm+velh+st 48 B read, FP64 velocity 24 B read (position
#            stepping), FP64 rates 48 B written                    = 120 B
#   density: pm+velh 32 B read, FP64 rho,p,cs 24 B + st 16 B written = 72 B
ALG_BYTES = {"RatesStage": 120.0, "DensityStage": 72.0, "ListStage": 8.0}
# Compulsory HBM bytes of a whole RK2 step per particle (3D): cell keys,
# counting sort, reorder, density + Tait, momentum, per evaluation, plus the
# predictor and final integrator updates
STEP_ALG_BYTES = 694.0
# FLOPs per neighbour pair: density 24, momentum 72 (FMA = 2)
PAIR_FLOPS = {"RatesStage": 72.0, "DensityStage": 24.0, "ListStage": 12.0}
FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12
# DRAM bytes per particle per launch (dram__bytes_read.sum + dram__bytes_write.sum
# of one ncu capture of the 1M-particle lattice, brick-staged passes at cell
# subdivision 2); the traffic grows with the particle count, so it is scaled
# by n
NCU_TRAFFIC_PER_PARTICLE = {"DensityStage": 222.3, "RatesStage": 286.1}
# The unit that bounds each pair kernel in the same capture, as a fraction of
# that unit's peak: the rates pass is bound by the L1 / shared-memory pipe
# that serves its staged-record reads (and their latency), the density pass
# by instruction issue
NCU_LIMITER = {
    "RatesStage": {"kernel": "k_brates", "unit": "L1 / shared-memory pipe", "frac": 0.702,
                   "issue_frac": 0.618, "dram_frac": 0.141},
    "DensityStage": {"kernel": "k_bdensity", "unit": "instruction issue", "frac": 0.646,
                     "l1_frac": 0.603, "dram_frac": 0.179},
}


def fp32_peak_tflops():
    """FP32 FMA peak: 152 SMs x 128 lanes x 2 FLOP x the maximum SM clock
    measured on this machine (MEASURED_PEAKS.json sm_max_mhz), else 2070 MHz."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            mhz = float(json.load(fh)["sm_max_mhz"])
        kind = "nominal lanes x measured max SM clock"
    except (OSError, KeyError, ValueError):
        mhz, kind = 2070.0, "nominal"
    return 152 * 128 * 2 * mhz * 1e6 / 1e12, kind


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# clocks sampler
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, interval_ms=50):
        self.gpu = gpu_index
        self.interval_ms = interval_ms
        self.proc = None
        self.lines = []
        self.window = None

    def start(self, wait_s=5.0):
        """Start sampling and wait (up to wait_s) for the first sample."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", str(self.interval_ms)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
            return
        t0 = time.monotonic()
        while not self.lines and time.monotonic() - t0 < wait_s and self.proc.poll() is None:
            time.sleep(0.01)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.monotonic(), line.strip()))

    def mark(self, begin, end):
        """The timed region (time.monotonic() values): samples inside it are
        the ones reported (the nearest one when the region is shorter than
        the sampling interval)."""
        self.window = (begin, end)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        lines = self.lines
        if self.window is not None and lines:
            b, e = self.window
            inside = [x for x in lines if b <= x[0] <= e]
            if not inside:
                inside = [min(lines, key=lambda x: abs(x[0] - 0.5 * (b + e)))]
            lines = inside
        for _, ln in lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        out = {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
               "reasons": sorted(reasons), "samples": len(sm),
               "interval_ms": self.interval_ms}
        if self.window is not None:
            out["timed_s"] = round(self.window[1] - self.window[0], 3)
        return out


# ---------------------------------------------------------------------------
# CPU baseline: the reference's own Cython path (or the oracle port)
# ---------------------------------------------------------------------------
SAMPLE_N = 32768


def _reference_api():
    sys.path.insert(0, os.path.join(ROOT, "oracle", "_ref", "src"))
    import types
    import pysph.base.api as rbase  # noqa: F401
    import pysph.sph.api as rsph
    import pysph.solver.api as rsolver
    return types.SimpleNamespace(base=rbase, sph=rsph, solver=rsolver)


def reference_available():
    try:
        import sysconfig
        ext = sysconfig.get_config_var("EXT_SUFFIX")
        return os.path.exists(os.path.join(ROOT, "oracle", "_ref", "src", "pysph", "sph",
                                           "sph_calc" + ext))
    except Exception:
        return False


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the ISA)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def _pin(core):
    """Pin this process to one core (returns the previous set, or None)."""
    if not hasattr(os, "sched_setaffinity"):
        return None
    try:
        prev = os.sched_getaffinity(0)
        os.sched_setaffinity(0, {core % (os.cpu_count() or 1)})
        return prev
    except OSError:
        return None


def _cpu_worker(args):
    """Time ``steps`` RK2 steps of the sample after ``warmup`` (one process,
    pinned to its own core)."""
    kind, n, warmup, steps, seed, core = args
    import numpy as np
    # the reference's Cython is single-threaded; the oracle port uses OpenMP
    prev = _pin(core) if kind == "reference" else None

    from pysph_gb300 import workloads as W
    props = W.cube_lattice(n, seed=seed)
    import oracle
    off, _ = oracle.neighbors(props, props, 2.0 * props["h"].max(), same=True)
    kbar = float(np.diff(off).mean())
    if kind == "reference":
        import io
        import contextlib
        api = _reference_api()
        with contextlib.redirect_stdout(io.StringIO()):
            s, particles = W.setup_cube(api, props)
        step = lambda: s.integrator.integrate(DT)  # noqa: E731
    else:
        prob = oracle.Problem({"fluid": props}, oracle.cube_ops(), dim=3)
        step = lambda: prob.integrate_rk2(DT)  # noqa: E731
    for _ in range(warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    dt = time.perf_counter() - t0
    if prev is not None:
        os.sched_setaffinity(0, prev)
    return {"pairs": 4.0 * kbar * n * steps, "seconds": dt, "kbar": kbar}


def cpu_baseline(procs, warmup, steps, n=SAMPLE_N):
    kind = "reference" if reference_available() else "port"
    import multiprocessing as mp
    jobs = [(kind, n, warmup, steps, 100 + i, i) for i in range(procs)]
    if procs == 1:
        res = [_cpu_worker(jobs[0])]
    else:
        ctx = mp.get_context("spawn")
        with ctx.Pool(procs) as pool:
            t0 = time.perf_counter()
            res = pool.map(_cpu_worker, jobs)
            wall = time.perf_counter() - t0
    total_pairs = sum(r["pairs"] for r in res)
    if procs == 1:
        value = total_pairs / res[0]["seconds"]
    else:
        # aggregate over concurrently running processes: slowest one bounds it
        value = total_pairs / max(r["seconds"] for r in res)
    cores = procs
    if kind == "port":
        import oracle
        cores = procs * oracle.num_threads()
    return {
        "value": value, "unit": UNIT, "cores": cores, "kind": kind, "cpu": cpu_model(),
        "ms_per_step": max(r["seconds"] for r in res) / steps * 1e3,
        "particles_per_process": n,
        "pinning": "process i on core i" if kind == "reference" else "none (OpenMP)",
        "sample": "%d independent %s processes, each %d RK2 steps of a %d-particle "
                  "jittered lattice (h=1.2dx, same physics), after %d warm-up steps; "
                  "mean neighbours %.1f" % (procs, "reference PySPH Cython" if kind == "reference"
                                            else "oracle C port", steps, n, warmup,
                                            statistics.mean(r["kbar"] for r in res)),
    }


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value, pg):
    """The largest of one float per rank (all ranks get it): whole-job time
    is the slowest replica's.  ``pg`` is torch.distributed or None (one
    process); the reduction runs on the device of the process group's
    backend (CUDA for NCCL, the host for gloo)."""
    if pg is None:
        return float(value)
    import torch
    dev = "cuda" if pg.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], device=dev, dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def replicas_value(units_per_rank, world, seconds):
    """Whole-job throughput of independent replicas (weak scaling): the units
    all ranks processed over the slowest rank's time."""
    return world * units_per_rank / seconds


def _timed_window(integ, cm, steps, flush, stages=False):
    """Time ``steps`` integrator steps with CUDA events on the current
    stream, L2 flushed (outside the events) before each.  Returns the step
    times (ms), the per-stage times (ms lists, with ``stages``: CUDA events
    around every stage, which runs the steps call by call instead of as
    recorded step graphs), the full builds / light refreshes in the window
    and the library launches."""
    import torch
    from pysph_gb300 import native
    torch.cuda.synchronize()
    launches0 = native.launch_count()
    builds0 = cm.build_stats()
    integ.stage_events = [] if stages else None
    step_ms = []
    for _ in range(steps):
        flush.fill_(1.0)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        integ.integrate(DT)
        b.record()
        b.synchronize()
        step_ms.append(a.elapsed_time(b))
    torch.cuda.synchronize()
    launches = native.launch_count() - launches0
    events = integ.stage_events or []
    integ.stage_events = None
    stage_ms = {}
    for name, a, b in events:
        stage_ms.setdefault(name, []).append(a.elapsed_time(b))
    builds = cm.build_stats()
    return step_ms, stage_ms, (builds[0] - builds0[0], builds[1] - builds0[1]), launches


def _full_rebuild_leg(api, props, steps, warmup, flush, pairs_per_step):
    """The same step with no neighbour-list skin: every update is a full
    neighbour build (box, counting sort, reorder, the density pass that
    writes the lists), as the reference rebuilds at every
    ``particles.update()`` (base/nnps.pyx:581-620)."""
    from pysph_gb300 import workloads as W
    prev = os.environ.get("PYSPH_GB300_SKIN")
    os.environ["PYSPH_GB300_SKIN"] = "0"
    try:
        s, particles = W.setup_cube(api, props)
    finally:
        if prev is None:
            os.environ.pop("PYSPH_GB300_SKIN", None)
        else:
            os.environ["PYSPH_GB300_SKIN"] = prev
    integ = s.integrator
    for _ in range(warmup):
        integ.integrate(DT)
    step_ms, stage_ms, builds, launches = _timed_window(integ, particles.cell_manager, steps, flush)
    _, stage_ms, _, _ = _timed_window(integ, particles.cell_manager, min(steps, 5), flush,
                                      stages=True)
    ms = statistics.mean(step_ms)
    return {"value": pairs_per_step / (ms / 1e3), "unit": UNIT, "steps": steps,
            "ms_per_step": ms, "stage_ms": {k: statistics.mean(v) for k, v in stage_ms.items()},
            "timed_full": builds[0], "timed_light": builds[1], "gpu_launches": launches,
            "skin": 0.0}


def run_gpu(args):
    import torch

    import pysph_gb300
    from pysph_gb300 import native
    from pysph_gb300 import workloads as W

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl")
        pg = dist

    api = pysph_gb300.api()
    props = W.cube_lattice(args.n, seed=rank)
    n = len(props["x"])
    s, particles = W.setup_cube(api, props)
    integ = s.integrator
    for _ in range(args.warmup):
        integ.integrate(DT)
    torch.cuda.synchronize()

    cm = particles.cell_manager
    import ctypes
    kb = ctypes.c_double()
    native.check(native.lib().sph_mean_neighbours(cm.context(), 0, 0, ctypes.byref(kb)))
    kbar = kb.value
    pairs_per_step = 4.0 * kbar * n

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    clocks = ClockSampler(local, interval_ms=20)
    clocks.start()
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    deferred0 = cm.deferred_stats()
    t_begin = time.monotonic()
    step_ms, _, builds, launches = _timed_window(integ, cm, args.steps, flush)
    if pg:
        pg.barrier()
    t_end = time.monotonic()
    replay_stats = integ.step_stats()
    # the per-stage breakdown: 50 steps call by call with events around
    # every stage (outside the headline window)
    eager_ms, stage_ms, _, _ = _timed_window(integ, cm, min(args.steps, 50), flush, stages=True)
    deferred = cm.deferred_stats()
    deferred = (deferred[0] - deferred0[0], deferred[1] - deferred0[1])
    t_total = max_over_ranks(sum(step_ms) / 1e3, pg)
    life = cm.build_stats()          # every update of this context so far
    # the reference-equivalent step: a full neighbour build at every update
    full_leg = None
    if not args.no_full_rebuild_leg:
        t_fb = time.monotonic()
        full_leg = _full_rebuild_leg(api, props, min(args.steps, 20), 3, flush, pairs_per_step)
        full_leg["clock_window_s"] = round(time.monotonic() - t_fb, 3)
    clocks.mark(t_begin, t_end)
    clk = clocks.stop()

    # e2e through the public API with host buffers: every step uploads the
    # state from page-locked memory and reads its results back.  Staged: the
    # upload of step k+1 and the read-back of step k cross the link on copy
    # streams while step k / k+1 computes.  Serial: set -> integrate -> get.
    fields_in = ("x", "y", "z", "u", "v", "w")
    fields_out = ("x", "y", "z", "u", "v", "w", "rho", "p")
    pa = particles.arrays[0]
    host = {f: torch.from_numpy(pa.get(f)).pin_memory() for f in fields_in}
    e2e_steps = max(1, args.steps)

    def staged_loop(nsteps):
        up = pa.upload(**host)
        pending = None
        for k in range(nsteps):
            pa.set_staged(up)
            if k + 1 < nsteps:
                up = pa.upload(**host)
            integ.integrate(DT)
            dl = pa.download(*fields_out)
            if pending is not None:
                pending.result()
            pending = dl
        return pending.result()

    staged_loop(args.warmup)    # untimed: first use of the copy streams and buffers
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    out = staged_loop(e2e_steps)
    torch.cuda.synchronize()
    e2e_t = max_over_ranks(time.perf_counter() - t0, pg)
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        pa.set(**host)
        integ.integrate(DT)
        out = pa.get(*fields_out)
    torch.cuda.synchronize()
    e2e_serial_t = max_over_ranks(time.perf_counter() - t0, pg)
    del out

    steps = args.steps
    value = replicas_value(pairs_per_step * steps, world, t_total)
    e2e_value = replicas_value(pairs_per_step * e2e_steps, world, e2e_t)
    e2e_serial = replicas_value(pairs_per_step * e2e_steps, world, e2e_serial_t)
    peak, peak_kind = measured_peaks()
    # dominant kernel by device time
    dom = max(ALG_BYTES, key=lambda k: sum(stage_ms.get(k, [0.0])))
    launches_dom = len(stage_ms.get(dom, []))
    # the kernel's launch duration: the median over the sampled evaluations
    # (the occasional full neighbour build falls inside a stage's events)
    avg_ms = statistics.median(stage_ms[dom]) if launches_dom else float("nan")
    achieved = ALG_BYTES[dom] * n / (avg_ms / 1e3) / 1e9
    flops = PAIR_FLOPS[dom] * kbar * n / (avg_ms / 1e3) / 1e12
    fp32_peak, fp32_src = fp32_peak_tflops()
    step_s = t_total / steps
    # whole-step rooflines: B_alg = 694 B and F_alg = 2 K (24 + 72) FLOP per
    # particle per RK2 step (compulsory bytes; density + momentum pair FLOPs)
    f_alg = 2.0 * kbar * (PAIR_FLOPS["DensityStage"] + PAIR_FLOPS["RatesStage"])
    hbm_frac = STEP_ALG_BYTES * n / step_s / 1e9 / peak
    fp32_frac = f_alg * n / step_s / 1e12 / fp32_peak
    rebuild_frac = life[0] / max(1, life[0] + life[1])
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair sums, f64 integration",
        "data": "synthetic (seeded jittered lattice)",
        "config": {"workload": "3D jittered lattice, %d particles (%d^3), h=1.2dx, RK2, "
                               "NNPS+SPHRho+Tait+PGrad+MonaghanAV" % (n, round(n ** (1 / 3))),
                   "particles_per_gpu": n, "mean_neighbours": kbar,
                   "pair_passes_per_step": 4, "dt": DT,
                   "cache": "L2 flushed between timed steps (256 MiB write outside the events)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "steps_per_s": 1.0 / step_s,
        # the reference counts each SPHFunction's pair loop separately:
        # SPHRho, PGrad and AV over every neighbour, twice per RK2 step
        "reference_equivalent": {"value": value * 6.0 / 4.0, "unit": UNIT,
                                 "per_step": "6 K N (SPHRho, PGrad, AV x 2 evaluations)"},
        "stage_ms": {k: statistics.mean(v) for k, v in stage_ms.items()},
        "stage_ms_median": {k: statistics.median(v) for k, v in stage_ms.items()},
        "step_graphs": replay_stats,
        "eager_ms_per_step": statistics.mean(eager_ms),
        "nnps_builds": {"timed_full": builds[0], "timed_light": builds[1],
                        "deferred": deferred[0], "deferred_stale": deferred[1],
                        "skin": "list skin %.3g of the search radius" % cm.list_skin()},
        "gpu_launches": launches,
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": 8 * n * len(fields_in),
                "d2h_bytes_per_step": 8 * n * len(fields_out),
                "ms_per_step": e2e_t / e2e_steps * 1e3,
                "transfers": "staged: ParticleArray.upload / set_staged / download, the "
                             "link overlapped with the neighbouring steps",
                "serial": {"value": e2e_serial,
                           "ms_per_step": e2e_serial_t / e2e_steps * 1e3,
                           "transfers": "ParticleArray.set -> integrate -> get"}},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak,
                     "traffic": (NCU_TRAFFIC_PER_PARTICLE[dom] * n
                                 if dom in NCU_TRAFFIC_PER_PARTICLE else None),
                     "traffic_source": "ncu capture at 1M particles, scaled by n",
                     "peak_kind": peak_kind,
                     "alg_bytes_per_particle": ALG_BYTES[dom],
                     "note": "brick-staged pair kernels bound by issue (density) and the "
                             "L1 / shared-memory pipe (rates: staged-record reads), not HBM; "
                             "fp32 context in fp32_context",
                     "limiter": dict(NCU_LIMITER.get(dom, {}),
                                     source="ncu --set full capture at 1M particles")},
        "fp32_context": {"kernel": dom, "achieved_tflops": flops,
                         "nominal_peak_tflops": FP32_NOMINAL_TFLOPS,
                         "frac_of_nominal": flops / FP32_NOMINAL_TFLOPS},
        "step_roofline": {"alg_bytes_per_particle_step": STEP_ALG_BYTES,
                          "alg_flops_per_particle_step": f_alg,
                          "achieved_gbs": STEP_ALG_BYTES * n / step_s / 1e9,
                          "achieved_tflops": f_alg * n / step_s / 1e12,
                          "frac": hbm_frac,
                          "hbm": hbm_frac, "fp32": fp32_frac,
                          "achieved": max(hbm_frac, fp32_frac),
                          "hbm_peak_gbs": peak, "hbm_peak_kind": peak_kind,
                          "fp32_peak_tflops": fp32_peak, "fp32_peak_kind": fp32_src},
        "clocks": clk,
    }
    line["roofline"]["fp32"] = {"achieved_tflops": flops, "peak_tflops": fp32_peak,
                                "frac": flops / fp32_peak, "peak_kind": fp32_src,
                                "flops_per_pair": PAIR_FLOPS[dom]}
    line["nnps_builds"]["rebuild_fraction_all_updates"] = rebuild_frac
    line["nnps_builds"]["updates_all"] = life[0] + life[1]
    if full_leg is not None:
        line["full_rebuild"] = full_leg
        # amortised step at the rebuild rate this context has seen so far
        ms_skin = step_s * 1e3
        line["nnps_builds"]["amortised_ms_per_step"] = (
            ms_skin + rebuild_frac * (full_leg["ms_per_step"] - ms_skin))
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(1, 1, args.cpu_steps)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()


# ---------------------------------------------------------------------------
# batched elliptical drops (many independent simulations per launch)
# ---------------------------------------------------------------------------
DROPS_DT = 1e-5
DROPS_METRIC = "instance steps/s (batched 2D elliptical drops, Euler, SPHRho+Tait+PGrad+AV+XSPH)"
DROPS_UNIT = "instance-steps/s"


def _drops(args):
    from pysph_gb300 import workloads as W
    return W.drop_batch(args.drops, seed=0, c0=args.drop_c0)


def _drop_sample(drops, count, spread=0.25):
    """Indices of ``count`` instances spread over the smallest ``spread``
    fraction of the size range (bounded CPU work)."""
    import numpy as np
    sizes = np.array([len(d["x"]) for d in drops])
    order = np.argsort(sizes)
    pick = order[np.linspace(0, int((len(order) - 1) * spread), count).astype(int)]
    return [int(i) for i in pick]


def _drop_ref_worker(args):
    """Reference Cython drop run: (props, steps) -> (seconds, final arrays)."""
    props, steps, c0 = args
    import io
    import contextlib
    from pysph_gb300 import workloads as W
    if reference_available():
        api = _reference_api()
        with contextlib.redirect_stdout(io.StringIO()):
            s, particles = W.setup_drop(api, props, c0=c0)
        step = lambda: s.integrator.integrate(DROPS_DT)  # noqa: E731
        fetch = lambda: {k: particles.arrays[0].get(k).copy()  # noqa: E731
                         for k in ("x", "y", "u", "v", "rho", "p")}
        kind = "reference"
    else:
        import oracle
        prob = oracle.Problem({"fluid": props}, oracle.drop_ops(c0=c0), dim=2)
        step = lambda: prob.integrate_euler(DROPS_DT)  # noqa: E731
        fetch = lambda: {k: prob.arrays["fluid"][k].copy()  # noqa: E731
                         for k in ("x", "y", "u", "v", "rho", "p")}
        kind = "port"
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    return kind, time.perf_counter() - t0, fetch()


def drops_cpu_baseline(drops, sample, steps, c0, procs=1):
    import multiprocessing as mp
    jobs = [(drops[i], steps, c0) for i in sample]
    if procs == 1:
        res = [_drop_ref_worker(j) for j in jobs]
        seconds = sum(r[1] for r in res)
    else:
        with mp.get_context("spawn").Pool(procs) as pool:
            res = pool.map(_drop_ref_worker, jobs)
        seconds = max(r[1] for r in res)
    kind = res[0][0]
    npart = sum(len(drops[i]["x"]) for i in sample)
    mean_batch = sum(len(d["x"]) for d in drops) / len(drops)
    return {"value": len(sample) * steps / seconds, "unit": DROPS_UNIT, "cores": procs,
            "particle_steps_per_s": npart * steps / seconds,
            "size_normalised_value": npart * steps / seconds / mean_batch,
            "kind": kind,
            "sample": "%d drops of %s particles, %d Euler steps each (%s)" % (
                len(sample), "/".join(str(len(drops[i]["x"])) for i in sample), steps,
                "reference PySPH Cython" if kind == "reference" else "oracle C port"),
            "particles": sum(len(drops[i]["x"]) for i in sample)}, [r[2] for r in res]


def run_gpu_drops(args):
    import numpy as np
    import torch

    from pysph_gb300 import native, tuning
    from pysph_gb300.batch import SimulationBatch

    torch.cuda.set_device(0)
    drops = _drops(args)
    n = sum(len(d["x"]) for d in drops)
    recipe = dict(dim=2, dt=DROPS_DT, co=args.drop_c0)
    best, tune = tuning.autotune_batch(drops, candidates=(1, 2, 3), steps=5, **recipe)
    batch = SimulationBatch(drops, subdiv=best, **recipe)
    stats0 = batch.stats()
    st = batch.stream()
    batch.step(args.warmup)
    pairs = batch.pair_counts()
    pairs_per_step = 2.0 * float(pairs.sum())       # density + rates pass, Euler
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    clocks = ClockSampler(0)
    clocks.start()
    torch.cuda.synchronize()
    launches0 = native.launch_count()
    step_ms = []
    t_begin = time.monotonic()
    for _ in range(args.steps):
        with torch.cuda.stream(st):
            flush.fill_(1.0)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(st)
        batch.step(1, check=False)
        b.record(st)
        b.synchronize()
        step_ms.append(a.elapsed_time(b))
    batch.check()
    torch.cuda.synchronize()
    launches = native.launch_count() - launches0
    clocks.mark(t_begin, time.monotonic())
    clk = clocks.stop()
    t_total = sum(step_ms) / 1e3
    steps = args.steps

    # e2e: host state in, one graph step, host state out -- staged (the
    # upload of step k+1 and the read-back of step k on copy streams beside
    # the steps), and serial (set -> step -> get_all) for comparison
    fin = ("x", "y", "u", "v")
    fout = ("x", "y", "u", "v", "rho", "p")
    host = {f: torch.from_numpy(batch.get_all(f)).pin_memory() for f in fin}

    def staged_loop(nsteps):
        up = batch.upload(**host)
        pending = None
        for k in range(nsteps):
            batch.set_staged(up)
            if k + 1 < nsteps:
                up = batch.upload(**host)
            batch.step(1, check=False)
            dl = batch.download(*fout)
            if pending is not None:
                pending.result()
            pending = dl
        return pending.result()

    staged_loop(max(1, args.warmup))     # untimed: first use of the copy streams
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = staged_loop(steps)
    torch.cuda.synchronize()
    e2e_t = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(steps):
        batch.set(**host)
        batch.step(1, check=False)
        out = batch.get_all(*fout)
    e2e_serial_t = time.perf_counter() - t0
    batch.check()
    del out

    line = {
        "metric": DROPS_METRIC, "value": len(drops) * steps / t_total, "unit": DROPS_UNIT,
        "n_gpus": 1, "steps": steps, "warmup": args.warmup,
        "ms_per_step": t_total / steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 pair sums, f64 integration",
        "data": "synthetic (seeded drop radii and spacings)",
        "config": {"workload": "%d independent 2D elliptical drops, radius U[0.5,1.5], "
                               "dx U[0.01,0.04], %d particles in total, c0=%g, Euler dt=%g"
                               % (len(drops), n, args.drop_c0, DROPS_DT),
                   "instances": len(drops), "particles": n,
                   "min_particles": min(len(d["x"]) for d in drops),
                   "max_particles": max(len(d["x"]) for d in drops),
                   "subdivision": {str(k): int(sum(1 for v in best if v == k)) for k in (1, 2, 3)},
                   "autotune": tune,
                   "regions": {"margin": 0.25, "cells_at_setup": stats0["cells"],
                               "cells_now": batch.stats()["cells"],
                               "regrids": batch.stats()["regrids"],
                               "pair_launch_groups": stats0["groups"]},
                   "cache": "L2 flushed between timed steps (256 MiB write outside the events)",
                   "launch": "one CUDA graph per step"},
        "pair_interactions_per_s": pairs_per_step * steps / t_total,
        "particle_steps_per_s": n * steps / t_total,
        "gpu_launches": launches,
        "e2e": {"value": len(drops) * steps / e2e_t, "unit": DROPS_UNIT,
                "h2d_bytes_per_step": 8 * n * len(fin), "d2h_bytes_per_step": 8 * n * len(fout),
                "ms_per_step": e2e_t / steps * 1e3,
                "transfers": "staged: SimulationBatch.upload / set_staged / download",
                "serial": {"value": len(drops) * steps / e2e_serial_t,
                           "ms_per_step": e2e_serial_t / steps * 1e3,
                           "transfers": "SimulationBatch.set -> step -> get_all"}},
        "clocks": clk,
    }
    if args.drop_error_steps > 0:
        line["instance_error_vs_f64"] = drops_long_error(drops, best, recipe, args)
    if not args.no_cpu_baseline:
        sample = _drop_sample(drops, args.drop_sample)
        cb, ref_states = drops_cpu_baseline(drops, sample, args.cpu_steps, args.drop_c0)
        # the same instances on the GPU from the initial state, for the error
        fresh = SimulationBatch(drops, subdiv=best, **recipe)
        fresh.step(args.cpu_steps)
        errs = []
        for i, ref in zip(sample, ref_states):
            e = {}
            for p in ("x", "y", "u", "v"):
                d0 = drops[i][p]
                got = fresh.get(i, p) - d0
                want = ref[p] - d0
                e[p] = float(np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300))
            for p in ("rho", "p"):
                got, want = fresh.get(i, p), ref[p]
                e[p] = float(np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300))
            errs.append({"instance": i, "particles": len(drops[i]["x"]), "max_rel": max(e.values())})
        line["cpu_baseline"] = cb
        line["instance_error_vs_reference"] = {"steps": args.cpu_steps,
                                               "norm": "||gpu-ref||/||ref|| (displacements for "
                                                       "x,y,u,v)", "instances": errs}
    print(json.dumps(line), flush=True)


def normwise(a, ref):
    """max |a - ref| / max |ref| (the per-field parity metric)."""
    import numpy as np
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = np.abs(ref).max()
    return float(np.abs(a - ref).max() / scale) if scale > 0 else float(np.abs(a).max())


def drops_long_error(drops, subdiv, recipe, args):
    """Per-instance error after ``args.drop_error_steps`` batch steps against
    FP64 runs of each drop alone (the oracle's C restatement, OpenMP), for a
    sample stratified over the size range (smallest, largest, evenly
    between)."""
    import numpy as np

    import oracle
    from pysph_gb300.batch import SimulationBatch
    sizes = np.array([len(d["x"]) for d in drops])
    order = np.argsort(sizes)
    pick = [int(order[i]) for i in np.linspace(0, len(order) - 1, args.drop_error_sample).astype(int)]
    fresh = SimulationBatch(drops, subdiv=subdiv, **recipe)
    fresh.step(args.drop_error_steps)
    fresh.check()
    out = []
    for i in pick:
        d = drops[i]
        prob = oracle.Problem({"fluid": d}, oracle.drop_ops(c0=args.drop_c0), dim=2)
        for _ in range(args.drop_error_steps):
            prob.integrate_euler(DROPS_DT)
        ref = prob.arrays["fluid"]
        e = {p: normwise(fresh.get(i, p) - d[p], ref[p] - d[p]) for p in ("x", "y")}
        e.update({p: normwise(fresh.get(i, p), ref[p]) for p in ("u", "v", "rho", "p")})
        out.append({"instance": i, "particles": len(d["x"]), "errors": e,
                    "max": max(e.values())})
    return {"steps": args.drop_error_steps, "reference": "oracle C restatement, FP64",
            "norm": "max|gpu-ref|/max|ref| per field (x, y as displacements)",
            "sample": "stratified over the size range, %d of %d instances"
                      % (len(pick), len(drops)),
            "instances": out}


def run_reference_drops(args):
    world, rank, local = dist_setup()
    if rank != 0:
        return
    drops = _drops(args)
    procs = args.procs or os.cpu_count() or 1
    sample = _drop_sample(drops, procs, spread=1.0)
    cb, _ = drops_cpu_baseline(drops, sample, args.steps, args.drop_c0, procs=procs)
    # the sample's drops are smaller or larger than the batch's mean: report
    # particle-steps/s divided by the batch's mean drop size
    cb["value"] = cb["size_normalised_value"]
    line = {"metric": DROPS_METRIC, "value": cb["value"], "unit": DROPS_UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "impl": "reference", "data": "synthetic (seeded drop radii and spacings)",
            "config": {"workload": "bounded sample of the %d-drop batch (one drop per process)"
                                   % len(drops)},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": DROPS_UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# learned momentum closure on the 80,000-particle dam break
# ---------------------------------------------------------------------------
CLOSURE_METRIC = "steps/s (2D dam break dx=0.005, RK2, learned closure vs plain)"


def run_gpu_closure(args):
    import numpy as np
    import torch

    import pysph_gb300
    from pysph_gb300 import learned as L
    from pysph_gb300 import native
    from pysph_gb300 import workloads as W

    torch.cuda.set_device(0)
    api = pysph_gb300.api()
    log = (lambda m: print(m, file=sys.stderr, flush=True))
    rng = np.random.default_rng(0)
    aspects = sorted(rng.uniform(0.3, 1.0, 5).tolist())
    t0 = time.perf_counter()
    raw, targ, c0 = L.dam_break_samples(api, aspects, dx=0.01, dt=args.train_dt,
                                        steps=args.train_steps, every=args.every,
                                        capacity=args.samples, log=log)
    x, t, norm = L.standardise(raw, targ, c0)
    del raw, targ
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    model = L.MomentumMLP(seed=0)
    t0 = time.perf_counter()
    losses = L.train(model, x, t, epochs=args.epochs, batch=8192, lr=2e-3, log=log)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    # training throughput of the tensor-core kernels: forward + backward
    nb = x.shape[0] // 8192
    flops = 6.0 * (192 * 128 + 128 * 128 + 128 * 2) * nb * 8192 * args.epochs
    del x, t

    nsteps = args.closure_steps
    ckpt = max(1, nsteps // 10)

    def errs_of(a, r):
        d = (a - r).abs()
        return float((d.max() / r.abs().max()).item()), float((d / r.abs()).max().item())

    def deploy(dx, dt, column):
        """Plain, surrogate-only and guarded runs of one dam break."""
        def fresh():
            fluid, wall = W.dam_break(dx=dx, column=column)
            return W.setup_dam_break(api, fluid, wall, dx, c0)

        def plain_run():
            s, particles = fresh()
            fl = particles.arrays[0]
            for _ in range(3):
                s.integrator.integrate(dt)
            torch.cuda.synchronize()
            refs = []
            t1 = time.perf_counter()
            for k in range(1, nsteps + 1):
                s.integrator.integrate(dt)
                if k % ckpt == 0:
                    refs.append(fl.get_device("rho").clone())
            torch.cuda.synchronize()
            return time.perf_counter() - t1, refs, fl.get_number_of_particles()

        # The comparison runs rebuild the neighbour lists at every update
        # (no list skin): the FP32 summation order then depends on the state
        # alone, so a guarded window that falls back reproduces the plain
        # run bit for bit.  With a skin the order follows the rebuild
        # history; the difference of the two plain runs is the noise floor
        # of each metric in this free-surface flow.
        skin_env = os.environ.get("PYSPH_GB300_SKIN")
        os.environ["PYSPH_GB300_SKIN"] = "0.03"
        _, refs_skin, _ = plain_run()
        os.environ["PYSPH_GB300_SKIN"] = "0"
        t_plain, refs, n = plain_run()
        log("dx %g plain: %.3f s for %d steps" % (dx, t_plain, nsteps))
        floor = [errs_of(a, r) for a, r in zip(refs_skin, refs)]

        def surrogate_run(k=None):
            s, particles = fresh()
            fl = particles.arrays[0]
            for _ in range(3):
                s.integrator.integrate(dt)
            closure = L.LearnedClosure(s.integrator, fl, model, norm)
            errs = []
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            runner = None
            try:
                if k is None:
                    for j in range(1, nsteps + 1):
                        s.integrator.integrate(dt)
                        if j % ckpt == 0:
                            errs.append(errs_of(fl.get_device("rho"), refs[j // ckpt - 1]))
                else:
                    runner = L.GuardedRunner(s, particles, closure, k=k, tol=args.tol)
                    done = 0
                    while done < nsteps:
                        runner.window(dt)
                        done += k
                        if done % ckpt == 0:
                            errs.append(errs_of(fl.get_device("rho"), refs[done // ckpt - 1]))
                torch.cuda.synchronize()
                el = time.perf_counter() - t1
                out = {"steps_per_s": nsteps / el, "vs_plain": (nsteps / el) / (nsteps / t_plain),
                       "max_normwise_density_error": max(e[0] for e in errs) if errs else None,
                       "max_relative_density_error": max(e[1] for e in errs) if errs else None,
                       "normwise_at_checkpoints": [e[0] for e in errs],
                       "max_relative_at_checkpoints": [e[1] for e in errs]}
            except RuntimeError as e:
                out = {"failed": str(e)[:120]}
            if runner is not None:
                out["guard"] = runner.stats()
            closure.detach()
            return out

        res = {"surrogate_only": surrogate_run(None)}
        # (no k = 1: with summation density the density at the end of one
        # RK2 step is that of its midpoint positions x + dt/2 v, which the
        # step's accelerations do not reach, so a one-step window's check
        # sees no difference)
        for k in (2, 5, 10, 20):
            res["guarded_k%d" % k] = surrogate_run(k)
            log("dx %g k=%d: %s" % (dx, k, {q: v for q, v in res["guarded_k%d" % k].items()
                                            if not q.endswith("checkpoints")}))
        if skin_env is None:
            os.environ.pop("PYSPH_GB300_SKIN", None)
        else:
            os.environ["PYSPH_GB300_SKIN"] = skin_env
        return {"dx": dx, "dt": dt, "column": list(column), "fluid_particles": n,
                "plain_steps_per_s": nsteps / t_plain,
                "plain_noise_floor": {
                    "what": "density difference between the plain run with and without a "
                            "neighbour-list skin (two exact summation orders)",
                    "normwise_at_checkpoints": [f[0] for f in floor],
                    "max_relative_at_checkpoints": [f[1] for f in floor]},
                "closure": res}

    def term_timings(dx, dt, column, reps=50):
        """CUDA-event times of what one rates evaluation of the closure
        runs against the pair loop it replaces (the fluid-on-itself PGrad +
        AV pass), at the state after three plain steps."""
        import ctypes

        from pysph_gb300.sph import gpu
        fluid, wall = W.dam_break(dx=dx, column=column)
        s, particles = W.setup_dam_break(api, fluid, wall, dx, c0)
        for _ in range(3):
            s.integrator.integrate(dt)
        fl = particles.arrays[0]
        cm = particles.cell_manager
        term = dict(L._self_term(L._fluid_stage(s.integrator, fl)))
        term["kinds"] = set(L.SELF_KINDS)
        n = fl.get_number_of_particles()
        dev = fl.get_device("x").device
        acc = tuple(torch.zeros(n, dtype=torch.float64, device=dev) for _ in range(3))
        st = torch.cuda.current_stream()

        def timed(fn):
            """(device ms, wall ms) per call: the device time with the
            calls queued behind a spin kernel (so the host has enqueued them
            all before the first runs), the wall time of calls made one
            after another from Python."""
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            for _ in range(reps):
                fn()
            torch.cuda.synchronize()
            wall = (time.perf_counter() - t1) * 1e3 / reps
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            torch.cuda._sleep(int(4e7))
            a.record(st)
            for _ in range(reps):
                fn()
            b.record(st)
            b.synchronize()
            return a.elapsed_time(b) / reps, wall

        out = {"fluid_particles": n, "what": "per call: [device ms, wall ms of calls from Python]"}
        out["pair_loop_ms"] = timed(lambda: gpu.rates(cm, fl, [term], 2, acc=acc))
        x = L.features(cm, fl, norm)
        out["features_ms"] = timed(lambda: L.features(cm, fl, norm, out=x))
        prev = os.environ.get("SPH_FEATURES_THREAD")
        os.environ["SPH_FEATURES_THREAD"] = "1"
        out["features_thread_per_destination_ms"] = timed(lambda: L.features(cm, fl, norm, out=x))
        if prev is None:
            os.environ.pop("SPH_FEATURES_THREAD", None)
        else:
            os.environ["SPH_FEATURES_THREAD"] = prev
        out["network_ms"] = timed(lambda: model.forward(x))
        y = model.forward(x)
        scale = (ctypes.c_double * 2)(*norm.targ_std)
        mean = (ctypes.c_double * 2)(*norm.targ_mean)
        ptrs = (ctypes.c_void_p * 3)(*[a.data_ptr() for a in acc])

        def apply():
            native.check(native.lib().sph_mlp_apply(cm.context(), cm.slot(fl), y.data_ptr(), c0,
                                                    scale, mean, ptrs, 1), "mlp apply")

        out["apply_ms"] = timed(apply)
        dev = out["features_ms"][0] + out["network_ms"][0] + out["apply_ms"][0]
        out["closure_device_ms"] = dev
        out["closure_device_vs_pair_loop"] = dev / out["pair_loop_ms"][0]
        return out

    # cross-resolution (trained at dx = 0.01, deployed at dx = 0.005, the
    # 80,000-particle case) and in-distribution (trained and deployed at
    # dx = 0.01; the column's aspect ratio 0.5 lies inside the training
    # range but is not one of the training runs)
    terms = term_timings(0.005, args.dt, (1.0, 2.0))
    log("per-term times at dx 0.005: %s" % terms)
    cross = deploy(0.005, args.dt, (1.0, 2.0))
    indist = deploy(0.01, args.train_dt, (1.0, 2.0))
    plain_sps = cross["plain_steps_per_s"]
    n, dx, dt = cross["fluid_particles"], cross["dx"], cross["dt"]
    line = {
        "metric": CLOSURE_METRIC, "value": plain_sps, "unit": "steps/s", "n_gpus": 1,
        "steps": nsteps, "warmup": 3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "ms_per_step": 1e3 / plain_sps, "dtype": "bf16 network (fp32 accumulate), f32 pair sums, f64 integration",
        "data": "synthetic (dam-break lattices)",
        "config": {"workload": "2D dam break, dx=%g, %d fluid particles, RK2 dt=%g; closure "
                               "trained on dx=0.01 runs at aspect ratios %s" % (
                                   dx, n, dt, ["%.3f" % a for a in aspects]),
                   "tolerance": args.tol, "tolerance_metric": "normwise max|d rho|/max|rho|",
                   "train_steps": args.train_steps, "every": args.every,
                   "lists": "rebuilt at every update (no skin) in the timed comparison runs"},
        "plain_steps_per_s": plain_sps,
        "cross_resolution": cross,
        "in_distribution": indist,
        "terms_ms": terms,
        "training": {"samples": int(nb * 8192), "epochs": args.epochs, "loss_first": losses[0],
                     "loss_last": losses[-1], "seconds": t_train, "data_seconds": t_data,
                     "tflops_fwd_bwd": flops / t_train / 1e12},
        "gpu_launches": None,
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# the closure network's tensor-core kernels on their own
# ---------------------------------------------------------------------------
MLP_FWD_FLOPS = 2.0 * (192 * 128 + 128 * 128 + 128 * 2)            # per sample
MLP_BWD_FLOPS = 2.0 * (128 * 128 + 128 * 144 + 128 * 208) + 4.0 * 128 * 2


def measured_bf16():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback"


def run_gpu_mlp(args):
    import torch

    from pysph_gb300 import learned as L
    from pysph_gb300 import native

    torch.cuda.set_device(0)
    n = args.mlp_n
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    x = torch.randn((n, 192), generator=g, device="cuda").to(torch.bfloat16)
    t = torch.randn((n, 2), generator=g, device="cuda")
    model = L.MomentumMLP(seed=0)
    st = torch.cuda.current_stream()

    def timed(fn, reps):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(reps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(st)
            fn()
            b.record(st)
            b.synchronize()
            ms.append(a.elapsed_time(b))
        return statistics.mean(ms)

    launches0 = native.launch_count()
    fwd_ms = timed(lambda: model.forward(x), args.steps)
    y, cache = model.forward(x, save=True)
    bwd_ms = timed(lambda: model.backward(x, cache, y, t), args.steps)
    train_ms = timed(lambda: _train_step(model, x, t), args.steps)
    launches = native.launch_count() - launches0
    model.check()
    peak, kind = measured_bf16()
    fwd_tf = MLP_FWD_FLOPS * n / (fwd_ms / 1e3) / 1e12
    bwd_tf = MLP_BWD_FLOPS * n / (bwd_ms / 1e3) / 1e12
    line = {
        "metric": "closure network samples/s (forward, BF16 tensor cores)",
        "value": n / (fwd_ms / 1e3), "unit": "samples/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": fwd_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (fp32 accumulate)",
        "data": "synthetic (seeded normal features)",
        "config": {"workload": "network 192-128-128-2 GELU, %d samples per launch" % n},
        "forward": {"ms": fwd_ms, "tflops": fwd_tf},
        "backward": {"ms": bwd_ms, "tflops": bwd_tf},
        "train_step_ms": train_ms,
        "roofline": {"bound": "tensor", "kernel": "k_mlp_fwd_tma", "achieved": fwd_tf, "peak": peak,
                     "unit": "TFLOP/s", "frac": fwd_tf / peak, "traffic": None,
                     "peak_kind": kind},
        "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)


def _train_step(model, x, t):
    y, cache = model.forward(x, save=True)
    model.backward(x, cache, y, t)
    model.adam(1e-4)


# ---------------------------------------------------------------------------
# single small simulations: host-bound call by call, one graph per step
# ---------------------------------------------------------------------------
SMALL_METRIC = "steps/s (single small simulations: 2D drop 5k Euler, 2D dam break 20k/80k RK2)"


def run_gpu_small(args):
    """Wall-clock and device time per step of the small single-simulation
    configurations, their steps replayed as one CUDA graph each (the default
    below 500 000 particles) and run call by call (PYSPH_GB300_GRAPHS=0).
    device_ms_per_step: CUDA events around the timed steps on the stream the
    steps run on (the device timeline, idle gaps the host leaves included);
    replay_device_ms_per_step: CUDA events around each graph launch, the
    device's own time for a replayed step -- a step is device-bound when the
    wall time per step approaches it."""
    import torch

    import pysph_gb300
    from pysph_gb300 import native
    from pysph_gb300 import workloads as W

    torch.cuda.set_device(0)
    api = pysph_gb300.api()

    def drop():
        props = W.elliptical_drop(dx=0.025, c0=100.0)
        return W.setup_drop(api, props, c0=100.0), 1e-5, len(props["x"])

    def dam(dx, dt):
        def make():
            fluid, wall = W.dam_break(dx=dx)
            return (W.setup_dam_break(api, fluid, wall, dx, W.dam_break_c0()), dt,
                    len(fluid["x"]) + len(wall["x"]))
        return make

    cases = [("2D elliptical drop dx=0.025, Euler, c0=100", drop),
             ("2D dam break dx=0.01 (20k fluid + walls), RK2 dt=2.5e-5", dam(0.01, 2.5e-5)),
             ("2D dam break dx=0.005 (80k fluid + walls), RK2 dt=1.25e-5", dam(0.005, 1.25e-5))]
    out = []
    for name, make in cases:
        row = {"case": name}
        for mode in ("graphs", "calls"):
            os.environ["PYSPH_GB300_GRAPHS"] = "1" if mode == "graphs" else "0"
            (s, particles), dt, n = make()
            integ = s.integrator
            for _ in range(args.warmup + 2):
                integ.integrate(dt)
            torch.cuda.synchronize()
            st0 = integ.step_stats() or {}
            b0 = particles.cell_manager.build_stats()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            l0 = native.launch_count()
            t0 = time.perf_counter()
            a.record()
            for _ in range(args.steps):
                integ.integrate(dt)
            b.record()
            b.synchronize()
            wall = (time.perf_counter() - t0) / args.steps * 1e3
            dev = a.elapsed_time(b) / args.steps
            st1 = integ.step_stats() or {}
            b1 = particles.cell_manager.build_stats()
            row["particles"] = n
            row[mode] = {"wall_ms_per_step": wall, "device_ms_per_step": dev,
                         "steps_per_s": 1e3 / wall,
                         "launches_per_step": (native.launch_count() - l0) / args.steps,
                         "list_skin": particles.cell_manager.list_skin(),
                         "full_builds_per_step": (b1[0] - b0[0]) / args.steps,
                         "light_refreshes_per_step": (b1[1] - b0[1]) / args.steps,
                         "step_graphs": st1 or None}
            g = st1.get("graph_steps", 0) - st0.get("graph_steps", 0)
            if g > 0:
                # device time of a replayed step: CUDA events around each
                # graph launch (no host work inside a graph)
                row[mode]["timed_graph_steps"] = g
                row[mode]["replay_device_ms_per_step"] = (
                    (st1["replay_device_us"] - st0.get("replay_device_us", 0)) / g / 1e3)
        os.environ.pop("PYSPH_GB300_GRAPHS", None)
        row["speedup_graphs"] = row["calls"]["wall_ms_per_step"] / row["graphs"]["wall_ms_per_step"]
        out.append(row)
    line = {"metric": SMALL_METRIC, "value": out[0]["graphs"]["steps_per_s"], "unit": "steps/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": out[0]["graphs"]["wall_ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair sums, f64 integration",
            "data": "synthetic (drop and dam-break lattices)",
            "config": {"workload": "single small simulations", "cases": [c for c, _ in cases]},
            "cases": out, "gpu_launches": None}
    print(json.dumps(line), flush=True)


def run_reference(args):
    world, rank, local = dist_setup()
    if rank != 0:
        return
    procs = args.procs or os.cpu_count() or 1
    cb = cpu_baseline(procs, args.warmup, args.steps)
    # the bench's own size on one pinned core: whole RK2 steps of the
    # 1,000,000-particle lattice (each rebuilds the neighbour cache)
    full = None
    if args.ref_1m_steps > 0:
        if reference_available():
            r = _cpu_worker(("reference", 1_000_000, 0, args.ref_1m_steps, 0, 0))
            full = {"value": r["pairs"] / r["seconds"], "unit": UNIT, "cores": 1,
                    "particles": 1_000_000, "steps": args.ref_1m_steps,
                    "ms_per_step": r["seconds"] / args.ref_1m_steps * 1e3,
                    "mean_neighbours": r["kbar"], "pinning": "core 0",
                    "kind": "reference"}
        else:
            full = {"unavailable": "the compiled reference is not built on this host"}
    line = {
        "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "ms_per_step": cb["ms_per_step"],
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
        "data": "synthetic (seeded jittered lattice)",
        "config": {"workload": "3D jittered lattice, h=1.2dx, RK2, NNPS+SPHRho+Tait+PGrad+"
                               "MonaghanAV; bounded sample of %d particles per process"
                               % SAMPLE_N},
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "ms_per_step_note": "wall time per RK2 step of the slowest process (its %d-particle "
                            "sample)" % SAMPLE_N,
    }
    if full is not None:
        line["single_core_1M"] = full
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # default: 300 timed GPU steps of the 1M-particle lattice or of the drops
    # batch (a third to half a second, long enough for several clock
    # samples), 20 elsewhere
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--procs", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-full-rebuild-leg", action="store_true")
    ap.add_argument("--ref-1m-steps", type=int, default=3)
    ap.add_argument("--workload", default="cube",
                    choices=["cube", "drops", "closure", "mlp", "small"])
    ap.add_argument("--mlp-n", type=int, default=1 << 20)
    ap.add_argument("--samples", type=int, default=10_000_000)
    ap.add_argument("--epochs", type=int, default=10)
    ap.add_argument("--train-steps", type=int, default=2000)
    ap.add_argument("--train-dt", type=float, default=2.5e-5)
    ap.add_argument("--every", type=int, default=20)
    ap.add_argument("--dt", type=float, default=1.25e-5)
    ap.add_argument("--tol", type=float, default=1e-3)
    ap.add_argument("--closure-steps", type=int, default=1000)
    ap.add_argument("--drops", type=int, default=256)
    ap.add_argument("--drop-c0", type=float, default=100.0)
    ap.add_argument("--drop-sample", type=int, default=8)
    # the supersonic drops (c0 = 100, |v| up to 150) blow up in FP64 within
    # ~770 steps for the largest ones: the error is compared at 500
    ap.add_argument("--drop-error-steps", type=int, default=500)
    ap.add_argument("--drop-error-sample", type=int, default=8)
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 300 if (args.workload in ("cube", "drops") and args.impl == "gb300") else 20
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.workload == "drops":
        (run_reference_drops if args.impl == "reference" else run_gpu_drops)(args)
    elif args.workload == "small":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the small cases' reference "
                              "timings are the cube and drops reference arms"}))
        else:
            run_gpu_small(args)
    elif args.workload == "mlp":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no network"}))
        else:
            run_gpu_mlp(args)
    elif args.workload == "closure":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned "
                              "closure; its plain dam break is the cube/drops reference arm"}))
        else:
            run_gpu_closure(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
