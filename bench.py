#!/usr/bin/env python3
"""Throughput benchmark of the 3D plain C-PML workload on GB300.

Workload (the reference's 3D program, run as one domain): 276^3 grid
(256^3 interior + 10-point C-PML on all faces), DELTA = 10 m, homogeneous
cp = 3300 m/s, cs = cp/1.732, rho = 2800, DELTAT = 1.6 ms, NSTEP = 2500,
Ricker f0 = 7 Hz at the centre, 64 receivers on the x line through the
centre. One bench step = one whole simulation (NSTEP time steps, from zeroed
fields to the last seismogram sample). Inputs are synthetic (parameters only;
the model is homogeneous). The working set (two 757 MB buffer sets) is far
larger than L2, so no flush is needed between steps.

metric: Mcell-updates/s (cells x time steps / s), higher is better.
  value : device time of K steps through the resident handle
          (cpml_reset + cpml_run), CUDA events on the handle's stream.
  e2e   : the C ABI as a caller uses it, per step: cpml_create (parameters and
          receiver indices host->device), cpml_run, cpml_get_seismograms and
          cpml_get_energy (device->host), cpml_destroy.
  roofline: the fused step kernel, HBM-bound; achieved = algorithmic bytes per
          launch (every field read and written once, per-cell model once,
          every C-PML memory variable read and written where its a != 0)
          / average launch duration over the timed region.
  cpu_baseline: the FP64 C++ restatement of the reference time loop with
          OpenMP on every host core, on a bounded sample of the same grid:
          as many time steps as take about 10 s (and the same on one thread).

--impl reference times the reference's own 3D program on the host cores, on
the same config and metric, each step a bounded sample of 40 time steps. No
Fortran compiler exists on either machine, so the program's statements are
translated to C (oracle/ref_f90c.py, from its Fortran source; gcc -O3 as
the reference Makefile builds it) and run on 12 MPI ranks emulated as
processes. Its time loop is timed. Where that
translated C is absent, the C++ restatement is timed instead (kind "port";
also with --reference-port).

Multi-GPU: the path has no exchange step in this build (one domain per GPU);
N ranks run N independent replicas of the workload ("replicas only").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PROFILE_TRAFFIC = os.path.join(ROOT, "profiles", "fused3d_276cube.json")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--nstep", type=int, default=None, help="time steps per bench step")
    ap.add_argument("--tuning", type=str, default=None, help="kernel,tile_y,zchunk,depth (skips autotune)")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--cpu-sample-steps", type=int, default=None,
                    help="time steps per CPU sample (default: about 10 s of work; the reference arm: 40)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--reference-port", action="store_true",
                    help="--impl reference: time the C++ restatement even where the translated "
                         "reference program exists")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", choices=["3d_plain", "3d_large", "2d_plain", "batch2d", "surrogate"],
                    default="3d_plain")
    ap.add_argument("--train-shots", type=int, default=20000)
    ap.add_argument("--test-shots", type=int, default=2000)
    ap.add_argument("--train-seconds", type=float, default=600.0)
    ap.add_argument("--epochs", type=int, default=200)
    ap.add_argument("--threshold", type=float, default=0.05)
    return ap.parse_args()


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend)
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def n_chunks(nstep, it_display):
    """Chunks of the runtime's time loop: ends at it = 5 and every display step."""
    it, n = 0, 0
    while it < nstep:
        nd = (it // it_display + 1) * it_display
        if it < 5:
            nd = min(nd, 5)
        it = min(nstep, nd, it + 128)
        n += 1
    return n


def cpu_baseline(p, nthreads, sample_steps=None, target_s=10.0, max_steps=400):
    """The FP64 C++ restatement of the time loop on `nthreads` host threads:
    `sample_steps` timed time steps, or by default as many as take about
    `target_s` seconds (estimated from two timed steps, at most `max_steps`).
    Returns (Mcell-updates/s, seconds, time steps)."""
    from oracle import oracle_c
    sess = oracle_c.Session(p, nthreads=nthreads)
    sess.run(1)  # touch every page once
    if sample_steps is None:
        t = time.perf_counter()
        sess.run(2)
        per_step = max((time.perf_counter() - t) / 2, 1e-6)
        sample_steps = int(min(max_steps, max(2, -(-target_s // per_step))))
    t = time.perf_counter()
    sess.run(sample_steps)
    dt = time.perf_counter() - t
    sess.close()
    ncell = p.nx * p.ny * p.nz
    return ncell * sample_steps / dt / 1e6, dt, sample_steps


# ---------------------------------------------------------------------------
def reference_program():
    """The reference's 3D program translated to C (oracle/_ref: its own
    statements, parameter lines set to the 3D plain workload with a
    40-step time loop), compiled for this machine; None where that C is
    absent (it is made from the reference sources, which only some machines
    have) or no C compiler exists."""
    import shutil
    from oracle import ref_f90c
    if shutil.which("gcc") is None or not ref_f90c.translated_exists(ref_f90c.BENCH_TAG):
        return None
    return ref_f90c.compile_translated(ref_f90c.BENCH_TAG)


def run_reference(args, world, rank, pg):
    from seismic_cpml_gb300 import params as P
    p, _ = P.config_3d_plain()
    if rank != 0:
        return 0
    ncell = p.nx * p.ny * p.nz
    note = None
    try:
        prog = None if args.reference_port else reference_program()
        if prog is not None:
            # each bench step runs the program once; its time loop (not the
            # process start or the zeroing of its arrays) is timed, as the
            # slowest rank saw it
            from oracle import ref_f90c
            sample, cores = ref_f90c.BENCH_SAMPLE_STEPS, ref_f90c.PLAIN_3D_RANKS

            def one():
                return max(r["loop_seconds"] for r in prog.run(nprocs=cores, timeout=1800))
            for _ in range(args.warmup):
                one()
            dt = sum(one() for _ in range(args.steps))
    except (OSError, RuntimeError, subprocess.SubprocessError) as e:
        note = f"translated reference program failed, C++ restatement timed instead: {e}"[:300]
        print(note, file=sys.stderr)
        prog = None
    if prog is not None:
        kind = "reference"
        what = (f"{sample} time steps of the 276^3 grid per bench step: the reference 3D "
                f"program's own statements (translated from its Fortran source to C, gcc -O3 as "
                f"its Makefile, FP64) on {cores} MPI ranks of 23 planes emulated as processes; "
                f"the time loop is timed")
    else:
        cores = os.cpu_count() or 1
        sample = args.cpu_sample_steps or 40
        from oracle import oracle_c
        sess = oracle_c.Session(p, nthreads=cores)
        sess.run(1)
        for _ in range(args.warmup):
            sess.run(sample)
        t = time.perf_counter()
        for _ in range(args.steps):
            sess.run(sample)
        dt = time.perf_counter() - t
        sess.close()
        kind = "port"
        what = (f"{sample} time steps of the 276^3 grid per bench step, FP64 C++ restatement "
                f"of the reference time loop, OpenMP")
    value = ncell * sample * args.steps / dt / 1e6
    line = {
        "impl": "reference",
        "metric": "Mcell-updates/s", "value": round(value, 3), "unit": "Mcell-updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "3d_plain_276cube", "grid": [p.nx, p.ny, p.nz],
                   "nstep_per_bench_step": sample, "parallelism": "replicas"},
        "cpu_baseline": {"value": round(value, 3), "unit": "Mcell-updates/s", "cores": cores,
                         "kind": kind, "sample": what},
        "e2e": {"value": round(value, 3), "unit": "Mcell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    if note:
        line["note"] = note
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, world, rank, local, pg):
    import torch
    from seismic_cpml_gb300 import params as P
    from seismic_cpml_gb300.solver import Solver
    torch.cuda.set_device(local)
    model = None
    if args.workload == "3d_large":
        # 820^3 per-cell layered model with anomalies, generated on the device
        # and handed to the C ABI as host arrays like any caller's model
        from seismic_cpml_gb300.earth import layered_model_3d_device
        p, rec = P.config_3d_large(nstep=args.nstep or 400)
        model = tuple(t.cpu().numpy() for t in layered_model_3d_device((p.nz, p.ny, p.nx)))
        torch.cuda.empty_cache()
    else:
        p, rec = P.config_3d_plain()
    if args.nstep:
        p.nstep = args.nstep
    tuning = tuple(int(x) for x in args.tuning.split(",")) if args.tuning else None
    ncell = p.nx * p.ny * p.nz

    s = Solver(p, rec, model=model, tuning=tuning)
    if s.tuning()[0] != 2 and (tuning is None or tuning[0] != 1):
        # the fused one-sweep step needs the driver's tensor-map encoder; a
        # handle without it runs the two-sweep kernels (108 instead of 72 B
        # per cell), which is not the path this line describes
        s.close()
        raise SystemExit("bench.py: the fused 3D step is unavailable on this device; "
                         "the handle fell back to the two-sweep kernels")
    tune = None
    if tuning is None and not args.no_autotune:
        tune = s.autotune(trial_steps=20)        # outside the timed region
        tuning = s.tuning()
    stream = torch.cuda.ExternalStream(s.stream_ptr())
    for _ in range(args.warmup):
        s.reset()
        s.run()
    torch.cuda.synchronize()
    barrier(pg)
    clocks = ClockSampler(local)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    barrier(pg)
    t0 = time.perf_counter()
    ev0.record(stream)
    for _ in range(args.steps):
        s.reset()
        s.run()
    ev1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    barrier(pg)
    clk = clocks.stop()
    dev_ms = ev0.elapsed_time(ev1)
    dev_ms = max_over_ranks(pg, dev_ms)
    bytes_step = s.algorithmic_bytes_per_step()
    kern = s.tuning()
    k_step, k_chunk = s.launches_per_step()
    vx, vy, vz = s.seismograms()
    s.close()

    value = world * ncell * p.nstep * args.steps / (dev_ms / 1e3) / 1e6
    launch_ms = dev_ms / (args.steps * p.nstep)
    achieved = bytes_step / (launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    traffic = None
    traffic_tuning = None
    try:
        with open(PROFILE_TRAFFIC) as f:
            prof = json.load(f)
        if prof.get("grid") == [p.nx, p.ny, p.nz] and prof.get("tuning", [None])[0] == kern[0]:
            traffic = prof.get("dram_bytes_per_launch")
            traffic_tuning = prof.get("tuning")
    except (OSError, ValueError):
        pass

    # end to end through the C ABI: host inputs in, seismograms and energy out
    e2e = None
    chunks_e2e = n_chunks(p.nstep, p.it_display)
    if not args.no_e2e:
        h2d = d2h = 0
        torch.cuda.synchronize()
        barrier(pg)
        t = time.perf_counter()
        for _ in range(args.steps):
            with Solver(p, rec, model=model, tuning=tuning) as e:
                e.run()
                sx, sy, sz = e.seismograms()
                ek, ep = e.energy()
        torch.cuda.synchronize()
        e2e_s = max_over_ranks(pg, time.perf_counter() - t)
        # host->device: source increments (2 x nstep FP32), receiver cells (int32)
        h2d = 2 * 4 * p.nstep + 4 * len(rec) + (3 * 4 * ncell if model is not None else 0)
        # device->host: samples (3 x nrec x nstep FP32), energy (2 x nstep FP64),
        # FP64 profiles read back for the slab extents (3 axes x 10 x n), and
        # the per-chunk max|v| and finiteness words
        d2h = (3 * 4 * len(rec) * p.nstep + 2 * 8 * p.nstep + 3 * 10 * 8 * p.nx +
               chunks_e2e * (8 + 4 * 100))
        e2e = {"value": round(world * ncell * p.nstep * args.steps / e2e_s / 1e6, 3),
               "unit": "Mcell-updates/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and model is None:
        cores = os.cpu_count() or 1
        v, dt, n = cpu_baseline(p, cores, args.cpu_sample_steps)
        v1, dt1, n1 = cpu_baseline(p, 1, 2 if args.cpu_sample_steps else None)
        cpu = {"value": round(v, 3), "unit": "Mcell-updates/s", "cores": cores, "kind": "port",
               "sample": f"{n} time steps of the 276^3 grid ({dt:.1f} s), FP64 C++ "
                         "restatement of the reference time loop, OpenMP",
               "value_1core": round(v1, 3), "sample_1core": f"{n1} time steps on one thread ({dt1:.1f} s)"}

    chunks = n_chunks(p.nstep, p.it_display)
    line = {
        "metric": "Mcell-updates/s", "value": round(value, 3), "unit": "Mcell-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dev_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "3d_large_820cube_het" if model is not None else "3d_plain_276cube",
                   "grid": [p.nx, p.ny, p.nz], "nstep": p.nstep, "deltat": p.deltat,
                   "receivers": len(rec), "parallelism": "replicas" if world > 1 else "single",
                   "l2": "inputs larger than L2 (%.1f GB of wavefields)" % (18 * 4 * ncell / 1e9),
                   "kernel": {"kind": ["auto", "two_sweep", "fused"][kern[0]], "tile_y": kern[1],
                              "zchunk": kern[2], "tma_lookahead": kern[3],
                              "autotuned": tune is not None}},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "traffic_source": ("ncu DRAM bytes of one step, tuning %s (profiles/fused3d_276cube.md)"
                                        % traffic_tuning) if traffic else None,
                     "peak_source": peak_kind,
                     "bytes_per_launch": bytes_step, "launch_ms": round(launch_ms, 5)},
        "cpu_baseline": cpu,
        "e2e": e2e,
        # the step kernels of every time step (interior + one per general class, or
        # stress + velocity), plus the chunk reduction and step-counter kernels
        "gpu_launches": args.steps * (k_step * p.nstep + k_chunk * chunks),
        "clocks": clk,
        "wall_s": round(wall, 3),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_2d_plain(args, world, rank, local, pg):
    """The 2D plain workload (101 x 641, 10-point C-PML on all edges but the
    top, homogeneous, 2000 steps, Ricker at the centre, 45 degrees, two
    receivers): one bench step = one whole run, on the handle's automatic
    kernel choice (for this grid, 324 tiles in one resident wave: the two
    sweep kernels replayed from CUDA graphs). Its 3.8 MB working set lives in
    L2, so the step is launch- and latency-bound: the line reports
    Mcell-updates/s and ms per run; the roofline fraction is quoted against
    HBM only for comparison."""
    import torch
    from seismic_cpml_gb300 import params as P
    from seismic_cpml_gb300.solver import Solver
    torch.cuda.set_device(local)
    p, rec = P.config_2d_plain()
    ncell = p.nx * p.ny
    s = Solver(p, rec)
    stream = torch.cuda.ExternalStream(s.stream_ptr())
    for _ in range(args.warmup):
        s.reset(); s.run()
    torch.cuda.synchronize()
    barrier(pg)
    clocks = ClockSampler(local)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        s.reset(); s.run()
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    dev_ms = max_over_ranks(pg, ev0.elapsed_time(ev1))
    bytes_step = s.algorithmic_bytes_per_step()
    kern = s.tuning()[0]
    k_step, k_chunk = s.launches_per_step()
    s.close()
    value = world * ncell * p.nstep * args.steps / (dev_ms / 1e3) / 1e6
    t = time.perf_counter()
    for _ in range(args.steps):
        with Solver(p, rec) as e:
            e.run()
            e.seismograms()
            e.energy()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(pg, time.perf_counter() - t)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle_c
        cores = os.cpu_count() or 1
        res = {}
        for nth in (cores, 1):
            sess = oracle_c.Session(p, nthreads=nth)
            sess.run(1)
            t0 = time.perf_counter()
            sess.run(p.nstep - 1)
            res[nth] = ncell * (p.nstep - 1) / (time.perf_counter() - t0) / 1e6
            sess.close()
        cpu = {"value": round(res[cores], 3), "unit": "Mcell-updates/s", "cores": cores, "kind": "port",
               "sample": "the whole 2000-step run, FP64 C++ restatement, OpenMP",
               "value_1core": round(res[1], 3)}
    step_ms = dev_ms / args.steps
    peak, peak_kind = measured_peak()
    achieved = bytes_step * p.nstep / (step_ms / 1e3) / 1e9
    line = {
        "metric": "Mcell-updates/s", "value": round(value, 3), "unit": "Mcell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "2d_plain_101x641", "grid": [p.nx, p.ny], "nstep": p.nstep, "receivers": len(rec),
                   "l2": "working set (3.8 MB) is L2-resident by design of the workload",
                   "kernel": {1: "two_sweep", 3: "persistent"}.get(kern, str(kern))},
        "latency_us_per_time_step": round(step_ms * 1e3 / p.nstep, 3),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_kind,
                     "note": "L2-resident and launch-bound; the fraction is not a kernel-quality figure"},
        "cpu_baseline": cpu,
        "e2e": {"value": round(world * ncell * p.nstep * args.steps / e2e_s / 1e6, 3), "unit": "Mcell-updates/s",
                "h2d_bytes_per_step": 2 * 4 * p.nstep + 4 * len(rec),
                "d2h_bytes_per_step": 2 * 4 * len(rec) * p.nstep + 2 * 8 * p.nstep},
        "gpu_launches": args.steps * (k_step * p.nstep + k_chunk * n_chunks(p.nstep, p.it_display)),
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_batch2d(args, world, rank, local, pg):
    """Batched 2D multi-shot FD: 256 seeded shots of 240-1240 cells per side
    (20-point C-PML), layered models, DELTAT from a Courant number of 0.5 and
    NSTEP covering 2 s, in one persistent launch. One bench step = the whole
    batch. `sequential` is the same shots run one after another through
    single-shot handles (measured once, outside the timed region)."""
    import torch
    from seismic_cpml_gb300.batch import Batch
    from seismic_cpml_gb300.solver import Solver
    from seismic_cpml_gb300.workloads import batch2d_shots
    torch.cuda.set_device(local)
    shots = batch2d_shots()
    cells = sum(sh[0].nx * sh[0].ny * sh[0].nstep for sh in shots)
    b = Batch([sh[0] for sh in shots], models=[sh[1] for sh in shots], receivers=[sh[2] for sh in shots])
    if args.tuning:
        b.set_tuning(*(int(x) for x in args.tuning.split(",")[:2]))
        tune = None
    else:
        tune = b.autotune(trial_steps=200)       # outside the timed region
    depth, tile_y = b.tuning()
    for _ in range(args.warmup):
        b.run()
    torch.cuda.synchronize()
    barrier(pg)
    clocks = ClockSampler(local)
    clocks.start()
    ms = []
    for _ in range(args.steps):
        b.run()
        ms.append(b.last_run_ms())
    clk = clocks.stop()
    dev_ms = max_over_ranks(pg, sum(ms))
    b.close()
    value = world * cells * args.steps / (dev_ms / 1e3) / 1e6
    seq_ms = 0.0
    for sh in shots:
        with Solver(sh[0], sh[2], model=sh[1]) as s1:
            s1.run()
            seq_ms += s1.last_run_ms()
    seq = cells / (seq_ms / 1e3) / 1e6
    t = time.perf_counter()
    for _ in range(args.steps):
        with Batch([sh[0] for sh in shots], models=[sh[1] for sh in shots],
                   receivers=[sh[2] for sh in shots]) as e:
            e.set_tuning(depth, tile_y)
            e.run()
            for q in range(len(shots)):
                e.seismograms(q)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(pg, time.perf_counter() - t)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle_c
        cores = os.cpu_count() or 1
        p, m = shots[0][0], shots[0][1]
        sess = oracle_c.Session(p, nthreads=cores, lam=m[0], mu=m[1], rho=m[2])
        sess.run(1)
        t0 = time.perf_counter()
        sess.run(200)
        dt = time.perf_counter() - t0
        sess.close()
        cpu = {"value": round(p.nx * p.ny * 200 / dt / 1e6, 3), "unit": "Mcell-updates/s", "cores": cores,
               "kind": "port", "sample": f"200 time steps of shot 0 ({p.nx} x {p.ny}), FP64 C++ restatement, "
                                         "OpenMP"}
    bytes_cell = 52.0
    peak, peak_kind = measured_peak()
    achieved = value * 1e6 * bytes_cell / 1e9
    line = {
        "metric": "Mcell-updates/s", "value": round(value, 3), "unit": "Mcell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dev_ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batch2d_256_shots", "shots": len(shots), "cell_updates": cells,
                   "l2": "inputs larger than L2 (about 4.5 GB of shot state)",
                   "kernel": {"depth": depth, "tile_y": tile_y, "autotuned": tune is not None,
                              "autotune_ms_per_step": tune["ms_per_step"] if tune else None}},
        "sequential_single_shot": {"value": round(seq, 3), "unit": "Mcell-updates/s",
                                   "speedup_of_batch": round(value / seq, 3)},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_kind,
                     "bytes_per_cell_update": "52 (fields and per-cell model; C-PML memory variables not counted)"},
        "cpu_baseline": cpu,
        "e2e": {"value": round(world * cells * args.steps / e2e_s / 1e6, 3), "unit": "Mcell-updates/s",
                "h2d_bytes_per_step": sum(12 * sh[0].nx * sh[0].ny for sh in shots),
                "d2h_bytes_per_step": sum(2 * 8 * len(sh[2]) * sh[0].nstep for sh in shots)},
        "gpu_launches": args.steps,
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def surrogate_flops_per_shot(cfg):
    """Multiply-add FLOPs of one shot's forward pass (all GEMMs)."""
    f = 0
    for (h, w, ci, co) in cfg.levels():
        f += 2 * ((h + 1) // 2) * ((w + 1) // 2) * co * 9 * ci
    f += 2 * cfg.flat() * cfg.latent + 2 * cfg.latent * (cfg.noff() * cfg.modes + 1)
    f += 2 * cfg.noff() * cfg.modes * cfg.nt
    return f


def run_surrogate(args, world, rank, local, pg):
    """Learned surrogate with FD fallback against the batched FD engine.

    Data: --train-shots training and --test-shots held-out seeded shots
    (seeds 5 and 50005) of the 296^2 surrogate workload, each run by the
    batched FD engine. The network trains for --epochs or --train-seconds.
    value : surrogate inference shots/s over the held-out inputs resident in
            HBM (K steps, CUDA events), without fallback.
    pipeline: surrogate + FD re-run of every shot whose predicted misfit is
            above --threshold, wall clock, held-out set.
    e2e   : the pipeline with host inputs: bf16 inputs host->device, traces
            device->host, FD re-runs of flagged shots."""
    import numpy as np
    import torch
    from seismic_cpml_gb300.surrogate import (NetConfig, ShotSpec, Surrogate, fd_seismograms,
                                              run_with_fallback)
    torch.cuda.set_device(local)
    spec, cfg = ShotSpec(), NetConfig()
    log = (lambda m: print(m, file=sys.stderr, flush=True)) if rank == 0 else None
    t0 = time.perf_counter()
    tm_train, tm_test = [], []
    Xtr, Str, Ytr = fd_seismograms(spec, 5, range(args.train_shots), timing=tm_train)
    gen_train_s = time.perf_counter() - t0
    t1 = time.perf_counter()
    Xte, Ste, Yte = fd_seismograms(spec, 50005, range(args.test_shots), timing=tm_test)
    fd_test_wall = time.perf_counter() - t1
    fd_dev_rate = args.test_shots / (sum(tm_test) / 1e3)
    fd_wall_rate = args.test_shots / fd_test_wall
    if log:
        log(f"FD: {args.train_shots} training shots in {gen_train_s:.1f} s, held-out {fd_dev_rate:.1f} "
            f"shots/s device, {fd_wall_rate:.1f} shots/s wall")
    scale = float(np.sqrt(np.mean(Ytr.astype(np.float64) ** 2)))
    Xt = torch.from_numpy(Xtr).to(torch.bfloat16).cuda()
    St = torch.from_numpy(Str).cuda()
    Tt = torch.from_numpy(Ytr.reshape(len(Ytr), -1) / scale).cuda()
    del Xtr, Ytr
    Xv = torch.from_numpy(Xte).to(torch.bfloat16).cuda()
    Sv = torch.from_numpy(Ste).cuda()
    Tv = torch.from_numpy(Yte.reshape(len(Yte), -1) / scale).cuda()
    net = Surrogate(cfg, seed=0)
    t2 = time.perf_counter()
    hist = net.train(Xt, St, Tt, epochs=args.epochs, batch=64, lr=1e-3, lr_min=1e-5,
                     time_budget_s=args.train_seconds, log=log)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t2
    P, head = net.predict(Xv, Sv)
    mis = net.misfit(P, Tv).sqrt().cpu().numpy().astype(np.float64)
    pred = np.exp(0.5 * head.cpu().numpy().astype(np.float64))
    train_mis = None
    if len(Xt):
        Pt, _ = net.predict(Xt[:2000], St[:2000])
        train_mis = float(np.median(net.misfit(Pt, Tt[:2000]).sqrt().cpu().numpy()))
        del Pt

    # timed region: inference on resident inputs
    for _ in range(args.warmup):
        net.predict(Xv, Sv, out=P)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = net.launches
    ev0.record()
    for _ in range(args.steps):
        net.predict(Xv, Sv, out=P)
    ev1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = net.launches - launches0
    dev_ms = ev0.elapsed_time(ev1)
    nn_rate = args.steps * args.test_shots / (dev_ms / 1e3)
    flops = surrogate_flops_per_shot(cfg)
    tflops = flops * nn_rate / 1e12
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak, peak_kind = float(json.load(f)["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        peak, peak_kind = 1900.0, "fallback"

    # surrogate + fallback, inputs resident
    idx = list(range(args.test_shots))
    out, mask, s_nn, s_fd = run_with_fallback(net, spec, 50005, idx, Xv, Sv, threshold=args.threshold,
                                              scale=scale)
    final = net.misfit(out, Tv).sqrt().cpu().numpy().astype(np.float64)
    pipe_rate = args.test_shots / (s_nn + s_fd)

    # end to end: host inputs, host outputs
    e2e = None
    if not args.no_e2e:
        Xh = torch.from_numpy(Xte).to(torch.bfloat16).pin_memory()
        Sh = torch.from_numpy(Ste).pin_memory()
        Ph = torch.empty((args.test_shots, cfg.nrec * cfg.nt), dtype=torch.float32).pin_memory()
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        Xd = Xh.cuda(non_blocking=True)
        Sd = Sh.cuda(non_blocking=True)
        outd, mask2, _, _ = run_with_fallback(net, spec, 50005, idx, Xd, Sd, threshold=args.threshold,
                                              scale=scale)
        Ph.copy_(outd, non_blocking=True)
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t3
        e2e = {"value": round(args.test_shots / e2e_s, 2), "unit": "shots/s",
               "h2d_bytes_per_step": Xh.numel() * 2 + Sh.numel() * 4, "d2h_bytes_per_step": Ph.numel() * 4 + args.test_shots,
               "fd_fallback_shots": int(mask2.sum())}

    thr = args.threshold
    line = {
        "metric": "surrogate shots/s", "value": round(nn_rate, 1), "unit": "shots/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dev_ms / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
        "config": {"workload": "surrogate_296sq_2000steps", "train_shots": args.train_shots,
                   "test_shots": args.test_shots, "network": "source-frame 5-level conv encoder + dense + DCT offset-trace synthesis",
                   "params": cfg.n_params(), "batch": 64, "epochs_run": len(hist),
                   "train_seconds": round(train_s, 1), "threshold": thr,
                   "l2": "inputs and activations larger than L2"},
        "quality": {"median_rel_l2": round(float(np.median(mis)), 4),
                    "p90_rel_l2": round(float(np.percentile(mis, 90)), 4),
                    "frac_le_threshold": round(float(np.mean(mis <= thr)), 4),
                    "train_median_rel_l2": round(train_mis, 4) if train_mis is not None else None,
                    "head_corr": round(float(np.corrcoef(np.log(pred), np.log(mis))[0, 1]), 3),
                    "fallback_frac": round(float(mask.mean()), 4),
                    "after_fallback_median_rel_l2": round(float(np.median(final)), 4),
                    "after_fallback_frac_le_threshold": round(float(np.mean(final <= thr)), 4)},
        "fd": {"device_shots_per_s": round(fd_dev_rate, 2), "wall_shots_per_s": round(fd_wall_rate, 2),
               "engine": "batched persistent 2D FD, 1024 shots per launch"},
        "pipeline": {"shots_per_s": round(pipe_rate, 2), "surrogate_s": round(s_nn, 3),
                     "fd_s": round(s_fd, 3), "speedup_vs_fd_wall": round(pipe_rate / fd_wall_rate, 2)},
        "speedup_surrogate_only_vs_fd_device": round(nn_rate / fd_dev_rate, 1),
        "roofline": {"bound": "tensor", "achieved": round(tflops, 2), "peak": peak, "unit": "TFLOP/s",
                     "frac": round(tflops / peak, 4), "traffic": None, "peak_source": peak_kind,
                     "flops_per_shot": flops},
        "cpu_baseline": None,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    world, rank, local, pg = dist_setup(args)
    try:
        if args.workload in ("2d_plain", "batch2d") and args.impl != "reference":
            return (run_2d_plain if args.workload == "2d_plain" else run_batch2d)(args, world, rank, local, pg)
        if args.workload in ("2d_plain", "batch2d"):
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the CPU restatement is timed inside "
                                  "this workload's own line (cpu_baseline)"}))
            return 0
        if args.workload == "surrogate":
            if args.impl == "reference":
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned "
                                  "surrogate; its batched-FD comparison is in the surrogate line"}))
                return 0
            return run_surrogate(args, world, rank, local, pg)
        if args.impl == "reference":
            if args.workload == "3d_large":
                if rank == 0:
                    print(json.dumps({"impl": "reference", "unavailable": "the FP64 CPU restatement is "
                                      "timed on the 3d_plain workload; 551 M cells in FP64 exceed a "
                                      "bounded CPU sample"}))
                return 0
            return run_reference(args, world, rank, pg)
        return run_ours(args, world, rank, local, pg)
    finally:
        if pg is not None:
            pg.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
