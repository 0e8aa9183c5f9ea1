#!/usr/bin/env python
"""Benchmark of the SPH step: particle-steps/s on the 1,048,576-particle
double dam break, with the HBM roofline of the dominant kernel.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step is one cSPH::Update (integrate, hash, sort, cell ranges, density,
force) over all particles.  Inputs are synthetic and seeded
(pibiti_gb300/configs.py).  Our arm times K steps with CUDA events on the
handle's stream, an event before each stage, each step started with a cold
L2 (a 256 MiB buffer is written before each timed step, outside the events),
so the per-stage times and the roofline come from the same steps as the
headline; the state 800 steps in (the crowded phase of the workload) is
timed the same way and reported beside it.  `e2e` repeats the steps through
the public API with positions and velocities uploaded from and read back to
pinned host memory every step.  Under torchrun every rank runs an
independent replica (the scene does not shard) and rank 0 prints one JSON
line with the whole-job throughput.

`--impl reference` times the CPU restatement of the reference's step (the
oracle; the reference itself has no CPU path) on all host cores, on the same
1,048,576-particle workload with the same warm-up and step counts, with the
SimParams the reference's own scene loader derived for it (recorded in
tests/golden/scenes.npz); where the reference's kernels were compiled to PTX
(oracle/_ref), their GPU step on the same workload is timed beside it
(`reference_gpu`).  Nothing of the product library is loaded on that arm.
"""
from __future__ import annotations

import argparse
import json
import math

import numpy as np
import os
import platform
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s at 1M (plain vs learned, ≤1% density err); % HBM roofline"
UNIT = "particle-steps/s"
# Algorithmic bytes per particle (and per cell) each stage moves, every array
# read or written once (intermediate arrays such as the neighbour masks are
# not counted).
STAGE_BYTES = {  # stage: (bytes per particle, bytes per cell)
    "integrate_count": (40, 12),
    "scan": (0, 8),
    "scatter_ids": (20, 0),
    "place": (88, 0),
    "density": (24, 8),
    "force": (56, 8),
}
KERNELS_PER_STEP = 9  # integrate_count, 2 scan kernels (which also list the crowded cells),
#                      scatter_ids, rank_cells, rank_big_cells, place, density, force


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), \
        int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(value: float, device=None) -> float:
    """Largest `value` over all ranks (the job's time is its slowest rank's);
    the value itself when no process group is initialised."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(particles_per_rank: int, steps: int, world: int, max_ms: float) -> float:
    """Whole-job particle-steps/s: every rank steps its own replica."""
    return world * particles_per_rank * steps / (max_ms / 1e3)


def shard_scenes(sizes, world: int, rank: int) -> list:
    """Scenes of `rank` when the ensemble's independent scenes are split over
    `world` GPUs: largest first to the least-loaded rank (ties to the lower
    rank), so the ranks' particle totals differ by at most one scene.  The
    same plan on every rank; returned in scene order."""
    load = [0] * world
    owner = [0] * len(sizes)
    for k in sorted(range(len(sizes)), key=lambda q: (-sizes[q], q)):
        r = min(range(world), key=lambda q: (load[q], q))
        owner[k] = r
        load[r] += sizes[k]
    return [k for k in range(len(sizes)) if owner[k] == rank]


def barrier() -> None:
    """All ranks meet (no-op without a process group)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def ensemble_throughput(total_particles: int, steps: int, max_ms: float) -> float:
    """Whole-job particle-steps/s of the sharded ensemble: every scene of the
    job over the slowest rank's time."""
    return total_particles * steps / (max_ms / 1e3)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


CROWDED_STEP = 800      # the crowded phase, timed beside the headline steps
ENSEMBLE_STEPS = 500    # steps of the ensemble measurement (one CUDA graph)
WALK_PROFILE = os.path.join("profiles", "walk_kernels_double_dambreak_1M.md")
SMS = 152               # GB300 multiprocessors
ISSUE_PER_SM_CLOCK = 4  # warp instructions issued per SM per clock (4 schedulers)


def ncu_summary(key: str, kernel: str, state: str):
    """A per-launch figure of `kernel` at `state` ("early", "crowded") from
    the committed ncu summary of this workload: `traffic` (DRAM bytes read +
    written), `instructions` (warp instructions executed) or `issue`
    (fraction of issue slots busy); None if it has no entry."""
    path = os.path.join(ROOT, WALK_PROFILE)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(f"{key} {kernel} {state}:"):
            return float(line.split(":")[1].split()[0])
    return None


def timed_steps(sysm, stream, flush, steps: int):
    """`steps` steps, each after a write of `flush` (larger than L2) and with
    a CUDA event before each stage on the handle's stream: per-step ms and
    per-stage lists of ms."""
    import torch
    from pibiti_gb300.sph import SPH
    step_ms, stages = [], {k: [] for k in SPH.STAGES}
    with torch.cuda.stream(stream):
        for k in range(steps):
            flush.fill_(k & 0xff)
            st = sysm.step_timed()
            for name, v in st.items():
                stages[name].append(v)
            step_ms.append(sum(st.values()))
    return step_ms, stages


def stage_roofline(stages: dict, n: int, cells: int, peak: float, peak_kind: str, walk: dict,
                   state: str, sm_mhz, where: str) -> dict:
    """HBM roofline of the dominant stage (median over the given steps):
    its algorithmic bytes per launch over its CUDA-event time, against the
    measured copy bandwidth; beside it the issue-slot roof of the same
    kernel: its warp instructions per launch (the committed ncu summary of
    the same state) over SMS x 4 issue slots per clock at the sampled SM
    clock."""
    stage_ms = {k: statistics.median(v) for k, v in stages.items()}
    dom = max(stage_ms, key=stage_ms.get)
    bp, bc = STAGE_BYTES[dom]
    alg = bp * n + bc * cells
    achieved = alg / (stage_ms[dom] / 1e3) / 1e9
    kernel = walk.get("kernels", {}).get(dom, f"k_{dom}")
    traffic = ncu_summary("traffic", kernel, state)
    instr = ncu_summary("instructions", kernel, state)
    binding = None
    if instr and sm_mhz:
        issue_ms = instr / (SMS * ISSUE_PER_SM_CLOCK * sm_mhz * 1e3)
        binding = {"resource": "instruction issue", "warp_instructions": instr,
                   "issue_roof_ms": issue_ms, "frac": issue_ms / stage_ms[dom],
                   "sm_mhz": sm_mhz, "source": f"{WALK_PROFILE} ({state} state)"}
    return {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "traffic_state": state,
            "algorithmic_bytes": alg, "peak_source": peak_kind, "stage_ms": stage_ms,
            "stage_ms_sum": sum(stage_ms.values()), "steps": where, "binding": binding}


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.gpu = gpu_index
        self.out = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def reference_params(xml: str) -> bytes:
    """SimParams bytes the reference's own scene loader (Scene.cpp,
    Scene_Load.cpp, run through oracle/ref_emu) derived for the scene element
    `xml`, as recorded in tests/golden/scenes.npz by
    tests/golden/make_golden.py.  The reference arm takes its parameters
    from here, not from the product's loader."""
    with np.load(os.path.join(ROOT, "tests", "golden", "scenes.npz")) as z:
        xmls = [str(x) for x in z["xml"]]
        if xml not in xmls:
            raise KeyError("workload scene element not in tests/golden/scenes.npz "
                           "(regenerate it with tests/golden/make_golden.py)")
        return z["params"][xmls.index(xml)].tobytes()


def time_cpu_oracle(params: bytes, pos, vel, warmup: int, steps: int):
    """The oracle's single-precision step (OpenMP, all host threads) on the
    full workload: `warmup` untimed steps, then `steps` timed steps in one
    call.  Returns (particle-steps/s, seconds, threads)."""
    import oracle
    if warmup:
        pos, vel = oracle.step(params, pos, vel, steps=warmup)
    t0 = time.perf_counter()
    oracle.step(params, pos, vel, steps=steps)
    dt = time.perf_counter() - t0
    return len(pos) * steps / dt, dt, oracle.threads()


def time_reference_gpu(params: bytes, pos, vel, warmup: int, steps: int):
    """The reference's own CUDA kernels (System.cu, radixsort_kernel.cu,
    compiled to PTX with nvcc's default flags by oracle/ref_gpu/build_ref_gpu.sh)
    stepping the same workload on this GPU as cSPH::Update does, every
    wrapper ending with a device synchronisation (SPH_Update.cpp:39-76,
    System.cu:653-756): wall time of `steps` steps after `warmup`.  None
    where the PTX or the GPU is missing."""
    try:
        import torch
        import oracle.ref_gpu as rg
        if not torch.cuda.is_available() or not rg.available():
            return None
    except Exception:  # no harness on this machine
        return None
    from pibiti_gb300.params import SimParams  # the ABI struct's layout only (ctypes)
    p = SimParams.from_bytes(params)
    r = rg.RefStep(p, pos, vel, fast=True)
    r.update(warmup)
    torch.cuda.synchronize()
    stage = {}
    t0 = time.perf_counter()
    r.update(steps, stage)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return {"value": len(pos) * steps / dt, "unit": UNIT, "ms_per_step": 1e3 * dt / steps,
            "stage_ms": {k: 1e3 * v / steps for k, v in stage.items()},
            "note": "the reference's own kernels on this GPU, launched with its wrappers' grids "
                    "and a device synchronisation after each wrapper; same workload, warm-up "
                    "and step count as this line"}


def run_cpu_configs(args) -> int:
    """The oracle's single-precision step (OpenMP, all host threads) on the
    full workloads, one JSON line each: the 32,768-particle dam break, the
    1,048,576-particle double dam break and, with fewer steps, the
    16,777,216-particle uniform block.  One untimed step first."""
    import oracle
    from pibiti_gb300 import configs
    from pibiti_gb300.sph import Scene
    cases = (("dam break, 32,768 particles", configs.dambreak_small, 100),
             ("double dam break, 1,048,576 particles", configs.dambreak_double, 5),
             ("uniform block, 16,777,216 particles", configs.uniform_stress, 2))
    for name, make, k in cases:
        w = make()
        p = Scene.parse(w.xml).params
        pos, vel = oracle.step(p, w.pos, w.vel, steps=1)
        t0 = time.perf_counter()
        pos, vel = oracle.step(p, pos, vel, steps=k)
        t = time.perf_counter() - t0
        print(json.dumps({"impl": "reference", "kind": "port", "workload": name, "particles": w.n,
                          "steps": k, "value": w.n * k / t, "unit": UNIT, "ms_per_step": 1e3 * t / k,
                          "cores": oracle.threads(), "cpu": platform.machine()}), flush=True)
        del w, pos, vel
    return 0


def run_reference(args):
    """The reference arm: the oracle's CPU step on the full workload (the
    reference has no CPU path of its own), rank 0 only; the reference's own
    GPU kernels on the same workload beside it where they are built."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from pibiti_gb300 import configs
    w = configs.dambreak_double()
    params = reference_params(w.xml)
    value, dt, threads = time_cpu_oracle(params, w.pos, w.vel, args.warmup, args.steps)
    sample = (f"the full workload ({w.n} particles), {args.warmup} untimed then {args.steps} "
              f"timed steps, oracle single-precision restatement, SimParams from the "
              f"reference's scene loader")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": workload_config(None),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_gpu": time_reference_gpu(params, w.pos, w.vel, args.warmup, args.steps),
        "notes": "The reference has no CPU implementation of its step; this is the oracle's "
                 "single-precision restatement of it (oracle/sph_oracle.c), OpenMP on all "
                 "host threads, on the same workload as our arm.",
    }
    print(json.dumps(line), flush=True)
    return 0


def ensemble_single(e, ps, stream, warmup: int, steps: int) -> dict:
    """The ensemble `e` (scene parameters `ps`) in one handle on this GPU:
    `warmup` steps, the autotuner, then `steps` steps captured as one CUDA
    graph and launched once (CUDA events); beside it the same steps as one
    persistent cooperative launch, and the first 32 scenes stepped one
    handle each."""
    import torch
    from pibiti_gb300.sph import ARRAY_POS, ARRAY_VEL, SPH
    sysm = SPH(ps, stream=stream)
    sysm.set_array(ARRAY_POS, e.pos)
    sysm.set_array(ARRAY_VEL, e.vel)
    sysm.update(warmup)
    chosen, tune_ms = sysm.autotune(trial_steps=5)
    sysm.set_graph_steps(steps)
    sysm.update(steps)  # builds and runs the graph once (untimed)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sysm.update(steps)  # one graph launch
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    st = sysm.stats()
    sysm.close()
    # the same steps as one persistent cooperative launch, from the same start
    with SPH(ps, stream=stream) as ph:
        ph.set_array(ARRAY_POS, e.pos)
        ph.set_array(ARRAY_VEL, e.vel)
        ph.set_persistent(True)
        ph.update(warmup)
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        ph.update(steps)  # one launch
        p1.record(stream)
        torch.cuda.synchronize()
        pms = p0.elapsed_time(p1)
        persistent = {"value": ph.n * steps / (pms / 1e3), "unit": UNIT, "ms_per_step": pms / steps,
                      "barrier_timeout": bool(ph.flags() & 4),
                      "note": f"{steps} steps in one cooperative launch (grid barrier between stages)"}
    # the same scenes, one handle each, for the first 32 scenes
    sub = 32
    t_sep, n_sep = 0.0, 0
    off = 0
    for k in range(sub):
        nk = e.sizes[k]
        with SPH(ps[k], stream=stream) as one:
            one.set_array(ARRAY_POS, e.pos[off:off + nk])
            one.set_array(ARRAY_VEL, e.vel[off:off + nk])
            one.update(4)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            one.update(50)
            b.record(stream)
            torch.cuda.synchronize()
            t_sep += a.elapsed_time(b) / 1e3
            n_sep += nk * 50
        off += nk
    return {
        "metric": "ensemble particle-steps/s", "value": e.n * steps / (ms / 1e3), "unit": UNIT,
        "steps": steps, "warmup": warmup, "ms_per_step": ms / steps,
        "config": {"workload": f"batched ensemble: {len(ps)} dam-break scenes, "
                               f"{min(e.sizes)}-{max(e.sizes)} particles (log-uniform, x512), "
                               f"k in [1,5], mu in [1,6]", "particles": e.n,
                   "cells": int(sum(p.numCells for p in ps)),
                   "graph": f"{steps} steps captured as one CUDA graph, one launch"},
        "autotune": {"chosen_shape": chosen, "chosen_threads": SPH.WALK_THREADS[chosen],
                     "staged": SPH.WALK_STAGED[chosen], "ms_per_step": tune_ms},
        "separate_handles": {"scenes": sub, "value": n_sep / t_sep, "unit": UNIT},
        "persistent": persistent,
        "state_check": {"max_density_dev": float(st[:, 2].max()), "nonfinite": float(st[:, 3].sum())},
    }


def measure_ensemble(warmup: int, steps: int) -> dict:
    """The 256-scene ensemble on this GPU (ensemble_single)."""
    import torch
    from pibiti_gb300 import configs
    from pibiti_gb300.sph import Scene
    e = configs.ensemble(steps=steps)
    ps = [Scene.parse(x).params for x in e.xmls]
    return ensemble_single(e, ps, torch.cuda.Stream(), warmup, steps + (steps % 2))


def run_ensemble(args):
    """256 independent dam-break scenes (4k-64k particles, k in [1,5], mu in
    [1,6]) stepped together in one handle per GPU: `steps` steps captured as
    one CUDA graph and launched once, after the autotuner picked the walk
    shape.  Under torchrun the scenes are split over the ranks with no
    exchange."""
    import torch
    from pibiti_gb300 import configs
    from pibiti_gb300.sph import ARRAY_POS, ARRAY_VEL, SPH, Scene
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    steps = args.steps + (args.steps % 2)
    if world == 1:
        clocks = ClockSampler(local)
        clocks.start()
        line = measure_ensemble(args.warmup, steps)
        line.update({"n_gpus": 1, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
                     "clocks": clocks.stop()})
        print(json.dumps(line), flush=True)
        return 0
    import torch.distributed as dist
    dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    e = configs.ensemble(steps=args.steps)
    total = e.n
    mine = shard_scenes(e.sizes, world, rank)  # independent scenes: no exchange
    offs = np.concatenate([[0], np.cumsum(e.sizes)])
    sel = np.concatenate([np.arange(offs[k], offs[k + 1]) for k in mine])
    e = configs.Ensemble(e.name, [e.xmls[k] for k in mine], e.pos[sel], e.vel[sel],
                         [e.sizes[k] for k in mine], e.steps, dict(e.notes, scenes=mine))
    ps = [Scene.parse(x).params for x in e.xmls]
    stream = torch.cuda.Stream()
    sysm = SPH(ps, stream=stream)
    sysm.set_array(ARRAY_POS, e.pos)
    sysm.set_array(ARRAY_VEL, e.vel)
    sysm.update(args.warmup)
    sysm.autotune(trial_steps=5)
    sysm.set_graph_steps(steps)
    sysm.update(steps)  # builds and runs the graph once (untimed)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sysm.update(steps)  # one graph launch
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = max_over_ranks(e0.elapsed_time(e1), device="cuda")
    value = ensemble_throughput(total, steps, ms)
    sysm.close()
    if rank == 0:
        print(json.dumps({
            "metric": "ensemble particle-steps/s", "value": value, "unit": UNIT, "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": ms / steps,
            "higher_is_better": True, "scaling": "strong", "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batched ensemble: 256 dam-break scenes split over the GPUs by "
                                   "particle count (no exchange)", "particles": total,
                       "graph": f"{steps} steps captured as one CUDA graph per rank"},
            "clocks": clk}), flush=True)
    dist.destroy_process_group()
    return 0


def measure_learned(w, p, stream, fine_steps: int = 2000, substeps: int = 4, tol: float = 0.02):
    """The learned 4x dt form on the 1M-particle double dam break from its
    initial state, over the configuration's 2000 steps of dt: simulated-time
    throughput (particle-steps of dt per second, CUDA events on the handle's
    stream, one call of 500 coarse steps) against 2000 plain steps from the
    same state, and the mean-density error relative to that fine run,
    sampled every coarse step in separate untimed runs (time-mean, worst
    instant, end), with and without the network."""
    import torch
    from pibiti_gb300 import learned
    from pibiti_gb300.sph import ARRAY_POS, ARRAY_VEL, SPH
    if not os.path.exists(learned.MODEL_PATH):
        return {"unavailable": "no trained model at pibiti_gb300/models/corrector.npz"}
    model = learned.Model.load()
    n = len(w.pos)
    coarse_steps = fine_steps // substeps

    def fresh(mode):
        h = SPH(p, stream=stream)
        h.set_array(ARRAY_POS, w.pos)
        h.set_array(ARRAY_VEL, w.vel)
        if mode != "fine":
            (model if mode == "learned" else learned.zero_model()).install(h)
            learned.learned_step(h, 0, substeps, tol)  # buffers allocated outside the timing
        return h

    res = {}
    for mode in ("fine", "learned"):
        h = fresh(mode)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fb = 0
        if mode == "fine":
            h.update(fine_steps)
        else:
            fb = learned.learned_step(h, coarse_steps, substeps, tol)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        res[mode] = {"value": n * fine_steps / (ms / 1e3), "ms": ms, "fallbacks": fb}
        h.close()
    rho = {}
    for mode in ("fine", "learned", "drift"):
        h = fresh(mode)
        traj = []
        for _ in range(coarse_steps):
            if mode == "fine":
                h.update(substeps)
            else:
                learned.learned_step(h, 1, substeps, tol if mode == "learned" else 1e9)
            traj.append(h.stats()[0][1])
        rho[mode] = np.asarray(traj)
        h.close()
    err = {k: np.abs(rho[k] - rho["fine"]) / rho["fine"] for k in ("learned", "drift")}
    return {"unit": UNIT, "value": res["learned"]["value"], "fine_value": res["fine"]["value"],
            "speedup_vs_fine": res["learned"]["value"] / res["fine"]["value"],
            "ms": res["learned"]["ms"], "fine_ms": res["fine"]["ms"],
            "mean_density_err": {"time_mean": float(err["learned"].mean()),
                                 "max": float(err["learned"].max()),
                                 "end": float(err["learned"][-1])},
            "without_network": {"time_mean": float(err["drift"].mean()),
                                "max": float(err["drift"].max()),
                                "end": float(err["drift"][-1])},
            "fallbacks": res["learned"]["fallbacks"], "coarse_steps": coarse_steps,
            "substeps": substeps, "tol": tol,
            "note": "simulated-time throughput: particle-steps of dt per second over 2000 steps "
                    "of dt from the initial state; mean-density error relative to the fine-dt "
                    "plain run, sampled every coarse step; without_network = the same coarse "
                    "step with the drift correction and a zero network, no density check"}


def measure_render(sysm, p, stream, width: int = 1920, height: int = 1080, iterations: int = 8,
                   frames: int = 10):
    """The headless renderer on the state the timed steps left (advanced by
    one step with the colour output on, for the foam overlay's input):
    curvature flow with `iterations` passes at width x height, wall time per
    frame (each frame is synchronous), then the foam overlay alone."""
    import torch
    from pibiti_gb300.render import Renderer, look_at, perspective
    from pibiti_gb300.sph import ARRAY_POS
    pos = torch.empty((sysm.n, 4), dtype=torch.float32, device="cuda")
    clr = torch.empty((sysm.n, 4), dtype=torch.float32, device="cuda")
    sysm.set_color_output(clr)
    sysm.update(1)
    sysm.set_color_output(None)
    sysm.get_array(ARRAY_POS, out=pos)
    torch.cuda.synchronize()
    mv = look_at((3.0, 2.6, 6.8), (3.0, 0.6, 0.85))
    pr = perspective(60.0, width / height, 0.1, 20.0)
    with Renderer(width, height) as r:
        prm = r.params(mv, pr, radius=2.0 * p.particleR, method=1, iterations=iterations)
        for _ in range(2):
            r.frame_params(pos, prm)
        t0 = time.perf_counter()
        for _ in range(frames):
            r.frame_params(pos, prm)
        ms = 1e3 * (time.perf_counter() - t0) / frames
        frags = r.fragments
        rgba = r.frame_params(pos, prm)[2]
        r.foam_params(pos, clr, prm, rgba)
        t0 = time.perf_counter()
        for _ in range(frames):
            fdepth = r.foam_params(pos, clr, prm, rgba)
        foam_ms = 1e3 * (time.perf_counter() - t0) / frames
        foam_px = int((fdepth < 1).sum().item())
    return {"ms_per_frame": ms, "width": width, "height": height, "particles": sysm.n,
            "method": "curvature flow", "iterations": iterations, "fragments": int(frags),
            "fragments_per_s": frags / (ms / 1e3),
            "foam_ms": foam_ms, "foam_pixels": foam_px,
            "note": "depth + thickness G-buffer in draw order, smoothing, shading; wall time "
                    "of synchronous frames; foam_ms: the foam overlay (two sprites per "
                    "particle at most, last fragment wins) over the frame, colour from one "
                    "more step with the colour output on"}


def workload_config(p, n=None):
    cfg = {"workload": "double dam break, 1,048,576 particles: two 64x128x64 lattices at "
                       "spacing 0.5h (h=0.0457 m) in a 6.0x3.4x1.7 m box, +-1% jitter, "
                       "rho0=1000, k=3, mu=3.5, g=-9.8, dt=1e-3, maxParInCell=16",
           "particles": 1048576}
    if p is not None:
        cfg.update({"cells": int(p.numCells), "grid": [int(p.gridSize.x), int(p.gridSize.y),
                                                         int(p.gridSize.z)],
                    "l2": "flushed before every timed step (256 MiB write)"})
    return cfg


def run_state_tool(args) -> int:
    """Saved states for profiling: a capture can then start at the crowded
    phase of the workload after a handful of launches instead of thousands."""
    import numpy as np
    import torch
    from pibiti_gb300 import configs
    from pibiti_gb300.sph import ARRAY_POS, ARRAY_VEL, SPH, Scene
    torch.cuda.set_device(0)
    w = configs.dambreak_double()
    p = Scene.parse(w.xml).params
    with SPH(p) as s:
        if args.save_state:
            s.set_array(ARRAY_POS, w.pos)
            s.set_array(ARRAY_VEL, w.vel)
            s.update(args.warm_steps)
            np.savez(args.save_state, pos=s.get_array(ARRAY_POS), vel=s.get_array(ARRAY_VEL))
            print(json.dumps({"saved": args.save_state, "steps": args.warm_steps}))
            return 0
        z = np.load(args.stages)
        s.set_array(ARRAY_POS, z["pos"])
        s.set_array(ARRAY_VEL, z["vel"])
        if args.walk_shape is not None:
            s.set_walk_shape(args.walk_shape)
        for _ in range(args.steps):
            print(json.dumps({"stage_ms": s.step_timed()}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--warm-steps", type=int, default=200)
    ap.add_argument("--workload", choices=["double_dambreak", "ensemble"], default="double_dambreak",
                    help="ensemble: the 256-scene batched ensemble (a separate measurement)")
    ap.add_argument("--cpu-budget", type=float, default=12.0, help="seconds of CPU baseline work")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-form measurement")
    ap.add_argument("--no-render", action="store_true", help="skip the render measurement")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the ensemble measurement")
    ap.add_argument("--save-state", metavar="NPZ",
                    help="profiling aid: run --warm-steps steps of the workload, save the state, exit")
    ap.add_argument("--walk-shape", type=int, default=None,
                    help="profiling aid: walk shape for --stages (sph_set_walk_shape)")
    ap.add_argument("--stages", metavar="NPZ",
                    help="profiling aid: load a saved state, print --steps per-stage step times")
    ap.add_argument("--cpu-configs", action="store_true",
                    help="time the oracle's CPU step on the full 32K, 1M and 16.7M workloads and exit")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.cpu_configs:
        return run_cpu_configs(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.save_state or args.stages:
        return run_state_tool(args)
    if args.workload == "ensemble":
        return run_ensemble(args)

    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from pibiti_gb300 import configs
    from pibiti_gb300.sph import ARRAY_POS, ARRAY_VEL, SPH, Scene

    w = configs.dambreak_double(seed=42 + rank)

    # CPU baseline first (no GPU work has started; rank 0 at N=1 only): the
    # oracle on the full workload for about --cpu-budget seconds
    cpu = None
    if rank == 0 and world == 1 and args.cpu_budget > 0:
        params = reference_params(configs.dambreak_double().xml)
        v1, t1, _ = time_cpu_oracle(params, w.pos, w.vel, 1, 1)
        k = max(3, int(args.cpu_budget / max(t1, 1e-3)))
        v, _, threads = time_cpu_oracle(params, w.pos, w.vel, 1, k)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"the full workload ({w.n} particles), steps 2-{k + 1}, oracle "
                         f"single-precision restatement, OpenMP on all host threads"}

    p = Scene.parse(w.xml).params
    stream = torch.cuda.Stream()
    sysm = SPH(p, stream=stream)
    sysm.set_array(ARRAY_POS, w.pos)
    sysm.set_array(ARRAY_VEL, w.vel)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    shape = sysm.walk_shape()
    walk = {"shape": shape, "threads": SPH.WALK_THREADS[shape], "staged": SPH.WALK_STAGED[shape],
            "kernels": dict(zip(("density", "force"), SPH.WALK_KERNELS[shape]))}

    with torch.cuda.stream(stream):
        sysm.update(args.warmup)
    torch.cuda.synchronize()
    stepped = args.warmup

    clocks = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    wall0 = time.perf_counter()
    step_ms, stages = timed_steps(sysm, stream, flush, args.steps)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    stepped += args.steps
    total_ms = max_over_ranks(sum(step_ms), device="cuda")
    n = sysm.n
    value = job_throughput(n, args.steps, world, total_ms)
    peak, peak_kind = measured_peaks()
    state = "early" if stepped <= 400 else "crowded"
    roofline = stage_roofline(stages, n, p.numCells, peak, peak_kind, walk, state,
                              clk.get("sm_mhz"), f"steps {args.warmup}-{stepped} (the timed steps)")
    P = 4 if p.numCells >= 65536 else 2
    model_b = 256 + 24 * P + 12 * p.numCells / n
    step_gbs = model_b * n / (total_ms / args.steps / 1e3) / 1e9
    roofline_step = {"bytes_per_particle_step": model_b, "achieved": step_gbs, "peak": peak,
                     "unit": "GB/s", "frac": step_gbs / peak,
                     "note": "reference dataflow byte model B = 256 + 24P + 12C/N"}

    # warm multi-step throughput (graph replay, L2 not flushed): informative
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    warm_steps = max(args.warm_steps, 2)
    e0.record(stream)
    sysm.update(warm_steps)
    e1.record(stream)
    torch.cuda.synchronize()
    warm_ms = e0.elapsed_time(e1) / warm_steps
    stepped += warm_steps

    # end to end through the public API with pinned host buffers
    hpos = torch.empty((n, 4), dtype=torch.float32).pin_memory()
    hvel = torch.empty((n, 4), dtype=torch.float32).pin_memory()
    sysm.get_array(ARRAY_POS, hpos.numpy())
    sysm.get_array(ARRAY_VEL, hvel.numpy())
    es, ee = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    es.record(stream)
    for _ in range(args.e2e_steps):
        sysm.set_array(ARRAY_POS, hpos.numpy())
        sysm.set_array(ARRAY_VEL, hvel.numpy())
        sysm.update(1)
        sysm.get_array(ARRAY_POS, hpos.numpy())
        sysm.get_array(ARRAY_VEL, hvel.numpy())
    ee.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(es.elapsed_time(ee), device="cuda")
    e2e_value = job_throughput(n, args.e2e_steps, world, e2e_ms)
    stepped += args.e2e_steps

    # the crowded phase: the same handle stepped on to step CROWDED_STEP,
    # then timed as the headline steps are
    crowded = None
    if rank == 0 and stepped < CROWDED_STEP:
        sysm.update(CROWDED_STEP - stepped)
        stepped = CROWDED_STEP
        cms, cst = timed_steps(sysm, stream, flush, 10)
        stepped += 10
        crowded = {"steps": f"{CROWDED_STEP}-{stepped}", "ms_per_step": sum(cms) / len(cms),
                   "value": n * len(cms) / (sum(cms) / 1e3), "unit": UNIT,
                   "roofline": stage_roofline(cst, n, p.numCells, peak, peak_kind, walk, "crowded",
                                              clk.get("sm_mhz"), f"steps {CROWDED_STEP}-{stepped}")}

    learned = measure_learned(w, p, stream) if rank == 0 and not args.no_learned else None
    render = measure_render(sysm, p, stream) if rank == 0 and not args.no_render else None
    ensemble = None
    if rank == 0 and world == 1 and not args.no_ensemble:
        sysm_state = sysm.stats()[0]
        ensemble = measure_ensemble(args.warmup, ENSEMBLE_STEPS)
    else:
        sysm_state = sysm.stats()[0]

    st = sysm_state
    flags = sysm.flags()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(p),
            "parallelism": f"replicas x{world}" if world > 1 else "single",
            "walk": walk,
            "e2e": {"value": e2e_value, "unit": UNIT, "steps": args.e2e_steps,
                    "h2d_bytes_per_step": 2 * n * 16, "d2h_bytes_per_step": 2 * n * 16},
            "roofline": roofline, "roofline_step": roofline_step,
            "crowded": crowded,
            "cpu_baseline": cpu, "clocks": clk,
            "gpu_launches": KERNELS_PER_STEP * args.steps,
            "warm_ms_per_step": warm_ms,
            "wall_s_timed_loop": wall,
            "learned": learned,
            "ensemble": ensemble,
            "render": render,
            "state_check": {"kinetic_energy": st[0], "mean_density": st[1],
                            "max_density_dev": st[2], "nonfinite": st[3], "flags": flags},
        }
        print(json.dumps(line), flush=True)
    sysm.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0

if __name__ == "__main__":
    sys.exit(main())
