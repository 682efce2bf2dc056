"""Benchmark of the coupled SPH + wave step on GB300.

Metric: particle + wave-cell updates per second (one update = one particle
or one wave cell advanced one step).  Workload: the 1,048,576-particle
dam-break (128x64x128 lattice, s = 0.0075, h = 2s, 67^3 grid cells) coupled to a
1024^2 height field, float32 with compensated neighbour sums, synthetic
seeded inputs.  Each timed step is one full cwa_step (grid sort -> rho_pres
-> force -> integrate + coupling -> wave) with the state resident in HBM;
L2 is flushed (256 MiB write on the sim's stream) before every step, outside
the per-step CUDA events.  The timed steps are steps warmup + 2 ..
warmup + steps + 1 of the run: a checkpoint taken after the warm-up is
reloaded once the clock sampler is logging, and the per-pass profile
restarts from it, so both cover the same simulated steps.

`e2e` runs the same steps through the public C ABI with host buffers: each
step uploads the particle records and both wave fields from pinned host
memory, steps, and downloads the particle records and u^n.

N > 1 (torchrun): every rank runs an independent replica (the single-scene
step does not shard); value = all ranks' updates / the slowest rank's time.

`--impl reference` times the reference algorithm on the host cores instead:
the reference's GLSL cannot run here (no graphics stack), so its CPU
restatement (oracle/, FP64, OpenMP over all host threads) runs on the same
workload, a bounded number of steps.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle+wave-cell updates/s on 1 GB300, batched vs plain, % of HBM roofline"
UNIT = "updates/s"
# Algorithmic bytes per unit of work (one particle or grid/wave cell per step).
# Per-step mode: integrate also hashes and counts the new positions (20 B of
# the sort's 160), so the grid pass carries the reorder's 140.
BYTES_PER_PARTICLE = {"grid": 140, "rho_pres": 24, "force": 64, "integrate": 100 + 20}
BYTES_PER_GRID_CELL = {"grid": 28}
# The neighbour passes' second bound: algorithmic FP32 flops per particle of
# the 27-cell search (216 candidates x 7 flop for the distance test, plus
# ~33 hits x 10 for the density or x 40 for the pressure/viscosity pair).
FLOP_PER_PARTICLE = {"rho_pres": 216 * 7 + 33 * 10, "force": 216 * 7 + 33 * 40}
# FP32 non-tensor peak: 152 SMs x 128 lanes x 2 flop (FMA) x the maximum SM clock
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


def _fp32_gemm_tflops(dev) -> float | None:
    """FP32 (non-tensor) throughput of a cuBLAS SGEMM on this GPU with TF32
    off: the measured ceiling the neighbour passes' FP32 fraction is quoted
    against, as the bf16 peak is a measured cuBLAS GEMM.  None if the GEMM
    runs above the FMA pipes' nominal rate (a library emulating FP32 on the
    tensor cores would)."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        n = 8192
        a = torch.randn(n, n, device=dev)
        b = torch.randn(n, n, device=dev)
        c = torch.empty(n, n, device=dev)
        for _ in range(3):
            torch.mm(a, b, out=c)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(10):
            torch.mm(a, b, out=c)
        e1.record()
        torch.cuda.synchronize()
        tflops = 2.0 * n ** 3 / (e0.elapsed_time(e1) / 10 * 1e-3) / 1e12
        del a, b, c
        return tflops if tflops <= 1.05 * FP32_PEAK_TFLOPS else None
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
BYTES_PER_WAVE_CELL = {"wave": 20}
FALLBACK_HBM_GBS = 6800.0


def _peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def _profiled_traffic() -> dict:
    """Per-launch DRAM bytes per pass from the committed ncu summaries."""
    out = {}
    for f in sorted((ROOT / "profiles").glob("*.md")):
        for m in re.finditer(r"^traffic_per_launch\s+(\w+)\s+(\d+)\s*$", f.read_text(), re.M):
            out[m.group(1)] = int(m.group(2))
    return out


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"cwa_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def lines(self) -> int:
        try:
            self.fh.flush()
            return len(self.path.read_text().splitlines())
        except Exception:
            return 99

    def summary(self) -> dict:
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(k)
        self.path.unlink(missing_ok=True)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# The CPU legs time the oracle on its own fastest sort grid (z cells of h/2;
# measured per step on 8 cores: 0.47 / 0.45 / 0.57 s for z cells of h, h/2,
# h/4), which need not be the GPU's.
CPU_ZSUB = 2


def _cpu_leg(workload, max_seconds: float, min_steps: int = 1):
    """Time the oracle (FP64 CPU restatement) on the workload's first scene."""
    from oracle import oracle as orc
    sc = workload.scenes[0]
    d = sc.desc
    p16 = orc.to_f64(sc.particles.view(np.float32).reshape(-1, 16))
    un = sc.wave.astype(np.float64)
    unm1 = un.copy()
    orc.step(d, p16, un, unm1, 1)  # warm-up (page-in, thread pool)
    steps, t0 = 0, time.perf_counter()
    while steps < min_steps or (time.perf_counter() - t0) < max_seconds * 0.5:
        orc.step(d, p16, un, unm1, 1)
        steps += 1
        if time.perf_counter() - t0 > max_seconds:
            break
    dt = time.perf_counter() - t0
    units = (d.n_particles + d.wave_nx * d.wave_nz) * steps
    return units / dt, steps, dt, orc.threads()


def run_reference(args) -> None:
    ws, rank, _ = _dist()
    if rank != 0:
        return
    from coupledwateranimation_gb300 import scenes
    wl = scenes.with_zsub(scenes.CONFIGS[args.config](), CPU_ZSUB)
    budget = float(os.environ.get("CWA_REF_SECONDS", "120"))
    value, steps, secs, cores = _cpu_leg(wl, budget, min_steps=1)
    d = wl.scenes[0].desc
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs / steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded dam-break + Gaussian bumps)",
        "config": {"workload": wl.name, "particles": d.n_particles, "wave": f"{d.wave_nx}x{d.wave_nz}"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{steps} full steps of the workload ({secs:.1f} s; sort grid z cells "
                                   f"of h/{CPU_ZSUB}, the oracle's fastest) on the FP64 OpenMP "
                                   f"restatement of the reference shaders; the GLSL itself cannot run "
                                   f"(no graphics stack)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def batched_vs_plain(args, torch, ws: int = 1, rank: int = 0, local: int = 0, config: int = 3) -> dict:
    """A batched workload (256 small scenes, or 64 large ones) stepped as one
    batched sim (one launch per pass over all scenes, CUDA graph) and as
    single-scene sims run one at a time (each its own graph).  Host
    wall-clock around the GPU work, with a synchronise at the end of every
    scene's steps in the plain leg.  Under N ranks each rank steps its shard
    of the scenes (greedy by device footprint); times are the max over
    ranks, units the sum."""
    from coupledwateranimation_gb300 import Sim, scenes, shard
    full = scenes.with_zsub(scenes.CONFIGS[config](), args.zsub)
    _, mine = shard.shard_scenes(full, rank, ws)
    wl = scenes.Workload(full.name, mine, full.steps)
    steps = max(3, min(args.steps, 10))
    dev = f"cuda:{local}"
    n_units = shard.sum_over_ranks(wl.n_particles + wl.n_wave_cells, dev)
    alg_bytes = shard.sum_over_ranks(sum(
        sum(BYTES_PER_PARTICLE.values()) * s.desc.n_particles
        + sum(BYTES_PER_GRID_CELL.values()) * shard.grid_cells(s.desc)
        + sum(BYTES_PER_WAVE_CELL.values()) * s.desc.wave_nx * s.desc.wave_nz for s in wl.scenes), dev)
    with Sim([s.desc for s in wl.scenes], precision=args.precision, use_graph=True, device=local) as sim:
        for k, s in enumerate(wl.scenes):
            sim.upload_particles(k, s.particles)
            sim.upload_wave(k, s.wave, s.wave)
        if not args.no_tune:
            sim.autotune(trial_steps=2)
        sim.step(3)
        sim.synchronize()
        t0 = time.perf_counter()
        sim.step(steps)
        sim.synchronize()
        t_batched = shard.max_over_ranks(time.perf_counter() - t0, dev)
        launches = sim.launch_count
    plain = []
    try:
        for s in wl.scenes:
            p = Sim(s.desc, precision=args.precision, use_graph=True, device=local)
            p.upload_particles(0, s.particles)
            p.upload_wave(0, s.wave, s.wave)
            p.step(3)
            p.synchronize()
            plain.append(p)
        t0 = time.perf_counter()
        for p in plain:
            p.step(steps)
            p.synchronize()
        t_plain = shard.max_over_ranks(time.perf_counter() - t0, dev)
    finally:
        for p in plain:
            p.close()
    return {"workload": wl.name, "scenes": len(full.scenes), "particles": full.n_particles,
            "wave_cells": full.n_wave_cells, "steps": steps, "ranks": ws,
            "scenes_per_rank_max": int(shard.max_over_ranks(len(wl.scenes), dev)),
            "batched_updates_per_s": n_units * steps / t_batched,
            "plain_updates_per_s": n_units * steps / t_plain,
            "speedup": t_plain / t_batched,
            "batched_algorithmic_gbs": alg_bytes * steps / t_batched / 1e9,
            "batched_ms_per_step": t_batched / steps * 1e3, "plain_ms_per_step": t_plain / steps * 1e3}


def run_gpu(args) -> None:
    import torch
    import torch.distributed as dist

    import coupledwateranimation_gb300 as cwa
    from coupledwateranimation_gb300 import PARTICLE_DTYPE, Sim, scenes

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    wl = scenes.with_zsub(scenes.CONFIGS[args.config](), args.zsub)
    sims = []
    sim = Sim([s.desc for s in wl.scenes], precision=args.precision, use_graph=True, device=local)
    for k, s in enumerate(wl.scenes):
        sim.upload_particles(k, s.particles)
        sim.upload_wave(k, s.wave, s.wave)
    view = sim.device_view(0)
    stream = torch.cuda.ExternalStream(view.stream, device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    n_units = wl.n_particles + wl.n_wave_cells

    tune = None
    if not args.no_tune:  # pick the kernel variants on this workload (state restored)
        tune = sim.autotune(trial_steps=4)
    clk = ClockSampler(local).__enter__()  # samples across warm-up, timed steps, profile and e2e
    # warm-up (graph capture happens here), then a checkpoint: the GPU is kept
    # loaded until the clock sampler is logging (at most ~5 s), and the timed
    # and profiled windows both restart from the checkpoint, so they cover the
    # same steps (warmup + 1 .. warmup + steps) of the run on every call
    sim.step(args.warmup)
    sim.synchronize()
    ckpt_fd, ckpt = tempfile.mkstemp(prefix=f"cwa_bench_r{rank}_", suffix=".ckpt")
    os.close(ckpt_fd)
    sim.save(ckpt)
    t_w = time.perf_counter()
    while clk.lines() < 3 and time.perf_counter() - t_w < 5.0:
        sim.step(20)
        sim.synchronize()

    def rewind():
        """Back to the checkpoint, then one untimed step (it hashes the
        loaded positions and replays the step graph of that phase)."""
        sim.load(ckpt)
        sim.step(1)
        sim.synchronize()

    rewind()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = sim.launch_count
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.fill_(k & 0xFF)
            starts[k].record(stream)
            sim.step(1)
            ends[k].record(stream)
    torch.cuda.synchronize()
    launches = sim.launch_count - l0
    sim.synchronize()
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    if ws > 1:
        t = torch.tensor([ms], device=f"cuda:{local}", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    value = n_units * ws * args.steps / (ms * 1e-3)

    # per-pass profile over the first steps of the same window (CUDA events
    # on the sim's stream, eager launches)
    rewind()
    os.unlink(ckpt)
    sim.set_profiling(True)
    acc = {p: 0.0 for p in cwa.PASSES}
    prof_steps = max(3, min(args.steps, 10))
    with torch.cuda.stream(stream):
        for k in range(prof_steps):
            flush.fill_(k & 0xFF)
            sim.step(1)
            for p, v in sim.pass_times().items():
                acc[p] += v
    sim.set_profiling(False)
    pass_ms = {p: v / prof_steps for p, v in acc.items()}
    top = max(pass_ms, key=pass_ms.get)
    n_p, n_c, n_w = wl.n_particles, sum(int(np.prod(sim.grid_dims(k))) for k in range(len(wl.scenes))), \
        wl.n_wave_cells
    alg = {p: BYTES_PER_PARTICLE.get(p, 0) * n_p + BYTES_PER_GRID_CELL.get(p, 0) * n_c
           + BYTES_PER_WAVE_CELL.get(p, 0) * n_w for p in cwa.PASSES}
    peak, peak_kind = _peaks()
    achieved = alg[top] / (pass_ms[top] * 1e-3) / 1e9
    fp32_achieved = (FLOP_PER_PARTICLE[top] * n_p / (pass_ms[top] * 1e-3) / 1e12
                     if top in FLOP_PER_PARTICLE else None)
    traffic = _profiled_traffic().get(top)

    # end-to-end through the C ABI with pinned host buffers
    e2e_steps = max(3, min(args.steps, 10))
    pin = []
    for s in wl.scenes:
        hp = torch.empty(s.desc.n_particles * 64, dtype=torch.uint8, pin_memory=True)
        hp.numpy()[:] = s.particles.view(np.uint8)
        hu = torch.empty((s.desc.wave_nz, s.desc.wave_nx), dtype=torch.float32, pin_memory=True)
        hu.numpy()[:] = s.wave
        hu2 = hu.clone().pin_memory()
        pin.append((hp, hu, hu2))
    h2d = sum(hp.numel() + hu.numel() * 8 for hp, hu, _ in pin)
    d2h = sum(hp.numel() + hu.numel() * 4 for hp, hu, _ in pin)
    lib = cwa.load()
    import ctypes as C
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for k, (hp, hu, hu2) in enumerate(pin):
            cwa._abi.check(lib.cwa_upload_particles(sim.handle, k, C.c_void_p(hp.data_ptr()),
                                                    wl.scenes[k].desc.n_particles), "upload")
            cwa._abi.check(lib.cwa_upload_wave(sim.handle, k, C.c_void_p(hu.data_ptr()),
                                               C.c_void_p(hu2.data_ptr()), hu.shape[1], hu.shape[0]),
                           "upload_wave")
        sim.step(1)
        for k, (hp, hu, hu2) in enumerate(pin):
            cwa._abi.check(lib.cwa_download_particles(sim.handle, k, C.c_void_p(hp.data_ptr()),
                                                      wl.scenes[k].desc.n_particles), "download")
            cwa._abi.check(lib.cwa_download_wave(sim.handle, k, C.c_void_p(hu.data_ptr()), None,
                                                 hu.shape[1], hu.shape[0]), "download_wave")
    e2e_s = time.perf_counter() - t0
    if ws > 1:
        t = torch.tensor([e2e_s], device=f"cuda:{local}", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = n_units * ws * e2e_steps / e2e_s
    clk.__exit__(None, None, None)
    # outside the clock sampler's window: the GEMM draws more power than the step
    fp32_peak = _fp32_gemm_tflops(f"cuda:{local}") if rank == 0 else None
    fp32_peak_kind = "measured (cuBLAS FP32 GEMM, TF32 off)" if fp32_peak else "nominal"
    fp32_peak = fp32_peak or FP32_PEAK_TFLOPS

    batched = None
    if not args.no_batched:
        batched = batched_vs_plain(args, torch, ws, rank, local)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu_wl = scenes.with_zsub(scenes.CONFIGS[args.config](), CPU_ZSUB)
        v, steps, secs, cores = _cpu_leg(cpu_wl, float(os.environ.get("CWA_CPU_SECONDS", "20")))
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{steps} full step(s) of the same workload ({secs:.1f} s; sort grid z cells "
                         f"of h/{CPU_ZSUB}, the oracle's fastest), FP64 OpenMP restatement of the "
                         f"reference shaders (oracle/)"}
    sim.close()
    del sims
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded dam-break + Gaussian bumps)",
            "config": {"workload": wl.name, "particles": wl.n_particles, "wave_cells": wl.n_wave_cells,
                       "grid_cells": n_c, "precision": ["fp32", "fp32-compensated", "fp64"][args.precision],
                       "grid_cell": f"h x h x h/{args.zsub}",
                       "l2": "flushed before every step (256 MiB write, outside the step events)",
                       "timed_steps": [args.warmup + 2, args.warmup + args.steps + 1],
                       "parallelism": f"replicas x{ws}"},
            "roofline": {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "algorithmic_bytes_per_launch": alg[top],
                         "ms_per_launch": pass_ms[top]},
            "roofline_fp32": {"bound": "fp32", "kernel": top, "unit": "TFLOP/s",
                              "achieved": fp32_achieved, "peak": fp32_peak, "peak_kind": fp32_peak_kind,
                              "nominal_peak": FP32_PEAK_TFLOPS,
                              "frac": fp32_achieved / fp32_peak if fp32_achieved else None,
                              "flop_per_particle": FLOP_PER_PARTICLE.get(top)},
            "pass_ms": pass_ms,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": e2e_steps},
            "gpu_launches": launches,
            "autotune": None if tune is None else {"best": tune["best"], "best_ms": tune["best_ms"],
                                                  "entry_ms": tune["entry_ms"], "tried": len(tune["tried"])},
            "clocks": clk.summary(),
        }
        if cpu:
            line["cpu_baseline"] = cpu
        if batched:
            line["batched_vs_plain"] = batched
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def run_profile(args) -> None:
    """Plain eager steps of the workload for ncu captures: no timing, no L2
    flush, each kernel a separate launch (the launch order of one step is
    hash, scan, list insert, reorder, rho_pres, force, integrate, wave)."""
    from coupledwateranimation_gb300 import Sim, scenes
    wl = scenes.with_zsub(scenes.CONFIGS[args.config](), args.zsub)
    with Sim([s.desc for s in wl.scenes], precision=args.precision, use_graph=False) as sim:
        for k, s in enumerate(wl.scenes):
            sim.upload_particles(k, s.particles)
            sim.upload_wave(k, s.wave, s.wave)
        sim.step(args.warmup + args.steps)
        sim.synchronize()
        print(json.dumps({"mode": "profile", "workload": wl.name, "steps": args.warmup + args.steps,
                          "launches": sim.launch_count}))


def run_batched(args) -> None:
    """`--mode batched`: the batched-vs-plain comparison alone for --config 3
    (256 small scenes) or 4 (64 large scenes), one JSON line."""
    import torch
    import torch.distributed as dist

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    cfg = args.config if args.config in (3, 4) else 3
    r = batched_vs_plain(args, torch, ws, rank, local, cfg)
    if rank == 0:
        peak, kind = _peaks()
        r["batched_hbm_frac"] = r["batched_algorithmic_gbs"] / peak
        r["peak_gbs"] = peak
        print(json.dumps({"mode": "batched", **r}), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def _synthetic_cube_map(size: int, seed: int = 12345) -> np.ndarray:
    """Six size x size RGBA8 faces: a seeded base colour per face plus
    smooth ramps along both texel axes."""
    rng = np.random.default_rng(seed)
    base = rng.integers(40, 200, (6, 1, 1, 3))
    ramp = np.linspace(0, 40, size)[None, :, None, None] + np.linspace(0, 25, size)[None, None, :, None]
    faces = np.empty((6, size, size, 4), np.uint8)
    faces[..., :3] = np.clip(base + ramp, 0, 255).astype(np.uint8)
    faces[..., 3] = 255
    return faces


def run_render(args) -> None:
    """`--mode render`: one headless frame (cwa_render, the reference's
    display()) of the workload's first scene after --warmup steps, at
    --width x --height with the reference's startup view; host wall-clock of
    the synchronous call (best of --steps).  --png writes the last frame.
    --skybox N sets a synthetic N x N cube map (smooth colour ramps, seeded)
    and draws it, so every fragment samples the cube map twice, as the
    reference's shaders do with its LoadCubemap textures."""
    from coupledwateranimation_gb300 import Sim, images, scenes
    from coupledwateranimation_gb300.sim import render_defaults
    wl = scenes.with_zsub(scenes.CONFIGS[args.config](), args.zsub)
    sc = wl.scenes[0]
    with Sim(sc.desc, precision=args.precision) as sim:
        sim.upload_particles(0, sc.particles)
        sim.upload_wave(0, sc.wave, sc.wave)
        sim.step(args.warmup)
        cam, prm = render_defaults(args.width, args.height)
        if args.skybox > 0:
            sim.set_skybox(_synthetic_cube_map(args.skybox))
            prm.draw_skybox = 1
        img = sim.render(0, camera=cam, params=prm)  # warm-up
        best = None
        for _ in range(max(1, args.steps)):
            t0 = time.perf_counter()
            img = sim.render(0, camera=cam, params=prm)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
    if args.png:
        with open(args.png, "wb") as f:
            f.write(images.encode_png(images.gl_rows(img)))
    print(json.dumps({"mode": "render", "workload": wl.name, "particles": sc.desc.n_particles,
                      "image": f"{args.width}x{args.height}", "surface_res": prm.surface_res,
                      "skybox": args.skybox,
                      "ms_per_frame": best * 1e3, "frames_per_s": 1.0 / best,
                      "lit_pixels": int((img[..., :3] != 0).any(axis=2).sum())}), flush=True)


def run_sph2d(args) -> None:
    """`--mode sph2d`: the 2D solver family (SphWave2D's scene: 4096 particles,
    32 x 32 grid, 128 wave cells), frames per second on the GPU (CUDA-graph
    frames, host clock around a synchronised batch) and of the CPU
    restatement on the host cores (the same passes, bounded sample)."""
    import torch  # noqa: F401 (CUDA context first, as the other modes)

    from coupledwateranimation_gb300 import _abi
    from coupledwateranimation_gb300.sim2d import WAVE2D_1D, WAVE2D_SHALLOW, Sim2D, defaults2d
    wave1d = args.wave_kind == "wave1d"
    p = defaults2d(WAVE2D_1D if wave1d else WAVE2D_SHALLOW)
    frames = max(10, args.steps)
    with Sim2D(p) as sim:
        sim.splash()
        sim.step(max(3, args.warmup))
        sim.synchronize()
        t0 = time.perf_counter()
        sim.step(frames)
        sim.synchronize()
        gpu_s = (time.perf_counter() - t0) / frames
        parts = sim.download_particles()
        wave = sim.download_wave()
    out = {"mode": "sph2d", "wave_kind": args.wave_kind, "particles": p.n_particles, "wave_cells": p.wave_cells,
           "sph_substeps": p.sph_substeps, "wave_substeps": p.wave_substeps, "frames": frames,
           "gpu_ms_per_frame": gpu_s * 1e3,
           "gpu_frames_per_s": 1.0 / gpu_s, "gpu_particle_substeps_per_s": p.n_particles * p.sph_substeps / gpu_s}
    if not args.no_cpu:
        from oracle import oracle as orc
        cpu_frames, t0 = 0, time.perf_counter()
        older = wave.copy()
        while cpu_frames < 3 or time.perf_counter() - t0 < 5.0:
            for _ in range(p.sph_substeps):
                parts = orc.force_2d(p, orc.density_2d(p, parts, wave), wave)
            for _ in range(p.wave_substeps):
                if wave1d:
                    wave, older = orc.wave1d_iter_2d_f32(p, wave, older), wave
                else:
                    a = orc.wave_iter_2d_f32(p, wave, 0)
                    wave = orc.wave_iter_2d_f32(p, a, 1, out_prev=wave)
            cpu_frames += 1
        cpu_s = (time.perf_counter() - t0) / cpu_frames
        out["cpu_baseline"] = {"ms_per_frame": cpu_s * 1e3, "cores": orc.threads(), "kind": "port",
                               "sample": f"{cpu_frames} frames of the FP64/float32 restatement (oracle/)"}
        out["gpu_vs_cpu"] = cpu_s / gpu_s
    assert _abi.PARTICLE2D_DTYPE.itemsize == 48
    print(json.dumps(out), flush=True)


def run_pbd(args) -> None:
    """`--mode pbd`: the PBD box demo (4096 boxes, 16^3 grid) and, with
    --boxes, larger piles; frames per second on the GPU (CUDA-graph frames)
    and of the float32 CPU restatement on the host (bounded sample)."""
    import torch  # noqa: F401 (CUDA context first, as the other modes)

    from coupledwateranimation_gb300.pbd import PbdSim, make_boxes, pbd_defaults
    p = pbd_defaults()
    if args.boxes:
        p.n_boxes = args.boxes
        p.max_contacts = 256  # the demo's initial block gets denser with the count
    boxes = make_boxes(p, 12345)
    frames = max(10, args.steps)
    with PbdSim(p) as sim:
        sim.upload(boxes)
        sim.step(max(3, args.warmup))
        sim.download()
        t0 = time.perf_counter()
        sim.step(frames)
        state = sim.download()
        gpu_s = (time.perf_counter() - t0) / frames
        pairs = sim.pair_count()
    out = {"mode": "pbd", "boxes": p.n_boxes, "frames": frames, "contacts_last_frame": pairs,
           "gpu_ms_per_frame": gpu_s * 1e3, "gpu_box_updates_per_s": p.n_boxes / gpu_s}
    if not args.no_cpu:
        from oracle import oracle as orc
        cpu_frames, t0 = 0, time.perf_counter()
        while cpu_frames < 2 or time.perf_counter() - t0 < 5.0:
            state = orc.pbd_step(p, state, 1)
            cpu_frames += 1
        cpu_s = (time.perf_counter() - t0) / cpu_frames
        out["cpu_baseline"] = {"ms_per_frame": cpu_s * 1e3, "cores": 1, "kind": "port",
                               "sample": f"{cpu_frames} frames of the float32 restatement (oracle/), one thread"}
        out["gpu_vs_cpu"] = cpu_s / gpu_s
    print(json.dumps(out), flush=True)


def run_wave(args) -> None:
    """The wave module stepped alone (no particle passes) on an nx x nz field:
    `--steps` single wave passes against cwa_wave_advance over the same steps
    with each blocked variant (128 x H boxes, K steps per launch, TMA-loaded
    tiles) and the wave tuner's pick; CUDA events on the sim's stream, fields
    larger than L2 unless --wave-n is small.  Prints one JSON line."""
    import torch

    from coupledwateranimation_gb300 import Sim, scenes
    from coupledwateranimation_gb300._abi import WAVE_BLOCKS
    n = args.wave_n
    d = scenes.reference().desc  # the reference's wave module: no deposits, splash init
    d.n_particles = 0
    d.wave_nx = d.wave_nz = n
    steps = max(8, args.steps // 8 * 8)
    out = {"mode": "wave", "field": f"{n}x{n}", "steps": steps}

    def timed(sim, fn):
        stream = torch.cuda.ExternalStream(sim.device_view(0).stream)
        fn()  # warm-up
        sim.synchronize()
        best = None
        for _ in range(max(3, args.warmup)):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            with torch.cuda.stream(stream):
                e0.record(stream)
                fn()
                e1.record(stream)
            sim.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        cells = n * n * steps
        return {"us_per_step": best / steps * 1e3, "cell_updates_per_s": cells / (best * 1e-3),
                "effective_gbs_at_12B": 12 * cells / (best * 1e-3) / 1e9}

    with Sim(d, use_graph=False) as sim:
        sim.wave_reinit(0)
        out["single"] = timed(sim, lambda: [sim.wave() for _ in range(steps)])
        tune = sim.autotune_wave(steps)
        out["tuner"] = {"pick": tune["best_name"], "ms_per_step": tune["ms_per_step"]}
    for v, name in enumerate(WAVE_BLOCKS):
        with Sim(d, use_graph=False, wave_block=v) as sim:
            sim.wave_reinit(0)
            out[f"blocked_{name}"] = timed(sim, lambda: sim.wave_advance(steps))
    out["blocked"] = out[f"blocked_{tune['best_name']}"]
    out["speedup"] = out["single"]["us_per_step"] / out["blocked"]["us_per_step"]
    print(json.dumps(out), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="bench",
                    choices=["bench", "profile", "wave", "batched", "render", "sph2d", "pbd"])
    ap.add_argument("--boxes", type=int, default=0, help="--mode pbd: number of boxes (default 4096)")
    ap.add_argument("--width", type=int, default=1920, help="image width for --mode render")
    ap.add_argument("--height", type=int, default=1080, help="image height for --mode render")
    ap.add_argument("--png", default="", help="--mode render: write the frame to this PNG")
    ap.add_argument("--skybox", type=int, default=0,
                    help="--mode render: draw a synthetic cube map with faces of this many texels a side")
    ap.add_argument("--wave-n", type=int, default=4096, help="field edge for --mode wave")
    ap.add_argument("--wave-kind", default="shallow", choices=["shallow", "wave1d"],
                    help="--mode sph2d: the 1D field the SPH samples")
    ap.add_argument("--config", type=int, default=1, choices=[0, 1, 2, 3, 4])
    ap.add_argument("--precision", type=int, default=1, choices=[0, 1, 2])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--zsub", type=int, default=4, help="z sub-cells per h of the sort grid")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.mode == "profile":
        run_profile(args)
    elif args.mode == "wave":
        run_wave(args)
    elif args.mode == "batched":
        run_batched(args)
    elif args.mode == "render":
        run_render(args)
    elif args.mode == "sph2d":
        run_sph2d(args)
    elif args.mode == "pbd":
        run_pbd(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
