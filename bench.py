"""Benchmark of the coupled SPH + wave step on GB300.

Metric: particle + wave-cell updates per second (one update = one particle
or one wave cell advanced one step).  Workload: the 1,048,576-particle
dam-break (128x64x128 lattice, s = 0.0075, h = 2s) coupled to a 1024^2
height field over its stated 500 steps, float32 with cascaded two-sum
neighbour sums, synthetic seeded inputs.  Each timed step is one full
cwa_step (grid sort -> rho_pres -> force -> integrate + coupling -> wave)
with the state resident in HBM; L2 is flushed (256 MiB write on the sim's
stream) before every timed step, outside its CUDA events.  After --warmup
untimed steps the run continues to the workload's last step, and exactly
--steps of those steps, evenly spaced from warmup + 1 to the last, are
timed, so the figure covers the early dam-break, the collapse and the late
sloshing state alike (config.timed_steps lists them).

`e2e` runs the same step through the public C ABI with host buffers: the
host owns the state, so each step uploads the particle records and both
wave fields from pinned host memory, steps, and downloads the records and
both wave fields, which the next step uploads.

`--gpus N` without torchrun re-launches itself under torch.distributed.run
with N ranks; every rank runs an independent replica (the single-scene step
does not shard) and value = all ranks' updates / the slowest rank's time.

`--impl reference` times the reference algorithm on the host cores instead:
the reference's GLSL cannot run through OpenGL here (no graphics stack), and
its shaders compiled for the CPU exist only beside the reference checkout and
loop over a fixed 20,480 particles, so its CPU restatement (oracle/, FP64,
OpenMP over all host threads; pinned to those shaders by
tests/test_ref_shaders.py), with inputs from the oracle's own generators,
runs --warmup untimed and exactly --steps timed steps of the same workload.
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
WORKLOAD_NAMES = {0: "c0: 32^3 particles s=0.02, 256^2 wave",
                  1: "c1: 1,048,576 particles (128x64x128, s=0.0075), 1024^2 wave",
                  2: "c2: 256x128x128 particles s=0.004, 2048^2 wave",
                  3: "c3: 256 batched small scenes", 4: "c4: 64 batched large scenes"}
WORKLOAD_STEPS = {0: 200, 1: 500, 2: 100, 3: 200, 4: 100}
PRECISION_NAMES = ["fp32", "fp32 with cascaded two-sum neighbour sums", "fp64"]
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


def _free_port() -> int:
    import socket
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _launch_ranks(n: int) -> int:
    """Re-runs this command under torch.distributed.run with n ranks on this
    node (rendezvous on 127.0.0.1); returns the launcher's exit code."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), str(Path(__file__).resolve())]
    return subprocess.call(cmd + sys.argv[1:])


# The CPU legs time the oracle on its own fastest sort grid (z cells of h/2;
# measured per step on 8 cores: 0.47 / 0.45 / 0.57 s for z cells of h, h/2,
# h/4), which need not be the GPU's.
CPU_ZSUB = 2


def _oracle_workload(config: int):
    """The workload built by the oracle's own generators (no library code)."""
    from oracle import workloads
    return workloads.with_zsub(workloads.CONFIGS[config](), CPU_ZSUB)


def _cpu_steps(wl, warmup: int, steps: int | None, max_seconds: float, timed: list[int] | None = None):
    """Times the oracle (FP64 CPU restatement) on the workload's first scene
    from its initial state.  timed: the step numbers (1-based) to time, the
    others run untimed up to the last of them.  Otherwise `warmup` untimed
    steps, then exactly `steps` timed steps, or (steps None) as many as fit
    in about max_seconds.  Returns (updates/s, timed steps, seconds, threads)."""
    from oracle import oracle as orc
    orc.set_threads(os.cpu_count() or 1)  # every host thread (torchrun sets OMP_NUM_THREADS=1 per rank)
    sc = wl.scenes[0]
    d = sc.desc
    p16 = orc.to_f64(sc.particles)
    un = sc.wave.astype(np.float64)
    unm1 = un.copy()
    if timed is not None:
        want, n, dt = set(timed), 0, 0.0
        for k in range(1, max(timed) + 1):
            if k in want:
                t0 = time.perf_counter()
                orc.step(d, p16, un, unm1, 1)
                dt += time.perf_counter() - t0
                n += 1
            else:
                orc.step(d, p16, un, unm1, 1)
    else:
        orc.step(d, p16, un, unm1, max(1, warmup))  # untimed (page-in, thread pool)
        n, t0 = 0, time.perf_counter()
        while True:
            orc.step(d, p16, un, unm1, 1)
            n += 1
            if steps is not None:
                if n >= steps:
                    break
            elif time.perf_counter() - t0 > max_seconds * 0.5:
                break
        dt = time.perf_counter() - t0
    units = (d.n_particles + d.wave_nx * d.wave_nz) * n
    return units / dt, n, dt, orc.threads()


def _config(args, n_particles: int, n_wave: int, grid_cells: int, timed: list[int], ws: int) -> dict:
    """The bench line's `config`: the same dict on both arms."""
    return {"workload": WORKLOAD_NAMES.get(args.config, str(args.config)), "particles": n_particles,
            "wave_cells": n_wave, "grid_cells": grid_cells, "workload_steps": WORKLOAD_STEPS[args.config],
            "precision": PRECISION_NAMES[args.precision], "grid_cell": f"h x h x h/{args.zsub}",
            "l2": "flushed before every timed step (256 MiB write, outside the step events)",
            "timed_steps": timed, "parallelism": f"replicas x{ws}"}


def _timed_steps(warmup: int, k: int, last: int) -> list[int]:
    """k step numbers evenly spaced over warmup + 1 .. last (1-based)."""
    first = warmup + 1
    last = max(last, first + k - 1)
    if k == 1:
        return [last]
    return sorted({first + round(i * (last - first) / (k - 1)) for i in range(k)})


def run_reference(args) -> None:
    """The reference arm: the same workload, the same warm-up and the same
    timed step numbers as the GPU arm, on the FP64 CPU restatement."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    wl = _oracle_workload(args.config)
    timed = _timed_steps(args.warmup, args.steps, max(wl.steps, args.warmup + args.steps))
    value, steps, secs, cores = _cpu_steps(wl, args.warmup, None, 0.0, timed=timed)
    d = wl.scenes[0].desc
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": steps, "warmup": args.warmup, "ms_per_step": secs / steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded dam-break + Gaussian bumps)",
        "config": _config(args, wl.n_particles, wl.n_wave_cells, orc_grid_cells(d, args.zsub), timed, ws),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"the {steps} timed steps of the workload's run (the GPU arm's step numbers; "
                                   f"{secs:.1f} s timed; sort grid z cells of h/{CPU_ZSUB}, the oracle's "
                                   f"fastest) on the FP64 OpenMP restatement of the reference shaders, inputs "
                                   f"from the oracle's own generators (the restatement is pinned to the "
                                   f"reference's shaders compiled for the CPU; those run only beside the "
                                   f"reference checkout, over a fixed 20,480 particles)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def orc_grid_cells(desc, zsub: int) -> int:
    """Cells of the scene's sort grid with z cells of h / zsub (oracle's count)."""
    from oracle import oracle as orc
    d = type(desc).from_buffer_copy(desc)
    d.cell_size_z = d.cell_size / zsub
    return int(np.prod(orc.grid_dims(d)))


def batched_vs_plain(args, torch, ws: int = 1, rank: int = 0, local: int = 0, config: int = 3,
                     steps: int | None = None) -> dict:
    """A batched workload (256 small scenes, or 64 large ones) stepped as one
    batched sim (one launch per pass over all scenes, CUDA graph; the
    neighbour passes once with one CTA a tile and once as persistent CTAs fed
    by the work queue, the faster form reported) and as
    single-scene sims run one at a time (each its own graph), both over the
    workload's stated step count unless `steps` is given.  Device time: CUDA
    events on each sim's stream around its steps (summed over the plain
    sims), after 3 untimed steps each.  Under N ranks each rank steps its
    shard of the scenes (greedy by device footprint); times are the max over
    ranks, units the sum."""
    from coupledwateranimation_gb300 import Sim, scenes, shard
    full = scenes.with_zsub(scenes.CONFIGS[config](), args.zsub)
    _, mine = shard.shard_scenes(full, rank, ws)
    wl = scenes.Workload(full.name, mine, full.steps)
    steps = steps or full.steps
    dev = f"cuda:{local}"
    n_units = shard.sum_over_ranks(wl.n_particles + wl.n_wave_cells, dev)
    alg_bytes = shard.sum_over_ranks(sum(
        sum(BYTES_PER_PARTICLE.values()) * s.desc.n_particles
        + sum(BYTES_PER_GRID_CELL.values()) * shard.grid_cells(s.desc)
        + sum(BYTES_PER_WAVE_CELL.values()) * s.desc.wave_nx * s.desc.wave_nz for s in wl.scenes), dev)

    def timed(sim, n):
        stream = torch.cuda.ExternalStream(sim.device_view(0).stream, device=torch.device("cuda", local))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.step(n)
        e1.record(stream)
        return e0, e1

    t_forms, wall_forms = {}, {}
    for form, queue in (("tile_list", 0), ("work_queue", 1)):
        with Sim([s.desc for s in wl.scenes], precision=args.precision, use_graph=True, device=local,
                 nb_queue=queue) as sim:
            for k, s in enumerate(wl.scenes):
                sim.upload_particles(k, s.particles)
                sim.upload_wave(k, s.wave, s.wave)
            if not args.no_tune:
                sim.autotune(trial_steps=2)
            sim.step(3)
            sim.synchronize()
            w0 = time.perf_counter()
            e0, e1 = timed(sim, steps)
            sim.synchronize()
            wall_forms[form] = time.perf_counter() - w0
            t_forms[form] = shard.max_over_ranks(e0.elapsed_time(e1) * 1e-3, dev)
    best = min(t_forms, key=t_forms.get)
    t_batched, wall_b = t_forms[best], wall_forms[best]
    plain, evs = [], []
    try:
        for s in wl.scenes:
            p = Sim(s.desc, precision=args.precision, use_graph=True, device=local)
            p.upload_particles(0, s.particles)
            p.upload_wave(0, s.wave, s.wave)
            p.step(3)
            p.synchronize()
            plain.append(p)
        w0 = time.perf_counter()
        for p in plain:  # one scene after another, as a caller of the plain path steps them
            evs.append(timed(p, steps))
            p.synchronize()
        wall_p = time.perf_counter() - w0
        t_plain = shard.max_over_ranks(sum(a.elapsed_time(b) for a, b in evs) * 1e-3, dev)
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
            "batched_ms_per_step": t_batched / steps * 1e3, "plain_ms_per_step": t_plain / steps * 1e3,
            "batched_form": best,
            "batched_ms_per_step_by_form": {f: t / steps * 1e3 for f, t in t_forms.items()},
            "host_wall_ms_per_step": {"batched": wall_b / steps * 1e3, "plain": wall_p / steps * 1e3}}


def run_gpu(args) -> None:
    import torch
    import torch.distributed as dist

    import coupledwateranimation_gb300 as cwa
    from coupledwateranimation_gb300 import Sim, scenes

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    wl = scenes.with_zsub(scenes.CONFIGS[args.config](), args.zsub)
    last_step = max(wl.steps, args.warmup + args.steps)
    timed_steps = _timed_steps(args.warmup, args.steps, last_step)
    sim = Sim([s.desc for s in wl.scenes], precision=args.precision, use_graph=True, device=local)
    for k, s in enumerate(wl.scenes):
        sim.upload_particles(k, s.particles)
        sim.upload_wave(k, s.wave, s.wave)
    view = sim.device_view(0)
    stream = torch.cuda.ExternalStream(view.stream, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    n_units = wl.n_particles + wl.n_wave_cells

    tune = None
    if not args.no_tune:  # pick the kernel variants on this workload (state restored)
        tune = sim.autotune(trial_steps=8)
    clk = ClockSampler(local).__enter__()  # samples across warm-up, timed steps, profile and e2e
    # warm-up (graph capture happens here), then a checkpoint: the GPU is kept
    # loaded until the clock sampler is logging (at most ~5 s), and the timed
    # run and the per-pass profile both restart from the checkpoint, so they
    # cover the same steps of the workload
    sim.step(args.warmup)
    sim.synchronize()
    ckpt_fd, ckpt = tempfile.mkstemp(prefix=f"cwa_bench_r{rank}_", suffix=".ckpt")
    os.close(ckpt_fd)
    sim.save(ckpt)
    t_w = time.perf_counter()
    while clk.lines() < 3 and time.perf_counter() - t_w < 5.0:
        sim.step(20)
        sim.synchronize()

    def run_to_end(on_timed):
        """From the checkpoint (step warmup) to the workload's last step;
        on_timed(k) brackets the k-th timed step, the rest run untimed."""
        sim.load(ckpt)
        sim.synchronize()
        want = set(timed_steps)
        k = 0
        with torch.cuda.stream(stream):
            for n in range(args.warmup + 1, last_step + 1):
                if n in want:
                    on_timed(k)
                    k += 1
                else:
                    sim.step(1)

    starts = [torch.cuda.Event(enable_timing=True) for _ in timed_steps]
    ends = [torch.cuda.Event(enable_timing=True) for _ in timed_steps]

    def one_timed(k):
        flush.fill_(k & 0xFF)
        starts[k].record(stream)
        sim.step(1)
        ends[k].record(stream)

    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = sim.launch_count
    w0 = time.perf_counter()
    run_to_end(one_timed)
    torch.cuda.synchronize()
    run_wall = time.perf_counter() - w0
    launches_run = sim.launch_count - l0
    sim.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    ms = sum(step_ms)
    if ws > 1:
        t = torch.tensor([ms], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    value = n_units * ws * len(timed_steps) / (ms * 1e-3)
    # one graph replay per step: the timed steps' share of the run's launches
    launches = launches_run * len(timed_steps) // max(1, last_step - args.warmup)
    thirds = np.array_split(np.array(step_ms), 3)
    window = {"early_ms": float(thirds[0].mean()), "mid_ms": float(thirds[1].mean()),
              "late_ms": float(thirds[2].mean()), "min_ms": min(step_ms), "max_ms": max(step_ms)}

    # per-pass profile over the same timed steps (CUDA events on the sim's
    # stream, eager launches)
    sim.set_profiling(True)
    acc = {p: 0.0 for p in cwa.PASSES}

    def one_profiled(k):
        flush.fill_(k & 0xFF)
        sim.step(1)
        for p, v in sim.pass_times().items():
            acc[p] += v

    run_to_end(one_profiled)
    sim.set_profiling(False)
    os.unlink(ckpt)
    pass_ms = {p: v / len(timed_steps) for p, v in acc.items()}
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

    # end-to-end through the C ABI with pinned host buffers (from the
    # workload's last state)
    e2e_steps = max(3, min(args.steps, 10))
    pin = []
    for s in wl.scenes:
        hp = torch.empty(s.desc.n_particles * 64, dtype=torch.uint8, pin_memory=True)
        hu = torch.empty((s.desc.wave_nz, s.desc.wave_nx), dtype=torch.float32, pin_memory=True)
        hu2 = torch.empty((s.desc.wave_nz, s.desc.wave_nx), dtype=torch.float32, pin_memory=True)
        pin.append((hp, hu, hu2))
    lib = cwa.load()
    import ctypes as C
    for k, (hp, hu, hu2) in enumerate(pin):  # the host copy of the current state
        cwa._abi.check(lib.cwa_download_particles(sim.handle, k, C.c_void_p(hp.data_ptr()),
                                                  wl.scenes[k].desc.n_particles), "download")
        cwa._abi.check(lib.cwa_download_wave(sim.handle, k, C.c_void_p(hu.data_ptr()), C.c_void_p(hu2.data_ptr()),
                                             hu.shape[1], hu.shape[0]), "download_wave")
    h2d = sum(hp.numel() + hu.numel() * 8 for hp, hu, _ in pin)
    d2h = sum(hp.numel() + hu.numel() * 8 for hp, hu, _ in pin)
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
            cwa._abi.check(lib.cwa_download_wave(sim.handle, k, C.c_void_p(hu.data_ptr()), C.c_void_p(hu2.data_ptr()),
                                                 hu.shape[1], hu.shape[0]), "download_wave")
    e2e_s = time.perf_counter() - t0
    if ws > 1:
        t = torch.tensor([e2e_s], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = n_units * ws * e2e_steps / e2e_s
    clk.__exit__(None, None, None)
    # outside the clock sampler's window: the GEMM draws more power than the step
    fp32_peak = _fp32_gemm_tflops(f"cuda:{local}") if rank == 0 else None
    fp32_peak_kind = "measured (cuBLAS FP32 GEMM, TF32 off)" if fp32_peak else "nominal"
    fp32_peak = fp32_peak or FP32_PEAK_TFLOPS
    sim.close()

    batched = []
    if not args.no_batched:
        for cfg in (3, 4):
            batched.append(batched_vs_plain(args, torch, ws, rank, local, cfg))
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        v, steps, secs, cores = _cpu_steps(_oracle_workload(args.config), 1, None,
                                           float(os.environ.get("CWA_CPU_SECONDS", "20")))
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"steps 2-{steps + 1} of the same workload ({secs:.1f} s; sort grid z cells "
                         f"of h/{CPU_ZSUB}, the oracle's fastest), FP64 OpenMP restatement of the "
                         f"reference shaders (oracle/), inputs from the oracle's own generators"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": len(timed_steps),
            "warmup": args.warmup, "ms_per_step": ms / len(timed_steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded dam-break + Gaussian bumps)",
            "config": _config(args, wl.n_particles, wl.n_wave_cells, n_c, timed_steps, ws),
            "window": window,
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
            "run": {"steps": [args.warmup + 1, last_step], "wall_s": run_wall, "launches": launches_run},
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


def run_dry(args) -> None:
    """`--dry-run`: the rank plumbing alone, on CPU (gloo): every rank joins
    the group, the timing reductions run, rank 0 prints a line with the
    rank count.  No GPU work; used to test the --gpus launcher."""
    import torch.distributed as dist

    from coupledwateranimation_gb300 import shard
    ws, rank, _ = _dist()
    if ws > 1:
        dist.init_process_group("gloo")
    slowest = shard.max_over_ranks(1.0 + rank, None)
    total = shard.sum_over_ranks(1.0, None)
    if rank == 0:
        print(json.dumps({"mode": "dry-run", "n_gpus": ws, "ranks_reporting": int(total), "slowest": slowest,
                          "config": {"parallelism": f"replicas x{ws}"}}), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def run_profile(args) -> None:
    """Plain eager steps of the workload for ncu captures: no timing, no L2
    flush, each kernel a separate launch (the launch order of one step is
    the count scan's tile totals and tile scans, list insert, reorder,
    rho_pres, force, integrate with the next step's hash and count, wave)."""
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
                parts = orc.force_2d(p, orc.density_2d(p, parts, wave), wave, grid_from=parts)
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


def run_refscene(args) -> None:
    """`--mode refscene`: the reference app's own scene (20,480 particles on
    its 64 x 5 x 64 cube, 64^2 wave, the shaders' constants,
    CoupledWaterAnimation/Main.cpp:28-35, 184-204): updates/s of the GPU step
    (CUDA events around --steps graph-launched steps after --warmup) beside
    the reference's own algorithm on the host cores, the O(N^2) all-pairs
    loops of rho_pres_comp.glsl:60-68 / force_comp.glsl:74-88 in the FP64
    restatement (bounded sample), and the same restatement on its grid."""
    import torch

    from coupledwateranimation_gb300 import Sim, scenes
    sc = scenes.reference()
    d = sc.desc
    units = d.n_particles + d.wave_nx * d.wave_nz
    with Sim(d) as sim:
        sim.upload_particles(0, sc.particles)
        sim.wave_reinit(0)
        stream = torch.cuda.ExternalStream(sim.device_view(0).stream)
        sim.step(args.warmup)
        sim.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.step(args.steps)
        e1.record(stream)
        sim.synchronize()
        gpu_ms = e0.elapsed_time(e1) / args.steps
    out = {"mode": "refscene", "particles": d.n_particles, "wave": f"{d.wave_nx}x{d.wave_nz}",
           "gpu_ms_per_step": gpu_ms, "gpu_updates_per_s": units / (gpu_ms * 1e-3)}
    if not args.no_cpu:
        from oracle import oracle as orc
        from oracle import workloads
        orc.set_threads(os.cpu_count() or 1)
        for brute, key in ((True, "cpu_all_pairs"), (False, "cpu_grid")):
            r = workloads.reference_preset()
            p16 = orc.to_f64(r.particles)
            un = r.wave.astype(np.float64)
            unm1 = un.copy()
            orc.step(r.desc, p16, un, unm1, 1, brute=brute)  # untimed
            n, t0 = 0, time.perf_counter()
            while n < 2 or time.perf_counter() - t0 < float(os.environ.get("CWA_CPU_SECONDS", "10")):
                orc.step(r.desc, p16, un, unm1, 1, brute=brute)
                n += 1
            sec = (time.perf_counter() - t0) / n
            out[key] = {"ms_per_step": sec * 1e3, "updates_per_s": units / sec, "steps": n,
                        "cores": orc.threads(), "kind": "port"}
        out["gpu_vs_cpu_all_pairs"] = out["cpu_all_pairs"]["ms_per_step"] / gpu_ms
    print(json.dumps(out), flush=True)


def run_wave_profile(args) -> None:
    """`--mode wave-profile`: a capture target for ncu.  A sim with
    wave_block = --wave-block on an --wave-n squared field of the reference
    preset (InitWave splash, no particles) calls wave_advance(8) four times;
    no timing."""
    from coupledwateranimation_gb300 import Sim, scenes
    d = scenes.reference().desc
    d.n_particles = 0
    d.wave_nx = d.wave_nz = args.wave_n
    with Sim(d, use_graph=False, wave_block=args.wave_block) as sim:
        sim.wave_reinit(0)
        for _ in range(4):
            sim.wave_advance(8)
        sim.synchronize()
    print(json.dumps({"mode": "wave-profile", "field": f"{args.wave_n}x{args.wave_n}",
                      "wave_block": args.wave_block, "advances": 4, "steps_each": 8}), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="bench",
                    choices=["bench", "profile", "wave", "wave-profile", "refscene", "batched", "render", "sph2d",
                             "pbd"])
    ap.add_argument("--wave-block", type=int, default=0, help="--mode wave-profile: CWA_WAVE_BLOCK_* variant")
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
    ap.add_argument("--dry-run", action="store_true", help="rank plumbing only, on CPU (tests the launcher)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(_launch_ranks(args.gpus))
    if args.dry_run:
        run_dry(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.mode == "profile":
        run_profile(args)
    elif args.mode == "wave":
        run_wave(args)
    elif args.mode == "wave-profile":
        run_wave_profile(args)
    elif args.mode == "refscene":
        run_refscene(args)
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
