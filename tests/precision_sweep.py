"""Precision sweep of the neighbour sums (FP32, FP32 with cascaded two-sum
accumulation, FP64).

For one workload (default: the 4,194,304-particle dam-break, 256x128x128
lattice at s = 0.004 with a 2048^2 wave) this measures, per precision mode:
- the one-pass error of rho, pressure and force against the FP64 oracle on
  the same input state (taken after `--warm` coupled steps, so velocities
  and the surface are non-trivial): max per-particle relative error of rho,
  normwise relative error of p and of each force component, and the median
  per-particle relative force error;
- the time per coupled step (CUDA events on the sim's stream);
- after `--steps` coupled steps: mass (exact), kinetic / potential / wave
  energy, their relative difference to the FP64 run, and the L1 distance of
  the density histogram to the FP64 run's.

The oracle only provides the comparisons; it is not timed.  Usage (GPU required):
    python tests/precision_sweep.py [--config 2] [--steps 100] [--warm 20] [--zsub 4]
Prints one JSON line per mode and a summary line.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

MODES = (("fp32", 0), ("fp32-cascaded-two-sum", 1), ("fp64", 2))


def _records(p: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(p).view(np.float32).reshape(-1, 16).copy()


def _load(sim, wl, parts=None, waves=None) -> None:
    for k, s in enumerate(wl.scenes):
        sim.upload_particles(k, s.particles if parts is None else parts[k])
        if waves is None:
            sim.upload_wave(k, s.wave, s.wave)
        else:
            sim.upload_wave(k, waves[k][0], waves[k][1])


def sweep(config: int = 2, steps: int = 100, warm: int = 20, zsub: int = 4, workload=None) -> list[dict]:
    import torch

    from coupledwateranimation_gb300 import Sim, scenes
    from oracle import oracle as orc

    wl = workload if workload is not None else scenes.with_zsub(scenes.CONFIGS[config](), zsub)
    d = wl.scenes[0].desc
    # common input state: `warm` coupled steps of the FP64 sim
    with Sim([s.desc for s in wl.scenes], precision=2) as sim:
        _load(sim, wl)
        sim.step(warm)
        sim.synchronize()
        parts = [sim.download_particles(k) for k in range(len(wl.scenes))]
        waves = [sim.download_wave(k) for k in range(len(wl.scenes))]
    u_n = waves[0][0]
    ref = orc.to_f64(_records(parts[0]))
    t0 = time.perf_counter()
    orc.rho_pres(d, ref, u_n.astype(np.float64))
    orc.force(d, ref, u_n.astype(np.float64))
    oracle_s = time.perf_counter() - t0

    out = []
    finals = {}
    for name, prec in MODES:
        with Sim([s.desc for s in wl.scenes], precision=prec) as sim:
            _load(sim, wl, parts, waves)
            sim.grid()
            sim.rho_pres()
            sim.force()
            got = _records(sim.download_particles(0))
            rho_err = float(np.max(np.abs(got[:, 12] - ref[:, 12]) / np.abs(ref[:, 12])))
            p_err = float(np.abs(got[:, 13] - ref[:, 13]).max() / max(np.abs(ref[:, 13]).max(), 1e-300))
            f_err = [float(np.abs(got[:, 8 + c] - ref[:, 8 + c]).max() / np.abs(ref[:, 8 + c]).max())
                     for c in range(3)]
            fn = np.linalg.norm(ref[:, 8:11], axis=1)
            fe = np.linalg.norm(got[:, 8:11].astype(np.float64) - ref[:, 8:11], axis=1)
            f_med = float(np.median(fe[fn > 0] / fn[fn > 0]))
            # timed coupled steps from the initial workload state
            _load(sim, wl)
            tot0 = sim.totals(0)
            view = sim.device_view(0)
            stream = torch.cuda.ExternalStream(view.stream)
            sim.step(3)
            sim.synchronize()
            _load(sim, wl)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            with torch.cuda.stream(stream):
                e0.record(stream)
                sim.step(steps)
                e1.record(stream)
            sim.synchronize()
            ms = e0.elapsed_time(e1) / steps
            tot = sim.totals(0)
            rho_final = _records(sim.download_particles(0))[:, 12].astype(np.float64)
        finals[name] = (tot, rho_final)
        out.append({"mode": name, "rho_max_rel": rho_err, "p_normwise": p_err, "force_normwise": f_err,
                    "force_median_rel": f_med, "ms_per_step": ms, "mass_change": tot["mass"] - tot0["mass"],
                    "kinetic": tot["kinetic"], "potential": tot["potential"], "wave_energy": tot["wave_energy"]})
    ref_tot, ref_rho = finals["fp64"]
    lo, hi = np.percentile(ref_rho, [0.5, 99.5])
    bins = np.linspace(lo, hi, 101)
    h_ref = np.histogram(ref_rho, bins)[0] / ref_rho.size
    for row in out:
        tot, rho = finals[row["mode"]]
        for key in ("kinetic", "potential", "wave_energy"):
            row[f"{key}_vs_fp64"] = abs(tot[key] - ref_tot[key]) / max(abs(ref_tot[key]), 1e-300)
        row["rho_hist_l1_vs_fp64"] = float(np.abs(np.histogram(rho, bins)[0] / rho.size - h_ref).sum())
    summary = {"workload": wl.name, "particles": int(sum(s.desc.n_particles for s in wl.scenes)),
               "warm_steps": warm, "steps": steps, "oracle_seconds": oracle_s,
               "oracle_threads": orc.threads()}
    return out + [summary]


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, default=2)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warm", type=int, default=20)
    ap.add_argument("--zsub", type=int, default=4)
    a = ap.parse_args()
    for row in sweep(a.config, a.steps, a.warm, a.zsub):
        print(json.dumps(row), flush=True)


if __name__ == "__main__":
    main()
