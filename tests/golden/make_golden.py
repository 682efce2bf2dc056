"""Regenerate the golden fixtures in tests/golden/.

parallel_scan_kat.json — the reference's only known-answer test: the input
vectors of ParallelScanTest (SphWave2D/ParallelScan.cpp:129 and the all-ones
variant at UniformGrid2D/ParallelScan.cpp:117), read from the reference's
source text, with the truth computed by the test's own serial rule
(SphWave2D/ParallelScan.cpp:130-137: truth[i] = sum of x[0..i-1]).

init_textures.npz — the reference's three InitFromImage textures
(CoupledWaterAnimation/init-textures/{splash,wake,breaking-wave}.png, 64x64)
decoded to RGBA8 by coupledwateranimation_gb300.images (rows top-down, as
stored in the files), so the GPU tests can run the init-from-image path on
them without the reference checkout.

oracle_regression.json — outputs of the CPU oracle on small fixed scenes
(hashes of float32 bit patterns and int arrays).  These pin the oracle
against accidental change; they are not reference outputs (those are in
ref_shader_outputs.npz, made by make_ref_shader_golden.py from the
reference's shaders compiled for the CPU).

Usage:  python tests/golden/make_golden.py [/path/to/reference]
The reference checkout is needed only for the KAT file.
"""
from __future__ import annotations

import hashlib
import json
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))


def _vectors(path: Path) -> list[list[int]]:
    out = []
    for line in path.read_text().splitlines():
        s = line.strip()
        if s.startswith("//"):
            continue
        m = re.search(r"std::vector<int>\s+x\s*=\s*\{([^}]*)\}", s)
        if m:
            out.append([int(v) for v in m.group(1).split(",")])
    return out


def make_kat(reference: Path) -> None:
    cases = []
    for rel in ("SphWave2D/ParallelScan.cpp", "UniformGrid2D/ParallelScan.cpp"):
        for x in _vectors(reference / rel):
            truth, acc = [], 0
            for v in x:
                truth.append(acc)
                acc += v
            cases.append({"source": rel, "input": x, "exclusive_scan": truth})
    (HERE / "parallel_scan_kat.json").write_text(json.dumps({"cases": cases}, indent=1) + "\n")


def make_init_textures(reference: Path) -> None:
    from coupledwateranimation_gb300 import images

    src = reference / "CoupledWaterAnimation" / "init-textures"
    arrays = {name.replace("-", "_"): images.read_png(src / f"{name}.png")
              for name in ("splash", "wake", "breaking-wave")}
    np.savez_compressed(HERE / "init_textures.npz", **arrays)


def _h(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make_oracle_regression() -> None:
    from oracle import oracle as orc
    import coupledwateranimation_gb300._abi as abi

    out = {}
    d = orc.scene_defaults(abi.PRESET_REFERENCE_3D, 0.0, abi.SceneDesc)
    cube = orc.make_reference_cube(d, d.n_particles)
    dims = orc.grid_dims(d)
    start, order, cell_of = orc.grid_build(cube[:, 0:4], list(d.box_lo), orc.cell_edges(d), dims)
    out["reference_cube"] = {"dims": dims, "cell_start_sha256": _h(start), "order_sha256": _h(order),
                             "cube_sha256": _h(cube)}
    u0 = orc.wave_init_f32(d)
    out["reference_wave_init"] = {"sha256": _h(u0), "sum": float(u0.astype(np.float64).sum())}
    p16 = orc.to_f64(cube)
    orc.rho_pres(d, p16, u0.astype(np.float64))
    out["reference_rho_pres"] = {"rho_sum": float(p16[:, 12].sum()), "p_sum": float(p16[:, 13].sum())}

    m = orc.scene_defaults(abi.PRESET_MULLER, 0.02, abi.SceneDesc)
    orc.scene_set_wave_grid(m, 256, 256)
    m.n_particles = 4096
    pm = orc.make_dam_break(m, (16, 16, 16), 0.02, 0.05, 12345, 4096)
    um = orc.make_bumps(m, 8, 12345 + 1_000_003, 256, 256)
    out["muller_dam_break"] = {"particles_sha256": _h(pm), "bumps_sha256": _h(um),
                               "deposit_shift": int(m.deposit_shift),
                               "couple_gain": float(m.couple_gain)}
    (HERE / "oracle_regression.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    # usage: make_golden.py [REFERENCE_CHECKOUT]
    # With the reference's source tree given, the scan KAT and the init
    # textures are read from it; the oracle regression needs no reference.
    if len(sys.argv) > 1:
        ref = Path(sys.argv[1])
        if not ref.is_dir():
            sys.exit(f"not a directory: {ref}")
        make_kat(ref)
        make_init_textures(ref)
    make_oracle_regression()
    print("golden fixtures written to", HERE)
