"""Regenerate tests/golden/ref_shader_outputs.npz: outputs of the reference's
own compute shaders (CoupledWaterAnimation/rho_pres_comp.glsl,
force_comp.glsl, integrate_comp.glsl, wave_comp.glsl;
UniformGrid2D/ugrid_particles_cs.glsl, prefix_sum_cs.glsl and
uniform_grid_pbd_3D_cs.glsl; the SphWave2D family) run on the CPU, on the
seeded inputs of oracle/ref.py.

The shaders are compiled as C++ (oracle/ref_shaders/: the GLSL source with
its declarations rewritten, against a GLSL types-and-built-ins header) in
two precisions: "f32", the shaders' float arithmetic with one rounding per
operation, and "f64", the same source with float promoted to double.  The
reference's constants stay float literals in both.

Cases (every input regenerates from oracle/ref.py; its SHA-256 is stored):
  sph      20,480 particles (the reference's 64 x 5 x 64 cube, jittered) on a
           64 x 64 height field: rho_pres, then force on each precision's own
           rho_pres output; stored for every 20th particle;
  integ    512 particles spread over the box and past its walls (foam,
           walls and surface branches): integrate, all outputs, in wave
           mode 1 and in mode 0.5 (which adds the ceiling);
  evolve   EvolveWave on 64 x 64 fields (wave modes 1 and 0.5) and on a
           67 x 45 field (mode 0.5: the line source at x = 33);
  init     InitWave for modes 1, 0 and 0.5 on 64 x 64 and mode 0.5 on 67 x 45;
  image    InitFromImage of the reference's splash texture on a 32 x 64 field;
  grid     UniformGrid2D/ugrid_particles_cs.glsl COMPUTE_COUNTS, the scan
           (prefix_sum_cs.glsl dispatched as ParallelScan::Compute) and
           INSERT_PARTICLES, as UniformGridGpu2D.cpp sequences them, on 20,000
           scattered points (16 x 8 x 16 cells, points past every wall and on
           cell faces) and a jittered 24 x 20 x 24 lattice (32^3 cells): counts,
           offsets and index list;
  scan     the scan alone on the reference's ParallelScanTest vector and on
           2^10 and 2^14 values;
  s2d      the 2D family (SphWave2D): InitParticle; one SphUgrid substep
           (the grid of uniform_grid_sph_cs.glsl, then the density and force
           modes of SphWaveKoschier2D_grid_cs.glsl on that grid) of a jittered
           lattice with particles past the grid and below the floor, stored
           for every 4th particle; Shallow1D InitWave, Splash, predictor and
           corrector; Wave1D InitWave (modes 0 and 1) and one iteration.  The
           bit-exact ones are stored as SHA-256 of their float32 bytes;
  pbd      one frame of UniformGrid2D/uniform_grid_pbd_3D_cs.glsl (the box
           grid, PreAnimate, the collision query, PostAnimate, as
           GridTestPbdGpu3D::Animate sequences them) on the demo's 4096
           boxes: the constraint counts and colours as SHA-256, every 8th
           box's record;
  frag     particle_fs.glsl (pass 0) and wave_fs.glsl for 2000 fragments
           each: a camera, a seeded cube map and depth image, fragments over
           the window (about a fifth outside the sprite: discarded).

Usage:  python tests/golden/make_ref_shader_golden.py
        (needs the reference checkout; CWA_REFERENCE names it if it is not
        at the default place oracle/ref.py looks)
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

OUT = HERE / "ref_shader_outputs.npz"
SPH_SAMPLE = np.arange(0, 20480, 20)
WAVE_MODES = {"m1": 1.0, "m0": 0.0, "m05": 0.5}


def sha(a: np.ndarray) -> str:
    """SHA-256 of an array's bytes, every NaN as the positive quiet NaN
    (a NaN's sign and payload differ between x86, Arm and the GPU)."""
    a = np.ascontiguousarray(a).copy()
    if a.dtype.kind == "f":
        a[np.isnan(a)] = np.nan
    return hashlib.sha256(a.tobytes()).hexdigest()


def reference_desc():
    import coupledwateranimation_gb300._abi as abi
    from oracle import oracle as orc
    return orc.scene_defaults(abi.PRESET_REFERENCE_3D, 0.0, abi.SceneDesc)


def inputs() -> dict[str, np.ndarray]:
    from oracle import ref
    return ref.fixture_inputs(np.load(HERE / "init_textures.npz")["splash"])


S2D_SAMPLE = np.arange(0, 4096, 4)


def sph2d_cases(ref, x, out) -> None:
    """The 2D family (SphWave2D): bit-exact cases as SHA-256 of their float32
    bytes, the SPH passes on a sample of particles."""
    from coupledwateranimation_gb300._abi import WAVE2D_1D
    from coupledwateranimation_gb300.sim2d import defaults2d
    p = defaults2d()
    u = ref.uniforms_2d(p)
    n = p.n_particles
    z = np.zeros((p.wave_cells, 4), np.float32)
    init = ref.sph2d(ref.F32, 0, np.zeros((n, 12)), z, u).astype(np.float32)
    out["s2d_init_sha"] = np.array(sha(init))
    out["s2d_sample"] = S2D_SAMPLE
    st = x["s2d_state"].astype(np.float64)
    for prec, tag, dt in ((ref.F32, "f32", np.float32), (ref.F64, "f64", np.float64)):
        dens, force = ref.substep2d(prec, st, x["s2d_wave"], u)
        out[f"s2d_density_{tag}"] = dens[S2D_SAMPLE].astype(dt)
        out[f"s2d_force_{tag}"] = force[S2D_SAMPLE].astype(dt)
    # Shallow1D: InitWave, Splash on it, the predictor (into the buffer that
    # held the splash), the corrector (into the buffer that held the splash)
    init0 = ref.field2d(0, 0, z, None, z, u)
    splash = ref.field2d(0, 1, init0, None, init0, u)
    pred = ref.field2d(0, 2, splash, None, splash, u)
    corr = ref.field2d(0, 3, pred, None, splash, u)
    for name, a in (("init", init0), ("splash", splash), ("corr", corr)):
        out[f"s2d_shallow_{name}_sha"] = np.array(sha(a))
    out["s2d_shallow_init"], out["s2d_shallow_splash"] = init0, splash  # the GPU's inputs (expf-free steps)
    out["s2d_shallow_pred_sha"] = np.array(sha(pred[1:]))  # cell 0: see the test
    # Wave1D on the app's 1024 cells
    p1 = defaults2d(WAVE2D_1D)
    u1 = ref.uniforms_2d(p1)
    z1 = np.zeros((p1.wave_cells, 4), np.float32)
    w0 = ref.field2d(1, 0, z1, z1, z1, u1)
    w1 = ref.field2d(1, 1, w0, z1, w0, u1)
    it = ref.field2d(1, 2, w1, w0, z1, u1)
    for name, a in (("init0", w0), ("init1", w1), ("iter", it)):
        out[f"s2d_wave1d_{name}_sha"] = np.array(sha(a))
    out["s2d_wave1d_init0"], out["s2d_wave1d_init1"] = w0, w1


PBD_SAMPLE = np.arange(0, 4096, 8)


def pbd_cases(ref, x, out) -> None:
    """One frame of the PBD demo in float: the constraint counts and colours
    (the contact set) as SHA-256, every 8th box's record in full."""
    from coupledwateranimation_gb300.pbd import pbd_defaults
    q = ref.pbd_params(pbd_defaults())
    r = ref.pbd(ref.F32, x["pbd_boxes"].astype(np.float64), 1, q).astype(np.float32)
    out["pbd_counts_sha"] = np.array(sha(r[:, 29]))
    out["pbd_colors_sha"] = np.array(sha(r[:, 0:4]))
    out["pbd_sample"] = PBD_SAMPLE
    out["pbd_frame1_f32"] = r[PBD_SAMPLE]


def fragment_cases(ref, x, out) -> None:
    """particle_fs.glsl pass 0 and wave_fs.glsl, one fragment at a time."""
    inp = ref.render_inputs_struct(x)
    n = len(x["rfs_px"])
    part = np.zeros((n, 4), np.float32)
    disc = np.zeros(n, bool)
    for k in range(n):
        part[k], disc[k] = ref.particle_fragment(inp, x["rfs_pp"][k], 0.5, x["rfs_px"][k] + 0.5,
                                                 x["rfs_py"][k] + 0.5, x["rfs_pc"][k])
    part[disc] = 0.0
    up = np.array([0.0, 1.0, 0.0], np.float32)  # -normal_attrib: Surf.cpp's normals are (0, -1, 0)
    wave = np.stack([ref.wave_fragment(inp, x["rfs_pw"][k], up, float(x["rfs_v"][k])) for k in range(n)])
    out["rfs_particle"], out["rfs_discard"], out["rfs_wave"] = part, disc, wave


def main() -> None:
    from oracle import ref
    if ref.build() is None or ref.load() is None:
        sys.exit("the reference checkout is needed (set CWA_REFERENCE)")
    d = reference_desc()
    x = inputs()
    out: dict[str, np.ndarray] = {"sph_sample": SPH_SAMPLE}
    for k, v in x.items():
        out[f"sha_{k}"] = np.array(sha(v))
    u = ref.uniforms(d)
    sph64 = x["sph"].astype(np.float64)
    for prec, tag, dt in ((ref.F32, "f32", np.float32), (ref.F64, "f64", np.float64)):
        r = ref.rho_pres(prec, sph64, x["sph_wave"], u)
        f = ref.force(prec, r, x["sph_wave"], u)
        out[f"rho_{tag}"] = r[SPH_SAMPLE, 12:14].astype(dt)
        out[f"force_{tag}"] = f[SPH_SAMPLE, 8:12].astype(dt)
        out[f"integ_{tag}"] = ref.integrate(prec, x["integ"].astype(np.float64), x["sph_wave"], u).astype(dt)
        d.wave_mode = 0.5  # the line-source mode adds the ceiling (integrate_comp.glsl:170-177)
        out[f"integ_m05_{tag}"] = ref.integrate(prec, x["integ"].astype(np.float64), x["sph_wave"],
                                                ref.uniforms(d)).astype(dt)
        d.wave_mode = 1.0
    for size in ("64", "67"):
        un, unm1 = x[f"evolve{size}_un"], x[f"evolve{size}_unm1"]
        for mk, mode in WAVE_MODES.items():
            if mk == "m0" or (size == "67" and mk != "m05"):
                continue
            d.wave_mode = mode
            uw = ref.uniforms(d, mode=2)
            out[f"evolve{size}_{mk}_f32"] = ref.wave(ref.F32, un, unm1, uw).astype(np.float32)
            if size == "64":
                out[f"evolve{size}_{mk}_f64"] = ref.wave(ref.F64, un, unm1, uw)
    for size, (w, h) in (("64", (64, 64)), ("67", (67, 45))):
        z = np.zeros((h, w))
        for mk, mode in WAVE_MODES.items():
            if size == "67" and mk != "m05":
                continue
            d.wave_mode = mode
            out[f"init{size}_{mk}_f32"] = ref.wave(ref.F32, z, z, ref.uniforms(d, mode=0)).astype(np.float32)
    d.wave_mode = 1.0
    z = np.zeros((64, 32))
    out["image_f32"] = ref.wave(ref.F32, z, z, ref.uniforms(d, mode=1), init_rgba=x["image_rgba"]).astype(np.float32)
    for name, (_, lo, hi, cell, dims) in ref.GRID_CASES.items():
        counts, offsets, lst = ref.grid_build(x[name], lo, hi, (cell, cell, cell), dims)
        out[f"{name}_counts"], out[f"{name}_offsets"], out[f"{name}_list"] = counts, offsets, lst
    for name in ref.scan_inputs():
        out[f"{name}_out"] = ref.exclusive_scan(x[name])
    sph2d_cases(ref, x, out)
    pbd_cases(ref, x, out)
    fragment_cases(ref, x, out)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
