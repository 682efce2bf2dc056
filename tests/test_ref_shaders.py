"""The oracle against the reference's own compute shaders.

tests/golden/ref_shader_outputs.npz holds outputs of
CoupledWaterAnimation/{rho_pres,force,integrate,wave}_comp.glsl and of the
grid and scan shaders UniformGrid2D/{ugrid_particles,prefix_sum}_cs.glsl
compiled as C++ and run on the CPU (tests/golden/make_ref_shader_golden.py),
in the shaders' float arithmetic ("f32") and with float promoted to double
("f64").  These tests pin the oracle to them:
  * the grid build (counts, offsets, index list) and the exclusive scan
    equal the reference's shaders bit for bit;
  * the FP64 oracle (brute-force neighbour loops, integrate, EvolveWave)
    computes the shaders' expressions on the shaders' constants: it equals
    the f64 shader outputs to a few units of double rounding;
  * the float32 restatements (integrate_f32, wave_f32, wave_init_f32,
    wave_from_image_f32) equal the f32 shader outputs bit for bit, except
    where the restatement associates a sum differently (the bilinear texture
    weights, the stencil's neighbour sum), where they agree within a few
    float32 roundings of the operands;
  * where the reference checkout is present, the shaders are rebuilt and
    rerun and reproduce the fixtures bit for bit.
"""
from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np
import pytest

from coupledwateranimation_gb300 import _abi

GOLDEN = Path(__file__).resolve().parent / "golden"
G = np.load(GOLDEN / "ref_shader_outputs.npz")


def _sha(a: np.ndarray) -> str:
    """SHA-256 of the bytes, NaNs as the positive quiet NaN (as the fixtures)."""
    a = np.ascontiguousarray(a).copy()
    if a.dtype.kind == "f":
        a[np.isnan(a)] = np.nan
    return hashlib.sha256(a.tobytes()).hexdigest()


@pytest.fixture(scope="module")
def x():
    from oracle import ref
    return ref.fixture_inputs(np.load(GOLDEN / "init_textures.npz")["splash"])


@pytest.fixture(scope="module")
def desc(orc):
    return orc.scene_defaults(_abi.PRESET_REFERENCE_3D, 0.0, _abi.SceneDesc)


def _normwise(got, want):
    return float(np.max(np.abs(got - want)) / np.max(np.abs(want)))


def _ulps(got32, want32):
    """Distance in float32 ulps, element-wise."""
    a = np.ascontiguousarray(got32, np.float32).view(np.int32).astype(np.int64)
    b = np.ascontiguousarray(want32, np.float32).view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)  # two's-complement order of floats
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return np.abs(a - b)


def test_inputs_regenerate_bit_exactly(x):
    for k, v in x.items():
        assert _sha(v) == str(G[f"sha_{k}"]), f"input {k} differs from the one the fixtures were made on"


def test_fp64_oracle_density_and_force_equal_the_shaders(orc, x, desc):
    """rho_pres_comp.glsl:49-81 and force_comp.glsl:62-115 over all 20,480
    particles (the shaders' all-pairs loops) against the oracle's brute-force
    mode: per-particle relative 1e-14 for rho, normwise 1e-14 for p and force."""
    s = G["sph_sample"]
    p = x["sph"].astype(np.float64)
    w = x["sph_wave"].astype(np.float64)
    orc.rho_pres(desc, p, w, brute=True)
    want = G["rho_f64"]
    assert np.max(np.abs(p[s, 12] - want[:, 0]) / want[:, 0]) <= 1e-14
    assert _normwise(p[s, 13], want[:, 1]) <= 1e-14
    orc.force(desc, p, w, brute=True)
    for c in range(3):
        assert _normwise(p[s, 8 + c], G["force_f64"][:, c]) <= 1e-14, c
    assert np.array_equal(p[s, 11], G["force_f64"][:, 3])  # w: the stored force's w, / 0.25 on crests
    # the float32 shaders are within float rounding of it
    assert np.max(np.abs(G["rho_f32"][:, 0] - want[:, 0]) / want[:, 0]) <= 1e-6
    for c in range(3):
        assert _normwise(G["force_f32"][:, c].astype(np.float64), G["force_f64"][:, c]) <= 1e-6


@pytest.mark.parametrize("mode", [1.0, 0.5])
def test_fp64_oracle_integrate_equals_the_shader(orc, x, desc, mode):
    """integrate_comp.glsl:56-92 with CheckBoundary (:135-177)."""
    desc.wave_mode = mode
    try:
        p = x["integ"].astype(np.float64)
        orc.integrate(desc, p, x["sph_wave"].astype(np.float64))
    finally:
        desc.wave_mode = 1.0
    want = G["integ_f64" if mode == 1.0 else "integ_m05_f64"]
    scale = np.maximum(np.abs(want), 1.0)
    assert np.max(np.abs(p - want) / scale) <= 1e-14


@pytest.mark.parametrize("case,mode", [("evolve64_m1", 1.0), ("evolve64_m05", 0.5)])
def test_fp64_oracle_wave_equals_the_shader(orc, x, desc, case, mode):
    """EvolveWave with get_clamp and the line source (wave_comp.glsl:171-206)."""
    desc.wave_mode = mode
    try:
        got = orc.wave(desc, x["evolve64_un"], x["evolve64_unm1"])
    finally:
        desc.wave_mode = 1.0
    assert np.max(np.abs(got - G[f"{case}_f64"])) <= 1e-16


@pytest.mark.parametrize("mode", [1.0, 0.5])
def test_float32_integrate_equals_the_shader(orc, x, desc, mode):
    """The float32 restatement (the CUDA kernel's arithmetic) against the f32
    shader: bit-exact but for the bilinear surface sample, whose weights the
    restatement applies as two nested lerps, not the GL formula's four
    products (a few ulps of the height field on the rows projected to the
    surface)."""
    desc.wave_mode = mode
    try:
        got, _ = orc.integrate_f32(desc, x["integ"], x["sph_wave"], with_deposits=False)
    finally:
        desc.wave_mode = 1.0
    want = G["integ_f32" if mode == 1.0 else "integ_m05_f32"]
    # the sample only sets y = height - radius (integrate_comp.glsl:79-83)
    other = [c for c in range(16) if c != 1]
    assert np.array_equal(got[:, other].view(np.uint32), want[:, other].view(np.uint32))
    dy = np.abs(got[:, 1].astype(np.float64) - want[:, 1])
    assert np.count_nonzero(dy) <= len(got) // 20, f"{np.count_nonzero(dy)} heights differ"
    assert dy.max() <= 4 * np.finfo(np.float32).eps * np.abs(x["sph_wave"]).max()


@pytest.mark.parametrize("case,size,mode", [("evolve64_m1", "64", 1.0), ("evolve64_m05", "64", 0.5),
                                            ("evolve67_m05", "67", 0.5)])
def test_float32_wave_equals_the_shader(orc, x, desc, case, size, mode):
    """The float32 stencil (the CUDA kernels' arithmetic) sums the four
    neighbours as (n + s) + (e + w) and folds the constant coefficients in
    double; the shader sums left to right in float: within two float32
    roundings of the field's magnitude."""
    un = x[f"evolve{size}_un"]
    desc.wave_nx, desc.wave_nz = un.shape[1], un.shape[0]
    desc.wave_mode = mode
    try:
        got = orc.wave_f32(desc, un, x[f"evolve{size}_unm1"])
    finally:
        desc.wave_nx = desc.wave_nz = 64
        desc.wave_mode = 1.0
    want = G[f"{case}_f32"]
    scale = float(np.abs(un).max())
    assert scale > 0.1
    # a rounding of the neighbour sum, scaled by lambda and the attenuation
    assert np.abs(got.astype(np.float64) - want).max() <= 2 * np.finfo(np.float32).eps * scale
    assert np.mean(got == want) >= 0.9  # most cells round the same way
    if mode == 0.5:  # the line source lifted the middle column in both
        col = un.shape[1] // 2
        lifted = want[:, col] > 0.0001 + 0.001
        assert lifted.any() and np.array_equal(got[lifted, col] > 0.0011, lifted[lifted])


@pytest.mark.parametrize("case,w,h,mode", [("init64_m1", 64, 64, 1.0), ("init64_m0", 64, 64, 0.0),
                                           ("init64_m05", 64, 64, 0.5), ("init67_m05", 67, 45, 0.5)])
def test_float32_wave_init_equals_the_shader_bit_exactly(orc, desc, case, w, h, mode):
    """InitWave (wave_comp.glsl:82-140) for the splash, wave and wake modes."""
    desc.wave_nx, desc.wave_nz, desc.wave_mode = w, h, mode
    try:
        got = orc.wave_init_f32(desc)
    finally:
        desc.wave_nx = desc.wave_nz = 64
        desc.wave_mode = 1.0
    assert np.array_equal(got.view(np.uint32), G[f"{case}_f32"].view(np.uint32))


def test_float32_init_from_image_equals_the_shader_bit_exactly(orc):
    """InitFromImage (wave_comp.glsl:76-80) of the reference's splash texture."""
    tex = np.load(GOLDEN / "init_textures.npz")["splash"]
    got = orc.wave_from_image_f32(32, 64, tex)
    assert np.array_equal(got.view(np.uint32), G["image_f32"].view(np.uint32))


@pytest.mark.parametrize("name", ["grid_a", "grid_b"])
def test_grid_build_equals_the_reference_grid_shader(orc, x, name):
    """UniformGrid2D/ugrid_particles_cs.glsl (cell = clamp(floor((p - min) /
    cell size)), counts by atomicAdd, insert at offset + atomicAdd) with the
    reference's scan between, invocations in index order: the oracle's
    counts, cell starts and stable order equal it bit for bit."""
    from oracle import ref
    _, lo, hi, cell, dims = ref.GRID_CASES[name]
    start, order, _ = orc.grid_build(x[name], list(lo), (cell, cell, cell), dims)
    assert np.array_equal(np.diff(start), G[f"{name}_counts"])
    assert np.array_equal(start[:-1], G[f"{name}_offsets"])
    assert np.array_equal(order, G[f"{name}_list"])
    assert G[f"{name}_counts"].sum() == len(x[name]) and start[-1] == len(x[name])


@pytest.mark.parametrize("name", ["scan_kat", "scan_1k", "scan_16k"])
def test_exclusive_scan_equals_the_reference_scan_shader(orc, x, name):
    """prefix_sum_cs.glsl dispatched as ParallelScan::Compute (up-sweep, then
    down-sweep, UniformGrid2D/ParallelScan.cpp:43-95)."""
    assert np.array_equal(orc.exclusive_scan(x[name]), G[f"{name}_out"])


def test_live_shaders_reproduce_the_fixtures(x, desc):
    """With the reference checkout present: rebuild the shaders from its
    source, rerun every case, and get the committed fixtures back bit for bit."""
    from oracle import ref
    if ref.build() is None or ref.load() is None:
        pytest.skip("the reference checkout is not on this host")
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_ref_shader_golden", GOLDEN / "make_ref_shader_golden.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    u = ref.uniforms(desc)
    r = ref.rho_pres(ref.F64, x["sph"].astype(np.float64), x["sph_wave"], u)
    assert np.array_equal(r[G["sph_sample"], 12:14], G["rho_f64"])
    f = ref.force(ref.F32, ref.rho_pres(ref.F32, x["sph"].astype(np.float64), x["sph_wave"], u), x["sph_wave"], u)
    assert np.array_equal(f[G["sph_sample"], 8:12].astype(np.float32), G["force_f32"])
    i = ref.integrate(ref.F32, x["integ"].astype(np.float64), x["sph_wave"], u)
    assert np.array_equal(i.astype(np.float32), G["integ_f32"])
    desc.wave_mode = 0.5
    try:
        wv = ref.wave(ref.F64, x["evolve64_un"], x["evolve64_unm1"], ref.uniforms(desc, mode=2))
    finally:
        desc.wave_mode = 1.0
    assert np.array_equal(wv, G["evolve64_m05_f64"])
    assert mk.SPH_SAMPLE.tolist() == G["sph_sample"].tolist()
    for name, (_, lo, hi, cell, dims) in ref.GRID_CASES.items():
        got = ref.grid_build(x[name], lo, hi, (cell, cell, cell), dims)
        for part, a in zip(("counts", "offsets", "list"), got):
            assert np.array_equal(a, G[f"{name}_{part}"])
    for name in ref.scan_inputs():
        assert np.array_equal(ref.exclusive_scan(x[name]), G[f"{name}_out"])


# ---- the 2D family (SphWave2D) ---------------------------------------------
@pytest.fixture(scope="module")
def p2d():
    from coupledwateranimation_gb300.sim2d import defaults2d
    return defaults2d()


def _records2d(a):
    from coupledwateranimation_gb300._abi import PARTICLE2D_DTYPE
    return np.ascontiguousarray(a, np.float32).view(PARTICLE2D_DTYPE).reshape(-1)


def _f12(rec):
    return np.ascontiguousarray(rec).view(np.float32).reshape(-1, 12)


def test_2d_init_particles_equal_the_shader_bit_exactly(orc, p2d):
    """InitParticle (SphWaveKoschier2D_grid_cs.glsl:308-333)."""
    from coupledwateranimation_gb300._abi import PARTICLE2D_DTYPE
    got = _f12(orc.init_particles_2d(p2d, PARTICLE2D_DTYPE))
    assert _sha(got) == str(G["s2d_init_sha"])


def test_2d_substep_equals_the_shaders(orc, x, p2d):
    """One SphUgrid::Compute substep (SphWave2D/StencilBuffer.cpp:150-179):
    the grid of uniform_grid_sph_cs.glsl, then ComputeDensityPressure and
    ComputeForces on that grid.  The state holds particles outside the grid
    (in no cell list, so they see no neighbour, not even themselves) and
    below the floor (moved by the density pass, after the grid was built).
    FP64 oracle against the double shaders, within 1e-5 (rho, per particle)
    and 5e-5 (forces, normwise): the oracle forms the wall planes' offsets
    in float and stores float32 records, the double shaders compute the
    offsets in double, and the forces' pressure and viscous differences
    amplify both.  (A particle wrongly in or out of a cell list moves rho by
    10-30%.)"""
    s = G["s2d_sample"]
    st = _records2d(x["s2d_state"])
    dens = orc.density_2d(p2d, st, x["s2d_wave"])
    d = _f12(dens).astype(np.float64)
    want = G["s2d_density_f64"]
    assert np.array_equal(d[s][:, 3], want[:, 3])  # enable flags
    assert np.max(np.abs(d[s][:, 11] - want[:, 11]) / want[:, 11]) <= 1e-5  # rho
    assert np.max(np.abs(d[s][:, 7] - want[:, 7])) / np.max(np.abs(want[:, 7])) <= 2e-5  # pressure
    assert np.max(np.abs(d[s][:, :2] - want[:, :2])) <= 1e-6  # positions after the wall projection
    forc = _f12(orc.force_2d(p2d, dens, x["s2d_wave"], grid_from=st)).astype(np.float64)
    wf = G["s2d_force_f64"]
    for k in (8, 9):  # acceleration
        assert np.max(np.abs(forc[s][:, k] - wf[:, k])) / np.max(np.abs(wf[:, k])) <= 5e-5, k
    for k in (0, 1, 4, 5):  # the Euler update's positions and velocities
        assert np.max(np.abs(forc[s][:, k] - wf[:, k])) / np.max(np.abs(wf[:, k])) <= 1e-5, k
    # the particles outside the grid: density from the wall term alone
    assert np.all(want[:2, 11] >= 1000.0)


def test_2d_fields_equal_the_shaders_bit_exactly(orc):
    """Shallow1D (InitWave, Splash, the Lax-Wendroff predictor and corrector,
    Shallow1D_cs.glsl:88-174) and Wave1D (InitWave in modes 0 and 1, one
    iteration, Wave1D_cs.glsl:92-207) in float32.  The predictor's cell 0 is
    written by two invocations (its own final store and cell 1's FreeBC copy,
    Shallow1D_cs.glsl:146-152, 195-201), an order GLSL leaves open: the
    restatement keeps the own store, as a warp executing both in lockstep
    does; the CPU dispatch runs cell 1 last.  It is left out."""
    from coupledwateranimation_gb300._abi import WAVE2D_1D
    from coupledwateranimation_gb300.sim2d import defaults2d
    p = defaults2d()
    z = np.zeros((p.wave_cells, 4), np.float32)
    init0 = orc.wave_init_2d_f32(p, z, splash=False)
    splash = orc.wave_init_2d_f32(p, init0, splash=True)
    pred = orc.wave_iter_2d_f32(p, splash, 0, out_prev=splash)
    corr = orc.wave_iter_2d_f32(p, pred, 1, out_prev=splash)
    assert _sha(init0) == str(G["s2d_shallow_init_sha"])
    assert _sha(splash) == str(G["s2d_shallow_splash_sha"])
    assert _sha(pred[1:]) == str(G["s2d_shallow_pred_sha"])
    assert _sha(corr) == str(G["s2d_shallow_corr_sha"])
    p1 = defaults2d(WAVE2D_1D)
    z1 = np.zeros((p1.wave_cells, 4), np.float32)
    w0 = orc.wave1d_init_2d_f32(p1, 0, z1, z1)
    w1 = orc.wave1d_init_2d_f32(p1, 1, w0, z1)
    it = orc.wave1d_iter_2d_f32(p1, w1, w0)
    assert _sha(w0) == str(G["s2d_wave1d_init0_sha"])
    assert _sha(w1) == str(G["s2d_wave1d_init1_sha"])
    assert _sha(it) == str(G["s2d_wave1d_iter_sha"])


# ---- PBD boxes ---------------------------------------------------------------
def _pbd_close(got32, want32):
    """One frame: the contact set exact (constraint counts, colours); the
    continuous fields within the float rounding of the shader's atomic adds,
    which the restatement makes in another (fixed) order."""
    g = np.asarray(got32, np.float64)
    w = np.asarray(want32, np.float64)
    assert np.array_equal(g[:, 29], w[:, 29]) and np.array_equal(g[:, 0:4], w[:, 0:4])
    for sl, tol in ((slice(4, 7), 1e-6), (slice(12, 15), 1e-6), (slice(8, 11), 1e-5),
                    (slice(16, 19), 1e-5), (slice(20, 23), 1e-5)):
        assert np.max(np.abs(g[:, sl] - w[:, sl])) <= tol * np.max(np.abs(w[:, sl])), sl
    assert np.array_equal(g[:, 24:29], w[:, 24:29])  # half widths and 1 / mass


def test_pbd_frame_equals_the_shader(orc, x):
    """One frame of uniform_grid_pbd_3D_cs.glsl as GridTestPbdGpu3D::Animate
    runs it (UniformGridGpu3D.cpp:120-183, 338-346) on the demo's 4096
    boxes: the float32 restatement finds the same contacts (the constraint
    count of every box, the colours) and lands within the rounding of the
    shader's float atomics."""
    from coupledwateranimation_gb300._abi import PBD_BOX_DTYPE
    from coupledwateranimation_gb300.pbd import pbd_defaults
    got = orc.pbd_step(pbd_defaults(), np.ascontiguousarray(x["pbd_boxes"]).view(PBD_BOX_DTYPE).reshape(-1), 1)
    got = np.ascontiguousarray(got).view(np.float32).reshape(-1, 32)
    assert _sha(got[:, 29]) == str(G["pbd_counts_sha"]) and _sha(got[:, 0:4]) == str(G["pbd_colors_sha"])
    assert got[:, 29].sum() > 20000  # a dense pile: tens of thousands of contacts
    _pbd_close(got[G["pbd_sample"]], G["pbd_frame1_f32"])


# ---- the renderer's fragment shaders -----------------------------------------
def test_fragment_shading_equals_the_shaders(orc, x):
    """particle_fs.glsl pass 0 (:47-68 and its reflection / refraction /
    lighting helpers) and wave_fs.glsl (:36-88) for 2000 fragments each,
    against the render oracle's per-fragment shading (the arithmetic the
    CUDA renderer follows): the same discards (gl_PointCoord outside the
    sprite), colours and alpha within 1e-5 (float rounding; colours reach
    ~2 before blending)."""
    from oracle import ref
    r = ref.point_radius(x["rfs_pc"])
    assert np.array_equal(r >= 0.5, G["rfs_discard"])
    assert 0.1 < G["rfs_discard"].mean() < 0.4
    sky, size = x["rfs_sky"], x["rfs_sky"].shape[1]
    for k in np.nonzero(~G["rfs_discard"])[0]:
        got = orc.shade_particle(x["rfs_inv_p"], x["rfs_inv_v"], x["rfs_eye"], sky, size, x["rfs_depth"],
                                 int(x["rfs_px"][k]), int(x["rfs_py"][k]), float(r[k]), x["rfs_pp"][k])
        assert np.max(np.abs(got - G["rfs_particle"][k])) <= 1e-5, k
    for k in range(len(x["rfs_v"])):
        got = orc.shade_wave(x["rfs_eye"], sky, size, x["rfs_pw"][k], float(x["rfs_v"][k]))
        assert np.max(np.abs(got - G["rfs_wave"][k])) <= 1e-5, k
