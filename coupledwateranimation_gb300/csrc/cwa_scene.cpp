// cwa_scene.cpp — scene presets and the seeded scene generators of libcwa.
// Host code, compiled with -ffp-contract=off so the float expressions here
// round the same way on x86_64 and aarch64.
#include <math.h>
#include <string.h>

#include <vector>

#include "../../include/cwa.h"
#include "cwa_internal.h"

namespace {

// splitmix64 seeding xoshiro256** (Blackman & Vigna); uniform doubles from
// the top 53 bits of each draw.
class Xoshiro256ss {
 public:
  explicit Xoshiro256ss(uint64_t seed) {
    uint64_t x = seed;
    for (uint64_t& w : s_) {
      uint64_t z = (x += 0x9e3779b97f4a7c15ULL);
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
      w = z ^ (z >> 31);
    }
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }

 private:
  static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s_[1] * 5, 7) * 9;
    const uint64_t t = s_[1] << 17;
    s_[2] ^= s_[0];
    s_[3] ^= s_[1];
    s_[1] ^= s_[2];
    s_[0] ^= s_[3];
    s_[2] ^= t;
    s_[3] = rotl(s_[3], 45);
    return r;
  }
  uint64_t s_[4];
};

void set_wave_grid(cwa_scene_desc* o, int32_t nx, int32_t nz) {
  o->wave_nx = nx;
  o->wave_nz = nz;
  if (o->preset != CWA_PRESET_MULLER) return;
  // u_tt = c^2 lap(u) - 0.01 u_t on a unit square: dx = 1/nx, dt_w = dx/2,
  // c = 1 -> lambda = (c dt_w/dx)^2 = 1/4, beta = 0.01 dt_w, atten = 1.
  const double dx = 1.0 / nx;
  const double dtw = 0.5 * dx;
  const double ex = (double)o->box_hi[0] - o->box_lo[0];
  const double ez = (double)o->box_hi[2] - o->box_lo[2];
  o->wave_lambda = 0.25f;
  o->wave_beta = (float)(0.01 * dtw);
  o->wave_uv_scale[0] = (float)(1.0 / ex);
  o->wave_uv_scale[1] = (float)(1.0 / ez);
  o->wave_uv_offset[0] = (float)(-o->box_lo[0] / ex);
  o->wave_uv_offset[1] = (float)(-o->box_lo[2] / ez);
  // A deposited vertical momentum P raises the column under it by
  // P dt_w / (rho0 * cell area * unit depth).
  const double area = (ex / nx) * (ez / nz);
  o->couple_gain = (float)(dtw / ((double)o->rest_rho * area * 1.0));
  // Fixed-point quantum: a particle at 10 m/s deposits about 2^40 units.
  const double mv = 10.0 * (double)o->mass;
  int shift = 40 - (int)ceil(log2(mv));
  o->deposit_shift = shift < 0 ? 0 : (shift > 62 ? 62 : shift);
}

}  // namespace

extern "C" {

// REFERENCE_3D: CoupledWaterAnimation/Main.cpp:28-35 (#defines) and :184-204
// (uniform-block defaults), rho_pres_comp.glsl:41-43, force_comp.glsl:5-7,52,
// integrate_comp.glsl:8,51, StencilImage2DTripleBuffered.h:39 (64x64 wave).
// MULLER: the benchmark physics for lattice spacing s (h = 2s, m = rho0 s^3).
cwa_status cwa_scene_defaults(int32_t preset, float spacing, cwa_scene_desc* o) {
  if (!o) return CWA_ERR_INVALID_ARG;
  if (preset != CWA_PRESET_REFERENCE_3D && preset != CWA_PRESET_MULLER) return CWA_ERR_INVALID_ARG;
  if (preset == CWA_PRESET_MULLER && !(spacing > 0.0f)) return CWA_ERR_INVALID_ARG;
  memset(o, 0, sizeof(*o));
  o->preset = preset;
  if (preset == CWA_PRESET_REFERENCE_3D) {
    o->n_particles = 20480;
    o->box_lo[0] = 0.0f;
    o->box_lo[1] = -0.02f;
    o->box_lo[2] = 0.0f;
    o->box_hi[0] = 0.48f;
    o->box_hi[1] = 1.0f;
    o->box_hi[2] = 0.48f;
    o->particle_radius = 0.005f;
    o->smoothing_length = 2.0f * 0.005f;  // smoothing_coeff * PARTICLE_RADIUS
    o->cell_size = o->smoothing_length;
    o->cell_size_z = o->cell_size;
    o->mass = 0.02f;
    o->visc = 3000.0f;
    o->rest_rho = 1000.0f;
    o->gas_const = 4000.0f;
    o->dt = 0.00005f;
    o->gravity[1] = -9806.65f;
    o->wall_restitution = 0.3f;   // DAMPING
    o->velocity_damping = 0.3f;   // v *= 1 - DAMPING dt
    o->crest_height = 0.01f;      // CREST_THRESHOLD
    o->foam_speed = 25.0f;
    o->wave_lambda = 0.01f;
    o->wave_atten = 0.985f;
    o->wave_beta = 0.001f;
    o->wave_mode = 1.0f;
    o->wave_uv_scale[0] = 2.0f;   // texture(wave_tex, 2 * pos.xz)
    o->wave_uv_scale[1] = 2.0f;
    o->wave_nx = 64;
    o->wave_nz = 64;
  } else {
    const double s = spacing;
    o->box_hi[0] = o->box_hi[1] = o->box_hi[2] = 1.0f;
    o->particle_radius = (float)(0.5 * s);
    o->smoothing_length = (float)(2.0 * s);
    o->cell_size = o->smoothing_length;
    o->cell_size_z = o->cell_size;
    o->rest_rho = 1000.0f;
    o->mass = (float)(1000.0 * s * s * s);
    o->visc = 0.1f;
    o->gas_const = 50.0f;
    o->dt = 1e-4f;
    o->gravity[1] = -9.81f;
    o->wall_restitution = 0.5f;
    o->surface_restitution = 0.5f;
    o->wave_atten = 1.0f;
    o->wave_mode = 1.0f;
    o->surface_y0 = 0.0f;
    set_wave_grid(o, 256, 256);
  }
  return CWA_OK;
}

cwa_status cwa_scene_set_wave_grid(cwa_scene_desc* o, int32_t nx, int32_t nz) {
  if (!o || nx < 1 || nz < 1) return CWA_ERR_INVALID_ARG;
  set_wave_grid(o, nx, nz);
  return CWA_OK;
}

cwa_status cwa_grid_dims(const cwa_scene_desc* sc, int32_t dims[3]) {
  if (!sc || !dims) return CWA_ERR_INVALID_ARG;
  if (!(sc->cell_size > 0.0f)) return CWA_ERR_INVALID_ARG;
  const float csz = sc->cell_size_z > 0.0f ? sc->cell_size_z : sc->cell_size;
  for (int a = 0; a < 3; ++a) {
    const float ext = sc->box_hi[a] - sc->box_lo[a];
    if (!(ext > 0.0f)) return CWA_ERR_INVALID_ARG;
    const float q = ext / (a == 2 ? csz : sc->cell_size);
    if (!(q < 1.0e7f)) return CWA_ERR_CAPACITY;
    const int d = (int)ceilf(q);
    dims[a] = d < 1 ? 1 : d;
  }
  return CWA_OK;
}

// make_cube + init_particles (CoupledWaterAnimation/Main.cpp:735-794):
// 64 x 5 x 64 lattice at spacing smoothing_coeff * 0.85 * PARTICLE_RADIUS,
// i (x) outer, j (y), k (z) inner; extras = (rho0, 0, 500, 50).
cwa_status cwa_make_reference_cube(const cwa_scene_desc* sc, cwa_particle* out, int32_t n) {
  if (!sc || !out || n < 0 || n > 64 * 5 * 64) return CWA_ERR_INVALID_ARG;
  const float spacing = 2.0f * 0.85f * 0.005f;
  int32_t idx = 0;
  for (int i = 0; i < 64 && idx < n; ++i)
    for (int j = 0; j < 5 && idx < n; ++j)
      for (int k = 0; k < 64 && idx < n; ++k, ++idx) {
        cwa_particle& q = out[idx];
        memset(&q, 0, sizeof(q));
        q.pos[0] = 0.0f + (float)i * spacing;
        q.pos[1] = (float)j * spacing;
        q.pos[2] = 0.0f + (float)k * spacing;
        q.pos[3] = 1.0f;
        q.extras[0] = sc->rest_rho;
        q.extras[2] = 500.0f;
        q.extras[3] = 50.0f;
      }
  return CWA_OK;
}

cwa_status cwa_make_dam_break(const cwa_scene_desc* sc, const int32_t dims[3], float spacing, float jitter,
                              uint64_t seed, cwa_particle* out, int32_t n) {
  if (!sc || !dims || !out || n < 0) return CWA_ERR_INVALID_ARG;
  if (dims[0] < 1 || dims[1] < 1 || dims[2] < 1) return CWA_ERR_INVALID_ARG;
  if ((int64_t)dims[0] * dims[1] * dims[2] < n) return CWA_ERR_INVALID_ARG;
  Xoshiro256ss rng(seed);
  const double s = spacing, jj = (double)jitter * s;
  for (int32_t idx = 0; idx < n; ++idx) {
    const int i = idx % dims[0];
    const int j = (idx / dims[0]) % dims[1];
    const int k = idx / (dims[0] * dims[1]);
    const double jx = (2.0 * rng.uniform() - 1.0) * jj;
    const double jy = (2.0 * rng.uniform() - 1.0) * jj;
    const double jz = (2.0 * rng.uniform() - 1.0) * jj;
    cwa_particle& q = out[idx];
    memset(&q, 0, sizeof(q));
    q.pos[0] = (float)((double)sc->box_lo[0] + (i + 0.5) * s + jx);
    q.pos[1] = (float)((double)sc->box_lo[1] + (j + 0.5) * s + jy);
    q.pos[2] = (float)((double)sc->box_lo[2] + (k + 0.5) * s + jz);
    q.pos[3] = 1.0f;
    q.extras[0] = sc->rest_rho;
  }
  return CWA_OK;
}

cwa_status cwa_make_bumps(const cwa_scene_desc* sc, int32_t n_bumps, uint64_t seed, float* u, int32_t nx,
                          int32_t nz) {
  if (!sc || !u || n_bumps < 0 || nx < 1 || nz < 1) return CWA_ERR_INVALID_ARG;
  Xoshiro256ss rng(seed);
  std::vector<double> A(n_bumps), S(n_bumps), CX(n_bumps), CZ(n_bumps);
  for (int b = 0; b < n_bumps; ++b) {
    A[b] = 0.01 + 0.04 * rng.uniform();
    S[b] = 0.02 + 0.08 * rng.uniform();
    CX[b] = rng.uniform();
    CZ[b] = rng.uniform();
  }
  for (int k = 0; k < nz; ++k)
    for (int i = 0; i < nx; ++i) {
      const double s = (i + 0.5) / nx, t = (k + 0.5) / nz;
      double acc = 0.0;
      for (int b = 0; b < n_bumps; ++b) {
        const double dx = s - CX[b], dz = t - CZ[b];
        acc += A[b] * exp(-(dx * dx + dz * dz) / (2.0 * S[b] * S[b]));
      }
      u[(size_t)k * nx + i] = (float)acc;
    }
  return CWA_OK;
}

cwa_status cwa_pbd_defaults(cwa_pbd_params* p) {
  if (!p) return CWA_ERR_INVALID_ARG;
  *p = cwa_pbd_params{};
  p->n_boxes = 4 * 1024;
  p->grid_cells[0] = p->grid_cells[1] = p->grid_cells[2] = 16;
  for (int c = 0; c < 3; ++c) {
    p->extents_lo[c] = -1.0f;
    p->extents_hi[c] = 1.0f;
  }
  p->g[1] = -0.1f;
  p->dt = 0.02f;
  p->damping = 0.999f;
  p->k = 1.75f;
  p->k_static = 10.0f;
  p->sleep_thresh = 0.0005f;
  p->mu_k = 0.4f;
  p->mu_s = 0.5f;
  p->e = 0.75f;
  p->substeps = 1;
  return CWA_OK;
}

cwa_status cwa_pbd_make_boxes(const cwa_pbd_params* p, uint64_t seed, cwa_pbd_box* out, int32_t n) {
  if (!p || !out || n < 0 || p->grid_cells[0] < 1) return CWA_ERR_INVALID_ARG;
  Xoshiro256ss rng(seed);
  // UniformGridPbdGpu3D: cell edge = extent / cells; half widths drawn from
  // [0.15, 0.45] cell edges (x axis), positions 0.5 U(-1, 1), velocities 0.1 U(-1, 1)
  const float cell = (p->extents_hi[0] - p->extents_lo[0]) / (float)p->grid_cells[0];
  auto upos = [&]() { return (float)(2.0 * rng.uniform() - 1.0); };
  auto usize = [&]() { return (float)(0.15 * cell + (0.45 * cell - 0.15 * cell) * rng.uniform()); };
  for (int32_t i = 0; i < n; ++i) {
    cwa_pbd_box& b = out[i];
    memset(&b, 0, sizeof(b));
    const float x = 0.5f * upos(), y = 0.5f * upos(), z = 0.5f * upos();
    const float vx = upos(), vy = upos(), vz = upos();
    const float hx = usize(), hy = usize(), hz = usize();
    for (int c = 0; c < 4; ++c) b.color[c] = 1.0f;
    b.x[0] = b.p[0] = x;
    b.x[1] = b.p[1] = y;
    b.x[2] = b.p[2] = z;
    b.x[3] = b.p[3] = 1.0f;
    b.v[0] = 0.1f * vx;
    b.v[1] = 0.1f * vy;
    b.v[2] = 0.1f * vz;
    b.hw[0] = hx;
    b.hw[1] = hy;
    b.hw[2] = hz;
    b.rm = 1.0f / (hx * hy * hz);
    b.n = 0.0f;
    b.e = 1.0f;
  }
  return CWA_OK;
}

}  // extern "C"
