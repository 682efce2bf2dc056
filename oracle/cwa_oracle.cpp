// cwa_oracle.cpp — CPU oracle of the coupled SPH + wave step.
//
// TEST INFRASTRUCTURE ONLY: what the tests compare against, and the timed
// CPU baseline.  The product never links or calls this file.  Every function
// cites the reference shader or host code it restates (paths relative to the
// reference project root).  Built with -ffp-contract=off so each float
// operation of the *_f32 routines is rounded on its own, like the CUDA
// kernels' __f*_rn intrinsics.
//
// Parity: the exclusive scan is pinned to the reference's ParallelScanTest
// vector (SphWave2D/ParallelScan.cpp:124-155).  The REFERENCE_3D density,
// force, integrate and wave routines are pinned to the reference's own
// compute shaders compiled for the CPU (oracle/ref_shaders/,
// tests/test_ref_shaders.py): the FP64 routines equal the shaders run in
// double to 1e-14, the float32 routines equal them run in float bit for bit
// or within a few roundings where a sum is associated differently.  The
// MULLER coupling terms have no reference counterpart.

#include "cwa_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

namespace {

// The shaders' float literals as the doubles they round to: the FP64 passes
// compute the shaders' expressions on the shaders' own constant values.
const double kRefPi = (double)3.141592741f;  // PI #define of the shaders (rho_pres_comp.glsl:8)
const double kWaveStep = (double)0.01f;      // WaveVelocity's h (force_comp.glsl:119)
const double kFoamScale = (double)0.1f;      // foam damping (integrate_comp.glsl:73,75)
const double kCeilMargin = (double)0.1f;     // line-source ceiling (integrate_comp.glsl:172-174)
const double kLineThreshold = (double)0.0001f, kLineLift = (double)0.001f;  // wave_comp.glsl:177,182

// ---------------------------------------------------------------- RNG ----
// splitmix64 seeding xoshiro256** (Blackman & Vigna), uniform doubles from
// the top 53 bits.  Same definition as the library's generator.
struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t x = seed;
    for (int i = 0; i < 4; ++i) {
      uint64_t z = (x += 0x9e3779b97f4a7c15ULL);
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
      s[i] = z ^ (z >> 31);
    }
  }
  static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
  uint64_t next() {
    uint64_t r = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// ------------------------------------------------------- wave sampling ----
// texture(sampler2D, uv) with GL_LINEAR + GL_CLAMP_TO_EDGE
// (StencilImage2DTripleBuffered.cpp:25-26): texel centres at (i+0.5)/W.
double sample64(const double* u, int w, int h, double s, double t) {
  double tx = s * w - 0.5, ty = t * h - 0.5;
  tx = std::min(std::max(tx, -1.0), (double)w);
  ty = std::min(std::max(ty, -1.0), (double)h);
  if (tx != tx) tx = -1.0;
  if (ty != ty) ty = -1.0;
  double fx = floor(tx), fy = floor(ty);
  double ax = tx - fx, ay = ty - fy;
  int x0 = (int)fx, y0 = (int)fy;
  int x1 = std::min(std::max(x0 + 1, 0), w - 1), y1 = std::min(std::max(y0 + 1, 0), h - 1);
  x0 = std::min(std::max(x0, 0), w - 1);
  y0 = std::min(std::max(y0, 0), h - 1);
  double v00 = u[(size_t)y0 * w + x0], v10 = u[(size_t)y0 * w + x1];
  double v01 = u[(size_t)y1 * w + x0], v11 = u[(size_t)y1 * w + x1];
  double top = (1.0 - ax) * v00 + ax * v10;
  double bot = (1.0 - ax) * v01 + ax * v11;
  return (1.0 - ay) * top + ay * bot;
}

// Bilinear value plus its derivatives along the texel axes.
void sample64_grad(const double* u, int w, int h, double s, double t, double* val, double* dtx,
                   double* dty) {
  double tx = s * w - 0.5, ty = t * h - 0.5;
  tx = std::min(std::max(tx, -1.0), (double)w);
  ty = std::min(std::max(ty, -1.0), (double)h);
  if (tx != tx) tx = -1.0;
  if (ty != ty) ty = -1.0;
  double fx = floor(tx), fy = floor(ty);
  double ax = tx - fx, ay = ty - fy;
  int x0 = (int)fx, y0 = (int)fy;
  int x1 = std::min(std::max(x0 + 1, 0), w - 1), y1 = std::min(std::max(y0 + 1, 0), h - 1);
  x0 = std::min(std::max(x0, 0), w - 1);
  y0 = std::min(std::max(y0, 0), h - 1);
  double v00 = u[(size_t)y0 * w + x0], v10 = u[(size_t)y0 * w + x1];
  double v01 = u[(size_t)y1 * w + x0], v11 = u[(size_t)y1 * w + x1];
  double top = (1.0 - ax) * v00 + ax * v10;
  double bot = (1.0 - ax) * v01 + ax * v11;
  *val = (1.0 - ay) * top + ay * bot;
  *dtx = (1.0 - ay) * (v10 - v00) + ay * (v11 - v01);
  *dty = bot - top;
}

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// ------------------------------------------------------ FP64 grid -------
struct Grid64 {
  int dims[3];
  std::vector<int> start;   // ncells + 1
  std::vector<int> order;   // particle indices sorted by cell
  std::vector<int> cell;    // cell of each particle
};

double cell_edge(const cwa_scene_desc* sc, int a) {
  return (a == 2 && sc->cell_size_z > 0.0f) ? sc->cell_size_z : sc->cell_size;
}

int cell_axis64(const cwa_scene_desc* sc, const int dims[3], int a, double x) {
  double t = floor((x - sc->box_lo[a]) / cell_edge(sc, a));
  if (!(t >= 0.0)) t = 0.0;
  if (t > dims[a] - 1) t = dims[a] - 1;
  return (int)t;
}

void cell_coords64(const cwa_scene_desc* sc, const int dims[3], const double* p, int c[3]) {
  for (int a = 0; a < 3; ++a) {
    double t = floor((p[a] - sc->box_lo[a]) / cell_edge(sc, a));
    if (!(t >= 0.0)) t = 0.0;
    if (t > dims[a] - 1) t = dims[a] - 1;
    c[a] = (int)t;
  }
}

inline int cell_index(const int dims[3], int cx, int cy, int cz) {
  // (x*ny + y)*nz + z: UniformGrid2D/ugrid_particles_cs.glsl:105-108 (which
  // multiplies by Nx; identical for the square grids it is used with).
  return (cx * dims[1] + cy) * dims[2] + cz;
}

void build_grid64(const cwa_scene_desc* sc, int n, const double* p16, Grid64* g) {
  orc_grid_dims(sc, g->dims);
  size_t nc = (size_t)g->dims[0] * g->dims[1] * g->dims[2];
  g->start.assign(nc + 1, 0);
  g->cell.resize(n);
  g->order.resize(n);
  std::vector<int> count(nc, 0);
  for (int i = 0; i < n; ++i) {
    int c[3];
    cell_coords64(sc, g->dims, p16 + 16 * (size_t)i, c);
    g->cell[i] = cell_index(g->dims, c[0], c[1], c[2]);
    count[g->cell[i]]++;
  }
  int sum = 0;
  for (size_t c = 0; c < nc; ++c) {
    g->start[c] = sum;
    sum += count[c];
  }
  g->start[nc] = sum;
  std::fill(count.begin(), count.end(), 0);
  for (int i = 0; i < n; ++i) g->order[g->start[g->cell[i]] + count[g->cell[i]]++] = i;
}

// Calls fn(j) for every j whose cell is in the 27-cell block around p.
template <class Fn>
inline void for_neighbours(const cwa_scene_desc* sc, const Grid64& g, const double* p, Fn fn) {
  int c[3];
  cell_coords64(sc, g.dims, p, c);
  for (int dx = -1; dx <= 1; ++dx) {
    int x = c[0] + dx;
    if (x < 0 || x >= g.dims[0]) continue;
    for (int dy = -1; dy <= 1; ++dy) {
      int y = c[1] + dy;
      if (y < 0 || y >= g.dims[1]) continue;
      // every z cell a neighbour within h can occupy
      int z0 = cell_axis64(sc, g.dims, 2, p[2] - sc->smoothing_length);
      int z1 = cell_axis64(sc, g.dims, 2, p[2] + sc->smoothing_length);
      int b = g.start[cell_index(g.dims, x, y, z0)];
      int e = g.start[cell_index(g.dims, x, y, z1) + 1];
      for (int k = b; k < e; ++k) fn(g.order[k]);
    }
  }
}

double surface_uv(const cwa_scene_desc* sc, const double* u, double x, double z) {
  return sample64(u, sc->wave_nx, sc->wave_nz, x * sc->wave_uv_scale[0] + sc->wave_uv_offset[0],
                  z * sc->wave_uv_scale[1] + sc->wave_uv_offset[1]);
}

// ------------------------------------------------------ FP32 helpers ----
float sample32(const float* u, int w, int h, float s, float t) {
  float tx = s * (float)w - 0.5f;
  float ty = t * (float)h - 0.5f;
  tx = fminf(fmaxf(tx, -1.0f), (float)w);
  ty = fminf(fmaxf(ty, -1.0f), (float)h);
  float fx = floorf(tx), fy = floorf(ty);
  float ax = tx - fx, ay = ty - fy;
  int x0 = (int)fx, y0 = (int)fy;
  int x1 = clampi(x0 + 1, 0, w - 1), y1 = clampi(y0 + 1, 0, h - 1);
  x0 = clampi(x0, 0, w - 1);
  y0 = clampi(y0, 0, h - 1);
  float v00 = u[(size_t)y0 * w + x0], v10 = u[(size_t)y0 * w + x1];
  float v01 = u[(size_t)y1 * w + x0], v11 = u[(size_t)y1 * w + x1];
  float bx = 1.0f - ax;
  float top = bx * v00 + ax * v10;
  float bot = bx * v01 + ax * v11;
  return (1.0f - ay) * top + ay * bot;
}

// Same patch as sample32 plus texel-axis derivatives (float32, op by op).
void sample32_grad(const float* u, int w, int h, float s, float t, float* val, float* dtx,
                   float* dty) {
  float tx = s * (float)w - 0.5f;
  float ty = t * (float)h - 0.5f;
  tx = fminf(fmaxf(tx, -1.0f), (float)w);
  ty = fminf(fmaxf(ty, -1.0f), (float)h);
  float fx = floorf(tx), fy = floorf(ty);
  float ax = tx - fx, ay = ty - fy;
  int x0 = (int)fx, y0 = (int)fy;
  int x1 = clampi(x0 + 1, 0, w - 1), y1 = clampi(y0 + 1, 0, h - 1);
  x0 = clampi(x0, 0, w - 1);
  y0 = clampi(y0, 0, h - 1);
  float v00 = u[(size_t)y0 * w + x0], v10 = u[(size_t)y0 * w + x1];
  float v01 = u[(size_t)y1 * w + x0], v11 = u[(size_t)y1 * w + x1];
  float bx = 1.0f - ax;
  float by = 1.0f - ay;
  float top = bx * v00 + ax * v10;
  float bot = bx * v01 + ax * v11;
  *val = by * top + ay * bot;
  *dtx = by * (v10 - v00) + ay * (v11 - v01);
  *dty = bot - top;
}

int cell_axis_f32(float p, float lo, float cell, int n) {
  float t = (p - lo) / cell;
  float f = floorf(t);
  f = fminf(fmaxf(f, 0.0f), (float)(n - 1));
  return (int)f;
}

}  // namespace

extern "C" {

int orc_num_threads(void) { return omp_get_max_threads(); }
void orc_set_num_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
}

// ---------------------------------------------------------------- scan ----
// SphWave2D/ParallelScan.cpp:130-137: truth[i] = sum of x[0..i-1].
void orc_exclusive_scan_i32(const int32_t* in, int32_t* out, int32_t n) {
  int32_t sum = 0;
  for (int32_t i = 0; i < n; ++i) {
    int32_t v = in[i];
    out[i] = sum;
    sum += v;
  }
}

// UniformGrid2D/ugrid_particles_cs.glsl:97-108, in float32:
// cell = clamp(floor((p - lo) / cell_size), 0, n - 1), id = (x*ny + y)*nz + z.
int32_t orc_cell_id_f32(const float p[3], const float lo[3], const float cell[3], const int32_t dims[3]) {
  int cx = cell_axis_f32(p[0], lo[0], cell[0], dims[0]);
  int cy = cell_axis_f32(p[1], lo[1], cell[1], dims[1]);
  int cz = cell_axis_f32(p[2], lo[2], cell[2], dims[2]);
  return (cx * dims[1] + cy) * dims[2] + cz;
}

// UniformGrid2D/UniformGrid2D.cpp:33-92 with one cell per point: count,
// exclusive offsets, insert in input order (stable).
void orc_grid_build_f32(const float* pos4, int32_t n, const float lo[3], const float cell[3],
                        const int32_t dims[3], int32_t* cell_start, int32_t* sorted_index,
                        int32_t* cell_of) {
  size_t nc = (size_t)dims[0] * dims[1] * dims[2];
  std::vector<int32_t> count(nc, 0), key(n);
  for (int32_t i = 0; i < n; ++i) {
    key[i] = orc_cell_id_f32(pos4 + 4 * (size_t)i, lo, cell, dims);
    count[key[i]]++;
    if (cell_of) cell_of[i] = key[i];
  }
  orc_exclusive_scan_i32(count.data(), cell_start, (int32_t)nc);
  cell_start[nc] = n;
  std::fill(count.begin(), count.end(), 0);
  for (int32_t i = 0; i < n; ++i) sorted_index[cell_start[key[i]] + count[key[i]]++] = i;
}

void orc_grid_dims(const cwa_scene_desc* sc, int32_t dims[3]) {
  const float csz = sc->cell_size_z > 0.0f ? sc->cell_size_z : sc->cell_size;
  for (int a = 0; a < 3; ++a) {
    float ext = sc->box_hi[a] - sc->box_lo[a];
    float q = ext / (a == 2 ? csz : sc->cell_size);
    int d = (int)ceilf(q);
    dims[a] = d < 1 ? 1 : d;
  }
}

// ------------------------------------------------------------ scenes ----
// REFERENCE_3D: Main.cpp:28-35 (#defines), :184-204 (uniform defaults) and the
// shader consts (rho_pres_comp.glsl:41-43, force_comp.glsl:5-7,52,
// integrate_comp.glsl:8,51).  MULLER: the benchmark physics.
void orc_scene_defaults(int32_t preset, float spacing, cwa_scene_desc* o) {
  memset(o, 0, sizeof(*o));
  o->preset = preset;
  if (preset == CWA_PRESET_REFERENCE_3D) {
    o->n_particles = 20480;
    o->box_lo[0] = 0.0f; o->box_lo[1] = -0.02f; o->box_lo[2] = 0.0f;
    o->box_hi[0] = 0.48f; o->box_hi[1] = 1.0f; o->box_hi[2] = 0.48f;
    o->particle_radius = 0.005f;
    o->smoothing_length = 2.0f * 0.005f;
    o->cell_size = o->smoothing_length;
    o->cell_size_z = o->cell_size;
    o->mass = 0.02f;
    o->visc = 3000.0f;
    o->rest_rho = 1000.0f;
    o->gas_const = 4000.0f;
    o->dt = 0.00005f;
    o->gravity[1] = -9806.65f;
    o->wall_restitution = 0.3f;
    o->velocity_damping = 0.3f;
    o->crest_height = 0.01f;
    o->foam_speed = 25.0f;
    o->wave_lambda = 0.01f;
    o->wave_atten = 0.985f;
    o->wave_beta = 0.001f;
    o->wave_mode = 1.0f;
    o->wave_uv_scale[0] = 2.0f;
    o->wave_uv_scale[1] = 2.0f;
    o->wave_nx = 64;
    o->wave_nz = 64;
  } else {
    double s = spacing;
    o->n_particles = 0;
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
    o->wave_lambda = 0.25f;
    o->wave_atten = 1.0f;
    o->wave_mode = 1.0f;
    o->surface_y0 = 0.0f;
    orc_scene_set_wave_grid(o, 256, 256);
  }
}

// Wave grid of a MULLER scene: dx = 1/nx, dt_w = 0.5 dx, c = 1 so
// lambda = (c dt_w / dx)^2 = 0.25; damping 0.01 u_t as beta = 0.01 dt_w;
// uv maps the box's x-z extent onto the texture; a deposit of momentum P
// changes the height by P dt_w / (rho0 * cell area * unit depth).
void orc_scene_set_wave_grid(cwa_scene_desc* o, int32_t nx, int32_t nz) {
  o->wave_nx = nx;
  o->wave_nz = nz;
  if (o->preset != CWA_PRESET_MULLER) return;
  double dx = 1.0 / nx;
  double dtw = 0.5 * dx;
  double ex = (double)o->box_hi[0] - o->box_lo[0];
  double ez = (double)o->box_hi[2] - o->box_lo[2];
  o->wave_lambda = 0.25f;
  o->wave_beta = (float)(0.01 * dtw);
  o->wave_uv_scale[0] = (float)(1.0 / ex);
  o->wave_uv_scale[1] = (float)(1.0 / ez);
  o->wave_uv_offset[0] = (float)(-o->box_lo[0] / ex);
  o->wave_uv_offset[1] = (float)(-o->box_lo[2] / ez);
  double area = (ex / nx) * (ez / nz);
  o->couple_gain = (float)(dtw / ((double)o->rest_rho * area * 1.0));
  double mv = 10.0 * (double)o->mass;
  int shift = 40 - (int)ceil(log2(mv));
  o->deposit_shift = shift < 0 ? 0 : (shift > 62 ? 62 : shift);
}

// Main.cpp:735-759 (make_cube) and :764-778 (init_particles).
void orc_make_reference_cube(const cwa_scene_desc* sc, float* p16f, int32_t n) {
  (void)sc;
  const float spacing = 2.0f * 0.85f * 0.005f;
  int idx = 0;
  for (int i = 0; i < 64 && idx < n; ++i)
    for (int j = 0; j < 5 && idx < n; ++j)
      for (int k = 0; k < 64 && idx < n; ++k, ++idx) {
        float* q = p16f + 16 * (size_t)idx;
        memset(q, 0, 16 * sizeof(float));
        q[0] = 0.0f + (float)i * spacing;
        q[1] = (float)j * spacing;
        q[2] = 0.0f + (float)k * spacing;
        q[3] = 1.0f;
        q[12] = sc->rest_rho;
        q[13] = 0.0f;
        q[14] = 500.0f;
        q[15] = 50.0f;
      }
}

void orc_make_dam_break(const cwa_scene_desc* sc, const int32_t dims[3], float spacing,
                        float jitter, uint64_t seed, float* p16f, int32_t n) {
  Rng rng(seed);
  double s = spacing, jj = (double)jitter * s;
  for (int32_t idx = 0; idx < n; ++idx) {
    int i = idx % dims[0];
    int j = (idx / dims[0]) % dims[1];
    int k = idx / (dims[0] * dims[1]);
    double jx = (2.0 * rng.uniform() - 1.0) * jj;
    double jy = (2.0 * rng.uniform() - 1.0) * jj;
    double jz = (2.0 * rng.uniform() - 1.0) * jj;
    float* q = p16f + 16 * (size_t)idx;
    memset(q, 0, 16 * sizeof(float));
    q[0] = (float)((double)sc->box_lo[0] + (i + 0.5) * s + jx);
    q[1] = (float)((double)sc->box_lo[1] + (j + 0.5) * s + jy);
    q[2] = (float)((double)sc->box_lo[2] + (k + 0.5) * s + jz);
    q[3] = 1.0f;
    q[12] = sc->rest_rho;
  }
}

void orc_make_bumps(const cwa_scene_desc* sc, int32_t n_bumps, uint64_t seed, float* u,
                    int32_t nx, int32_t nz) {
  (void)sc;
  Rng rng(seed);
  std::vector<double> A(n_bumps), S(n_bumps), CX(n_bumps), CZ(n_bumps);
  for (int b = 0; b < n_bumps; ++b) {
    A[b] = 0.01 + 0.04 * rng.uniform();
    S[b] = 0.02 + 0.08 * rng.uniform();
    CX[b] = rng.uniform();
    CZ[b] = rng.uniform();
  }
  for (int k = 0; k < nz; ++k)
    for (int i = 0; i < nx; ++i) {
      double s = (i + 0.5) / nx, t = (k + 0.5) / nz, acc = 0.0;
      for (int b = 0; b < n_bumps; ++b) {
        double dx = s - CX[b], dz = t - CZ[b];
        acc += A[b] * exp(-(dx * dx + dz * dz) / (2.0 * S[b] * S[b]));
      }
      u[(size_t)k * nx + i] = (float)acc;
    }
}

// --------------------------------------------------------- rho_pres ----
// rho_pres_comp.glsl:49-81 (REFERENCE_3D) / Mueller poly6 + p = k(rho-rho0).
void orc_rho_pres(const cwa_scene_desc* sc, int32_t n, double* p16, const double* u_n,
                  int32_t brute) {
  const bool ref = sc->preset == CWA_PRESET_REFERENCE_3D;
  const double h = sc->smoothing_length, h2 = h * h;
  const double pi = ref ? kRefPi : M_PI;
  const double c6 = (double)sc->mass * 315.0 / (64.0 * pi * pow(h, 9));
  Grid64 g;
  if (!brute) build_grid64(sc, n, p16, &g);
  std::vector<double> rho(n);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; ++i) {
    const double* pi_ = p16 + 16 * (size_t)i;
    double acc = 0.0;
    auto add = [&](int j) {
      const double* pj = p16 + 16 * (size_t)j;
      double dx = pi_[0] - pj[0], dy = pi_[1] - pj[1], dz = pi_[2] - pj[2];
      double r2 = dx * dx + dy * dy + dz * dz;
      if (sqrt(r2) < h) {
        double q = h2 - r2;
        acc += q * q * q;
      }
    };
    if (brute)
      for (int j = 0; j < n; ++j) add(j);
    else
      for_neighbours(sc, g, pi_, add);
    rho[i] = c6 * acc;
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    double* q = p16 + 16 * (size_t)i;
    double r = rho[i];
    double p = (double)sc->gas_const * (r - sc->rest_rho);
    if (ref) {
      p = std::max(p, 0.0);
      double H = surface_uv(sc, u_n, q[0], q[2]);
      double wf = H * r;
      p += wf;
      r += wf / ((double)sc->gas_const * sc->particle_radius);
      r = std::max((double)sc->rest_rho, r);
    }
    q[12] = r;
    q[13] = p;
  }
}

// ------------------------------------------------------------ force ----
// force_comp.glsl:62-139 (REFERENCE_3D: spiky constant -20/(pi h^6), crest,
// torque, drag, wave normal) / Mueller: -45/(pi h^6), viscosity, gravity.
void orc_force(const cwa_scene_desc* sc, int32_t n, double* p16, const double* u_n,
               int32_t brute) {
  const bool ref = sc->preset == CWA_PRESET_REFERENCE_3D;
  const double h = sc->smoothing_length;
  const double pi = ref ? kRefPi : M_PI;
  const double kgrad = (ref ? 20.0 : 45.0) / (pi * pow(h, 6));
  const double m = sc->mass;
  Grid64 g;
  if (!brute) build_grid64(sc, n, p16, &g);
  std::vector<double> out(4 * (size_t)n);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; ++i) {
    const double* a = p16 + 16 * (size_t)i;
    double fp[3] = {0, 0, 0}, fv[3] = {0, 0, 0};
    auto add = [&](int j) {
      if (j == i) return;
      const double* b = p16 + 16 * (size_t)j;
      double d[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
      double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      if (!(r < h)) return;
      double hr = h - r;
      double sp = m * (a[13] + b[13]) / (2.0 * b[12]) * kgrad * hr * hr;
      double inv_r = r > 0.0 ? 1.0 / r : 0.0;  // normalize(0) := 0
      double sv = m / b[12] * kgrad * hr;
      for (int c = 0; c < 3; ++c) {
        fp[c] += sp * d[c] * inv_r;
        fv[c] += sv * (b[4 + c] - a[4 + c]);
      }
    };
    if (brute)
      for (int j = 0; j < n; ++j) add(j);
    else
      for_neighbours(sc, g, a, add);
    double* o = &out[4 * (size_t)i];
    double fw = a[11];
    if (ref) {
      double fprev[3] = {a[8], a[9], a[10]};
      double visc_scale = sc->visc;
      if (a[1] > sc->crest_height) {  // force /= BREAKING_MASS_FACTOR (0.25)
        for (int c = 0; c < 3; ++c) fprev[c] /= 0.25;
        fw /= 0.25;
        visc_scale *= 0.5;  // BREAKING_VISC_FACTOR
      }
      double s = a[0] * sc->wave_uv_scale[0] + sc->wave_uv_offset[0];
      double t = a[2] * sc->wave_uv_scale[1] + sc->wave_uv_offset[1];
      int W = sc->wave_nx, Hh = sc->wave_nz;
      double H = sample64(u_n, W, Hh, s, t);
      double torque[3] = {0.25 * (a[1] * fprev[2] - a[2] * fprev[1]),
                          0.25 * (a[2] * fprev[0] - a[0] * fprev[2]),
                          0.25 * (a[0] * fprev[1] - a[1] * fprev[0])};
      // WaveVelocity (force_comp.glsl:117-128): step 0.01 in uv, shader dt.
      double hx = sample64(u_n, W, Hh, s + kWaveStep, t), hy = sample64(u_n, W, Hh, s, t + kWaveStep);
      double wv[3] = {(hx - H) / sc->dt, (hy - H) / sc->dt, (hx - hy) / kWaveStep};
      // WaveNormal (force_comp.glsl:130-139): cross((0,1,hT-h),(1,0,hR-h)).
      double hR = sample64(u_n, W, Hh, s + 1.0, t) - H;
      double hT = sample64(u_n, W, Hh, s, t + 1.0) - H;
      double nrm[3] = {hR, hT, -1.0};
      for (int c = 0; c < 3; ++c) {
        double drag = -0.25 * (a[4 + c] - wv[c]);
        double wave = -H * nrm[c] * 0.5;
        o[c] = fp[c] + fv[c] * visc_scale + a[12] * sc->gravity[c] + torque[c] + drag + wave;
      }
      o[3] = fw;
    } else {
      for (int c = 0; c < 3; ++c) o[c] = fp[c] + fv[c] * sc->visc + a[12] * sc->gravity[c];
      o[3] = 0.0;
    }
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 4; ++c) p16[16 * (size_t)i + 8 + c] = out[4 * (size_t)i + c];
}

// -------------------------------------------------------- integrate ----
// integrate_comp.glsl:56-92 and CheckBoundary :135-178 (REFERENCE_3D), or
// symplectic Euler + heightfield coupling + restitution walls (MULLER).
static inline int64_t quantize64(double mv, int shift) {
  double s = ldexp(mv, shift);
  const double lim = 4611686018427387904.0;  // 2^62
  if (s > lim) s = lim;
  if (s < -lim) s = -lim;
  if (s != s) s = 0.0;
  return (int64_t)llrint(s);
}

void orc_integrate(const cwa_scene_desc* sc, int32_t n, double* p16, const double* u_n,
                   int64_t* deposits) {
  const bool ref = sc->preset == CWA_PRESET_REFERENCE_3D;
  const int W = sc->wave_nx, Hh = sc->wave_nz;
  const double dt = sc->dt;
  for (int i = 0; i < n; ++i) {
    double* q = p16 + 16 * (size_t)i;
    double v[3], x[3];
    for (int c = 0; c < 3; ++c) {
      double a = q[8 + c] / q[12];
      v[c] = q[4 + c] + dt * a;
      x[c] = q[c] + dt * v[c];
    }
    double damp = 1.0 - (double)sc->velocity_damping * dt;
    for (int c = 0; c < 3; ++c) v[c] *= damp;
    double s = x[0] * sc->wave_uv_scale[0] + sc->wave_uv_offset[0];
    double t = x[2] * sc->wave_uv_scale[1] + sc->wave_uv_offset[1];
    if (ref) {
      if (sc->foam_speed > 0.0f && sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) > sc->foam_speed) {
        for (int c = 0; c < 4; ++c) q[8 + c] *= 0.5;
        q[12] *= kFoamScale;
        q[13] *= 0.25;
        for (int c = 0; c < 3; ++c) v[c] *= kFoamScale;
      }
      double H = sample64(u_n, W, Hh, s, t);
      if (x[1] < H) x[1] = H - sc->particle_radius;
    } else {
      double val, gx, gz;
      sample64_grad(u_n, W, Hh, s, t, &val, &gx, &gz);
      double H = sc->surface_y0 + val;
      if (x[1] < H) {
        if (deposits) {
          int ci = clampi((int)std::max(std::min(floor(s * W), (double)W), -1.0), 0, W - 1);
          int ck = clampi((int)std::max(std::min(floor(t * Hh), (double)Hh), -1.0), 0, Hh - 1);
          deposits[(size_t)ck * W + ci] += quantize64((double)sc->mass * v[1], sc->deposit_shift);
        }
        double nx_ = -gx * W * sc->wave_uv_scale[0];
        double nz_ = -gz * Hh * sc->wave_uv_scale[1];
        double inv = 1.0 / sqrt(nx_ * nx_ + 1.0 + nz_ * nz_);
        double nrm[3] = {nx_ * inv, inv, nz_ * inv};
        double vn = v[0] * nrm[0] + v[1] * nrm[1] + v[2] * nrm[2];
        if (vn < 0.0) {
          double k = (1.0 + sc->surface_restitution) * vn;
          for (int c = 0; c < 3; ++c) v[c] -= k * nrm[c];
        }
        x[1] = H;
      }
    }
    const double e = sc->wall_restitution;
    for (int c = 0; c < 3; ++c) {
      if (x[c] < sc->box_lo[c]) {
        x[c] = sc->box_lo[c];
        v[c] *= -e;
      } else if (x[c] > sc->box_hi[c]) {
        x[c] = sc->box_hi[c];
        v[c] *= -e;
      }
    }
    if (ref && sc->wave_mode > 0.0f && sc->wave_mode < 1.0f) {
      double ceil_y = (double)sc->box_hi[1] + kCeilMargin;
      if (x[1] > ceil_y) {
        x[1] = ceil_y;
        v[1] *= -e;
      }
    }
    for (int c = 0; c < 3; ++c) {
      q[c] = x[c];
      q[4 + c] = v[c];
    }
  }
}

// ------------------------------------------------------------- wave ----
// wave_comp.glsl:171-206: EvolveWave with get_clamp (clamped 5-point
// neighbourhood) and the line source of modes 0 < w < 1; plus the particle
// deposits of the MULLER coupling.
void orc_wave(const cwa_scene_desc* sc, const double* u_n, const double* u_nm1, double* u_out,
              const int64_t* deposits) {
  const int W = sc->wave_nx, H = sc->wave_nz;
  const double lam = sc->wave_lambda, att = sc->wave_atten, beta = sc->wave_beta;
  const bool line = sc->wave_mode > 0.0f && sc->wave_mode < 1.0f;
  const double dq = ldexp(1.0, -sc->deposit_shift) * (double)sc->couple_gain;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < H; ++j)
    for (int i = 0; i < W; ++i) {
      size_t c = (size_t)j * W + i;
      double c0 = u_n[c], c1 = u_nm1[c];
      double nn = u_n[(size_t)std::min(j + 1, H - 1) * W + i];
      double ss = u_n[(size_t)std::max(j - 1, 0) * W + i];
      double ee = u_n[(size_t)j * W + std::min(i + 1, W - 1)];
      double ww = u_n[(size_t)j * W + std::max(i - 1, 0)];
      double w = (2.0 - 4.0 * lam - beta) * c0 + lam * (nn + ss + ee + ww) - (1.0 - beta) * c1;
      w *= att;
      if (line && w > kLineThreshold && i == W / 2) w += kLineLift;
      if (deposits) w += (double)deposits[c] * dq;
      u_out[c] = w;
    }
}

void orc_step(const cwa_scene_desc* sc, int32_t n, double* p16, double* u_n, double* u_nm1,
              int32_t n_steps, int32_t brute) {
  const size_t nw = (size_t)sc->wave_nx * sc->wave_nz;
  std::vector<double> nxt(nw);
  std::vector<int64_t> dep(nw);
  for (int s = 0; s < n_steps; ++s) {
    std::fill(dep.begin(), dep.end(), 0);
    orc_rho_pres(sc, n, p16, u_n, brute);
    orc_force(sc, n, p16, u_n, brute);
    orc_integrate(sc, n, p16, u_n, sc->preset == CWA_PRESET_MULLER ? dep.data() : nullptr);
    orc_wave(sc, u_n, u_nm1, nxt.data(), sc->preset == CWA_PRESET_MULLER ? dep.data() : nullptr);
    // StencilImage2DTripleBuffered::PingPong (:33-40): u^(n-1) <- u^n <- new.
    memcpy(u_nm1, u_n, nw * sizeof(double));
    memcpy(u_n, nxt.data(), nw * sizeof(double));
  }
}

void orc_totals(const cwa_scene_desc* sc, int32_t n, const double* p16, const double* u_n,
                const double* u_nm1, double out[CWA_TOTALS_COUNT]) {
  double t[CWA_TOTALS_COUNT] = {0};
  const double m = sc->mass;
  for (int i = 0; i < n; ++i) {
    const double* q = p16 + 16 * (size_t)i;
    t[CWA_TOTAL_MASS] += m;
    double v2 = 0.0;
    for (int c = 0; c < 3; ++c) {
      t[CWA_TOTAL_MOMENTUM_X + c] += m * q[4 + c];
      v2 += q[4 + c] * q[4 + c];
      t[CWA_TOTAL_POTENTIAL] -= m * sc->gravity[c] * (q[c] - sc->box_lo[c]);
    }
    t[CWA_TOTAL_KINETIC] += 0.5 * m * v2;
  }
  const int W = sc->wave_nx, H = sc->wave_nz;
  double area = ((double)sc->box_hi[0] - sc->box_lo[0]) / W * (((double)sc->box_hi[2] - sc->box_lo[2]) / H);
  for (size_t c = 0; c < (size_t)W * H; ++c) {
    t[CWA_TOTAL_WAVE_VOLUME] += u_n[c] * area;
    double d = u_n[c] - u_nm1[c];
    t[CWA_TOTAL_WAVE_ENERGY] += 0.5 * (u_n[c] * u_n[c] + d * d) * area;
  }
  memcpy(out, t, sizeof(t));
}

// --------------------------------------------------- FP32-exact passes ----
// The integrate pass in float32, one rounding per operation, in the order
// the CUDA kernel uses.  Deposits: q = rint(clamp(m*vy * 2^shift, +-2^62)).
void orc_integrate_f32(const cwa_scene_desc* sc, int32_t n, float* p16f, const float* u_n,
                       int64_t* deposits) {
  const bool ref = sc->preset == CWA_PRESET_REFERENCE_3D;
  const int W = sc->wave_nx, Hh = sc->wave_nz;
  const float dt = sc->dt;
  const float damp = 1.0f - sc->velocity_damping * dt;
  const float e = sc->wall_restitution;
  const float qscale = ldexpf(1.0f, sc->deposit_shift);
  for (int i = 0; i < n; ++i) {
    float* q = p16f + 16 * (size_t)i;
    float v[3], x[3];
    for (int c = 0; c < 3; ++c) {
      float a = q[8 + c] / q[12];
      v[c] = q[4 + c] + dt * a;
      x[c] = q[c] + dt * v[c];
    }
    for (int c = 0; c < 3; ++c) v[c] = v[c] * damp;
    float s = x[0] * sc->wave_uv_scale[0] + sc->wave_uv_offset[0];
    float t = x[2] * sc->wave_uv_scale[1] + sc->wave_uv_offset[1];
    if (ref) {
      float sp2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
      if (sc->foam_speed > 0.0f && sqrtf(sp2) > sc->foam_speed) {
        for (int c = 0; c < 4; ++c) q[8 + c] = q[8 + c] * 0.5f;
        q[12] = q[12] * 0.1f;
        q[13] = q[13] * 0.25f;
        for (int c = 0; c < 3; ++c) v[c] = v[c] * 0.1f;
      }
      float H = sample32(u_n, W, Hh, s, t);
      if (x[1] < H) x[1] = H - sc->particle_radius;
    } else {
      float val, gx, gz;
      sample32_grad(u_n, W, Hh, s, t, &val, &gx, &gz);
      float H = sc->surface_y0 + val;
      if (x[1] < H) {
        if (deposits) {
          float fs = fminf(fmaxf(floorf(s * (float)W), -1.0f), (float)W);
          float ft = fminf(fmaxf(floorf(t * (float)Hh), -1.0f), (float)Hh);
          int ci = clampi((int)fs, 0, W - 1), ck = clampi((int)ft, 0, Hh - 1);
          float mv = sc->mass * v[1];
          float sq = mv * qscale;
          const float lim = 4611686018427387904.0f;
          sq = fminf(fmaxf(sq, -lim), lim);
          deposits[(size_t)ck * W + ci] += (int64_t)llrintf(sq);
        }
        float nx_ = -(gx * ((float)W * sc->wave_uv_scale[0]));
        float nz_ = -(gz * ((float)Hh * sc->wave_uv_scale[1]));
        float len2 = nx_ * nx_ + 1.0f + nz_ * nz_;
        float inv = 1.0f / sqrtf(len2);
        float nrm[3] = {nx_ * inv, inv, nz_ * inv};
        float vn = v[0] * nrm[0] + v[1] * nrm[1] + v[2] * nrm[2];
        if (vn < 0.0f) {
          float k = (1.0f + sc->surface_restitution) * vn;
          for (int c = 0; c < 3; ++c) v[c] = v[c] - k * nrm[c];
        }
        x[1] = H;
      }
    }
    for (int c = 0; c < 3; ++c) {
      if (x[c] < sc->box_lo[c]) {
        x[c] = sc->box_lo[c];
        v[c] = v[c] * -e;
      } else if (x[c] > sc->box_hi[c]) {
        x[c] = sc->box_hi[c];
        v[c] = v[c] * -e;
      }
    }
    if (ref && sc->wave_mode > 0.0f && sc->wave_mode < 1.0f) {
      float ceil_y = sc->box_hi[1] + 0.1f;
      if (x[1] > ceil_y) {
        x[1] = ceil_y;
        v[1] = v[1] * -e;
      }
    }
    for (int c = 0; c < 3; ++c) {
      q[c] = x[c];
      q[4 + c] = v[c];
    }
  }
}

// EvolveWave in float32 (wave_comp.glsl:171-187) with the deposit source:
// w = atten*((a*c0 + lam*((n+s)+(e+w))) - b*c1); line source; + gain*dep.
void orc_wave_f32(const cwa_scene_desc* sc, const float* u_n, const float* u_nm1, float* u_out,
                  const int64_t* deposits) {
  const int W = sc->wave_nx, H = sc->wave_nz;
  const float lam = sc->wave_lambda, att = sc->wave_atten;
  const float a = (float)(2.0 - 4.0 * (double)sc->wave_lambda - (double)sc->wave_beta);
  const float b = (float)(1.0 - (double)sc->wave_beta);
  const bool line = sc->wave_mode > 0.0f && sc->wave_mode < 1.0f;
  const float dq = ldexpf(1.0f, -sc->deposit_shift);
  for (int j = 0; j < H; ++j)
    for (int i = 0; i < W; ++i) {
      size_t c = (size_t)j * W + i;
      float c0 = u_n[c], c1 = u_nm1[c];
      float nn = u_n[(size_t)std::min(j + 1, H - 1) * W + i];
      float ss = u_n[(size_t)std::max(j - 1, 0) * W + i];
      float ee = u_n[(size_t)j * W + std::min(i + 1, W - 1)];
      float ww = u_n[(size_t)j * W + std::max(i - 1, 0)];
      float nb = (nn + ss) + (ee + ww);
      float w = a * c0 + lam * nb;
      w = w - b * c1;
      w = att * w;
      if (line && w > 0.0001f && i == W / 2) w = w + 0.001f;
      if (deposits) {
        float d = (float)deposits[c];
        w = w + sc->couple_gain * (d * dq);
      }
      u_out[c] = w;
    }
}

// InitFromImage (wave_comp.glsl:76-80): texelFetch(uInitImage, coord * (2, 1)).r
// of an RGBA8 texture is c / 255 in float; past the image, 0.
void orc_wave_from_image_f32(int32_t nx, int32_t nz, const uint8_t* rgba, int32_t w, int32_t h, float* u) {
  for (int32_t y = 0; y < nz; ++y)
    for (int32_t x = 0; x < nx; ++x) {
      const int32_t tx = 2 * x;
      u[(size_t)y * nx + x] = (tx < w && y < h) ? (float)rgba[((size_t)y * w + tx) * 4] / 255.0f : 0.0f;
    }
}

// InitWave (wave_comp.glsl:82-140) in float32.
void orc_wave_init_f32(const cwa_scene_desc* sc, float* u) {
  const int W = sc->wave_nx, H = sc->wave_nz;
  const float mode = sc->wave_mode;
  int c0x, c0y, c1x, c1y, c2x, c2y;
  float peak;
  bool three = true;
  if (mode == 1.0f) {
    c0x = (int)(0.25f * (float)W); c0y = (int)(0.25f * (float)H);
    c1x = (int)(0.75f * (float)W); c1y = (int)(0.75f * (float)H);
    c2x = c0x; c2y = c0y;
    peak = 0.5f;
    three = false;
  } else if (mode == 0.0f) {
    c0x = (int)(0.25f * (float)W); c0y = H;
    c2x = (int)(0.5f * (float)W); c2y = H;
    c1x = (int)(0.75f * (float)W); c1y = H;
    peak = 1.0f;
  } else {
    c0x = (int)(0.5f * (float)W); c0y = (int)(0.1f * (float)H);
    c1x = c2x = c0x; c1y = c2y = c0y;
    peak = 0.1f;
  }
  for (int j = 0; j < H; ++j)
    for (int i = 0; i < W; ++i) {
      auto dist = [&](int cx, int cy) {
        float dx = (float)i - (float)cx, dy = (float)j - (float)cy;
        return sqrtf(dx * dx + dy * dy);
      };
      float d = fminf(dist(c0x, c0y), dist(c1x, c1y));
      if (three) d = fminf(d, dist(c2x, c2y));
      float t = (d - 5.0f) / (0.0f - 5.0f);
      t = fminf(fmaxf(t, 0.0f), 1.0f);
      float sm = (t * t) * (3.0f - 2.0f * t);
      u[(size_t)j * W + i] = peak * sm;
    }
}

float orc_sample_f32(const float* u, int32_t w, int32_t h, float s, float t) {
  return sample32(u, w, h, s, t);
}

}  // extern "C"
