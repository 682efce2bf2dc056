// ref_sph2d.cpp — the reference's 2D solver family (SphWave2D) compiled as
// C++: SphWaveKoschier2D_grid_cs.glsl over the uniform grid of
// uniform_grid_sph_cs.glsl (COMPUTE_COUNTS, the scan of prefix_sum_cs.glsl,
// INSERT_BOXES), and the 1D fields Shallow1D_cs.glsl and Wave1D_cs.glsl.
// Dispatched the way the host code runs them: SphUgrid::Compute
// (SphWave2D/StencilBuffer.cpp:150-179) builds the grid from the read
// buffer, then runs the density and force modes, each reading one particle
// buffer and writing the other, both on that one grid (its 32 x 32 cells
// over [0, 9.6]^2, StencilBuffer.cpp:138); UniformGridSph2D::CollisionQuery
// (UniformGridGpu2D.cpp:220-265) clears, counts, scans, clears and inserts.
// TEST INFRASTRUCTURE ONLY.
#include <algorithm>
#include <vector>

#include "glsl.h"
#include "ref_shaders.h"

#define GLSL_CONST(name, init) (init)

#undef M_PI  // the shader declares its own M_PI constant

namespace ref2d_grid {
GLSL_PRELUDE(f32)
#include "SphWave2D_uniform_grid_sph_cs.inc"
void dispatch(int m, int count) {
  mode = m;
  glsl_init_globals();
  const int groups = (count + 1023) / 1024;
  for (int i = 0; i < groups * 1024; ++i) {
    gl_GlobalInvocationID = uvec3((unsigned)i, 0u, 0u);
    main();
  }
}
}  // namespace ref2d_grid

namespace ref2d_scan {
GLSL_PRELUDE(f32)
#include "SphWave2D_prefix_sum_cs.inc"
void dispatch(int count) {
  glsl_init_globals();
  const int groups = (int)ceil(count / 1024.0f);
  for (int i = 0; i < groups * 1024; ++i) {
    gl_GlobalInvocationID = uvec3((unsigned)i, 0u, 0u);
    main();
  }
}
// ParallelScan::Compute (SphWave2D/ParallelScan.cpp:43-95), in place
void compute(int* data, int count) {
  x = data;
  n = count;
  int m = count / 2, pass = 0;
  phase = UPSWEEP_PHASE;
  for (;;) {
    stride = 2 << pass;
    dispatch(m);
    if (m == 1) break;
    m = m / 2;
    pass = pass + 1;
  }
  phase = DOWNSWEEP_PHASE;
  for (;;) {
    stride = 2 << pass;
    dispatch(m);
    if (m == count / 2) break;
    m = m * 2;
    pass = pass - 1;
  }
  x = nullptr;
}
}  // namespace ref2d_scan

namespace {

struct Grid2 {
  std::vector<int> counter, offset, list;
};

// The grid of the particles `p12` (n records of 12 doubles): clear, count,
// scan, clear, insert.  The grid shader reads float positions.
bool build_grid(const double* p12, int n, const ref2d_uniforms* u, Grid2& g) {
  using namespace ref2d_grid;
  const int nc = u->grid_cells[0] * u->grid_cells[1];
  if (nc < 2 || (nc & (nc - 1))) return false;  // the scan needs a power of two
  std::vector<Particle> buf((size_t)n);
  for (int i = 0; i < n; ++i) {
    const double* q = p12 + 12 * (size_t)i;
    buf[i].pos = vec4(q[0], q[1], q[2], q[3]);
    buf[i].vel = vec4(q[4], q[5], q[6], q[7]);
    buf[i].acc = vec4(q[8], q[9], q[10], q[11]);
  }
  g.counter.assign((size_t)nc, 0);
  g.offset.assign((size_t)nc, 0);
  g.list.assign((size_t)n, -1);
  mParticles = buf.data();
  mGridCounter = g.counter.data();
  mGridOffset = g.offset.data();
  mIndexList = g.list.data();
  num_boxes = n;
  mExtents.mMin = vec2(0.0f, 0.0f);
  mExtents.mMax = vec2(u->extent_max[0], u->extent_max[1]);
  mNumCells = ivec2(u->grid_cells[0], u->grid_cells[1]);
  // UniformGridSph2D: (mMax - mMin) / vec2(mNumCells), in float
  mCellSize = vec2(u->extent_max[0] / (float)u->grid_cells[0], u->extent_max[1] / (float)u->grid_cells[1]);
  dispatch(COMPUTE_COUNTS, n);
  std::copy(g.counter.begin(), g.counter.end(), g.offset.begin());
  ref2d_scan::compute(g.offset.data(), nc);
  std::fill(g.counter.begin(), g.counter.end(), 0);
  dispatch(INSERT_BOXES, n);
  mParticles = nullptr;
  mGridCounter = mGridOffset = mIndexList = nullptr;
  return true;
}

}  // namespace

// One SPH mode over the particles, reading `in` and writing `out`, with the
// grid g bound (the same grid for both modes of a substep).
#define REF_SPH2D_RUN                                                                          \
  void run(int m, const double* in12, double* out12, int n, const float* wave4, int wave_n,   \
           const ref2d_uniforms* u, Grid2& g) {                                                \
    std::vector<Particle> a((size_t)n), b((size_t)n);                                          \
    for (int i = 0; i < n; ++i) {                                                              \
      const double* q = in12 + 12 * (size_t)i;                                                 \
      a[i].pos = vec4(q[0], q[1], q[2], q[3]);                                                 \
      a[i].vel = vec4(q[4], q[5], q[6], q[7]);                                                 \
      a[i].acc = vec4(q[8], q[9], q[10], q[11]);                                               \
    }                                                                                          \
    particles_in = a.data();                                                                   \
    particles_out = b.data();                                                                  \
    mGridCounter = g.counter.data();                                                           \
    mGridOffset = g.offset.data();                                                             \
    mIndexList = g.list.data();                                                                \
    mExtents.mMin = vec2(0.0f, 0.0f);                                                          \
    mExtents.mMax = vec2(u->extent_max[0], u->extent_max[1]);                                  \
    mNumCells = ivec2(u->grid_cells[0], u->grid_cells[1]);                                     \
    mCellSize = vec2(u->extent_max[0] / (float)u->grid_cells[0],                               \
                     u->extent_max[1] / (float)u->grid_cells[1]);                              \
    wave_tex = sampler1D{wave4, wave_n, 4};                                                    \
    uMode = m;                                                                                 \
    num_particles = n;                                                                         \
    time = u->time;                                                                            \
    bottom = u->bottom;                                                                        \
    glsl_init_globals();                                                                       \
    _Pragma("omp parallel for schedule(dynamic, 64)")                                          \
    for (int i = 0; i < ((n + 1023) / 1024) * 1024; ++i) {                                     \
      gl_GlobalInvocationID = uvec3((unsigned)i, 0u, 0u);                                      \
      main();                                                                                  \
    }                                                                                          \
    for (int i = 0; i < n; ++i) {                                                              \
      double* q = out12 + 12 * (size_t)i;                                                      \
      for (int c = 0; c < 4; ++c) {                                                            \
        q[c] = b[i].pos.e[c];                                                                  \
        q[4 + c] = b[i].vel.e[c];                                                              \
        q[8 + c] = b[i].acc.e[c];                                                              \
      }                                                                                        \
    }                                                                                          \
    particles_in = particles_out = nullptr;                                                    \
  }

namespace ref2d_sph_f32 {
GLSL_PRELUDE(f32)
#include "SphWave2D_SphWaveKoschier2D_grid_cs.inc"
REF_SPH2D_RUN
}  // namespace ref2d_sph_f32

#undef GLSL_CONST
#define GLSL_CONST(name, init) (ref2d_sph_f32::name)
namespace ref2d_sph_f64 {
GLSL_PRELUDE(f64)
#define float double
#include "SphWave2D_SphWaveKoschier2D_grid_cs.inc"
#undef float
REF_SPH2D_RUN
}  // namespace ref2d_sph_f64
#undef GLSL_CONST
#define GLSL_CONST(name, init) (init)

// The 1D fields: one dispatch over the image, invocations in order (the
// shaders write invocation-private globals).
#define REF_FIELD1D_RUN(...)                                                                    \
  void run(int m, int n, const float* init4, int init_n, const ref2d_uniforms* u) {            \
    uOutputImage = image1D{out_img, n, false};                                                 \
    uInitImage = sampler1D{init4, init_n, 4};                                                  \
    uMode = m;                                                                                 \
    time = u->time;                                                                            \
    lambda = u->lambda;                                                                        \
    beta = u->beta;                                                                            \
    boundary = vec2(u->boundary[0], u->boundary[1]);                                           \
    __VA_ARGS__                                                                                \
    for (int i = 0; i < ((n + 1023) / 1024) * 1024; ++i) {                                     \
      gl_GlobalInvocationID = uvec3((unsigned)i, 0u, 0u);                                      \
      glsl_init_globals();                                                                     \
      main();                                                                                  \
    }                                                                                          \
  }

namespace ref2d_shallow {
GLSL_PRELUDE(f32)
#include "SphWave2D_Shallow1D_cs.inc"
float* out_img = nullptr;
REF_FIELD1D_RUN(dx = u->dx;)
}  // namespace ref2d_shallow

namespace ref2d_wave1d {
GLSL_PRELUDE(f32)
#include "SphWave2D_Wave1D_cs.inc"
float* out_img = nullptr;
REF_FIELD1D_RUN(atten = u->atten;)
}  // namespace ref2d_wave1d

extern "C" int32_t ref2d_sph(int32_t prec, int32_t mode, const double* in12, double* out12, int32_t n,
                             const float* wave4, int32_t wave_n, const ref2d_uniforms* u) {
  Grid2 g;
  if (n < 0 || !build_grid(in12, n, u, g)) return -1;
  if (prec)
    ref2d_sph_f64::run(mode, in12, out12, n, wave4, wave_n, u, g);
  else
    ref2d_sph_f32::run(mode, in12, out12, n, wave4, wave_n, u, g);
  return 0;
}

extern "C" int32_t ref2d_substep(int32_t prec, const double* in12, double* dens12, double* force12, int32_t n,
                                 const float* wave4, int32_t wave_n, const ref2d_uniforms* u) {
  Grid2 g;
  if (n < 0 || !build_grid(in12, n, u, g)) return -1;
  // MODE_COMPUTE_DENSITY_PRESSURE = 1, MODE_COMPUTE_FORCES = 2
  if (prec) {
    ref2d_sph_f64::run(1, in12, dens12, n, wave4, wave_n, u, g);
    ref2d_sph_f64::run(2, dens12, force12, n, wave4, wave_n, u, g);
  } else {
    ref2d_sph_f32::run(1, in12, dens12, n, wave4, wave_n, u, g);
    ref2d_sph_f32::run(2, dens12, force12, n, wave4, wave_n, u, g);
  }
  return 0;
}

extern "C" int32_t ref2d_field(int32_t kind, int32_t mode, const float* in0, const float* in1, float* out4, int32_t n,
                               const float* init4, int32_t init_n, const ref2d_uniforms* u) {
  // the output image starts as the previous output (cells a dispatch does not write keep it)
  if (kind == 0) {
    ref2d_shallow::uInputImage = glsl::image1D{const_cast<float*>(in0), n, false};
    ref2d_shallow::out_img = out4;
    ref2d_shallow::run(mode, n, init4, init_n, u);
  } else {
    ref2d_wave1d::uInputImage0 = glsl::image1D{const_cast<float*>(in0), n, false};
    ref2d_wave1d::uInputImage1 = glsl::image1D{const_cast<float*>(in1), n, false};
    ref2d_wave1d::out_img = out4;
    ref2d_wave1d::run(mode, n, init4, init_n, u);
  }
  return 0;
}
