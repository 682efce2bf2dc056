// ref_pbd.cpp — the reference's PBD box collisions compiled as C++:
// UniformGrid2D/uniform_grid_pbd_3D_cs.glsl, a frame dispatched as
// GridTestPbdGpu3D::Animate runs it (UniformGridGpu3D.cpp:338-346): per
// substep, UniformGridPbdGpu3D::CollisionQuery (UniformGridGpu3D.cpp:120-183)
// clears the counters and offsets, counts, scans (prefix_sum_cs.glsl as
// ParallelScan::Compute), clears, inserts the boxes, then PreAnimate, the
// collision query and PostAnimate.  Invocations run in index order, so the
// shader's float atomics add in that order.  TEST INFRASTRUCTURE ONLY.
#include <algorithm>
#include <vector>

#include "glsl.h"
#include "ref_shaders.h"

#define GLSL_CONST(name, init) (init)
namespace ref_pbd_scan {
GLSL_PRELUDE(f32)
#include "prefix_sum_cs.inc"
void dispatch(int count) {
  glsl_init_globals();
  const int groups = (int)ceil(count / 1024.0f);
  for (int i = 0; i < groups * 1024; ++i) {
    gl_GlobalInvocationID = uvec3((unsigned)i, 0u, 0u);
    main();
  }
}
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
}  // namespace ref_pbd_scan

// n boxes of 32 doubles (color, x, v, p, dp_t, dp_n, hw, (rm, n, e, pad)).
#define REF_PBD_RUN                                                                              \
  void dispatch(int m, int count) {                                                              \
    mode = m;                                                                                    \
    glsl_init_globals();                                                                         \
    for (int i = 0; i < ((count + 1023) / 1024) * 1024; ++i) {                                   \
      gl_GlobalInvocationID = uvec3((unsigned)i, 0u, 0u);                                        \
      main();                                                                                    \
    }                                                                                            \
  }                                                                                              \
  int run(double* b32, int nb, int frames, const ref_pbd_params* q) {                            \
    const int nc = q->grid_cells[0] * q->grid_cells[1] * q->grid_cells[2];                       \
    if (nc < 2 || (nc & (nc - 1)) || q->grid_cells[0] != q->grid_cells[2]) return -1;            \
    std::vector<PbdObj> objs((size_t)nb);                                                        \
    for (int i = 0; i < nb; ++i) {                                                               \
      const double* r = b32 + 32 * (size_t)i;                                                    \
      vec4* v[7] = {&objs[i].color, &objs[i].x, &objs[i].v, &objs[i].p, &objs[i].dp_t, &objs[i].dp_n, &objs[i].hw}; \
      for (int f = 0; f < 7; ++f) *v[f] = vec4(r[4 * f], r[4 * f + 1], r[4 * f + 2], r[4 * f + 3]); \
      objs[i].rm = r[28];                                                                        \
      objs[i].n = r[29];                                                                         \
      objs[i].e = r[30];                                                                         \
      objs[i].padding = r[31];                                                                   \
    }                                                                                            \
    std::vector<int> counter((size_t)nc), offset((size_t)nc), list;                              \
    mObj = objs.data();                                                                          \
    mExtents.mMin = vec4(q->lo[0], q->lo[1], q->lo[2], 0.0f);                                    \
    mExtents.mMax = vec4(q->hi[0], q->hi[1], q->hi[2], 0.0f);                                    \
    mNumCells = ivec4(q->grid_cells[0], q->grid_cells[1], q->grid_cells[2], 0);                  \
    /* UniformGridPbdGpu3D: (mMax - mMin) / vec3(mNumCells), in float */                         \
    mCellSize = vec4((q->hi[0] - q->lo[0]) / (float)q->grid_cells[0],                            \
                     (q->hi[1] - q->lo[1]) / (float)q->grid_cells[1],                            \
                     (q->hi[2] - q->lo[2]) / (float)q->grid_cells[2], 0.0f);                     \
    mParams.g = vec4(q->g[0], q->g[1], q->g[2], 0.0f);                                           \
    mParams.dt = q->dt;                                                                          \
    mParams.damping = q->damping;                                                                \
    mParams.k = q->k;                                                                            \
    mParams.k_static = q->k_static;                                                              \
    mParams.sleep_thresh = q->sleep_thresh;                                                      \
    mParams.mu_k = q->mu_k;                                                                      \
    mParams.mu_s = q->mu_s;                                                                      \
    mParams.e = q->e;                                                                            \
    mParams.n = nb;                                                                              \
    mParams.substeps = q->substeps;                                                              \
    for (int f = 0; f < frames * q->substeps; ++f) {                                             \
      std::fill(counter.begin(), counter.end(), 0);                                              \
      std::fill(offset.begin(), offset.end(), 0);                                                \
      mGridCounter = counter.data();                                                             \
      mGridOffset = offset.data();                                                               \
      dispatch(COMPUTE_COUNTS, nb);                                                              \
      std::copy(counter.begin(), counter.end(), offset.begin());                                 \
      ref_pbd_scan::compute(offset.data(), nc);                                                  \
      list.assign((size_t)offset[nc - 1] + counter[nc - 1], -1);                                 \
      mIndexList = list.data();                                                                  \
      std::fill(counter.begin(), counter.end(), 0);                                              \
      dispatch(INSERT_BOXES, nb);                                                                \
      dispatch(PREANIMATE, nb);                                                                  \
      dispatch(COLLISION_QUERY, nb);                                                             \
      dispatch(POSTANIMATE, nb);                                                                 \
    }                                                                                            \
    for (int i = 0; i < nb; ++i) {                                                               \
      double* r = b32 + 32 * (size_t)i;                                                          \
      const vec4* v[7] = {&objs[i].color, &objs[i].x, &objs[i].v, &objs[i].p, &objs[i].dp_t, &objs[i].dp_n, &objs[i].hw}; \
      for (int f = 0; f < 7; ++f)                                                                \
        for (int c = 0; c < 4; ++c) r[4 * f + c] = v[f]->e[c];                                   \
      r[28] = objs[i].rm;                                                                        \
      r[29] = objs[i].n;                                                                         \
      r[30] = objs[i].e;                                                                         \
      r[31] = objs[i].padding;                                                                   \
    }                                                                                            \
    mObj = nullptr;                                                                              \
    mGridCounter = mGridOffset = mIndexList = nullptr;                                           \
    return 0;                                                                                    \
  }

namespace ref_pbd_f32 {
GLSL_PRELUDE(f32)
#include "uniform_grid_pbd_3D_cs.inc"
REF_PBD_RUN
}  // namespace ref_pbd_f32

#undef GLSL_CONST
#define GLSL_CONST(name, init) (ref_pbd_f32::name)
namespace ref_pbd_f64 {
GLSL_PRELUDE(f64)
#define float double
#include "uniform_grid_pbd_3D_cs.inc"
#undef float
REF_PBD_RUN
}  // namespace ref_pbd_f64

extern "C" int32_t ref_pbd(int32_t prec, double* b32, int32_t n, int32_t frames, const ref_pbd_params* q) {
  return prec ? ref_pbd_f64::run(b32, n, frames, q) : ref_pbd_f32::run(b32, n, frames, q);
}
