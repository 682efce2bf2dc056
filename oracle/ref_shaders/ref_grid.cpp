// ref_grid.cpp — the reference's GPU uniform-grid build compiled as C++:
// UniformGrid2D/ugrid_particles_cs.glsl (COMPUTE_COUNTS, INSERT_PARTICLES)
// and UniformGrid2D/prefix_sum_cs.glsl dispatched the way the host code
// dispatches them (UniformGrid2D/UniformGridGpu2D.cpp:96-125: clear the
// counters, count, scan the counts into offsets, clear the counters,
// insert; ParallelScan::Compute, UniformGrid2D/ParallelScan.cpp:43-95).
// TEST INFRASTRUCTURE ONLY.
#include <algorithm>
#include <vector>

#include "glsl.h"
#include "ref_shaders.h"

#define GLSL_CONST(name, init) (init)

namespace ref_ugrid {
GLSL_PRELUDE(f32)
#include "ugrid_particles_cs.inc"
// one dispatch of work groups of 1024 covering `count` invocations; the
// invocations run in order, so each cell's atomicAdd slots go to particles
// in index order
void dispatch(int m, int count) {
  mode = m;
  glsl_init_globals();
  const int groups = (count + 1023) / 1024;
  for (int i = 0; i < groups * 1024; ++i) {
    gl_GlobalInvocationID = uvec3((unsigned)i, 0u, 0u);
    main();
  }
}
}  // namespace ref_ugrid

namespace ref_scan {
GLSL_PRELUDE(f32)
#include "prefix_sum_cs.inc"
void dispatch(int count) {
  glsl_init_globals();
  const int groups = (int)ceil(count / 1024.0f);  // glm::ceil(n / float(mMaxWorkGroup))
  for (int i = 0; i < groups * 1024; ++i) {
    gl_GlobalInvocationID = uvec3((unsigned)i, 0u, 0u);
    main();
  }
}
// ParallelScan::Compute on `count` (a power of two) ints, in place.
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
}  // namespace ref_scan

namespace {
bool pow2(long v) { return v >= 2 && (v & (v - 1)) == 0; }
}  // namespace

extern "C" int32_t ref_exclusive_scan(const int32_t* in, int32_t* out, int32_t n) {
  if (!pow2(n)) return -1;  // ParallelScan::Init asserts a power of two (ParallelScan.cpp:14-16)
  std::copy(in, in + n, out);
  ref_scan::compute(out, n);
  return 0;
}

extern "C" int32_t ref_grid_build(const float* pos4, int32_t n, const float lo[3], const float hi[3],
                                  const float cell[3], const int32_t dims[3], int32_t* counts, int32_t* offsets,
                                  int32_t* index_list) {
  using namespace ref_ugrid;
  const long nc = (long)dims[0] * dims[1] * dims[2];
  // the scan needs a power of two cells; the shader's Index() multiplies by
  // mNumCells.x where the z extent belongs, a cell id only when nx == nz
  if (!pow2(nc) || dims[0] != dims[2] || n < 0) return -1;
  std::vector<Particle> buf((size_t)n);
  for (int i = 0; i < n; ++i) buf[i].pos = vec4(pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2], pos4[4 * i + 3]);
  std::vector<int> counter((size_t)nc, 0), offset((size_t)nc, 0), list((size_t)n, -1);
  particles = buf.data();
  mGridCounter = counter.data();
  mGridOffset = offset.data();
  mIndexList = list.data();
  num_particles = n;
  mExtents.mMin = vec4(lo[0], lo[1], lo[2], 0.0f);
  mExtents.mMax = vec4(hi[0], hi[1], hi[2], 0.0f);
  mNumCells = ivec4(dims[0], dims[1], dims[2], 0);
  mCellSize = vec4(cell[0], cell[1], cell[2], 0.0f);
  dispatch(COMPUTE_COUNTS, n);
  std::copy(counter.begin(), counter.end(), counts);
  std::copy(counter.begin(), counter.end(), offset.begin());
  ref_scan::compute(offset.data(), (int)nc);
  std::copy(offset.begin(), offset.end(), offsets);
  std::fill(counter.begin(), counter.end(), 0);
  dispatch(INSERT_PARTICLES, n);
  std::copy(list.begin(), list.end(), index_list);
  particles = nullptr;
  mGridCounter = mGridOffset = mIndexList = nullptr;
  return 0;
}
