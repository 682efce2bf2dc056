// cwa_device.cuh — device helpers shared by the kernels: the float32 cell
// hash and the bilinear height-field sample, both written one rounding per
// operation (__f*_rn) so results do not depend on FMA contraction.
#pragma once

#include <cuda_runtime.h>

#include "cwa_internal.h"

namespace cwa {

// clamp(floor((p - lo) / cell), 0, n - 1)  (UniformGrid2D/ugrid_particles_cs.glsl:97-103)
__device__ __forceinline__ int cell_axis(float p, float lo, float cell, int n) {
  float t = __fdiv_rn(__fsub_rn(p, lo), cell);
  float f = floorf(t);
  f = fminf(fmaxf(f, 0.0f), (float)(n - 1));
  return (int)f;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Programmatic dependent launch across a step's kernel chain.  Every kernel
// of the chain first waits for the kernel before it to complete (a no-op
// when it was launched without the chaining attribute), then lets the next
// kernel be launched, whose blocks take the SMs this grid's last wave frees
// and wait there: launch latency and ramp-up overlap this grid's tail.  The
// wait covers every earlier kernel, since each one waited for its own
// predecessor before it could complete.
__device__ __forceinline__ void chain_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Index checks of the debug build (compiled with CWA_DEBUG_CHECKS): a failed
// check records kStatusBounds in the status word and evaluates to true, so
// the caller skips the access; release builds compile every check to false.
// They stand in for a memory checker: no trap, the context stays usable.
__device__ __forceinline__ bool dcheck_failed(bool ok, int32_t* status) {
  if (!ok && status) atomicOr(status, kStatusBounds);
  return !ok;
}
#ifdef CWA_DEBUG_CHECKS
#define CWA_DCHECK_FAILED(cond, status) (::cwa::dcheck_failed((cond), (status)))
#else
#define CWA_DCHECK_FAILED(cond, status) (false)
#endif

__device__ __forceinline__ bool finite3(float4 p) {
  return isfinite(p.x) && isfinite(p.y) && isfinite(p.z);
}

// Warp-aggregated count: lanes with the same key share one atomicAdd; each
// lane's slot is its arrival rank within the cell.
__device__ __forceinline__ int count_slot(int32_t* count, int key) {
  const unsigned int active = __activemask();
  const unsigned int peers = __match_any_sync(active, key);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  const int rank = __popc(peers & ((1u << lane) - 1u));
  int base = 0;
  if (lane == leader) base = atomicAdd(count + key, __popc(peers));
  base = __shfl_sync(peers, base, leader);
  return base + rank;
}

// texture(wave_tex, uv) with GL_LINEAR / GL_CLAMP_TO_EDGE on an R32F image
// (StencilImage2DTripleBuffered.cpp:21-26): texel centres at (i + 0.5) / W.
struct Bilinear {
  float v00, v10, v01, v11, ax, ay;
};

__device__ __forceinline__ Bilinear bilinear_patch(const float* __restrict__ u, int w, int h, float s,
                                                   float t) {
  float tx = __fsub_rn(__fmul_rn(s, (float)w), 0.5f);
  float ty = __fsub_rn(__fmul_rn(t, (float)h), 0.5f);
  tx = fminf(fmaxf(tx, -1.0f), (float)w);
  ty = fminf(fmaxf(ty, -1.0f), (float)h);
  float fx = floorf(tx), fy = floorf(ty);
  Bilinear b;
  b.ax = __fsub_rn(tx, fx);
  b.ay = __fsub_rn(ty, fy);
  int x0 = (int)fx, y0 = (int)fy;
  int x1 = clampi(x0 + 1, 0, w - 1), y1 = clampi(y0 + 1, 0, h - 1);
  x0 = clampi(x0, 0, w - 1);
  y0 = clampi(y0, 0, h - 1);
  b.v00 = __ldg(u + (size_t)y0 * w + x0);
  b.v10 = __ldg(u + (size_t)y0 * w + x1);
  b.v01 = __ldg(u + (size_t)y1 * w + x0);
  b.v11 = __ldg(u + (size_t)y1 * w + x1);
  return b;
}

__device__ __forceinline__ float bilinear_value(const Bilinear& b, float* top_out = nullptr,
                                                float* bot_out = nullptr) {
  float bx = __fsub_rn(1.0f, b.ax);
  float top = __fadd_rn(__fmul_rn(bx, b.v00), __fmul_rn(b.ax, b.v10));
  float bot = __fadd_rn(__fmul_rn(bx, b.v01), __fmul_rn(b.ax, b.v11));
  if (top_out) *top_out = top;
  if (bot_out) *bot_out = bot;
  return __fadd_rn(__fmul_rn(__fsub_rn(1.0f, b.ay), top), __fmul_rn(b.ay, bot));
}

__device__ __forceinline__ float sample_height(const float* __restrict__ u, int w, int h, float s, float t) {
  return bilinear_value(bilinear_patch(u, w, h, s, t));
}

// Value and derivatives along the texel axes of the same bilinear patch.
__device__ __forceinline__ void sample_height_grad(const float* __restrict__ u, int w, int h, float s,
                                                   float t, float* val, float* dtx, float* dty) {
  Bilinear b = bilinear_patch(u, w, h, s, t);
  float top, bot;
  float by = __fsub_rn(1.0f, b.ay);
  *val = bilinear_value(b, &top, &bot);
  *dtx = __fadd_rn(__fmul_rn(by, __fsub_rn(b.v10, b.v00)), __fmul_rn(b.ay, __fsub_rn(b.v11, b.v01)));
  *dty = __fsub_rn(bot, top);
}

}  // namespace cwa
