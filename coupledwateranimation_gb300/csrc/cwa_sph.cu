// cwa_sph.cu — SPH neighbour passes over the cell-sorted particle arrays.
//
//   rho_pres: poly6 density, equation of state, and (REFERENCE_3D) the wave
//             density / pressure terms — CoupledWaterAnimation/rho_pres_comp.glsl:49-81.
//   force:    spiky pressure gradient + viscosity Laplacian, then either the
//             reference's crest / torque / drag / wave-normal terms
//             (force_comp.glsl:160-237) or gravity only (MULLER).
//
// The reference loops over all N particles per particle (O(N^2)).  Here the
// particles are sorted by uniform-grid cell (cell edge >= h), so the 27-cell
// block around a particle is 9 contiguous z-rows of the sorted arrays; the
// loop visits exactly those rows.  Every pair with r < h lies inside them,
// so the neighbour sets equal the shaders'.  Lanes of a warp that sit in the
// same cell walk the same rows in lock step, so their loads broadcast.
//
// Sums are accumulated in one of three precisions (template P):
//   CWA_PREC_FP32 plain float, CWA_PREC_COMPENSATED float with a two-sum
//   error term (Knuth), CWA_PREC_FP64 double pair math and sums.
#include <cuda_runtime.h>

#include <type_traits>

#include "cwa_device.cuh"
#include "cwa_internal.h"

namespace cwa {
namespace {

template <int P>
struct Sum {
  float s = 0.0f;
  __device__ __forceinline__ void add(float x) { s += x; }
  __device__ __forceinline__ float get() const { return s; }
};

template <>
struct Sum<CWA_PREC_COMPENSATED> {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float x) {
    float t = __fadd_rn(s, x);
    float bp = __fsub_rn(t, s);
    c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(x, bp)));
    s = t;
  }
  __device__ __forceinline__ float get() const { return s + c; }
};

template <>
struct Sum<CWA_PREC_FP64> {
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ double get() const { return s; }
};

template <int P>
using Real = typename std::conditional<P == CWA_PREC_FP64, double, float>::type;

__device__ __forceinline__ float inv_sqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double inv_sqrt(double x) { return rsqrt(x); }
__device__ __forceinline__ float recip(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ double recip(double x) { return 1.0 / x; }

struct CellCoord {
  int x, y, z;
};

__device__ __forceinline__ CellCoord cell_of(const SceneDev* S, float4 p) {
  CellCoord c;
  c.x = cell_axis(p.x, S->lo[0], S->cell, S->dims[0]);
  c.y = cell_axis(p.y, S->lo[1], S->cell, S->dims[1]);
  c.z = cell_axis(p.z, S->lo[2], S->cell, S->dims[2]);
  return c;
}

// Calls body(j) for every sorted index j of the 27 cells around c, row by
// row (x outer, y inner, contiguous z range).
template <class Body>
__device__ __forceinline__ void for_block27(const SceneDev* S, const int32_t* __restrict__ start,
                                            CellCoord c, Body body) {
  const int nx = S->dims[0], ny = S->dims[1], nz = S->dims[2];
  const int z0 = max(c.z - 1, 0), z1 = min(c.z + 1, nz - 1);
  const int x0 = max(c.x - 1, 0), x1 = min(c.x + 1, nx - 1);
  const int y0 = max(c.y - 1, 0), y1 = min(c.y + 1, ny - 1);
  for (int x = x0; x <= x1; ++x) {
    for (int y = y0; y <= y1; ++y) {
      const int row = S->coff + (x * ny + y) * nz;
      const int b = __ldg(start + row + z0);
      const int e = __ldg(start + row + z1 + 1);
      for (int j = b; j < e; ++j) body(j);
    }
  }
}

__device__ __forceinline__ float uv_s(const SceneDev* S, float x) { return x * S->uvs[0] + S->uvo[0]; }
__device__ __forceinline__ float uv_t(const SceneDev* S, float z) { return z * S->uvs[1] + S->uvo[1]; }

template <int P>
__global__ void __launch_bounds__(128)
    k_rho_pres(const float4* __restrict__ pos, const int32_t* __restrict__ start,
               const Tile* __restrict__ tiles, const SceneDev* __restrict__ scenes,
               const float* __restrict__ wave, float2* __restrict__ rho_p) {
  using T = Real<P>;
  const Tile tl = tiles[blockIdx.x];
  const int i = tl.begin + threadIdx.x;
  if (i >= tl.end) return;
  const SceneDev* S = scenes + tl.scene;
  const float4 pi = __ldg(pos + i);
  const T hh = (T)S->h;
  const T h2 = hh * hh;
  const T px = pi.x, py = pi.y, pz = pi.z;
  Sum<P> acc;
  for_block27(S, start, cell_of(S, pi), [&](int j) {
    const float4 pj = __ldg(pos + j);
    const T dx = px - (T)pj.x, dy = py - (T)pj.y, dz = pz - (T)pj.z;
    const T r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < h2) {
      const T q = h2 - r2;
      acc.add(q * q * q);
    }
  });
  const T rho_t = (P == CWA_PREC_FP64 ? (T)S->c_poly6_d : (T)S->c_poly6) * acc.get();
  float rho = (float)rho_t;
  float p = S->k * (rho - S->rho0);
  if (S->preset == CWA_PRESET_REFERENCE_3D) {
    // rho_pres_comp.glsl:70-80
    p = fmaxf(p, 0.0f);
    const float H = sample_height(wave + S->woff, S->nx, S->nz, uv_s(S, pi.x), uv_t(S, pi.z));
    const float wf = H * rho;
    p += wf;
    rho += wf * S->inv_kr;
    rho = fmaxf(S->rho0, rho);
  }
  rho_p[i] = make_float2(rho, p);
}

template <int P>
__global__ void __launch_bounds__(128)
    k_force(const float4* __restrict__ pos, const float4* __restrict__ vel,
            const float2* __restrict__ rho_p, const int32_t* __restrict__ start,
            const Tile* __restrict__ tiles, const SceneDev* __restrict__ scenes,
            const float* __restrict__ wave, float4* __restrict__ force) {
  using T = Real<P>;
  const Tile tl = tiles[blockIdx.x];
  const int i = tl.begin + threadIdx.x;
  if (i >= tl.end) return;
  const SceneDev* S = scenes + tl.scene;
  const float4 pi = __ldg(pos + i);
  const float4 vi = __ldg(vel + i);
  const float2 rpi = __ldg(rho_p + i);
  const T hh = (T)S->h;
  const T h2 = hh * hh;
  const T px = pi.x, py = pi.y, pz = pi.z;
  const T vx = vi.x, vy = vi.y, vz = vi.z, pres_i = rpi.y;
  Sum<P> fpx, fpy, fpz, fvx, fvy, fvz;
  for_block27(S, start, cell_of(S, pi), [&](int j) {
    const float4 pj = __ldg(pos + j);
    const T dx = px - (T)pj.x, dy = py - (T)pj.y, dz = pz - (T)pj.z;
    const T r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < h2 && j != i) {
      const float4 vj = __ldg(vel + j);
      const float2 rpj = __ldg(rho_p + j);
      const T inv_r = r2 > (T)0 ? inv_sqrt(r2) : (T)0;  // normalize(0) := 0
      const T r = r2 * inv_r;
      const T hr = hh - r;
      const T irho = recip((T)rpj.x);
      const T sp = (pres_i + (T)rpj.y) * irho * hr * hr * inv_r;
      fpx.add(sp * dx);
      fpy.add(sp * dy);
      fpz.add(sp * dz);
      const T sv = irho * hr;
      fvx.add(sv * ((T)vj.x - vx));
      fvy.add(sv * ((T)vj.y - vy));
      fvz.add(sv * ((T)vj.z - vz));
    }
  });
  const T cg = P == CWA_PREC_FP64 ? (T)S->k_grad_d * (T)S->mass : (T)(S->k_grad * S->mass);
  const T cp = (T)0.5 * cg;
  float fp[3] = {(float)(cp * fpx.get()), (float)(cp * fpy.get()), (float)(cp * fpz.get())};
  float fv[3] = {(float)(cg * fvx.get()), (float)(cg * fvy.get()), (float)(cg * fvz.get())};
  const float rho = rpi.x;
  float4 out;
  if (S->preset == CWA_PRESET_REFERENCE_3D) {
    // force_comp.glsl:188-212
    float4 fprev = force[i];
    float vs = S->visc;
    if (pi.y > S->crest) {
      fprev.x /= 0.25f;
      fprev.y /= 0.25f;
      fprev.z /= 0.25f;
      fprev.w /= 0.25f;
      vs *= 0.5f;
    }
    const float* u = wave + S->woff;
    const int W = S->nx, Hn = S->nz;
    const float s = uv_s(S, pi.x), t = uv_t(S, pi.z);
    const float H = sample_height(u, W, Hn, s, t);
    const float tq[3] = {0.25f * (pi.y * fprev.z - pi.z * fprev.y), 0.25f * (pi.z * fprev.x - pi.x * fprev.z),
                         0.25f * (pi.x * fprev.y - pi.y * fprev.x)};
    // WaveVelocity (:215-226) and WaveNormal (:229-237)
    const float hx = sample_height(u, W, Hn, s + 0.01f, t);
    const float hy = sample_height(u, W, Hn, s, t + 0.01f);
    const float wv[3] = {(hx - H) / S->dt, (hy - H) / S->dt, (hx - hy) / 0.01f};
    const float hR = sample_height(u, W, Hn, s + 1.0f, t) - H;
    const float hT = sample_height(u, W, Hn, s, t + 1.0f) - H;
    const float nrm[3] = {hR, hT, -1.0f};
    const float vv[3] = {vi.x, vi.y, vi.z};
    float f[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float drag = -0.25f * (vv[c] - wv[c]);
      const float wf = -H * nrm[c] * 0.5f;
      f[c] = fp[c] + fv[c] * vs + rho * S->g[c] + tq[c] + drag + wf;
    }
    out = make_float4(f[0], f[1], f[2], fprev.w);
  } else {
    out = make_float4(fp[0] + fv[0] * S->visc + rho * S->g[0], fp[1] + fv[1] * S->visc + rho * S->g[1],
                      fp[2] + fv[2] * S->visc + rho * S->g[2], 0.0f);
  }
  force[i] = out;
}

}  // namespace

cudaError_t launch_rho_pres(int precision, const float4* pos, const int32_t* start, const Tile* tiles,
                            int32_t n_tiles, int32_t tile_size, const SceneDev* scenes,
                            const float* wave_u, float2* rho_p, cudaStream_t stream) {
  if (n_tiles <= 0) return cudaSuccess;
  switch (precision) {
    case CWA_PREC_FP32:
      k_rho_pres<CWA_PREC_FP32><<<n_tiles, tile_size, 0, stream>>>(pos, start, tiles, scenes, wave_u, rho_p);
      break;
    case CWA_PREC_FP64:
      k_rho_pres<CWA_PREC_FP64><<<n_tiles, tile_size, 0, stream>>>(pos, start, tiles, scenes, wave_u, rho_p);
      break;
    default:
      k_rho_pres<CWA_PREC_COMPENSATED><<<n_tiles, tile_size, 0, stream>>>(pos, start, tiles, scenes, wave_u,
                                                                          rho_p);
  }
  return cudaGetLastError();
}

cudaError_t launch_force(int precision, const float4* pos, const float4* vel, const float2* rho_p,
                         const int32_t* start, const Tile* tiles, int32_t n_tiles, int32_t tile_size,
                         const SceneDev* scenes, const float* wave_u, float4* force,
                         cudaStream_t stream) {
  if (n_tiles <= 0) return cudaSuccess;
  switch (precision) {
    case CWA_PREC_FP32:
      k_force<CWA_PREC_FP32><<<n_tiles, tile_size, 0, stream>>>(pos, vel, rho_p, start, tiles, scenes, wave_u,
                                                                force);
      break;
    case CWA_PREC_FP64:
      k_force<CWA_PREC_FP64><<<n_tiles, tile_size, 0, stream>>>(pos, vel, rho_p, start, tiles, scenes, wave_u,
                                                                force);
      break;
    default:
      k_force<CWA_PREC_COMPENSATED><<<n_tiles, tile_size, 0, stream>>>(pos, vel, rho_p, start, tiles, scenes,
                                                                       wave_u, force);
  }
  return cudaGetLastError();
}

}  // namespace cwa
