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
// rho_pres does the candidate tests once and leaves each particle's hits as
// a neighbour list; force then runs its pair terms over that list only.
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

// Sorted-index ranges [b, e) of the 9 z-rows that hold the 27 cells around
// c (x outer, y inner); rows outside the grid are empty.  All 18 loads are
// independent, so they overlap.
__device__ __forceinline__ void row_ranges(const SceneDev* S, const int32_t* __restrict__ start, CellCoord c,
                                           int b[9], int e[9]) {
  const int nx = S->dims[0], ny = S->dims[1], nz = S->dims[2];
  const int z0 = max(c.z - 1, 0), z1 = min(c.z + 1, nz - 1);
#pragma unroll
  for (int dx = -1; dx <= 1; ++dx) {
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy) {
      const int r = (dx + 1) * 3 + (dy + 1);
      const int x = c.x + dx, y = c.y + dy;
      const bool ok = x >= 0 && x < nx && y >= 0 && y < ny;
      const int row = S->coff + (x * ny + y) * nz;
      b[r] = ok ? __ldg(start + row + z0) : 0;
      e[r] = ok ? __ldg(start + row + z1 + 1) : 0;
    }
  }
}

__device__ __forceinline__ float uv_s(const SceneDev* S, float x) { return x * S->uvs[0] + S->uvo[0]; }
__device__ __forceinline__ float uv_t(const SceneDev* S, float z) { return z * S->uvs[1] + S->uvo[1]; }

// Neighbour-list capacity per particle.  ~33 neighbours at rest density with
// h = 2 s; a particle with more falls back to the candidate scan in force.
constexpr int kNbThreads = 128;

// rho_pres: tests every candidate of the 27-cell block once, accumulates
// the poly6 sum branch-free per row (q = max(h^2 - r^2, 0), sum of q^3 in
// float within a row, rows combined by the precision mode's accumulator),
// and writes the hits (r < h, j != i) as the particle's neighbour list
// nbr[k * n_total + i], k < kMaxNbr, which the force pass consumes.
template <int P>
__global__ void __launch_bounds__(kNbThreads)
    k_rho_pres(const float4* __restrict__ pos, const int32_t* __restrict__ start,
               const Tile* __restrict__ tiles, const SceneDev* __restrict__ scenes,
               const float* __restrict__ wave, float2* __restrict__ rho_p, int32_t* __restrict__ nbr,
               int32_t* __restrict__ nbr_cnt, int32_t n_total) {
  using T = Real<P>;
  const Tile tl = tiles[blockIdx.x];
  const int i = tl.begin + threadIdx.x;
  if (i >= tl.end) return;
  const SceneDev* S = scenes + tl.scene;
  const float4 pi = __ldg(pos + i);
  const T hh = (T)S->h;
  const T h2 = hh * hh;
  const T px = pi.x, py = pi.y, pz = pi.z;
  int b[9], e[9];
  row_ranges(S, start, cell_of(S, pi), b, e);
  Sum<P> acc;
  int cnt = 0;
#pragma unroll
  for (int r = 0; r < 9; ++r) {
    T part = (T)0;
#pragma unroll 4
    for (int j = b[r]; j < e[r]; ++j) {
      const float4 pj = __ldg(pos + j);
      const T dx = px - (T)pj.x, dy = py - (T)pj.y, dz = pz - (T)pj.z;
      const T q = h2 - (dx * dx + dy * dy + dz * dz);
      const T qp = q > (T)0 ? q : (T)0;
      part += qp * qp * qp;
      if (q > (T)0 && j != i) {
        if (cnt < kMaxNbr) nbr[(size_t)cnt * n_total + i] = j;
        ++cnt;
      }
    }
    acc.add(part);
  }
  nbr_cnt[i] = cnt;
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

// Three-component sum in the precision mode: COMPENSATED adds pair terms
// in float into a partial that is folded into a two-sum accumulator every
// 8 terms (cascaded summation); FP32 is plain; FP64 is double.
template <int P>
struct Acc3 {
  Sum<P> x, y, z;
  Real<P> px = 0, py = 0, pz = 0;
  int n = 0;
  __device__ __forceinline__ void add(Real<P> a, Real<P> b, Real<P> c) {
    if (P == CWA_PREC_COMPENSATED) {
      px += a;
      py += b;
      pz += c;
      if (++n == 8) flush();
    } else {
      x.add(a);
      y.add(b);
      z.add(c);
    }
  }
  __device__ __forceinline__ void flush() {
    if (P == CWA_PREC_COMPENSATED) {
      x.add(px);
      y.add(py);
      z.add(pz);
      px = py = pz = 0;
      n = 0;
    }
  }
};

// force: spiky pressure gradient + viscosity Laplacian over the neighbour
// list written by rho_pres (same pairs, same order as the candidate scan),
// then the preset's extra terms.  A particle whose list overflowed rescans
// its 27-cell block.
template <int P>
__global__ void __launch_bounds__(kNbThreads)
    k_force(const float4* __restrict__ pos, const float4* __restrict__ vel,
            const float2* __restrict__ rho_p, const int32_t* __restrict__ start,
            const Tile* __restrict__ tiles, const SceneDev* __restrict__ scenes,
            const float* __restrict__ wave, float4* __restrict__ force, const int32_t* __restrict__ nbr,
            const int32_t* __restrict__ nbr_cnt, int32_t n_total) {
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
  Acc3<P> fp, fv;
  auto pair = [&](int j) {
    const float4 pj = __ldg(pos + j);
    const float4 vj = __ldg(vel + j);
    const float2 rpj = __ldg(rho_p + j);
    const T dx = px - (T)pj.x, dy = py - (T)pj.y, dz = pz - (T)pj.z;
    const T r2 = dx * dx + dy * dy + dz * dz;
    const T inv_r = r2 > (T)0 ? inv_sqrt(r2) : (T)0;  // normalize(0) := 0
    const T r = r2 * inv_r;
    const T hr = hh - r;
    const T irho = recip((T)rpj.x);
    const T sp = (pres_i + (T)rpj.y) * irho * hr * hr * inv_r;
    fp.add(sp * dx, sp * dy, sp * dz);
    const T sv = irho * hr;
    fv.add(sv * ((T)vj.x - vx), sv * ((T)vj.y - vy), sv * ((T)vj.z - vz));
  };
  const int cnt = __ldg(nbr_cnt + i);
  if (cnt <= kMaxNbr) {
    int jn = cnt > 0 ? __ldg(nbr + i) : 0;
    for (int k = 0; k < cnt; ++k) {
      const int j = jn;
      if (k + 1 < cnt) jn = __ldg(nbr + (size_t)(k + 1) * n_total + i);
      pair(j);
    }
  } else {
    int b[9], e[9];
    row_ranges(S, start, cell_of(S, pi), b, e);
    for (int r = 0; r < 9; ++r)
      for (int j = b[r]; j < e[r]; ++j) {
        const float4 pj = __ldg(pos + j);
        const T dx = px - (T)pj.x, dy = py - (T)pj.y, dz = pz - (T)pj.z;
        if (h2 - (dx * dx + dy * dy + dz * dz) > (T)0 && j != i) pair(j);
      }
  }
  fp.flush();
  fv.flush();
  const T cg = P == CWA_PREC_FP64 ? (T)S->k_grad_d * (T)S->mass : (T)(S->k_grad * S->mass);
  const T cp = (T)0.5 * cg;
  float fpr[3] = {(float)(cp * fp.x.get()), (float)(cp * fp.y.get()), (float)(cp * fp.z.get())};
  float fvr[3] = {(float)(cg * fv.x.get()), (float)(cg * fv.y.get()), (float)(cg * fv.z.get())};
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
      f[c] = fpr[c] + fvr[c] * vs + rho * S->g[c] + tq[c] + drag + wf;
    }
    out = make_float4(f[0], f[1], f[2], fprev.w);
  } else {
    out = make_float4(fpr[0] + fvr[0] * S->visc + rho * S->g[0], fpr[1] + fvr[1] * S->visc + rho * S->g[1],
                      fpr[2] + fvr[2] * S->visc + rho * S->g[2], 0.0f);
  }
  force[i] = out;
}

}  // namespace

cudaError_t launch_rho_pres(int precision, const float4* pos, const int32_t* start, const Tile* tiles,
                            int32_t n_tiles, int32_t tile_size, const SceneDev* scenes,
                            const float* wave_u, float2* rho_p, int32_t* nbr, int32_t* nbr_cnt,
                            int32_t n_total, cudaStream_t stream) {
  if (n_tiles <= 0) return cudaSuccess;
  switch (precision) {
    case CWA_PREC_FP32:
      k_rho_pres<CWA_PREC_FP32><<<n_tiles, tile_size, 0, stream>>>(pos, start, tiles, scenes, wave_u, rho_p, nbr,
                                                                   nbr_cnt, n_total);
      break;
    case CWA_PREC_FP64:
      k_rho_pres<CWA_PREC_FP64><<<n_tiles, tile_size, 0, stream>>>(pos, start, tiles, scenes, wave_u, rho_p, nbr,
                                                                   nbr_cnt, n_total);
      break;
    default:
      k_rho_pres<CWA_PREC_COMPENSATED><<<n_tiles, tile_size, 0, stream>>>(pos, start, tiles, scenes, wave_u,
                                                                          rho_p, nbr, nbr_cnt, n_total);
  }
  return cudaGetLastError();
}

cudaError_t launch_force(int precision, const float4* pos, const float4* vel, const float2* rho_p,
                         const int32_t* start, const Tile* tiles, int32_t n_tiles, int32_t tile_size,
                         const SceneDev* scenes, const float* wave_u, float4* force, const int32_t* nbr,
                         const int32_t* nbr_cnt, int32_t n_total, cudaStream_t stream) {
  if (n_tiles <= 0) return cudaSuccess;
  switch (precision) {
    case CWA_PREC_FP32:
      k_force<CWA_PREC_FP32><<<n_tiles, tile_size, 0, stream>>>(pos, vel, rho_p, start, tiles, scenes, wave_u,
                                                                force, nbr, nbr_cnt, n_total);
      break;
    case CWA_PREC_FP64:
      k_force<CWA_PREC_FP64><<<n_tiles, tile_size, 0, stream>>>(pos, vel, rho_p, start, tiles, scenes, wave_u,
                                                                force, nbr, nbr_cnt, n_total);
      break;
    default:
      k_force<CWA_PREC_COMPENSATED><<<n_tiles, tile_size, 0, stream>>>(pos, vel, rho_p, start, tiles, scenes,
                                                                       wave_u, force, nbr, nbr_cnt, n_total);
  }
  return cudaGetLastError();
}

}  // namespace cwa
