// cwa_step.cu — element-wise passes of the step: integrate + particle<->
// heightfield coupling, the wave leapfrog stencil, wave init, AoS<->SoA
// packing and the FP64 conservation totals.
//
// Integrate and wave are written one rounding per operation (__f*_rn, no FMA
// contraction) so that a float32 restatement of the same operation order on
// the CPU reproduces them bit for bit, deposits included.
#include <cuda_runtime.h>

#include "cwa_device.cuh"
#include "cwa_internal.h"

namespace cwa {
namespace {

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

// integrate_comp.glsl:56-92 + CheckBoundary :135-178 (REFERENCE_3D), or
// symplectic Euler, heightfield coupling and restitution walls (MULLER).
// Coupling (MULLER): a particle that ends the Euler update below the surface
// y0 + u(x, z) deposits its vertical momentum m*vy into the wave cell under
// it as a fixed-point int64 (q = rint(m vy 2^shift), summed with integer
// atomics, so the total is order independent), is pushed back along the
// surface normal (v -= (1+e) (v.n) n when v.n < 0) and placed on the surface.
__global__ void __launch_bounds__(128)
    k_integrate(float4* __restrict__ pos, float4* __restrict__ vel, float4* __restrict__ force,
                float2* __restrict__ rho_p, const Tile* __restrict__ tiles,
                const SceneDev* __restrict__ scenes, const float* __restrict__ wave,
                unsigned long long* __restrict__ deposits, const float4* __restrict__ xref, int32_t* flag,
                int32_t* __restrict__ key, int32_t* __restrict__ slot, int32_t* __restrict__ count,
                int32_t* status) {
  chain_enter();
  const Tile tl = tiles[blockIdx.x];
  const int i = tl.begin + threadIdx.x;
  if (i >= tl.end) return;
  const SceneDev* S = scenes + tl.scene;
  const float4 p = pos[i];
  const float4 v0 = vel[i];
  float4 f = force[i];
  float2 rp = rho_p[i];
  const float dt = S->dt;
  float v[3], x[3];
  {
    const float pp[3] = {p.x, p.y, p.z}, vv[3] = {v0.x, v0.y, v0.z}, ff[3] = {f.x, f.y, f.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float a = __fdiv_rn(ff[c], rp.x);
      v[c] = fadd(vv[c], fmul(dt, a));
      x[c] = fadd(pp[c], fmul(dt, v[c]));
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) v[c] = fmul(v[c], S->damp);
  const float s = fadd(fmul(x[0], S->uvs[0]), S->uvo[0]);
  const float t = fadd(fmul(x[2], S->uvs[1]), S->uvo[1]);
  const float* u = wave + S->woff;
  const int W = S->nx, Hn = S->nz;
  if (S->preset == CWA_PRESET_REFERENCE_3D) {
    const float sp2 = fadd(fadd(fmul(v[0], v[0]), fmul(v[1], v[1])), fmul(v[2], v[2]));
    if (S->foam > 0.0f && __fsqrt_rn(sp2) > S->foam) {
      f.x = fmul(f.x, 0.5f);
      f.y = fmul(f.y, 0.5f);
      f.z = fmul(f.z, 0.5f);
      f.w = fmul(f.w, 0.5f);
      rp.x = fmul(rp.x, 0.1f);
      rp.y = fmul(rp.y, 0.25f);
#pragma unroll
      for (int c = 0; c < 3; ++c) v[c] = fmul(v[c], 0.1f);
      force[i] = f;
      rho_p[i] = rp;
    }
    const float H = sample_height(u, W, Hn, s, t);
    if (x[1] < H) x[1] = fsub(H, S->radius);
  } else {
    float val, gx, gz;
    sample_height_grad(u, W, Hn, s, t, &val, &gx, &gz);
    const float H = fadd(S->y0, val);
    if (x[1] < H) {
      if (S->coupled) {
        const float fs = fminf(fmaxf(floorf(fmul(s, (float)W)), -1.0f), (float)W);
        const float ft = fminf(fmaxf(floorf(fmul(t, (float)Hn)), -1.0f), (float)Hn);
        const int ci = clampi((int)fs, 0, W - 1), ck = clampi((int)ft, 0, Hn - 1);
        const float mv = fmul(S->mass, v[1]);
        float sq = fmul(mv, S->qscale);
        const float lim = 4611686018427387904.0f;  // 2^62
        sq = fminf(fmaxf(sq, -lim), lim);
        const long long q = __float2ll_rn(sq);
        if (!CWA_DCHECK_FAILED(ci >= 0 && ci < W && ck >= 0 && ck < Hn, status))
          atomicAdd(deposits + S->woff + (size_t)ck * W + ci, (unsigned long long)q);
      }
      const float nx = -fmul(gx, fmul((float)W, S->uvs[0]));
      const float nz = -fmul(gz, fmul((float)Hn, S->uvs[1]));
      const float len2 = fadd(fadd(fmul(nx, nx), 1.0f), fmul(nz, nz));
      const float inv = __fdiv_rn(1.0f, __fsqrt_rn(len2));
      const float nrm[3] = {fmul(nx, inv), inv, fmul(nz, inv)};
      const float vn = fadd(fadd(fmul(v[0], nrm[0]), fmul(v[1], nrm[1])), fmul(v[2], nrm[2]));
      if (vn < 0.0f) {
        const float k = fmul(fadd(1.0f, S->e_surf), vn);
#pragma unroll
        for (int c = 0; c < 3; ++c) v[c] = fsub(v[c], fmul(k, nrm[c]));
      }
      x[1] = H;
    }
  }
  const float e = S->e_wall;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (x[c] < S->lo[c]) {
      x[c] = S->lo[c];
      v[c] = fmul(v[c], -e);
    } else if (x[c] > S->hi[c]) {
      x[c] = S->hi[c];
      v[c] = fmul(v[c], -e);
    }
  }
  if (S->line_source && S->preset == CWA_PRESET_REFERENCE_3D) {  // integrate_comp.glsl:170-177
    const float ceil_y = fadd(S->hi[1], 0.1f);
    if (x[1] > ceil_y) {
      x[1] = ceil_y;
      v[1] = fmul(v[1], -e);
    }
  }
  const float4 pn = make_float4(x[0], x[1], x[2], p.w);
  pos[i] = pn;
  vel[i] = make_float4(v[0], v[1], v[2], v0.w);
  if (key) {  // the next grid build's cell hash + count, on the position just written
    if (!finite3(pn)) atomicOr(status, kStatusNonFinite);
    const int ny = S->dims[1], nz = S->dims[2];
    const int k = S->coff + (cell_axis(pn.x, S->lo[0], S->cell, S->dims[0]) * ny +
                             cell_axis(pn.y, S->lo[1], S->cell, ny)) * nz +
                  cell_axis(pn.z, S->lo[2], S->cellz, nz);
    if (CWA_DCHECK_FAILED(k >= S->coff && k < S->coff + S->ncells, status)) return;
    key[i] = k;
    slot[i] = count_slot(count, k);
  }
  if (xref) {  // Verlet mode: has this particle left its skin?
    const float4 r = xref[i];
    const float dx = x[0] - r.x, dy = x[1] - r.y, dz = x[2] - r.z;
    const bool far = dx * dx + dy * dy + dz * dz > S->disp2;
    if (__any_sync(__activemask(), far) && far) atomicOr(flag, 1);
  }
}

// One cell of EvolveWave (wave_comp.glsl:171-206) with get_clamp borders,
// plus the particle deposit d: one rounding per operation, in the order the
// float32 restatement uses.
__device__ __forceinline__ float evolve_cell(const SceneDev* S, float c0, float c1, float nn, float ss, float ee,
                                             float ww, int i, long long d) {
  const float nb = fadd(fadd(nn, ss), fadd(ee, ww));
  float w = fadd(fmul(S->wa, c0), fmul(S->lam, nb));
  w = fsub(w, fmul(S->wb, c1));
  w = fmul(S->atten, w);
  if (S->line_source && w > 0.0001f && i == S->nx / 2) w = fadd(w, 0.001f);
  if (S->coupled) w = fadd(w, fmul(S->gain, fmul(__ll2float_rn(d), S->dq)));
  return w;
}

// The wave pass over every scene: a tile is kWaveCellsPerThread x blockDim
// cells of one scene.  Rows whose width is a multiple of 4 take the float4
// path (4 cells per thread: three float4 rows, two edge scalars, the
// previous field and two 16-byte deposit loads, all independent); other
// widths take the scalar path.  Deposits are read and cleared here.
constexpr int kWaveCellsPerThread = 4;

__global__ void __launch_bounds__(256)
    k_wave(const float* __restrict__ un, const float* __restrict__ unm1, float* __restrict__ uout,
           unsigned long long* __restrict__ deposits, const Tile* __restrict__ tiles,
           const SceneDev* __restrict__ scenes, int32_t* status) {
  chain_enter();
  const Tile tl = tiles[blockIdx.x];
  const SceneDev* S = scenes + tl.scene;
  const int W = S->nx, H = S->nz, woff = S->woff;
  const int local0 = tl.begin - woff + threadIdx.x * kWaveCellsPerThread;
  if (local0 + woff >= tl.end) return;
  if (CWA_DCHECK_FAILED(local0 >= 0 && local0 < W * H && ((W & 3) != 0 || local0 + 3 < W * H), status)) return;
  const float* u = un + woff;
  const float* um = unm1 + woff;
  float* uo = uout + woff;
  unsigned long long* dep = deposits + woff;
  if ((W & 3) == 0) {
    const int j = local0 / W, i = local0 - j * W;
    const float4 C = __ldg(reinterpret_cast<const float4*>(u + local0));
    const float4 N = j + 1 < H ? __ldg(reinterpret_cast<const float4*>(u + local0 + W)) : C;
    const float4 Sd = j > 0 ? __ldg(reinterpret_cast<const float4*>(u + local0 - W)) : C;
    const float west = i > 0 ? __ldg(u + local0 - 1) : C.x;
    const float east = i + 4 < W ? __ldg(u + local0 + 4) : C.w;
    const float4 P = __ldg(reinterpret_cast<const float4*>(um + local0));
    long long d[4] = {0, 0, 0, 0};
    if (S->coupled) {
      const longlong2 a = *reinterpret_cast<const longlong2*>(dep + local0);
      const longlong2 b = *reinterpret_cast<const longlong2*>(dep + local0 + 2);
      d[0] = a.x;
      d[1] = a.y;
      d[2] = b.x;
      d[3] = b.y;
      // clear only what holds a deposit: most cells have none, and a skipped
      // store saves its 16 bytes of DRAM write
      if ((a.x | a.y) != 0) *reinterpret_cast<longlong2*>(dep + local0) = make_longlong2(0, 0);
      if ((b.x | b.y) != 0) *reinterpret_cast<longlong2*>(dep + local0 + 2) = make_longlong2(0, 0);
    }
    float4 o;
    o.x = evolve_cell(S, C.x, P.x, N.x, Sd.x, C.y, west, i, d[0]);
    o.y = evolve_cell(S, C.y, P.y, N.y, Sd.y, C.z, C.x, i + 1, d[1]);
    o.z = evolve_cell(S, C.z, P.z, N.z, Sd.z, C.w, C.y, i + 2, d[2]);
    o.w = evolve_cell(S, C.w, P.w, N.w, Sd.w, east, C.z, i + 3, d[3]);
    *reinterpret_cast<float4*>(uo + local0) = o;
  } else {
    const int ncell = W * H;
#pragma unroll
    for (int k = 0; k < kWaveCellsPerThread; ++k) {
      const int local = local0 + k;
      if (local >= ncell) break;
      const int j = local / W, i = local - j * W;
      long long d = 0;
      if (S->coupled) {
        d = (long long)dep[local];
        if (d != 0) dep[local] = 0ull;
      }
      uo[local] = evolve_cell(S, u[local], um[local], u[min(j + 1, H - 1) * W + i], u[max(j - 1, 0) * W + i],
                              u[j * W + min(i + 1, W - 1)], u[j * W + max(i - 1, 0)], i, d);
    }
  }
}

// InitWave (wave_comp.glsl:82-140): peak * smoothstep(5, 0, d) around two
// (splash) or three (wave, wake) centres.
__global__ void k_wave_init(float* __restrict__ u, int32_t nx, int32_t nz, float mode) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nx * nz) return;
  const int j = c / nx, i = c - j * nx;
  int c0x, c0y, c1x, c1y, c2x, c2y;
  float peak;
  bool three = true;
  if (mode == 1.0f) {
    c0x = (int)fmul(0.25f, (float)nx);
    c0y = (int)fmul(0.25f, (float)nz);
    c1x = (int)fmul(0.75f, (float)nx);
    c1y = (int)fmul(0.75f, (float)nz);
    c2x = c0x;
    c2y = c0y;
    peak = 0.5f;
    three = false;
  } else if (mode == 0.0f) {
    c0x = (int)fmul(0.25f, (float)nx);
    c0y = nz;
    c2x = (int)fmul(0.5f, (float)nx);
    c2y = nz;
    c1x = (int)fmul(0.75f, (float)nx);
    c1y = nz;
    peak = 1.0f;
  } else {
    c0x = (int)fmul(0.5f, (float)nx);
    c0y = (int)fmul(0.1f, (float)nz);
    c1x = c2x = c0x;
    c1y = c2y = c0y;
    peak = 0.1f;
  }
  auto dist = [&](int cx, int cy) {
    const float dx = fsub((float)i, (float)cx), dy = fsub((float)j, (float)cy);
    return __fsqrt_rn(fadd(fmul(dx, dx), fmul(dy, dy)));
  };
  float d = fminf(dist(c0x, c0y), dist(c1x, c1y));
  if (three) d = fminf(d, dist(c2x, c2y));
  float t = __fdiv_rn(fsub(d, 5.0f), fsub(0.0f, 5.0f));
  t = fminf(fmaxf(t, 0.0f), 1.0f);
  const float sm = fmul(fmul(t, t), fsub(3.0f, fmul(2.0f, t)));
  u[c] = fmul(peak, sm);
}

// One thread a 16-byte quarter of a record: a warp reads 512 contiguous
// bytes (8 records) of the source, which may be page-locked host memory
// read over the host link, and writes each quarter's 8 words to its array as
// 128 contiguous bytes.
__global__ void k_unpack(const float4* __restrict__ aos, int32_t n, int32_t poff, float4* __restrict__ pos,
                         float4* __restrict__ vel, float4* __restrict__ force, float2* __restrict__ rho_p,
                         float2* __restrict__ extra, int32_t* __restrict__ id) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= 4L * n) return;
  const int i = (int)(t >> 2), q = (int)(t & 3);
  const float4 v = aos[t];
  if (q == 3) {
    rho_p[poff + i] = make_float2(v.x, v.y);
    extra[poff + i] = make_float2(v.z, v.w);
    id[poff + i] = i;
  } else {
    (q == 0 ? pos : q == 1 ? vel : force)[poff + i] = v;
  }
}

// Contiguous copy of n floats, both pointers 16-byte aligned, either side
// device memory or page-locked host memory: one 16-byte word a thread, and
// the thread past the last whole word copies the 0-3 floats left.
__global__ void k_copy_f32(const float* __restrict__ src, float* __restrict__ dst, long n) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long n4 = n >> 2;
  if (t < n4)
    reinterpret_cast<float4*>(dst)[t] = reinterpret_cast<const float4*>(src)[t];
  else if (t == n4)
    for (long k = n4 * 4; k < n; ++k) dst[k] = src[k];
}

__global__ void k_pack(cwa_particle* __restrict__ aos, int32_t n, int32_t poff, const float4* __restrict__ pos,
                       const float4* __restrict__ vel, const float4* __restrict__ force,
                       const float2* __restrict__ rho_p, const float2* __restrict__ extra,
                       const int32_t* __restrict__ id) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = id[poff + i];
  if (k < 0 || k >= n) return;
  float4* q = reinterpret_cast<float4*>(aos + k);
  const float2 rp = rho_p[poff + i];
  const float2 ex = extra[poff + k];
  q[0] = pos[poff + i];
  q[1] = vel[poff + i];
  q[2] = force[poff + i];
  q[3] = make_float4(rp.x, rp.y, ex.x, ex.y);
}

constexpr int kTotBlocks = kTotalsBlocks;
constexpr int kTotThreads = 256;

// Per-block FP64 partial sums in a fixed order, then one block adds the
// partials in block order: the totals are deterministic run to run.
__global__ void __launch_bounds__(kTotThreads)
    k_totals_partial(const float4* __restrict__ pos, const float4* __restrict__ vel, int32_t poff, int32_t n,
                     const float* __restrict__ un, const float* __restrict__ unm1, int32_t woff, int32_t nw,
                     const SceneDev* __restrict__ scenes, int32_t scene, double* __restrict__ partial) {
  const SceneDev* S = scenes + scene;
  double t[CWA_TOTALS_COUNT] = {0, 0, 0, 0, 0, 0, 0, 0};
  const double m = S->mass;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = pos[poff + i], v = vel[poff + i];
    t[CWA_TOTAL_MASS] += m;
    t[CWA_TOTAL_MOMENTUM_X] += m * v.x;
    t[CWA_TOTAL_MOMENTUM_Y] += m * v.y;
    t[CWA_TOTAL_MOMENTUM_Z] += m * v.z;
    t[CWA_TOTAL_KINETIC] += 0.5 * m * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
    t[CWA_TOTAL_POTENTIAL] -= m * ((double)S->g[0] * ((double)p.x - S->lo[0]) +
                                   (double)S->g[1] * ((double)p.y - S->lo[1]) +
                                   (double)S->g[2] * ((double)p.z - S->lo[2]));
  }
  const double area = ((double)S->hi[0] - S->lo[0]) / S->nx * (((double)S->hi[2] - S->lo[2]) / S->nz);
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nw; c += gridDim.x * blockDim.x) {
    const double a = un[woff + c], b = unm1[woff + c];
    t[CWA_TOTAL_WAVE_VOLUME] += a * area;
    t[CWA_TOTAL_WAVE_ENERGY] += 0.5 * (a * a + (a - b) * (a - b)) * area;
  }
  __shared__ double sh[kTotThreads / 32][CWA_TOTALS_COUNT];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < CWA_TOTALS_COUNT; ++k) {
    double x = t[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[warp][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < CWA_TOTALS_COUNT) {
    double x = 0.0;
    for (int w = 0; w < kTotThreads / 32; ++w) x += sh[w][threadIdx.x];
    partial[blockIdx.x * CWA_TOTALS_COUNT + threadIdx.x] = x;
  }
}

__global__ void k_totals_final(const double* __restrict__ partial, double* __restrict__ out) {
  if (threadIdx.x < CWA_TOTALS_COUNT) {
    double x = 0.0;
    for (int b = 0; b < kTotBlocks; ++b) x += partial[b * CWA_TOTALS_COUNT + threadIdx.x];
    out[threadIdx.x] = x;
  }
}

inline int blocks_for(long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

cudaError_t launch_integrate(float4* pos, float4* vel, float4* force, float2* rho_p, const Tile* tiles,
                             int32_t n_tiles, int32_t tile_size, const SceneDev* scenes,
                             const float* wave_u, unsigned long long* deposits, const float4* xref,
                             int32_t* flag, int32_t* key, int32_t* slot, int32_t* count, int32_t* status,
                             cudaStream_t stream) {
  if (n_tiles <= 0) return cudaSuccess;
  k_integrate<<<n_tiles, tile_size, 0, stream>>>(pos, vel, force, rho_p, tiles, scenes, wave_u, deposits, xref,
                                                 flag, key, slot, count, status);
  return cudaGetLastError();
}

cudaError_t launch_wave(const float* u_n, const float* u_nm1, float* u_out, unsigned long long* deposits,
                        const Tile* wtiles, int32_t n_wtiles, int32_t wtile_size, const SceneDev* scenes,
                        cudaStream_t stream, int32_t* status) {
  if (n_wtiles <= 0) return cudaSuccess;
  launch_chained(k_wave, dim3(n_wtiles), dim3(wtile_size / kWaveCellsPerThread), 0, stream, u_n, u_nm1, u_out,
                 deposits, wtiles, scenes, status);
  return cudaGetLastError();
}

// InitFromImage (wave_comp.glsl:76-80): cell (x, y) takes the red channel of
// texel (2x, y) of an RGBA8 texture as a normalised float, c / 255.  The
// shader's texelFetch past the image is undefined; here it reads 0.
__global__ void k_wave_from_image(float* __restrict__ u, int32_t nx, int32_t nz,
                                  const uint8_t* __restrict__ rgba, int32_t w, int32_t h) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nx * nz) return;
  const int y = c / nx, x = c - y * nx;
  const int tx = 2 * x;
  u[c] = (tx < w && y < h) ? __fdiv_rn((float)rgba[((size_t)y * w + tx) * 4], 255.0f) : 0.0f;
}

cudaError_t launch_wave_from_image(float* u, int32_t nx, int32_t nz, const uint8_t* rgba, int32_t w, int32_t h,
                                   cudaStream_t stream) {
  long n = (long)nx * nz;
  if (n <= 0) return cudaSuccess;
  k_wave_from_image<<<blocks_for(n, 256), 256, 0, stream>>>(u, nx, nz, rgba, w, h);
  return cudaGetLastError();
}

cudaError_t launch_wave_init(float* u, int32_t nx, int32_t nz, float mode, cudaStream_t stream) {
  long n = (long)nx * nz;
  if (n <= 0) return cudaSuccess;
  k_wave_init<<<blocks_for(n, 256), 256, 0, stream>>>(u, nx, nz, mode);
  return cudaGetLastError();
}

cudaError_t launch_unpack(const cwa_particle* aos, int32_t n, int32_t poff, float4* pos, float4* vel,
                          float4* force, float2* rho_p, float2* extra, int32_t* id, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_unpack<<<blocks_for(4L * n, 256), 256, 0, stream>>>(reinterpret_cast<const float4*>(aos), n, poff, pos, vel,
                                                         force, rho_p, extra, id);
  return cudaGetLastError();
}

cudaError_t launch_copy_f32(const float* src, float* dst, long n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  if ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) return cudaErrorInvalidValue;
  k_copy_f32<<<blocks_for((n >> 2) + 1, 256), 256, 0, stream>>>(src, dst, n);
  return cudaGetLastError();
}

cudaError_t launch_pack(cwa_particle* aos, int32_t n, int32_t poff, const float4* pos, const float4* vel,
                        const float4* force, const float2* rho_p, const float2* extra,
                        const int32_t* id, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_pack<<<blocks_for(n, 256), 256, 0, stream>>>(aos, n, poff, pos, vel, force, rho_p, extra, id);
  return cudaGetLastError();
}

cudaError_t launch_totals(const float4* pos, const float4* vel, int32_t poff, int32_t n,
                          const float* u_n, const float* u_nm1, int32_t woff, int32_t nw,
                          const SceneDev* scenes, int32_t scene, double* out, cudaStream_t stream) {
  // `out` holds kTotBlocks * 8 partials followed by the 8 totals.
  k_totals_partial<<<kTotBlocks, kTotThreads, 0, stream>>>(pos, vel, poff, n, u_n, u_nm1, woff, nw, scenes,
                                                           scene, out);
  k_totals_final<<<1, 32, 0, stream>>>(out, out + kTotBlocks * CWA_TOTALS_COUNT);
  return cudaGetLastError();
}

}  // namespace cwa
