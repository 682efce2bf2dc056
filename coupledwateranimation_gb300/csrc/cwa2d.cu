// cwa2d.cu — the 2D solver family (the reference's SphWave2D app).
//
// Cubic-spline SPH with signed-distance walls (SphWaveKoschier2D_grid_cs.glsl
// :233-627) over a uniform grid (SphUgrid::Compute, StencilBuffer.cpp:150-179:
// per substep a grid build, the density pass and the force pass, each pass
// reading one particle buffer and writing the other), driven by a 1D
// shallow-water field advanced with a two-phase Lax-Wendroff step
// (Shallow1D_cs.glsl:110-167, ImageStencil::Compute,
// StencilImage2D.cpp:141-163).  A frame is the SPH substeps followed by the
// wave substeps (SphWave2D/Main.cpp:220-241: the SPH of frame n samples the
// field left by frame n - 1).
//
// GB300 form: structure-of-arrays particle state, the grid built with the
// library's stable counting sort (hash + warp-aggregated count, single-pass
// scan, stable insert / rank), so each cell's members come in upload order
// and every sum is deterministic; the whole frame replays from a CUDA graph.
// Differences from the shader, by design:
//   * texture(wave_tex, x) is exact float linear interpolation with
//     CLAMP_TO_EDGE (texture units use 8-bit weights);
//   * a coincident distinct neighbour (r = 0) contributes no pressure or
//     viscosity term (rij / r is NaN in the shader);
//   * the predictor's two stores to cells 0 and size-1 race in the shader
//     (FreeBC's neighbour copy and the unconditional store); the cell's own
//     half-step value is kept, the one the corrector at cell 1 needs.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <string>

#include "cwa_device.cuh"
#include "cwa_internal.h"

namespace cwa {
namespace {

// Constants of the shader, evaluated once on the host in float.
struct Sph2dConst {
  int n, ncx, ncy, wave_n, cols;
  float R, H, HSQ, rest, visc, mass, dt, gas, k2, psi;
  float view_w, view_h;
  float cell_x, cell_y;
  float plane0_c;  // floor plane offset: -0.5 VIEW_HEIGHT + 15 R - R + bottom
  float lambda, dx;
  int wave_kind;
  float w1_a, w1_b, w1_atten, w1_half;  // Wave1D: 2 - 2 lambda - beta, 1 - beta, atten, 0.5 lambda
};

__device__ __forceinline__ float w_cubic(const Sph2dConst& c, float r) {
  const float q = r / c.H;
  if (q >= 1.0f) return 0.0f;
  if (q <= 0.5f) return c.k2 * (6.0f * q * q * (q - 1.0f) + 1.0f);
  const float q1 = 1.0f - q;
  return c.k2 * 2.0f * q1 * q1 * q1;
}

__device__ __forceinline__ float w_cubic_grad(const Sph2dConst& c, float r) {
  const float q = r / c.H;
  if (q >= 1.0f) return 0.0f;
  if (q <= 0.5f) return 6.0f * c.k2 * q * (3.0f * q - 2.0f) / c.H;
  const float q1 = 1.0f - q;
  return -6.0f * c.k2 * (q1 * q1) / c.H;
}

__device__ __forceinline__ float smoothstepf(float e0, float e1, float x) {
  float t = (x - e0) / (e1 - e0);
  t = fminf(fmaxf(t, 0.0f), 1.0f);
  return t * t * (3.0f - 2.0f * t);
}

// boundary_sdf (:187-213): the nearest of four planes, (nx, ny, distance).
__device__ __forceinline__ float3 boundary_sdf(const Sph2dConst& c, float px, float py) {
  const float d0 = 0.0f * px + 1.0f * py + c.plane0_c;
  const float d1 = 1.0f * px + 0.0f * py - c.R;
  const float d2 = -1.0f * px + 0.0f * py + (c.view_w - c.R);
  const float d3 = 0.0f * px + -1.0f * py + (c.view_h - c.R);
  float3 r = make_float3(0.0f, 1.0f, d0);
  if (d1 < r.z) r = make_float3(1.0f, 0.0f, d1);
  if (d2 < r.z) r = make_float3(-1.0f, 0.0f, d2);
  if (d3 < r.z) r = make_float3(0.0f, -1.0f, d3);
  return r;
}

// texture(wave_tex, coord) on the 1D RGBA32F field: linear, clamp to edge.
__device__ __forceinline__ float2 wave_tex(const float4* __restrict__ w, int n, float coord) {
  const float u = coord * (float)n - 0.5f;
  const float u0 = floorf(u), f = u - u0;
  const int i0 = min(max((int)u0, 0), n - 1), i1 = min(max((int)u0 + 1, 0), n - 1);
  const float4 a = w[i0], b = w[i1];
  return make_float2((1.0f - f) * a.x + f * b.x, (1.0f - f) * a.y + f * b.y);
}

// GetWaveNormalHeight (:280-297): normal (nx, ny), height, and uh / h.
__device__ __forceinline__ void wave_normal_height(const Sph2dConst& c, const float4* __restrict__ w, float x,
                                                   float* nx, float* ny, float* h, float* xvel) {
  const float coord = x / c.view_w;
  const float inv = 1.0f / (float)c.wave_n;
  const float2 m = wave_tex(w, c.wave_n, coord);
  const float2 e = wave_tex(w, c.wave_n, coord - inv);
  const float2 ww = wave_tex(w, c.wave_n, coord + inv);
  const float ax = e.x - ww.x, len = sqrtf(ax * ax + 1.0f);
  *nx = ax / len;
  *ny = 1.0f / len;
  *h = m.x;
  *xvel = m.y / m.x;
}

__device__ __forceinline__ int cell_i(const Sph2dConst& c, float p, int axis) {
  const float lo = 0.0f;
  return axis == 0 ? cell_axis(p, lo, c.cell_x, c.ncx) : cell_axis(p, lo, c.cell_y, c.ncy);
}

// A point enters the cell of its position only when it lies strictly inside
// the grid's extents [0, view] (point_in_aabb, uniform_grid_sph_cs.glsl:19-23,
// 101-105); the others go to bucket ncx * ncy past the last cell, which no
// neighbour search visits, so they are invisible, to themselves too.
__global__ void k2_hash(Sph2dConst c, const float4* __restrict__ pos, int32_t* __restrict__ key,
                        int32_t* __restrict__ slot, int32_t* __restrict__ count, int32_t* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  const float4 p = pos[i];
  if (!finite3(make_float4(p.x, p.y, 0.0f, 0.0f))) atomicOr(status, kStatusNonFinite);
  const bool inside = p.x > 0.0f && p.y > 0.0f && p.x < c.view_w && p.y < c.view_h;
  const int k = inside ? cell_i(c, p.x, 0) * c.ncy + cell_i(c, p.y, 1)  // Index(i, j) = i * ny + j
                       : c.ncx * c.ncy;
  key[i] = k;
  slot[i] = count_slot(count, k);
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One warp per particle: the lanes split each neighbour cell's members
// (member k goes to lane k mod 32) and the partial sums meet in a fixed
// butterfly, so the result does not depend on scheduling.  (A thread per
// particle walked ~80 candidates through dependent loads: 16 CTAs on a
// 4096-particle scene, latency bound.)
constexpr int kWarpsPerBlock = 8;

// ComputeDensityPressure (:372-479).
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    k2_density(Sph2dConst c, const float4* __restrict__ pin, const float4* __restrict__ vin,
               const float4* __restrict__ ain, float4* __restrict__ pout, float4* __restrict__ vout,
               float4* __restrict__ aout, const int32_t* __restrict__ start, const int32_t* __restrict__ sorted,
               const float4* __restrict__ wave) {
  const int ix = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (ix >= c.n) return;  // whole warps leave together
  float4 p = pin[ix], v = vin[ix], a = ain[ix];
  float nx, ny, h, xvel;
  wave_normal_height(c, wave, p.x, &nx, &ny, &h, &xvel);
  const float thresh = 0.05f;
  if (p.w == 0.0f && fabsf(xvel) > thresh) p.w = 1.0f;  // enable inside the moving wave
  if (p.w == 1.0f && fabsf(xvel) < thresh) p.w = 0.0f;  // disable where it is at rest
  const float3 db = boundary_sdf(c, p.x, p.y);
  if (db.z < 0.0f) {
    p.x -= 0.75f * db.z * db.x;  // unpenetrate
    p.y -= 0.75f * db.z * db.y;
    const float vn = fminf(0.0f, v.x * db.x + v.y * db.y);
    v.x -= 1.75f * vn * db.x;
    v.y -= 1.75f * vn * db.y;
  }
  if (p.y > c.view_h) {
    if (lane == 0) {
      pout[ix] = p;
      vout[ix] = v;
      aout[ix] = a;
    }
    return;
  }
  float rho = 0.0f;
  const int x0 = cell_i(c, p.x - c.H, 0), x1 = cell_i(c, p.x + c.H, 0);
  const int y0 = cell_i(c, p.y - c.H, 1), y1 = cell_i(c, p.y + c.H, 1);
  for (int ci = x0; ci <= x1; ++ci)
    for (int cj = y0; cj <= y1; ++cj) {
      const int cell = ci * c.ncy + cj;
      for (int k = start[cell] + lane; k < start[cell + 1]; k += 32) {
        const float4 q = pin[sorted[k]];
        const float rx = p.x - q.x, ry = p.y - q.y;
        const float r2 = rx * rx + ry * ry;
        if (r2 < c.HSQ) rho += w_cubic(c, sqrtf(r2));
      }
    }
  rho = warp_sum_f(rho);
  if (lane != 0) return;
  rho = c.mass * rho;
  if (db.z < c.H) rho += c.psi * w_cubic(c, fmaxf(0.0f, db.z + 0.0f * c.R));
  rho = fmaxf(c.rest, rho);
  a.w = rho;
  v.w = c.gas * (powf(rho / c.rest, 3.0f) - 1.0f);  // WeaklyCompressibleStateEqn, gamma 3
  pout[ix] = p;
  vout[ix] = v;
  aout[ix] = a;
}

// ComputeForces (:482-627), forward Euler at the end; one warp per particle.
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    k2_force(Sph2dConst c, const float4* __restrict__ pin, const float4* __restrict__ vin,
             const float4* __restrict__ ain, float4* __restrict__ pout, float4* __restrict__ vout,
             float4* __restrict__ aout, const int32_t* __restrict__ start, const int32_t* __restrict__ sorted,
             const float4* __restrict__ wave) {
  const int ix = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (ix >= c.n) return;
  float4 p = pin[ix], v = vin[ix], a = ain[ix];
  if (p.w == 0.0f) {
    if (lane == 0) {
      pout[ix] = p;
      vout[ix] = v;
      aout[ix] = a;
    }
    return;
  }
  const float rho_i = a.w;
  float apx = 0.0f, apy = 0.0f, avx = 0.0f, avy = 0.0f;
  const float c_visc = -c.visc * 8.0f * c.mass;
  const float c_press = c.mass;
  const float api = v.w / (rho_i * rho_i);
  const int x0 = cell_i(c, p.x - c.H, 0), x1 = cell_i(c, p.x + c.H, 0);
  const int y0 = cell_i(c, p.y - c.H, 1), y1 = cell_i(c, p.y + c.H, 1);
  for (int ci = x0; ci <= x1; ++ci)
    for (int cj = y0; cj <= y1; ++cj) {
      const int cell = ci * c.ncy + cj;
      for (int k = start[cell] + lane; k < start[cell + 1]; k += 32) {
        const int jx = sorted[k];
        if (jx == ix) continue;
        const float4 q = pin[jx];
        const float rx = p.x - q.x, ry = p.y - q.y;
        const float r = sqrtf(rx * rx + ry * ry);
        if (r < c.H && r > 0.0f) {
          const float wg = w_cubic_grad(c, r);
          const float ux = rx / r, uy = ry / r;
          const float4 vj = vin[jx];
          const float rho_j = ain[jx].w;
          const float sp = (api + vj.w / (rho_j * rho_j)) * wg;
          apx -= sp * ux;
          apy -= sp * uy;
          const float vxij = v.x - vj.x, vyij = v.y - vj.y;
          const float sv = 1.0f / rho_j * (vxij * rx + vyij * ry) / (r * r + 0.01f * c.HSQ) * wg;
          avx -= sv * ux;
          avy -= sv * uy;
        }
      }
    }
  apx = warp_sum_f(apx);
  apy = warp_sum_f(apy);
  avx = warp_sum_f(avx);
  avy = warp_sum_f(avy);
  if (lane != 0) return;
  avx *= c_visc;
  avy *= c_visc;
  apx *= c_press;
  apy *= c_press;
  const float3 db = boundary_sdf(c, p.x, p.y);
  if (db.z < c.H) {
    const float wg = w_cubic_grad(c, fmaxf(0.0f, db.z + 0.0f * c.R));
    apx += c.psi * api * wg * -db.x;
    apy += c.psi * api * wg * -db.y;
  }
  float nx, ny, h, vx;
  wave_normal_height(c, wave, p.x, &nx, &ny, &h, &vx);
  const float dh = h - c.view_h / 2.0f;
  const float wave_mask = smoothstepf(0.0f, 0.2f, fabsf(vx));
  float dy = p.y - h;
  dy -= 0.5f * dh;
  float tro_y = 0.0f;
  if (ix % 5 < 4) tro_y -= wave_mask * 500000.0f * smoothstepf(0.0f, 10.0f, dy);  // wave pressure
  a.x = apx + avx + 0.0f + 0.0f;
  a.y = apy + avy + -9.8f + tro_y;
  v.x += c.dt * a.x;
  v.y += c.dt * a.y;
  p.x += c.dt * v.x;
  p.y += c.dt * v.y;
  pout[ix] = p;
  vout[ix] = v;
  aout[ix] = a;
}

// InitParticle / init_grid (:308-333).
__global__ void k2_init_particles(Sph2dConst c, float4* __restrict__ pos, float4* __restrict__ vel,
                                  float4* __restrict__ acc) {
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;
  if (ix >= c.n) return;
  const int cols = c.cols, rows = c.n / cols;
  const float xy0 = __fdiv_rn((float)(ix % cols), (float)cols), xy1 = __fdiv_rn((float)(ix / cols), (float)rows);
  const float px = __fadd_rn(__fmul_rn(c.view_w, xy0), c.R);
  const float y0 = __fadd_rn(__fsub_rn(__fmul_rn(0.5f, c.view_h), __fmul_rn(15.0f, c.R)), c.R);
  const float py = __fadd_rn(__fmul_rn(__fmul_rn(18.0f, c.H), xy1), y0);
  pos[ix] = make_float4(px, py, 0.0f, 1.0f);
  vel[ix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  acc[ix] = make_float4(0.0f, 0.0f, 0.0f, c.rest);
}

// Shallow1D InitWave (mode 0) and Splash (mode 1), Shallow1D_cs.glsl:88-117.
__global__ void k2_wave_init(Sph2dConst c, const float4* __restrict__ in, float4* __restrict__ out, int splash) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.wave_n) return;
  const float x = (float)i / (float)(c.wave_n - 1), xc = x - 0.5f;
  const float sgn = xc > 0.0f ? 1.0f : (xc < 0.0f ? -1.0f : 0.0f);
  if (splash) {
    float4 o = in[i];
    const float h = -c.view_h * 0.1f * expf(-xc * xc / 0.005f);
    o.x += h;
    o.y += 0.2f * fabsf(h) * sgn;
    out[i] = o;
  } else {
    const float h = c.view_h * 0.1f * expf(-xc * xc / 0.005f);
    out[i] = make_float4(c.view_h * 0.5f + h, 0.5f * fabsf(h) * sgn, 0.0f, 0.0f);
  }
}

__device__ __forceinline__ float4 load_or_zero(const float4* w, int i, int n) {
  return (i >= 0 && i < n) ? w[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// IterateWave (:119-148) with FreeBC (:157-174).  Phase 0: half-step values
// (hm, uhm) between cells i and i+1; phase 1: the full step from them.
__global__ void k2_wave_iter(Sph2dConst c, const float4* __restrict__ in, float4* __restrict__ out, int phase) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = c.wave_n;
  if (i >= n) return;
  const float G = 9.8f, lam = c.lambda, dx = c.dx;
  const float hl = __fdiv_rn(lam, 2.0f);
  // flux of (h, uh): uh^2 / h + g h^2 / 2, one rounding per operation
  auto flux = [G](float h, float uh) {
    return __fadd_rn(__fdiv_rn(__fmul_rn(uh, uh), h), __fmul_rn(__fmul_rn(__fmul_rn(0.5f, G), h), h));
  };
  const float4 cc = in[i];
  float4 w = cc;
  if (phase == 0) {
    const float4 e = load_or_zero(in, i + 1, n);
    w.z = __fsub_rn(__fdiv_rn(__fadd_rn(cc.x, e.x), 2.0f), __fdiv_rn(__fmul_rn(hl, __fsub_rn(e.y, cc.y)), dx));
    w.w = __fsub_rn(__fdiv_rn(__fadd_rn(cc.y, e.y), 2.0f),
                    __fdiv_rn(__fmul_rn(hl, __fsub_rn(flux(e.x, e.y), flux(cc.x, cc.y))), dx));
    out[i] = w;  // every cell keeps its own half-step value (cells 0 and size-1 included)
  } else {
    const float4 ww = load_or_zero(in, i - 1, n);
    w.x = __fsub_rn(cc.x, __fdiv_rn(__fmul_rn(lam, __fsub_rn(cc.w, ww.w)), dx));
    w.y = __fsub_rn(cc.y, __fdiv_rn(__fmul_rn(lam, __fsub_rn(flux(cc.z, cc.w), flux(ww.z, ww.w))), dx));
    if (i == 0 || i == n - 1) return;  // FreeBC: written by the neighbours
    out[i] = w;
    if (i == 1) out[0] = w;
    if (i == n - 2) out[n - 1] = w;
  }
}

// Wave1D_cs.glsl (the 2D app's other wave kind), one rounding per operation.
// get_n (:198-207): c1 from the older field, c0 / e0 / w0 from the newest,
// out-of-range loads read zero.  FreeBC (:148-166): cells 0 and n-1 store
// nothing themselves; cells 1 and n-2 copy their value outward.
__device__ __forceinline__ void w1_vel_acc(float4& w, float c0x, float c1x) {
  const float v = __fdiv_rn(__fsub_rn(w.x, c1x), 2.0f);
  const float a = __fadd_rn(__fsub_rn(w.x, __fmul_rn(2.0f, c0x)), c1x);
  w.y = v;
  w.z = a;
}

__device__ __forceinline__ void w1_store_free(float4* out, int i, int n, const float4& w) {
  if (i == 0 || i == n - 1) return;
  out[i] = w;
  if (i == 1) out[0] = w;
  if (i == n - 2) out[n - 1] = w;
}

// InitWave (:98-118).  Mode 0: the Gaussian bump at int(0.25 n).  Mode 1:
// the invocation's Gaussian store is overwritten by its later FreeBC stores
// of w = c0 - 0.5 lambda (e0 - 2 c0 + w0), so only those are made.
__global__ void k1_wave_init(Sph2dConst c, const float4* __restrict__ cur, const float4* __restrict__ prev,
                             float4* __restrict__ out, int mode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = c.wave_n;
  if (i >= n) return;
  if (mode == 0) {
    const int x = (int)(0.25f * (float)n) - i;
    const int xx = (int)((uint32_t)(-x) * (uint32_t)x);  // the shader's int product, wrapping
    const float h = __fadd_rn(0.0f, __fmul_rn(0.1f, expf(__fdiv_rn((float)xx, 5000.0f))));
    out[i] = make_float4(h, 0.0f, 0.0f, 0.0f);
    return;
  }
  const float4 c0 = cur[i], c1 = prev[i];
  const float4 e0 = load_or_zero(cur, i + 1, n), w0 = load_or_zero(cur, i - 1, n);
  auto half = [&c](float cc, float e, float w) {
    return __fsub_rn(cc, __fmul_rn(c.w1_half, __fadd_rn(__fsub_rn(e, __fmul_rn(2.0f, cc)), w)));
  };
  float4 w = make_float4(half(c0.x, e0.x, w0.x), half(c0.y, e0.y, w0.y), half(c0.z, e0.z, w0.z),
                         half(c0.w, e0.w, w0.w));
  w1_vel_acc(w, c0.x, c1.x);
  w1_store_free(out, i, n, w);
}

// IterateWave (:120-131): w = atten ((2 - 2 lambda - beta) c0 + lambda (e0 + w0)
// - (1 - beta) c1), then velocity and acceleration, then FreeBC.
__global__ void k1_wave_iter(Sph2dConst c, const float4* __restrict__ cur, const float4* __restrict__ prev,
                             float4* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = c.wave_n;
  if (i >= n || i == 0 || i == n - 1) return;  // FreeBC: cells 0 and n-1 are written by their neighbours
  const float4 c0 = cur[i], c1 = prev[i], e0 = cur[i + 1], w0 = cur[i - 1];
  auto step = [&c](float cc, float cp, float e, float w) {
    const float t = __fadd_rn(__fmul_rn(c.w1_a, cc), __fmul_rn(c.lambda, __fadd_rn(e, w)));
    return __fmul_rn(c.w1_atten, __fsub_rn(t, __fmul_rn(c.w1_b, cp)));
  };
  float4 w = make_float4(step(c0.x, c1.x, e0.x, w0.x), step(c0.y, c1.y, e0.y, w0.y), step(c0.z, c1.z, e0.z, w0.z),
                         step(c0.w, c1.w, e0.w, w0.w));
  w1_vel_acc(w, c0.x, c1.x);
  w1_store_free(out, i, n, w);
}

constexpr int kBlock = 256;
inline unsigned blocks(int n) { return (unsigned)((n + kBlock - 1) / kBlock); }

}  // namespace
}  // namespace cwa

using namespace cwa;

struct cwa2d_sim {
  int device = 0;
  cwa2d_params prm{};
  Sph2dConst k{};
  cudaStream_t stream = nullptr;
  float4 *P[2] = {}, *V[2] = {}, *A[2] = {};
  // wave buffers: W[wcur] is the newest field; the shallow-water kind
  // writes W[wcur ^ 1], Wave1D writes W[(wcur + 1) % 3] and reads the older
  // field from W[(wcur + 2) % 3]
  float4* W[3] = {};
  int cur = 0, wcur = 0;
  int32_t *key = nullptr, *slot = nullptr, *count = nullptr, *start = nullptr, *list = nullptr, *sorted = nullptr;
  void* scan_ws = nullptr;
  ScanWorkspace scan{};
  int32_t* d_status = nullptr;
  bool grid_fresh = false;
  cudaGraphExec_t graph[3] = {};  // one frame, per wave-buffer phase wcur
  cwa2d_particle* staging = nullptr;
};

namespace {

cwa_status err2(const std::string& m, cwa_status s = CWA_ERR_INVALID_ARG) {
  cwa::set_error(m);
  return s;
}

#define CWA2_CUDA(expr)                                                  \
  do {                                                                   \
    cudaError_t e_ = (expr);                                             \
    if (e_ != cudaSuccess) {                                             \
      cwa::set_error(std::string(#expr) + ": " + cudaGetErrorString(e_)); \
      cudaGetLastError(); /* clear a non-sticky error for the next call */ \
      return e_ == cudaErrorMemoryAllocation ? CWA_ERR_OOM : CWA_ERR_CUDA; \
    }                                                                    \
  } while (0)

void free2d(cwa2d_sim* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (cudaGraphExec_t& g : s->graph)
    if (g) cudaGraphExecDestroy(g);
  for (int b = 0; b < 2; ++b) {
    cudaFree(s->P[b]);
    cudaFree(s->V[b]);
    cudaFree(s->A[b]);
  }
  for (float4* w : s->W) cudaFree(w);
  cudaFree(s->key);
  cudaFree(s->slot);
  cudaFree(s->count);
  cudaFree(s->start);
  cudaFree(s->list);
  cudaFree(s->sorted);
  cudaFree(s->scan_ws);
  cudaFree(s->d_status);
  cudaFree(s->staging);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

cwa_status pass_grid(cwa2d_sim* s) {
  const Sph2dConst& c = s->k;
  const int nb = c.ncx * c.ncy + 1;  // the cells and the outside bucket
  k2_hash<<<blocks(c.n), kBlock, 0, s->stream>>>(c, s->P[s->cur], s->key, s->slot, s->count, s->d_status);
  CWA2_CUDA(cudaGetLastError());
  CWA2_CUDA(scan_launch(s->count, s->start, nb, nb + 1, true, s->scan, s->d_status, s->stream, nullptr));
  CWA2_CUDA(launch_list_insert(s->key, s->slot, s->start, s->list, c.n, nullptr, s->stream));
  CWA2_CUDA(launch_point_rank(s->key, s->slot, s->start, s->list, c.n, s->sorted, s->d_status, s->stream));
  s->grid_fresh = true;
  return CWA_OK;
}

cwa_status pass_sph(cwa2d_sim* s, bool density) {
  const int a = s->cur, b = a ^ 1;
  const unsigned grid = (unsigned)((s->k.n + kWarpsPerBlock - 1) / kWarpsPerBlock);
  if (density)
    k2_density<<<grid, 32 * kWarpsPerBlock, 0, s->stream>>>(s->k, s->P[a], s->V[a], s->A[a], s->P[b], s->V[b],
                                                              s->A[b], s->start, s->sorted, s->W[s->wcur]);
  else
    k2_force<<<grid, 32 * kWarpsPerBlock, 0, s->stream>>>(s->k, s->P[a], s->V[a], s->A[a], s->P[b], s->V[b],
                                                            s->A[b], s->start, s->sorted, s->W[s->wcur]);
  CWA2_CUDA(cudaGetLastError());
  s->cur = b;  // StencilBuffer::PingPong
  if (!density) s->grid_fresh = false;
  return CWA_OK;
}

cwa_status pass_wave(cwa2d_sim* s, int phase) {
  k2_wave_iter<<<blocks(s->k.wave_n), kBlock, 0, s->stream>>>(s->k, s->W[s->wcur], s->W[s->wcur ^ 1], phase);
  CWA2_CUDA(cudaGetLastError());
  s->wcur ^= 1;  // ImageStencil::PingPong
  return CWA_OK;
}

// Wave1D: one dispatch into the write buffer, then the three-buffer rotation
// (ImageStencil::PingPong with two read images: the new field becomes the
// newest, the newest the older one).
cwa_status pass_wave1d(cwa2d_sim* s, int init_mode) {
  const int w = s->wcur, nxt = (w + 1) % 3, old = (w + 2) % 3;
  if (init_mode >= 0)
    k1_wave_init<<<blocks(s->k.wave_n), kBlock, 0, s->stream>>>(s->k, s->W[w], s->W[old], s->W[nxt], init_mode);
  else
    k1_wave_iter<<<blocks(s->k.wave_n), kBlock, 0, s->stream>>>(s->k, s->W[w], s->W[old], s->W[nxt]);
  CWA2_CUDA(cudaGetLastError());
  s->wcur = nxt;
  return CWA_OK;
}

void drop_graphs2(cwa2d_sim* s) {
  for (cudaGraphExec_t& g : s->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

cwa_status enqueue_frame(cwa2d_sim* s) {
  for (int sub = 0; sub < s->prm.sph_substeps; ++sub) {
    cwa_status st = pass_grid(s);
    if (st == CWA_OK) st = pass_sph(s, true);
    if (st == CWA_OK) st = pass_sph(s, false);
    if (st != CWA_OK) return st;
  }
  for (int sub = 0; sub < s->prm.wave_substeps; ++sub) {
    cwa_status st = CWA_OK;
    if (s->k.wave_kind == CWA2D_WAVE_1D) {
      st = pass_wave1d(s, -1);
    } else {
      st = pass_wave(s, 0);
      if (st == CWA_OK) st = pass_wave(s, 1);
    }
    if (st != CWA_OK) return st;
  }
  return CWA_OK;
}

cwa_status read_status2(cwa2d_sim* s) {
  int32_t v = 0;
  CWA2_CUDA(cudaMemcpyAsync(&v, s->d_status, 4, cudaMemcpyDeviceToHost, s->stream));
  CWA2_CUDA(cudaStreamSynchronize(s->stream));
  if (v == 0) return CWA_OK;
  CWA2_CUDA(cudaMemsetAsync(s->d_status, 0, 4, s->stream));
  CWA2_CUDA(cudaStreamSynchronize(s->stream));
  if (v & kStatusTimeout) return err2("a bounded device wait (scan look-back) timed out", CWA_ERR_TIMEOUT);
  if (v & kStatusNonFinite) return err2("non-finite particle position", CWA_ERR_NONFINITE);
  return err2("a grid cell held more than 1024 particles; its insert order fell back to arrival order",
              CWA_ERR_CAPACITY);
}

cwa_status check2(cwa2d_sim* s) {
  if (!s) return err2("null sim");
  CWA2_CUDA(cudaSetDevice(s->device));
  return CWA_OK;
}

}  // namespace

extern "C" {

cwa_status cwa2d_defaults(cwa2d_params* p) {
  if (!p) return err2("null params");
  *p = cwa2d_params{};
  p->n_particles = 32 * 128;
  p->wave_cells = 128;
  p->sph_substeps = 2;
  p->wave_substeps = 1;
  p->grid_cells[0] = p->grid_cells[1] = 32;
  p->init_columns = 128;
  p->view_size[0] = p->view_size[1] = 2.0f * 4.8f;
  p->particle_radius = 0.025f;
  p->rest_density = 1000.0f;
  p->visc = 0.05f;
  p->dt = 0.002f;
  p->gas_const = 35000.0f;
  p->bottom = 0.3f;
  p->wave_lambda = 0.001f;
  p->wave_dx = 0.1f;
  p->wave_kind = CWA2D_WAVE_SHALLOW;
  p->wave_atten = 0.9995f;
  p->wave_beta = 0.001f;
  return CWA_OK;
}

cwa_status cwa2d_create(const cwa2d_params* p, int32_t device, cwa2d_sim** out) {
  if (!p || !out) return err2("null params or output");
  *out = nullptr;
  if (p->n_particles < 1 || p->n_particles > (1 << 26)) return err2("n_particles must be in [1, 2^26]");
  if (p->init_columns < 1 || p->n_particles % p->init_columns) return err2("n_particles must be a multiple of init_columns");
  if (p->wave_cells < 3 || p->wave_cells > (1 << 24)) return err2("wave_cells must be in [3, 2^24]");
  if (p->grid_cells[0] < 1 || p->grid_cells[1] < 1 || (int64_t)p->grid_cells[0] * p->grid_cells[1] > (1 << 26))
    return err2("grid_cells must be positive, at most 2^26 cells");
  if (p->sph_substeps < 0 || p->wave_substeps < 0) return err2("substeps must be >= 0");
  if (p->wave_kind != CWA2D_WAVE_SHALLOW && p->wave_kind != CWA2D_WAVE_1D) return err2("unknown wave_kind");
  if (!(p->view_size[0] > 0.0f && p->view_size[1] > 0.0f && p->particle_radius > 0.0f && p->rest_density > 0.0f &&
        p->dt > 0.0f && p->wave_dx > 0.0f))
    return err2("sizes, radius, rest density, dt and dx must be positive");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return err2("no such CUDA device", CWA_ERR_NO_DEVICE);
  cwa2d_sim* s = new cwa2d_sim();
  s->device = device;
  s->prm = *p;
  Sph2dConst& k = s->k;
  k.n = p->n_particles;
  k.ncx = p->grid_cells[0];
  k.ncy = p->grid_cells[1];
  k.wave_n = p->wave_cells;
  k.cols = p->init_columns;
  k.R = p->particle_radius;
  k.H = 4.0f * k.R;
  k.HSQ = k.H * k.H;
  k.rest = p->rest_density;
  k.visc = p->visc;
  k.mass = (2.0f * k.R) * (2.0f * k.R) * k.rest;
  k.dt = p->dt;
  k.gas = p->gas_const;
  const float pi = 3.14159265f;  // the shader's M_PI
  k.k2 = 40.0f / (7.0f * pi * k.HSQ);
  k.psi = k.rest / (1.5f * k.k2);
  k.view_w = p->view_size[0];
  k.view_h = p->view_size[1];
  k.cell_x = k.view_w / (float)k.ncx;  // UniformGridGpu2D: extents / cells
  k.cell_y = k.view_h / (float)k.ncy;
  k.plane0_c = -0.5f * k.view_h + 15.0f * k.R - k.R + p->bottom;
  k.lambda = p->wave_lambda;
  k.dx = p->wave_dx;
  k.wave_kind = p->wave_kind;
  // Wave1D's coefficients as the shader forms them (Wave1D_cs.glsl:109, 125)
  k.w1_a = (2.0f - 2.0f * p->wave_lambda) - p->wave_beta;
  k.w1_b = 1.0f - p->wave_beta;
  k.w1_atten = p->wave_atten;
  k.w1_half = 0.5f * p->wave_lambda;
  const int nb = k.ncx * k.ncy + 1;  // grid cells + the bucket of points outside the grid
  auto fail = [&](cudaError_t e) {
    cwa::set_error(std::string("cwa2d_create: ") + cudaGetErrorString(e));
    free2d(s);
    return e == cudaErrorMemoryAllocation ? CWA_ERR_OOM : CWA_ERR_CUDA;
  };
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(e);
  for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
    e = cudaMalloc((void**)&s->P[b], sizeof(float4) * k.n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&s->V[b], sizeof(float4) * k.n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&s->A[b], sizeof(float4) * k.n);
  }
  for (int b = 0; b < 3 && e == cudaSuccess; ++b) {
    e = cudaMalloc((void**)&s->W[b], sizeof(float4) * k.wave_n);
    if (e == cudaSuccess) e = cudaMemset(s->W[b], 0, sizeof(float4) * k.wave_n);  // images start at zero
  }
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->key, 4 * (size_t)k.n);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->slot, 4 * (size_t)k.n);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->list, 4 * (size_t)k.n);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->sorted, 4 * (size_t)k.n);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->count, 4 * (size_t)nb);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->start, 4 * ((size_t)nb + 1));
  if (e == cudaSuccess) e = cudaMalloc(&s->scan_ws, scan_workspace_bytes(nb + 1));
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->d_status, 4);
  if (e == cudaSuccess) e = cudaMalloc((void**)&s->staging, sizeof(cwa2d_particle) * k.n);
  if (e == cudaSuccess) e = cudaMemset(s->count, 0, 4 * (size_t)nb);
  if (e == cudaSuccess) e = cudaMemset(s->d_status, 0, 4);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(e);
  scan_bind_workspace(s->scan_ws, nb + 1, &s->scan);
  const cwa_status st = cwa2d_reinit(s);
  if (st != CWA_OK) {
    free2d(s);
    return st;
  }
  *out = s;
  return CWA_OK;
}

cwa_status cwa2d_destroy(cwa2d_sim* s) {
  if (!s) return err2("null sim");
  free2d(s);
  return CWA_OK;
}

cwa_status cwa2d_reinit(cwa2d_sim* s) {
  cwa_status st = check2(s);
  if (st != CWA_OK) return st;
  k2_init_particles<<<blocks(s->k.n), kBlock, 0, s->stream>>>(s->k, s->P[s->cur], s->V[s->cur], s->A[s->cur]);
  // ImageStencil::Reinit: MODE_INIT_FIRST + i into the write image, then
  // PingPong, for each read image (one for shallow water, two for Wave1D)
  if (s->k.wave_kind == CWA2D_WAVE_1D) {
    st = pass_wave1d(s, 0);
    if (st == CWA_OK) st = pass_wave1d(s, 1);
    if (st != CWA_OK) return st;
  } else {
    k2_wave_init<<<blocks(s->k.wave_n), kBlock, 0, s->stream>>>(s->k, s->W[s->wcur], s->W[s->wcur ^ 1], 0);
    CWA2_CUDA(cudaGetLastError());
    s->wcur ^= 1;
  }
  s->grid_fresh = false;
  drop_graphs2(s);  // the particle phase may have changed
  return read_status2(s);
}

cwa_status cwa2d_splash(cwa2d_sim* s) {
  cwa_status st = check2(s);
  if (st != CWA_OK) return st;
  if (s->k.wave_kind == CWA2D_WAVE_1D) {
    st = pass_wave1d(s, 1);
    if (st != CWA_OK) return st;
  } else {
    k2_wave_init<<<blocks(s->k.wave_n), kBlock, 0, s->stream>>>(s->k, s->W[s->wcur], s->W[s->wcur ^ 1], 1);
    CWA2_CUDA(cudaGetLastError());
    s->wcur ^= 1;
  }
  return CWA_OK;
}

cwa_status cwa2d_step(cwa2d_sim* s, int32_t n) {
  cwa_status st = check2(s);
  if (st != CWA_OK) return st;
  if (n < 0) return err2("n_steps < 0");
  for (int32_t k = 0; k < n; ++k) {
    // A frame flips the particle buffers an even number of times (two passes
    // per substep); the wave phase advances by 0 (shallow water: two passes
    // per substep) or by wave_substeps mod 3 (Wave1D), so frames replay one
    // graph per wave phase.
    const int cur0 = s->cur, w0 = s->wcur;
    cudaGraphExec_t& ge = s->graph[w0];
    int w1 = w0;
    if (s->k.wave_kind == CWA2D_WAVE_1D) w1 = (w0 + s->prm.wave_substeps) % 3;
    if (!ge) {
      cudaGraph_t g = nullptr;
      CWA2_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
      st = enqueue_frame(s);
      cudaError_t e = cudaStreamEndCapture(s->stream, &g);
      s->cur = cur0;
      s->wcur = w0;
      if (st != CWA_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
      }
      CWA2_CUDA(e);
      e = cudaGraphInstantiate(&ge, g, 0);
      cudaGraphDestroy(g);
      CWA2_CUDA(e);
    }
    CWA2_CUDA(cudaGraphLaunch(ge, s->stream));
    s->wcur = w1;
    s->grid_fresh = false;
  }
  return CWA_OK;
}

cwa_status cwa2d_pass(cwa2d_sim* s, int32_t pass) {
  cwa_status st = check2(s);
  if (st != CWA_OK) return st;
  if (pass != CWA2D_PASS_GRID) drop_graphs2(s);  // single passes change the particle phase
  const bool w1 = s->k.wave_kind == CWA2D_WAVE_1D;
  if ((pass == CWA2D_PASS_WAVE_PREDICT || pass == CWA2D_PASS_WAVE_CORRECT) && w1)
    return err2("the predictor and corrector passes belong to the shallow-water kind");
  if (pass == CWA2D_PASS_WAVE_ITERATE && !w1) return err2("the iterate pass belongs to the Wave1D kind");
  switch (pass) {
    case CWA2D_PASS_GRID: return pass_grid(s);
    case CWA2D_PASS_DENSITY:
      if (!s->grid_fresh) return err2("the grid pass must precede the density pass");
      return pass_sph(s, true);
    case CWA2D_PASS_FORCE:
      if (!s->grid_fresh) return err2("the grid pass must precede the force pass");
      return pass_sph(s, false);
    case CWA2D_PASS_WAVE_PREDICT: return pass_wave(s, 0);
    case CWA2D_PASS_WAVE_CORRECT: return pass_wave(s, 1);
    case CWA2D_PASS_WAVE_ITERATE: return pass_wave1d(s, -1);
    default: return err2("unknown pass");
  }
}

cwa_status cwa2d_upload_particles(cwa2d_sim* s, const cwa2d_particle* host, int32_t n) {
  cwa_status st = check2(s);
  if (st != CWA_OK) return st;
  if (!host || n != s->k.n) return err2("upload size must equal n_particles");
  // host AoS (48 B) -> device SoA through pitched 2D copies
  const size_t es = sizeof(cwa2d_particle);
  CWA2_CUDA(cudaMemcpy2DAsync(s->P[s->cur], 16, &host[0].pos, es, 16, n, cudaMemcpyHostToDevice, s->stream));
  CWA2_CUDA(cudaMemcpy2DAsync(s->V[s->cur], 16, &host[0].vel, es, 16, n, cudaMemcpyHostToDevice, s->stream));
  CWA2_CUDA(cudaMemcpy2DAsync(s->A[s->cur], 16, &host[0].acc, es, 16, n, cudaMemcpyHostToDevice, s->stream));
  s->grid_fresh = false;
  CWA2_CUDA(cudaStreamSynchronize(s->stream));
  return CWA_OK;
}

cwa_status cwa2d_download_particles(cwa2d_sim* s, cwa2d_particle* host, int32_t n) {
  cwa_status st = check2(s);
  if (st != CWA_OK) return st;
  if (!host || n != s->k.n) return err2("download size must equal n_particles");
  const size_t es = sizeof(cwa2d_particle);
  CWA2_CUDA(cudaMemcpy2DAsync(&host[0].pos, es, s->P[s->cur], 16, 16, n, cudaMemcpyDeviceToHost, s->stream));
  CWA2_CUDA(cudaMemcpy2DAsync(&host[0].vel, es, s->V[s->cur], 16, 16, n, cudaMemcpyDeviceToHost, s->stream));
  CWA2_CUDA(cudaMemcpy2DAsync(&host[0].acc, es, s->A[s->cur], 16, 16, n, cudaMemcpyDeviceToHost, s->stream));
  CWA2_CUDA(cudaStreamSynchronize(s->stream));
  return read_status2(s);
}

cwa_status cwa2d_upload_wave(cwa2d_sim* s, const float* cells4, int32_t n) {
  cwa_status st = check2(s);
  if (st != CWA_OK) return st;
  if (!cells4 || n != s->k.wave_n) return err2("upload size must equal wave_cells");
  CWA2_CUDA(cudaMemcpyAsync(s->W[s->wcur], cells4, sizeof(float4) * n, cudaMemcpyHostToDevice, s->stream));
  CWA2_CUDA(cudaStreamSynchronize(s->stream));
  return CWA_OK;
}

cwa_status cwa2d_download_wave(cwa2d_sim* s, float* cells4, int32_t n) {
  cwa_status st = check2(s);
  if (st != CWA_OK) return st;
  if (!cells4 || n != s->k.wave_n) return err2("download size must equal wave_cells");
  CWA2_CUDA(cudaMemcpyAsync(cells4, s->W[s->wcur], sizeof(float4) * n, cudaMemcpyDeviceToHost, s->stream));
  CWA2_CUDA(cudaStreamSynchronize(s->stream));
  return CWA_OK;
}

cwa_status cwa2d_upload_wave_prev(cwa2d_sim* s, const float* cells4, int32_t n) {
  cwa_status st = check2(s);
  if (st != CWA_OK) return st;
  if (s->k.wave_kind != CWA2D_WAVE_1D) return err2("only the Wave1D kind keeps an older field");
  if (!cells4 || n != s->k.wave_n) return err2("upload size must equal wave_cells");
  CWA2_CUDA(cudaMemcpyAsync(s->W[(s->wcur + 2) % 3], cells4, sizeof(float4) * n, cudaMemcpyHostToDevice,
                            s->stream));
  CWA2_CUDA(cudaStreamSynchronize(s->stream));
  return CWA_OK;
}

cwa_status cwa2d_download_wave_prev(cwa2d_sim* s, float* cells4, int32_t n) {
  cwa_status st = check2(s);
  if (st != CWA_OK) return st;
  if (s->k.wave_kind != CWA2D_WAVE_1D) return err2("only the Wave1D kind keeps an older field");
  if (!cells4 || n != s->k.wave_n) return err2("download size must equal wave_cells");
  CWA2_CUDA(cudaMemcpyAsync(cells4, s->W[(s->wcur + 2) % 3], sizeof(float4) * n, cudaMemcpyDeviceToHost,
                            s->stream));
  CWA2_CUDA(cudaStreamSynchronize(s->stream));
  return CWA_OK;
}

cwa_status cwa2d_synchronize(cwa2d_sim* s) {
  cwa_status st = check2(s);
  if (st != CWA_OK) return st;
  CWA2_CUDA(cudaStreamSynchronize(s->stream));
  return read_status2(s);
}

}  // extern "C"
