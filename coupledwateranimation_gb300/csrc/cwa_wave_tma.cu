// cwa_wave_tma.cu — temporally blocked wave stencil over every scene.
//
// Advances the height fields K leapfrog steps per launch with no new
// particle deposits: the stand-alone wave module's job (the reference's
// StencilImage2DTripleBuffered driving wave_comp.glsl EvolveWave, :171-206,
// one dispatch per step; the 2D wave demo Wave2DSimp/Wave2D_cs.glsl:78-84).
//
// One launch covers all scenes through a list of block tiles.  A block tile
// owns a (128 - 2K) x (BOX_H - 2K) patch of one scene's field and works on a
// 128 x BOX_H box: the patch plus a K-cell halo.  Three variants exist
// (BOX_H, K) = (32, 4), (64, 4), (64, 8); the wave tuner times them and keeps
// the fastest.  Scenes whose row width is a multiple of 4 cells load the box
// of u^n and u^(n-1) with two 2D TMA copies (cp.async.bulk.tensor, completion
// counted on an mbarrier; the box's x origin is patch_x - K, a multiple of 4
// floats = 16 bytes for K = 4 and 8); other widths load it with plain loads.
// The K steps then run in shared memory — step s is computed on the box
// shrunk by s cells, which is exactly the region whose inputs are still
// exact — and the patch of u^(n+K) and u^(n+K-1) is stored with coalesced
// writes into two buffers that no CTA of this launch reads.  DRAM traffic
// per cell-step drops from 12 bytes (single step: read u^n, u^(n-1), write
// u^(n+1)) to 16 x box / (K x patch) bytes: 4.9 for (32, 4), 4.1 for (64, 4),
// 2.6 for (64, 8).
//
// Each cell runs the single-step kernel's operation sequence with the same
// clamped (Neumann) neighbour indices, so one launch equals K single wave
// passes bit for bit.  Box cells outside the domain (TMA zero fill) are
// never read by an in-domain cell: neighbour indices clamp to the domain.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include "cwa_internal.h"

namespace cwa {
namespace {

constexpr int kBoxW = 128;               // box width in cells
constexpr int kWaveTmaThreads = kBoxW;  // one thread per box column

// The block variants the tuner chooses from: box height and steps per launch
// (= halo).  Output patch (128 - 2K) x (BOX_H - 2K).
constexpr int kVarBoxW[kWaveVariants] = {128, 128, 128, 128, 128, 128, 256, 128};
constexpr int kVarBoxH[kWaveVariants] = {32, 64, 64, 32, 64, 64, 32, 32};
constexpr int kVarK[kWaveVariants] = {4, 4, 8, 4, 4, 8, 4, 4};

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool bar_try_wait(uint32_t bar, uint32_t parity = 0) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on the barrier's phase with the given parity: false after
// ~2^20 polls.
__device__ __forceinline__ bool bar_wait_bounded(uint32_t bar, uint32_t parity = 0) {
  for (int k = 0; k < (1 << 20); ++k)
    if (bar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Loads the box of u^n (box 0) and u^(n-1) (box 1) at origin (ox, oy): two
// TMA copies counted on the mbarrier, or plain loads with zero fill outside
// the domain.  Returns false (after flagging a timeout) when the copies do
// not land within the bounded wait; the caller's CTA then exits.
template <int kBoxH, int kBW>
__device__ __forceinline__ bool load_box(const WaveBlockArgs& a, const WaveBlockTile& t, const SceneDev* S,
                                         float (*box)[kBoxH][kBW], uint64_t& bar, int ox, int oy) {
  const int W = S->nx, H = S->nz;
  if (t.tma) {
    constexpr uint32_t kBoxBytes = kBW * kBoxH * sizeof(float);
    const uint32_t b = smem_u32(&bar);
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(2 * kBoxBytes)
                   : "memory");
      tma_load_2d(smem_u32(&box[0][0][0]), a.map_cur + t.scene, ox, oy, b);
      tma_load_2d(smem_u32(&box[1][0][0]), a.map_prev + t.scene, ox, oy, b);
    }
    if (!bar_wait_bounded(b)) {
      if (threadIdx.x == 0) atomicOr(a.status, kStatusTimeout);
      bar_wait_bounded(b);  // give copies still in flight a chance to land before the CTA exits
      return false;
    }
  } else {
    const float* uc = a.in_cur + S->woff;
    const float* up = a.in_prev + S->woff;
    for (int lx = threadIdx.x; lx < kBW; lx += kWaveTmaThreads) {
      const int gx = ox + lx;
      for (int ly = 0; ly < kBoxH; ++ly) {
        const int gy = oy + ly;
        const bool in = gx >= 0 && gx < W && gy >= 0 && gy < H;
        box[0][ly][lx] = in ? __ldg(uc + (size_t)gy * W + gx) : 0.0f;
        box[1][ly][lx] = in ? __ldg(up + (size_t)gy * W + gx) : 0.0f;
      }
    }
    __syncthreads();
  }
  return true;
}

// The column walk of an interior box: every step's row range is a constant,
// so the walks unroll completely and need no domain clamps (the box lies
// inside the domain's rows).
template <int kBoxH, int kK>
__device__ __forceinline__ void walk_interior(float (*box)[kBoxH][kBoxW], int lx, int le, int lw, bool col_in,
                                              float wa, float wb, float lam, float atten, bool coupled,
                                              float zero_deposit) {
#pragma unroll
  for (int s = 1; s <= kK; ++s) {
    const float(*A)[kBoxW] = box[(s - 1) & 1];
    float(*B)[kBoxW] = box[s & 1];
    if (col_in && lx >= s && lx < kBoxW - s) {
      float south = A[s - 1][lx];
      float mid = A[s][lx];
#pragma unroll
      for (int ly = s; ly < kBoxH - s; ++ly) {
        const float north = A[ly + 1][lx];
        const float nb = fadd(fadd(north, south), fadd(A[ly][le], A[ly][lw]));
        float w = fadd(fmul(wa, mid), fmul(lam, nb));
        w = fsub(w, fmul(wb, B[ly][lx]));
        w = fmul(atten, w);
        if (coupled) w = fadd(w, zero_deposit);
        B[ly][lx] = w;
        south = mid;
        mid = north;
      }
    }
    __syncthreads();
  }
}

// Stores the patch of u^(n+K) (box[0]; K is even) and u^(n+K-1) (box[1]).
template <int kBoxH, int kK>
__device__ __forceinline__ void store_patch(const WaveBlockArgs& a, const SceneDev* S, float (*box)[kBoxH][kBoxW],
                                            int oy, int gx, int W, int H) {
  static_assert(kK % 2 == 0, "u^(n+K) lands in box[0] for even K");
  const int lx = threadIdx.x;
  float* oc = a.out_cur + S->woff;
  float* op = a.out_prev + S->woff;
  if (lx >= kK && lx < kBoxW - kK && gx < W) {
    const int r1 = min(kBoxH - kK, H - oy);
    for (int ly = kK; ly < r1; ++ly) {
      const size_t g = (size_t)(oy + ly) * W + gx;
      oc[g] = box[0][ly][lx];
      op[g] = box[1][ly][lx];
    }
  }
}

template <int kBoxH, int kK>
__global__ void __launch_bounds__(kWaveTmaThreads)
    k_wave_block(WaveBlockArgs a) {
  constexpr int kTileW = kBoxW - 2 * kK, kTileH = kBoxH - 2 * kK;
  // Dynamic shared memory only, so the boxes start at the window's base
  // (the TMA destinations want 128-byte alignment); the mbarrier follows them.
  extern __shared__ __align__(128) float box_mem[];  // [2][kBoxH][kBoxW], then the barrier
  float(*box)[kBoxH][kBoxW] = reinterpret_cast<float(*)[kBoxH][kBoxW]>(box_mem);
  uint64_t& bar = *reinterpret_cast<uint64_t*>(box_mem + 2 * kBoxH * kBoxW);
  const WaveBlockTile t = a.tiles[blockIdx.x];
  const SceneDev* S = a.scenes + t.scene;
  const int W = S->nx, H = S->nz;
  const int ox = t.bx * kTileW - kK, oy = t.by * kTileH - kK;  // box origin; ox % 4 == 0
  if (!load_box<kBoxH, kBoxW>(a, t, S, box, bar, ox, oy)) return;
  // Each thread owns one box column and walks it top to bottom with the
  // column's north / centre / south values in registers; east and west come
  // from the neighbouring columns in shared memory.  Domain borders clamp
  // (the clamped neighbour is the cell itself).
  const float wa = S->wa, wb = S->wb, lam = S->lam, atten = S->atten;
  const bool coupled = S->coupled != 0;
  const float zero_deposit = coupled ? fmul(S->gain, fmul(0.0f, S->dq)) : 0.0f;
  const int lx = threadIdx.x, gx = ox + lx;
  const bool src_col = S->line_source && gx == W / 2;
  const bool col_in = gx >= 0 && gx < W;
  const int le = gx + 1 < W ? lx + 1 : lx, lw = gx > 0 ? lx - 1 : lx;
  // Interior boxes (inside the domain's rows, no line-source column) take
  // the unrolled walk without row clamps.
  if (!(oy < 0 || oy + kBoxH > H || (S->line_source && W / 2 >= ox && W / 2 < ox + kBoxW))) {
    walk_interior<kBoxH, kK>(box, lx, le, lw, col_in, wa, wb, lam, atten, coupled, zero_deposit);
    store_patch<kBoxH, kK>(a, S, box, oy, gx, W, H);
    return;
  }
  int c = 0;  // box[c] = u^t, box[c ^ 1] = u^(t-1), overwritten in place by u^(t+1)
#pragma unroll 1
  for (int s = 1; s <= kK; ++s) {
    const float(*A)[kBoxW] = box[c];
    float(*B)[kBoxW] = box[c ^ 1];
    // rows whose inputs are still exact after s - 1 steps, inside the domain
    const int r0 = max(s, -oy), r1 = min(kBoxH - s, H - oy);
    if (col_in && lx >= s && lx < kBoxW - s && r0 < r1) {
      float south = oy + r0 > 0 ? A[r0 - 1][lx] : A[r0][lx];
      float mid = A[r0][lx];
#pragma unroll 4
      for (int ly = r0; ly < r1; ++ly) {
        const int gy = oy + ly;
        const float north = gy + 1 < H ? A[ly + 1][lx] : mid;
        const float nb = fadd(fadd(north, south), fadd(A[ly][le], A[ly][lw]));
        float w = fadd(fmul(wa, mid), fmul(lam, nb));
        w = fsub(w, fmul(wb, B[ly][lx]));
        w = fmul(atten, w);
        if (src_col && w > 0.0001f) w = fadd(w, 0.001f);
        if (coupled) w = fadd(w, zero_deposit);
        B[ly][lx] = w;
        south = mid;
        mid = north;
      }
    }
    __syncthreads();
    c ^= 1;
  }
  store_patch<kBoxH, kK>(a, S, box, oy, gx, W, H);  // K even: box[0] = u^(n+K)
}

// Register-column form of the same block: each thread keeps its box column
// of u^t and u^(t-1) in registers (rows fully unrolled), so a cell update
// reads only its east and west neighbours from shared memory and writes its
// own new value there for the neighbours' next step: 2 loads + 1 store per
// cell-step instead of 4 + 1.  Every box cell is updated every step (the
// invalid rim grows by one cell per step and is never stored); neighbour
// indices clamp at the domain border exactly as the single pass does and at
// the box border, where the values are outside the stored patch anyway.
// kEdge = false is the interior form: the box lies inside the domain's rows
// (no north / south clamp) and holds no line-source column.
template <int kBoxH, bool kEdge>
__device__ __forceinline__ void reg_step(const float (&cu)[kBoxH], float (&pv)[kBoxH], const float (*src)[kBoxW],
                                         float (*dst)[kBoxW], int lx, int le, int lw, int ytop, int ybot,
                                         float wa, float wb, float lam, float atten, bool src_col, bool coupled,
                                         float zero_deposit) {
#pragma unroll
  for (int ly = 0; ly < kBoxH; ++ly) {
    const float mid = cu[ly];
    float north = ly + 1 < kBoxH ? cu[ly + 1 < kBoxH ? ly + 1 : ly] : mid;
    float south = ly > 0 ? cu[ly > 0 ? ly - 1 : 0] : mid;
    if (kEdge) {
      if (ly + 1 >= ytop) north = mid;
      if (ly <= ybot) south = mid;
    }
    const float nb = fadd(fadd(north, south), fadd(src[ly][le], src[ly][lw]));
    float w = fadd(fmul(wa, mid), fmul(lam, nb));
    w = fsub(w, fmul(wb, pv[ly]));
    w = fmul(atten, w);
    if (kEdge && src_col && w > 0.0001f) w = fadd(w, 0.001f);
    if (coupled) w = fadd(w, zero_deposit);
    pv[ly] = w;
    dst[ly][lx] = w;
  }
}

template <int kBoxH, int kK, bool kEdge>
__device__ __forceinline__ void reg_steps(float (&cu)[kBoxH], float (&pv)[kBoxH], float (*b0)[kBoxW],
                                          float (*b1)[kBoxW], int lx, int le, int lw, int ytop, int ybot, float wa,
                                          float wb, float lam, float atten, bool src_col, bool coupled,
                                          float zero_deposit) {
#pragma unroll 1
  for (int s = 0; s < kK; s += 2) {
    reg_step<kBoxH, kEdge>(cu, pv, b0, b1, lx, le, lw, ytop, ybot, wa, wb, lam, atten, src_col, coupled,
                           zero_deposit);
    __syncthreads();
    reg_step<kBoxH, kEdge>(pv, cu, b1, b0, lx, le, lw, ytop, ybot, wa, wb, lam, atten, src_col, coupled,
                           zero_deposit);
    __syncthreads();
  }
}

template <int kBoxH, int kK>
__global__ void __launch_bounds__(kWaveTmaThreads)
    k_wave_reg(WaveBlockArgs a) {
  static_assert(kK % 2 == 0, "steps run in pairs");
  constexpr int kTileW = kBoxW - 2 * kK, kTileH = kBoxH - 2 * kK;
  extern __shared__ __align__(128) float box_mem[];  // [2][kBoxH][kBoxW], then the barrier
  float(*box)[kBoxH][kBoxW] = reinterpret_cast<float(*)[kBoxH][kBoxW]>(box_mem);
  uint64_t& bar = *reinterpret_cast<uint64_t*>(box_mem + 2 * kBoxH * kBoxW);
  const WaveBlockTile t = a.tiles[blockIdx.x];
  const SceneDev* S = a.scenes + t.scene;
  const int W = S->nx, H = S->nz;
  const int ox = t.bx * kTileW - kK, oy = t.by * kTileH - kK;  // box origin; ox % 4 == 0
  const int lx = threadIdx.x, gx = ox + lx;
  if (!load_box<kBoxH, kBoxW>(a, t, S, box, bar, ox, oy)) return;
  float cu[kBoxH], pv[kBoxH];
#pragma unroll
  for (int ly = 0; ly < kBoxH; ++ly) {
    cu[ly] = box[0][ly][lx];
    pv[ly] = box[1][ly][lx];
  }
  __syncthreads();  // box[1] is overwritten by the first step
  const float wa = S->wa, wb = S->wb, lam = S->lam, atten = S->atten;
  const bool coupled = S->coupled != 0;
  const float zero_deposit = coupled ? fmul(S->gain, fmul(0.0f, S->dq)) : 0.0f;
  const bool src_col = S->line_source && gx == W / 2;
  // east / west: the neighbour column inside the domain and the box, else the
  // column itself (the single pass's clamp at the domain border)
  const int le = (gx + 1 < W && lx + 1 < kBoxW) ? lx + 1 : lx;
  const int lw = (gx > 0 && lx > 0) ? lx - 1 : lx;
  const int ytop = H - oy, ybot = -oy;  // local rows in the domain: (ybot - 1, ytop)
  const bool edge = oy < 0 || oy + kBoxH > H || (S->line_source && W / 2 >= ox && W / 2 < ox + kBoxW);
  if (edge)
    reg_steps<kBoxH, kK, true>(cu, pv, box[0], box[1], lx, le, lw, ytop, ybot, wa, wb, lam, atten, src_col, coupled,
                               zero_deposit);
  else
    reg_steps<kBoxH, kK, false>(cu, pv, box[0], box[1], lx, le, lw, ytop, ybot, wa, wb, lam, atten, src_col,
                                coupled, zero_deposit);
  // cu = u^(n+K), pv = u^(n+K-1)
  float* oc = a.out_cur + S->woff;
  float* op = a.out_prev + S->woff;
  if (lx >= kK && lx < kBoxW - kK && gx < W) {
#pragma unroll
    for (int ly = kK; ly < kBoxH - kK; ++ly) {
      if (ly < ytop) {
        const size_t g = (size_t)(oy + ly) * W + gx;
        oc[g] = cu[ly];
        op[g] = pv[ly];
      }
    }
  }
}

// Column-pair form: a 256 x kBoxH box, each of the 128 threads holding two
// adjacent columns (2t, 2t+1) of u^t and u^(t-1) in registers.  Inside the
// pair the east / west neighbours are registers; across pairs a thread reads
// the right column of thread t-1 and the left column of thread t+1 from two
// exchange arrays, written once per row and side.  A cell-step costs one
// shared-memory access (the shared walk: 5, the one-column register form:
// 3).  The exchange arrays reuse the boxes' shared memory once the columns
// are in registers.
constexpr int kPairW = 2 * kWaveTmaThreads;

struct PairCtx {
  int th, tw, te;             // this thread, the thread west / east of it
  bool self_w, self_e, pair_in;  // domain clamps of column 2t's west, 2t+1's east, 2t's east
  int ytop, ybot;
  float wa, wb, lam, atten, zero_deposit;
  bool src0, src1, coupled;
};

template <int kBoxH, bool kEdge>
__device__ __forceinline__ void pair_step(const float (&c0)[kBoxH], const float (&c1)[kBoxH], float (&p0)[kBoxH],
                                          float (&p1)[kBoxH], const float (*sl)[kWaveTmaThreads],
                                          const float (*sr)[kWaveTmaThreads], float (*dl)[kWaveTmaThreads],
                                          float (*dr)[kWaveTmaThreads], const PairCtx& c) {
#pragma unroll
  for (int ly = 0; ly < kBoxH; ++ly) {
    const float m0 = c0[ly], m1 = c1[ly];
    float n0 = ly + 1 < kBoxH ? c0[ly + 1 < kBoxH ? ly + 1 : ly] : m0;
    float n1 = ly + 1 < kBoxH ? c1[ly + 1 < kBoxH ? ly + 1 : ly] : m1;
    float s0 = ly > 0 ? c0[ly > 0 ? ly - 1 : 0] : m0;
    float s1 = ly > 0 ? c1[ly > 0 ? ly - 1 : 0] : m1;
    float w0 = sr[ly][c.tw];  // column 2t - 1
    float e1 = sl[ly][c.te];  // column 2t + 2
    float e0 = m1, w1 = m0;
    if (kEdge) {
      if (ly + 1 >= c.ytop) {
        n0 = m0;
        n1 = m1;
      }
      if (ly <= c.ybot) {
        s0 = m0;
        s1 = m1;
      }
      if (c.self_w) w0 = m0;
      if (c.self_e) e1 = m1;
      if (!c.pair_in) e0 = m0;
    }
    const float nb0 = fadd(fadd(n0, s0), fadd(e0, w0));
    const float nb1 = fadd(fadd(n1, s1), fadd(e1, w1));
    float u0 = fadd(fmul(c.wa, m0), fmul(c.lam, nb0));
    float u1 = fadd(fmul(c.wa, m1), fmul(c.lam, nb1));
    u0 = fmul(c.atten, fsub(u0, fmul(c.wb, p0[ly])));
    u1 = fmul(c.atten, fsub(u1, fmul(c.wb, p1[ly])));
    if (kEdge) {
      if (c.src0 && u0 > 0.0001f) u0 = fadd(u0, 0.001f);
      if (c.src1 && u1 > 0.0001f) u1 = fadd(u1, 0.001f);
    }
    if (c.coupled) {
      u0 = fadd(u0, c.zero_deposit);
      u1 = fadd(u1, c.zero_deposit);
    }
    p0[ly] = u0;
    p1[ly] = u1;
    dl[ly][c.th] = u0;
    dr[ly][c.th] = u1;
  }
}

template <int kBoxH, int kK, bool kEdge>
__device__ __forceinline__ void pair_steps(float (&c0)[kBoxH], float (&c1)[kBoxH], float (&p0)[kBoxH],
                                           float (&p1)[kBoxH], float (*ex)[2][kBoxH][kWaveTmaThreads],
                                           const PairCtx& c) {
#pragma unroll 1
  for (int s = 0; s < kK; s += 2) {
    pair_step<kBoxH, kEdge>(c0, c1, p0, p1, ex[0][0], ex[0][1], ex[1][0], ex[1][1], c);
    __syncthreads();
    pair_step<kBoxH, kEdge>(p0, p1, c0, c1, ex[1][0], ex[1][1], ex[0][0], ex[0][1], c);
    __syncthreads();
  }
}

template <int kBoxH, int kK>
__global__ void __launch_bounds__(kWaveTmaThreads)
    k_wave_pair(WaveBlockArgs a) {
  static_assert(kK % 2 == 0, "steps run in pairs");
  constexpr int kTileW = kPairW - 2 * kK, kTileH = kBoxH - 2 * kK;
  extern __shared__ __align__(128) float box_mem[];  // [2][kBoxH][kPairW], then the barrier
  float(*box)[kBoxH][kPairW] = reinterpret_cast<float(*)[kBoxH][kPairW]>(box_mem);
  uint64_t& bar = *reinterpret_cast<uint64_t*>(box_mem + 2 * kBoxH * kPairW);
  const WaveBlockTile t = a.tiles[blockIdx.x];
  const SceneDev* S = a.scenes + t.scene;
  const int W = S->nx, H = S->nz;
  const int ox = t.bx * kTileW - kK, oy = t.by * kTileH - kK;  // box origin; ox % 4 == 0
  if (!load_box<kBoxH, kPairW>(a, t, S, box, bar, ox, oy)) return;
  const int th = threadIdx.x, lx0 = 2 * th, gx0 = ox + lx0;
  float c0[kBoxH], c1[kBoxH], p0[kBoxH], p1[kBoxH];
#pragma unroll
  for (int ly = 0; ly < kBoxH; ++ly) {
    const float2 u = *reinterpret_cast<const float2*>(&box[0][ly][lx0]);
    const float2 v = *reinterpret_cast<const float2*>(&box[1][ly][lx0]);
    c0[ly] = u.x;
    c1[ly] = u.y;
    p0[ly] = v.x;
    p1[ly] = v.y;
  }
  __syncthreads();  // the exchange arrays overwrite the boxes
  float(*ex)[2][kBoxH][kWaveTmaThreads] = reinterpret_cast<float(*)[2][kBoxH][kWaveTmaThreads]>(box_mem);
#pragma unroll
  for (int ly = 0; ly < kBoxH; ++ly) {
    ex[0][0][ly][th] = c0[ly];
    ex[0][1][ly][th] = c1[ly];
  }
  __syncthreads();
  PairCtx c;
  c.th = th;
  c.tw = th > 0 ? th - 1 : th;
  c.te = th + 1 < kWaveTmaThreads ? th + 1 : th;
  c.self_w = !(gx0 > 0) || th == 0;
  c.self_e = !(gx0 + 2 < W) || th + 1 == kWaveTmaThreads;
  c.pair_in = gx0 + 1 < W;
  c.ytop = H - oy;
  c.ybot = -oy;
  c.wa = S->wa;
  c.wb = S->wb;
  c.lam = S->lam;
  c.atten = S->atten;
  c.coupled = S->coupled != 0;
  c.zero_deposit = c.coupled ? fmul(S->gain, fmul(0.0f, S->dq)) : 0.0f;
  c.src0 = S->line_source && gx0 == W / 2;
  c.src1 = S->line_source && gx0 + 1 == W / 2;
  // interior: TMA scene (even width), the box clear of the domain's first and
  // last columns and inside its rows, no line-source column
  const bool edge = !t.tma || ox <= 0 || ox + kPairW >= W || oy < 0 || oy + kBoxH > H ||
                    (S->line_source && W / 2 >= ox && W / 2 < ox + kPairW);
  if (edge)
    pair_steps<kBoxH, kK, true>(c0, c1, p0, p1, ex, c);
  else
    pair_steps<kBoxH, kK, false>(c0, c1, p0, p1, ex, c);
  // c = u^(n+K), p = u^(n+K-1)
  float* oc = a.out_cur + S->woff;
  float* op = a.out_prev + S->woff;
  const bool st0 = lx0 >= kK && lx0 < kPairW - kK && gx0 < W;
  const bool st1 = lx0 + 1 >= kK && lx0 + 1 < kPairW - kK && gx0 + 1 < W;
  const bool vec = t.tma && st0 && st1;  // 8-byte aligned: gx0 even, width a multiple of 4, base 16-byte aligned
#pragma unroll
  for (int ly = kK; ly < kBoxH - kK; ++ly) {
    if (ly < c.ytop) {
      const size_t g = (size_t)(oy + ly) * W + gx0;
      if (vec) {
        *reinterpret_cast<float2*>(oc + g) = make_float2(c0[ly], c1[ly]);
        *reinterpret_cast<float2*>(op + g) = make_float2(p0[ly], p1[ly]);
      } else {
        if (st0) {
          oc[g] = c0[ly];
          op[g] = p0[ly];
        }
        if (st1) {
          oc[g + 1] = c1[ly];
          op[g + 1] = p1[ly];
        }
      }
    }
  }
}

// Persistent form of the register-column block: a grid of resident CTAs,
// each taking tiles blockIdx.x, blockIdx.x + gridDim.x, ... .  A CTA owns two
// box stages; while it walks the box of one tile, the TMA copies of its next
// tile land in the other stage (completion on that stage's mbarrier, whose
// phase parity flips at each reuse).  The stage of the current tile, once
// its columns are in registers, serves as the east / west exchange arrays.
template <int kBoxH, int kK>
__global__ void __launch_bounds__(kWaveTmaThreads)
    k_wave_stream(WaveBlockArgs a, int32_t n_tiles) {
  static_assert(kK % 2 == 0, "steps run in pairs");
  constexpr int kTileW = kBoxW - 2 * kK, kTileH = kBoxH - 2 * kK;
  constexpr uint32_t kBoxBytes = kBoxW * kBoxH * sizeof(float);
  extern __shared__ __align__(128) float box_mem[];  // [stage][2][kBoxH][kBoxW], then two barriers
  float(*stage_box)[2][kBoxH][kBoxW] = reinterpret_cast<float(*)[2][kBoxH][kBoxW]>(box_mem);
  uint64_t* bars = reinterpret_cast<uint64_t*>(box_mem + 4 * kBoxH * kBoxW);
  const int lx = threadIdx.x;
  if (lx == 0) {
    for (int st = 0; st < 2; ++st)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[st])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto origin = [](const WaveBlockTile& t, int& ox, int& oy) {
    ox = t.bx * kTileW - kK;  // a multiple of 4 floats: 16-byte TMA x coordinate
    oy = t.by * kTileH - kK;
  };
  // thread 0: the two TMA copies of tile t into stage st.  The stage last
  // held the previous tile's exchange arrays (generic-proxy stores, ordered
  // by that tile's final barrier); the proxy fence orders them before the
  // async-proxy writes of the copies.
  auto issue = [&](const WaveBlockTile& t, int st) {
    int ox, oy;
    origin(t, ox, oy);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const uint32_t b = smem_u32(&bars[st]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(2 * kBoxBytes) : "memory");
    tma_load_2d(smem_u32(&stage_box[st][0][0][0]), a.map_cur + t.scene, ox, oy, b);
    tma_load_2d(smem_u32(&stage_box[st][1][0][0]), a.map_prev + t.scene, ox, oy, b);
  };
  // bit st: parity of the next phase of stage st's barrier / copies of
  // stage st in flight (thread 0 issues them; every thread tracks them)
  uint32_t parity = 0, inflight = 0;
  int tile = blockIdx.x;
  if (tile < n_tiles && a.tiles[tile].tma) {
    if (lx == 0) issue(a.tiles[tile], 0);
    inflight |= 1u;
  }
  for (int i = 0; tile < n_tiles; ++i, tile += gridDim.x) {
    const int st = i & 1;
    const WaveBlockTile t = a.tiles[tile];
    const int next = tile + gridDim.x;
    // prefetch the next tile into the other stage (its last use, as the
    // exchange arrays of the previous tile, ended at that tile's final sync)
    if (next < n_tiles && a.tiles[next].tma) {
      if (lx == 0) issue(a.tiles[next], st ^ 1);
      inflight |= 2u >> st;  // bit st ^ 1
    }
    const SceneDev* S = a.scenes + t.scene;
    const int W = S->nx, H = S->nz;
    int ox, oy;
    origin(t, ox, oy);
    float(*box)[kBoxH][kBoxW] = stage_box[st];
    if (t.tma) {
      const uint32_t b = smem_u32(&bars[st]);
      const uint32_t ph = (parity >> st) & 1u;
      if (!bar_wait_bounded(b, ph)) {
        if (lx == 0) atomicOr(a.status, kStatusTimeout);
        // let every copy this CTA issued land before it exits
        bar_wait_bounded(b, ph);
        if ((inflight >> (st ^ 1)) & 1u) bar_wait_bounded(smem_u32(&bars[st ^ 1]), (parity >> (st ^ 1)) & 1u);
        return;
      }
      parity ^= 1u << st;
      inflight &= ~(1u << st);
    } else {
      const float* uc = a.in_cur + S->woff;
      const float* up = a.in_prev + S->woff;
      const int gx = ox + lx;
      for (int ly = 0; ly < kBoxH; ++ly) {
        const int gy = oy + ly;
        const bool in = gx >= 0 && gx < W && gy >= 0 && gy < H;
        box[0][ly][lx] = in ? __ldg(uc + (size_t)gy * W + gx) : 0.0f;
        box[1][ly][lx] = in ? __ldg(up + (size_t)gy * W + gx) : 0.0f;
      }
      __syncthreads();
    }
    float cu[kBoxH], pv[kBoxH];
#pragma unroll
    for (int ly = 0; ly < kBoxH; ++ly) {
      cu[ly] = box[0][ly][lx];
      pv[ly] = box[1][ly][lx];
    }
    __syncthreads();  // the stage becomes the exchange arrays
    const int gx = ox + lx;
    const float wa = S->wa, wb = S->wb, lam = S->lam, atten = S->atten;
    const bool coupled = S->coupled != 0;
    const float zero_deposit = coupled ? fmul(S->gain, fmul(0.0f, S->dq)) : 0.0f;
    const bool src_col = S->line_source && gx == W / 2;
    const int le = (gx + 1 < W && lx + 1 < kBoxW) ? lx + 1 : lx;
    const int lw = (gx > 0 && lx > 0) ? lx - 1 : lx;
    const int ytop = H - oy, ybot = -oy;
    const bool edge = oy < 0 || oy + kBoxH > H || (S->line_source && W / 2 >= ox && W / 2 < ox + kBoxW);
    if (edge)
      reg_steps<kBoxH, kK, true>(cu, pv, box[0], box[1], lx, le, lw, ytop, ybot, wa, wb, lam, atten, src_col,
                                 coupled, zero_deposit);
    else
      reg_steps<kBoxH, kK, false>(cu, pv, box[0], box[1], lx, le, lw, ytop, ybot, wa, wb, lam, atten, src_col,
                                  coupled, zero_deposit);
    float* oc = a.out_cur + S->woff;
    float* op = a.out_prev + S->woff;
    if (lx >= kK && lx < kBoxW - kK && gx < W) {
#pragma unroll
      for (int ly = kK; ly < kBoxH - kK; ++ly) {
        if (ly < ytop) {
          const size_t g = (size_t)(oy + ly) * W + gx;
          oc[g] = cu[ly];
          op[g] = pv[ly];
        }
      }
    }
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

}  // namespace

int wave_variant_steps(int v) { return kVarK[v]; }

bool wave_block_encode(CUtensorMap* map, float* base, int W, int H, int variant) {
  if (W < 1 || H < 1 || (W % 4) != 0 || (reinterpret_cast<uintptr_t>(base) & 15) != 0) return false;
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)W, (cuuint64_t)H};
  const cuuint64_t strides[1] = {(cuuint64_t)W * sizeof(float)};
  const cuuint32_t boxdim[2] = {(cuuint32_t)kVarBoxW[variant], (cuuint32_t)kVarBoxH[variant]};
  const cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, boxdim, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

void wave_block_tiles(const SceneDev& d, int32_t scene, bool tma, int variant, std::vector<WaveBlockTile>* out) {
  const int tw = kVarBoxW[variant] - 2 * kVarK[variant], th = kVarBoxH[variant] - 2 * kVarK[variant];
  const int nbx = (d.nx + tw - 1) / tw, nby = (d.nz + th - 1) / th;
  for (int by = 0; by < nby; ++by)
    for (int bx = 0; bx < nbx; ++bx) out->push_back(WaveBlockTile{scene, bx, by, tma ? 1 : 0});
}

namespace {
enum Form { kShared, kReg, kPair };

template <int kBoxH, int kK, Form kForm>
cudaError_t launch_variant(const WaveBlockArgs& a, int32_t n_tiles, cudaStream_t stream) {
  constexpr int bytes = 2 * kBoxH * (kForm == kPair ? kPairW : kBoxW) * (int)sizeof(float) + 16;
  void (*kern)(WaveBlockArgs);
  if constexpr (kForm == kPair)
    kern = k_wave_pair<kBoxH, kK>;
  else if constexpr (kForm == kReg)
    kern = k_wave_reg<kBoxH, kK>;
  else
    kern = k_wave_block<kBoxH, kK>;
  static bool raised = false;  // dynamic shared memory above 48 KB needs the opt-in
  if (bytes > 48 * 1024 && !raised) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    raised = true;
  }
  kern<<<n_tiles, kWaveTmaThreads, bytes, stream>>>(a);
  return cudaGetLastError();
}
}  // namespace

// The persistent form: as many resident CTAs as fit, at most one per tile.
cudaError_t launch_stream(const WaveBlockArgs& a, int32_t n_tiles, cudaStream_t stream) {
  constexpr int kH = 32, kK = 4;
  constexpr int bytes = 4 * kH * kBoxW * (int)sizeof(float) + 16;
  static int grid_cap = 0;
  if (grid_cap == 0) {
    cudaError_t e = cudaFuncSetAttribute(k_wave_stream<kH, kK>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    int dev = 0, sms = 0, per_sm = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_wave_stream<kH, kK>, kWaveTmaThreads, bytes);
    if (e != cudaSuccess) return e;
    grid_cap = sms * (per_sm > 0 ? per_sm : 1);
  }
  const int grid = n_tiles < grid_cap ? n_tiles : grid_cap;
  k_wave_stream<kH, kK><<<grid, kWaveTmaThreads, bytes, stream>>>(a, n_tiles);
  return cudaGetLastError();
}

cudaError_t launch_wave_block(const WaveBlockArgs& a, int32_t n_tiles, int variant, cudaStream_t stream) {
  if (n_tiles <= 0) return cudaSuccess;
  switch (variant) {
    case 7: return launch_stream(a, n_tiles, stream);
    case 1: return launch_variant<64, 4, kShared>(a, n_tiles, stream);
    case 2: return launch_variant<64, 8, kShared>(a, n_tiles, stream);
    case 3: return launch_variant<32, 4, kReg>(a, n_tiles, stream);
    case 4: return launch_variant<64, 4, kReg>(a, n_tiles, stream);
    case 5: return launch_variant<64, 8, kReg>(a, n_tiles, stream);
    case 6: return launch_variant<32, 4, kPair>(a, n_tiles, stream);
    default: return launch_variant<32, 4, kShared>(a, n_tiles, stream);
  }
}

}  // namespace cwa
