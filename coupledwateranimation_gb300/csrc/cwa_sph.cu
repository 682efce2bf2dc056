// cwa_sph.cu — SPH neighbour passes over the cell-sorted particle arrays.
//
//   rho_pres: poly6 density, equation of state, and (REFERENCE_3D) the wave
//             density / pressure terms — CoupledWaterAnimation/rho_pres_comp.glsl:49-81.
//   force:    spiky pressure gradient + viscosity Laplacian, then either the
//             reference's crest / torque / drag / wave-normal terms
//             (force_comp.glsl:62-139) or gravity only (MULLER).
//
// The reference loops over all N particles per particle (O(N^2)).  Here the
// particles are sorted by uniform-grid cell (x/y cell edge >= the search
// radius), so the candidates of a particle lie in 9 rows (columns x-1..x+1,
// y-1..y+1) of the sorted arrays, each a contiguous z range.  Every pair with
// r < h lies inside them, so the neighbour sets equal the shaders'.
//
// Two modes (cwa_sim_options.verlet_skin):
//  * per-step (skin 0): k_scan_cands tests every candidate of the particle's
//    rows once, accumulates the density and keeps the hits as this step's
//    neighbour list;
//  * Verlet (skin > 0): the grid and a list of every pair within
//    h (1 + skin) are rebuilt only when some particle has moved more than
//    skin h / 2 since the last rebuild (integrate raises a device flag);
//    k_rho_list walks that list each step, tests r < h and keeps the hits.
// Either way force runs its pair terms over the step's hits only.
//
// A row's cell-based start is start[row + max(cz - rz, 0)], decodable from
// the particle's sorted cell key alone.  The step's hits are nine 64-bit
// row masks per particle (bit b = the row's candidate at that start + b):
// the density pass sets bits in registers, with no per-hit store, and force
// walks the set bits.  The Verlet list holds 16-bit codes (row << 12 |
// offset from the same start), so it stays valid while the particles move.
// The candidate scan can stage the CTA's rows in shared memory with bulk
// TMA copies (cp.async.bulk, completion on an mbarrier).
//
// Sums are accumulated in one of three precisions (template P):
//   CWA_PREC_FP32 plain float; CWA_PREC_COMPENSATED float partial sums (per
//   row or per 8 pairs) folded into a Knuth two-sum accumulator;
//   CWA_PREC_FP64 double pair math and sums.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
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

// Cell coordinates of a global cell id (the two divisions by the scene's
// grid dimensions as multiply-highs with the scene's exact magic numbers).
__device__ __forceinline__ CellCoord cell_of_key(const SceneDev* S, int key) {
  const int local = key - S->coff, nz = S->dims[2], ny = S->dims[1];
  const int xy = (int)(((unsigned long long)(uint32_t)local * S->mz) >> S->sz);
  CellCoord c;
  c.z = local - xy * nz;
  c.x = (int)(((unsigned long long)(uint32_t)xy * S->my) >> S->sy);
  c.y = xy - c.x * ny;
  return c;
}

__device__ __forceinline__ bool row_valid(const SceneDev* S, CellCoord c, int r) {
  const int x = c.x + r / 3 - 1, y = c.y + r % 3 - 1;
  return x >= 0 && x < S->dims[0] && y >= 0 && y < S->dims[1];
}

__device__ __forceinline__ int row_id(const SceneDev* S, CellCoord c, int r) {
  return S->coff + ((c.x + r / 3 - 1) * S->dims[1] + (c.y + r % 3 - 1)) * S->dims[2];
}

// Cell-based start of each row: the base that row-mask bits and Verlet codes are relative
// to.  rz z cells below the particle's cell cover every window.
__device__ __forceinline__ void row_bases(const SceneDev* S, const int32_t* __restrict__ start, CellCoord c,
                                          int base[9]) {
  const int z0 = max(c.z - S->rz, 0);
#pragma unroll
  for (int r = 0; r < 9; ++r) base[r] = row_valid(S, c, r) ? __ldg(start + row_id(S, c, r) + z0) : 0;
}

// Sorted-index ranges [b, e) of the candidates within radius sqrt(rad2) of
// p, row by row.  A row whose column is farther than the radius in (x, y)
// is empty; the others cover the z cells of the window
// |z - pz| < sqrt(rad2 - d^2), d = the column's (x, y) distance.  The
// radius carries a 2^-10 margin (about h / 1024 of slack in the window), so
// neither float rounding nor the approximate square root t * rsqrt(t)
// (relative error ~1e-7) ever drops a pair.
__device__ __forceinline__ void row_ranges(const SceneDev* S, const int32_t* __restrict__ start, float4 p,
                                           CellCoord c, float rad2, int b[9], int e[9]) {
  const int nz = S->dims[2];
  const float x0f = S->lo[0] + (float)c.x * S->cell;
  const float y0f = S->lo[1] + (float)c.y * S->cell;
  const float dxm = fmaxf(p.x - x0f, 0.0f), dxp = fmaxf(x0f + S->cell - p.x, 0.0f);
  const float dym = fmaxf(p.y - y0f, 0.0f), dyp = fmaxf(y0f + S->cell - p.y, 0.0f);
  const float zl = p.z - S->lo[2], izc = S->inv_cellz, zmax = (float)(nz - 1);
#pragma unroll
  for (int r = 0; r < 9; ++r) {
    const int dx = r / 3 - 1, dy = r % 3 - 1;
    const float ddx = dx < 0 ? dxm : (dx > 0 ? dxp : 0.0f);
    const float ddy = dy < 0 ? dym : (dy > 0 ? dyp : 0.0f);
    const float d2 = ddx * ddx + ddy * ddy;
    const bool ok = row_valid(S, c, r) && d2 < rad2;
    const float t = fmaxf(rad2 - d2, 0.0f);
    const float w = ok ? t * rsqrtf(t) : 0.0f;  // ok implies t > 0
    const int z0 = (int)fminf(fmaxf(floorf((zl - w) * izc), 0.0f), zmax);
    const int z1 = (int)fminf(fmaxf(floorf((zl + w) * izc), 0.0f), zmax);
    const int row = row_id(S, c, r);
    b[r] = ok ? __ldg(start + row + z0) : 0;
    e[r] = ok ? __ldg(start + row + z1 + 1) : 0;
  }
}

__device__ __forceinline__ float uv_s(const SceneDev* S, float x) { return x * S->uvs[0] + S->uvo[0]; }
__device__ __forceinline__ float uv_t(const SceneDev* S, float z) { return z * S->uvs[1] + S->uvo[1]; }

// rho, p and the reference's wave terms (rho_pres_comp.glsl:70-80).
__device__ __forceinline__ float2 eos(const SceneDev* S, float rho, float4 pi, const float* __restrict__ wave) {
  float p = S->k * (rho - S->rho0);
  if (S->preset == CWA_PRESET_REFERENCE_3D) {
    p = fmaxf(p, 0.0f);
    const float H = sample_height(wave + S->woff, S->nx, S->nz, uv_s(S, pi.x), uv_t(S, pi.z));
    const float wf = H * rho;
    p += wf;
    rho += wf * S->inv_kr;
    rho = fmaxf(S->rho0, rho);
  }
  return make_float2(rho, p);
}

// Force's gather records of particle i: (x, y, z, p) and (vx, vy, vz, 1/rho),
// so a pair costs two aligned 16-byte gathers; 1/rho uses force's recip.
__device__ __forceinline__ void write_pair_rec(float4* __restrict__ xp, float4* __restrict__ vp,
                                               const float4* __restrict__ vel, int i, float4 pi, float2 rp) {
  if (!xp) return;
  const float4 v = __ldg(vel + i);
  xp[i] = make_float4(pi.x, pi.y, pi.z, rp.y);
  vp[i] = make_float4(v.x, v.y, v.z, recip(rp.x));
}

// ---- shared-memory staging with bulk TMA copies --------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// One 128-bit shared load of a staged candidate at shared-window address a,
// so a quarter warp's eight lanes move 128 bytes per wavefront (the compiler
// would otherwise split the load when the fourth component is unused).  The
// row loop steps a 32-bit address: in place of converting a generic pointer
// at every candidate, that saves 113 instructions a warp and took the
// density pass from 154 to 147 us at 1M particles.
__device__ __forceinline__ float4 lds128(uint32_t a) {
  float4 v;
  asm("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a));
  return v;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on one phase of the staging barrier (phase parity 0 for a
// CTA's first stage, alternating in the work-queue form).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity = 0) {
  for (int k = 0; k < (1 << 20); ++k)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

constexpr int kNbThreads = 128;
constexpr int kStageCap = 1536;   // staged candidates per CTA (24 KB)
constexpr int kRowCodeBits = 12;  // a hit is (row << 12) | offset from the row's cell-based start
constexpr int kRowCodeMax = 1 << kRowCodeBits;
constexpr int kMaxCols = 3;       // columns a CTA's particles may span and still be staged
constexpr int kMaxSegs = 9 * kMaxCols;  // 27 row segments: one planning warp covers them

// Verlet lists hold codes in pairs: code k of particle i is half (k & 1) of
// the 32-bit word (k >> 1) * n + i, so a warp writes its lanes' k-th pairs as
// one 128-byte store and readers load two codes per load.
__device__ __forceinline__ uint32_t code_pair(const uint16_t* __restrict__ list, int k, int i, int n) {
  return __ldg(reinterpret_cast<const uint32_t*>(list) + (size_t)(k >> 1) * n + i);
}

struct StagePlan {
  int32_t seg_b[kMaxSegs];        // global sorted index of each staged segment
  int32_t seg_off[kMaxSegs + 1];  // staged offset (prefix of lengths)
  int32_t seg_delta[kMaxSegs];    // seg_off - seg_b: a staged candidate sits at its sorted index + delta
  int32_t col0;                   // first column (x*ny + y) of the CTA
  int32_t ncols;                  // 1 .. kMaxCols; 0 = read from global memory
};

// Warp 0 plans the CTA's staging: the columns its particles occupy and, per
// column, the candidate rows over the z cells its particles' windows can
// reach (rz cells beyond the particles' own).
__device__ __forceinline__ void plan_stage(const SceneDev* S, const int32_t* __restrict__ start,
                                           const int32_t* __restrict__ keys, const Tile& tl, StagePlan& sp) {
  const int lane = threadIdx.x & 31;
  const CellCoord a = cell_of_key(S, __ldg(keys + tl.begin));
  const CellCoord b = cell_of_key(S, __ldg(keys + tl.end - 1));
  const int nx = S->dims[0], ny = S->dims[1], nz = S->dims[2];
  const int colA = a.x * ny + a.y, colB = b.x * ny + b.y;
  const int ncols = colB - colA + 1;
  const int R = S->rz;
  int len = 0, gb = 0;
  if (ncols <= kMaxCols && lane < 9 * ncols) {
    const int g = lane / 9, r = lane % 9;
    const int col = colA + g;
    const int cx = (int)(((unsigned long long)(uint32_t)col * S->my) >> S->sy), cy = col - cx * ny;
    const int zlo = g == 0 ? max(a.z - R, 0) : 0;
    const int zhi = (g == ncols - 1) ? min(b.z + R, nz - 1) : nz - 1;
    const int x = cx + r / 3 - 1, y = cy + r % 3 - 1;
    if (x >= 0 && x < nx && y >= 0 && y < ny) {
      const int row = S->coff + (x * ny + y) * nz;
      gb = __ldg(start + row + zlo);
      len = __ldg(start + row + zhi + 1) - gb;
    }
  }
  int incl = len;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  if (lane < kMaxSegs) {
    sp.seg_b[lane] = gb;
    sp.seg_off[lane] = incl - len;
    sp.seg_delta[lane] = incl - len - gb;
  }
  if (lane == 0) {
    sp.seg_off[kMaxSegs] = total;
    sp.col0 = colA;
    sp.ncols = (ncols <= kMaxCols && total <= kStageCap) ? ncols : 0;
  }
}

// Candidate test of one row.  DENSITY: q = max(h^2 - r^2, 0) and the sum of
// q^3.  A hit (q > 0 for the radius hit2) is appended to the lane's code
// list, the particle itself included.  CLAMP: the list pointer is clamped
// at the overflow slot after every candidate; rows that cannot reach it
// (the common case, checked once per row) skip the clamp.
template <bool DENSITY, bool CLAMP, class T, class Load>
__device__ __forceinline__ T scan_row_impl(Load load, int len, uint32_t code0, T px, T py, T pz, T hit2,
                                           uint16_t*& hp, uint16_t* hp_end) {
  T part = (T)0;
#pragma unroll 4
  for (int o = 0; o < len; ++o) {
    const float4 pj = load(o);
    const T dx = px - (T)pj.x, dy = py - (T)pj.y, dz = pz - (T)pj.z;
    T q = fma(-dx, dx, hit2);
    q = fma(-dy, dy, q);
    q = fma(-dz, dz, q);
    if (q > (T)0) {  // a miss would add (+0)^3: the sum is unchanged
      if (DENSITY) part = fma(q * q, q, part);
      *hp = (uint16_t)(code0 + (uint32_t)o);
      hp += kNbThreads;
    }
    if (CLAMP) hp = hp < hp_end ? hp : hp_end;
  }
  return part;
}

template <bool DENSITY, class T, class Load>
__device__ __forceinline__ T scan_row(Load load, int len, uint32_t code0, T px, T py, T pz, T hit2,
                                      uint16_t*& hp, uint16_t* hp_end) {
  if (hp + (size_t)len * kNbThreads <= hp_end)
    return scan_row_impl<DENSITY, false, T>(load, len, code0, px, py, pz, hit2, hp, hp_end);
  return scan_row_impl<DENSITY, true, T>(load, len, code0, px, py, pz, hit2, hp, hp_end);
}

// Candidate test of one row for the density pass: the sum of q^3 over the
// hits and the hits themselves as bits of the row window (bit o = candidate
// o; candidates 64 and up are tested and summed but get no bit).  The tests
// only set register bits, so no lane stores anything per candidate.
template <class T, class Load>
__device__ __forceinline__ T scan_row_bits(Load load, int len, T px, T py, T pz, T hit2, RowMask& bits) {
  T part = (T)0;
  uint32_t lo = 0u, hi = 0u;
  for (int c0 = 0; c0 < len; c0 += 32) {
    const int n = min(len - c0, 32);
    uint32_t m = 0u, bit = 1u;
    // Unrolled by 2: a row holds ~12 candidates at C1 (z cells of h/4), so
    // a deeper unroll spends its time in the remainder loop.  The candidate
    // pass took 168 us unrolled by 4, 154 by 2, 165 by 1, 167 by 3 and 192
    // by 8 at C1.
#pragma unroll 2
    for (int o = 0; o < n; ++o) {
      const float4 pj = load(c0 + o);
      const T dx = px - (T)pj.x, dy = py - (T)pj.y, dz = pz - (T)pj.z;
      T q = fma(-dx, dx, hit2);
      q = fma(-dy, dy, q);
      q = fma(-dz, dz, q);
      if (q > (T)0) {  // a miss would add (+0)^3: the sum is unchanged
        part = fma(q * q, q, part);
        m |= bit;
      }
      bit <<= 1;
    }
    if (c0 == 0)
      lo = m;
    else if (c0 == 32)
      hi = m;
  }
  bits = ((RowMask)hi << 32) | lo;
  return part;
}

// Candidate scan.  MODE_DENSITY (per-step mode): radius h, density + this
// step's row masks.  MODE_LIST (Verlet mode, only when the rebuild flag is
// up): radius h (1 + skin), the Verlet list and the rebuild positions.
constexpr int MODE_DENSITY = 0;
constexpr int MODE_LIST = 1;

// Shared memory of the candidate scan.
template <int MODE>
struct ScanShared {
  static constexpr bool kCanStage = MODE == MODE_DENSITY;
  __align__(128) float4 cand[kCanStage ? kStageCap : 1];
  // the Verlet list build stages its codes (+ the overflow slot); the
  // density pass keeps its hits in registers
  uint16_t hit[MODE == MODE_LIST ? kMaxVerlet + 1 : 1][kNbThreads];
  StagePlan sp;
  __align__(8) uint64_t bar;
};

// One tile of the candidate scan.  Stages the tile's rows (bulk copies that
// complete phase `parity` of the CTA's barrier) and scans them.  Returns 1
// when the tile was staged (a barrier phase was used), plus 2 when the
// staging wait timed out (then nothing was computed).  Contains CTA-wide
// barriers: every thread of the CTA calls it.
template <int P, int MODE>
__device__ __forceinline__ int scan_tile(
    ScanShared<MODE>& sh, const Tile tl, uint32_t parity, const float4* __restrict__ pos,
    const int32_t* __restrict__ start, const int32_t* __restrict__ keys, const SceneDev* __restrict__ scenes,
    const float* __restrict__ wave, float2* __restrict__ rho_p, uint16_t* __restrict__ list,
    int32_t* __restrict__ list_cnt, RowMask* __restrict__ masks, float4* __restrict__ xref, int32_t n_total,
    int32_t* status, int32_t allow_stage, const float4* __restrict__ vel, float4* __restrict__ xpair,
    float4* __restrict__ vpair) {
  using T = Real<P>;
  constexpr int kCap = kMaxVerlet;  // the Verlet list build's codes per particle
  // The list build (rare: Verlet rebuilds only) reads candidates from global
  // memory, which keeps its static shared memory under 48 KB.
  constexpr bool kCanStage = ScanShared<MODE>::kCanStage;
  float4* const s_cand = sh.cand;
  StagePlan& sp = sh.sp;
  const SceneDev* S = scenes + tl.scene;
  if (threadIdx.x < 32) plan_stage(S, start, keys, tl, sp);
  __syncthreads();
  const bool staged = kCanStage && allow_stage && sp.ncols > 0;
  if (staged && threadIdx.x < 32) {
    // thread 0 arms the barrier with the stage's bytes, then lane s issues
    // segment s's copy (at most 27 segments: one warp issues them all at once)
    if (threadIdx.x == 0) mbar_expect_tx(&sh.bar, (uint32_t)sp.seg_off[kMaxSegs] * 16u);
    __syncwarp();
    const int s = threadIdx.x;
    if (s < 9 * sp.ncols) {
      const int len = sp.seg_off[s + 1] - sp.seg_off[s];
      if (len > 0) bulk_g2s(&s_cand[sp.seg_off[s]], pos + sp.seg_b[s], (uint32_t)len * 16u, &sh.bar);
    }
  }
  bool ready = true;
  if (staged && !mbar_wait_bounded(&sh.bar, parity)) {
    ready = false;
    if (threadIdx.x == 0) atomicOr(status, kStatusTimeout);
    mbar_wait_bounded(&sh.bar, parity);  // let copies in flight land before the CTA moves on
  }
  const int used = (staged ? 1 : 0) | (ready ? 0 : 2);
  const int i = tl.begin + threadIdx.x;
  if (i >= tl.end || !ready) return used;

  const float4 pi = __ldg(pos + i);
  const T hh = (T)S->h;
  const T hit2 = MODE == MODE_DENSITY ? hh * hh : (T)S->hl2;
  const T px = pi.x, py = pi.y, pz = pi.z;
  const CellCoord c = cell_of_key(S, __ldg(keys + i));
  int b[9], e[9], base[9];
  row_ranges(S, start, pi, c, S->hl2, b, e);
  row_bases(S, start, c, base);
  const int g = staged ? c.x * S->dims[1] + c.y - sp.col0 : 0;
  uint16_t* const hit_col = &sh.hit[0][threadIdx.x];
  uint16_t* const hp_end = hit_col + kCap * kNbThreads;  // the overflow slot (list build)
  uint16_t* hp = hit_col;
  Sum<P> acc;
  bool overflow = false;
  int hits = 0;  // rows with a nonzero mask (bit r)
#pragma unroll
  for (int r = 0; r < 9; ++r) {
    int len = e[r] - b[r];
    if (CWA_DCHECK_FAILED(len == 0 || (b[r] >= 0 && len > 0 && e[r] <= n_total), status)) len = 0;
    const int off0 = b[r] - base[r];
    const float4* cand = pos + b[r];
    bool in_stage = staged && len > 0;
    if (in_stage) {
      const int so = b[r] + sp.seg_delta[g * 9 + r];
      if (CWA_DCHECK_FAILED(g >= 0 && g < sp.ncols && so >= 0 && so + len <= sp.seg_off[kMaxSegs], status))
        len = 0;
      cand = s_cand + so;
    }
    if (MODE == MODE_DENSITY) {
      // row r's hits as bits relative to the row's cell-based start
      RowMask bits = 0u;
      T part = (T)0;
      if (len > 0) {
        if (in_stage) {
          const uint32_t a0 = smem_u32(cand);
          part = scan_row_bits<T>([&](int o) { return lds128(a0 + 16u * (uint32_t)o); }, len, px, py, pz, hit2,
                                  bits);
        } else
          part = scan_row_bits<T>([&](int o) { return __ldg(cand + o); }, len, px, py, pz, hit2, bits);
      }
      overflow |= off0 + len > kMaskBits;
      const RowMask m = off0 < kMaskBits ? bits << off0 : 0u;
      // every row is stored (whole sectors: skipping the zero rows would make
      // each store a partial-sector write that DRAM reads back to merge);
      // force reads only the rows the bitmap names
      masks[(size_t)r * n_total + i] = m;
      if (m != 0u) hits |= 1 << r;
      acc.add(part);
    } else {
      overflow |= off0 + len > kRowCodeMax;
      const uint32_t code0 = ((uint32_t)r << kRowCodeBits) + (uint32_t)off0;
      if (len > 0) {
        if (in_stage)
          scan_row<false, T>([&](int o) { return cand[o]; }, len, code0, px, py, pz, hit2, hp, hp_end);
        else
          scan_row<false, T>([&](int o) { return __ldg(cand + o); }, len, code0, px, py, pz, hit2, hp, hp_end);
      }
    }
  }
  if (MODE == MODE_LIST) {
    // Coalesced list write: the pair (k, k+1) of every lane is one 128-byte
    // store per warp.  (Row k+1 <= kCap exists: s_hit has the overflow row.)
    const int cnt = (int)(hp - hit_col) / kNbThreads;
    overflow |= cnt >= kCap;
    uint32_t* const list32 = reinterpret_cast<uint32_t*>(list);
    for (int k = 0; k < cnt; k += 2)
      list32[(size_t)(k >> 1) * n_total + i] =
          (uint32_t)hit_col[k * kNbThreads] | ((uint32_t)hit_col[(k + 1) * kNbThreads] << 16);
    list_cnt[i] = overflow ? kCap + 1 : cnt;
    xref[i] = pi;
  } else {
    list_cnt[i] = overflow ? -1 : hits;
    const T rho_t = (P == CWA_PREC_FP64 ? (T)S->c_poly6_d : (T)S->c_poly6) * acc.get();
    const float2 rp = eos(S, (float)rho_t, pi, wave);
    rho_p[i] = rp;
    write_pair_rec(xpair, vpair, vel, i, pi, rp);
  }
  return used;
}

// The candidate scan over the tile list, one CTA a tile; or (queue set,
// density mode only) as the work-queue form: resident CTAs take tile
// numbers from the counter *queue and scan tiles[order[t]] until the
// n_tiles of the launch are taken.
template <int P, int MODE, int MINB, bool WQ>
__global__ void __launch_bounds__(kNbThreads, MINB)
    k_scan_cands(const float4* __restrict__ pos, const int32_t* __restrict__ start,
                 const int32_t* __restrict__ keys, const Tile* __restrict__ tiles,
                 const SceneDev* __restrict__ scenes, const float* __restrict__ wave,
                 float2* __restrict__ rho_p, uint16_t* __restrict__ list, int32_t* __restrict__ list_cnt,
                 RowMask* __restrict__ masks, float4* __restrict__ xref, int32_t n_total, int32_t* status,
                 const int32_t* __restrict__ flag,
                 int32_t allow_stage, const float4* __restrict__ vel, float4* __restrict__ xpair,
                 float4* __restrict__ vpair, const int32_t* __restrict__ order, int32_t* queue, int32_t n_tiles) {
  __shared__ ScanShared<MODE> sh;
  __shared__ int32_t s_next;
  if (MODE == MODE_LIST && flag && __ldg(flag) == 0) return;  // no rebuild this step
  if (threadIdx.x == 0) mbar_init(&sh.bar, 1);
  if constexpr (!WQ || MODE != MODE_DENSITY) {
    scan_tile<P, MODE>(sh, tiles[blockIdx.x], 0u, pos, start, keys, scenes, wave, rho_p, list, list_cnt, masks,
                       xref, n_total, status, allow_stage, vel, xpair, vpair);
    return;
  }
  uint32_t parity = 0u;
  for (;;) {
    if (threadIdx.x == 0) s_next = atomicAdd(queue, 1);
    __syncthreads();  // also: every thread is done with the previous tile's stage and plan
    const int t = s_next;
    __syncthreads();  // s_next read by all before thread 0 may take the next number
    if (t >= n_tiles) break;
    const int used = scan_tile<P, MODE>(sh, tiles[__ldg(order + t)], parity, pos, start, keys, scenes, wave, rho_p,
                                        list, list_cnt, masks, xref, n_total, status, allow_stage, vel, xpair,
                                        vpair);
    if (__syncthreads_or(used & 2)) break;  // a staging wait timed out (status set): stop taking tiles
    if (used & 1) parity ^= 1u;
  }
}

// Verlet density: walks the particle's list (pairs within h (1 + skin) at
// the last rebuild), accumulates the poly6 sum over r < h in groups of 8
// (partials folded into the precision mode's accumulator), and writes this
// step's row masks for force.  A particle whose Verlet list overflowed
// rescans the rows of its rebuild cell.
template <int P>
__global__ void __launch_bounds__(kNbThreads, 8)
    k_rho_list(const float4* __restrict__ pos, const int32_t* __restrict__ start,
               const int32_t* __restrict__ keys, const Tile* __restrict__ tiles,
               const SceneDev* __restrict__ scenes, const float* __restrict__ wave,
               float2* __restrict__ rho_p, const uint16_t* __restrict__ vlist,
               const int32_t* __restrict__ vcnt, RowMask* __restrict__ nbm, int32_t* __restrict__ nbr_cnt,
               int32_t n_total, const float4* __restrict__ vel, float4* __restrict__ xpair,
               float4* __restrict__ vpair) {
  using T = Real<P>;
  __shared__ int32_t s_rb[9][kNbThreads];
  __shared__ RowMask s_m[kNbRows][kNbThreads];  // this step's row masks
  const Tile tl = tiles[blockIdx.x];
  const int i = tl.begin + threadIdx.x;
  if (i >= tl.end) return;
  const SceneDev* S = scenes + tl.scene;
  const float4 pi = __ldg(pos + i);
  const T hh = (T)S->h;
  const T h2 = hh * hh;
  const T px = pi.x, py = pi.y, pz = pi.z;
  const CellCoord c = cell_of_key(S, __ldg(keys + i));
  int base[9];
  row_bases(S, start, c, base);
  Sum<P> acc;
  bool overflow = false;
  const int vn = __ldg(vcnt + i);
#pragma unroll
  for (int r = 0; r < kNbRows; ++r) s_m[r][threadIdx.x] = 0u;
  // candidate j at offset off of row r (r < 9): a hit sets its row-mask
  // bit, or marks the particle overflowed when off is past the mask's last bit
  auto test = [&](int j, int r, uint32_t off) {
    const float4 pj = __ldg(pos + j);
    const T dx = px - (T)pj.x, dy = py - (T)pj.y, dz = pz - (T)pj.z;
    T q = fma(-dx, dx, h2);
    q = fma(-dy, dy, q);
    q = fma(-dz, dz, q);
    const T qp = q > (T)0 ? q : (T)0;
    if (q > (T)0) {
      if (off < (uint32_t)kMaskBits)
        s_m[r][threadIdx.x] |= (RowMask)1u << off;
      else
        overflow = true;
    }
    return qp * qp * qp;
  };
  if (vn <= kMaxVerlet) {
#pragma unroll
    for (int r = 0; r < 9; ++r) s_rb[r][threadIdx.x] = base[r];
    for (int k0 = 0; k0 < vn; k0 += 8) {
      uint32_t code[8];
#pragma unroll
      for (int u = 0; u < 8; u += 2) {
        const uint32_t w = k0 + u < vn ? code_pair(vlist, k0 + u, i, n_total) : 0u;
        code[u] = w & 0xFFFFu;
        code[u + 1] = k0 + u + 1 < vn ? w >> 16 : 0u;
      }
      T part = (T)0;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int rr = (int)(code[u] >> kRowCodeBits);
        const uint32_t off = code[u] & (kRowCodeMax - 1);
        const int j = s_rb[rr][threadIdx.x] + (int)off;
        if (k0 + u < vn) part += test(j, rr, off);
      }
      acc.add(part);
    }
  } else {
    // the rows of the rebuild cell over every z cell a pair within
    // h (1 + skin) could occupy; hits take bits against the same bases
    const int z1 = min(c.z + S->rz, S->dims[2] - 1);
#pragma unroll
    for (int r = 0; r < 9; ++r) {
      if (!row_valid(S, c, r)) continue;
      const int e = __ldg(start + row_id(S, c, r) + z1 + 1);
      T part = (T)0;
      for (int j = base[r]; j < e; ++j) part += test(j, r, (uint32_t)(j - base[r]));
      acc.add(part);
    }
  }
  int rows = 0;  // rows with a nonzero mask (bit r)
#pragma unroll
  for (int r = 0; r < kNbRows; ++r) {
    const RowMask m = s_m[r][threadIdx.x];
    nbm[(size_t)r * n_total + i] = m;
    if (m != 0u) rows |= 1 << r;
  }
  nbr_cnt[i] = overflow ? -1 : rows;
  const T rho_t = (P == CWA_PREC_FP64 ? (T)S->c_poly6_d : (T)S->c_poly6) * acc.get();
  const float2 rp = eos(S, (float)rho_t, pi, wave);
  rho_p[i] = rp;
  write_pair_rec(xpair, vpair, vel, i, pi, rp);
}

// The force a particle stores: pressure + viscosity sums (already scaled,
// fpr / fvr) plus gravity, and for REFERENCE_3D the shader's crest, torque,
// drag and wave-normal terms (force_comp.glsl:90-114).
__device__ __forceinline__ float4 force_out(const SceneDev* S, int i, float4 pi, float4 vi, float rho,
                                            const float fpr[3], const float fvr[3], const float4* force,
                                            const float* __restrict__ wave) {
  float4 out;
  if (S->preset == CWA_PRESET_REFERENCE_3D) {
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
    // WaveVelocity (:117-128) and WaveNormal (:130-139)
    const float hx = sample_height(u, W, Hn, s + 0.01f, t);
    const float hy = sample_height(u, W, Hn, s, t + 0.01f);
    const float wv[3] = {(hx - H) / S->dt, (hy - H) / S->dt, (hx - hy) / 0.01f};
    const float hR = sample_height(u, W, Hn, s + 1.0f, t) - H;
    const float hT = sample_height(u, W, Hn, s, t + 1.0f) - H;
    const float nrm[3] = {hR, hT, -1.0f};
    const float vv[3] = {vi.x, vi.y, vi.z};
    float f[3];
#pragma unroll
    for (int c2 = 0; c2 < 3; ++c2) {
      const float drag = -0.25f * (vv[c2] - wv[c2]);
      const float wf = -H * nrm[c2] * 0.5f;
      f[c2] = fpr[c2] + fvr[c2] * vs + rho * S->g[c2] + tq[c2] + drag + wf;
    }
    out = make_float4(f[0], f[1], f[2], fprev.w);
  } else {
    out = make_float4(fpr[0] + fvr[0] * S->visc + rho * S->g[0], fpr[1] + fvr[1] * S->visc + rho * S->g[1],
                      fpr[2] + fvr[2] * S->visc + rho * S->g[2], 0.0f);
  }
  return out;
}

// Three-component sum in the precision mode: COMPENSATED adds pair terms
// in float into a partial that the caller folds into a two-sum accumulator
// after every group of 8 pairs (cascaded summation); FP32 is plain; FP64 is
// double.
template <int P>
struct Acc3 {
  Sum<P> x, y, z;
  Real<P> px = 0, py = 0, pz = 0;
  __device__ __forceinline__ void add(Real<P> a, Real<P> b, Real<P> c) {
    if (P == CWA_PREC_COMPENSATED) {
      px += a;
      py += b;
      pz += c;
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
    }
  }
};

// force: spiky pressure gradient + viscosity Laplacian over the step's hits
// (the row masks), then the preset's extra terms.  A particle whose masks
// overflowed rescans the rows of its cell over every z cell a neighbour can
// occupy.  Neighbour data comes from global memory (L1-resident for the most
// part: a CTA's particles share their candidate rows).  Staging the rows'
// records in shared memory, as the candidate scan does, measured slower
// here: 48 KB of stage per CTA halves the resident warps this latency-bound
// loop needs.
template <int P>
__device__ __forceinline__ void force_tile(
    RowMask (&s_w)[kNbRows][kNbThreads], int32_t (&s_jb)[kNbRows][kNbThreads], const Tile tl,
    const float4* __restrict__ pos, const float4* __restrict__ vel, const float2* __restrict__ rho_p,
    const int32_t* __restrict__ start, const int32_t* __restrict__ keys, const SceneDev* __restrict__ scenes,
    const float* __restrict__ wave, float4* __restrict__ force, const RowMask* __restrict__ nbm,
    const int32_t* __restrict__ nbr_cnt, int32_t n_total, const float4* __restrict__ xpair,
    const float4* __restrict__ vpair, int32_t* status) {
  using T = Real<P>;
  const SceneDev* S = scenes + tl.scene;
  const int i = tl.begin + threadIdx.x;
  if (i >= tl.end) return;
  // FP32 modes read the particle's own position and velocity from its gather
  // records (the same floats, and lines its neighbours' gathers share)
  const float4 pi = P == CWA_PREC_FP64 ? __ldg(pos + i) : __ldg(xpair + i);
  const float4 vi = P == CWA_PREC_FP64 ? __ldg(vel + i) : __ldg(vpair + i);
  const float2 rpi = __ldg(rho_p + i);
  const T hh = (T)S->h;
  const T h2 = hh * hh;
  const T px = pi.x, py = pi.y, pz = pi.z;
  const T vx = vi.x, vy = vi.y, vz = vi.z, pres_i = rpi.y;
  Acc3<P> fp, fv;
  auto pair = [&](float4 pj, float4 vj, T irho, T pres_j) {
    const T dx = px - (T)pj.x, dy = py - (T)pj.y, dz = pz - (T)pj.z;
    const T r2 = dx * dx + dy * dy + dz * dz;
    const T inv_r = r2 > (T)0 ? inv_sqrt(r2) : (T)0;  // normalize(0) := 0
    const T r = r2 * inv_r;
    const T hr = hh - r;
    const T sp = (pres_i + pres_j) * irho * hr * hr * inv_r;
    fp.add(sp * dx, sp * dy, sp * dz);
    const T sv = irho * hr;
    fv.add(sv * ((T)vj.x - vx), sv * ((T)vj.y - vy), sv * ((T)vj.z - vz));
  };
  // FP32 modes read the density pass's records; FP64 gathers pos, vel and
  // (rho, p) and divides in double.
  auto pair_global = [&](int j) {
    if (P == CWA_PREC_FP64) {
      const float2 rpj = __ldg(rho_p + j);
      pair(__ldg(pos + j), __ldg(vel + j), recip((T)rpj.x), (T)rpj.y);
    } else {
      const float4 xj = __ldg(xpair + j), vj = __ldg(vpair + j);
      pair(xj, vj, (T)vj.w, (T)xj.w);
    }
  };
  const int cnt = __ldg(nbr_cnt + i);
  const CellCoord c = cell_of_key(S, __ldg(keys + i));
  int base[9];
  row_bases(S, start, c, base);
  if (cnt >= 0) {
    // The row masks hold the particle itself: row 4 (its own column) at bit
    // i - base[4], cleared here.  Only the nonzero masks are loaded, back to
    // back, and compacted in row order, and
    // hits are then popped in row then bit order, in groups of 8 whose
    // neighbour indexes are found first so the gathers overlap.
    int nw = 0, left = 0;
#pragma unroll
    for (int r = 0; r < kNbRows; ++r) {
      // cnt: the rows with hits, as bits; the zero rows are not read
      RowMask m = (cnt >> r) & 1 ? __ldg(nbm + (size_t)r * n_total + i) : (RowMask)0u;
      if (r == 4 && i - base[4] < kMaskBits) m &= ~((RowMask)1u << (i - base[4]));
      if (m) {
        s_w[nw][threadIdx.x] = m;
        s_jb[nw][threadIdx.x] = base[r];
        ++nw;
      }
      left += __popcll(m);
    }
    int wi = 0;
    RowMask cw = nw > 0 ? s_w[0][threadIdx.x] : 0u;
    int jb = nw > 0 ? s_jb[0][threadIdx.x] : 0;
    for (int k0 = 0; k0 < left; k0 += 8) {
      int js[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        js[u] = -1;
        if (k0 + u < left) {
          if (cw == 0u) {  // the next mask (every compacted mask holds a hit)
            ++wi;
            cw = s_w[wi][threadIdx.x];
            jb = s_jb[wi][threadIdx.x];
          }
          js[u] = jb + __ffsll((long long)cw) - 1;
          cw &= cw - 1u;
        }
      }
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (js[u] >= 0 && !CWA_DCHECK_FAILED(js[u] < n_total, status)) pair_global(js[u]);
      fp.flush();
      fv.flush();
    }
  } else {
    const int z1 = min(c.z + S->rz, S->dims[2] - 1);
#pragma unroll
    for (int r = 0; r < 9; ++r) {
      if (!row_valid(S, c, r)) continue;
      const int e = __ldg(start + row_id(S, c, r) + z1 + 1);
      for (int j = base[r]; j < e; ++j) {
        const float4 pj = __ldg(pos + j);
        const T dx = px - (T)pj.x, dy = py - (T)pj.y, dz = pz - (T)pj.z;
        T q = fma(-dx, dx, h2);
        q = fma(-dy, dy, q);
        q = fma(-dz, dz, q);
        if (q > (T)0 && j != i) pair_global(j);
      }
      fp.flush();
      fv.flush();
    }
  }
  fp.flush();
  fv.flush();
  const T cg = P == CWA_PREC_FP64 ? (T)S->k_grad_d * (T)S->mass : (T)(S->k_grad * S->mass);
  const T cp = (T)0.5 * cg;
  float fpr[3] = {(float)(cp * fp.x.get()), (float)(cp * fp.y.get()), (float)(cp * fp.z.get())};
  float fvr[3] = {(float)(cg * fv.x.get()), (float)(cg * fv.y.get()), (float)(cg * fv.z.get())};
  force[i] = force_out(S, i, pi, vi, rpi.x, fpr, fvr, force, wave);
}

// The force pass over the tile list, one CTA a tile, or (queue set) in the
// work-queue form.
template <int P, int MINB, bool WQ>
__global__ void __launch_bounds__(kNbThreads, MINB)
    k_force(const float4* __restrict__ pos, const float4* __restrict__ vel,
            const float2* __restrict__ rho_p, const int32_t* __restrict__ start,
            const int32_t* __restrict__ keys, const Tile* __restrict__ tiles,
            const SceneDev* __restrict__ scenes, const float* __restrict__ wave, float4* __restrict__ force,
            const RowMask* __restrict__ nbm, const int32_t* __restrict__ nbr_cnt, int32_t n_total,
            const float4* __restrict__ xpair, const float4* __restrict__ vpair, int32_t* status,
            const int32_t* __restrict__ order, int32_t* queue, int32_t n_tiles) {
  // the particle's nonzero row masks and the index of each mask's bit 0
  // (13.8 KB a CTA; 32-bit masks, 9.2 KB a CTA, measured slower: 209 against
  // 143 us over the C1 run).  The default variant runs nine CTAs a SM at 56
  // registers: 135.9 against 139.2 us at eight (64 registers), though nine
  // CTAs' arrays leave the L1 a smaller share of the SM's 256 KB.
  __shared__ RowMask s_w[kNbRows][kNbThreads];
  __shared__ int32_t s_jb[kNbRows][kNbThreads];
  if constexpr (!WQ) {
    force_tile<P>(s_w, s_jb, tiles[blockIdx.x], pos, vel, rho_p, start, keys, scenes, wave, force, nbm, nbr_cnt,
                  n_total, xpair, vpair, status);
  } else {
    // work-queue form: resident CTAs take tile numbers from *queue
    __shared__ int32_t s_next[2];
    for (int it = 0;; ++it) {
      if (threadIdx.x == 0) s_next[it & 1] = atomicAdd(queue, 1);
      __syncthreads();  // (two slots: thread 0 refills one while the other is still being read)
      const int t = s_next[it & 1];
      if (t >= n_tiles) break;
      force_tile<P>(s_w, s_jb, tiles[__ldg(order + t)], pos, vel, rho_p, start, keys, scenes, wave, force, nbm,
                    nbr_cnt, n_total, xpair, vpair, status);
    }
  }
}

// Grid of a work-queue launch: the CTAs of `kernel` that fit the device at
// once (occupancy x SMs), at most n_tiles.
template <typename K>
int queue_grid(K kernel, int block, int n_tiles) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess || per_sm < 1)
    return n_tiles;
  return std::min(n_tiles, per_sm * sms);
}

// Launch-bound variants (min CTAs per SM): the register budget trades
// occupancy against loads in flight per warp; the autotuner picks one.
// queue (density mode): the work-queue form, its counter zeroed first.
template <int P, int MODE, int MB>
void scan_launch_one(const NbArgs& a, uint16_t* list, int32_t* cnt, RowMask* masks, float4* xref,
                     const int32_t* flag, int32_t* queue, cudaStream_t st) {
  auto kern = queue ? k_scan_cands<P, MODE, MB, true> : k_scan_cands<P, MODE, MB, false>;
  int grid = a.n_tiles;
  if (queue) {
    cudaMemsetAsync(queue, 0, sizeof(int32_t), st);
    grid = queue_grid(kern, a.tile_size, a.n_tiles);
  }
  kern<<<grid, a.tile_size, 0, st>>>(a.pos, a.start, a.keys, a.tiles, a.scenes, a.wave, a.rho_p, list, cnt, masks,
                                     xref, a.n_total, a.status, flag, a.stage, a.vel, a.xpair, a.vpair, a.order,
                                     queue, a.n_tiles);
}

template <int P, int MODE>
void scan_variant(int minb, const NbArgs& a, uint16_t* list, int32_t* cnt, RowMask* masks, float4* xref,
                  const int32_t* flag, int32_t* queue, cudaStream_t st) {
  if (minb >= 8)
    scan_launch_one<P, MODE, 8>(a, list, cnt, masks, xref, flag, queue, st);
  else if (minb >= 6)
    scan_launch_one<P, MODE, 6>(a, list, cnt, masks, xref, flag, queue, st);
  else
    scan_launch_one<P, MODE, 4>(a, list, cnt, masks, xref, flag, queue, st);
}

template <int P>
void dispatch_scan(bool list_mode, const NbArgs& a, cudaStream_t st) {
  if (list_mode)
    scan_variant<P, MODE_LIST>(a.scan_minb, a, a.vlist, a.vcnt, nullptr, a.xref, a.flag, nullptr, st);
  else
    scan_variant<P, MODE_DENSITY>(a.scan_minb, a, nullptr, a.nbr_cnt, a.nbm, nullptr, nullptr,
                                  a.queue, st);
}

template <int P, int MB>
void force_variant(const NbArgs& a, cudaStream_t st) {
  int32_t* queue = a.queue ? a.queue + 1 : nullptr;
  auto kern = queue ? k_force<P, MB, true> : k_force<P, MB, false>;
  int grid = a.n_tiles;
  if (queue) {
    cudaMemsetAsync(queue, 0, sizeof(int32_t), st);
    grid = queue_grid(kern, a.tile_size, a.n_tiles);
  }
  kern<<<grid, a.tile_size, 0, st>>>(a.pos, a.vel, a.rho_p, a.start, a.keys, a.tiles, a.scenes, a.wave, a.force,
                                     a.nbm, a.nbr_cnt, a.n_total, a.xpair, a.vpair, a.status, a.order, queue,
                                     a.n_tiles);
}

template <int P>
void dispatch_force(const NbArgs& a, cudaStream_t st) {
  // FP64 keeps eight CTAs a SM for nine: its 56-register form spills more
  if constexpr (P != CWA_PREC_FP64) {
    if (a.force_minb >= 9) {
      force_variant<P, 9>(a, st);
      return;
    }
  }
  if (a.force_minb >= 8)
    force_variant<P, 8>(a, st);
  else
    force_variant<P, 6>(a, st);
}

}  // namespace

cudaError_t launch_scan_cands(int precision, bool list_mode, const NbArgs& a, cudaStream_t stream) {
  if (a.n_tiles <= 0) return cudaSuccess;
  switch (precision) {
    case CWA_PREC_FP32: dispatch_scan<CWA_PREC_FP32>(list_mode, a, stream); break;
    case CWA_PREC_FP64: dispatch_scan<CWA_PREC_FP64>(list_mode, a, stream); break;
    default: dispatch_scan<CWA_PREC_COMPENSATED>(list_mode, a, stream);
  }
  return cudaGetLastError();
}

cudaError_t launch_rho_list(int precision, const NbArgs& a, cudaStream_t stream) {
  if (a.n_tiles <= 0) return cudaSuccess;
#define CWA_RHO_LIST(P)                                                                                     \
  k_rho_list<P><<<a.n_tiles, a.tile_size, 0, stream>>>(a.pos, a.start, a.keys, a.tiles, a.scenes, a.wave,  \
                                                       a.rho_p, a.vlist, a.vcnt, a.nbm, a.nbr_cnt, a.n_total, \
                                                       a.vel, a.xpair, a.vpair)
  switch (precision) {
    case CWA_PREC_FP32: CWA_RHO_LIST(CWA_PREC_FP32); break;
    case CWA_PREC_FP64: CWA_RHO_LIST(CWA_PREC_FP64); break;
    default: CWA_RHO_LIST(CWA_PREC_COMPENSATED);
  }
#undef CWA_RHO_LIST
  return cudaGetLastError();
}

cudaError_t launch_force(int precision, const NbArgs& a, cudaStream_t stream) {
  if (a.n_tiles <= 0) return cudaSuccess;
  switch (precision) {
    case CWA_PREC_FP32: dispatch_force<CWA_PREC_FP32>(a, stream); break;
    case CWA_PREC_FP64: dispatch_force<CWA_PREC_FP64>(a, stream); break;
    default: dispatch_force<CWA_PREC_COMPENSATED>(a, stream);
  }
  return cudaGetLastError();
}

}  // namespace cwa
