// cwa_grid.cu — uniform-grid counting sort: cell hash + count, single-pass
// exclusive scan (decoupled look-back), stable insert, reorder.
//
// Replaces the reference's COMPUTE_COUNTS / ParallelScan / INSERT sequence
// (SphWave2D/UniformGridGpu2D.cpp:220-265, SphWave2D/uniform_grid_sph_cs.glsl:112-165,
// UniformGrid2D/ugrid_particles_cs.glsl:90-117, SphWave2D/ParallelScan.cpp:43-95,
// SphWave2D/prefix_sum_cs.glsl:18-43).  Differences by design:
//   * the insert is stable (input order within a cell) instead of atomic
//     arrival order, so the sorted order is deterministic;
//   * the scan is one launch for any n instead of 2*log2(n) dispatches over
//     a power-of-two array;
//   * particle state is moved into sorted order so the neighbour passes read
//     contiguous cell ranges.
#include <cuda_runtime.h>

#include "cwa_device.cuh"
#include "cwa_internal.h"

namespace cwa {
namespace {

constexpr int kScanBlock = 512;
constexpr int kScanItems = 16;  // 8192-item tiles: 147 tiles for the 1.2M cells of the 1M-particle grid, one wave
constexpr int kScanTile = kScanBlock * kScanItems;
static_assert(kScanTile == kScanTileItems, "workspace sizes assume kScanTileItems items a tile");
constexpr unsigned long long kFlagAgg = 1ull << 32;
constexpr unsigned long long kFlagInc = 2ull << 32;
constexpr long kSpinLimit = 1l << 22;
constexpr int kLookBack = 128;  // predecessor states a look-back round reads (4 a lane)

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One tile of kScanTile items per CTA; tiles are ticketed in start order so a
// CTA only ever waits on CTAs that are already running.  A ticket at or past
// n_tiles (possible only when scans sharing one workspace overlap on the GPU)
// sets the time-out bit and touches nothing, so the tile-state writes never
// leave the workspace.  kVec: in and out
// are 16-byte aligned, so each thread moves its 16 items as four int4s
// (a vector that would cross n_in / n_out falls back to scalar accesses).
template <bool kZero, bool kVec>
__global__ void __launch_bounds__(kScanBlock)
    k_scan(int32_t* in, int32_t* out, int32_t n_in, int32_t n_out, unsigned int* counter,
           unsigned long long* state, int32_t n_tiles, int32_t* status, const int32_t* flag) {
  chain_enter();
  __shared__ int s_tile, s_prefix;
  if (flag && __ldg(flag) == 0) return;  // grid kept this step (Verlet mode)
  __shared__ int s_warp[kScanBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(counter, 1u);
  __syncthreads();
  const int tile = s_tile;
  if (tile >= n_tiles) {
    if (threadIdx.x == 0) atomicOr(status, kStatusTimeout);
    return;
  }
  const long base = (long)tile * kScanTile + (long)threadIdx.x * kScanItems;

  int v[kScanItems];
  if (kVec) {
#pragma unroll
    for (int q = 0; q < kScanItems / 4; ++q) {
      const long idx = base + 4 * q;
      if (idx + 3 < n_in) {
        const int4 x = *reinterpret_cast<const int4*>(in + idx);
        v[4 * q] = x.x;
        v[4 * q + 1] = x.y;
        v[4 * q + 2] = x.z;
        v[4 * q + 3] = x.w;
        if (kZero) *reinterpret_cast<int4*>(in + idx) = make_int4(0, 0, 0, 0);
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          v[4 * q + k] = idx + k < n_in ? in[idx + k] : 0;
          if (kZero && idx + k < n_in) in[idx + k] = 0;
        }
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      long idx = base + k;
      v[k] = idx < n_in ? in[idx] : 0;
    }
    if (kZero) {
#pragma unroll
      for (int k = 0; k < kScanItems; ++k)
        if (base + k < n_in) in[base + k] = 0;
    }
  }
  int tsum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    int x = v[k];
    v[k] = tsum;
    tsum += x;
  }
  int incl = tsum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  int warp_excl = 0, total = 0;
#pragma unroll
  for (int w = 0; w < kScanBlock / 32; ++w) {
    int s = s_warp[w];
    if (w < warp) warp_excl += s;
    total += s;
  }
  const int thread_excl = warp_excl + incl - tsum;

  if (warp == 0) {
    if (tile == 0) {
      if (lane == 0) {
        st_relaxed(state, kFlagInc | (unsigned int)total);
        s_prefix = 0;
      }
    } else {
      if (lane == 0) st_relaxed(state + tile, kFlagAgg | (unsigned int)total);
      // Look back over windows of kLookBack predecessors (4 a lane, one
      // round trip of loads): sum the aggregates nearer than the nearest
      // inclusive prefix, plus that prefix; wait only while one of those
      // nearer tiles has published nothing.  Tiles before 0 read as an
      // inclusive prefix of 0.
      int pred = tile - 1;
      int excl = 0;
      long spins = 0;
      while (true) {
        unsigned long long sv[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int idx = pred - (q * 32 + lane);
          sv[q] = idx >= 0 ? ld_relaxed(state + idx) : kFlagInc;
        }
        int near_inc = kLookBack;  // distance of the nearest inclusive prefix
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if ((unsigned int)(sv[q] >> 32) == 2u) near_inc = min(near_inc, q * 32 + lane);
        near_inc = __reduce_min_sync(0xffffffffu, near_inc);
        bool pending = false;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          pending |= q * 32 + lane < near_inc && (unsigned int)(sv[q] >> 32) == 0u;
        if (__any_sync(0xffffffffu, pending)) {
          if (++spins > kSpinLimit) {
            if (lane == 0) atomicOr(status, kStatusTimeout);
            break;
          }
          __nanosleep(32);
          continue;
        }
        int part = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (q * 32 + lane <= near_inc) part += (int)(unsigned int)sv[q];
        excl += warp_sum(part);
        if (near_inc < kLookBack) break;
        pred -= kLookBack;
      }
      if (lane == 0) {
        st_relaxed(state + tile, kFlagInc | (unsigned int)(excl + total));
        s_prefix = excl;
      }
    }
  }
  __syncthreads();
  const int prefix = s_prefix + thread_excl;
  if (kVec) {
#pragma unroll
    for (int q = 0; q < kScanItems / 4; ++q) {
      const long idx = base + 4 * q;
      if (idx + 3 < n_out) {
        *reinterpret_cast<int4*>(out + idx) =
            make_int4(prefix + v[4 * q], prefix + v[4 * q + 1], prefix + v[4 * q + 2], prefix + v[4 * q + 3]);
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (idx + k < n_out) out[idx + k] = prefix + v[4 * q + k];
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      long idx = base + k;
      if (idx < n_out) out[idx] = prefix + v[k];
    }
  }
}

// Two-pass form of the same exclusive scan, for the sim's grid pass: first
// every tile's total (k_tile_sum), then every tile adds the totals of the
// tiles before it to its own local scan (k_tile_scan).  The input is read
// twice (4.8 MB at the 1M-particle grid, from L2 the second time) but no
// tile waits on another, where the look-back chain of k_scan kept each CTA
// resident ~12 us for a ~5 us job.
template <bool kVec>
__device__ __forceinline__ void load_tile_items(const int32_t* in, int32_t n_in, long base, int (&v)[kScanItems]) {
  if (kVec) {
#pragma unroll
    for (int q = 0; q < kScanItems / 4; ++q) {
      const long idx = base + 4 * q;
      if (idx + 3 < n_in) {
        const int4 x = *reinterpret_cast<const int4*>(in + idx);
        v[4 * q] = x.x;
        v[4 * q + 1] = x.y;
        v[4 * q + 2] = x.z;
        v[4 * q + 3] = x.w;
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) v[4 * q + k] = idx + k < n_in ? in[idx + k] : 0;
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) v[k] = base + k < n_in ? in[base + k] : 0;
  }
}

template <bool kVec>
__global__ void __launch_bounds__(kScanBlock)
    k_tile_sum(const int32_t* in, int32_t n_in, int32_t* __restrict__ sums, const int32_t* flag) {
  chain_enter();
  if (flag && __ldg(flag) == 0) return;  // grid kept this step (Verlet mode)
  __shared__ int s_warp[kScanBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long base = (long)blockIdx.x * kScanTile + (long)threadIdx.x * kScanItems;
  int v[kScanItems];
  load_tile_items<kVec>(in, n_in, base, v);
  int t = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) t += v[k];
  t = warp_sum(t);
  if (lane == 0) s_warp[warp] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    int total = 0;
#pragma unroll
    for (int w = 0; w < kScanBlock / 32; ++w) total += s_warp[w];
    sums[blockIdx.x] = total;
  }
}

template <bool kZero, bool kVec>
__global__ void __launch_bounds__(kScanBlock)
    k_tile_scan(int32_t* in, int32_t* out, int32_t n_in, int32_t n_out, const int32_t* __restrict__ sums,
                const int32_t* flag) {
  chain_enter();
  if (flag && __ldg(flag) == 0) return;
  __shared__ int s_warp[kScanBlock / 32];
  __shared__ int s_prefix;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int tile = blockIdx.x;
  if (warp == 0) {  // the totals of the tiles before this one
    int p = 0;
    for (int t = lane; t < tile; t += 32) p += sums[t];
    p = warp_sum(p);
    if (lane == 0) s_prefix = p;
  }
  const long base = (long)tile * kScanTile + (long)threadIdx.x * kScanItems;
  int v[kScanItems];
  load_tile_items<kVec>(in, n_in, base, v);
  if (kZero) {
    if (kVec) {
#pragma unroll
      for (int q = 0; q < kScanItems / 4; ++q) {
        const long idx = base + 4 * q;
        if (idx + 3 < n_in)
          *reinterpret_cast<int4*>(in + idx) = make_int4(0, 0, 0, 0);
        else
          for (int k = 0; k < 4; ++k)
            if (idx + k < n_in) in[idx + k] = 0;
      }
    } else {
#pragma unroll
      for (int k = 0; k < kScanItems; ++k)
        if (base + k < n_in) in[base + k] = 0;
    }
  }
  int tsum = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const int x = v[k];
    v[k] = tsum;
    tsum += x;
  }
  int incl = tsum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  int warp_excl = 0;
#pragma unroll
  for (int w = 0; w < kScanBlock / 32; ++w)
    if (w < warp) warp_excl += s_warp[w];
  const int prefix = s_prefix + warp_excl + incl - tsum;
  if (kVec) {
#pragma unroll
    for (int q = 0; q < kScanItems / 4; ++q) {
      const long idx = base + 4 * q;
      if (idx + 3 < n_out) {
        *reinterpret_cast<int4*>(out + idx) =
            make_int4(prefix + v[4 * q], prefix + v[4 * q + 1], prefix + v[4 * q + 2], prefix + v[4 * q + 3]);
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (idx + k < n_out) out[idx + k] = prefix + v[4 * q + k];
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
      if (base + k < n_out) out[base + k] = prefix + v[k];
  }
}

__global__ void __launch_bounds__(256)
    k_hash_count(const float4* __restrict__ pos, const Tile* __restrict__ tiles,
                 const SceneDev* __restrict__ scenes, int32_t* __restrict__ key,
                 int32_t* __restrict__ slot, int32_t* __restrict__ count, int32_t* status,
                 const int32_t* flag) {
  chain_enter();
  if (flag && __ldg(flag) == 0) return;
  const Tile t = tiles[blockIdx.x];
  const SceneDev* S = scenes + t.scene;
  const float lx = S->lo[0], ly = S->lo[1], lz = S->lo[2], cs = S->cell, csz = S->cellz;
  const int nx = S->dims[0], ny = S->dims[1], nz = S->dims[2], coff = S->coff;
  for (int i = t.begin + threadIdx.x; i < t.end; i += blockDim.x) {
    float4 p = pos[i];
    if (!finite3(p)) atomicOr(status, kStatusNonFinite);
    int cx = cell_axis(p.x, lx, cs, nx);
    int cy = cell_axis(p.y, ly, cs, ny);
    int cz = cell_axis(p.z, lz, csz, nz);
    int k = coff + (cx * ny + cy) * nz + cz;
    if (CWA_DCHECK_FAILED(k >= coff && k < coff + nx * ny * nz, status)) continue;
    key[i] = k;
    slot[i] = count_slot(count, k);
  }
}

__global__ void k_point_hash(const float4* __restrict__ pos, int32_t n, float lx, float ly, float lz,
                             float cs, int32_t nx, int32_t ny, int32_t nz, int32_t* __restrict__ key,
                             int32_t* __restrict__ slot, int32_t* __restrict__ count, int32_t* status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float4 p = pos[i];
  if (!finite3(p)) atomicOr(status, kStatusNonFinite);
  int k = (cell_axis(p.x, lx, cs, nx) * ny + cell_axis(p.y, ly, cs, ny)) * nz + cell_axis(p.z, lz, cs, nz);
  key[i] = k;
  slot[i] = count_slot(count, k);
}

__global__ void k_list_insert(const int32_t* __restrict__ key, const int32_t* __restrict__ slot,
                              const int32_t* __restrict__ start, int32_t* __restrict__ list, int32_t n,
                              const int32_t* flag, int32_t* status) {
  chain_enter();
  if (flag && __ldg(flag) == 0) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = key[i], dst = start[k] + slot[i];
  if (CWA_DCHECK_FAILED(k >= 0 && dst >= start[k] && dst < start[k + 1] && dst < n, status)) return;
  list[dst] = i;
}

// Stable rank of particle i in its cell = members with a smaller index.
__device__ __forceinline__ int stable_rank(const int32_t* __restrict__ list, int b, int e, int i,
                                           int slot, int32_t* status) {
  if (e - b > kMaxStableCell) {
    if (slot == 0) atomicOr(status, kStatusBigCell);
    return slot;
  }
  int r = 0;
  for (int m = b; m < e; ++m) r += list[m] < i;
  return r;
}

__global__ void __launch_bounds__(256)
    k_rank_reorder(const int32_t* __restrict__ key, const int32_t* __restrict__ slot,
                   const int32_t* __restrict__ start, const int32_t* __restrict__ list,
                   const float4* __restrict__ pin, const float4* __restrict__ vin,
                   const float4* __restrict__ fin, const int32_t* __restrict__ idin,
                   float4* __restrict__ pout, float4* __restrict__ vout, float4* __restrict__ fout,
                   int32_t* __restrict__ idout, int32_t* __restrict__ kout, int32_t n, int32_t* status,
                   const int32_t* flag) {
  chain_enter();
  if (flag && __ldg(flag) == 0) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int k = key[i];
  int b = start[k], e = start[k + 1];
  int dst = b + stable_rank(list, b, e, i, slot[i], status);
  if (CWA_DCHECK_FAILED(dst >= b && dst < e && dst < n, status)) return;
  pout[dst] = pin[i];
  vout[dst] = vin[i];
  if (fout) fout[dst] = fin[i];
  idout[dst] = idin[i];
  kout[dst] = k;
}

__global__ void __launch_bounds__(256)
    k_copy_back(const float4* __restrict__ p2, const float4* __restrict__ v2, const float4* __restrict__ f2,
                const int32_t* __restrict__ id2, float4* __restrict__ p, float4* __restrict__ v,
                float4* __restrict__ f, int32_t* __restrict__ id, int32_t n, const int32_t* flag,
                unsigned long long* rebuilds) {
  chain_enter();
  if (__ldg(flag) == 0) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(rebuilds, 1ull);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    p[i] = p2[i];
    v[i] = v2[i];
    if (f) f[i] = f2[i];
    id[i] = id2[i];
  }
}

__global__ void k_point_rank(const int32_t* __restrict__ key, const int32_t* __restrict__ slot,
                             const int32_t* __restrict__ start, const int32_t* __restrict__ list,
                             int32_t n, int32_t* __restrict__ sorted_index, int32_t* status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int k = key[i];
  int b = start[k], e = start[k + 1];
  sorted_index[b + stable_rank(list, b, e, i, slot[i], status)] = i;
}

inline int blocks_for(long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

int scan_tile_items() { return kScanTile; }

size_t scan_workspace_bytes(int32_t n_out) {
  long tiles = blocks_for(n_out > 0 ? n_out : 1, kScanTile);
  return 256 + (size_t)tiles * sizeof(unsigned long long);
}

void scan_bind_workspace(void* ws, int32_t n_out, ScanWorkspace* out) {
  out->counter = reinterpret_cast<unsigned int*>(ws);
  out->state = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(ws) + 256);
  out->n_tiles = blocks_for(n_out > 0 ? n_out : 1, kScanTile);
}

cudaError_t scan_launch(const int32_t* in, int32_t* out, int32_t n_in, int32_t n_out, bool zero_input,
                        const ScanWorkspace& ws, int32_t* status, cudaStream_t stream, int64_t* launches,
                        const int32_t* flag) {
  if (n_out <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(ws.counter, 0, 256 + (size_t)ws.n_tiles * 8, stream);
  if (e != cudaSuccess) return e;
  int32_t* inw = const_cast<int32_t*>(in);
  const bool vec = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
#define CWA_SCAN_K(Z, V) \
  k_scan<Z, V><<<ws.n_tiles, kScanBlock, 0, stream>>>(inw, out, n_in, n_out, ws.counter, ws.state, ws.n_tiles, \
                                                       status, flag)
  if (zero_input) {
    if (vec)
      CWA_SCAN_K(true, true);
    else
      CWA_SCAN_K(true, false);
  } else {
    if (vec)
      CWA_SCAN_K(false, true);
    else
      CWA_SCAN_K(false, false);
  }
#undef CWA_SCAN_K
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t scan_launch_two_pass(int32_t* in, int32_t* out, int32_t n_in, int32_t n_out, bool zero_input,
                                 const ScanWorkspace& ws, cudaStream_t stream, int64_t* launches,
                                 const int32_t* flag) {
  if (n_out <= 0) return cudaSuccess;
  int32_t* sums = reinterpret_cast<int32_t*>(ws.state);  // n_tiles ints in the tile-state area
  const bool vec = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
  const dim3 grid(ws.n_tiles), block(kScanBlock);
  cudaError_t e;
  if (vec)
    e = launch_chained(k_tile_sum<true>, grid, block, 0, stream, in, n_in, sums, flag);
  else
    e = launch_chained(k_tile_sum<false>, grid, block, 0, stream, in, n_in, sums, flag);
  if (e != cudaSuccess) return e;
  if (zero_input) {
    if (vec)
      e = launch_chained(k_tile_scan<true, true>, grid, block, 0, stream, in, out, n_in, n_out, sums, flag);
    else
      e = launch_chained(k_tile_scan<true, false>, grid, block, 0, stream, in, out, n_in, n_out, sums, flag);
  } else {
    if (vec)
      e = launch_chained(k_tile_scan<false, true>, grid, block, 0, stream, in, out, n_in, n_out, sums, flag);
    else
      e = launch_chained(k_tile_scan<false, false>, grid, block, 0, stream, in, out, n_in, n_out, sums, flag);
  }
  if (launches) *launches += 2;
  return e;
}

cudaError_t launch_hash_count(const float4* pos, const Tile* tiles, int32_t n_tiles, int32_t tile_size,
                              const SceneDev* scenes, int32_t* key, int32_t* slot, int32_t* count,
                              int32_t* status, const int32_t* flag, cudaStream_t stream) {
  if (n_tiles <= 0) return cudaSuccess;
  launch_chained(k_hash_count, dim3(n_tiles), dim3(tile_size), 0, stream, pos, tiles, scenes, key, slot, count,
                 status, flag);
  return cudaGetLastError();
}

cudaError_t launch_list_insert(const int32_t* key, const int32_t* slot, const int32_t* start, int32_t* list,
                               int32_t n, const int32_t* flag, cudaStream_t stream, int32_t* status) {
  if (n <= 0) return cudaSuccess;
  launch_chained(k_list_insert, dim3(blocks_for(n, 256)), dim3(256), 0, stream, key, slot, start, list, n, flag,
                 status);
  return cudaGetLastError();
}

cudaError_t launch_rank_reorder(const int32_t* key, const int32_t* slot, const int32_t* start,
                                const int32_t* list, const float4* pin, const float4* vin,
                                const float4* fin, const int32_t* idin, float4* pout, float4* vout,
                                float4* fout, int32_t* idout, int32_t* kout, int32_t n, int32_t* status,
                                const int32_t* flag, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  launch_chained(k_rank_reorder, dim3(blocks_for(n, 256)), dim3(256), 0, stream, key, slot, start, list, pin,
                 vin, fin, idin, pout, vout, fout, idout, kout, n, status, flag);
  return cudaGetLastError();
}

cudaError_t launch_copy_back(const float4* p2, const float4* v2, const float4* f2, const int32_t* id2,
                             float4* p, float4* v, float4* f, int32_t* id, int32_t n, const int32_t* flag,
                             unsigned long long* rebuilds, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  launch_chained(k_copy_back, dim3(min(blocks_for(n, 256), 1216)), dim3(256), 0, stream, p2, v2, f2, id2, p, v,
                 f, id, n, flag, rebuilds);
  return cudaGetLastError();
}

cudaError_t launch_point_hash(const float4* pos, int32_t n, float lx, float ly, float lz, float cell,
                              int32_t dx, int32_t dy, int32_t dz, int32_t* key, int32_t* slot,
                              int32_t* count, int32_t* status, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_point_hash<<<blocks_for(n, 256), 256, 0, stream>>>(pos, n, lx, ly, lz, cell, dx, dy, dz, key, slot,
                                                       count, status);
  return cudaGetLastError();
}

cudaError_t launch_point_rank(const int32_t* key, const int32_t* slot, const int32_t* start,
                              const int32_t* list, int32_t n, int32_t* sorted_index, int32_t* status,
                              cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  k_point_rank<<<blocks_for(n, 256), 256, 0, stream>>>(key, slot, start, list, n, sorted_index, status);
  return cudaGetLastError();
}

}  // namespace cwa
