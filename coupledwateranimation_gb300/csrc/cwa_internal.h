// cwa_internal.h — device-side scene descriptors, work tiles and the kernel
// launchers shared by the translation units of libcwa.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/cwa.h"

namespace cwa {

// Launches `kernel` as a link of the step's chain (programmatic stream
// serialization): it may start while the previous kernel drains, and waits
// for it in chain_enter().  Only kernels that call chain_enter() first are
// launched this way.
template <typename... KArgs, typename... Args>
cudaError_t launch_chained(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                           Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Device status bits (atomicOr'ed by kernels, read by cwa_synchronize).
enum : int32_t {
  kStatusNonFinite = 1,  // a NaN/Inf position reached the cell hash
  kStatusTimeout = 2,    // a bounded spin (scan look-back) gave up
  kStatusBigCell = 4,    // a cell above kMaxStableCell members: insert order not stable
  kStatusBounds = 8      // a debug-build index check failed (the access was skipped)
};

// Members above which a cell's insert order falls back to arrival order.
constexpr int kMaxStableCell = 1024;

// Per-scene constants, precomputed on the host from cwa_scene_desc.
struct SceneDev {
  // particles
  int32_t poff, n;
  // uniform grid (z fastest: id = (x*ny + y)*nz + z)
  int32_t coff, ncells;
  int32_t dims[3];
  // division by dims[2] and dims[1] of a cell id below 2^31: q = (n * m) >> s
  // (round-up reciprocal, exact for every such n; see div_magic)
  uint32_t mz, my;
  int32_t sz, sy;
  float lo[3], hi[3];
  float cell, cellz, inv_cell, inv_cellz;  // x/y and z cell edges
  float hs, hs2;  // h * (1 + 2^-10): float rounding never drops a pair
  float hl, hl2;  // candidate-scan radius: hs, or h (1 + skin)(1 + 2^-10) in Verlet mode
  int32_t rz;     // z cells below a particle's cell that cover its scan window
  float disp2;    // Verlet rebuild threshold (skin h / 2)^2; 0 = per-step mode
  // physics
  int32_t preset;
  float h, h2, mass, visc, rho0, k, dt;
  float g[3];
  float e_wall, damp, radius, crest, foam;
  float c_poly6;  // mass * 315 / (64 pi h^9)
  float k_grad;   // (20 | 45) / (pi h^6)
  float inv_kr;   // 1 / (gas_const * particle_radius)  (reference wave density term)
  double c_poly6_d, k_grad_d;  // the same two constants in double (FP64 mode)
  // wave
  int32_t woff, nx, nz;
  float lam, atten, wa, wb;  // wa = 2 - 4 lam - beta, wb = 1 - beta
  float mode;
  float uvs[2], uvo[2];
  float y0, e_surf, gain;
  int32_t shift;
  float qscale, dq;  // 2^shift, 2^-shift
  int32_t line_source;
  int32_t coupled;   // MULLER: deposits on
};

// Multiplier and shift for dividing numbers below 2^31 by d >= 1 with a
// multiply-high: m = ceil(2^(31 + l) / d), l = ceil(log2 d), then
// n / d = (n * m) >> (31 + l) for every 0 <= n < 2^31 (Granlund and
// Montgomery, "Division by invariant integers using multiplication", 1994,
// with N = 31 so that m fits in 32 bits).
inline void div_magic(int32_t d, uint32_t* m, int32_t* shift) {
  int l = 0;
  while ((1ll << l) < d) ++l;
  const unsigned long long num = 1ull << (31 + l);
  *m = (uint32_t)((num + (unsigned long long)d - 1) / (unsigned long long)d);
  *shift = 31 + l;
}

// A contiguous run of particles (or wave cells) that belongs to one scene.
struct Tile {
  int32_t scene;
  int32_t begin;
  int32_t end;
};

struct ScanWorkspace {
  unsigned int* counter;  // dynamic tile ticket
  unsigned long long* state;  // one (flag<<32 | value) word per tile
  int32_t n_tiles;
};

// Maps a nonzero device status word to its cwa_status (and sets the error
// text); 0 maps to CWA_OK.
cwa_status status_from_bits(int32_t bits);

// ---- grid / sort kernels (cwa_grid.cu) ----
// Items per scan tile: the workspace holds one 8-byte state per tile.
constexpr int kScanTileItems = 8192;
int scan_tile_items();
size_t scan_workspace_bytes(int32_t n_out);
void scan_bind_workspace(void* ws, int32_t n_out, ScanWorkspace* out);
// Exclusive scan of n_in ints into n_out outputs (n_out >= n_in, tail reads 0).
// zero_input clears `in` as it is read.  Workspace must be zeroed first
// (scan_launch does it with a memset on `stream`).
cudaError_t scan_launch(const int32_t* in, int32_t* out, int32_t n_in, int32_t n_out, bool zero_input,
                        const ScanWorkspace& ws, int32_t* status, cudaStream_t stream, int64_t* launches,
                        const int32_t* flag = nullptr);

// The same scan as two chained kernels (tile totals, then every tile's
// scan plus the totals before it); uses the workspace's tile-state area for
// the totals, needs no zeroing and has no wait that can time out.
cudaError_t scan_launch_two_pass(int32_t* in, int32_t* out, int32_t n_in, int32_t n_out, bool zero_input,
                                 const ScanWorkspace& ws, cudaStream_t stream, int64_t* launches,
                                 const int32_t* flag = nullptr);

// The grid-build kernels take the Verlet rebuild flag (null = always run).
cudaError_t launch_hash_count(const float4* pos, const Tile* tiles, int32_t n_tiles, int32_t tile_size,
                              const SceneDev* scenes, int32_t* key, int32_t* slot, int32_t* count,
                              int32_t* status, const int32_t* flag, cudaStream_t stream);
cudaError_t launch_list_insert(const int32_t* key, const int32_t* slot, const int32_t* start, int32_t* list,
                               int32_t n, const int32_t* flag, cudaStream_t stream, int32_t* status = nullptr);
// Moves the particle state into sorted order and writes each particle's cell
// key (kout) in that order.
cudaError_t launch_rank_reorder(const int32_t* key, const int32_t* slot, const int32_t* start,
                                const int32_t* list, const float4* pin, const float4* vin,
                                const float4* fin, const int32_t* idin, float4* pout, float4* vout,
                                float4* fout, int32_t* idout, int32_t* kout, int32_t n, int32_t* status,
                                const int32_t* flag, cudaStream_t stream);
// Verlet mode: copies the reordered state back into the live buffers (when
// the flag is set) and counts rebuilds.
cudaError_t launch_copy_back(const float4* p2, const float4* v2, const float4* f2, const int32_t* id2,
                             float4* p, float4* v, float4* f, int32_t* id, int32_t n, const int32_t* flag,
                             unsigned long long* rebuilds, cudaStream_t stream);
// Plain point grid for cwa_grid_build (one scene, no reorder).
cudaError_t launch_point_hash(const float4* pos, int32_t n, float lx, float ly, float lz, float cell,
                              int32_t dx, int32_t dy, int32_t dz, int32_t* key, int32_t* slot,
                              int32_t* count, int32_t* status, cudaStream_t stream);
cudaError_t launch_point_rank(const int32_t* key, const int32_t* slot, const int32_t* start,
                              const int32_t* list, int32_t n, int32_t* sorted_index, int32_t* status,
                              cudaStream_t stream);

// ---- SPH kernels (cwa_sph.cu) ----
// This step's hits (r < h, the particle itself included), written by the
// density pass and read by force: nine row masks per particle, word
// r * n_total + i holding particle i's hits in candidate row r as bits
// (bit b = the candidate at the row's cell-based start + b).  nbr_cnt holds
// the rows with a nonzero mask (bit r), the only words force reads, or -1
// when some row's window reaches past bit 63 (force then rescans the
// particle's rows).
// The Verlet list (pairs within h (1 + skin) at the last rebuild) holds
// 16-bit codes (row << 12 | offset from the row's cell-based start), entry k
// of particle i at list[k * n_total + i]; a count of kMaxVerlet + 1 marks an
// overflowed list, whose reader rescans the particle's rows.
constexpr int kNbRows = 9;
constexpr int kMaskBits = 64;
typedef uint64_t RowMask;  // one candidate row's hits, bit b = the candidate at the row's cell-based start + b
constexpr int kMaxVerlet = 128;
struct NbArgs {
  const float4* pos;
  const float4* vel;
  float4* force;
  float2* rho_p;
  const int32_t* start;
  const int32_t* keys;  // sorted cell key of each particle (at the last grid build)
  const Tile* tiles;
  int32_t n_tiles, tile_size;
  const SceneDev* scenes;
  const float* wave;
  RowMask* nbm;         // row masks, kNbRows x n_total
  int32_t* nbr_cnt;
  uint16_t* vlist;
  int32_t* vcnt;
  float4* xref;         // positions at the last rebuild (Verlet mode)
  // (x, y, z, p) and (vx, vy, vz, 1/rho) of every particle, written by the
  // density pass for force's neighbour gathers (FP32 modes; null in FP64)
  float4* xpair;
  float4* vpair;
  int32_t n_total;
  int32_t* status;
  const int32_t* flag;  // rebuild flag (Verlet mode), else null
  int32_t stage;        // candidate scan may stage rows in shared memory
  int32_t scan_minb;    // launch-bound variant of the candidate scan (4, 6, 8)
  int32_t force_minb;   // launch-bound variant of force (6, 8, 10)
  // Work-queue form of the per-step density pass and of force (null: one
  // CTA a tile): resident CTAs take numbers t from queue[0] (density) or
  // queue[1] (force), zeroed before each launch, and run tiles[order[t]].
  const int32_t* order;
  int32_t* queue;
};
// Candidate scan: the per-step density + row masks, or (list_mode) the
// Verlet list, run only when *flag is set.
cudaError_t launch_scan_cands(int precision, bool list_mode, const NbArgs& a, cudaStream_t stream);
// Verlet-mode density over the Verlet list; writes the step's row masks.
cudaError_t launch_rho_list(int precision, const NbArgs& a, cudaStream_t stream);
cudaError_t launch_force(int precision, const NbArgs& a, cudaStream_t stream);

// ---- integrate / wave / packing kernels (cwa_step.cu) ----
// xref/flag (Verlet mode): raises *flag when a particle has moved more than
// skin h / 2 from its rebuild position; null otherwise.  key/slot/count
// (per-step mode): the next grid build's cell hash and warp-aggregated
// count on the new positions (the work of the hash-count kernel), so that
// build starts at the scan; null to skip.
cudaError_t launch_integrate(float4* pos, float4* vel, float4* force, float2* rho_p, const Tile* tiles,
                             int32_t n_tiles, int32_t tile_size, const SceneDev* scenes,
                             const float* wave_u, unsigned long long* deposits, const float4* xref,
                             int32_t* flag, int32_t* key, int32_t* slot, int32_t* count, int32_t* status,
                             cudaStream_t stream);
cudaError_t launch_wave(const float* u_n, const float* u_nm1, float* u_out, unsigned long long* deposits,
                        const Tile* wtiles, int32_t n_wtiles, int32_t wtile_size, const SceneDev* scenes,
                        cudaStream_t stream, int32_t* status = nullptr);
cudaError_t launch_wave_init(float* u, int32_t nx, int32_t nz, float mode, cudaStream_t stream);
// u(x, y) = red(2x, y) / 255 of a w x h RGBA8 image (device memory), 0 past it.
cudaError_t launch_wave_from_image(float* u, int32_t nx, int32_t nz, const uint8_t* rgba, int32_t w, int32_t h,
                                   cudaStream_t stream);
// `aos` (16-byte aligned) may be device memory or the device address of
// page-locked host memory.
cudaError_t launch_unpack(const cwa_particle* aos, int32_t n, int32_t poff, float4* pos, float4* vel,
                          float4* force, float2* rho_p, float2* extra, int32_t* id, cudaStream_t stream);
// n floats from src to dst, both 16-byte aligned (cudaErrorInvalidValue
// otherwise); either may be the device address of page-locked host memory.
cudaError_t launch_copy_f32(const float* src, float* dst, long n, cudaStream_t stream);
cudaError_t launch_pack(cwa_particle* aos, int32_t n, int32_t poff, const float4* pos, const float4* vel,
                        const float4* force, const float2* rho_p, const float2* extra,
                        const int32_t* id, cudaStream_t stream);
// `out` must hold (kTotalsBlocks + 1) * CWA_TOTALS_COUNT doubles; the totals
// land in the last CWA_TOTALS_COUNT entries.
constexpr int kTotalsBlocks = 304;
cudaError_t launch_totals(const float4* pos, const float4* vel, int32_t poff, int32_t n,
                          const float* u_n, const float* u_nm1, int32_t woff, int32_t nw,
                          const SceneDev* scenes, int32_t scene, double* out, cudaStream_t stream);

// ---- temporally blocked wave advance (cwa_wave_tma.cu) ----
// Block variants (box 128 x 32 / K 4, 128 x 64 / K 4, 128 x 64 / K 8, each
// with the column walk in shared memory or held in registers, and a 256 x 32
// / K 4 box with column pairs in registers, and a persistent register-column
// form that prefetches each CTA's next 128 x 32 box): K wave steps per
// launch, equal to the halo width.
constexpr int kWaveVariants = 8;
int wave_variant_steps(int variant);

// One block tile: patch (bx, by) of a scene's field; tma = rows load by TMA.
struct WaveBlockTile {
  int32_t scene, bx, by, tma;
};

struct WaveBlockArgs {
  const float* in_cur;           // u^n (all scenes, woff-offset inside)
  const float* in_prev;          // u^(n-1)
  float* out_cur;                // receives u^(n+K)
  float* out_prev;               // receives u^(n+K-1)
  const CUtensorMap* map_cur;    // per-scene tiled maps of in_cur / in_prev,
  const CUtensorMap* map_prev;   // in device memory
  const WaveBlockTile* tiles;
  const SceneDev* scenes;
  int32_t* status;
};

// Encodes the tiled map of one scene's field in one buffer for a variant's
// box; false when the row width is not a multiple of 4 floats (those scenes
// load without TMA).
bool wave_block_encode(CUtensorMap* map, float* base, int W, int H, int variant);
void wave_block_tiles(const SceneDev& d, int32_t scene, bool tma, int variant, std::vector<WaveBlockTile>* out);
cudaError_t launch_wave_block(const WaveBlockArgs& a, int32_t n_tiles, int variant, cudaStream_t stream);

// ---- headless rendering (cwa_render.cu) ----
struct RenderMatrices {  // row-major 4x4
  float mvp_p[16], m_p[16], mvp_w[16], m_w[16], inv_p[16], inv_v[16];
};
struct RenderState;
RenderState* render_state_new();
// True when cwa_debug_fail_alloc's countdown says this device allocation fails.
bool debug_alloc_should_fail();
void render_state_free(RenderState* r);
cudaError_t render_set_skybox(RenderState* r, const uint8_t* faces, int size, cudaStream_t stream);
void render_matrices(const cwa_camera& cam, const cwa_render_params& prm, RenderMatrices* m);
// One frame: particles given in the sim's sorted order with their upload
// indices (drawn in upload order), the scene's u^n, RGBA8 out to host memory.
cudaError_t render_frame(RenderState* r, const cwa_camera& cam, const cwa_render_params& prm,
                         const float4* sorted_pos, const int32_t* sorted_id, int32_t n, const float* wave,
                         int32_t nx, int32_t nz, uint8_t* host_out, int32_t* status, cudaStream_t stream,
                         int64_t* launches);

// Host-side thread-local error text.
void set_error(const std::string& msg);

}  // namespace cwa
