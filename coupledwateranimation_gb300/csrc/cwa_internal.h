// cwa_internal.h — device-side scene descriptors, work tiles and the kernel
// launchers shared by the translation units of libcwa.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/cwa.h"

namespace cwa {

// Device status bits (atomicOr'ed by kernels, read by cwa_synchronize).
enum : int32_t {
  kStatusNonFinite = 1,  // a NaN/Inf position reached the cell hash
  kStatusTimeout = 2,    // a bounded spin (scan look-back) gave up
  kStatusBigCell = 4     // a cell above kMaxStableCell members: insert order not stable
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
  float lo[3], hi[3];
  float cell, cellz, inv_cell, inv_cellz;  // x/y and z cell edges
  float hs, hs2;  // search radius: h * (1 + 2^-10), so float rounding never drops a pair
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

// ---- grid / sort kernels (cwa_grid.cu) ----
int scan_tile_items();
size_t scan_workspace_bytes(int32_t n_out);
void scan_bind_workspace(void* ws, int32_t n_out, ScanWorkspace* out);
// Exclusive scan of n_in ints into n_out outputs (n_out >= n_in, tail reads 0).
// zero_input clears `in` as it is read.  Workspace must be zeroed first
// (scan_launch does it with a memset on `stream`).
cudaError_t scan_launch(const int32_t* in, int32_t* out, int32_t n_in, int32_t n_out, bool zero_input,
                        const ScanWorkspace& ws, int32_t* status, cudaStream_t stream, int64_t* launches);

cudaError_t launch_hash_count(const float4* pos, const Tile* tiles, int32_t n_tiles, int32_t tile_size,
                              const SceneDev* scenes, int32_t* key, int32_t* slot, int32_t* count,
                              int32_t* status, cudaStream_t stream);
cudaError_t launch_list_insert(const int32_t* key, const int32_t* slot, const int32_t* start, int32_t* list,
                               int32_t n, cudaStream_t stream);
cudaError_t launch_rank_reorder(const int32_t* key, const int32_t* slot, const int32_t* start,
                                const int32_t* list, const float4* pin, const float4* vin,
                                const float4* fin, const int32_t* idin, float4* pout, float4* vout,
                                float4* fout, int32_t* idout, int32_t n, int32_t* status,
                                cudaStream_t stream);
// Plain point grid for cwa_grid_build (one scene, no reorder).
cudaError_t launch_point_hash(const float4* pos, int32_t n, float lx, float ly, float lz, float cell,
                              int32_t dx, int32_t dy, int32_t dz, int32_t* key, int32_t* slot,
                              int32_t* count, int32_t* status, cudaStream_t stream);
cudaError_t launch_point_rank(const int32_t* key, const int32_t* slot, const int32_t* start,
                              const int32_t* list, int32_t n, int32_t* sorted_index, int32_t* status,
                              cudaStream_t stream);

// ---- SPH kernels (cwa_sph.cu) ----
// Neighbour list: nbr[k * n_total + i] (k < kMaxNbr) holds 16-bit hit codes
// (row << 12 | offset in the row's sorted range; the particle itself is one
// of them) and nbr_cnt[i] their count (kMaxNbr + 1 = overflow, force
// rescans); written by rho_pres, read by force.  stage != 0 lets rho_pres
// stage candidate rows in shared memory.
constexpr int kMaxNbr = 64;
cudaError_t launch_rho_pres(int precision, const float4* pos, const int32_t* start, const Tile* tiles,
                            int32_t n_tiles, int32_t tile_size, const SceneDev* scenes,
                            const float* wave_u, float2* rho_p, uint16_t* nbr, int32_t* nbr_cnt,
                            int32_t n_total, int32_t* status, int32_t stage, cudaStream_t stream);
cudaError_t launch_force(int precision, const float4* pos, const float4* vel, const float2* rho_p,
                         const int32_t* start, const Tile* tiles, int32_t n_tiles, int32_t tile_size,
                         const SceneDev* scenes, const float* wave_u, float4* force, const uint16_t* nbr,
                         const int32_t* nbr_cnt, int32_t n_total, cudaStream_t stream);

// ---- integrate / wave / packing kernels (cwa_step.cu) ----
cudaError_t launch_integrate(float4* pos, float4* vel, float4* force, float2* rho_p, const Tile* tiles,
                             int32_t n_tiles, int32_t tile_size, const SceneDev* scenes,
                             const float* wave_u, unsigned long long* deposits, cudaStream_t stream);
cudaError_t launch_wave(const float* u_n, const float* u_nm1, float* u_out, unsigned long long* deposits,
                        const Tile* wtiles, int32_t n_wtiles, int32_t wtile_size, const SceneDev* scenes,
                        cudaStream_t stream);
cudaError_t launch_wave_init(float* u, int32_t nx, int32_t nz, float mode, cudaStream_t stream);
cudaError_t launch_unpack(const cwa_particle* aos, int32_t n, int32_t poff, float4* pos, float4* vel,
                          float4* force, float2* rho_p, float2* extra, int32_t* id, cudaStream_t stream);
cudaError_t launch_pack(cwa_particle* aos, int32_t n, int32_t poff, const float4* pos, const float4* vel,
                        const float4* force, const float2* rho_p, const float2* extra,
                        const int32_t* id, cudaStream_t stream);
// `out` must hold (kTotalsBlocks + 1) * CWA_TOTALS_COUNT doubles; the totals
// land in the last CWA_TOTALS_COUNT entries.
constexpr int kTotalsBlocks = 304;
cudaError_t launch_totals(const float4* pos, const float4* vel, int32_t poff, int32_t n,
                          const float* u_n, const float* u_nm1, int32_t woff, int32_t nw,
                          const SceneDev* scenes, int32_t scene, double* out, cudaStream_t stream);

// Host-side thread-local error text.
void set_error(const std::string& msg);

}  // namespace cwa
