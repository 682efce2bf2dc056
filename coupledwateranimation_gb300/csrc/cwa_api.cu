// cwa_api.cu — the C ABI (include/cwa.h): simulation lifecycle, the pass
// sequence of one step, CUDA-graph replay, host<->device transfer,
// checkpoints and the stand-alone scan / grid operators.
//
// Pass sequence of a step (CoupledWaterAnimation/Main.cpp:549-560 plus the
// grid sort): grid -> rho_pres -> force -> integrate -> wave.  All scenes of
// a sim are concatenated: particles, grid cells and wave cells of scene s
// occupy [poff, poff+n), [coff, coff+ncells), [woff, woff+nx*nz) of shared
// arrays, so each pass is one launch over every scene, fed by a table of
// per-scene tiles.
#include <cuda_runtime.h>
#include <math.h>
#include <nvtx3/nvToolsExt.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <string>
#include <vector>

#include "cwa_internal.h"

namespace cwa {
namespace {
thread_local std::string g_error;
}
void set_error(const std::string& msg) { g_error = msg; }
}  // namespace cwa

using namespace cwa;

struct cwa_sim {
  int device = 0;
  cwa_sim_options opt{};
  cudaStream_t stream = nullptr;
  std::vector<cwa_scene_desc> desc;
  std::vector<SceneDev> sd;
  SceneDev* d_scenes = nullptr;
  int32_t n_total = 0, c_total = 0, w_total = 0, n_max = 0;
  bool move_force = false;
  // particle state, cell-sorted; P/V/ID (and F when the reference torque
  // needs last step's force) ping-pong through the reorder.
  float4* P[2] = {nullptr, nullptr};
  float4* V[2] = {nullptr, nullptr};
  float4* F[2] = {nullptr, nullptr};
  float2* RP = nullptr;  // (rho, pressure)
  float2* EX = nullptr;  // extras.zw, indexed by upload id
  int32_t* ID[2] = {nullptr, nullptr};
  int cur = 0;
  // grid
  int32_t* key = nullptr;
  int32_t* slot = nullptr;
  int32_t* list = nullptr;
  int32_t* count = nullptr;
  int32_t* start = nullptr;
  RowMask* nbm = nullptr;      // this step's hits: kNbRows row masks per particle
  int32_t* nbr_cnt = nullptr;
  int32_t* KS = nullptr;       // sorted cell key of each particle (last grid build)
  // Verlet mode
  bool verlet = false;
  uint16_t* vlist = nullptr;   // kMaxVerlet x n_total codes
  int32_t* vcnt = nullptr;
  float4* XR = nullptr;        // positions at the last rebuild
  // force's gather records (x, y, z, p), (vx, vy, vz, 1/rho); FP32 modes only
  float4* XP = nullptr;
  float4* VP = nullptr;
  int32_t* d_flag = nullptr;   // rebuild flag, raised by integrate / uploads
  unsigned long long* d_rebuilds = nullptr;
  void* scan_ws = nullptr;
  ScanWorkspace scan{};
  // wave: U[wcur] = u^n, U[(wcur+2)%3] = u^(n-1), U[(wcur+1)%3] = next
  float* U[3] = {nullptr, nullptr, nullptr};
  int wcur = 0;
  unsigned long long* D = nullptr;
  // wave advance (cwa_wave_advance): physical buffers UB[0..3], slot -> buffer
  // map uid (slots 0-2 are U[0..2], slot 3 the spare); per variant, tensor
  // maps [variant][buffer][scene] and block tiles wb_off[v] .. wb_off[v+1]
  float* UB[4] = {nullptr, nullptr, nullptr, nullptr};
  int uid[4] = {0, 1, 2, 3};
  CUtensorMap* d_wmaps = nullptr;
  WaveBlockTile* d_wbtiles = nullptr;
  int32_t wb_off[kWaveVariants + 1] = {};
  // work tiles
  Tile* d_ptiles = nullptr;
  int32_t* d_porder = nullptr;  // work-queue order of the particle tiles (capacity porder_cap)
  size_t porder_cap = 0;
  int32_t* d_queue = nullptr;   // work-queue counters: density, force
  int32_t n_ptiles = 0, ptile = 128;
  Tile* d_wtiles = nullptr;
  int32_t n_wtiles = 0, wtile = 1024;
  // staging / status / totals
  cwa_particle* staging = nullptr;
  int32_t* d_status = nullptr;
  int32_t* h_status = nullptr;
  double* d_totals = nullptr;
  double* h_totals = nullptr;
  int64_t steps = 0;
  int64_t launches = 0;
  bool grid_fresh = false;
  // per-step mode: integrate has already hashed and counted the current
  // positions for the next grid build (count holds those counts)
  bool counts_pending = false;
  // an integrate pass has deposited into D since the last wave pass
  bool deposits_pending = false;
  bool profiling = false;
  bool pass_times_valid = false;
  cudaEvent_t ev[CWA_PASS_COUNT + 1] = {};
  cudaGraphExec_t graph[6] = {};
  int64_t graph_launches[6] = {};
  std::vector<void*> dev_allocs;
  RenderState* render = nullptr;  // cube map for cwa_render, created on first use
};

namespace {

#define CWA_CUDA(expr)                                                        \
  do {                                                                        \
    cudaError_t e_ = (expr);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      set_error(std::string(#expr) + ": " + cudaGetErrorString(e_));          \
      cudaGetLastError(); /* a non-sticky error must not fail the next call */ \
      return e_ == cudaErrorMemoryAllocation ? CWA_ERR_OOM : CWA_ERR_CUDA;    \
    }                                                                         \
  } while (0)

#define CWA_TRY(expr)                  \
  do {                                 \
    cwa_status s_ = (expr);            \
    if (s_ != CWA_OK) return s_;       \
  } while (0)

cwa_status arg_error(const std::string& msg) {
  set_error(msg);
  return CWA_ERR_INVALID_ARG;
}

constexpr int kMaxScenes = 1 << 20;
constexpr double kPi = 3.14159265358979323846;
constexpr double kShaderPi = 3.141592741;  // PI #define of the reference shaders

// Fault injection for tests (cwa_debug_fail_alloc): the countdown's n-th
// device allocation from now on fails as if the device were out of memory.
std::atomic<int64_t> g_fail_alloc_in{-1};

bool injected_alloc_failure() {
  int64_t v = g_fail_alloc_in.load();
  while (v >= 0) {
    if (g_fail_alloc_in.compare_exchange_weak(v, v - 1)) return v == 0;
  }
  return false;
}

template <class T>
cwa_status dev_alloc(cwa_sim* s, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  if (injected_alloc_failure()) {
    set_error("cudaMalloc: out of memory (injected by cwa_debug_fail_alloc)");
    return CWA_ERR_OOM;
  }
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    *p = nullptr;
    return CWA_ERR_OOM;
  }
  s->dev_allocs.push_back(*p);
  e = cudaMemset(*p, 0, count * sizeof(T));
  if (e != cudaSuccess) {
    set_error(std::string("cudaMemset: ") + cudaGetErrorString(e));
    return CWA_ERR_CUDA;
  }
  return CWA_OK;
}

cwa_status validate_scene(const cwa_scene_desc& d, int idx) {
  auto bad = [&](const char* what) {
    char buf[160];
    snprintf(buf, sizeof(buf), "scene %d: %s", idx, what);
    return arg_error(buf);
  };
  if (d.preset != CWA_PRESET_REFERENCE_3D && d.preset != CWA_PRESET_MULLER) return bad("unknown preset");
  if (d.n_particles < 0) return bad("n_particles < 0");
  if (d.wave_nx < 1 || d.wave_nz < 1) return bad("wave grid must be at least 1x1");
  if ((int64_t)d.wave_nx * d.wave_nz > (1ll << 28)) return bad("wave grid above 2^28 cells");
  if (!(d.smoothing_length > 0.0f) || !(d.cell_size >= d.smoothing_length))
    return bad("need 0 < smoothing_length <= cell_size");
  if (d.cell_size_z > 0.0f && !(d.cell_size_z * 64.0f >= d.smoothing_length))
    return bad("cell_size_z below smoothing_length / 64");
  if (!(d.mass > 0.0f) || !(d.rest_rho > 0.0f) || !(d.dt > 0.0f)) return bad("mass, rest_rho, dt must be > 0");
  for (int a = 0; a < 3; ++a)
    if (!(d.box_hi[a] > d.box_lo[a])) return bad("box_hi must exceed box_lo");
  if (d.deposit_shift < 0 || d.deposit_shift > 62) return bad("deposit_shift outside [0, 62]");
  if (d.flags != 0) return bad("flags must be 0");
  if (d.preset == CWA_PRESET_REFERENCE_3D && !(d.gas_const * d.particle_radius != 0.0f))
    return bad("reference preset needs gas_const * particle_radius != 0");
  return CWA_OK;
}

SceneDev make_scene_dev(const cwa_scene_desc& d, const int32_t dims[3], int32_t poff, int32_t coff,
                        int32_t woff, float skin) {
  SceneDev s;
  memset(&s, 0, sizeof(s));
  const bool ref = d.preset == CWA_PRESET_REFERENCE_3D;
  s.poff = poff;
  s.n = d.n_particles;
  s.coff = coff;
  s.ncells = dims[0] * dims[1] * dims[2];
  for (int a = 0; a < 3; ++a) {
    s.dims[a] = dims[a];
    s.lo[a] = d.box_lo[a];
    s.hi[a] = d.box_hi[a];
    s.g[a] = d.gravity[a];
  }
  div_magic(dims[2], &s.mz, &s.sz);
  div_magic(dims[1], &s.my, &s.sy);
  s.cell = d.cell_size;
  s.cellz = d.cell_size_z > 0.0f ? d.cell_size_z : d.cell_size;
  s.inv_cell = 1.0f / s.cell;
  s.inv_cellz = 1.0f / s.cellz;
  s.hs = (float)((double)d.smoothing_length * (1.0 + 1.0 / 1024.0));
  s.hs2 = s.hs * s.hs;
  s.hl = skin > 0.0f ? (float)((double)d.smoothing_length * (1.0 + skin) * (1.0 + 1.0 / 1024.0)) : s.hs;
  s.hl2 = s.hl * s.hl;
  s.rz = (int32_t)ceilf(s.hl * s.inv_cellz) + 1;
  // The rebuild threshold uses the skin the x/y cells really hold, so every
  // pair that can come within h before the next rebuild is in the list.
  const double skin_eff = std::min((double)skin, (double)d.cell_size / (double)d.smoothing_length - 1.0);
  s.disp2 = skin > 0.0f ? (float)(0.25 * skin_eff * skin_eff * (double)d.smoothing_length * d.smoothing_length)
                        : 0.0f;
  s.preset = d.preset;
  s.h = d.smoothing_length;
  s.h2 = d.smoothing_length * d.smoothing_length;
  s.mass = d.mass;
  s.visc = d.visc;
  s.rho0 = d.rest_rho;
  s.k = d.gas_const;
  s.dt = d.dt;
  s.e_wall = d.wall_restitution;
  s.damp = 1.0f - d.velocity_damping * d.dt;
  s.radius = d.particle_radius;
  s.crest = d.crest_height;
  s.foam = d.foam_speed;
  const double pi = ref ? kShaderPi : kPi;
  const double h = d.smoothing_length;
  s.c_poly6_d = (double)d.mass * 315.0 / (64.0 * pi * pow(h, 9));
  s.k_grad_d = (ref ? 20.0 : 45.0) / (pi * pow(h, 6));
  s.c_poly6 = (float)s.c_poly6_d;
  s.k_grad = (float)s.k_grad_d;
  s.inv_kr = ref ? (float)(1.0 / ((double)d.gas_const * d.particle_radius)) : 0.0f;
  s.woff = woff;
  s.nx = d.wave_nx;
  s.nz = d.wave_nz;
  s.lam = d.wave_lambda;
  s.atten = d.wave_atten;
  s.wa = (float)(2.0 - 4.0 * (double)d.wave_lambda - (double)d.wave_beta);
  s.wb = (float)(1.0 - (double)d.wave_beta);
  s.mode = d.wave_mode;
  s.uvs[0] = d.wave_uv_scale[0];
  s.uvs[1] = d.wave_uv_scale[1];
  s.uvo[0] = d.wave_uv_offset[0];
  s.uvo[1] = d.wave_uv_offset[1];
  s.y0 = d.surface_y0;
  s.e_surf = d.surface_restitution;
  s.gain = d.couple_gain;
  s.shift = d.deposit_shift;
  s.qscale = ldexpf(1.0f, d.deposit_shift);
  s.dq = ldexpf(1.0f, -d.deposit_shift);
  s.line_source = (d.wave_mode > 0.0f && d.wave_mode < 1.0f) ? 1 : 0;
  s.coupled = d.preset == CWA_PRESET_MULLER ? 1 : 0;
  return s;
}

cwa_status check_sim(cwa_sim* s) {
  if (!s) return arg_error("null sim");
  CWA_CUDA(cudaSetDevice(s->device));
  return CWA_OK;
}

cwa_status check_scene(cwa_sim* s, int32_t scene) {
  CWA_TRY(check_sim(s));
  if (scene < 0 || scene >= (int32_t)s->desc.size()) return arg_error("scene index out of range");
  return CWA_OK;
}

float4* cur_force(cwa_sim* s) { return s->move_force ? s->F[s->cur] : s->F[0]; }

// Device address of a page-locked host buffer of `bytes` bytes (cudaHostAlloc,
// or cudaHostRegister'd), or nullptr for pageable memory, a buffer that is not
// 16-byte aligned, or one whose last byte is not page-locked at the matching
// device address (a buffer that runs past its registration).  Kernels read and
// write such buffers directly over the host link (NVLink-C2C on Grace), which
// moves contiguous data faster than a copy-engine transfer does.
void* host_alias(const void* host, size_t bytes) {
  if (!host || bytes == 0 || (reinterpret_cast<uintptr_t>(host) & 15u)) return nullptr;
  auto mapped = [](const void* p, void** dev) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
      cudaGetLastError();  // not a pointer CUDA knows: plain pageable memory
      return false;
    }
    *dev = a.devicePointer;
    return a.type == cudaMemoryTypeHost && a.devicePointer != nullptr;
  };
  void* first = nullptr;
  void* last = nullptr;
  if (!mapped(host, &first) || (reinterpret_cast<uintptr_t>(first) & 15u)) return nullptr;
  if (!mapped(static_cast<const char*>(host) + bytes - 1, &last) ||
      static_cast<char*>(last) != static_cast<char*>(first) + bytes - 1)
    return nullptr;
  return first;
}

// One height field between the host and the device, on the sim's stream:
// a kernel copy when the host side is page-locked and both sides are 16-byte
// aligned, else cudaMemcpyAsync.
cwa_status copy_field(cwa_sim* s, const float* src, float* dst, long cells, cudaMemcpyKind kind) {
  const bool to_dev = kind == cudaMemcpyHostToDevice;
  void* alias = host_alias(to_dev ? static_cast<const void*>(src) : static_cast<const void*>(dst),
                           (size_t)cells * sizeof(float));
  const float* dev_side = to_dev ? dst : src;
  if (alias && !(reinterpret_cast<uintptr_t>(dev_side) & 15u)) {
    CWA_CUDA(launch_copy_f32(to_dev ? static_cast<const float*>(alias) : src,
                             to_dev ? dst : static_cast<float*>(alias), cells, s->stream));
    s->launches += 1;
    return CWA_OK;
  }
  CWA_CUDA(cudaMemcpyAsync(dst, src, (size_t)cells * sizeof(float), kind, s->stream));
  return CWA_OK;
}

// Particle work tiles of `size` particles, never straddling two scenes.
std::vector<Tile> particle_tiles(const cwa_sim* s, int32_t size) {
  std::vector<Tile> t;
  for (size_t i = 0; i < s->sd.size(); ++i) {
    const SceneDev& d = s->sd[i];
    for (int32_t b = 0; b < d.n; b += size)
      t.push_back(Tile{(int32_t)i, d.poff + b, d.poff + std::min(b + size, d.n)});
  }
  return t;
}

// Work-queue order of the tiles: the scenes from the most particles to the
// fewest (the longest work first, so the short scenes fill the tail), each
// scene's tiles in sorted order.
std::vector<int32_t> tile_order(const cwa_sim* s, const std::vector<Tile>& t) {
  std::vector<int32_t> scene_rank(s->sd.size());
  for (size_t i = 0; i < scene_rank.size(); ++i) scene_rank[i] = (int32_t)i;
  std::stable_sort(scene_rank.begin(), scene_rank.end(),
                   [&](int32_t a, int32_t b) { return s->sd[a].n > s->sd[b].n; });
  std::vector<int32_t> pos_of(s->sd.size());
  for (size_t k = 0; k < scene_rank.size(); ++k) pos_of[scene_rank[k]] = (int32_t)k;
  std::vector<int32_t> o(t.size());
  for (size_t k = 0; k < o.size(); ++k) o[k] = (int32_t)k;
  std::stable_sort(o.begin(), o.end(), [&](int32_t a, int32_t b) { return pos_of[t[a].scene] < pos_of[t[b].scene]; });
  return o;
}

cwa_status upload_tile_order(cwa_sim* s, const std::vector<Tile>& t) {
  const std::vector<int32_t> o = tile_order(s, t);
  if (o.size() > s->porder_cap) return arg_error("tile order above its capacity");
  if (!o.empty()) CWA_CUDA(cudaMemcpy(s->d_porder, o.data(), o.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
  return CWA_OK;
}

cwa_status set_particle_tiles(cwa_sim* s, int32_t size) {
  std::vector<Tile> t = particle_tiles(s, size);
  CWA_TRY(upload_tile_order(s, t));
  Tile* d = nullptr;
  CWA_CUDA(cudaMalloc((void**)&d, std::max<size_t>(t.size(), 1) * sizeof(Tile)));
  if (!t.empty()) {
    cudaError_t e = cudaMemcpy(d, t.data(), t.size() * sizeof(Tile), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(d);
      CWA_CUDA(e);
    }
  }
  for (auto& p : s->dev_allocs)
    if (p == s->d_ptiles) {
      cudaFree(p);
      p = d;
    }
  s->d_ptiles = d;
  s->n_ptiles = (int32_t)t.size();
  s->ptile = size;
  return CWA_OK;
}

void drop_graphs(cwa_sim* s) {
  for (auto& g : s->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

// ---- passes (enqueue only) ----
NbArgs nb_args(cwa_sim* s) {
  NbArgs a;
  a.pos = s->P[s->cur];
  a.vel = s->V[s->cur];
  a.force = cur_force(s);
  a.rho_p = s->RP;
  a.start = s->start;
  a.keys = s->KS;
  a.tiles = s->d_ptiles;
  a.n_tiles = s->n_ptiles;
  a.tile_size = s->ptile;
  a.scenes = s->d_scenes;
  a.wave = s->U[s->wcur];
  a.nbm = s->nbm;
  a.nbr_cnt = s->nbr_cnt;
  a.vlist = s->vlist;
  a.vcnt = s->vcnt;
  a.xref = s->XR;
  a.xpair = s->XP;
  a.vpair = s->VP;
  a.n_total = s->n_total;
  a.status = s->d_status;
  a.flag = s->verlet ? s->d_flag : nullptr;
  a.stage = s->opt.nb_stage >= 0 ? 1 : 0;
  a.scan_minb = s->opt.nb_scan_minb ? s->opt.nb_scan_minb : 4;
  a.force_minb = s->opt.nb_force_minb ? s->opt.nb_force_minb : 9;
  a.order = s->d_porder;
  a.queue = s->opt.nb_queue ? s->d_queue : nullptr;
  return a;
}

// Counts of an earlier fused hash are stale once the particles change
// outside a step (uploads, checkpoint loads, the autotuner's restores).
cwa_status drop_pending_counts(cwa_sim* s) {
  if (s->counts_pending) {
    CWA_CUDA(cudaMemsetAsync(s->count, 0, (size_t)s->c_total * sizeof(int32_t), s->stream));
    s->counts_pending = false;
  }
  return CWA_OK;
}

cwa_status run_hash(cwa_sim* s) {
  CWA_CUDA(launch_hash_count(s->P[s->cur], s->d_ptiles, s->n_ptiles, s->ptile, s->d_scenes, s->key, s->slot,
                             s->count, s->d_status, s->verlet ? s->d_flag : nullptr, s->stream));
  s->launches += s->n_ptiles > 0;
  return CWA_OK;
}

// Grid pass: hash + count (unless integrate has already done it), scan,
// stable insert, reorder.  Per-step mode
// flips the live buffers every step.  Verlet mode runs the same kernels
// only when the device rebuild flag is up (each kernel checks it), copies
// the reordered state back into the live buffers and rebuilds the Verlet
// list, so the host-side buffer roles never change.
cwa_status run_grid(cwa_sim* s) {
  cudaStream_t st = s->stream;
  const int cur = s->cur, nxt = cur ^ 1;
  const int32_t* flag = s->verlet ? s->d_flag : nullptr;
  if (!s->counts_pending) CWA_TRY(run_hash(s));
  s->counts_pending = false;  // the scan consumes (and clears) the counts
  CWA_CUDA(scan_launch_two_pass(s->count, s->start, s->c_total, s->c_total + 1, true, s->scan, st, &s->launches,
                                flag));
  CWA_CUDA(launch_list_insert(s->key, s->slot, s->start, s->list, s->n_total, flag, st, s->d_status));
  CWA_CUDA(launch_rank_reorder(s->key, s->slot, s->start, s->list, s->P[cur], s->V[cur],
                               s->move_force ? s->F[cur] : nullptr, s->ID[cur], s->P[nxt], s->V[nxt],
                               s->move_force ? s->F[nxt] : nullptr, s->ID[nxt], s->KS, s->n_total, s->d_status,
                               flag, st));
  s->launches += s->n_total > 0 ? 2 : 0;
  if (s->verlet) {
    CWA_CUDA(launch_copy_back(s->P[nxt], s->V[nxt], s->move_force ? s->F[nxt] : nullptr, s->ID[nxt], s->P[cur],
                              s->V[cur], s->move_force ? s->F[cur] : nullptr, s->ID[cur], s->n_total, s->d_flag,
                              s->d_rebuilds, st));
    CWA_CUDA(launch_scan_cands(s->opt.precision, true, nb_args(s), st));
    s->launches += s->n_total > 0 ? 2 : 0;
  } else {
    s->cur = nxt;
  }
  s->grid_fresh = true;
  return CWA_OK;
}

cwa_status run_rho_pres(cwa_sim* s) {
  if (s->verlet)
    CWA_CUDA(launch_rho_list(s->opt.precision, nb_args(s), s->stream));
  else
    CWA_CUDA(launch_scan_cands(s->opt.precision, false, nb_args(s), s->stream));
  s->launches += s->n_ptiles > 0;
  return CWA_OK;
}

cwa_status run_force(cwa_sim* s) {
  CWA_CUDA(launch_force(s->opt.precision, nb_args(s), s->stream));
  s->launches += s->n_ptiles > 0;
  return CWA_OK;
}

cwa_status run_integrate(cwa_sim* s) {
  if (s->verlet) CWA_CUDA(cudaMemsetAsync(s->d_flag, 0, sizeof(int32_t), s->stream));
  // Per-step mode hashes and counts the new positions here for the next
  // grid build.  (Verlet mode rebuilds rarely and keeps the separate pass.)
  const bool fuse = !s->verlet;
  if (fuse) CWA_TRY(drop_pending_counts(s));  // integrate twice without a grid in between
  CWA_CUDA(launch_integrate(s->P[s->cur], s->V[s->cur], cur_force(s), s->RP, s->d_ptiles, s->n_ptiles,
                            s->ptile, s->d_scenes, s->U[s->wcur], s->D, s->verlet ? s->XR : nullptr,
                            s->verlet ? s->d_flag : nullptr, fuse ? s->key : nullptr, fuse ? s->slot : nullptr,
                            fuse ? s->count : nullptr, s->d_status, s->stream));
  s->launches += s->n_ptiles > 0;
  s->counts_pending = fuse && s->n_ptiles > 0;
  s->deposits_pending = true;
  if (!s->verlet) s->grid_fresh = false;  // a Verlet list stays usable
  return CWA_OK;
}


cwa_status run_wave(cwa_sim* s) {
  const int w = s->wcur;
  CWA_CUDA(launch_wave(s->U[w], s->U[(w + 2) % 3], s->U[(w + 1) % 3], s->D, s->d_wtiles, s->n_wtiles, s->wtile,
                       s->d_scenes, s->stream, s->d_status));
  s->launches += 1;
  s->wcur = (w + 1) % 3;  // StencilImage2DTripleBuffered::PingPong (:33-40)
  s->steps += 1;
  s->deposits_pending = false;  // read and cleared
  return CWA_OK;
}

// Lazily set up the blocked wave advance: the spare buffer and, for every
// variant, a tensor map of every scene's field in each of the four buffers
// and the block tiles.
cwa_status prepare_wave_blocks(cwa_sim* s) {
  if (s->d_wbtiles) return CWA_OK;
  const int nsc = (int)s->sd.size();
  float* spare = nullptr;
  CWA_TRY(dev_alloc(s, &spare, (size_t)s->w_total));
  for (int b = 0; b < 3; ++b) s->UB[b] = s->U[b];
  s->UB[3] = spare;
  for (int b = 0; b < 4; ++b) s->uid[b] = b;
  std::vector<CUtensorMap> maps((size_t)kWaveVariants * 4 * nsc);
  memset(maps.data(), 0, maps.size() * sizeof(CUtensorMap));
  std::vector<WaveBlockTile> tiles;
  for (int v = 0; v < kWaveVariants; ++v) {
    s->wb_off[v] = (int32_t)tiles.size();
    for (int k = 0; k < nsc; ++k) {
      const SceneDev& d = s->sd[k];
      bool tma = true;
      for (int b = 0; b < 4 && tma; ++b)
        tma = wave_block_encode(&maps[((size_t)v * 4 + b) * nsc + k], s->UB[b] + d.woff, d.nx, d.nz, v);
      wave_block_tiles(d, k, tma, v, &tiles);
    }
  }
  s->wb_off[kWaveVariants] = (int32_t)tiles.size();
  CUtensorMap* dm = nullptr;
  WaveBlockTile* dt = nullptr;
  CWA_TRY(dev_alloc(s, &dm, maps.size()));
  CWA_TRY(dev_alloc(s, &dt, tiles.size()));
  CWA_CUDA(cudaMemcpy(dm, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice));
  CWA_CUDA(cudaMemcpy(dt, tiles.data(), tiles.size() * sizeof(WaveBlockTile), cudaMemcpyHostToDevice));
  CWA_CUDA(cudaDeviceSynchronize());  // the zero-fill memsets ran on the legacy stream
  s->d_wmaps = dm;
  s->d_wbtiles = dt;
  return CWA_OK;
}

// n wave passes: a single pass first when deposits are pending (it applies
// and clears them), K-step blocks of the sim's wave_block variant, single
// passes for the remainder.  A block writes u^(n+K) into the free slot and
// u^(n+K-1) into the spare; the slots are then renamed so U[wcur] /
// U[(wcur+2)%3] hold them, which is the state K single passes leave (up to
// the rotation of wcur).
cwa_status run_wave_advance(cwa_sim* s, int32_t n) {
  int32_t done = 0;
  bool coupled = false;
  for (const SceneDev& d : s->sd) coupled = coupled || d.coupled;
  if (coupled && s->deposits_pending && n > 0) {
    CWA_TRY(run_wave(s));
    done = 1;
  }
  const int v = s->opt.wave_block, K = wave_variant_steps(v);
  if (n - done >= K) {
    CWA_TRY(prepare_wave_blocks(s));
    const int w = s->wcur, cur = w, prev = (w + 2) % 3, nxt = (w + 1) % 3;
    const int32_t n_tiles = s->wb_off[v + 1] - s->wb_off[v];
    while (n - done >= K) {
      const int ic = s->uid[cur], ip = s->uid[prev], oc = s->uid[nxt], op = s->uid[3];
      const size_t nsc = s->sd.size();
      WaveBlockArgs a;
      a.in_cur = s->UB[ic];
      a.in_prev = s->UB[ip];
      a.out_cur = s->UB[oc];
      a.out_prev = s->UB[op];
      a.map_cur = s->d_wmaps + ((size_t)v * 4 + ic) * nsc;
      a.map_prev = s->d_wmaps + ((size_t)v * 4 + ip) * nsc;
      a.tiles = s->d_wbtiles + s->wb_off[v];
      a.scenes = s->d_scenes;
      a.status = s->d_status;
      CWA_CUDA(launch_wave_block(a, n_tiles, v, s->stream));
      s->launches += n_tiles > 0;
      s->uid[cur] = oc;
      s->uid[prev] = op;
      s->uid[nxt] = ic;
      s->uid[3] = ip;
      done += K;
      s->steps += K;
    }
    for (int b = 0; b < 3; ++b) s->U[b] = s->UB[s->uid[b]];
    drop_graphs(s);  // captured steps hold the old buffer pointers
  }
  for (; done < n; ++done) CWA_TRY(run_wave(s));
  return CWA_OK;
}

cwa_status record(cwa_sim* s, int idx) {
  if (s->profiling) CWA_CUDA(cudaEventRecord(s->ev[idx], s->stream));
  return CWA_OK;
}

// One NVTX range per pass on the host thread that enqueues it (eager steps;
// a graph replay shows as the enclosing cwa_step range).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

template <class F>
cwa_status traced(const char* name, F&& f) {
  NvtxRange r(name);
  return f();
}

cwa_status enqueue_step(cwa_sim* s) {
  CWA_TRY(record(s, 0));
  CWA_TRY(traced("cwa grid", [&] { return run_grid(s); }));
  CWA_TRY(record(s, 1));
  CWA_TRY(traced("cwa rho_pres", [&] { return run_rho_pres(s); }));
  CWA_TRY(record(s, 2));
  CWA_TRY(traced("cwa force", [&] { return run_force(s); }));
  CWA_TRY(record(s, 3));
  CWA_TRY(traced("cwa integrate", [&] { return run_integrate(s); }));
  CWA_TRY(record(s, 4));
  CWA_TRY(traced("cwa wave", [&] { return run_wave(s); }));
  CWA_TRY(record(s, 5));
  if (s->profiling) s->pass_times_valid = true;
  return CWA_OK;
}

// Capture one step for the current (cur, wcur) phase; the host-side state
// the capture advanced is rolled back, the graph launch advances it again.
cwa_status graph_step(cwa_sim* s) {
  // Graphs start at the scan: in per-step mode the counts come from the
  // previous step's integrate, or from this eager hash after an upload.
  if (!s->verlet && !s->counts_pending && s->n_ptiles > 0) {
    CWA_TRY(run_hash(s));
    s->counts_pending = true;
  }
  const int phase = s->cur * 3 + s->wcur;
  const int cur0 = s->cur, w0 = s->wcur;
  const int64_t steps0 = s->steps, launches0 = s->launches;
  if (!s->graph[phase]) {
    cudaGraph_t g = nullptr;
    CWA_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    cwa_status st = enqueue_step(s);
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    s->graph_launches[phase] = s->launches - launches0;
    s->cur = cur0;
    s->wcur = w0;
    s->steps = steps0;
    s->launches = launches0;
    if (st != CWA_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    CWA_CUDA(e);
    e = cudaGraphInstantiate(&s->graph[phase], g, 0);
    cudaGraphDestroy(g);
    CWA_CUDA(e);
  }
  // The launch-count and state bookkeeping of one step, as enqueue_step does.
  CWA_CUDA(cudaGraphLaunch(s->graph[phase], s->stream));
  s->launches += s->graph_launches[phase];
  if (!s->verlet) {
    s->cur ^= 1;
    s->grid_fresh = false;
  } else {
    s->grid_fresh = true;
  }
  s->wcur = (s->wcur + 1) % 3;
  s->steps += 1;
  s->counts_pending = !s->verlet && s->n_ptiles > 0;
  s->deposits_pending = false;  // the step ends with its wave pass
  return CWA_OK;
}

cwa_status read_status(cwa_sim* s) {
  CWA_CUDA(cudaMemcpyAsync(s->h_status, s->d_status, sizeof(int32_t), cudaMemcpyDeviceToHost, s->stream));
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  const int32_t v = *s->h_status;
  if (v == 0) return CWA_OK;
  CWA_CUDA(cudaMemsetAsync(s->d_status, 0, sizeof(int32_t), s->stream));
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  return status_from_bits(v);
}

// Waits for `stream`, then maps the status word at d_word (device memory)
// to a cwa_status.
cwa_status read_status_word(const int32_t* d_word, void* stream) {
  int32_t v = 0;
  CWA_CUDA(cudaMemcpyAsync(&v, d_word, sizeof(int32_t), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  CWA_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  return status_from_bits(v);
}

void free_sim(cwa_sim* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (auto& g : s->graph)
    if (g) cudaGraphExecDestroy(g);
  for (auto& e : s->ev)
    if (e) cudaEventDestroy(e);
  for (void* p : s->dev_allocs) cudaFree(p);
  render_state_free(s->render);
  if (s->h_status) cudaFreeHost(s->h_status);
  if (s->h_totals) cudaFreeHost(s->h_totals);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

}  // namespace

namespace cwa {
bool debug_alloc_should_fail() { return injected_alloc_failure(); }

cwa_status status_from_bits(int32_t v) {
  if (v == 0) return CWA_OK;
  if (v & kStatusBounds) {
    set_error("an index check of the debug build failed; the access was skipped");
    return CWA_ERR_BOUNDS;
  }
  if (v & kStatusTimeout) {
    set_error("a bounded device wait (scan look-back) timed out");
    return CWA_ERR_TIMEOUT;
  }
  if (v & kStatusNonFinite) {
    set_error("non-finite particle position");
    return CWA_ERR_NONFINITE;
  }
  set_error("a grid cell held more than 1024 particles; its insert order fell back to arrival order");
  return CWA_ERR_CAPACITY;
}
}  // namespace cwa

extern "C" {

const char* cwa_status_str(cwa_status s) {
  switch (s) {
    case CWA_OK: return "ok";
    case CWA_ERR_INVALID_ARG: return "invalid argument";
    case CWA_ERR_OOM: return "out of memory";
    case CWA_ERR_CUDA: return "CUDA error";
    case CWA_ERR_TIMEOUT: return "device wait timed out";
    case CWA_ERR_NONFINITE: return "non-finite value";
    case CWA_ERR_IO: return "I/O error";
    case CWA_ERR_NO_DEVICE: return "no CUDA device";
    case CWA_ERR_CAPACITY: return "capacity exceeded";
    case CWA_ERR_BOUNDS: return "debug index check failed";
  }
  return "unknown status";
}

int32_t cwa_abi_version(void) { return CWA_ABI_VERSION; }

const char* cwa_last_error(void) { return g_error.c_str(); }

cwa_status cwa_create(const cwa_sim_options* opt, const cwa_scene_desc* scenes, int32_t n_scenes,
                      cwa_sim** out) {
  if (!out) return arg_error("null output pointer");
  *out = nullptr;
  if (!scenes || n_scenes < 1 || n_scenes > kMaxScenes) return arg_error("need 1 <= n_scenes <= 2^20");
  cwa_sim_options o{};
  o.precision = CWA_PREC_COMPENSATED;
  o.use_graph = 1;
  if (opt) o = *opt;
  if (o.precision < CWA_PREC_FP32 || o.precision > CWA_PREC_FP64) return arg_error("unknown precision");
  if (o.nb_stage < -1 || o.nb_stage > 1) return arg_error("nb_stage must be -1, 0 or 1");
  if (!(o.verlet_skin >= 0.0f && o.verlet_skin <= 1.0f)) return arg_error("verlet_skin must be in [0, 1]");
  if (o.nb_scan_minb < 0 || o.nb_scan_minb > 8) return arg_error("nb_scan_minb must be 0..8");
  if (o.nb_force_minb < 0 || o.nb_force_minb > 9) return arg_error("nb_force_minb must be 0..9");
  if (o.nb_threads != 0 && (o.nb_threads < 32 || o.nb_threads > 128 || (o.nb_threads & 31)))
    return arg_error("nb_threads must be 0 or a multiple of 32 in [32, 128]");
  if (o.wave_block < 0 || o.wave_block >= CWA_WAVE_BLOCK_COUNT) return arg_error("unknown wave_block variant");
  if (o.nb_queue != 0 && o.nb_queue != 1) return arg_error("nb_queue must be 0 or 1");
  std::vector<int32_t> dims(3 * (size_t)n_scenes);
  int64_t np = 0, nc = 0, nw = 0;
  int32_t nmax = 0;
  for (int i = 0; i < n_scenes; ++i) {
    CWA_TRY(validate_scene(scenes[i], i));
    if (o.verlet_skin > 0.0f && !((double)scenes[i].cell_size >=
                                  (double)scenes[i].smoothing_length * (1.0 + o.verlet_skin) * (1.0 - 1e-5))) {
      char buf[160];
      snprintf(buf, sizeof(buf), "scene %d: Verlet mode needs cell_size >= h (1 + verlet_skin)", i);
      return arg_error(buf);
    }
    cwa_status st = cwa_grid_dims(&scenes[i], &dims[3 * (size_t)i]);
    if (st != CWA_OK) return st == CWA_ERR_CAPACITY ? st : arg_error("bad grid dimensions");
    np += scenes[i].n_particles;
    nc += (int64_t)dims[3 * i] * dims[3 * i + 1] * dims[3 * i + 2];
    nw += ((int64_t)scenes[i].wave_nx * scenes[i].wave_nz + 31) / 32 * 32;  // 128-byte aligned regions
    if (scenes[i].n_particles > nmax) nmax = scenes[i].n_particles;
  }
  const int64_t lim = (1ll << 31) - (1ll << 20);
  if (np > lim || nc > lim || nw > lim) {
    set_error("total particles, grid cells or wave cells above 2^31 - 2^20");
    return CWA_ERR_CAPACITY;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    set_error("no CUDA device");
    return CWA_ERR_NO_DEVICE;
  }
  if (o.device < 0 || o.device >= ndev) return arg_error("device ordinal out of range");

  cwa_sim* s = new cwa_sim();
  s->device = o.device;
  s->opt = o;
  s->desc.assign(scenes, scenes + n_scenes);
  s->n_total = (int32_t)np;
  s->c_total = (int32_t)nc;
  s->w_total = (int32_t)nw;
  s->n_max = nmax;
  s->ptile = o.nb_threads ? o.nb_threads : 128;
  s->verlet = o.verlet_skin > 0.0f;
  auto fail = [&](cwa_status st) {
    free_sim(s);
    return st;
  };
  if (cudaSetDevice(s->device) != cudaSuccess) return fail(CWA_ERR_CUDA);

  std::vector<Tile> ptiles, wtiles;
  int32_t poff = 0, coff = 0, woff = 0;
  for (int i = 0; i < n_scenes; ++i) {
    const cwa_scene_desc& d = scenes[i];
    s->sd.push_back(make_scene_dev(d, &dims[3 * (size_t)i], poff, coff, woff, o.verlet_skin));
    if (d.preset == CWA_PRESET_REFERENCE_3D) s->move_force = true;
    for (int32_t b = 0; b < d.n_particles; b += s->ptile)
      ptiles.push_back(Tile{i, poff + b, poff + std::min(b + s->ptile, d.n_particles)});
    const int32_t cells = d.wave_nx * d.wave_nz;
    for (int32_t b = 0; b < cells; b += s->wtile)
      wtiles.push_back(Tile{i, woff + b, woff + std::min(b + s->wtile, cells)});
    poff += d.n_particles;
    coff += s->sd.back().ncells;
    woff += (cells + 31) / 32 * 32;
  }
  s->n_ptiles = (int32_t)ptiles.size();
  s->n_wtiles = (int32_t)wtiles.size();

  cwa_status st = CWA_OK;
  const size_t N = (size_t)s->n_total;
#define ALLOC(ptr, cnt)                               \
  do {                                                \
    st = dev_alloc(s, &(ptr), (cnt));                 \
    if (st != CWA_OK) return fail(st);                \
  } while (0)
  for (int b = 0; b < 2; ++b) {
    ALLOC(s->P[b], N);
    ALLOC(s->V[b], N);
    ALLOC(s->ID[b], N);
  }
  ALLOC(s->F[0], N);
  if (s->move_force) ALLOC(s->F[1], N);
  ALLOC(s->RP, N);
  ALLOC(s->EX, N);
  ALLOC(s->key, N);
  ALLOC(s->slot, N);
  ALLOC(s->list, N);
  ALLOC(s->nbm, N * kNbRows);
  ALLOC(s->nbr_cnt, N);
  ALLOC(s->KS, N);
  if (s->opt.precision != CWA_PREC_FP64) {
    ALLOC(s->XP, N);
    ALLOC(s->VP, N);
  }
  ALLOC(s->d_flag, 1);
  ALLOC(s->d_rebuilds, 1);
  if (s->verlet) {
    ALLOC(s->vlist, N * kMaxVerlet);
    ALLOC(s->vcnt, N);
    ALLOC(s->XR, N);
  }
  ALLOC(s->count, (size_t)s->c_total);
  ALLOC(s->start, (size_t)s->c_total + 1);
  {
    char* ws = nullptr;
    ALLOC(ws, scan_workspace_bytes(s->c_total + 1));
    s->scan_ws = ws;
    scan_bind_workspace(ws, s->c_total + 1, &s->scan);
  }
  for (int b = 0; b < 3; ++b) ALLOC(s->U[b], (size_t)s->w_total);
  ALLOC(s->D, (size_t)s->w_total);
  ALLOC(s->d_scenes, s->sd.size());
  ALLOC(s->d_ptiles, ptiles.size());
  // tiles of 32 or more particles: at most N / 32 + one partial tile a scene
  s->porder_cap = N / 32 + s->sd.size() + 1;
  ALLOC(s->d_porder, s->porder_cap);
  ALLOC(s->d_queue, 2);
  ALLOC(s->d_wtiles, wtiles.size());
  ALLOC(s->staging, (size_t)s->n_max);
  ALLOC(s->d_status, 1);
  ALLOC(s->d_totals, (size_t)(kTotalsBlocks + 1) * CWA_TOTALS_COUNT);
#undef ALLOC
  if (cudaMallocHost((void**)&s->h_status, sizeof(int32_t)) != cudaSuccess ||
      cudaMallocHost((void**)&s->h_totals, CWA_TOTALS_COUNT * sizeof(double)) != cudaSuccess) {
    set_error("cudaMallocHost failed");
    return fail(CWA_ERR_OOM);
  }
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(CWA_ERR_CUDA);
  for (auto& e : s->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return fail(CWA_ERR_CUDA);
  if (s->verlet) {  // the first step builds the grid and the Verlet list
    const int32_t one = 1;
    if (cudaMemcpy(s->d_flag, &one, sizeof(one), cudaMemcpyHostToDevice) != cudaSuccess) return fail(CWA_ERR_CUDA);
  }
  std::vector<int32_t> ids(N);
  for (size_t i = 0; i < s->sd.size(); ++i)
    for (int32_t k = 0; k < s->sd[i].n; ++k) ids[(size_t)s->sd[i].poff + k] = k;
  bool ok = cudaMemcpy(s->d_scenes, s->sd.data(), s->sd.size() * sizeof(SceneDev), cudaMemcpyHostToDevice) ==
                cudaSuccess &&
            (ptiles.empty() || cudaMemcpy(s->d_ptiles, ptiles.data(), ptiles.size() * sizeof(Tile),
                                          cudaMemcpyHostToDevice) == cudaSuccess) &&
            upload_tile_order(s, ptiles) == CWA_OK &&
            cudaMemcpy(s->d_wtiles, wtiles.data(), wtiles.size() * sizeof(Tile), cudaMemcpyHostToDevice) ==
                cudaSuccess &&
            (N == 0 || (cudaMemcpy(s->ID[0], ids.data(), N * sizeof(int32_t), cudaMemcpyHostToDevice) ==
                            cudaSuccess &&
                        cudaMemcpy(s->ID[1], ids.data(), N * sizeof(int32_t), cudaMemcpyHostToDevice) ==
                            cudaSuccess));
  if (!ok) {
    set_error("initial upload failed");
    return fail(CWA_ERR_CUDA);
  }
  *out = s;
  return CWA_OK;
}

cwa_status cwa_destroy(cwa_sim* sim) {
  if (!sim) return arg_error("null sim");
  free_sim(sim);
  return CWA_OK;
}

cwa_status cwa_upload_particles(cwa_sim* s, int32_t scene, const cwa_particle* host, int32_t n) {
  CWA_TRY(check_scene(s, scene));
  const SceneDev& d = s->sd[scene];
  if (n != d.n || (!host && n > 0)) return arg_error("upload size must equal the scene's n_particles");
  if (n == 0) return CWA_OK;
  // page-locked records are read by the unpack kernel itself, over the host
  // link; pageable ones go through the staging buffer
  const cwa_particle* src = static_cast<const cwa_particle*>(host_alias(host, (size_t)n * sizeof(cwa_particle)));
  if (!src) {
    CWA_CUDA(cudaMemcpyAsync(s->staging, host, (size_t)n * sizeof(cwa_particle), cudaMemcpyHostToDevice,
                             s->stream));
    src = s->staging;
  }
  CWA_CUDA(launch_unpack(src, n, d.poff, s->P[s->cur], s->V[s->cur], cur_force(s), s->RP, s->EX, s->ID[s->cur],
                         s->stream));
  s->launches += 1;
  s->grid_fresh = false;
  CWA_TRY(drop_pending_counts(s));
  if (s->verlet) {  // the new particles need a fresh grid and Verlet list
    const int32_t one = 1;
    CWA_CUDA(cudaMemcpyAsync(s->d_flag, &one, sizeof(one), cudaMemcpyHostToDevice, s->stream));
  }
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  return CWA_OK;
}

cwa_status cwa_download_particles(cwa_sim* s, int32_t scene, cwa_particle* host, int32_t n) {
  CWA_TRY(check_scene(s, scene));
  const SceneDev& d = s->sd[scene];
  if (n != d.n || (!host && n > 0)) return arg_error("download size must equal the scene's n_particles");
  if (n == 0) return CWA_OK;
  CWA_CUDA(launch_pack(s->staging, n, d.poff, s->P[s->cur], s->V[s->cur], cur_force(s), s->RP, s->EX,
                       s->ID[s->cur], s->stream));
  s->launches += 1;
  // the pack scatters the records back to upload order in device memory; a
  // page-locked destination then takes them in one coalesced kernel copy
  if (void* dst = host_alias(host, (size_t)n * sizeof(cwa_particle))) {
    CWA_CUDA(launch_copy_f32(reinterpret_cast<const float*>(s->staging), static_cast<float*>(dst),
                             (long)n * (long)(sizeof(cwa_particle) / sizeof(float)), s->stream));
    s->launches += 1;
  } else {
    CWA_CUDA(cudaMemcpyAsync(host, s->staging, (size_t)n * sizeof(cwa_particle), cudaMemcpyDeviceToHost,
                             s->stream));
  }
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  return CWA_OK;
}

cwa_status cwa_upload_wave(cwa_sim* s, int32_t scene, const float* u_n, const float* u_nm1, int32_t nx,
                           int32_t nz) {
  CWA_TRY(check_scene(s, scene));
  const SceneDev& d = s->sd[scene];
  if (nx != d.nx || nz != d.nz || !u_n) return arg_error("wave upload size must equal the scene's grid");
  const long cells = (long)nx * nz;
  const int w = s->wcur;
  CWA_TRY(copy_field(s, u_n, s->U[w] + d.woff, cells, cudaMemcpyHostToDevice));
  CWA_TRY(copy_field(s, u_nm1 ? u_nm1 : u_n, s->U[(w + 2) % 3] + d.woff, cells, cudaMemcpyHostToDevice));
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  return CWA_OK;
}

cwa_status cwa_download_wave(cwa_sim* s, int32_t scene, float* u_n, float* u_nm1, int32_t nx, int32_t nz) {
  CWA_TRY(check_scene(s, scene));
  const SceneDev& d = s->sd[scene];
  if (nx != d.nx || nz != d.nz) return arg_error("wave download size must equal the scene's grid");
  const long cells = (long)nx * nz;
  const int w = s->wcur;
  if (u_n) CWA_TRY(copy_field(s, s->U[w] + d.woff, u_n, cells, cudaMemcpyDeviceToHost));
  if (u_nm1) CWA_TRY(copy_field(s, s->U[(w + 2) % 3] + d.woff, u_nm1, cells, cudaMemcpyDeviceToHost));
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  return CWA_OK;
}

cwa_status cwa_wave_reinit(cwa_sim* s, int32_t scene) {
  CWA_TRY(check_scene(s, scene));
  const SceneDev& d = s->sd[scene];
  const int w = s->wcur;
  CWA_CUDA(launch_wave_init(s->U[w] + d.woff, d.nx, d.nz, d.mode, s->stream));
  CWA_CUDA(launch_wave_init(s->U[(w + 2) % 3] + d.woff, d.nx, d.nz, d.mode, s->stream));
  s->launches += 2;
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  return CWA_OK;
}

cwa_status cwa_wave_init_from_image(cwa_sim* s, int32_t scene, const uint8_t* rgba, int32_t width,
                                    int32_t height) {
  CWA_TRY(check_scene(s, scene));
  if (width < 1 || height < 1 || !rgba) return arg_error("image must be at least 1x1 RGBA8 texels");
  if ((int64_t)width * height > (1ll << 28)) return arg_error("image above 2^28 texels");
  const SceneDev& d = s->sd[scene];
  const size_t bytes = (size_t)width * height * 4;
  const size_t cells = (size_t)d.nx * d.nz;
  const int w = s->wcur;
  uint8_t* img = nullptr;
  CWA_CUDA(cudaMalloc((void**)&img, bytes));
  cudaError_t e = cudaMemcpyAsync(img, rgba, bytes, cudaMemcpyHostToDevice, s->stream);
  // the rotation for this scene alone: u^(n-1) <- u^n, then u^n <- image
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->U[(w + 2) % 3] + d.woff, s->U[w] + d.woff, cells * sizeof(float),
                        cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess) e = launch_wave_from_image(s->U[w] + d.woff, d.nx, d.nz, img, width, height, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  cudaFree(img);
  CWA_CUDA(e);
  s->launches += 1;
  return CWA_OK;
}

cwa_status cwa_render_defaults(int32_t width, int32_t height, cwa_camera* cam, cwa_render_params* prm) {
  if (!cam || !prm) return arg_error("null output");
  if (width < 1 || height < 1) return arg_error("image must be at least 1x1");
  *cam = cwa_camera{};
  *prm = cwa_render_params{};
  cam->eye[0] = 7.0f;
  cam->eye[1] = 4.0f;
  cam->eye[2] = 0.0f;
  cam->center[0] = 0.0f;
  cam->center[1] = -1.0f;
  cam->center[2] = 0.0f;
  cam->up[1] = 1.0f;
  cam->fovy = 3.14159265358979323846f / 4.0f;
  cam->near_z = 0.1f;
  cam->far_z = 100.0f;
  prm->width = width;
  prm->height = height;
  prm->angle = 0.75f;
  prm->particle_scale = 5.0f;
  prm->wave_scale = 0.047f;
  prm->point_size = 8.0f;
  prm->surface_res = 512;
  prm->draw_surface = 1;
  prm->draw_particles = 1;
  prm->draw_skybox = 0;
  return CWA_OK;
}

cwa_status cwa_render_set_skybox(cwa_sim* s, const uint8_t* faces, int32_t face_size) {
  CWA_TRY(check_sim(s));
  if (!faces || face_size < 1 || face_size > 8192) return arg_error("face_size must be in [1, 8192]");
  if (!s->render) s->render = render_state_new();
  CWA_CUDA(render_set_skybox(s->render, faces, face_size, s->stream));
  return CWA_OK;
}

cwa_status cwa_render(cwa_sim* s, int32_t scene, const cwa_camera* cam, const cwa_render_params* prm,
                      uint8_t* out) {
  CWA_TRY(check_scene(s, scene));
  if (!cam || !prm || !out) return arg_error("null camera, params or output");
  if (prm->width < 1 || prm->height < 1 || (int64_t)prm->width * prm->height > (1ll << 26))
    return arg_error("image size must be in [1, 2^26] pixels");
  if (prm->surface_res < 3 || prm->surface_res > 8192) return arg_error("surface_res must be in [3, 8192]");
  if (!(prm->point_size > 0.0f && prm->point_size <= 256.0f)) return arg_error("point_size must be in (0, 256]");
  if (!(cam->near_z > 0.0f && cam->far_z > cam->near_z) || !(cam->fovy > 0.0f && cam->fovy < 3.14159f))
    return arg_error("camera needs 0 < near < far and 0 < fovy < pi");
  if (!s->render) s->render = render_state_new();
  const SceneDev& d = s->sd[scene];
  CWA_CUDA(render_frame(s->render, *cam, *prm, s->P[s->cur] + d.poff, s->ID[s->cur] + d.poff, d.n,
                        s->U[s->wcur] + d.woff, d.nx, d.nz, out, s->d_status, s->stream, &s->launches));
  return read_status(s);
}

cwa_status cwa_step(cwa_sim* s, int32_t n_steps) {
  CWA_TRY(check_sim(s));
  if (n_steps < 0) return arg_error("n_steps < 0");
  NvtxRange range("cwa_step");
  for (int32_t k = 0; k < n_steps; ++k) {
    if (s->opt.use_graph && !s->profiling)
      CWA_TRY(graph_step(s));
    else
      CWA_TRY(enqueue_step(s));
  }
  return CWA_OK;
}

cwa_status cwa_pass_grid(cwa_sim* s) {
  CWA_TRY(check_sim(s));
  if (s->verlet) {  // an explicit grid pass always rebuilds
    const int32_t one = 1;
    CWA_CUDA(cudaMemcpyAsync(s->d_flag, &one, sizeof(one), cudaMemcpyHostToDevice, s->stream));
    CWA_CUDA(cudaStreamSynchronize(s->stream));
  }
  return run_grid(s);
}

cwa_status cwa_get_rebuild_count(cwa_sim* s, int64_t* rebuilds) {
  CWA_TRY(check_sim(s));
  if (!rebuilds) return arg_error("null output");
  unsigned long long v = 0;
  CWA_CUDA(cudaMemcpyAsync(&v, s->d_rebuilds, sizeof(v), cudaMemcpyDeviceToHost, s->stream));
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  *rebuilds = (int64_t)v;
  return CWA_OK;
}

cwa_status cwa_pass_rho_pres(cwa_sim* s) {
  CWA_TRY(check_sim(s));
  if (!s->grid_fresh) return arg_error("cwa_pass_grid must run before rho_pres in each step");
  return run_rho_pres(s);
}

cwa_status cwa_pass_force(cwa_sim* s) {
  CWA_TRY(check_sim(s));
  if (!s->grid_fresh) return arg_error("cwa_pass_grid must run before force in each step");
  return run_force(s);
}

cwa_status cwa_pass_integrate(cwa_sim* s) {
  CWA_TRY(check_sim(s));
  return run_integrate(s);
}

cwa_status cwa_pass_wave(cwa_sim* s) {
  CWA_TRY(check_sim(s));
  return run_wave(s);
}

cwa_status cwa_wave_advance(cwa_sim* s, int32_t n_steps) {
  CWA_TRY(check_sim(s));
  if (n_steps < 0) return arg_error("n_steps < 0");
  NvtxRange range("cwa_wave_advance");
  return run_wave_advance(s, n_steps);
}

cwa_status cwa_synchronize(cwa_sim* s) {
  CWA_TRY(check_sim(s));
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  return read_status(s);
}

cwa_status cwa_get_step_count(cwa_sim* s, int64_t* steps) {
  CWA_TRY(check_sim(s));
  if (!steps) return arg_error("null output");
  *steps = s->steps;
  return CWA_OK;
}

cwa_status cwa_get_device_view(cwa_sim* s, int32_t scene, cwa_device_view* v) {
  CWA_TRY(check_scene(s, scene));
  if (!v) return arg_error("null output");
  const SceneDev& d = s->sd[scene];
  v->n_particles = d.n;
  v->n_cells = d.ncells;
  for (int a = 0; a < 3; ++a) v->grid_dims[a] = d.dims[a];
  v->wave_nx = d.nx;
  v->wave_nz = d.nz;
  v->pos = reinterpret_cast<float*>(s->P[s->cur] + d.poff);
  v->vel = reinterpret_cast<float*>(s->V[s->cur] + d.poff);
  v->force = reinterpret_cast<float*>(cur_force(s) + d.poff);
  v->rho_p = reinterpret_cast<float*>(s->RP + d.poff);
  v->particle_id = s->ID[s->cur] + d.poff;
  v->cell_start = s->start + d.coff;
  v->wave_u_n = s->U[s->wcur] + d.woff;
  v->wave_u_nm1 = s->U[(s->wcur + 2) % 3] + d.woff;
  v->stream = (void*)s->stream;
  return CWA_OK;
}

cwa_status cwa_download_grid(cwa_sim* s, int32_t scene, int32_t* cell_start, int32_t n_cells_p1,
                             int32_t* sorted_id, int32_t n) {
  CWA_TRY(check_scene(s, scene));
  const SceneDev& d = s->sd[scene];
  if (cell_start && n_cells_p1 != d.ncells + 1) return arg_error("cell_start needs n_cells + 1 entries");
  if (sorted_id && n != d.n) return arg_error("sorted_id needs n_particles entries");
  if (cell_start) {
    CWA_CUDA(cudaMemcpyAsync(cell_start, s->start + d.coff, (size_t)n_cells_p1 * sizeof(int32_t),
                             cudaMemcpyDeviceToHost, s->stream));
  }
  if (sorted_id && n > 0)
    CWA_CUDA(cudaMemcpyAsync(sorted_id, s->ID[s->cur] + d.poff, (size_t)n * sizeof(int32_t),
                             cudaMemcpyDeviceToHost, s->stream));
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  if (cell_start)
    for (int32_t c = 0; c < n_cells_p1; ++c) cell_start[c] -= d.poff;
  return CWA_OK;
}

cwa_status cwa_download_deposits(cwa_sim* s, int32_t scene, int64_t* out, int32_t nx, int32_t nz) {
  CWA_TRY(check_scene(s, scene));
  const SceneDev& d = s->sd[scene];
  if (!out || nx != d.nx || nz != d.nz) return arg_error("deposit download size must equal the wave grid");
  CWA_CUDA(cudaMemcpyAsync(out, s->D + d.woff, (size_t)nx * nz * sizeof(int64_t), cudaMemcpyDeviceToHost,
                           s->stream));
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  return CWA_OK;
}

cwa_status cwa_reduce_totals(cwa_sim* s, int32_t scene, double out[CWA_TOTALS_COUNT]) {
  CWA_TRY(check_scene(s, scene));
  if (!out) return arg_error("null output");
  const SceneDev& d = s->sd[scene];
  CWA_CUDA(launch_totals(s->P[s->cur], s->V[s->cur], d.poff, d.n, s->U[s->wcur], s->U[(s->wcur + 2) % 3],
                         d.woff, d.nx * d.nz, s->d_scenes, scene, s->d_totals, s->stream));
  s->launches += 2;
  CWA_CUDA(cudaMemcpyAsync(s->h_totals, s->d_totals + (size_t)kTotalsBlocks * CWA_TOTALS_COUNT,
                           CWA_TOTALS_COUNT * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  memcpy(out, s->h_totals, CWA_TOTALS_COUNT * sizeof(double));
  return CWA_OK;
}

// Checkpoint: "CWAS", version 2, n_scenes, step count, every scene's
// descriptor, then the sim's device state in a fixed order: the sorted
// particle arrays (pos, vel, force, rho_p, id), extras.zw, the sorted keys
// and cell starts of the last grid build, u^n and u^(n-1), and in Verlet
// mode the Verlet list, its counts, the rebuild positions and the rebuild
// flag.  Restoring the sorted order and the grid keeps a resumed run
// bit-identical to an uninterrupted one.
struct StateItem {
  void* dev;
  size_t bytes;
};

std::vector<StateItem> state_items(cwa_sim* s) {
  const size_t N = (size_t)s->n_total, W = (size_t)s->w_total;
  std::vector<StateItem> it = {
      {s->P[s->cur], N * 16}, {s->V[s->cur], N * 16}, {cur_force(s), N * 16}, {s->RP, N * 8},
      {s->ID[s->cur], N * 4}, {s->EX, N * 8},          {s->KS, N * 4},        {s->start, ((size_t)s->c_total + 1) * 4},
      {s->U[s->wcur], W * 4}, {s->U[(s->wcur + 2) % 3], W * 4},
  };
  if (s->verlet) {
    it.push_back({s->vlist, N * kMaxVerlet * 2});
    it.push_back({s->vcnt, N * 4});
    it.push_back({s->XR, N * 16});
    it.push_back({s->d_flag, 4});
  }
  return it;
}

cwa_status cwa_save(cwa_sim* s, const char* path) {
  CWA_TRY(check_sim(s));
  if (!path) return arg_error("null path");
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  FILE* f = fopen(path, "wb");
  if (!f) {
    set_error(std::string("cannot open ") + path);
    return CWA_ERR_IO;
  }
  bool ok = true;
  auto put = [&](const void* p, size_t b) { ok = ok && (b == 0 || fwrite(p, 1, b, f) == b); };
  const uint32_t magic = 0x53415743u, version = 2;  // "CWAS"
  const int32_t ns = (int32_t)s->desc.size(), verlet = s->verlet ? 1 : 0;
  put(&magic, 4);
  put(&version, 4);
  put(&ns, 4);
  put(&verlet, 4);
  put(&s->steps, 8);
  put(s->desc.data(), s->desc.size() * sizeof(cwa_scene_desc));
  std::vector<char> buf;
  for (const StateItem& it : state_items(s)) {
    if (!ok) break;
    buf.resize(it.bytes);
    if (it.bytes && cudaMemcpy(buf.data(), it.dev, it.bytes, cudaMemcpyDeviceToHost) != cudaSuccess) {
      fclose(f);
      set_error("checkpoint readback failed");
      return CWA_ERR_CUDA;
    }
    put(buf.data(), it.bytes);
  }
  if (fclose(f) != 0) ok = false;
  if (!ok) {
    set_error(std::string("write failed: ") + path);
    return CWA_ERR_IO;
  }
  return CWA_OK;
}

cwa_status cwa_load(cwa_sim* s, const char* path) {
  CWA_TRY(check_sim(s));
  if (!path) return arg_error("null path");
  FILE* f = fopen(path, "rb");
  if (!f) {
    set_error(std::string("cannot open ") + path);
    return CWA_ERR_IO;
  }
  bool ok = true;
  auto get = [&](void* p, size_t b) { ok = ok && (b == 0 || fread(p, 1, b, f) == b); };
  uint32_t magic = 0, version = 0;
  int32_t ns = 0, verlet = 0;
  int64_t steps = 0;
  get(&magic, 4);
  get(&version, 4);
  get(&ns, 4);
  get(&verlet, 4);
  get(&steps, 8);
  std::vector<cwa_scene_desc> desc(ns > 0 && ns == (int32_t)s->desc.size() ? ns : 0);
  if (ok) get(desc.data(), desc.size() * sizeof(cwa_scene_desc));
  if (!ok || magic != 0x53415743u || version != 2 || ns != (int32_t)s->desc.size() ||
      verlet != (s->verlet ? 1 : 0) ||
      memcmp(desc.data(), s->desc.data(), desc.size() * sizeof(cwa_scene_desc)) != 0) {
    fclose(f);
    set_error("checkpoint does not match this sim (scenes, mode or version)");
    return ok ? CWA_ERR_INVALID_ARG : CWA_ERR_IO;
  }
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  std::vector<char> buf;
  for (const StateItem& it : state_items(s)) {
    buf.resize(it.bytes);
    get(buf.data(), it.bytes);
    if (!ok) break;
    if (it.bytes && cudaMemcpy(it.dev, buf.data(), it.bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
      fclose(f);
      set_error("checkpoint upload failed");
      return CWA_ERR_CUDA;
    }
  }
  fclose(f);
  if (!ok) {
    set_error(std::string("truncated checkpoint: ") + path);
    return CWA_ERR_IO;
  }
  s->steps = steps;
  s->grid_fresh = s->verlet;  // per-step mode rebuilds its grid every step anyway
  CWA_TRY(drop_pending_counts(s));
  return CWA_OK;
}

cwa_status cwa_set_profiling(cwa_sim* s, int32_t enable) {
  CWA_TRY(check_sim(s));
  s->profiling = enable != 0;
  s->pass_times_valid = false;
  return CWA_OK;
}

cwa_status cwa_get_pass_times(cwa_sim* s, float* ms, int32_t n) {
  CWA_TRY(check_sim(s));
  if (!ms || n < CWA_PASS_COUNT) return arg_error("need CWA_PASS_COUNT outputs");
  if (!s->pass_times_valid) return arg_error("no profiled step yet (cwa_set_profiling, then cwa_step)");
  CWA_CUDA(cudaEventSynchronize(s->ev[CWA_PASS_COUNT]));
  for (int k = 0; k < CWA_PASS_COUNT; ++k) CWA_CUDA(cudaEventElapsedTime(ms + k, s->ev[k], s->ev[k + 1]));
  return CWA_OK;
}

cwa_status cwa_debug_fail_alloc(int32_t n) {
  if (n < -1) return arg_error("n must be -1 (off) or >= 0");
  g_fail_alloc_in.store(n);
  return CWA_OK;
}

cwa_status cwa_get_launch_count(cwa_sim* s, int64_t* launches) {
  CWA_TRY(check_sim(s));
  if (!launches) return arg_error("null output");
  *launches = s->launches;
  return CWA_OK;
}

// ---- autotuner ----
// Tries the kernel variants on the sim's own state: candidate staging on /
// off, the density-scan and force launch-bound variants and 128- or
// 64-particle CTAs.  Every trial starts from a device-side snapshot of the
// state and runs one warm-up step and `trial_steps` timed steps (CUDA
// events, eager launches); the fastest is kept and the state restored.
cwa_status cwa_autotune(cwa_sim* s, int32_t trial_steps, cwa_tune_report* out) {
  CWA_TRY(check_sim(s));
  if (trial_steps < 1 || trial_steps > 1000) return arg_error("trial_steps must be in [1, 1000]");
  CWA_TRY(drop_pending_counts(s));  // every trial starts from zero counts
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  std::vector<StateItem> items = state_items(s);
  size_t total = 0;
  for (const StateItem& it : items) total += (it.bytes + 255) & ~(size_t)255;
  char* snap = nullptr;
  CWA_CUDA(cudaMalloc((void**)&snap, std::max<size_t>(total, 1)));
  auto copy_state = [&](bool save) -> cudaError_t {
    size_t off = 0;
    for (const StateItem& it : items) {
      cudaError_t e = save ? cudaMemcpyAsync(snap + off, it.dev, it.bytes, cudaMemcpyDeviceToDevice, s->stream)
                           : cudaMemcpyAsync(it.dev, snap + off, it.bytes, cudaMemcpyDeviceToDevice, s->stream);
      if (e != cudaSuccess) return e;
      off += (it.bytes + 255) & ~(size_t)255;
    }
    return cudaSuccess;
  };
  const cwa_sim_options entry = s->opt;
  const int32_t entry_ptile = s->ptile;
  const int64_t steps0 = s->steps, launches0 = s->launches;
  const int cur0 = s->cur, w0 = s->wcur;
  const bool prof0 = s->profiling;
  s->profiling = false;
  cwa_tune_report rep;
  memset(&rep, 0, sizeof(rep));
  rep.best_ms = 1e30f;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t err = copy_state(true);
  if (err == cudaSuccess) err = cudaEventCreate(&e0);
  if (err == cudaSuccess) err = cudaEventCreate(&e1);
  const int stages[2] = {0, -1}, scans[3] = {4, 6, 8}, forces[2] = {8, 9}, ctas[2] = {128, 64};
  constexpr int kCombos = 2 * 3 * 2 * 2;
  // Two rounds, the second in reverse order; each combination keeps its
  // faster round, which damps clock and neighbour-load noise.
  float best_of[kCombos];
  for (float& v : best_of) v = 1e30f;
  for (int round = 0; round < 2 && err == cudaSuccess; ++round)
    for (int q = 0; q < kCombos && err == cudaSuccess; ++q) {
      const int idx = round == 0 ? q : kCombos - 1 - q;
      const int a = idx / 12, b = (idx / 4) % 3, c = (idx / 2) % 2, d = idx % 2;
      cwa_sim_options o = entry;
      o.nb_stage = stages[a];
      o.nb_scan_minb = scans[b];
      o.nb_force_minb = forces[c];
      o.nb_threads = ctas[d];
      s->opt = o;
      if (s->ptile != ctas[d]) {
        cwa_status st = set_particle_tiles(s, ctas[d]);
        if (st != CWA_OK) {
          err = cudaErrorMemoryAllocation;
          break;
        }
      }
      err = copy_state(false);
      s->cur = cur0;
      s->wcur = w0;
      s->counts_pending = true;  // the last trial's integrate counted its own positions
      if (err == cudaSuccess && drop_pending_counts(s) != CWA_OK) err = cudaErrorUnknown;
      if (err != cudaSuccess) break;
      cwa_status st = enqueue_step(s);  // warm-up
      if (st == CWA_OK) err = cudaEventRecord(e0, s->stream);
      for (int k = 0; k < trial_steps && st == CWA_OK && err == cudaSuccess; ++k) st = enqueue_step(s);
      if (st != CWA_OK) {
        err = cudaErrorLaunchFailure;
        break;
      }
      if (err == cudaSuccess) err = cudaEventRecord(e1, s->stream);
      if (err == cudaSuccess) err = cudaEventSynchronize(e1);
      float ms = 0.0f;
      if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
      ms /= (float)trial_steps;
      best_of[idx] = std::min(best_of[idx], ms);
      if (round == 1) {
        ms = best_of[idx];
        if (rep.n_tried < CWA_TUNE_MAX_TRIED) {
          rep.tried[rep.n_tried] = o;
          rep.tried_ms[rep.n_tried] = ms;
        }
        rep.n_tried++;
        // the entry options, with 0 read as each knob's default
        if ((o.nb_stage < 0) == (entry.nb_stage < 0) &&
            o.nb_scan_minb == (entry.nb_scan_minb ? entry.nb_scan_minb : 4) &&
            o.nb_force_minb == (entry.nb_force_minb ? entry.nb_force_minb : 9) &&
            o.nb_threads == (entry.nb_threads ? entry.nb_threads : 128))
          rep.entry_ms = ms;
        if (ms < rep.best_ms) {
          rep.best_ms = ms;
          rep.best = o;
        }
      }
    }
  // A winner within 1.5% of the entry options is trial noise (variants that
  // tie in short trials have differed by 10% over a long run): keep the
  // entry options then.
  if (err == cudaSuccess && rep.entry_ms > 0.0f && rep.best_ms > 0.985f * rep.entry_ms) {
    rep.best = entry;
    rep.best_ms = rep.entry_ms;
  }
  // keep the winner (or the entry options on failure) and restore the state
  s->opt = err == cudaSuccess ? rep.best : entry;
  const int32_t want_ptile = s->opt.nb_threads ? s->opt.nb_threads : entry_ptile;
  if (s->ptile != want_ptile) set_particle_tiles(s, want_ptile);
  cudaError_t e2 = copy_state(false);
  if (err == cudaSuccess) err = e2;
  s->counts_pending = true;
  if (drop_pending_counts(s) != CWA_OK && err == cudaSuccess) err = cudaErrorUnknown;
  cudaStreamSynchronize(s->stream);
  s->cur = cur0;
  s->wcur = w0;
  s->steps = steps0;
  s->launches = launches0;
  s->profiling = prof0;
  drop_graphs(s);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(snap);
  if (out) *out = rep;
  CWA_CUDA(err);
  return CWA_OK;
}

// Wave tuner: every blocked variant from the same snapshot of the two live
// wave slots (and the deposit buffer, when a pending integrate filled it),
// trial_steps wave steps each (rounded up to a multiple of 8, so every
// variant runs whole blocks), best of two rounds; keeps the fastest in
// opt.wave_block and restores the state, the slot map included.
cwa_status cwa_autotune_wave(cwa_sim* s, int32_t trial_steps, cwa_wave_tune_report* out) {
  CWA_TRY(check_sim(s));
  if (trial_steps < 1 || trial_steps > 4096) return arg_error("trial_steps must be in [1, 4096]");
  const int32_t steps = (trial_steps + 7) & ~7;
  CWA_TRY(prepare_wave_blocks(s));
  CWA_CUDA(cudaStreamSynchronize(s->stream));
  const size_t W = (size_t)s->w_total;
  const int w0 = s->wcur;
  int uid0[4];
  for (int b = 0; b < 4; ++b) uid0[b] = s->uid[b];
  float* live[2] = {s->U[w0], s->U[(w0 + 2) % 3]};
  const bool dep0 = s->deposits_pending;
  const int64_t steps0 = s->steps, launches0 = s->launches;
  const int32_t entry = s->opt.wave_block;
  char* snap = nullptr;
  CWA_CUDA(cudaMalloc((void**)&snap, W * 16 + 256));
  float* snap_u = reinterpret_cast<float*>(snap);
  unsigned long long* snap_d = reinterpret_cast<unsigned long long*>(snap + W * 8);
  auto copy_state = [&](bool save) -> cudaError_t {
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 2 && e == cudaSuccess; ++k)
      e = save ? cudaMemcpyAsync(snap_u + k * W, live[k], W * 4, cudaMemcpyDeviceToDevice, s->stream)
               : cudaMemcpyAsync(live[k], snap_u + k * W, W * 4, cudaMemcpyDeviceToDevice, s->stream);
    if (e == cudaSuccess && dep0)
      e = save ? cudaMemcpyAsync(snap_d, s->D, W * 8, cudaMemcpyDeviceToDevice, s->stream)
               : cudaMemcpyAsync(s->D, snap_d, W * 8, cudaMemcpyDeviceToDevice, s->stream);
    for (int b = 0; b < 4; ++b) s->uid[b] = uid0[b];
    for (int b = 0; b < 3; ++b) s->U[b] = s->UB[uid0[b]];
    s->wcur = w0;
    s->deposits_pending = dep0;
    return e;
  };
  cwa_wave_tune_report rep;
  memset(&rep, 0, sizeof(rep));
  rep.steps = steps;
  for (float& m : rep.ms_per_step) m = 1e30f;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t err = copy_state(true);
  if (err == cudaSuccess) err = cudaEventCreate(&e0);
  if (err == cudaSuccess) err = cudaEventCreate(&e1);
  for (int round = 0; round < 2 && err == cudaSuccess; ++round)
    for (int q = 0; q < CWA_WAVE_BLOCK_COUNT && err == cudaSuccess; ++q) {
      const int v = round == 0 ? q : CWA_WAVE_BLOCK_COUNT - 1 - q;
      s->opt.wave_block = v;
      err = copy_state(false);
      if (err != cudaSuccess) break;
      // a pending deposit is applied by an untimed single pass first
      if (dep0 && run_wave(s) != CWA_OK) err = cudaErrorLaunchFailure;
      if (err == cudaSuccess && run_wave_advance(s, 8) != CWA_OK) err = cudaErrorLaunchFailure;  // warm-up
      if (err == cudaSuccess) err = cudaEventRecord(e0, s->stream);
      if (err == cudaSuccess && run_wave_advance(s, steps) != CWA_OK) err = cudaErrorLaunchFailure;
      if (err == cudaSuccess) err = cudaEventRecord(e1, s->stream);
      if (err == cudaSuccess) err = cudaEventSynchronize(e1);
      float ms = 0.0f;
      if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
      if (err == cudaSuccess) rep.ms_per_step[v] = std::min(rep.ms_per_step[v], ms / (float)steps);
    }
  rep.best = entry;
  if (err == cudaSuccess)
    for (int v = 0; v < CWA_WAVE_BLOCK_COUNT; ++v)
      if (rep.ms_per_step[v] < rep.ms_per_step[rep.best]) rep.best = v;
  s->opt.wave_block = rep.best;
  cudaError_t e2 = copy_state(false);
  if (err == cudaSuccess) err = e2;
  cudaStreamSynchronize(s->stream);
  s->steps = steps0;
  s->launches = launches0;
  drop_graphs(s);  // captured steps hold the trials' buffer pointers
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(snap);
  if (out) *out = rep;
  CWA_CUDA(err);
  return read_status(s);
}

cwa_status cwa_get_options(cwa_sim* s, cwa_sim_options* out) {
  CWA_TRY(check_sim(s));
  if (!out) return arg_error("null output");
  *out = s->opt;
  return CWA_OK;
}

// ---- stand-alone operators ----
size_t cwa_scan_workspace_bytes(int32_t n) { return scan_workspace_bytes(n < 0 ? 0 : n) + 256; }

cwa_status cwa_exclusive_scan_i32(const int32_t* d_in, int32_t* d_out, int32_t n, void* d_workspace,
                                  size_t workspace_bytes, void* stream) {
  if (n < 0) return arg_error("n < 0");
  if (n == 0) return CWA_OK;
  if (!d_in || !d_out || !d_workspace) return arg_error("null device pointer");
  if (workspace_bytes < cwa_scan_workspace_bytes(n)) return arg_error("workspace too small");
  ScanWorkspace ws;
  scan_bind_workspace(d_workspace, n, &ws);
  // A status word follows the tile states; a look-back time-out sets it.
  int32_t* status = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(d_workspace) + scan_workspace_bytes(n));
  cudaStream_t st = (cudaStream_t)stream;
  CWA_CUDA(cudaMemsetAsync(status, 0, sizeof(int32_t), st));
  CWA_CUDA(scan_launch(d_in, d_out, n, n, false, ws, status, st, nullptr));
  return CWA_OK;
}

cwa_status cwa_scan_status(int32_t n, const void* d_workspace, void* stream) {
  if (n < 0 || !d_workspace) return arg_error("bad arguments");
  if (n == 0) return CWA_OK;
  return read_status_word(
      reinterpret_cast<const int32_t*>(reinterpret_cast<const char*>(d_workspace) + scan_workspace_bytes(n)), stream);
}

size_t cwa_grid_workspace_bytes(int32_t n, int32_t n_cells) {
  if (n < 0 || n_cells < 1) return 0;
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  return up(scan_workspace_bytes(n_cells + 1)) + up((size_t)n_cells * 4) + 3 * up((size_t)n * 4 + 4) + 256;
}

cwa_status cwa_grid_build(const float* d_pos4, int32_t n, const float lo[3], float cell_size,
                          const int32_t dims[3], int32_t* d_cell_start, int32_t* d_sorted_index,
                          int32_t* d_cell_of, void* d_workspace, size_t workspace_bytes, void* stream) {
  if (n < 0 || !lo || !dims || !d_cell_start) return arg_error("bad arguments");
  if (!(cell_size > 0.0f) || dims[0] < 1 || dims[1] < 1 || dims[2] < 1) return arg_error("bad grid");
  const int64_t nc64 = (int64_t)dims[0] * dims[1] * dims[2];
  if (nc64 > (1ll << 31) - (1ll << 20)) return arg_error("too many cells");
  const int32_t nc = (int32_t)nc64;
  if (!d_workspace || workspace_bytes < cwa_grid_workspace_bytes(n, nc)) return arg_error("workspace too small");
  if (n > 0 && (!d_pos4 || !d_sorted_index)) return arg_error("null device pointer");
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  char* w = reinterpret_cast<char*>(d_workspace);
  ScanWorkspace ws;
  scan_bind_workspace(w, nc + 1, &ws);
  w += up(scan_workspace_bytes(nc + 1));
  int32_t* count = reinterpret_cast<int32_t*>(w);
  w += up((size_t)nc * 4);
  int32_t* key = reinterpret_cast<int32_t*>(w);
  w += up((size_t)n * 4 + 4);
  int32_t* slot = reinterpret_cast<int32_t*>(w);
  w += up((size_t)n * 4 + 4);
  int32_t* list = reinterpret_cast<int32_t*>(w);
  w += up((size_t)n * 4 + 4);
  int32_t* status = reinterpret_cast<int32_t*>(w);  // cwa_grid_status reads it
  if (d_cell_of) key = d_cell_of;
  cudaStream_t st = (cudaStream_t)stream;
  CWA_CUDA(cudaMemsetAsync(count, 0, (size_t)nc * 4, st));
  CWA_CUDA(cudaMemsetAsync(status, 0, 4, st));
  CWA_CUDA(launch_point_hash(reinterpret_cast<const float4*>(d_pos4), n, lo[0], lo[1], lo[2], cell_size, dims[0],
                             dims[1], dims[2], key, slot, count, status, st));
  CWA_CUDA(scan_launch(count, d_cell_start, nc, nc + 1, false, ws, status, st, nullptr));
  CWA_CUDA(launch_list_insert(key, slot, d_cell_start, list, n, nullptr, st));
  CWA_CUDA(launch_point_rank(key, slot, d_cell_start, list, n, d_sorted_index, status, st));
  return CWA_OK;
}

cwa_status cwa_grid_status(int32_t n, int32_t n_cells, const void* d_workspace, void* stream) {
  if (n < 0 || n_cells < 1 || !d_workspace) return arg_error("bad arguments");
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t off = up(scan_workspace_bytes(n_cells + 1)) + up((size_t)n_cells * 4) + 3 * up((size_t)n * 4 + 4);
  return read_status_word(reinterpret_cast<const int32_t*>(reinterpret_cast<const char*>(d_workspace) + off),
                          stream);
}

}  // extern "C"
