// cwa_pbd.cu — position-based box collisions on the uniform grid: the
// reference's GridTestPbdGpu3D demo (UniformGrid2D/UniformGridGpu3D.cpp:
// 128-183, 292-346; uniform_grid_pbd_3D_cs.glsl:113-382).
//
// One substep: boxes are inserted into every cell their AABB overlaps
// (COMPUTE_COUNTS / scan / INSERT_BOXES), PreAnimate predicts p = x + dt v,
// the collision query finds each box's contacts with the extents and with
// the boxes of higher index (the home-cell test visits each pair once), and
// PostAnimate applies the averaged displacements with SOR factor k and
// restitution e.
//
// The shader accumulates every contact into both boxes with float atomics,
// so its sums (and the wall terms, added without atomics beside them) depend
// on thread order.  Here the accumulation is a gather: the query writes each
// contact once into the lower box's pair slots, a stable counting sort
// indexes the pairs by their higher box, and PostAnimate sums, per box, its
// wall terms, then the pairs it owns in slot order, then the pairs it is the
// partner of in slot order.  Every float operation is rounded to nearest in
// a fixed order (round-to-nearest intrinsics), so a step is deterministic
// and the float32 CPU restatement reproduces it bit for bit.  Cell ids are
// (i ny + j) nz + k; the shader's (i ny + j) nx + k is the same on its cubic
// grid.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <string>

#include "cwa_device.cuh"
#include "cwa_internal.h"

namespace cwa {
namespace {

__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }

struct PbdConst {
  int n, nx, ny, nz, maxc, pcap;
  float lo[3], hi[3], cell[3];
  float g[3], dt, damping, k, k_static, sleep, mu_k, mu_s, e;
};

struct PbdPair {
  int32_t i, j;
  float wi, wj;
  float disp[3];
  float frict[3];
};

__device__ __forceinline__ float len3(float x, float y, float z) {
  return __fsqrt_rn(fa(fa(fm(x, x), fm(y, y)), fm(z, z)));
}

__device__ __forceinline__ int cell_c(const PbdConst& c, float p, int a) {
  const int n = a == 0 ? c.nx : (a == 1 ? c.ny : c.nz);
  return cell_axis(p, c.lo[a], c.cell[a], n);
}

__device__ __forceinline__ int cell_id(const PbdConst& c, int i, int j, int k) { return (i * c.ny + j) * c.nz + k; }

// COMPUTE_COUNTS / INSERT_BOXES: item q = box * maxc + t is the box's t-th
// overlapped cell (x-major, z fastest); unused slots get key -1.
__global__ void k_pbd_cells(PbdConst c, cwa_pbd_box* __restrict__ boxes, int32_t* __restrict__ ikey,
                            int32_t* __restrict__ islot, int32_t* __restrict__ count, int32_t* status) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= c.n) return;
  cwa_pbd_box& o = boxes[b];
  int lo[3], hi[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    lo[a] = cell_c(c, fs(o.x[a], o.hw[a]), a);
    hi[a] = cell_c(c, fa(o.x[a], o.hw[a]), a);
  }
  int t = 0;
  for (int i = lo[0]; i <= hi[0]; ++i)
    for (int j = lo[1]; j <= hi[1]; ++j)
      for (int k = lo[2]; k <= hi[2]; ++k) {
        if (t < c.maxc) {
          const int key = cell_id(c, i, j, k);
          ikey[(size_t)b * c.maxc + t] = key;
          islot[(size_t)b * c.maxc + t] = count_slot(count, key);
        } else {
          atomicOr(status, kStatusBigCell);
        }
        ++t;
      }
  for (; t < c.maxc; ++t) ikey[(size_t)b * c.maxc + t] = -1;
#pragma unroll
  for (int a = 0; a < 4; ++a) o.color[a] = 1.0f;  // InsertBox resets the colour
}

// Arrival-order insert, then the stable rank (members with a smaller index).
__global__ void k_pbd_insert(const int32_t* __restrict__ key, const int32_t* __restrict__ slot,
                             const int32_t* __restrict__ start, int32_t* __restrict__ list, int32_t n_items) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n_items || key[q] < 0) return;
  list[start[key[q]] + slot[q]] = q;
}

__global__ void k_pbd_rank(const int32_t* __restrict__ key, const int32_t* __restrict__ start,
                           const int32_t* __restrict__ list, int32_t* __restrict__ sorted, int32_t n_items) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n_items || key[q] < 0) return;
  const int b = start[key[q]], e = start[key[q] + 1];
  int rank = 0;
  for (int m = b; m < e; ++m) rank += list[m] < q;
  sorted[b + rank] = q;
}

// PreAnimate (:354-370).
__global__ void k_pbd_pre(PbdConst c, cwa_pbd_box* __restrict__ boxes) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= c.n) return;
  cwa_pbd_box& o = boxes[b];
  float v[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const float ga = a < 3 ? c.g[a] : 0.0f;
    v[a] = fm(c.damping, fa(o.v[a], fm(c.dt, ga)));
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    o.dp_n[a] = 0.0f;
    o.dp_t[a] = 0.0f;
    o.p[a] = fa(o.x[a], fm(c.dt, v[a]));
    o.v[a] = v[a];
  }
  o.n = 0.0f;
}

// Collide (:293-351) for the ordered pair (i < j); false when they do not overlap.
__device__ bool collide(const PbdConst& c, const cwa_pbd_box& bi, const cwa_pbd_box& bj, const float qmin[3],
                        const float qmax[3], const float bmin[3], const float bmax[3], PbdPair* out) {
  float sz[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) sz[a] = fs(fminf(qmax[a], bmax[a]), fmaxf(qmin[a], bmin[a]));
  int comp = 0;
  if (sz[1] < sz[0] && sz[1] < sz[2]) comp = 1;
  if (sz[2] < sz[0] && sz[2] < sz[1]) comp = 2;
  const float dist = fm(0.5f, sz[comp]);
  if (dist < 0.0f) return false;
  const float eps = 1e-8f;
  float dij[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) dij[a] = fs(bj.p[a], bi.p[a]);
  const float den = fa(len3(dij[0], dij[1], dij[2]), eps);
  float ud[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) ud[a] = fd(dij[a], den);
  const float sg = dij[comp] > 0.0f ? 1.0f : (dij[comp] < 0.0f ? -1.0f : 0.0f);
#pragma unroll
  for (int a = 0; a < 3; ++a) out->disp[a] = 0.0f;
  out->disp[comp] = fm(sg, dist);
  const float rs = fa(bi.rm, bj.rm);
  out->wi = fd(bi.rm, rs);
  out->wj = fd(bj.rm, rs);
  float dp[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) dp[a] = fs(fs(bj.x[a], bj.p[a]), fs(bi.x[a], bi.p[a]));
  const float d = fa(fa(fm(dp[0], ud[0]), fm(dp[1], ud[1])), fm(dp[2], ud[2]));
#pragma unroll
  for (int a = 0; a < 3; ++a) dp[a] = fs(dp[a], fm(d, ud[a]));
  const float mag = len3(dp[0], dp[1], dp[2]);
  float s = 1.0f;
  if (mag < fm(c.mu_s, dist)) s = fminf(1.0f, fd(fm(c.mu_k, dist), mag));
#pragma unroll
  for (int a = 0; a < 3; ++a) out->frict[a] = s == 1.0f ? dp[a] : fm(dp[a], s);
  return true;
}

// CollisionQuery (:225-290) for box i against the boxes of higher index.
__global__ void k_pbd_query(PbdConst c, cwa_pbd_box* __restrict__ boxes, const int32_t* __restrict__ cstart,
                            const int32_t* __restrict__ csorted, PbdPair* __restrict__ pairs,
                            int32_t* __restrict__ npairs, int32_t* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.n) return;
  const cwa_pbd_box bi = boxes[i];
  float qmin[3], qmax[3];
  int lo[3], hi[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    qmin[a] = fs(bi.p[a], bi.hw[a]);
    qmax[a] = fa(bi.p[a], bi.hw[a]);
    lo[a] = cell_c(c, qmin[a], a);
    hi[a] = cell_c(c, qmax[a], a);
  }
  int t = 0;
  for (int ci = lo[0]; ci <= hi[0]; ++ci)
    for (int cj = lo[1]; cj <= hi[1]; ++cj)
      for (int ck = lo[2]; ck <= hi[2]; ++ck) {
        const int cell = cell_id(c, ci, cj, ck);
        for (int r = cstart[cell]; r < cstart[cell + 1]; ++r) {
          const int j = csorted[r] / c.maxc;
          if (j <= i) continue;  // Collide returns for i >= j
          const cwa_pbd_box& bj = boxes[j];
          float bmin[3], bmax[3];
          int home[3];
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            bmin[a] = fs(bj.x[a], bj.hw[a]);
            bmax[a] = fa(bj.x[a], bj.hw[a]);
            home[a] = max(lo[a], cell_c(c, bmin[a], a));
          }
          if (home[0] != ci || home[1] != cj || home[2] != ck) continue;
          PbdPair pr;
          if (!collide(c, bi, bj, qmin, qmax, bmin, bmax, &pr)) continue;
          pr.i = i;
          pr.j = j;
          if (t < c.pcap)
            pairs[(size_t)i * c.pcap + t] = pr;
          else
            atomicOr(status, kStatusBigCell);
          ++t;
          const float red[4] = {1.0f, 0.0f, 0.0f, 1.0f};
#pragma unroll
          for (int a = 0; a < 4; ++a) {
            boxes[i].color[a] = red[a];  // the same value from every writer
            boxes[j].color[a] = red[a];
          }
        }
      }
  npairs[i] = min(t, c.pcap);
}

// The pairs indexed by their higher box: key = j for the used slots.
__global__ void k_pbd_rev_key(PbdConst c, const PbdPair* __restrict__ pairs, const int32_t* __restrict__ npairs,
                              int32_t* __restrict__ rkey, int32_t* __restrict__ rslot, int32_t* __restrict__ rcount) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= c.n * c.pcap) return;
  const int i = q / c.pcap, t = q - i * c.pcap;
  if (t >= npairs[i]) {
    rkey[q] = -1;
    return;
  }
  const int j = pairs[q].j;
  rkey[q] = j;
  rslot[q] = count_slot(rcount, j);
}

// wall terms, then the own pairs, then the partner pairs; PostAnimate (:372-392)
__global__ void k_pbd_post(PbdConst c, cwa_pbd_box* __restrict__ boxes, const PbdPair* __restrict__ pairs,
                           const int32_t* __restrict__ npairs, const int32_t* __restrict__ rstart,
                           const int32_t* __restrict__ rsorted) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= c.n) return;
  cwa_pbd_box o = boxes[b];
  float dpn[3] = {0.0f, 0.0f, 0.0f}, dpt[3] = {0.0f, 0.0f, 0.0f}, nn = 0.0f;
  // collisions with the extents (:230-259)
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float qmin = fs(o.p[a], o.hw[a]), qmax = fa(o.p[a], o.hw[a]);
    const float ov[2] = {fs(c.lo[a], qmin), fs(qmax, c.hi[a])};
    const float dir[2] = {1.0f, -1.0f};
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      if (!(ov[m] > 0.0f)) continue;
      dpn[a] = fa(dpn[a], fm(fm(dir[m], c.k_static), ov[m]));
      nn = fa(nn, c.k_static);
      float dp[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) dp[q] = q == a ? 0.0f : fs(o.x[q], o.p[q]);
      const float mag = len3(dp[0], dp[1], dp[2]);
      float s = 1.0f;
      if (mag < fm(c.mu_s, ov[m])) s = fminf(1.0f, fd(fm(c.mu_k, ov[m]), mag));
#pragma unroll
      for (int q = 0; q < 3; ++q) dpt[q] = fa(dpt[q], s == 1.0f ? dp[q] : fm(dp[q], s));
    }
  }
  for (int t = 0; t < npairs[b]; ++t) {  // b is the lower box
    const PbdPair& pr = pairs[(size_t)b * c.pcap + t];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      dpn[a] = fa(dpn[a], fm(-pr.wi, pr.disp[a]));
      dpt[a] = fa(dpt[a], fm(-pr.wi, pr.frict[a]));
    }
    nn = fa(nn, 1.0f);
  }
  for (int r = rstart[b]; r < rstart[b + 1]; ++r) {  // b is the higher box
    const PbdPair& pr = pairs[rsorted[r]];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      dpn[a] = fa(dpn[a], fm(pr.wj, pr.disp[a]));
      dpt[a] = fa(dpt[a], fm(pr.wj, pr.frict[a]));
    }
    nn = fa(nn, 1.0f);
  }
  float p[3], pe[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    p[a] = o.p[a];
    pe[a] = o.p[a];
  }
  if (nn > 0.0f) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      p[a] = fa(p[a], fd(fm(c.k, fa(dpt[a], dpn[a])), nn));
      pe[a] = fa(pe[a], fd(fm(c.k, fa(dpt[a], fm(c.e, dpn[a]))), nn));
      o.p[a] = p[a];
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    o.v[a] = fd(fs(pe[a], o.x[a]), c.dt);
    o.dp_n[a] = dpn[a];
    o.dp_t[a] = dpt[a];
  }
  o.n = nn;
  if (len3(fs(o.x[0], p[0]), fs(o.x[1], p[1]), fs(o.x[2], p[2])) > c.sleep)
#pragma unroll
    for (int a = 0; a < 3; ++a) o.x[a] = p[a];
  boxes[b].x[0] = o.x[0];
  boxes[b].x[1] = o.x[1];
  boxes[b].x[2] = o.x[2];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    boxes[b].p[a] = o.p[a];
    boxes[b].v[a] = o.v[a];
    boxes[b].dp_n[a] = o.dp_n[a];
    boxes[b].dp_t[a] = o.dp_t[a];
  }
  boxes[b].n = o.n;
}

constexpr int kB = 128;
inline unsigned nb(long n) { return (unsigned)((n + kB - 1) / kB); }

}  // namespace
}  // namespace cwa

using namespace cwa;

struct cwa_pbd_sim {
  int device = 0;
  cwa_pbd_params prm{};
  PbdConst k{};
  cudaStream_t stream = nullptr;
  cwa_pbd_box* boxes = nullptr;
  int32_t *ikey = nullptr, *islot = nullptr, *ccount = nullptr, *cstart = nullptr, *clist = nullptr,
          *csorted = nullptr;
  PbdPair* pairs = nullptr;
  int32_t *npairs = nullptr, *rkey = nullptr, *rslot = nullptr, *rcount = nullptr, *rstart = nullptr,
          *rlist = nullptr, *rsorted = nullptr;
  void *ws_cells = nullptr, *ws_rev = nullptr;
  ScanWorkspace scan_cells{}, scan_rev{};
  int32_t* d_status = nullptr;
  int ncells = 0;
  bool uploaded = false;
  cudaGraphExec_t graph = nullptr;
};

namespace {

cwa_status perr(const std::string& m, cwa_status s = CWA_ERR_INVALID_ARG) {
  cwa::set_error(m);
  return s;
}

#define PBD_CUDA(expr)                                                   \
  do {                                                                   \
    cudaError_t e_ = (expr);                                             \
    if (e_ != cudaSuccess) {                                             \
      cwa::set_error(std::string(#expr) + ": " + cudaGetErrorString(e_)); \
      cudaGetLastError(); /* clear a non-sticky error for the next call */ \
      return e_ == cudaErrorMemoryAllocation ? CWA_ERR_OOM : CWA_ERR_CUDA; \
    }                                                                    \
  } while (0)

void free_items(cwa_pbd_sim* s) {
  cudaFree(s->ikey);
  cudaFree(s->islot);
  cudaFree(s->clist);
  cudaFree(s->csorted);
  s->ikey = s->islot = s->clist = s->csorted = nullptr;
}

void free_pbd(cwa_pbd_sim* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->graph) cudaGraphExecDestroy(s->graph);
  free_items(s);
  void* ps[] = {s->boxes, s->ccount, s->cstart, s->pairs, s->npairs, s->rkey, s->rslot, s->rcount,
                s->rstart, s->rlist, s->rsorted, s->ws_cells, s->ws_rev, s->d_status};
  for (void* p : ps) cudaFree(p);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

cwa_status enqueue_substep(cwa_pbd_sim* s) {
  const PbdConst& c = s->k;
  cudaStream_t st = s->stream;
  const long items = (long)c.n * c.maxc, slots = (long)c.n * c.pcap;
  k_pbd_cells<<<nb(c.n), kB, 0, st>>>(c, s->boxes, s->ikey, s->islot, s->ccount, s->d_status);
  PBD_CUDA(cudaGetLastError());
  PBD_CUDA(scan_launch(s->ccount, s->cstart, s->ncells, s->ncells + 1, true, s->scan_cells, s->d_status, st,
                       nullptr));
  k_pbd_insert<<<nb(items), kB, 0, st>>>(s->ikey, s->islot, s->cstart, s->clist, (int32_t)items);
  k_pbd_rank<<<nb(items), kB, 0, st>>>(s->ikey, s->cstart, s->clist, s->csorted, (int32_t)items);
  k_pbd_pre<<<nb(c.n), kB, 0, st>>>(c, s->boxes);
  k_pbd_query<<<nb(c.n), kB, 0, st>>>(c, s->boxes, s->cstart, s->csorted, s->pairs, s->npairs, s->d_status);
  k_pbd_rev_key<<<nb(slots), kB, 0, st>>>(c, s->pairs, s->npairs, s->rkey, s->rslot, s->rcount);
  PBD_CUDA(cudaGetLastError());
  PBD_CUDA(scan_launch(s->rcount, s->rstart, c.n, c.n + 1, true, s->scan_rev, s->d_status, st, nullptr));
  k_pbd_insert<<<nb(slots), kB, 0, st>>>(s->rkey, s->rslot, s->rstart, s->rlist, (int32_t)slots);
  k_pbd_rank<<<nb(slots), kB, 0, st>>>(s->rkey, s->rstart, s->rlist, s->rsorted, (int32_t)slots);
  k_pbd_post<<<nb(c.n), kB, 0, st>>>(c, s->boxes, s->pairs, s->npairs, s->rstart, s->rsorted);
  PBD_CUDA(cudaGetLastError());
  return CWA_OK;
}

cwa_status read_pbd_status(cwa_pbd_sim* s) {
  int32_t v = 0;
  PBD_CUDA(cudaMemcpyAsync(&v, s->d_status, 4, cudaMemcpyDeviceToHost, s->stream));
  PBD_CUDA(cudaStreamSynchronize(s->stream));
  if (v == 0) return CWA_OK;
  PBD_CUDA(cudaMemsetAsync(s->d_status, 0, 4, s->stream));
  PBD_CUDA(cudaStreamSynchronize(s->stream));
  if (v & kStatusTimeout) return perr("a bounded device wait (scan look-back) timed out", CWA_ERR_TIMEOUT);
  if (v & kStatusNonFinite) return perr("non-finite box position", CWA_ERR_NONFINITE);
  return perr("a box overlapped more cells, or had more contacts, than its slots hold", CWA_ERR_CAPACITY);
}

}  // namespace

extern "C" {

cwa_status cwa_pbd_create(const cwa_pbd_params* p, int32_t device, cwa_pbd_sim** out) {
  if (!p || !out) return perr("null params or output");
  *out = nullptr;
  if (p->n_boxes < 1 || p->n_boxes > (1 << 22)) return perr("n_boxes must be in [1, 2^22]");
  for (int a = 0; a < 3; ++a) {
    if (p->grid_cells[a] < 1 || p->grid_cells[a] > 1024) return perr("grid_cells must be in [1, 1024]");
    if (!(p->extents_hi[a] > p->extents_lo[a])) return perr("extents must have hi > lo");
  }
  if (!(p->dt > 0.0f) || p->substeps < 0) return perr("dt must be positive and substeps >= 0");
  if (p->max_contacts < 0 || p->max_contacts > 4096) return perr("max_contacts must be in [0, 4096]");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return perr("no such CUDA device", CWA_ERR_NO_DEVICE);
  cwa_pbd_sim* s = new cwa_pbd_sim();
  s->device = device;
  s->prm = *p;
  PbdConst& k = s->k;
  k.n = p->n_boxes;
  k.nx = p->grid_cells[0];
  k.ny = p->grid_cells[1];
  k.nz = p->grid_cells[2];
  for (int a = 0; a < 3; ++a) {
    k.lo[a] = p->extents_lo[a];
    k.hi[a] = p->extents_hi[a];
    k.cell[a] = (k.hi[a] - k.lo[a]) / (float)p->grid_cells[a];  // mCellSize = extents / cells
    k.g[a] = p->g[a];
  }
  k.dt = p->dt;
  k.damping = p->damping;
  k.k = p->k;
  k.k_static = p->k_static;
  k.sleep = p->sleep_thresh;
  k.mu_k = p->mu_k;
  k.mu_s = p->mu_s;
  k.e = p->e;
  k.maxc = 8;
  k.pcap = p->max_contacts > 0 ? p->max_contacts : 64;
  s->ncells = k.nx * k.ny * k.nz;
  const size_t slots = (size_t)k.n * k.pcap;
  cudaError_t e = cudaSetDevice(device);
  auto al = [&](void** ptr, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(ptr, bytes > 0 ? bytes : 4);
  };
  al((void**)&s->boxes, sizeof(cwa_pbd_box) * k.n);
  al((void**)&s->ccount, 4 * (size_t)s->ncells);
  al((void**)&s->cstart, 4 * ((size_t)s->ncells + 1));
  al((void**)&s->pairs, sizeof(PbdPair) * slots);
  al((void**)&s->npairs, 4 * (size_t)k.n);
  al((void**)&s->rkey, 4 * slots);
  al((void**)&s->rslot, 4 * slots);
  al((void**)&s->rlist, 4 * slots);
  al((void**)&s->rsorted, 4 * slots);
  al((void**)&s->rcount, 4 * (size_t)k.n);
  al((void**)&s->rstart, 4 * ((size_t)k.n + 1));
  al(&s->ws_cells, scan_workspace_bytes(s->ncells + 1));
  al(&s->ws_rev, scan_workspace_bytes(k.n + 1));
  al((void**)&s->d_status, 4);
  if (e == cudaSuccess) e = cudaMemset(s->ccount, 0, 4 * (size_t)s->ncells);
  if (e == cudaSuccess) e = cudaMemset(s->rcount, 0, 4 * (size_t)k.n);
  if (e == cudaSuccess) e = cudaMemset(s->npairs, 0, 4 * (size_t)k.n);
  if (e == cudaSuccess) e = cudaMemset(s->d_status, 0, 4);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    cwa::set_error(std::string("cwa_pbd_create: ") + cudaGetErrorString(e));
    free_pbd(s);
    return e == cudaErrorMemoryAllocation ? CWA_ERR_OOM : CWA_ERR_CUDA;
  }
  scan_bind_workspace(s->ws_cells, s->ncells + 1, &s->scan_cells);
  scan_bind_workspace(s->ws_rev, k.n + 1, &s->scan_rev);
  *out = s;
  return CWA_OK;
}

cwa_status cwa_pbd_destroy(cwa_pbd_sim* s) {
  if (!s) return perr("null sim");
  free_pbd(s);
  return CWA_OK;
}

cwa_status cwa_pbd_upload(cwa_pbd_sim* s, const cwa_pbd_box* host, int32_t n) {
  if (!s) return perr("null sim");
  if (!host || n != s->k.n) return perr("upload size must equal n_boxes");
  PBD_CUDA(cudaSetDevice(s->device));
  // cells a box can overlap: per axis floor(2 hw / cell) + 2, over the largest box
  float hmax[3] = {0.0f, 0.0f, 0.0f};
  for (int i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      if (!(host[i].hw[a] >= 0.0f) || !isfinite(host[i].hw[a])) return perr("half widths must be finite, >= 0");
      hmax[a] = std::max(hmax[a], host[i].hw[a]);
    }
  long maxc = 1;
  const int dims[3] = {s->k.nx, s->k.ny, s->k.nz};
  for (int a = 0; a < 3; ++a)
    maxc *= std::min<long>(dims[a], (long)floorf(2.0f * hmax[a] / s->k.cell[a]) + 2);
  if (maxc * n > (1l << 30)) return perr("boxes too large for the grid", CWA_ERR_CAPACITY);
  if (s->graph) {
    cudaGraphExecDestroy(s->graph);
    s->graph = nullptr;
  }
  if (maxc != s->k.maxc || !s->ikey) {
    free_items(s);
    s->k.maxc = (int)maxc;
    const size_t items = (size_t)maxc * n;
    PBD_CUDA(cudaMalloc((void**)&s->ikey, 4 * items));
    PBD_CUDA(cudaMalloc((void**)&s->islot, 4 * items));
    PBD_CUDA(cudaMalloc((void**)&s->clist, 4 * items));
    PBD_CUDA(cudaMalloc((void**)&s->csorted, 4 * items));
  }
  PBD_CUDA(cudaMemcpyAsync(s->boxes, host, sizeof(cwa_pbd_box) * n, cudaMemcpyHostToDevice, s->stream));
  PBD_CUDA(cudaStreamSynchronize(s->stream));
  s->uploaded = true;
  return CWA_OK;
}

cwa_status cwa_pbd_download(cwa_pbd_sim* s, cwa_pbd_box* host, int32_t n) {
  if (!s) return perr("null sim");
  if (!host || n != s->k.n) return perr("download size must equal n_boxes");
  PBD_CUDA(cudaSetDevice(s->device));
  PBD_CUDA(cudaMemcpyAsync(host, s->boxes, sizeof(cwa_pbd_box) * n, cudaMemcpyDeviceToHost, s->stream));
  PBD_CUDA(cudaStreamSynchronize(s->stream));
  return read_pbd_status(s);
}

cwa_status cwa_pbd_step(cwa_pbd_sim* s, int32_t n_steps) {
  if (!s) return perr("null sim");
  if (n_steps < 0) return perr("n_steps < 0");
  if (!s->uploaded) return perr("upload boxes first (cwa_pbd_upload)");
  PBD_CUDA(cudaSetDevice(s->device));
  if (!s->graph && s->prm.substeps > 0) {
    cudaGraph_t g = nullptr;
    PBD_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    cwa_status st = CWA_OK;
    for (int sub = 0; sub < s->prm.substeps && st == CWA_OK; ++sub) st = enqueue_substep(s);
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (st != CWA_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    PBD_CUDA(e);
    e = cudaGraphInstantiate(&s->graph, g, 0);
    cudaGraphDestroy(g);
    PBD_CUDA(e);
  }
  for (int32_t k = 0; k < n_steps && s->graph; ++k) PBD_CUDA(cudaGraphLaunch(s->graph, s->stream));
  return CWA_OK;
}

cwa_status cwa_pbd_pair_count(cwa_pbd_sim* s, int64_t* pairs) {
  if (!s || !pairs) return perr("null sim or output");
  PBD_CUDA(cudaSetDevice(s->device));
  int32_t v = 0;
  PBD_CUDA(cudaMemcpyAsync(&v, s->rstart + s->k.n, 4, cudaMemcpyDeviceToHost, s->stream));
  PBD_CUDA(cudaStreamSynchronize(s->stream));
  *pairs = v;
  return read_pbd_status(s);
}

}  // extern "C"
