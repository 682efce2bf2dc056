// cwa_render.cu — one frame of the reference's display() (Main.cpp:326-474)
// rendered headless with CUDA kernels instead of GL.
//
// Primitives, in the reference's draw order:
//   * the wave surface: the indexed triangle-strip mesh of Surf.cpp:68-190
//     (WAVE_RES vertices per side; vertex (a, b) sits at
//     (int(0.1 a), -1, int(0.1 b)) because START_INDEX * i is passed to int
//     parameters), displaced to y = 50 * u(tex) by wave_vs.glsl:30-42 and
//     shaded by wave_fs.glsl:30-88;
//   * the particles: 8-pixel point sprites (particle_vs.glsl, particle_fs.glsl
//     pass 0), with the depth image of pass 2 (eye_pos.z of the nearest
//     sprite) giving screen-space normals.
//
// GB300 form: a tiled rasteriser.  Primitives are binned into 8 x 4 pixel
// tiles (count, scan, fill: the grid sort's pieces); one warp then owns a
// tile, lane = pixel.  The depth image is the nearest particle fragment, an
// order-free minimum over the tile's list.  The colour pass sorts the tile's
// list into draw order (in shared memory; long lists by a radix sort in
// global scratch) and replays GL_LESS with depth writes and SRC_ALPHA /
// ONE_MINUS_SRC_ALPHA blending into an 8-bit target per pixel, so the result
// follows GL's ordered blending, not just the nearest fragment.  Fragments
// that pass the depth test are queued and shaded 32 at a time.
// Coverage, depths and projections use round-to-nearest intrinsics in a
// fixed order (the CPU restatement repeats them bit for bit); shading uses
// the CUDA math library.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <vector>

#include "cwa_device.cuh"
#include "cwa_internal.h"

namespace cwa {

namespace {

__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }

struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(float k, V3 a) { return v3(k * a.x, k * a.y, k * a.z); }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 normalize(V3 a) { return rsqrtf(dot(a, a)) * a; }
__device__ __forceinline__ V3 reflect(V3 i, V3 n) { return i - (2.0f * dot(n, i)) * n; }
__device__ __forceinline__ V3 refract(V3 i, V3 n, float eta) {
  const float d = dot(n, i);
  const float k = 1.0f - eta * eta * (1.0f - d * d);
  if (k < 0.0f) return v3(0.0f, 0.0f, 0.0f);
  return eta * i - (eta * d + sqrtf(k)) * n;
}

// Projection with a fixed operation order: clip_r = ((m0 x + m1 y) + m2 z) + m3.
__device__ __forceinline__ float row4(const float* m, float x, float y, float z) {
  return fa(fa(fa(fm(m[0], x), fm(m[1], y)), fm(m[2], z)), m[3]);
}

struct Win {
  float x, y, z, w;  // window x, y (pixels), window depth in [0, 1], clip w
  float cz;          // clip z (the depth image's value)
  bool ok;           // inside the clip volume (points) / in front of the eye
};

__device__ __forceinline__ Win project(const float* mvp, float x, float y, float z, int W, int H, bool point) {
  Win o;
  const float cx = row4(mvp, x, y, z), cy = row4(mvp + 4, x, y, z), cz = row4(mvp + 8, x, y, z),
              cw = row4(mvp + 12, x, y, z);
  o.w = cw;
  o.cz = cz;
  o.ok = cw > 0.0f && cz >= -cw && cz <= cw;
  if (point) o.ok = o.ok && cx >= -cw && cx <= cw && cy >= -cw && cy <= cw;
  const float nx = fd(cx, cw), ny = fd(cy, cw), nz = fd(cz, cw);
  o.x = fm(fm(fa(nx, 1.0f), 0.5f), (float)W);
  o.y = fm(fm(fa(ny, 1.0f), 0.5f), (float)H);
  o.z = fm(fa(nz, 1.0f), 0.5f);
  return o;
}

// Sprite pixel range: centres c with wx - S/2 <= c < wx + S/2.
__device__ __forceinline__ void sprite_range(float c, float half, int n, int* lo, int* hi) {
  *lo = max((int)ceilf(fs(fs(c, half), 0.5f)), 0);
  *hi = min((int)ceilf(fs(fa(c, half), 0.5f)) - 1, n - 1);
}

// Squared sprite radius of pixel centre (px, py) in point-coordinate units.
__device__ __forceinline__ float sprite_r2(int px, int py, float wx, float wy, float inv_s) {
  const float dx = fm(fs(fa((float)px, 0.5f), wx), inv_s), dy = fm(fs(fa((float)py, 0.5f), wy), inv_s);
  return fa(fm(dx, dx), fm(dy, dy));
}

// ---- the strip mesh ------------------------------------------------------
// Row i of the strip holds vertices (i, j), (i+1, j) for j < n-1; its
// triangles are consecutive vertex triples, 2n - 4 per row.
__device__ __forceinline__ void tri_vertices(int t, int n, int va[3], int vb[3]) {
  const int per_row = 2 * n - 4;
  const int i = t / per_row, k0 = t - i * per_row;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const int k = k0 + q;
    va[q] = i + (k & 1);
    vb[q] = k >> 1;
  }
}

struct MeshVert {
  float wx, wy, wz, iw;  // window position, depth, 1 / clip w
  float s, t;            // texture coordinates
  float px, py, pz;      // world position of the undisplaced vertex (wave_vs pw)
  int ok;
};

}  // namespace

struct RenderFrame {
  float mvp_p[16], m_p[16];  // particles: PV * M and M (row-major)
  float mvp_w[16], m_w[16];  // wave surface
  float inv_p[16], inv_v[16];
  float eye[3];
  int W, H;
  float point_size;
  int res, n_tris, n_particles;
  int draw_surface, draw_particles, draw_skybox;
  const float* wave;
  int nx, nz;
  const float4* pos;
  const uint8_t* sky;
  int sky_size;
};

namespace {

// ---- cube map (GL cube-map face selection, GL_LINEAR, clamp within face) --
// One 4-byte load per RGBA8 texel (the cube map's base is cudaMalloc-aligned).
__device__ V3 cube_texel(const RenderFrame& f, int face, int x, int y) {
  const uchar4 p = __ldg(reinterpret_cast<const uchar4*>(f.sky) + (((size_t)face * f.sky_size + y) * f.sky_size + x));
  return v3(p.x / 255.0f, p.y / 255.0f, p.z / 255.0f);
}

__device__ V3 cube_sample(const RenderFrame& f, V3 r) {
  if (!f.sky) return v3(0.0f, 0.0f, 0.0f);
  const float ax = fabsf(r.x), ay = fabsf(r.y), az = fabsf(r.z);
  int face;
  float sc, tc, ma;
  if (ax >= ay && ax >= az) {
    face = r.x >= 0.0f ? 0 : 1;
    sc = r.x >= 0.0f ? -r.z : r.z;
    tc = -r.y;
    ma = ax;
  } else if (ay >= az) {
    face = r.y >= 0.0f ? 2 : 3;
    sc = r.x;
    tc = r.y >= 0.0f ? r.z : -r.z;
    ma = ay;
  } else {
    face = r.z >= 0.0f ? 4 : 5;
    sc = r.z >= 0.0f ? r.x : -r.x;
    tc = -r.y;
    ma = az;
  }
  if (ma == 0.0f) return cube_texel(f, 0, f.sky_size / 2, f.sky_size / 2);
  const float s = 0.5f * (sc / ma + 1.0f), t = 0.5f * (tc / ma + 1.0f);
  const float u = s * f.sky_size - 0.5f, v = t * f.sky_size - 0.5f;
  const float u0 = floorf(u), v0 = floorf(v);
  const float au = u - u0, av = v - v0;
  const int n1 = f.sky_size - 1;
  const int x0 = min(max((int)u0, 0), n1), x1 = min(max((int)u0 + 1, 0), n1);
  const int y0 = min(max((int)v0, 0), n1), y1 = min(max((int)v0 + 1, 0), n1);
  const V3 c00 = cube_texel(f, face, x0, y0), c10 = cube_texel(f, face, x1, y0);
  const V3 c01 = cube_texel(f, face, x0, y1), c11 = cube_texel(f, face, x1, y1);
  return (1.0f - av) * ((1.0f - au) * c00 + au * c10) + av * ((1.0f - au) * c01 + au * c11);
}

__device__ __forceinline__ MeshVert mesh_vertex(const RenderFrame& f, int a, int b) {
  MeshVert m;
  const float fx = (float)(int)fm(0.1f, (float)a), fz = (float)(int)fm(0.1f, (float)b);
  m.s = fd((float)a, (float)(f.res - 1));
  m.t = fd((float)b, (float)(f.res - 1));
  const float h = sample_height(f.wave, f.nx, f.nz, m.s, m.t);
  const Win w = project(f.mvp_w, fx, fm(50.0f, h), fz, f.W, f.H, false);
  m.wx = w.x;
  m.wy = w.y;
  m.wz = w.z;
  m.iw = fd(1.0f, w.w);
  m.ok = w.ok;
  m.px = row4(f.m_w, fx, -1.0f, fz);
  m.py = row4(f.m_w + 4, fx, -1.0f, fz);
  m.pz = row4(f.m_w + 8, fx, -1.0f, fz);
  return m;
}

__device__ __forceinline__ float edge(float ax, float ay, float bx, float by, float px, float py) {
  return fs(fm(fs(bx, ax), fs(py, ay)), fm(fs(by, ay), fs(px, ax)));
}

// Pixel-centre coverage of a CCW-normalised triangle with the top-left rule.
__device__ __forceinline__ bool top_left(float ax, float ay, float bx, float by) {
  return (ay == by && bx < ax) || (by < ay);
}

struct TriSetup {
  float x[3], y[3];
  int order[3];  // mesh vertex slot of each CCW-normalised corner
  float area;
  int x0, x1, y0, y1;
  bool ok;
};

__device__ TriSetup tri_setup(const MeshVert* mv, int t, int W, int H) {
  TriSetup s;
  int o[3] = {0, 1, 2};
  float x[3] = {mv[0].wx, mv[1].wx, mv[2].wx}, y[3] = {mv[0].wy, mv[1].wy, mv[2].wy};
  float area = edge(x[0], y[0], x[1], y[1], x[2], y[2]);
  s.ok = mv[0].ok && mv[1].ok && mv[2].ok && area != 0.0f;
  if (area < 0.0f) {  // make it counter-clockwise: swap corners 1 and 2
    o[1] = 2;
    o[2] = 1;
    area = -area;
  }
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    s.x[q] = x[o[q]];
    s.y[q] = y[o[q]];
    s.order[q] = o[q];
  }
  s.area = area;
  const float minx = fminf(fminf(s.x[0], s.x[1]), s.x[2]), maxx = fmaxf(fmaxf(s.x[0], s.x[1]), s.x[2]);
  const float miny = fminf(fminf(s.y[0], s.y[1]), s.y[2]), maxy = fmaxf(fmaxf(s.y[0], s.y[1]), s.y[2]);
  s.x0 = max((int)floorf(minx - 0.5f), 0);
  s.x1 = min((int)ceilf(maxx - 0.5f), W - 1);
  s.y0 = max((int)floorf(miny - 0.5f), 0);
  s.y1 = min((int)ceilf(maxy - 0.5f), H - 1);
  if (s.x0 > s.x1 || s.y0 > s.y1) s.ok = false;
  return s;
}

// Barycentric weights (of the CCW corners x, y) of pixel (px, py), or false.
__device__ __forceinline__ bool tri_cover(const float* x, const float* y, float area, int px, int py,
                                          float l[3]) {
  const float cx = fa((float)px, 0.5f), cy = fa((float)py, 0.5f);
  const float e0 = edge(x[1], y[1], x[2], y[2], cx, cy);
  const float e1 = edge(x[2], y[2], x[0], y[0], cx, cy);
  const float e2 = edge(x[0], y[0], x[1], y[1], cx, cy);
  const bool in0 = e0 > 0.0f || (e0 == 0.0f && top_left(x[1], y[1], x[2], y[2]));
  const bool in1 = e1 > 0.0f || (e1 == 0.0f && top_left(x[2], y[2], x[0], y[0]));
  const bool in2 = e2 > 0.0f || (e2 == 0.0f && top_left(x[0], y[0], x[1], y[1]));
  if (!(in0 && in1 && in2)) return false;
  l[0] = fd(e0, area);
  l[1] = fd(e1, area);
  l[2] = fd(e2, area);
  return true;
}

__device__ __forceinline__ bool tri_cover(const TriSetup& s, int px, int py, float l[3]) {
  return tri_cover(s.x, s.y, s.area, px, py, l);
}

__device__ __forceinline__ void load_tri(const RenderFrame& f, const MeshVert* verts, int t, MeshVert mv[3]) {
  int va[3], vb[3];
  tri_vertices(t, f.res, va, vb);
#pragma unroll
  for (int q = 0; q < 3; ++q) mv[q] = verts[(size_t)va[q] * f.res + vb[q]];
}

// ---- kernels --------------------------------------------------------------
// The sim keeps particles cell-sorted; the reference draws its SSBO in
// upload order, which is what the blending order follows.
__global__ void k_upload_order(const float4* __restrict__ sorted, const int32_t* __restrict__ id, int n,
                               float4* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[id[k]] = sorted[k];
}

__global__ void k_mesh_vertices(RenderFrame f, MeshVert* __restrict__ verts) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= f.res * f.res) return;
  verts[v] = mesh_vertex(f, v / f.res, v % f.res);
}

// ---- tiled rasteriser ---------------------------------------------------------
// The screen is cut into 8 x 4 pixel tiles, one warp each: lane l owns pixel
// (l & 7, l >> 3) of its tile.  Every primitive is binned into each tile its
// pixel bounds touch; a tile's warp then tests its 32 pixels against the
// tile's primitives.  The depth image only needs the nearest particle, so its
// walk takes the list in any order; the colour walk sorts the list into draw
// order first and replays the depth test and blending per pixel, as GL does.
constexpr int kTileW = 8, kTileH = 4;
constexpr int kTileWarps = 4;     // tiles per block
constexpr int kTileCap = 512;     // longer tile lists are sorted in global memory
constexpr int kHaloW = kTileW + 2, kHaloH = kTileH + 2;  // a tile's depth image with a one-pixel border

enum : int { kPrimNone = 0, kPrimTri = 1, kPrimSprite = 2 };

// A primitive's coverage set-up (64 bytes, staged in shared memory).
struct __align__(16) PrimSetup {
  float x[3], y[3];  // triangle: CCW corners; sprite: centre x[0], y[0], position x[1], x[2], y[1]
  float area;        // triangle: twice the area; sprite: 1 / point size
  float z[3];        // triangle: window depth of each corner; sprite: z[0] depth, z[1] clip z
  int x0, x1, y0, y1;  // pixel bounds, inclusive, on screen
  int type;
  uint32_t prim;
};

// Primitive p: triangles first (p < n_tri), then the particles in upload order.
__device__ PrimSetup prim_setup(const RenderFrame& f, const MeshVert* __restrict__ verts, uint32_t p, int n_tri) {
  PrimSetup s;
  s.type = kPrimNone;
  s.prim = p;
  if ((int)p < n_tri) {
    MeshVert mv[3];
    load_tri(f, verts, (int)p, mv);
    const TriSetup t = tri_setup(mv, (int)p, f.W, f.H);
    if (!t.ok) return s;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      s.x[q] = t.x[q];
      s.y[q] = t.y[q];
      s.z[q] = mv[t.order[q]].wz;
    }
    s.area = t.area;
    s.x0 = t.x0;
    s.x1 = t.x1;
    s.y0 = t.y0;
    s.y1 = t.y1;
    s.type = kPrimTri;
  } else {
    const float4 q = f.pos[p - n_tri];
    const Win w = project(f.mvp_p, q.x, q.y, q.z, f.W, f.H, true);
    if (!w.ok) return s;
    const float half = 0.5f * f.point_size;
    sprite_range(w.x, half, f.W, &s.x0, &s.x1);
    sprite_range(w.y, half, f.H, &s.y0, &s.y1);
    if (s.x0 > s.x1 || s.y0 > s.y1) return s;
    s.x[0] = w.x;
    s.y[0] = w.y;
    s.z[0] = w.z;
    s.z[1] = w.cz;
    s.x[1] = q.x;  // the position, for the shading
    s.x[2] = q.y;
    s.y[1] = q.z;
    s.area = fd(1.0f, f.point_size);
    s.type = kPrimSprite;
  }
  return s;
}

// Window depth of s's fragment at pixel (px, py), or false where s does not
// cover the pixel centre.
__device__ __forceinline__ bool prim_fragment(const PrimSetup& s, int px, int py, float* z) {
  if (px < s.x0 || px > s.x1 || py < s.y0 || py > s.y1) return false;
  if (s.type == kPrimSprite) {
    if (!(sprite_r2(px, py, s.x[0], s.y[0], s.area) < 0.25f)) return false;  // r >= 0.5 is discarded
    *z = s.z[0];
    return true;
  }
  float l[3];
  if (!tri_cover(s.x, s.y, s.area, px, py, l)) return false;
  *z = fa(fa(fm(l[0], s.z[0]), fm(l[1], s.z[1])), fm(l[2], s.z[2]));
  return true;
}

// Counts (pairs == nullptr) or fills each tile's primitive list.
__global__ void k_bin(RenderFrame f, const MeshVert* __restrict__ verts, int n_tri, int n_prim, int tiles_x,
                      int32_t* __restrict__ cnt, const int32_t* __restrict__ off, uint32_t* __restrict__ pairs,
                      int32_t* __restrict__ status) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_prim) return;
  const PrimSetup s = prim_setup(f, verts, (uint32_t)p, n_tri);
  if (s.type == kPrimNone) return;
  const int tx0 = s.x0 / kTileW, tx1 = s.x1 / kTileW, ty0 = s.y0 / kTileH, ty1 = s.y1 / kTileH;
  for (int ty = ty0; ty <= ty1; ++ty)
    for (int tx = tx0; tx <= tx1; ++tx) {
      const int t = ty * tiles_x + tx;
      const int slot = atomicAdd(cnt + t, 1);
      if (pairs) {
        const int k = off[t] + slot;
        if (CWA_DCHECK_FAILED(k < off[t + 1], status)) continue;
        pairs[k] = (uint32_t)p;
      }
    }
}

// Ascending bitonic sort of a[0, m) by one warp (m a power of two).
__device__ void warp_bitonic(uint32_t* a, int m, int lane) {
  for (int k = 2; k <= m; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int c = lane; c < (m >> 1); c += 32) {
        const int i = ((c & ~(j - 1)) << 1) | (c & (j - 1)), l = i + j;
        const uint32_t x = a[i], y = a[l];
        if ((x > y) == ((i & k) == 0)) {
          a[i] = y;
          a[l] = x;
        }
      }
      __syncwarp();
    }
}

// Stable LSD radix sort (8-bit digits) of a[0, n) by one warp, through
// tmp[0, n); hist holds 256 counters.  Returns the buffer holding the result.
__device__ const uint32_t* warp_radix(uint32_t* a, uint32_t* tmp, int n, int bits, uint32_t* hist, int lane,
                                      int32_t* status) {
  uint32_t *src = a, *dst = tmp;
  for (int shift = 0; shift < bits; shift += 8) {
    for (int d = lane; d < 256; d += 32) hist[d] = 0;
    __syncwarp();
    for (int i = lane; i < n; i += 32) atomicAdd(&hist[(src[i] >> shift) & 255u], 1u);
    __syncwarp();
    uint32_t v[8], sum = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      v[q] = hist[lane * 8 + q];
      sum += v[q];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    uint32_t run = incl - sum;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      hist[lane * 8 + q] = run;
      run += v[q];
    }
    __syncwarp();
    for (int base = 0; base < n; base += 32) {
      const int i = base + lane;
      const bool valid = i < n;
      uint32_t x = 0, dg = 256u + (uint32_t)lane;  // lanes past the end never match a digit
      if (valid) {
        x = src[i];
        dg = (x >> shift) & 255u;
      }
      const unsigned peers = __match_any_sync(0xffffffffu, dg);
      const int rank = __popc(peers & ((1u << lane) - 1u));
      uint32_t pos = 0;
      if (valid) pos = hist[dg] + (uint32_t)rank;
      __syncwarp();
      if (valid) {
        if (!CWA_DCHECK_FAILED(pos < (uint32_t)n, status)) dst[pos] = x;
        if (rank == 0) hist[dg] += (uint32_t)__popc(peers);
      }
      __syncwarp();
    }
    uint32_t* t = src;
    src = dst;
    dst = t;
  }
  return src;
}

// The depth image of pass 2: eye_pos.z (clip z) of the particle fragment
// that wins GL_LESS, the first drawn among equal depths (0 where none).
// A sprite's set-up as the depth walk needs it (32 bytes): window position
// and depth, particle index, pixel bounds (empty for anything else).
struct __align__(16) SpriteStage {
  float wx, wy, z;
  uint32_t i;
  int x0, x1, y0, y1;
};

__global__ void __launch_bounds__(kTileWarps * 32)
    k_tile_depth(RenderFrame f, int n_tri, int tiles_x, int n_tiles, const int32_t* __restrict__ off,
                 const uint32_t* __restrict__ pairs, float* __restrict__ depth_img, int32_t* __restrict__ status) {
  __shared__ SpriteStage stage[kTileWarps][32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = blockIdx.x * kTileWarps + w;
  if (t >= n_tiles) return;
  const int px = (t % tiles_x) * kTileW + (lane & 7), py = (t / tiles_x) * kTileH + (lane >> 3);
  const float inv_s = fd(1.0f, f.point_size);
  const uint64_t none = (uint64_t)__float_as_uint(1.0f) << 32;
  uint64_t best = none;  // (depth bits, particle): window depths are in [0, 1]
  const int b = off[t], e = off[t + 1];
  for (int base = b; base < e; base += 32) {
    SpriteStage g = {0.0f, 0.0f, 0.0f, 0u, 1, 0, 1, 0};  // empty bounds: covers nothing
    if (base + lane < e) {
      const uint32_t p = pairs[base + lane];
      if ((int)p >= n_tri) {
        const PrimSetup s = prim_setup(f, nullptr, p, n_tri);
        if (s.type == kPrimSprite)
          g = SpriteStage{s.x[0], s.y[0], s.z[0], p - (uint32_t)n_tri, s.x0, s.x1, s.y0, s.y1};
      }
    }
    stage[w][lane] = g;
    __syncwarp();
    const int m = min(32, e - base);
    for (int j = 0; j < m; ++j) {
      const SpriteStage q = stage[w][j];  // two 16-byte loads
      if (px < q.x0 || px > q.x1 || py < q.y0 || py > q.y1) continue;
      if (!(sprite_r2(px, py, q.wx, q.wy, inv_s) < 0.25f)) continue;  // r >= 0.5 is discarded
      const uint64_t key = ((uint64_t)__float_as_uint(q.z) << 32) | q.i;
      best = key < best ? key : best;
    }
    __syncwarp();
  }
  if (px >= f.W || py >= f.H) return;
  float d = 0.0f;
  if (best < none && !CWA_DCHECK_FAILED((uint32_t)best < (uint32_t)f.n_particles, status)) {
    const float4 q = f.pos[(uint32_t)best];
    d = project(f.mvp_p, q.x, q.y, q.z, f.W, f.H, true).cz;
  }
  depth_img[py * f.W + px] = d;
}

__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }

__device__ __forceinline__ V3 mat3x(const float* m, V3 v, float w) {
  return v3(m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * w, m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * w,
            m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * w);
}

// wave_fs.glsl:30-88 for the fragment of triangle t at pixel (px, py).
__device__ void shade_surface(const RenderFrame& f, const MeshVert* verts, int t, int px, int py, V3* rgb,
                              float* alpha) {
  MeshVert mv[3];
  load_tri(f, verts, t, mv);
  const TriSetup s = tri_setup(mv, t, f.W, f.H);
  float l[3];
  tri_cover(s, px, py, l);
  // perspective-correct varyings
  float q[3], sum = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    q[k] = l[k] * mv[s.order[k]].iw;
    sum += q[k];
  }
  float ts = 0.0f, tt = 0.0f;
  V3 pw = v3(0.0f, 0.0f, 0.0f);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const MeshVert& m = mv[s.order[k]];
    const float wgt = q[k] / sum;
    ts += wgt * m.s;
    tt += wgt * m.t;
    pw = pw + wgt * v3(m.px, m.py, m.pz);
  }
  const float v = sample_height(f.wave, f.nx, f.nz, ts, tt);
  const V3 eye = v3(f.eye[0], f.eye[1], f.eye[2]);
  const V3 n = v3(0.0f, 1.0f, 0.0f);  // -normal_attrib of the flat strip mesh, normalised
  const V3 i = normalize(pw - eye);
  const V3 refl = cube_sample(f, reflect(i, n));
  const V3 refr = cube_sample(f, refract(i, n, 1.0f / 1.33f));
  const V3 light_col = v3(1.0f, 0.85f, 0.7f);
  const V3 light_dir = normalize(v3(0.0f, 1.0f, 0.0f) - pw);
  const float diff = fmaxf(dot(n, light_dir), 0.0f);
  const V3 view_dir = normalize(eye - pw);
  const V3 rdir = reflect(v3(-light_dir.x, -light_dir.y, -light_dir.z), n);
  const float spec = powf(fmaxf(dot(view_dir, rdir), 0.0f), 32.0f);
  const V3 lit = (0.8f * light_col + diff * light_col + (10.0f * spec) * light_col) * v3(0.6f, 0.8f, 1.0f);
  const V3 combine = 0.75f * (refl + refr) + 0.1f * lit;
  *rgb = v3(mixf(combine.x, 0.7f, v), mixf(combine.y, 0.9f, v), mixf(combine.z, 1.0f, v));
  *alpha = mixf(0.2f, 0.0f, v);
}

// particle_fs.glsl pass 0 for particle i at pixel (px, py).
// particle_fs.glsl pass 0 splits into terms of the pixel alone, which come
// from the depth image (the normal of GetNormalFromDepth and lighting() at
// WorldPosFromDepth), and terms of the particle.
//
// The pixel's terms.  sd is the depth image around the pixel's tile (a
// one-pixel halo, kHaloW floats a row, 0 off screen) and (hx, hy) the
// pixel's place in it.
__device__ void particle_pixel_terms(const RenderFrame& f, const float* sd, int hx, int hy, int px, int py,
                                     V3* n_out, V3* lit_out) {
  const V3 eye = v3(f.eye[0], f.eye[1], f.eye[2]);
  // GetNormalFromDepth
  const float* d = sd + hy * kHaloW + hx;
  const float dzdx = 0.5f * (d[1] - d[-1]);
  const float dzdy = 0.5f * (d[kHaloW] - d[-kHaloW]);
  const V3 n = normalize(v3(-dzdx, -dzdy, 1.0f));
  // lighting() with WorldPosFromDepth (gl_FragCoord * 2 - 1, as the shader writes it)
  const float dz = d[0];
  const float cx = (px + 0.5f) * 2.0f - 1.0f, cy = (py + 0.5f) * 2.0f - 1.0f, cz = dz * 2.0f - 1.0f;
  float vw = f.inv_p[12] * cx + f.inv_p[13] * cy + f.inv_p[14] * cz + f.inv_p[15];
  V3 view = mat3x(f.inv_p, v3(cx, cy, cz), 1.0f);
  view = (1.0f / vw) * view;
  const V3 pos = mat3x(f.inv_v, view, 1.0f);
  const V3 light_col = v3(1.0f, 0.85f, 0.7f);
  const V3 light_dir = normalize(v3(1.0f, 1.0f, 0.0f) - pos);
  const float diff = fmaxf(dot(n, light_dir), 0.0f);
  const V3 view_dir = normalize(eye - pos);
  const V3 rdir = reflect(v3(-light_dir.x, -light_dir.y, -light_dir.z), n);
  const float spec2 = powf(fmaxf(dot(view_dir, rdir), 0.0f), 32.0f);
  *n_out = n;
  *lit_out = (0.8f * light_col + diff * light_col + (0.9f * spec2) * light_col) * v3(0.4f, 0.7f, 1.0f);
}

// The particle's terms and the fragment's colour: q is the particle's
// position, (wx, wy) its window position, n and lit the pixel's terms.
__device__ void shade_particle(const RenderFrame& f, V3 n, V3 lit, float3 q, int px, int py, float wx, float wy,
                               float inv_s, V3* rgb, float* alpha) {
  const float r = sqrtf(sprite_r2(px, py, wx, wy, inv_s));
  const V3 pp = v3(row4(f.m_p, q.x, q.y, q.z), row4(f.m_p + 4, q.x, q.y, q.z), row4(f.m_p + 8, q.x, q.y, q.z));
  const V3 eye = v3(f.eye[0], f.eye[1], f.eye[2]);
  const float spec = powf(fmaxf(dot(normalize(pp), normalize(v3(1.0f, 1.0f, 0.0f))), 0.0f), 16.0f);
  const float a = expf(-12.0f * r) + 0.1f * expf(-2.0f * r);
  const V3 iv = normalize(eye - pp);
  const V3 refl = cube_sample(f, reflect(iv, n));
  const V3 refr = cube_sample(f, refract(iv, n, 1.0f / 1.33f));
  const V3 combine = 0.75f * (refl + refr) + 0.1f * lit;
  const float t = 2.0f * pp.y;
  *rgb = v3(mixf(combine.x, 1.0f, t) + spec, mixf(combine.y, 1.0f, t) + spec, mixf(combine.z, 1.0f, t) + spec);
  *alpha = mixf(0.1f, a, t);
}

__device__ __forceinline__ float unorm8(float x) { return floorf(fminf(fmaxf(x, 0.0f), 1.0f) * 255.0f + 0.5f); }

// SRC_ALPHA / ONE_MINUS_SRC_ALPHA into an 8-bit target: c is the 8-bit
// value, va = clamp(src) * clamp(alpha), oma = 1 - clamp(alpha) and
// div255[k] = k / 255 (the division, tabulated).  Every term is
// non-negative, so unorm8's lower clamp never acts and is left out; the
// floor and the conversion are one rounding-down conversion.
__device__ __forceinline__ int blend_channel(int c, float va, float oma, const float* div255) {
  return __float2int_rd(fminf(va + div255[c] * oma, 1.0f) * 255.0f + 0.5f);
}

// The colour pass: the tile's list sorted into draw order, each pixel's
// fragments through GL_LESS (depth writes on) and SRC_ALPHA /
// ONE_MINUS_SRC_ALPHA blending into an 8-bit target.  Fragments that pass
// the depth test are queued per warp (a 64-entry ring) and shaded 32 at a
// time, one per lane; each pixel's owner lane then blends that pixel's
// fragments into its colour in rounds, in queue order, which is draw order.
__global__ void __launch_bounds__(kTileWarps * 32, 7)
    k_tile_color(RenderFrame f, const MeshVert* __restrict__ verts, int n_tri, int tiles_x, int n_tiles,
                 const int32_t* __restrict__ off, uint32_t* __restrict__ pairs, int32_t n_pairs, int sort_bits,
                 const float* __restrict__ dimg, uint8_t* __restrict__ out, int32_t* __restrict__ status) {
  __shared__ uint32_t s_list[kTileWarps][kTileCap];
  __shared__ PrimSetup stage[kTileWarps][32];
  __shared__ uint32_t q_prim[kTileWarps][64];
  __shared__ int32_t q_lane[kTileWarps][64];
  __shared__ uint32_t s_mask[kTileWarps][32];  // per pixel: the flush's entries for it
  __shared__ float4 q_win[kTileWarps][64];   // sprites: window x, y and position x, y
  __shared__ float q_pz[kTileWarps][64];      // and position z
  __shared__ float s_depth[kTileWarps][kHaloW * kHaloH];
  __shared__ float s_px[kTileWarps][6][32];  // each pixel's particle terms: normal, lighting
  __shared__ float div255[256];
  for (int k = threadIdx.x; k < 256; k += blockDim.x) div255[k] = (float)k / 255.0f;
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = blockIdx.x * kTileWarps + w;
  if (t >= n_tiles) return;
  const int tx0 = (t % tiles_x) * kTileW, ty0 = (t / tiles_x) * kTileH;
  const int px = tx0 + (lane & 7), py = ty0 + (lane >> 3);
  const bool inside = px < f.W && py < f.H;
  const float inv_s = fd(1.0f, f.point_size);
  for (int k = lane; k < kHaloW * kHaloH; k += 32) {
    const int x = tx0 - 1 + k % kHaloW, y = ty0 - 1 + k / kHaloW;
    s_depth[w][k] = (x < 0 || y < 0 || x >= f.W || y >= f.H) ? 0.0f : dimg[y * f.W + x];
  }
  __syncwarp();
  if (f.draw_particles) {
    V3 n, lit;
    particle_pixel_terms(f, s_depth[w], (lane & 7) + 1, (lane >> 3) + 1, px, py, &n, &lit);
    s_px[w][0][lane] = n.x;
    s_px[w][1][lane] = n.y;
    s_px[w][2][lane] = n.z;
    s_px[w][3][lane] = lit.x;
    s_px[w][4][lane] = lit.y;
    s_px[w][5][lane] = lit.z;
  }
  // the colour target holds 8-bit values between blends
  int c[3] = {0, 0, 0};
  {
    if (f.draw_skybox && inside) {
      // view ray through the pixel centre: inverse(V) * inverse(P) * ndc
      const float nx = (px + 0.5f) / f.W * 2.0f - 1.0f, ny = (py + 0.5f) / f.H * 2.0f - 1.0f;
      const float vw = f.inv_p[12] * nx + f.inv_p[13] * ny + f.inv_p[14] + f.inv_p[15];
      V3 view = mat3x(f.inv_p, v3(nx, ny, 1.0f), 1.0f);
      view = (1.0f / vw) * view;
      const V3 dir = mat3x(f.inv_v, view, 0.0f);
      const V3 sky = cube_sample(f, dir);
      c[0] = (int)unorm8(sky.x);
      c[1] = (int)unorm8(sky.y);
      c[2] = (int)unorm8(sky.z);
    }
  }
  const int b = off[t], n = off[t + 1] - b;
  const uint32_t* list;
  if (n <= kTileCap) {
    int m = 1;
    while (m < n) m <<= 1;
    for (int i = lane; i < m; i += 32) s_list[w][i] = i < n ? pairs[b + i] : 0xffffffffu;
    __syncwarp();
    warp_bitonic(s_list[w], m, lane);
    list = s_list[w];
  } else {  // the second half of the pair buffer is this list's scratch
    list = warp_radix(pairs + b, pairs + n_pairs + b, n, sort_bits, s_list[w], lane, status);
  }
  float depth = 1.0f;
  int qh = 0, qn = 0;  // the queue's head and length (warp-uniform)
  auto flush = [&](int cnt) {
    __syncwarp();
    const bool mine = lane < cnt;
    const int qe = (qh + lane) & 63;
    const uint32_t p = mine ? q_prim[w][qe] : 0u;
    const int ql = mine ? q_lane[w][qe] : 32 + lane;  // lanes without an entry match nobody
    V3 rgb = v3(0.0f, 0.0f, 0.0f);
    float a = 0.0f;
    if (mine) {
      const int qx = tx0 + (ql & 7), qy = ty0 + (ql >> 3);
      if ((int)p < n_tri)
        shade_surface(f, verts, (int)p, qx, qy, &rgb, &a);
      else
      {
        const float4 v = q_win[w][qe];
        const float* pt = &s_px[w][0][ql];
        shade_particle(f, v3(pt[0], pt[32], pt[64]), v3(pt[96], pt[128], pt[160]),
                       make_float3(v.z, v.w, q_pz[w][qe]), qx, qy, v.x, v.y, inv_s, &rgb, &a);
      }
    }
    // premultiplied source terms, then each pixel's owner lane blends its
    // entries in queue order, one per round
    a = fminf(fmaxf(a, 0.0f), 1.0f);
    const float va0 = fminf(fmaxf(rgb.x, 0.0f), 1.0f) * a, va1 = fminf(fmaxf(rgb.y, 0.0f), 1.0f) * a,
                va2 = fminf(fmaxf(rgb.z, 0.0f), 1.0f) * a, oma = 1.0f - a;
    s_mask[w][lane] = 0u;
    __syncwarp();
    const unsigned peers = __match_any_sync(0xffffffffu, ql);
    if (mine && (peers & ((1u << lane) - 1u)) == 0u) s_mask[w][ql] = peers;
    __syncwarp();
    unsigned todo = s_mask[w][lane];
    const int rounds = (int)__reduce_max_sync(0xffffffffu, (unsigned)__popc(todo));
    for (int r = 0; r < rounds; ++r) {
      const int e = todo ? __ffs((int)todo) - 1 : lane;
      const float s0 = __shfl_sync(0xffffffffu, va0, e), s1 = __shfl_sync(0xffffffffu, va1, e),
                  s2 = __shfl_sync(0xffffffffu, va2, e), so = __shfl_sync(0xffffffffu, oma, e);
      if (todo) {
        c[0] = blend_channel(c[0], s0, so, div255);
        c[1] = blend_channel(c[1], s1, so, div255);
        c[2] = blend_channel(c[2], s2, so, div255);
        todo &= todo - 1u;
      }
    }
    __syncwarp();  // the ring's slots are free for new entries
    qh = (qh + cnt) & 63;
    qn -= cnt;
  };
  for (int base = 0; base < n; base += 32) {
    PrimSetup s;
    s.type = kPrimNone;
    if (base + lane < n) {
      const uint32_t p = list[base + lane];
      if (!CWA_DCHECK_FAILED(p < (uint32_t)n_tri + (f.draw_particles ? (uint32_t)f.n_particles : 0u), status))
        s = prim_setup(f, verts, p, n_tri);
    }
    stage[w][lane] = s;
    __syncwarp();
    const int m = min(32, n - base);
    for (int j = 0; j < m; ++j) {
      const PrimSetup q = stage[w][j];  // one 64-byte copy: the loads issue together
      if (q.type == kPrimNone) continue;
      float z;
      const bool pass = prim_fragment(q, px, py, &z) && z < depth;  // GL_LESS
      if (pass) depth = z;
      const unsigned bal = __ballot_sync(0xffffffffu, pass);
      if (bal) {
        if (pass) {
          const int slot = (qh + qn + __popc(bal & ((1u << lane) - 1u))) & 63;
          q_prim[w][slot] = q.prim;
          q_lane[w][slot] = lane;
          q_win[w][slot] = make_float4(q.x[0], q.y[0], q.x[1], q.x[2]);  // sprites only
          q_pz[w][slot] = q.y[1];
        }
        qn += __popc(bal);
        if (qn >= 32) flush(32);
      }
    }
    __syncwarp();
  }
  while (qn > 0) flush(min(qn, 32));
  __syncwarp();
  if (!inside) return;
  uchar4 o;
  o.x = (uint8_t)c[0];
  o.y = (uint8_t)c[1];
  o.z = (uint8_t)c[2];
  o.w = 255;
  reinterpret_cast<uchar4*>(out)[py * f.W + px] = o;
}

}  // namespace

// ---- host side --------------------------------------------------------------

struct RenderState {
  uint8_t* sky = nullptr;
  int sky_size = 0;
  // per-frame work buffers, kept between frames and grown on demand
  struct Buf {
    void* p = nullptr;
    size_t cap = 0;
  };
  Buf verts, upos, cnt, off, pairs, dimg, img, ws;
};

namespace {
cudaError_t ensure(RenderState::Buf& b, size_t bytes, size_t slack_div = 0) {
  if (b.p && bytes <= b.cap) return cudaSuccess;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  size_t want = bytes > 16 ? bytes : 16;
  if (slack_div) want += want / slack_div;
  if (debug_alloc_should_fail()) return cudaErrorMemoryAllocation;
  const cudaError_t e = cudaMalloc(&b.p, want);
  if (e == cudaSuccess) b.cap = want;
  return e;
}
}  // namespace

RenderState* render_state_new() { return new RenderState(); }

void render_state_free(RenderState* r) {
  if (!r) return;
  if (r->sky) cudaFree(r->sky);
  for (RenderState::Buf* b : {&r->verts, &r->upos, &r->cnt, &r->off, &r->pairs, &r->dimg, &r->img, &r->ws})
    if (b->p) cudaFree(b->p);
  delete r;
}

cudaError_t render_set_skybox(RenderState* r, const uint8_t* faces, int size, cudaStream_t stream) {
  if (r->sky) {
    cudaFree(r->sky);
    r->sky = nullptr;
    r->sky_size = 0;
  }
  const size_t bytes = (size_t)6 * size * size * 4;
  if (debug_alloc_should_fail()) return cudaErrorMemoryAllocation;
  cudaError_t e = cudaMalloc((void**)&r->sky, bytes);
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(r->sky, faces, bytes, cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e == cudaSuccess) r->sky_size = size;
  return e;
}

// glm's float formulas (lookAt, perspective, rotate, scale, mat4 product),
// column-major as glm stores them, in glm's operation order.
namespace {
struct F3 {
  float x, y, z;
};
F3 f3sub(F3 a, F3 b) { return F3{a.x - b.x, a.y - b.y, a.z - b.z}; }
float f3dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
F3 f3norm(F3 v) {
  const float inv = 1.0f / sqrtf(f3dot(v, v));
  return F3{v.x * inv, v.y * inv, v.z * inv};
}
F3 f3cross(F3 a, F3 b) { return F3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }

struct M4 {
  float c[4][4];  // c[column][row]
};
M4 m4_zero() {
  M4 m;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) m.c[i][j] = 0.0f;
  return m;
}
M4 m4_identity() {
  M4 m = m4_zero();
  for (int i = 0; i < 4; ++i) m.c[i][i] = 1.0f;
  return m;
}
M4 m4_mul(const M4& a, const M4& b) {
  M4 r;
  for (int j = 0; j < 4; ++j)
    for (int row = 0; row < 4; ++row)
      r.c[j][row] = ((a.c[0][row] * b.c[j][0] + a.c[1][row] * b.c[j][1]) + a.c[2][row] * b.c[j][2]) +
                    a.c[3][row] * b.c[j][3];
  return r;
}
M4 look_at(F3 eye, F3 center, F3 up) {
  const F3 f = f3norm(f3sub(center, eye));
  const F3 s = f3norm(f3cross(f, up));
  const F3 u = f3cross(s, f);
  M4 r = m4_identity();
  r.c[0][0] = s.x;
  r.c[1][0] = s.y;
  r.c[2][0] = s.z;
  r.c[0][1] = u.x;
  r.c[1][1] = u.y;
  r.c[2][1] = u.z;
  r.c[0][2] = -f.x;
  r.c[1][2] = -f.y;
  r.c[2][2] = -f.z;
  r.c[3][0] = -f3dot(s, eye);
  r.c[3][1] = -f3dot(u, eye);
  r.c[3][2] = f3dot(f, eye);
  return r;
}
M4 perspective(float fovy, float aspect, float zn, float zf) {
  const float th = tanf(fovy / 2.0f);
  M4 r = m4_zero();
  r.c[0][0] = 1.0f / (aspect * th);
  r.c[1][1] = 1.0f / th;
  r.c[2][2] = -(zf + zn) / (zf - zn);
  r.c[2][3] = -1.0f;
  r.c[3][2] = -(2.0f * zf * zn) / (zf - zn);
  return r;
}
// rotate(angle, (0, 1, 0)) * scale(vec3(k)), expanded as glm evaluates it
M4 rot_y_scale(float angle, float k) {
  const float c = cosf(angle), s = sinf(angle);
  M4 rot = m4_identity();
  rot.c[0][0] = c;
  rot.c[0][2] = -s;
  rot.c[1][1] = c + (1.0f - c);
  rot.c[2][0] = s;
  rot.c[2][2] = c;
  M4 sc = m4_identity();
  sc.c[0][0] = sc.c[1][1] = sc.c[2][2] = k;
  return m4_mul(rot, sc);
}
void to_rows(const M4& m, float* out) {
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) out[r * 4 + c] = m.c[c][r];
}
// General inverse (Gauss-Jordan in double), rows out.
void inverse_rows(const M4& m, float* out) {
  double a[4][8];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      a[r][c] = m.c[c][r];
      a[r][4 + c] = r == c ? 1.0 : 0.0;
    }
  for (int col = 0; col < 4; ++col) {
    int piv = col;
    for (int r = col + 1; r < 4; ++r)
      if (fabs(a[r][col]) > fabs(a[piv][col])) piv = r;
    for (int c = 0; c < 8; ++c) {
      const double t = a[col][c];
      a[col][c] = a[piv][c];
      a[piv][c] = t;
    }
    const double d = a[col][col];
    for (int c = 0; c < 8; ++c) a[col][c] /= d;
    for (int r = 0; r < 4; ++r)
      if (r != col) {
        const double k = a[r][col];
        for (int c = 0; c < 8; ++c) a[r][c] -= k * a[col][c];
      }
  }
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) out[r * 4 + c] = (float)a[r][4 + c];
}
}  // namespace

void render_matrices(const cwa_camera& cam, const cwa_render_params& prm, RenderMatrices* m) {
  const F3 eye{cam.eye[0], cam.eye[1], cam.eye[2]}, ctr{cam.center[0], cam.center[1], cam.center[2]},
      up{cam.up[0], cam.up[1], cam.up[2]};
  const M4 V = look_at(eye, ctr, up);
  const M4 P = perspective(cam.fovy, (float)prm.width / (float)prm.height, cam.near_z, cam.far_z);
  const M4 PV = m4_mul(P, V);
  const M4 Mp = rot_y_scale(prm.angle, prm.particle_scale);
  const M4 Mw = rot_y_scale(prm.angle, prm.wave_scale);
  to_rows(m4_mul(PV, Mp), m->mvp_p);
  to_rows(Mp, m->m_p);
  to_rows(m4_mul(PV, Mw), m->mvp_w);
  to_rows(Mw, m->m_w);
  inverse_rows(P, m->inv_p);
  inverse_rows(V, m->inv_v);
}

cudaError_t render_frame(RenderState* r, const cwa_camera& cam, const cwa_render_params& prm,
                         const float4* sorted_pos, const int32_t* sorted_id, int32_t n, const float* wave,
                         int32_t nx, int32_t nz, uint8_t* host_out, int32_t* status, cudaStream_t stream,
                         int64_t* launches) {
  RenderMatrices mats;
  render_matrices(cam, prm, &mats);
  RenderFrame f{};
  for (int k = 0; k < 16; ++k) {
    f.mvp_p[k] = mats.mvp_p[k];
    f.m_p[k] = mats.m_p[k];
    f.mvp_w[k] = mats.mvp_w[k];
    f.m_w[k] = mats.m_w[k];
    f.inv_p[k] = mats.inv_p[k];
    f.inv_v[k] = mats.inv_v[k];
  }
  for (int k = 0; k < 3; ++k) f.eye[k] = cam.eye[k];
  f.W = prm.width;
  f.H = prm.height;
  f.point_size = prm.point_size;
  f.res = prm.surface_res;
  f.n_tris = (prm.surface_res - 1) * (2 * prm.surface_res - 4);
  f.n_particles = n;
  f.draw_surface = prm.draw_surface != 0;
  f.draw_particles = prm.draw_particles != 0;
  f.draw_skybox = prm.draw_skybox != 0 && r->sky != nullptr;
  f.wave = wave;
  f.nx = nx;
  f.nz = nz;
  f.sky = r->sky;
  f.sky_size = r->sky_size;

  const int npix = f.W * f.H;
  const int tiles_x = (f.W + kTileW - 1) / kTileW, tiles_y = (f.H + kTileH - 1) / kTileH;
  const int n_tiles = tiles_x * tiles_y;
  const int n_tri = f.draw_surface ? f.n_tris : 0;
  const int nprim = n_tri + (f.draw_particles ? n : 0);
  const size_t nverts = (size_t)f.res * f.res;
  cudaError_t e = cudaSuccess;
  auto fail = [&](cudaError_t err) {
    cudaStreamSynchronize(stream);
    return err;
  };
  if ((e = ensure(r->verts, sizeof(MeshVert) * nverts)) != cudaSuccess) return fail(e);
  if ((e = ensure(r->upos, sizeof(float4) * (size_t)n)) != cudaSuccess) return fail(e);
  if ((e = ensure(r->cnt, sizeof(int32_t) * (size_t)n_tiles)) != cudaSuccess) return fail(e);
  if ((e = ensure(r->off, sizeof(int32_t) * ((size_t)n_tiles + 1))) != cudaSuccess) return fail(e);
  if ((e = ensure(r->dimg, sizeof(float) * (size_t)npix)) != cudaSuccess) return fail(e);
  if ((e = ensure(r->img, (size_t)npix * 4)) != cudaSuccess) return fail(e);
  if ((e = ensure(r->ws, scan_workspace_bytes(n_tiles + 1))) != cudaSuccess) return fail(e);
  MeshVert* verts = static_cast<MeshVert*>(r->verts.p);
  float4* upos = static_cast<float4*>(r->upos.p);
  int32_t* cnt = static_cast<int32_t*>(r->cnt.p);
  int32_t* off = static_cast<int32_t*>(r->off.p);
  ScanWorkspace sw;
  scan_bind_workspace(r->ws.p, n_tiles + 1, &sw);
  if (n > 0) {
    k_upload_order<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(sorted_pos, sorted_id, n, upos);
    *launches += 1;
  }
  f.pos = upos;
  if ((e = cudaMemsetAsync(cnt, 0, sizeof(int32_t) * n_tiles, stream)) != cudaSuccess) return fail(e);
  if (f.draw_surface && nverts) {
    k_mesh_vertices<<<(unsigned)((nverts + 255) / 256), 256, 0, stream>>>(f, verts);
    *launches += 1;
  }
  const unsigned pblocks = (unsigned)((nprim + 127) / 128);
  if (nprim > 0) {
    k_bin<<<pblocks, 128, 0, stream>>>(f, verts, n_tri, nprim, tiles_x, cnt, nullptr, nullptr, status);
    *launches += 1;
  }
  if ((e = scan_launch(cnt, off, n_tiles, n_tiles + 1, true, sw, status, stream, launches, nullptr)) !=
      cudaSuccess)
    return fail(e);
  int32_t total = 0;
  if ((e = cudaMemcpyAsync(&total, off + n_tiles, sizeof(int32_t), cudaMemcpyDeviceToHost, stream)) !=
      cudaSuccess)
    return fail(e);
  if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return fail(e);
  if (total < 0 || total > (1 << 30)) return fail(cudaErrorInvalidValue);  // pair buffer plus its sort scratch
  // the second half is the sort scratch of tile lists longer than kTileCap
  if ((e = ensure(r->pairs, sizeof(uint32_t) * 2 * (size_t)total, 8)) != cudaSuccess) return fail(e);
  uint32_t* pairs = static_cast<uint32_t*>(r->pairs.p);
  if (nprim > 0) {  // the scan cleared cnt: it now counts each tile's filled slots
    k_bin<<<pblocks, 128, 0, stream>>>(f, verts, n_tri, nprim, tiles_x, cnt, off, pairs, status);
    *launches += 1;
  }
  const unsigned tblocks = (unsigned)((n_tiles + kTileWarps - 1) / kTileWarps);
  int sort_bits = 0;
  while (nprim > 1 && ((nprim - 1) >> sort_bits) != 0) ++sort_bits;
  float* dimg = static_cast<float*>(r->dimg.p);
  uint8_t* img = static_cast<uint8_t*>(r->img.p);
  k_tile_depth<<<tblocks, kTileWarps * 32, 0, stream>>>(f, n_tri, tiles_x, n_tiles, off, pairs, dimg, status);
  k_tile_color<<<tblocks, kTileWarps * 32, 0, stream>>>(f, verts, n_tri, tiles_x, n_tiles, off, pairs, total,
                                                         sort_bits, dimg, img, status);
  *launches += 2;
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e);
  if ((e = cudaMemcpyAsync(host_out, img, (size_t)npix * 4, cudaMemcpyDeviceToHost, stream)) != cudaSuccess)
    return fail(e);
  return fail(cudaStreamSynchronize(stream));
}

}  // namespace cwa
