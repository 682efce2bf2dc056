// cwa_render_oracle.cpp — CPU restatement of one headless frame of the
// reference's display() (CoupledWaterAnimation/Main.cpp:326-474).  Test
// infrastructure only: the tests compare the renderer against it.
//
// It follows GL's pipeline directly.  Primitives (the strip mesh of
// Surf.cpp:68-190 displaced by wave_vs.glsl:30-42, then the particle
// sprites of particle_vs.glsl) are rasterised in draw order into per-pixel
// fragment lists.  Every pixel then replays its list through the GL_LESS
// depth test and SRC_ALPHA / ONE_MINUS_SRC_ALPHA blending into an 8-bit
// target, shading with wave_fs.glsl:30-88 and particle_fs.glsl (pass 0),
// whose normals come from the pass-2 depth image (:74-82, :104-118).
// Matrices restate glm's lookAt / perspective / rotate / scale / mat4
// product in float.  Coverage, depth and projection arithmetic is float32
// op by op (the library is built with -ffp-contract=off), so fragment sets
// match the GPU exactly; shading uses libm.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "cwa_oracle.h"

namespace {

struct V3 {
  float x, y, z;
};
V3 v3(float x, float y, float z) { return V3{x, y, z}; }
V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
V3 mul(float k, V3 a) { return v3(k * a.x, k * a.y, k * a.z); }
V3 hmul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 normalize(V3 a) { return mul(1.0f / sqrtf(dot(a, a)), a); }
V3 reflect(V3 i, V3 n) { return sub(i, mul(2.0f * dot(n, i), n)); }
V3 refract(V3 i, V3 n, float eta) {
  const float d = dot(n, i);
  const float k = 1.0f - eta * eta * (1.0f - d * d);
  if (k < 0.0f) return v3(0.0f, 0.0f, 0.0f);
  return sub(mul(eta, i), mul(eta * d + sqrtf(k), n));
}
float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }

// ---- glm in float, column-major ----
struct M4 {
  float c[4][4];
};
M4 zero4() {
  M4 m;
  memset(&m, 0, sizeof(m));
  return m;
}
M4 ident4() {
  M4 m = zero4();
  for (int i = 0; i < 4; ++i) m.c[i][i] = 1.0f;
  return m;
}
M4 mul4(const M4& a, const M4& b) {
  M4 r;
  for (int j = 0; j < 4; ++j)
    for (int row = 0; row < 4; ++row)
      r.c[j][row] = ((a.c[0][row] * b.c[j][0] + a.c[1][row] * b.c[j][1]) + a.c[2][row] * b.c[j][2]) +
                    a.c[3][row] * b.c[j][3];
  return r;
}
V3 cross(V3 a, V3 b) { return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
M4 look_at(V3 eye, V3 center, V3 up) {
  const V3 f = normalize(sub(center, eye));
  const V3 s = normalize(cross(f, up));
  const V3 u = cross(s, f);
  M4 r = ident4();
  r.c[0][0] = s.x;
  r.c[1][0] = s.y;
  r.c[2][0] = s.z;
  r.c[0][1] = u.x;
  r.c[1][1] = u.y;
  r.c[2][1] = u.z;
  r.c[0][2] = -f.x;
  r.c[1][2] = -f.y;
  r.c[2][2] = -f.z;
  r.c[3][0] = -dot(s, eye);
  r.c[3][1] = -dot(u, eye);
  r.c[3][2] = dot(f, eye);
  return r;
}
M4 perspective(float fovy, float aspect, float zn, float zf) {
  const float th = tanf(fovy / 2.0f);
  M4 r = zero4();
  r.c[0][0] = 1.0f / (aspect * th);
  r.c[1][1] = 1.0f / th;
  r.c[2][2] = -(zf + zn) / (zf - zn);
  r.c[2][3] = -1.0f;
  r.c[3][2] = -(2.0f * zf * zn) / (zf - zn);
  return r;
}
M4 rotate_y_scale(float angle, float k) {
  const float c = cosf(angle), s = sinf(angle);
  M4 rot = ident4();
  rot.c[0][0] = c;
  rot.c[0][2] = -s;
  rot.c[1][1] = c + (1.0f - c);
  rot.c[2][0] = s;
  rot.c[2][2] = c;
  M4 sc = ident4();
  sc.c[0][0] = sc.c[1][1] = sc.c[2][2] = k;
  return mul4(rot, sc);
}
void rows(const M4& m, float* o) {
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) o[r * 4 + c] = m.c[c][r];
}
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

float row4(const float* m, float x, float y, float z) { return ((m[0] * x + m[1] * y) + m[2] * z) + m[3]; }

struct Win {
  float x, y, z, w, cz;
  bool ok;
};
Win project(const float* mvp, float x, float y, float z, int W, int H, bool point) {
  Win o;
  const float cx = row4(mvp, x, y, z), cy = row4(mvp + 4, x, y, z), cz = row4(mvp + 8, x, y, z),
              cw = row4(mvp + 12, x, y, z);
  o.w = cw;
  o.cz = cz;
  o.ok = cw > 0.0f && cz >= -cw && cz <= cw;
  if (point) o.ok = o.ok && cx >= -cw && cx <= cw && cy >= -cw && cy <= cw;
  o.x = ((cx / cw + 1.0f) * 0.5f) * (float)W;
  o.y = ((cy / cw + 1.0f) * 0.5f) * (float)H;
  o.z = (cz / cw + 1.0f) * 0.5f;
  return o;
}

struct Vert {
  float wx, wy, wz, iw, s, t;
  V3 pw;
  bool ok;
};

struct Frame {
  float mvp_p[16], m_p[16], mvp_w[16], m_w[16], inv_p[16], inv_v[16];
  V3 eye;
  int W, H, res;
  float ps;
  const float* wave;
  int nx, nz;
  const uint8_t* sky;
  int sky_size;
};

V3 texel(const Frame& f, int face, int x, int y) {
  const uint8_t* p = f.sky + (((size_t)face * f.sky_size + y) * f.sky_size + x) * 4;
  return v3(p[0] / 255.0f, p[1] / 255.0f, p[2] / 255.0f);
}

// GL cube-map face selection; GL_LINEAR, clamped within the face.
V3 cube(const Frame& f, V3 r) {
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
  if (ma == 0.0f) return texel(f, 0, f.sky_size / 2, f.sky_size / 2);
  const float s = 0.5f * (sc / ma + 1.0f), t = 0.5f * (tc / ma + 1.0f);
  const float u = s * f.sky_size - 0.5f, v = t * f.sky_size - 0.5f;
  const float u0 = floorf(u), v0 = floorf(v), au = u - u0, av = v - v0;
  const int n1 = f.sky_size - 1;
  auto cl = [n1](int i) { return i < 0 ? 0 : (i > n1 ? n1 : i); };
  const int x0 = cl((int)u0), x1 = cl((int)u0 + 1), y0 = cl((int)v0), y1 = cl((int)v0 + 1);
  const V3 a = add(mul(1.0f - au, texel(f, face, x0, y0)), mul(au, texel(f, face, x1, y0)));
  const V3 b = add(mul(1.0f - au, texel(f, face, x0, y1)), mul(au, texel(f, face, x1, y1)));
  return add(mul(1.0f - av, a), mul(av, b));
}

Vert mesh_vertex(const Frame& f, int a, int b) {
  Vert v;
  const float fx = (float)(int)(0.1f * (float)a), fz = (float)(int)(0.1f * (float)b);
  v.s = (float)a / (float)(f.res - 1);
  v.t = (float)b / (float)(f.res - 1);
  const float h = orc_sample_f32(f.wave, f.nx, f.nz, v.s, v.t);
  const Win w = project(f.mvp_w, fx, 50.0f * h, fz, f.W, f.H, false);
  v.wx = w.x;
  v.wy = w.y;
  v.wz = w.z;
  v.iw = 1.0f / w.w;
  v.ok = w.ok;
  v.pw = v3(row4(f.m_w, fx, -1.0f, fz), row4(f.m_w + 4, fx, -1.0f, fz), row4(f.m_w + 8, fx, -1.0f, fz));
  return v;
}

float edge(float ax, float ay, float bx, float by, float px, float py) {
  return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}
bool top_left(float ax, float ay, float bx, float by) { return (ay == by && bx < ax) || (by < ay); }

struct Tri {
  float x[3], y[3], area;
  int o[3];
  int x0, x1, y0, y1;
  bool ok;
};

Tri setup(const Vert* mv, int W, int H) {
  Tri s;
  int o[3] = {0, 1, 2};
  float area = edge(mv[0].wx, mv[0].wy, mv[1].wx, mv[1].wy, mv[2].wx, mv[2].wy);
  s.ok = mv[0].ok && mv[1].ok && mv[2].ok && area != 0.0f;
  if (area < 0.0f) {
    o[1] = 2;
    o[2] = 1;
    area = -area;
  }
  for (int q = 0; q < 3; ++q) {
    s.x[q] = mv[o[q]].wx;
    s.y[q] = mv[o[q]].wy;
    s.o[q] = o[q];
  }
  s.area = area;
  const float minx = fminf(fminf(s.x[0], s.x[1]), s.x[2]), maxx = fmaxf(fmaxf(s.x[0], s.x[1]), s.x[2]);
  const float miny = fminf(fminf(s.y[0], s.y[1]), s.y[2]), maxy = fmaxf(fmaxf(s.y[0], s.y[1]), s.y[2]);
  auto lo = [](float v) { return v > 2e9f ? 2000000000 : (v < -2e9f ? -2000000000 : (int)v); };
  s.x0 = lo(floorf(minx - 0.5f));
  s.x1 = lo(ceilf(maxx - 0.5f));
  s.y0 = lo(floorf(miny - 0.5f));
  s.y1 = lo(ceilf(maxy - 0.5f));
  if (s.x0 < 0) s.x0 = 0;
  if (s.y0 < 0) s.y0 = 0;
  if (s.x1 > W - 1) s.x1 = W - 1;
  if (s.y1 > H - 1) s.y1 = H - 1;
  if (s.x0 > s.x1 || s.y0 > s.y1) s.ok = false;
  return s;
}

bool cover(const Tri& s, int px, int py, float l[3]) {
  const float cx = (float)px + 0.5f, cy = (float)py + 0.5f;
  const float e0 = edge(s.x[1], s.y[1], s.x[2], s.y[2], cx, cy);
  const float e1 = edge(s.x[2], s.y[2], s.x[0], s.y[0], cx, cy);
  const float e2 = edge(s.x[0], s.y[0], s.x[1], s.y[1], cx, cy);
  const bool in0 = e0 > 0.0f || (e0 == 0.0f && top_left(s.x[1], s.y[1], s.x[2], s.y[2]));
  const bool in1 = e1 > 0.0f || (e1 == 0.0f && top_left(s.x[2], s.y[2], s.x[0], s.y[0]));
  const bool in2 = e2 > 0.0f || (e2 == 0.0f && top_left(s.x[0], s.y[0], s.x[1], s.y[1]));
  if (!(in0 && in1 && in2)) return false;
  l[0] = e0 / s.area;
  l[1] = e1 / s.area;
  l[2] = e2 / s.area;
  return true;
}

void strip_tri(int t, int n, int va[3], int vb[3]) {
  const int per_row = 2 * n - 4, i = t / per_row, k0 = t - i * per_row;
  for (int q = 0; q < 3; ++q) {
    va[q] = i + ((k0 + q) & 1);
    vb[q] = (k0 + q) >> 1;
  }
}

struct Frag {
  int prim;
  float z;
};

float unorm8(float x) {
  x = x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x);
  return floorf(x * 255.0f + 0.5f);
}

V3 m3x(const float* m, V3 v, float w) {
  return v3(m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * w, m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * w,
            m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * w);
}

// wave_fs.glsl main (:36-50) for a fragment at world position p whose wave
// sample is v; the mesh normal is (0, 1, 0) (Surf.cpp:49-61 gives (0, -1, 0),
// wave_vs.glsl:40 negates it).  Colour before blending.
void shade_wave(const Frame& f, V3 p, float v, V3* rgb, float* a) {
  const V3 light_col = v3(1.0f, 0.85f, 0.7f), eye = f.eye;
  const V3 nrm = v3(0.0f, 1.0f, 0.0f);
  const V3 I = normalize(sub(p, eye));
  const V3 refl = cube(f, reflect(I, nrm)), refr = cube(f, refract(I, nrm, 1.0f / 1.33f));
  const V3 ld = normalize(sub(v3(0.0f, 1.0f, 0.0f), p));
  const float diff = fmaxf(dot(nrm, ld), 0.0f);
  const V3 vd = normalize(sub(eye, p));
  const float spec = powf(fmaxf(dot(vd, reflect(v3(-ld.x, -ld.y, -ld.z), nrm)), 0.0f), 32.0f);
  const V3 lit = hmul(add(add(mul(0.8f, light_col), mul(diff, light_col)), mul(10.0f * spec, light_col)),
                      v3(0.6f, 0.8f, 1.0f));
  const V3 comb = add(mul(0.75f, add(refl, refr)), mul(0.1f, lit));
  *rgb = v3(mixf(comb.x, 0.7f, v), mixf(comb.y, 0.9f, v), mixf(comb.z, 1.0f, v));
  *a = mixf(0.2f, 0.0f, v);
}

// particle_fs.glsl pass 0 (:47-68) for the fragment at pixel (px, py), r
// sprite widths from the sprite's centre, of the particle at world position
// pp; depth_at reads the pass-2 depth image (0 off the image).  Colour
// before blending.
template <class DepthAt>
void shade_particle(const Frame& f, int px, int py, float r, V3 pp, DepthAt depth_at, V3* rgb, float* a) {
  const V3 light_col = v3(1.0f, 0.85f, 0.7f), eye = f.eye;
  const float spec = powf(fmaxf(dot(normalize(pp), normalize(v3(1.0f, 1.0f, 0.0f))), 0.0f), 16.0f);
  const float aa = expf(-12.0f * r) + 0.1f * expf(-2.0f * r);
  const float dzdx = 0.5f * (depth_at(px + 1, py) - depth_at(px - 1, py));
  const float dzdy = 0.5f * (depth_at(px, py + 1) - depth_at(px, py - 1));
  const V3 nrm = normalize(v3(-dzdx, -dzdy, 1.0f));
  const V3 I = normalize(sub(eye, pp));
  const V3 refl = cube(f, reflect(I, nrm)), refr = cube(f, refract(I, nrm, 1.0f / 1.33f));
  const float dz = depth_at(px, py);
  const float cx = (px + 0.5f) * 2.0f - 1.0f, cy = (py + 0.5f) * 2.0f - 1.0f, cz = dz * 2.0f - 1.0f;
  const float vw = f.inv_p[12] * cx + f.inv_p[13] * cy + f.inv_p[14] * cz + f.inv_p[15];
  const V3 view = mul(1.0f / vw, m3x(f.inv_p, v3(cx, cy, cz), 1.0f));
  const V3 pos = m3x(f.inv_v, view, 1.0f);
  const V3 ld = normalize(sub(v3(1.0f, 1.0f, 0.0f), pos));
  const float diff = fmaxf(dot(nrm, ld), 0.0f);
  const V3 vd = normalize(sub(eye, pos));
  const float spec2 = powf(fmaxf(dot(vd, reflect(v3(-ld.x, -ld.y, -ld.z), nrm)), 0.0f), 32.0f);
  const V3 lit = hmul(add(add(mul(0.8f, light_col), mul(diff, light_col)), mul(0.9f * spec2, light_col)),
                      v3(0.4f, 0.7f, 1.0f));
  const V3 comb = add(mul(0.75f, add(refl, refr)), mul(0.1f, lit));
  const float t = 2.0f * pp.y;
  *rgb = v3(mixf(comb.x, 1.0f, t) + spec, mixf(comb.y, 1.0f, t) + spec, mixf(comb.z, 1.0f, t) + spec);
  *a = mixf(0.1f, aa, t);
}

Frame shade_frame(const float inv_p[16], const float inv_v[16], const float eye[3], const uint8_t* sky,
                  int32_t sky_size) {
  Frame f{};
  for (int k = 0; k < 16; ++k) {
    f.inv_p[k] = inv_p[k];
    f.inv_v[k] = inv_v[k];
  }
  f.eye = v3(eye[0], eye[1], eye[2]);
  f.sky = sky;
  f.sky_size = sky ? sky_size : 0;
  return f;
}

}  // namespace

void orc_render(const float* pos4, int32_t n, const float* wave, int32_t nx, int32_t nz, const cwa_camera* cam,
                const cwa_render_params* prm, const uint8_t* sky, int32_t sky_size, uint8_t* out) {
  Frame f;
  const V3 eye = v3(cam->eye[0], cam->eye[1], cam->eye[2]);
  const M4 V = look_at(eye, v3(cam->center[0], cam->center[1], cam->center[2]),
                       v3(cam->up[0], cam->up[1], cam->up[2]));
  const M4 P = perspective(cam->fovy, (float)prm->width / (float)prm->height, cam->near_z, cam->far_z);
  const M4 PV = mul4(P, V);
  const M4 Mp = rotate_y_scale(prm->angle, prm->particle_scale), Mw = rotate_y_scale(prm->angle, prm->wave_scale);
  rows(mul4(PV, Mp), f.mvp_p);
  rows(Mp, f.m_p);
  rows(mul4(PV, Mw), f.mvp_w);
  rows(Mw, f.m_w);
  inverse_rows(P, f.inv_p);
  inverse_rows(V, f.inv_v);
  f.eye = eye;
  f.W = prm->width;
  f.H = prm->height;
  f.res = prm->surface_res;
  f.ps = prm->point_size;
  f.wave = wave;
  f.nx = nx;
  f.nz = nz;
  f.sky = sky;
  f.sky_size = sky ? sky_size : 0;
  const int W = f.W, H = f.H, res = f.res;
  const int n_tris = (res - 1) * (2 * res - 4);
  const int first_particle = prm->draw_surface ? n_tris : 0;
  std::vector<std::vector<Frag>> lists((size_t)W * H);
  std::vector<Vert> verts;
  if (prm->draw_surface) {
    verts.resize((size_t)res * res);
    for (int a = 0; a < res; ++a)
      for (int b = 0; b < res; ++b) verts[(size_t)a * res + b] = mesh_vertex(f, a, b);
    for (int t = 0; t < n_tris; ++t) {
      int va[3], vb[3];
      strip_tri(t, res, va, vb);
      Vert mv[3] = {verts[(size_t)va[0] * res + vb[0]], verts[(size_t)va[1] * res + vb[1]],
                    verts[(size_t)va[2] * res + vb[2]]};
      const Tri s = setup(mv, W, H);
      if (!s.ok) continue;
      for (int py = s.y0; py <= s.y1; ++py)
        for (int px = s.x0; px <= s.x1; ++px) {
          float l[3];
          if (!cover(s, px, py, l)) continue;
          const float z = (l[0] * mv[s.o[0]].wz + l[1] * mv[s.o[1]].wz) + l[2] * mv[s.o[2]].wz;
          lists[(size_t)py * W + px].push_back(Frag{t, z});
        }
    }
  }
  const float half = 0.5f * f.ps, inv_s = 1.0f / f.ps;
  std::vector<Win> pw((size_t)n);
  for (int i = 0; i < n; ++i) pw[i] = project(f.mvp_p, pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2], W, H, true);
  if (prm->draw_particles) {
    for (int i = 0; i < n; ++i) {
      const Win& w = pw[i];
      if (!w.ok) continue;
      int x0 = (int)ceilf((w.x - half) - 0.5f), x1 = (int)ceilf((w.x + half) - 0.5f) - 1;
      int y0 = (int)ceilf((w.y - half) - 0.5f), y1 = (int)ceilf((w.y + half) - 0.5f) - 1;
      if (x0 < 0) x0 = 0;
      if (y0 < 0) y0 = 0;
      if (x1 > W - 1) x1 = W - 1;
      if (y1 > H - 1) y1 = H - 1;
      for (int py = y0; py <= y1; ++py)
        for (int px = x0; px <= x1; ++px) {
          const float dx = (((float)px + 0.5f) - w.x) * inv_s, dy = (((float)py + 0.5f) - w.y) * inv_s;
          if (!(dx * dx + dy * dy < 0.25f)) continue;
          lists[(size_t)py * W + px].push_back(Frag{first_particle + i, w.z});
        }
    }
  }
  // pass 2: depth image (eye_pos.z of the particle fragment that wins GL_LESS)
  std::vector<float> D((size_t)W * H, 0.0f);
  for (size_t p = 0; p < lists.size(); ++p) {
    float best = 1.0f;
    int win = -1;
    for (const Frag& fr : lists[p])
      if (fr.prim >= first_particle && fr.z < best) {
        best = fr.z;
        win = fr.prim - first_particle;
      }
    if (win >= 0) D[p] = pw[win].cz;
  }
  auto depth_at = [&](int x, int y) { return (x < 0 || y < 0 || x >= W || y >= H) ? 0.0f : D[(size_t)y * W + x]; };
  for (int py = 0; py < H; ++py)
    for (int px = 0; px < W; ++px) {
      float c[3] = {0.0f, 0.0f, 0.0f};
      if (prm->draw_skybox && f.sky) {
        const float ndx = (px + 0.5f) / W * 2.0f - 1.0f, ndy = (py + 0.5f) / H * 2.0f - 1.0f;
        const float vw = f.inv_p[12] * ndx + f.inv_p[13] * ndy + f.inv_p[14] + f.inv_p[15];
        const V3 view = mul(1.0f / vw, m3x(f.inv_p, v3(ndx, ndy, 1.0f), 1.0f));
        const V3 sk = cube(f, m3x(f.inv_v, view, 0.0f));
        c[0] = unorm8(sk.x);
        c[1] = unorm8(sk.y);
        c[2] = unorm8(sk.z);
      }
      float depth = 1.0f;
      for (const Frag& fr : lists[(size_t)py * W + px]) {
        if (!(fr.z < depth)) continue;
        depth = fr.z;
        V3 rgb;
        float a;
        if (fr.prim < first_particle) {  // wave_fs.glsl
          int va[3], vb[3];
          strip_tri(fr.prim, res, va, vb);
          Vert mv[3] = {verts[(size_t)va[0] * res + vb[0]], verts[(size_t)va[1] * res + vb[1]],
                        verts[(size_t)va[2] * res + vb[2]]};
          const Tri s = setup(mv, W, H);
          float l[3];
          cover(s, px, py, l);
          float q[3], sum = 0.0f;
          for (int k = 0; k < 3; ++k) {
            q[k] = l[k] * mv[s.o[k]].iw;
            sum += q[k];
          }
          float ts = 0.0f, tt = 0.0f;
          V3 p = v3(0.0f, 0.0f, 0.0f);
          for (int k = 0; k < 3; ++k) {
            const float wgt = q[k] / sum;
            ts += wgt * mv[s.o[k]].s;
            tt += wgt * mv[s.o[k]].t;
            p = add(p, mul(wgt, mv[s.o[k]].pw));
          }
          shade_wave(f, p, orc_sample_f32(wave, nx, nz, ts, tt), &rgb, &a);
        } else {  // particle_fs.glsl pass 0
          const int i = fr.prim - first_particle;
          const Win& w = pw[i];
          const float dx = (((float)px + 0.5f) - w.x) * inv_s, dy = (((float)py + 0.5f) - w.y) * inv_s;
          const float r = sqrtf(dx * dx + dy * dy);
          const float* q = pos4 + 4 * i;
          const V3 pp = v3(row4(f.m_p, q[0], q[1], q[2]), row4(f.m_p + 4, q[0], q[1], q[2]),
                           row4(f.m_p + 8, q[0], q[1], q[2]));
          shade_particle(f, px, py, r, pp, depth_at, &rgb, &a);
        }
        a = a < 0.0f ? 0.0f : (a > 1.0f ? 1.0f : a);
        const float src[3] = {rgb.x, rgb.y, rgb.z};
        for (int ch = 0; ch < 3; ++ch) {
          const float s = src[ch] < 0.0f ? 0.0f : (src[ch] > 1.0f ? 1.0f : src[ch]);
          c[ch] = unorm8(s * a + (c[ch] / 255.0f) * (1.0f - a));
        }
      }
      uint8_t* o = out + ((size_t)py * W + px) * 4;
      o[0] = (uint8_t)c[0];
      o[1] = (uint8_t)c[1];
      o[2] = (uint8_t)c[2];
      o[3] = 255;
    }
}

void orc_shade_particle(const float inv_p[16], const float inv_v[16], const float eye[3], const uint8_t* sky,
                        int32_t sky_size, const float* D, int32_t w, int32_t h, int32_t px, int32_t py, float r,
                        const float pp[3], float out[4]) {
  const Frame f = shade_frame(inv_p, inv_v, eye, sky, sky_size);
  auto depth_at = [&](int x, int y) { return (x < 0 || y < 0 || x >= w || y >= h) ? 0.0f : D[(size_t)y * w + x]; };
  V3 rgb;
  shade_particle(f, px, py, r, v3(pp[0], pp[1], pp[2]), depth_at, &rgb, &out[3]);
  out[0] = rgb.x;
  out[1] = rgb.y;
  out[2] = rgb.z;
}

void orc_shade_wave(const float eye[3], const uint8_t* sky, int32_t sky_size, const float p[3], float v,
                    float out[4]) {
  const float id[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  const Frame f = shade_frame(id, id, eye, sky, sky_size);
  V3 rgb;
  shade_wave(f, v3(p[0], p[1], p[2]), v, &rgb, &out[3]);
  out[0] = rgb.x;
  out[1] = rgb.y;
  out[2] = rgb.z;
}
