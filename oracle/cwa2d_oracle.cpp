// cwa2d_oracle.cpp — CPU restatement of the reference's 2D solver family
// (SphWave2D), test infrastructure only.
//
// SPH passes in FP64 (SphWaveKoschier2D_grid_cs.glsl ComputeDensityPressure
// :372-479 and ComputeForces :482-627, neighbours found by brute force over
// the same 3 x 3 block of grid cells); the shallow-water Lax-Wendroff step
// (Shallow1D_cs.glsl:110-174) in float32 op by op, and the initialisers
// (InitParticle :308-333, InitWave / Splash :88-117).  The shader's
// constants are float; they are formed in float here too, then widened.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "cwa_oracle.h"

namespace {

struct C2 {
  int n, ncx, ncy, wave_n, cols;
  float R, H, HSQ, rest, visc, mass, dt, gas, k2, psi, view_w, view_h, cell_x, cell_y, plane0_c, lambda, dx;
};

C2 consts(const cwa2d_params* p) {
  C2 c;
  c.n = p->n_particles;
  c.ncx = p->grid_cells[0];
  c.ncy = p->grid_cells[1];
  c.wave_n = p->wave_cells;
  c.cols = p->init_columns;
  c.R = p->particle_radius;
  c.H = 4.0f * c.R;
  c.HSQ = c.H * c.H;
  c.rest = p->rest_density;
  c.visc = p->visc;
  c.mass = (2.0f * c.R) * (2.0f * c.R) * c.rest;
  c.dt = p->dt;
  c.gas = p->gas_const;
  const float pi = 3.14159265f;
  c.k2 = 40.0f / (7.0f * pi * c.HSQ);
  c.psi = c.rest / (1.5f * c.k2);
  c.view_w = p->view_size[0];
  c.view_h = p->view_size[1];
  c.cell_x = c.view_w / (float)c.ncx;
  c.cell_y = c.view_h / (float)c.ncy;
  c.plane0_c = -0.5f * c.view_h + 15.0f * c.R - c.R + p->bottom;
  c.lambda = p->wave_lambda;
  c.dx = p->wave_dx;
  return c;
}

double w_cubic(const C2& c, double r) {
  const double q = r / c.H;
  if (q >= 1.0) return 0.0;
  if (q <= 0.5) return (double)c.k2 * (6.0 * q * q * (q - 1.0) + 1.0);
  const double q1 = 1.0 - q;
  return (double)c.k2 * 2.0 * q1 * q1 * q1;
}

double w_cubic_grad(const C2& c, double r) {
  const double q = r / c.H;
  if (q >= 1.0) return 0.0;
  if (q <= 0.5) return 6.0 * c.k2 * q * (3.0 * q - 2.0) / c.H;
  const double q1 = 1.0 - q;
  return -6.0 * c.k2 * (q1 * q1) / c.H;
}

double smoothstep(double e0, double e1, double x) {
  double t = (x - e0) / (e1 - e0);
  t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
  return t * t * (3.0 - 2.0 * t);
}

void sdf(const C2& c, double px, double py, double out[3]) {
  const double d[4] = {py + (double)c.plane0_c, px - (double)c.R, -px + (double)(c.view_w - c.R),
                       -py + (double)(c.view_h - c.R)};
  const double nx[4] = {0.0, 1.0, -1.0, 0.0}, ny[4] = {1.0, 0.0, 0.0, -1.0};
  int best = 0;
  for (int k = 1; k < 4; ++k)
    if (d[k] < d[best]) best = k;
  out[0] = nx[best];
  out[1] = ny[best];
  out[2] = d[best];
}

void tex(const float* w4, int n, double coord, double* x, double* y) {
  const double u = coord * n - 0.5, u0 = floor(u), f = u - u0;
  auto cl = [n](int i) { return i < 0 ? 0 : (i > n - 1 ? n - 1 : i); };
  const int i0 = cl((int)u0), i1 = cl((int)u0 + 1);
  *x = (1.0 - f) * w4[4 * i0] + f * w4[4 * i1];
  *y = (1.0 - f) * w4[4 * i0 + 1] + f * w4[4 * i1 + 1];
}

void wave_nh(const C2& c, const float* w4, double x, double* h, double* xvel) {
  const double coord = x / c.view_w;
  double mx, my;
  tex(w4, c.wave_n, coord, &mx, &my);
  *h = mx;
  *xvel = my / mx;
}

// ComputeCellIndex (uniform_grid_sph_cs.glsl:126-132) in float: the cell of
// a float coordinate, clamped to the grid.
int cell_of(float p, float cell, int n) {
  float t = floorf((p - 0.0f) / cell);
  t = t < 0.0f ? 0.0f : (t > (float)(n - 1) ? (float)(n - 1) : t);
  return (int)t;
}

// The cell lists of UniformGridSph2D::CollisionQuery (UniformGridGpu2D.cpp:
// 220-265): a point enters the cell of its position only when it lies
// strictly inside the grid's extents [0, view] (point_in_aabb,
// uniform_grid_sph_cs.glsl:19-23, 101-105); a point outside is in no list,
// so no neighbour search (its own included) sees it.  Members in index order.
std::vector<std::vector<int>> cell_lists(const C2& c, const cwa2d_particle* src) {
  std::vector<std::vector<int>> cells((size_t)c.ncx * c.ncy);
  for (int j = 0; j < c.n; ++j) {
    const float x = src[j].pos[0], y = src[j].pos[1];
    if (!(x > 0.0f && y > 0.0f && x < c.view_w && y < c.view_h)) continue;
    cells[(size_t)cell_of(x, c.cell_x, c.ncx) * c.ncy + cell_of(y, c.cell_y, c.ncy)].push_back(j);
  }
  return cells;
}

}  // namespace

extern "C" {

void orc2d_init_particles(const cwa2d_params* prm, cwa2d_particle* out) {
  const C2 c = consts(prm);
  const int cols = c.cols, rows = c.n / cols;
  for (int ix = 0; ix < c.n; ++ix) {
    const float px = c.view_w * ((float)(ix % cols) / (float)cols) + c.R;
    const float py = (18.0f * c.H) * ((float)(ix / cols) / (float)rows) + ((0.5f * c.view_h - 15.0f * c.R) + c.R);
    cwa2d_particle& q = out[ix];
    memset(&q, 0, sizeof(q));
    q.pos[0] = px;
    q.pos[1] = py;
    q.pos[3] = 1.0f;
    q.acc[3] = c.rest;
  }
}

void orc2d_wave_init_f32(const cwa2d_params* prm, const float* in4, float* out4, int32_t splash) {
  const C2 c = consts(prm);
  for (int i = 0; i < c.wave_n; ++i) {
    const float x = (float)i / (float)(c.wave_n - 1), xc = x - 0.5f;
    const float sgn = xc > 0.0f ? 1.0f : (xc < 0.0f ? -1.0f : 0.0f);
    float* o = out4 + 4 * i;
    if (splash) {
      for (int k = 0; k < 4; ++k) o[k] = in4[4 * i + k];
      const float h = -c.view_h * 0.1f * expf(-xc * xc / 0.005f);
      o[0] += h;
      o[1] += 0.2f * fabsf(h) * sgn;
    } else {
      const float h = c.view_h * 0.1f * expf(-xc * xc / 0.005f);
      o[0] = c.view_h * 0.5f + h;
      o[1] = 0.5f * fabsf(h) * sgn;
      o[2] = o[3] = 0.0f;
    }
  }
}

// One phase of the Lax-Wendroff step with FreeBC, float32 op by op; `out`
// holds the previous contents of the write buffer on entry.
void orc2d_wave_iter_f32(const cwa2d_params* prm, const float* in4, float* out4, int32_t phase) {
  const C2 c = consts(prm);
  const int n = c.wave_n;
  const float G = 9.8f, lam = c.lambda, dx = c.dx, hl = lam / 2.0f;
  auto at = [&](int i, int k) { return (i >= 0 && i < n) ? in4[4 * i + k] : 0.0f; };
  auto flux = [G](float h, float uh) { return uh * uh / h + 0.5f * G * h * h; };
  for (int i = 0; i < n; ++i) {
    float w[4] = {at(i, 0), at(i, 1), at(i, 2), at(i, 3)};
    if (phase == 0) {
      const float ex = at(i + 1, 0), ey = at(i + 1, 1);
      w[2] = (w[0] + ex) / 2.0f - hl * (ey - w[1]) / dx;
      w[3] = (w[1] + ey) / 2.0f - hl * (flux(ex, ey) - flux(w[0], w[1])) / dx;
      for (int k = 0; k < 4; ++k) out4[4 * i + k] = w[k];
    } else {
      const float wz = at(i - 1, 2), ww = at(i - 1, 3);
      const float h = w[0] - lam * (w[3] - ww) / dx;
      const float uh = w[1] - lam * (flux(w[2], w[3]) - flux(wz, ww)) / dx;
      w[0] = h;
      w[1] = uh;
      if (i == 0 || i == n - 1) continue;
      for (int k = 0; k < 4; ++k) out4[4 * i + k] = w[k];
      if (i == 1)
        for (int k = 0; k < 4; ++k) out4[k] = w[k];
      if (i == n - 2)
        for (int k = 0; k < 4; ++k) out4[4 * (n - 1) + k] = w[k];
    }
  }
}

// Wave1D_cs.glsl, float32 op by op.  get_n (:198-207) reads c1 from the
// older field and c0, e0, w0 from the newest; loads outside the field read
// zero (imageLoad out of range).  FreeBC (:148-166): cells 0 and n-1 keep no
// value of their own; cells 1 and n-2 copy theirs outward.
static void wave1d_store_free(const float (*w)[4], int n, float* out4) {
  for (int i = 1; i <= n - 2; ++i) {
    for (int k = 0; k < 4; ++k) out4[4 * i + k] = w[i][k];
    if (i == 1)
      for (int k = 0; k < 4; ++k) out4[k] = w[i][k];
    if (i == n - 2)
      for (int k = 0; k < 4; ++k) out4[4 * (n - 1) + k] = w[i][k];
  }
}

// ComputeVelocityAcceleration (:73-79) on w.
static void wave1d_vel_acc(float* w, float c0x, float c1x) {
  const float v = (w[0] - c1x) / 2.0f;
  const float a = (w[0] - 2.0f * c0x) + c1x;
  w[1] = v;
  w[2] = a;
}

// InitWave (:98-118).  Mode 0 stores the Gaussian bump centred at
// int(0.25 n); mode 1's Gaussian store is overwritten by FreeBC's stores of
// the half-step estimate w = c0 - 0.5 lambda (e0 - 2 c0 + w0) in every cell,
// which come later in each invocation.
void orc2d_wave1d_init_f32(const cwa2d_params* prm, const float* cur4, const float* prev4, float* out4, int32_t mode) {
  const int n = prm->wave_cells;
  const float lam = prm->wave_lambda;
  auto at = [&](const float* f, int i, int k) { return (i >= 0 && i < n) ? f[4 * i + k] : 0.0f; };
  if (mode == 0) {
    const int cen = (int)(0.25f * (float)n);
    for (int i = 0; i < n; ++i) {
      const int x = cen - i;
      const int xx = (int)((uint32_t)(-x) * (uint32_t)x);  // the shader's int product, wrapping
      const float h = 0.0f + 0.1f * expf((float)xx / 5000.0f);
      out4[4 * i + 0] = h;
      out4[4 * i + 1] = out4[4 * i + 2] = out4[4 * i + 3] = 0.0f;
    }
    return;
  }
  std::vector<float> w((size_t)4 * n);
  float(*wp)[4] = reinterpret_cast<float(*)[4]>(w.data());
  const float s = 0.5f * lam;
  for (int i = 0; i < n; ++i) {
    for (int k = 0; k < 4; ++k) {
      const float c0 = at(cur4, i, k), e0 = at(cur4, i + 1, k), w0 = at(cur4, i - 1, k);
      wp[i][k] = c0 - s * ((e0 - 2.0f * c0) + w0);
    }
    wave1d_vel_acc(wp[i], at(cur4, i, 0), at(prev4, i, 0));
  }
  wave1d_store_free(wp, n, out4);
}

// IterateWave (:120-131).
void orc2d_wave1d_iter_f32(const cwa2d_params* prm, const float* cur4, const float* prev4, float* out4) {
  const int n = prm->wave_cells;
  const float lam = prm->wave_lambda, beta = prm->wave_beta, atten = prm->wave_atten;
  const float a = (2.0f - 2.0f * lam) - beta, b = 1.0f - beta;
  auto at = [&](const float* f, int i, int k) { return (i >= 0 && i < n) ? f[4 * i + k] : 0.0f; };
  std::vector<float> w((size_t)4 * n);
  float(*wp)[4] = reinterpret_cast<float(*)[4]>(w.data());
  for (int i = 0; i < n; ++i) {
    for (int k = 0; k < 4; ++k) {
      const float c0 = at(cur4, i, k), c1 = at(prev4, i, k);
      const float e0 = at(cur4, i + 1, k), w0 = at(cur4, i - 1, k);
      wp[i][k] = atten * ((a * c0 + lam * (e0 + w0)) - b * c1);
    }
    wave1d_vel_acc(wp[i], at(cur4, i, 0), at(prev4, i, 0));
  }
  wave1d_store_free(wp, n, out4);
}

// ComputeDensityPressure in FP64: reads `in`, writes `out` (positions after
// the wall projection, enable flag, density, pressure).
void orc2d_density(const cwa2d_params* prm, const cwa2d_particle* in, const float* wave4, cwa2d_particle* out) {
  const C2 c = consts(prm);
  const std::vector<std::vector<int>> cells = cell_lists(c, in);
#pragma omp parallel for schedule(dynamic, 64)
  for (int ix = 0; ix < c.n; ++ix) {
    cwa2d_particle q = in[ix];
    double px = q.pos[0], py = q.pos[1], vx = q.vel[0], vy = q.vel[1];
    double h, xvel;
    wave_nh(c, wave4, px, &h, &xvel);
    if (q.pos[3] == 0.0f && fabs(xvel) > 0.05) q.pos[3] = 1.0f;
    if (q.pos[3] == 1.0f && fabs(xvel) < 0.05) q.pos[3] = 0.0f;
    double db[3];
    sdf(c, px, py, db);
    if (db[2] < 0.0) {
      px -= 0.75 * db[2] * db[0];
      py -= 0.75 * db[2] * db[1];
      const double vn = fmin(0.0, vx * db[0] + vy * db[1]);
      vx -= 1.75 * vn * db[0];
      vy -= 1.75 * vn * db[1];
    }
    q.pos[0] = (float)px;
    q.pos[1] = (float)py;
    q.vel[0] = (float)vx;
    q.vel[1] = (float)vy;
    if (py > c.view_h) {
      out[ix] = q;
      continue;
    }
    double rho = 0.0;
    // the query box around the stored (float) position, in float
    const int x0 = cell_of(q.pos[0] - c.H, c.cell_x, c.ncx), x1 = cell_of(q.pos[0] + c.H, c.cell_x, c.ncx);
    const int y0 = cell_of(q.pos[1] - c.H, c.cell_y, c.ncy), y1 = cell_of(q.pos[1] + c.H, c.cell_y, c.ncy);
    for (int ci = x0; ci <= x1; ++ci)
      for (int cj = y0; cj <= y1; ++cj)
        for (int j : cells[(size_t)ci * c.ncy + cj]) {
          const double rx = px - in[j].pos[0], ry = py - in[j].pos[1], r2 = rx * rx + ry * ry;
          if (r2 < (double)c.HSQ) rho += w_cubic(c, sqrt(r2));
        }
    rho = (double)c.mass * rho;
    if (db[2] < c.H) rho += (double)c.psi * w_cubic(c, fmax(0.0, db[2]));
    rho = fmax((double)c.rest, rho);
    q.acc[3] = (float)rho;
    q.vel[3] = (float)((double)c.gas * (pow(rho / c.rest, 3.0) - 1.0));
    out[ix] = q;
  }
}

// ComputeForces in FP64 (forward Euler at the end).  The neighbour lists are
// those of the grid built from `grid_src` (null: from `in`): SphUgrid::Compute
// (SphWave2D/StencilBuffer.cpp:150-179) builds one grid per substep, before
// the density pass, and the force pass searches that grid with the
// positions the density pass left.
void orc2d_force(const cwa2d_params* prm, const cwa2d_particle* in, const cwa2d_particle* grid_src,
                 const float* wave4, cwa2d_particle* out) {
  const C2 c = consts(prm);
  const std::vector<std::vector<int>> cells = cell_lists(c, grid_src ? grid_src : in);
#pragma omp parallel for schedule(dynamic, 64)
  for (int ix = 0; ix < c.n; ++ix) {
    cwa2d_particle q = in[ix];
    if (q.pos[3] == 0.0f) {
      out[ix] = q;
      continue;
    }
    const double px = q.pos[0], py = q.pos[1], vxi = q.vel[0], vyi = q.vel[1];
    const double rho_i = q.acc[3], api = (double)q.vel[3] / (rho_i * rho_i);
    double apx = 0, apy = 0, avx = 0, avy = 0;
    const int x0 = cell_of(q.pos[0] - c.H, c.cell_x, c.ncx), x1 = cell_of(q.pos[0] + c.H, c.cell_x, c.ncx);
    const int y0 = cell_of(q.pos[1] - c.H, c.cell_y, c.ncy), y1 = cell_of(q.pos[1] + c.H, c.cell_y, c.ncy);
    for (int ci = x0; ci <= x1; ++ci)
      for (int cj = y0; cj <= y1; ++cj)
        for (int j : cells[(size_t)ci * c.ncy + cj]) {
          if (j == ix) continue;
          const double rx = px - in[j].pos[0], ry = py - in[j].pos[1], r = sqrt(rx * rx + ry * ry);
          if (!(r < c.H && r > 0.0)) continue;
          const double wg = w_cubic_grad(c, r), ux = rx / r, uy = ry / r;
          const double rho_j = in[j].acc[3];
          const double sp = (api + (double)in[j].vel[3] / (rho_j * rho_j)) * wg;
          apx -= sp * ux;
          apy -= sp * uy;
          const double vx = vxi - in[j].vel[0], vy = vyi - in[j].vel[1];
          const double sv = 1.0 / rho_j * (vx * rx + vy * ry) / (r * r + 0.01 * c.HSQ) * wg;
          avx -= sv * ux;
          avy -= sv * uy;
        }
    const double cv = -(double)c.visc * 8.0 * c.mass;
    avx *= cv;
    avy *= cv;
    apx *= c.mass;
    apy *= c.mass;
    double db[3];
    sdf(c, px, py, db);
    if (db[2] < c.H) {
      const double wg = w_cubic_grad(c, fmax(0.0, db[2]));
      apx += c.psi * api * wg * -db[0];
      apy += c.psi * api * wg * -db[1];
    }
    double h, vxw;
    wave_nh(c, wave4, px, &h, &vxw);
    const double dh = h - c.view_h / 2.0, mask = smoothstep(0.0, 0.2, fabs(vxw));
    const double dy = (py - h) - 0.5 * dh;
    const double tro = (ix % 5 < 4) ? -mask * 500000.0 * smoothstep(0.0, 10.0, dy) : 0.0;
    const double ax = apx + avx, ay = apy + avy - 9.8 + tro;
    const double nvx = vxi + c.dt * ax, nvy = vyi + c.dt * ay;
    q.acc[0] = (float)ax;
    q.acc[1] = (float)ay;
    q.vel[0] = (float)nvx;
    q.vel[1] = (float)nvy;
    q.pos[0] = (float)(px + c.dt * nvx);
    q.pos[1] = (float)(py + c.dt * nvy);
    out[ix] = q;
  }
}

}  // extern "C"
