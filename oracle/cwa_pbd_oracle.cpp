// cwa_pbd_oracle.cpp — CPU restatement of the PBD box collisions
// (UniformGrid2D/uniform_grid_pbd_3D_cs.glsl, UniformGridGpu3D.cpp:128-183,
// 338-346), test infrastructure only.
//
// float32 op by op (the library is built with -ffp-contract=off), with the
// accumulation order the GPU path defines for the shader's atomics: per box,
// its wall terms, then the contacts it owns (it is the lower index) in
// discovery order, then the contacts it is the partner of, ordered by the
// owner's index and discovery order.  Contacts are discovered as
// CollisionQuery does: the cells of the box's predicted AABB in x, y, z
// order, each cell's boxes by index, a pair visited in its home cell only.
#include <math.h>
#include <stdint.h>

#include <vector>

#include "cwa_oracle.h"

namespace {

struct Pair {
  int i, j;
  float wi, wj, disp[3], frict[3];
};

struct K {
  int n, nd[3];
  float lo[3], hi[3], cell[3], g[3], dt, damping, k, k_static, sleep, mu_k, mu_s, e;
};

int cell_axis(float p, float lo, float cell, int n) {
  float f = floorf((p - lo) / cell);
  f = fminf(fmaxf(f, 0.0f), (float)(n - 1));
  return (int)f;
}

float len3(float x, float y, float z) { return sqrtf((x * x + y * y) + z * z); }

bool collide(const K& c, const cwa_pbd_box& bi, const cwa_pbd_box& bj, const float* qmin, const float* qmax,
             const float* bmin, const float* bmax, Pair* out) {
  float sz[3];
  for (int a = 0; a < 3; ++a) sz[a] = fminf(qmax[a], bmax[a]) - fmaxf(qmin[a], bmin[a]);
  int comp = 0;
  if (sz[1] < sz[0] && sz[1] < sz[2]) comp = 1;
  if (sz[2] < sz[0] && sz[2] < sz[1]) comp = 2;
  const float dist = 0.5f * sz[comp];
  if (dist < 0.0f) return false;
  float dij[3], ud[3];
  for (int a = 0; a < 3; ++a) dij[a] = bj.p[a] - bi.p[a];
  const float den = len3(dij[0], dij[1], dij[2]) + 1e-8f;
  for (int a = 0; a < 3; ++a) ud[a] = dij[a] / den;
  const float sg = dij[comp] > 0.0f ? 1.0f : (dij[comp] < 0.0f ? -1.0f : 0.0f);
  for (int a = 0; a < 3; ++a) out->disp[a] = 0.0f;
  out->disp[comp] = sg * dist;
  const float rs = bi.rm + bj.rm;
  out->wi = bi.rm / rs;
  out->wj = bj.rm / rs;
  float dp[3];
  for (int a = 0; a < 3; ++a) dp[a] = (bj.x[a] - bj.p[a]) - (bi.x[a] - bi.p[a]);
  const float d = (dp[0] * ud[0] + dp[1] * ud[1]) + dp[2] * ud[2];
  for (int a = 0; a < 3; ++a) dp[a] = dp[a] - d * ud[a];
  const float mag = len3(dp[0], dp[1], dp[2]);
  float s = 1.0f;
  if (mag < c.mu_s * dist) s = fminf(1.0f, (c.mu_k * dist) / mag);
  for (int a = 0; a < 3; ++a) out->frict[a] = s == 1.0f ? dp[a] : dp[a] * s;
  return true;
}

}  // namespace

extern "C" void orc_pbd_step(const cwa_pbd_params* p, cwa_pbd_box* b, int32_t n, int32_t steps) {
  K c;
  c.n = n;
  for (int a = 0; a < 3; ++a) {
    c.nd[a] = p->grid_cells[a];
    c.lo[a] = p->extents_lo[a];
    c.hi[a] = p->extents_hi[a];
    c.cell[a] = (c.hi[a] - c.lo[a]) / (float)c.nd[a];
    c.g[a] = p->g[a];
  }
  c.dt = p->dt;
  c.damping = p->damping;
  c.k = p->k;
  c.k_static = p->k_static;
  c.sleep = p->sleep_thresh;
  c.mu_k = p->mu_k;
  c.mu_s = p->mu_s;
  c.e = p->e;
  const int ncells = c.nd[0] * c.nd[1] * c.nd[2];
  auto cid = [&](int i, int j, int k) { return (i * c.nd[1] + j) * c.nd[2] + k; };
  for (int s = 0; s < steps; ++s)
    for (int sub = 0; sub < p->substeps; ++sub) {
      // grid of the current positions x (boxes by index in every cell)
      std::vector<std::vector<int>> cells(ncells);
      for (int i = 0; i < n; ++i) {
        int lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
          lo[a] = cell_axis(b[i].x[a] - b[i].hw[a], c.lo[a], c.cell[a], c.nd[a]);
          hi[a] = cell_axis(b[i].x[a] + b[i].hw[a], c.lo[a], c.cell[a], c.nd[a]);
        }
        for (int x = lo[0]; x <= hi[0]; ++x)
          for (int y = lo[1]; y <= hi[1]; ++y)
            for (int z = lo[2]; z <= hi[2]; ++z) cells[cid(x, y, z)].push_back(i);
        for (int a = 0; a < 4; ++a) b[i].color[a] = 1.0f;
      }
      // PreAnimate
      for (int i = 0; i < n; ++i) {
        float v[4];
        for (int a = 0; a < 4; ++a) v[a] = c.damping * (b[i].v[a] + c.dt * (a < 3 ? c.g[a] : 0.0f));
        for (int a = 0; a < 4; ++a) {
          b[i].dp_n[a] = 0.0f;
          b[i].dp_t[a] = 0.0f;
          b[i].p[a] = b[i].x[a] + c.dt * v[a];
          b[i].v[a] = v[a];
        }
        b[i].n = 0.0f;
      }
      // collision query: each box's contacts with the boxes of higher index
      std::vector<std::vector<Pair>> own(n);
      for (int i = 0; i < n; ++i) {
        float qmin[3], qmax[3];
        int lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
          qmin[a] = b[i].p[a] - b[i].hw[a];
          qmax[a] = b[i].p[a] + b[i].hw[a];
          lo[a] = cell_axis(qmin[a], c.lo[a], c.cell[a], c.nd[a]);
          hi[a] = cell_axis(qmax[a], c.lo[a], c.cell[a], c.nd[a]);
        }
        for (int x = lo[0]; x <= hi[0]; ++x)
          for (int y = lo[1]; y <= hi[1]; ++y)
            for (int z = lo[2]; z <= hi[2]; ++z)
              for (int j : cells[cid(x, y, z)]) {
                if (j <= i) continue;
                float bmin[3], bmax[3];
                int home[3];
                for (int a = 0; a < 3; ++a) {
                  bmin[a] = b[j].x[a] - b[j].hw[a];
                  bmax[a] = b[j].x[a] + b[j].hw[a];
                  const int cj = cell_axis(bmin[a], c.lo[a], c.cell[a], c.nd[a]);
                  home[a] = lo[a] > cj ? lo[a] : cj;
                }
                if (home[0] != x || home[1] != y || home[2] != z) continue;
                Pair pr;
                if (!collide(c, b[i], b[j], qmin, qmax, bmin, bmax, &pr)) continue;
                pr.i = i;
                pr.j = j;
                own[i].push_back(pr);
                for (int a = 0; a < 4; ++a) b[i].color[a] = b[j].color[a] = (a == 1 || a == 2) ? 0.0f : 1.0f;
              }
      }
      std::vector<std::vector<const Pair*>> partner(n);
      for (int i = 0; i < n; ++i)
        for (const Pair& pr : own[i]) partner[pr.j].push_back(&pr);
      // walls, own contacts, partner contacts; PostAnimate
      for (int o = 0; o < n; ++o) {
        cwa_pbd_box& q = b[o];
        float dpn[3] = {0, 0, 0}, dpt[3] = {0, 0, 0}, nn = 0.0f;
        for (int a = 0; a < 3; ++a) {
          const float qmin = q.p[a] - q.hw[a], qmax = q.p[a] + q.hw[a];
          const float ov[2] = {c.lo[a] - qmin, qmax - c.hi[a]}, dir[2] = {1.0f, -1.0f};
          for (int m = 0; m < 2; ++m) {
            if (!(ov[m] > 0.0f)) continue;
            dpn[a] = dpn[a] + (dir[m] * c.k_static) * ov[m];
            nn = nn + c.k_static;
            float dp[3];
            for (int r = 0; r < 3; ++r) dp[r] = r == a ? 0.0f : q.x[r] - q.p[r];
            const float mag = len3(dp[0], dp[1], dp[2]);
            float s = 1.0f;
            if (mag < c.mu_s * ov[m]) s = fminf(1.0f, (c.mu_k * ov[m]) / mag);
            for (int r = 0; r < 3; ++r) dpt[r] = dpt[r] + (s == 1.0f ? dp[r] : dp[r] * s);
          }
        }
        for (const Pair& pr : own[o]) {
          for (int a = 0; a < 3; ++a) {
            dpn[a] = dpn[a] + -pr.wi * pr.disp[a];
            dpt[a] = dpt[a] + -pr.wi * pr.frict[a];
          }
          nn = nn + 1.0f;
        }
        for (const Pair* pr : partner[o]) {
          for (int a = 0; a < 3; ++a) {
            dpn[a] = dpn[a] + pr->wj * pr->disp[a];
            dpt[a] = dpt[a] + pr->wj * pr->frict[a];
          }
          nn = nn + 1.0f;
        }
        float pp[3], pe[3];
        for (int a = 0; a < 3; ++a) pp[a] = pe[a] = q.p[a];
        if (nn > 0.0f)
          for (int a = 0; a < 3; ++a) {
            pp[a] = pp[a] + (c.k * (dpt[a] + dpn[a])) / nn;
            pe[a] = pe[a] + (c.k * (dpt[a] + c.e * dpn[a])) / nn;
            q.p[a] = pp[a];
          }
        for (int a = 0; a < 3; ++a) {
          q.v[a] = (pe[a] - q.x[a]) / c.dt;
          q.dp_n[a] = dpn[a];
          q.dp_t[a] = dpt[a];
        }
        q.n = nn;
        if (len3(q.x[0] - pp[0], q.x[1] - pp[1], q.x[2] - pp[2]) > c.sleep)
          for (int a = 0; a < 3; ++a) q.x[a] = pp[a];
      }
    }
}
