// ref_shaders.h — the reference's four compute shaders
// (CoupledWaterAnimation/{rho_pres,force,integrate,wave}_comp.glsl) compiled
// as C++ and dispatched on the CPU.  TEST INFRASTRUCTURE ONLY: the oracle's
// check against the reference's own code.  Built from the reference's
// sources into oracle/_ref/ (oracle/ref_shaders/Makefile); nothing under
// oracle/_ref/ is committed.
//
// prec 0 runs the shaders' float arithmetic, prec 1 the same source with
// float promoted to double.  Particles are n records of 16 doubles (pos,
// vel, force, extras: the shaders' Particle, CoupledWaterAnimation/
// rho_pres_comp.glsl:16-22); heights are the red channel of the wave image,
// row-major w x h (row = texture t).  Every call returns 0, or -1 when n is
// not what the shader's NUM_PARTICLES loop needs.
#pragma once

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// The uniform blocks the shaders read (Main.cpp binds them; names as in the
// shaders): ConstantsUniform, BoundaryUniform, WaveUniforms, and the loose
// uniforms time and uMode.
typedef struct ref_uniforms {
  float mass, smoothing_coeff, visc, resting_rho;
  float upper[4], lower[4];
  float attributes[4], mesh_ws_pos[4];
  float time;
  int32_t mode;
} ref_uniforms;

// rho_pres_comp.glsl over all NUM_PARTICLES (20480) particles: writes extras.x, .y.
int32_t ref_rho_pres(int32_t prec, double* p16, int32_t n, const float* wave, int32_t w, int32_t h,
                     const ref_uniforms* u);
// force_comp.glsl over all NUM_PARTICLES particles: writes force.
int32_t ref_force(int32_t prec, double* p16, int32_t n, const float* wave, int32_t w, int32_t h,
                  const ref_uniforms* u);
// integrate_comp.glsl over the first n <= NUM_PARTICLES particles.
int32_t ref_integrate(int32_t prec, double* p16, int32_t n, const float* wave, int32_t w, int32_t h,
                      const ref_uniforms* u);
// wave_comp.glsl in mode u->mode (0 InitWave, 1 InitFromImage, 2 EvolveWave)
// over a w x h image: u_n is image 0 (t-1), u_nm1 image 1 (t-2), the result
// the output image's red channel.  init_rgba: iw x ih RGBA texels (already
// normalised to [0, 1]) for InitFromImage, else null.
int32_t ref_wave(int32_t prec, const double* u_n, const double* u_nm1, double* out, int32_t w, int32_t h,
                 const float* init_rgba, int32_t iw, int32_t ih, const ref_uniforms* u);

// The 2D family (SphWave2D).  Particles are n records of 12 doubles (pos,
// vel, acc: SphWaveKoschier2D_grid_cs.glsl:39-44); fields are n cells of 4
// floats (rgba32f image1D).
typedef struct ref2d_uniforms {
  float time, bottom;                  // SphWaveKoschier2D_grid_cs.glsl uniforms
  int32_t grid_cells[2];               // UniformGridSph2D: 32 x 32
  float extent_max[2];                 // over [0, extent_max]: 9.6 x 9.6
  float lambda, dx, atten, beta;       // Shallow1D / Wave1D uniforms
  float boundary[2];
} ref2d_uniforms;

// The grid of `in`, then one mode (0 init, 1 density/pressure, 2 forces)
// reading `in`, writing `out`.  -1 unless the cell count is a power of two.
int32_t ref2d_sph(int32_t prec, int32_t mode, const double* in12, double* out12, int32_t n, const float* wave4,
                  int32_t wave_n, const ref2d_uniforms* u);
// One substep as SphUgrid::Compute runs it: the grid of `in`, density
// (in -> dens), forces (dens -> force) on that same grid.
int32_t ref2d_substep(int32_t prec, const double* in12, double* dens12, double* force12, int32_t n,
                      const float* wave4, int32_t wave_n, const ref2d_uniforms* u);
// One dispatch of Shallow1D_cs.glsl (kind 0; image in0) or Wave1D_cs.glsl
// (kind 1; images in0 = t-1, in1 = t-2) in `mode`; out4 holds the output
// image (cells the dispatch does not write keep their values).
int32_t ref2d_field(int32_t kind, int32_t mode, const float* in0, const float* in1, float* out4, int32_t n,
                    const float* init4, int32_t init_n, const ref2d_uniforms* u);

// PBD boxes (UniformGrid2D/uniform_grid_pbd_3D_cs.glsl): records of 32
// doubles (PbdObj: color, x, v, p, dp_t, dp_n, hw, then rm, n, e, padding).
typedef struct ref_pbd_params {
  int32_t grid_cells[3];
  float lo[3], hi[3];
  float g[3], dt, damping, k, k_static, sleep_thresh, mu_k, mu_s, e;
  int32_t substeps;
} ref_pbd_params;

// `frames` frames of GridTestPbdGpu3D::Animate.  -1 unless the grid has
// nx == nz and a power-of-two cell count.
int32_t ref_pbd(int32_t prec, double* b32, int32_t n, int32_t frames, const ref_pbd_params* q);

// The fragment shaders, one fragment at a time.  Matrices column-major (as
// GLSL stores them); sky: 6 faces of sky_size^2 RGBA8 (+x, -x, +y, -y, +z,
// -z); depth_image: the w x h pass-2 depth texture (its red channel).
typedef struct ref_render_inputs {
  float P[16], V[16], PV[16];
  float eye[3];
  const uint8_t* sky;
  int32_t sky_size;
  const float* depth_image;
  int32_t w, h;
} ref_render_inputs;

// particle_fs.glsl pass 0 at window position (px, py) (gl_FragCoord.xy)
// with gl_PointCoord point_coord: out = frag_color; returns 1 when the
// fragment was discarded.
int32_t ref_particle_fragment(const ref_render_inputs* in, const float pp[3], float depth, float px, float py,
                              const float point_coord[2], float out[4]);
// wave_fs.glsl with the interpolated world position pw, normal nw and wave
// sample v: out = fragcolor.
int32_t ref_wave_fragment(const ref_render_inputs* in, const float pw[3], const float nw[3], float v, float out[4]);

#ifdef __cplusplus
}

#include <stddef.h>

#include <vector>

namespace ref_shaders {

template <class P>
void load_particles(std::vector<P>& v, const double* p16, int n) {
  v.resize((size_t)n);
  for (int i = 0; i < n; ++i) {
    const double* q = p16 + 16 * (size_t)i;
    for (int c = 0; c < 4; ++c) {
      v[i].pos.e[c] = q[c];
      v[i].vel.e[c] = q[4 + c];
      v[i].force.e[c] = q[8 + c];
      v[i].extras.e[c] = q[12 + c];
    }
  }
}

template <class P>
void store_particles(const std::vector<P>& v, double* p16, int n) {
  for (int i = 0; i < n; ++i) {
    double* q = p16 + 16 * (size_t)i;
    for (int c = 0; c < 4; ++c) {
      q[c] = v[i].pos.e[c];
      q[4 + c] = v[i].vel.e[c];
      q[8 + c] = v[i].force.e[c];
      q[12 + c] = v[i].extras.e[c];
    }
  }
}

template <class V>
V vec4_of(const float* a) {
  return V(a[0], a[1], a[2], a[3]);
}

}  // namespace ref_shaders
#endif
