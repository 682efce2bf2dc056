/*
 * cwa_oracle.h — CPU oracle of the coupled SPH + wave step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the correctness checker and the timed
 * CPU baseline; the product (libcwa) never links, loads or calls it.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
 * legs may use it.
 *
 * It restates the reference's GLSL compute shaders in plain C++:
 *   - FP64 versions of every pass (rho_pres, force, integrate, wave) used for
 *     the tolerance checks and the CPU baseline;
 *   - FP32-exact versions of the integer / element-wise parts (cell hash,
 *     stable counting sort, exclusive scan, integrate + fixed-point deposits,
 *     wave stencil, wave init) that the GPU must reproduce bit for bit.
 * Build flags: -O3 -fopenmp -ffp-contract=off (no FMA contraction, so the
 * FP32-exact routines round every operation separately).
 *
 * Parity pinning: the reference's only known-answer test is the exclusive
 * scan (SphWave2D/ParallelScan.cpp:124-155); the scan restatement is pinned
 * to it.  The REFERENCE_3D SPH, integrate and wave restatements are pinned to
 * the reference's compute shaders themselves, compiled for the CPU
 * (oracle/ref_shaders/) and run on seeded inputs whose outputs are committed
 * as tests/golden/ref_shader_outputs.npz.  The MULLER coupling terms are new
 * physics with no reference output.
 *
 * Particle arrays are the 64-byte reference struct widened to double:
 * 16 doubles per particle = pos[4], vel[4], force[4], extras[4].
 */
#ifndef CWA_ORACLE_H
#define CWA_ORACLE_H

#include <stdint.h>

#include "../include/cwa.h"

#ifdef __cplusplus
extern "C" {
#endif

int orc_num_threads(void);
void orc_set_num_threads(int n);

/* ---- FP32-exact integer parts ------------------------------------------ */
/* Exclusive scan, the CPU truth of SphWave2D/ParallelScan.cpp:130-137. */
void orc_exclusive_scan_i32(const int32_t* in, int32_t* out, int32_t n);
/* Cell of a float32 point, UniformGrid2D/ugrid_particles_cs.glsl:97-103,
 * with a cell edge per axis. */
int32_t orc_cell_id_f32(const float p[3], const float lo[3], const float cell[3], const int32_t dims[3]);
/* Stable counting sort (UniformGrid2D/UniformGrid2D.cpp:33-92 with one cell
 * per point): cell_start[ncells+1], sorted_index[n], cell_of[n] (nullable). */
void orc_grid_build_f32(const float* pos4, int32_t n, const float lo[3], const float cell[3],
                        const int32_t dims[3], int32_t* cell_start, int32_t* sorted_index,
                        int32_t* cell_of);
void orc_grid_dims(const cwa_scene_desc* sc, int32_t dims[3]);

/* ---- scene generators (independent restatement of the library's) -------- */
void orc_scene_defaults(int32_t preset, float spacing, cwa_scene_desc* out);
void orc_scene_set_wave_grid(cwa_scene_desc* sc, int32_t nx, int32_t nz);
void orc_make_reference_cube(const cwa_scene_desc* sc, float* p16f, int32_t n);
void orc_make_dam_break(const cwa_scene_desc* sc, const int32_t dims[3], float spacing,
                        float jitter, uint64_t seed, float* p16f, int32_t n);
void orc_make_bumps(const cwa_scene_desc* sc, int32_t n_bumps, uint64_t seed, float* u,
                    int32_t nx, int32_t nz);

/* ---- FP64 passes (particles in any order; p16 = n x 16 doubles) -------- */
/* brute != 0: all-pairs O(N^2) loop as the shaders do; else uniform grid. */
void orc_rho_pres(const cwa_scene_desc* sc, int32_t n, double* p16, const double* u_n,
                  int32_t brute);
void orc_force(const cwa_scene_desc* sc, int32_t n, double* p16, const double* u_n,
               int32_t brute);
/* deposits: nx*nz int64 accumulated (not cleared), may be NULL. */
void orc_integrate(const cwa_scene_desc* sc, int32_t n, double* p16, const double* u_n,
                   int64_t* deposits);
/* u_out = evolve(u_n, u_nm1) + deposits (deposits may be NULL). */
void orc_wave(const cwa_scene_desc* sc, const double* u_n, const double* u_nm1, double* u_out,
              const int64_t* deposits);
/* Full steps in place; wave buffers rotate: after a step u_n holds u^(n+1). */
void orc_step(const cwa_scene_desc* sc, int32_t n, double* p16, double* u_n, double* u_nm1,
              int32_t n_steps, int32_t brute);
/* FP64 totals in CWA_TOTAL_* order. */
void orc_totals(const cwa_scene_desc* sc, int32_t n, const double* p16, const double* u_n,
                const double* u_nm1, double out[CWA_TOTALS_COUNT]);

/* ---- FP32-exact element-wise passes (p16f = n x 16 floats) ------------- */
void orc_integrate_f32(const cwa_scene_desc* sc, int32_t n, float* p16f, const float* u_n,
                       int64_t* deposits);
void orc_wave_f32(const cwa_scene_desc* sc, const float* u_n, const float* u_nm1, float* u_out,
                  const int64_t* deposits);
void orc_wave_init_f32(const cwa_scene_desc* sc, float* u);
/* InitFromImage (wave_comp.glsl:76-80): u(x, y) = red(2x, y) / 255 of an
 * RGBA8 image, 0 past the image. */
void orc_wave_from_image_f32(int32_t nx, int32_t nz, const uint8_t* rgba, int32_t w, int32_t h, float* u);
float orc_sample_f32(const float* u, int32_t w, int32_t h, float s, float t);
/* One headless frame of display() (cwa_render_oracle.cpp): pos4 = n float4
 * particle positions in upload (draw) order, u^n of the scene, optional cube
 * map (6 faces of sky_size^2 RGBA8, or NULL), out = width*height RGBA8. */
void orc_render(const float* pos4, int32_t n, const float* wave, int32_t nx, int32_t nz, const cwa_camera* cam,
                const cwa_render_params* prm, const uint8_t* sky, int32_t sky_size, uint8_t* out);
/* One fragment of each fragment shader, with the inputs the shader reads:
 * particle_fs.glsl pass 0 at pixel (px, py), r sprite widths from the
 * centre, particle at world position pp (inv_p, inv_v: the row-major
 * inverses of P and V; D: the w x h pass-2 depth image); wave_fs.glsl at
 * world position p with wave sample v.  out: r, g, b, a before blending. */
void orc_shade_particle(const float inv_p[16], const float inv_v[16], const float eye[3], const uint8_t* sky,
                        int32_t sky_size, const float* D, int32_t w, int32_t h, int32_t px, int32_t py, float r,
                        const float pp[3], float out[4]);
void orc_shade_wave(const float eye[3], const uint8_t* sky, int32_t sky_size, const float p[3], float v,
                    float out[4]);

/* The 2D solver family (cwa2d_oracle.cpp): SphWave2D's initialisers, one
 * phase of the shallow-water step (float32 op by op), and the two SPH passes
 * in FP64 from an input particle array to an output array. */
void orc2d_init_particles(const cwa2d_params* prm, cwa2d_particle* out);
void orc2d_wave_init_f32(const cwa2d_params* prm, const float* in4, float* out4, int32_t splash);
void orc2d_wave_iter_f32(const cwa2d_params* prm, const float* in4, float* out4, int32_t phase);
/* Wave1D (the 2D family's second wave kind): MODE_INIT_0 / MODE_INIT_1 and
 * one MODE_ITERATE step with free boundaries, float32 op by op; cur4 is the
 * newest field, prev4 the one before. */
void orc2d_wave1d_init_f32(const cwa2d_params* prm, const float* cur4, const float* prev4, float* out4, int32_t mode);
void orc2d_wave1d_iter_f32(const cwa2d_params* prm, const float* cur4, const float* prev4, float* out4);
void orc2d_density(const cwa2d_params* prm, const cwa2d_particle* in, const float* wave4, cwa2d_particle* out);
/* grid_src: the particles the substep's grid was built from (before the
 * density pass), or NULL for `in`. */
void orc2d_force(const cwa2d_params* prm, const cwa2d_particle* in, const cwa2d_particle* grid_src,
                 const float* wave4, cwa2d_particle* out);

/* PBD box collisions (cwa_pbd_oracle.cpp): `steps` frames in place, float32
 * op by op with the library's accumulation order. */
void orc_pbd_step(const cwa_pbd_params* p, cwa_pbd_box* boxes, int32_t n, int32_t steps);

#ifdef __cplusplus
}
#endif
#endif
