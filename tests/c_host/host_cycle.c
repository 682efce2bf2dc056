/* host_cycle.c — a plain C host driving libcwa through include/cwa.h only,
 * the way an integrator's application would (no Python, no CUDA headers).
 *
 *   host_cycle nodevice : a machine without a usable GPU; cwa_create must
 *                         fail cleanly with CWA_ERR_NO_DEVICE and argument
 *                         errors must be reported without touching a device.
 *   host_cycle gpu      : one coupled scene through its whole life: build,
 *                         upload, 20 graph steps, FP64 totals (mass exact),
 *                         download, size errors, checkpoint round trip,
 *                         destroy.
 * Exit status 0 on success; a failing check exits with its own code. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cwa.h"

#define CHECK(x)                                                                                \
  do {                                                                                          \
    cwa_status s_ = (x);                                                                        \
    if (s_ != CWA_OK) {                                                                         \
      fprintf(stderr, "%s: %s (%s)\n", #x, cwa_status_str(s_), cwa_last_error());              \
      return 100 + (int)s_;                                                                     \
    }                                                                                           \
  } while (0)

int main(int argc, char** argv) {
  const int gpu = argc > 1 && strcmp(argv[1], "gpu") == 0;
  if (cwa_abi_version() != CWA_ABI_VERSION) return 2;
  if (strcmp(cwa_status_str(CWA_OK), "ok") != 0) return 3;

  cwa_scene_desc d;
  CHECK(cwa_scene_defaults(CWA_PRESET_MULLER, 0.03f, &d));
  CHECK(cwa_scene_set_wave_grid(&d, 64, 48));
  const int32_t dims[3] = {10, 8, 9};
  const int32_t n = dims[0] * dims[1] * dims[2];
  d.n_particles = n;
  cwa_particle* p = (cwa_particle*)malloc(sizeof(cwa_particle) * (size_t)n);
  float* u = (float*)malloc(sizeof(float) * 64 * 48);
  CHECK(cwa_make_dam_break(&d, dims, 0.03f, 0.05f, 7u, p, n));
  CHECK(cwa_make_bumps(&d, 4, 11u, u, 64, 48));
  if (cwa_scene_defaults(7, 0.03f, &d) != CWA_ERR_INVALID_ARG) return 4;  /* unknown preset */
  CHECK(cwa_scene_defaults(CWA_PRESET_MULLER, 0.03f, &d));
  CHECK(cwa_scene_set_wave_grid(&d, 64, 48));
  d.n_particles = n;

  cwa_sim* sim = NULL;
  const cwa_status st = cwa_create(NULL, &d, 1, &sim);
  if (!gpu) {
    if (st != CWA_ERR_NO_DEVICE || sim != NULL) {
      fprintf(stderr, "cwa_create without a device: %s\n", cwa_status_str(st));
      return 5;
    }
    if (cwa_step(NULL, 1) != CWA_ERR_INVALID_ARG) return 6;
    if (cwa_create(NULL, &d, 0, &sim) != CWA_ERR_INVALID_ARG) return 7;
    printf("ok nodevice\n");
    return 0;
  }
  CHECK(st);
  CHECK(cwa_upload_particles(sim, 0, p, n));
  CHECK(cwa_upload_wave(sim, 0, u, u, 64, 48));
  double t0[CWA_TOTALS_COUNT], t1[CWA_TOTALS_COUNT];
  CHECK(cwa_reduce_totals(sim, 0, t0));
  CHECK(cwa_step(sim, 20));
  CHECK(cwa_synchronize(sim));
  CHECK(cwa_reduce_totals(sim, 0, t1));
  if (t0[CWA_TOTAL_MASS] != t1[CWA_TOTAL_MASS]) return 8; /* mass is exact */
  int64_t steps = 0;
  CHECK(cwa_get_step_count(sim, &steps));
  if (steps != 20) return 9;
  CHECK(cwa_download_particles(sim, 0, p, n));
  for (int32_t i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a)
      if (!isfinite(p[i].pos[a]) || p[i].pos[a] < d.box_lo[a] - 1e-4f || p[i].pos[a] > d.box_hi[a] + 1e-4f)
        return 10;
  if (cwa_upload_particles(sim, 0, p, n - 1) != CWA_ERR_INVALID_ARG) return 11;
  if (cwa_upload_particles(sim, 1, p, n) != CWA_ERR_INVALID_ARG) return 12;
  if (cwa_download_wave(sim, 0, u, NULL, 63, 48) != CWA_ERR_INVALID_ARG) return 13;

  /* checkpoint: save, step, load, step again: the two runs agree bit for bit */
  const char* path = argc > 2 ? argv[2] : "host_cycle.ckpt";
  cwa_particle* a = (cwa_particle*)malloc(sizeof(cwa_particle) * (size_t)n);
  CHECK(cwa_save(sim, path));
  CHECK(cwa_step(sim, 5));
  CHECK(cwa_download_particles(sim, 0, a, n));
  CHECK(cwa_load(sim, path));
  CHECK(cwa_step(sim, 5));
  CHECK(cwa_download_particles(sim, 0, p, n));
  if (memcmp(a, p, sizeof(cwa_particle) * (size_t)n) != 0) return 14;
  remove(path);
  CHECK(cwa_destroy(sim));
  printf("ok gpu: %d particles, mass %.9g conserved over 20 steps\n", n, t1[CWA_TOTAL_MASS]);
  free(a);
  free(p);
  free(u);
  return 0;
}
