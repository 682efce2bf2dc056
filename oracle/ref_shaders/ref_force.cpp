// ref_force.cpp — CoupledWaterAnimation/force_comp.glsl compiled as C++ and
// dispatched over NUM_PARTICLES invocations.  TEST INFRASTRUCTURE ONLY.
#include "glsl.h"
#include "ref_shaders.h"

// Invocation i reads every particle's position, velocity and extras and
// writes only its own force, so the invocations run in any order.
#define REF_FORCE_RUN                                                                    \
  int run(double* p16, int n, const float* wave, int w, int h, const ref_uniforms* u) {  \
    if (n != NUM_PARTICLES) return -1;                                                   \
    std::vector<Particle> buf;                                                           \
    ref_shaders::load_particles(buf, p16, n);                                            \
    particles = buf.data();                                                              \
    wave_tex = sampler2D{wave, w, h, 1};                                                 \
    time = u->time;                                                                      \
    mass = u->mass;                                                                      \
    smoothing_coeff = u->smoothing_coeff;                                                \
    visc = u->visc;                                                                      \
    resting_rho = u->resting_rho;                                                        \
    upper = ref_shaders::vec4_of<vec4>(u->upper);                                        \
    lower = ref_shaders::vec4_of<vec4>(u->lower);                                        \
    attributes = ref_shaders::vec4_of<vec4>(u->attributes);                              \
    glsl_init_globals();                                                                 \
    _Pragma("omp parallel for schedule(dynamic, 64)")                                    \
    for (int i = 0; i < n; ++i) {                                                        \
      gl_GlobalInvocationID = uvec3((unsigned)i, 0u, 0u);                                \
      main();                                                                            \
    }                                                                                    \
    ref_shaders::store_particles(buf, p16, n);                                           \
    particles = nullptr;                                                                 \
    return 0;                                                                            \
  }

#define GLSL_CONST(name, init) (init)
namespace ref_force_f32 {
GLSL_PRELUDE(f32)
#include "force_comp.inc"
REF_FORCE_RUN
}  // namespace ref_force_f32

#undef GLSL_CONST
#define GLSL_CONST(name, init) (ref_force_f32::name)
namespace ref_force_f64 {
GLSL_PRELUDE(f64)
#define float double
#include "force_comp.inc"
#undef float
REF_FORCE_RUN
}  // namespace ref_force_f64

extern "C" int32_t ref_force(int32_t prec, double* p16, int32_t n, const float* wave, int32_t w, int32_t h,
                             const ref_uniforms* u) {
  return prec ? ref_force_f64::run(p16, n, wave, w, h, u) : ref_force_f32::run(p16, n, wave, w, h, u);
}
