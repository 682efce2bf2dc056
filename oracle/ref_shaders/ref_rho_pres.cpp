// ref_rho_pres.cpp — CoupledWaterAnimation/rho_pres_comp.glsl compiled as C++
// (the generated rho_pres_comp.inc: the shader with its declarations
// rewritten by glsl_to_cpp.py) and dispatched over NUM_PARTICLES
// invocations.  TEST INFRASTRUCTURE ONLY.
#include "glsl.h"
#include "ref_shaders.h"

// One dispatch: bind the particle buffer, the wave texture and the uniform
// blocks, run every invocation (they write only their own particle), copy
// the buffer back.
#define REF_RHO_PRES_RUN                                                                 \
  int run(double* p16, int n, const float* wave, int w, int h, const ref_uniforms* u) {  \
    if (n != NUM_PARTICLES) return -1;                                                   \
    std::vector<Particle> buf;                                                           \
    ref_shaders::load_particles(buf, p16, n);                                            \
    particles = buf.data();                                                              \
    wave_tex = sampler2D{wave, w, h, 1};                                                 \
    mass = u->mass;                                                                      \
    smoothing_coeff = u->smoothing_coeff;                                                \
    visc = u->visc;                                                                      \
    resting_rho = u->resting_rho;                                                        \
    upper = ref_shaders::vec4_of<vec4>(u->upper);                                        \
    lower = ref_shaders::vec4_of<vec4>(u->lower);                                        \
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
namespace ref_rho_pres_f32 {
GLSL_PRELUDE(f32)
#include "rho_pres_comp.inc"
REF_RHO_PRES_RUN
}  // namespace ref_rho_pres_f32

#undef GLSL_CONST
#define GLSL_CONST(name, init) (ref_rho_pres_f32::name)
namespace ref_rho_pres_f64 {
GLSL_PRELUDE(f64)
#define float double
#include "rho_pres_comp.inc"
#undef float
REF_RHO_PRES_RUN
}  // namespace ref_rho_pres_f64

extern "C" int32_t ref_rho_pres(int32_t prec, double* p16, int32_t n, const float* wave, int32_t w, int32_t h,
                                const ref_uniforms* u) {
  return prec ? ref_rho_pres_f64::run(p16, n, wave, w, h, u) : ref_rho_pres_f32::run(p16, n, wave, w, h, u);
}
