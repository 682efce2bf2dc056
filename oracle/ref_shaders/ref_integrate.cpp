// ref_integrate.cpp — CoupledWaterAnimation/integrate_comp.glsl compiled as
// C++ and dispatched over the first n invocations.  TEST INFRASTRUCTURE ONLY.
#include "glsl.h"
#include "ref_shaders.h"

#define REF_INTEGRATE_RUN                                                                \
  int run(double* p16, int n, const float* wave, int w, int h, const ref_uniforms* u) {  \
    if (n < 0 || n > NUM_PARTICLES) return -1;                                           \
    std::vector<Particle> buf;                                                           \
    ref_shaders::load_particles(buf, p16, n);                                            \
    particles = buf.data();                                                              \
    wave_tex = sampler2D{wave, w, h, 1};                                                 \
    upper = ref_shaders::vec4_of<vec4>(u->upper);                                        \
    lower = ref_shaders::vec4_of<vec4>(u->lower);                                        \
    attributes = ref_shaders::vec4_of<vec4>(u->attributes);                              \
    mesh_ws_pos = ref_shaders::vec4_of<vec4>(u->mesh_ws_pos);                            \
    glsl_init_globals();                                                                 \
    _Pragma("omp parallel for schedule(static)")                                         \
    for (int i = 0; i < n; ++i) {                                                        \
      gl_GlobalInvocationID = uvec3((unsigned)i, 0u, 0u);                                \
      main();                                                                            \
    }                                                                                    \
    ref_shaders::store_particles(buf, p16, n);                                           \
    particles = nullptr;                                                                 \
    return 0;                                                                            \
  }

#define GLSL_CONST(name, init) (init)
namespace ref_integrate_f32 {
GLSL_PRELUDE(f32)
#include "integrate_comp.inc"
REF_INTEGRATE_RUN
}  // namespace ref_integrate_f32

#undef GLSL_CONST
#define GLSL_CONST(name, init) (ref_integrate_f32::name)
namespace ref_integrate_f64 {
GLSL_PRELUDE(f64)
#define float double
#include "integrate_comp.inc"
#undef float
REF_INTEGRATE_RUN
}  // namespace ref_integrate_f64

extern "C" int32_t ref_integrate(int32_t prec, double* p16, int32_t n, const float* wave, int32_t w, int32_t h,
                                 const ref_uniforms* u) {
  return prec ? ref_integrate_f64::run(p16, n, wave, w, h, u) : ref_integrate_f32::run(p16, n, wave, w, h, u);
}
