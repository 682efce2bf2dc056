// ref_wave.cpp — CoupledWaterAnimation/wave_comp.glsl compiled as C++ and
// dispatched over a w x h image.  TEST INFRASTRUCTURE ONLY.
#include "glsl.h"
#include "ref_shaders.h"

// The shader writes invocation-private globals (anim_mode), so the
// invocations run one after another, each from freshly initialised globals.
// Images are rgba32f: the heights go in the red channel, the others are 0.
#define REF_WAVE_RUN                                                                          \
  int run(const double* un, const double* unm1, double* out, int w, int h, const float* init_rgba, \
          int iw, int ih, const ref_uniforms* u) {                                            \
    using S = decltype(vec4().x);                                                             \
    const bool dbl = sizeof(S) == sizeof(double);                                             \
    std::vector<S> a((size_t)w * h * 4, (S)0), b((size_t)w * h * 4, (S)0), o((size_t)w * h * 4, (S)0); \
    for (size_t k = 0; k < (size_t)w * h; ++k) {                                              \
      a[4 * k] = (S)un[k];                                                                    \
      b[4 * k] = (S)unm1[k];                                                                  \
    }                                                                                         \
    uInputImage0 = image2D{a.data(), w, h, dbl};                                              \
    uInputImage1 = image2D{b.data(), w, h, dbl};                                              \
    uOutputImage = image2D{o.data(), w, h, dbl};                                              \
    uInitImage = sampler2D{init_rgba, iw, ih, 4};                                             \
    time = u->time;                                                                           \
    uMode = u->mode;                                                                          \
    attributes = ref_shaders::vec4_of<vec4>(u->attributes);                                   \
    mesh_ws_pos = ref_shaders::vec4_of<vec4>(u->mesh_ws_pos);                                 \
    for (int y = 0; y < h; ++y)                                                               \
      for (int x = 0; x < w; ++x) {                                                           \
        gl_GlobalInvocationID = uvec3((unsigned)x, (unsigned)y, 0u);                          \
        glsl_init_globals();                                                                  \
        main();                                                                               \
      }                                                                                       \
    for (size_t k = 0; k < (size_t)w * h; ++k) out[k] = (double)o[4 * k];                     \
    return 0;                                                                                 \
  }

#define GLSL_CONST(name, init) (init)
namespace ref_wave_f32 {
GLSL_PRELUDE(f32)
#include "wave_comp.inc"
REF_WAVE_RUN
}  // namespace ref_wave_f32

#undef GLSL_CONST
#define GLSL_CONST(name, init) (ref_wave_f32::name)
namespace ref_wave_f64 {
GLSL_PRELUDE(f64)
#define float double
#include "wave_comp.inc"
#undef float
REF_WAVE_RUN
}  // namespace ref_wave_f64

extern "C" int32_t ref_wave(int32_t prec, const double* u_n, const double* u_nm1, double* out, int32_t w,
                            int32_t h, const float* init_rgba, int32_t iw, int32_t ih, const ref_uniforms* u) {
  return prec ? ref_wave_f64::run(u_n, u_nm1, out, w, h, init_rgba, iw, ih, u)
              : ref_wave_f32::run(u_n, u_nm1, out, w, h, init_rgba, iw, ih, u);
}
