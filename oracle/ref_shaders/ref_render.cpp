// ref_render.cpp — the reference's fragment shaders compiled as C++:
// CoupledWaterAnimation/particle_fs.glsl (pass 0, the shaded sprite) and
// wave_fs.glsl, run for one fragment at a time with the inputs the raster
// pipeline would hand them (the interpolated VertexData block,
// gl_FragCoord, gl_PointCoord, the bound textures and uniforms).
// TEST INFRASTRUCTURE ONLY.
#include "glsl.h"
#include "ref_shaders.h"

#define GLSL_CONST(name, init) (init)

namespace ref_particle_fs {
GLSL_PRELUDE(f32)
vec4 gl_FragCoord;
vec2 gl_PointCoord;
bool glsl_discarded = false;
#define discard            \
  do {                     \
    glsl_discarded = true; \
    return;                \
  } while (0)
#include "particle_fs.inc"
#undef discard
}  // namespace ref_particle_fs

namespace ref_wave_fs {
GLSL_PRELUDE(f32)
#include "wave_fs.inc"
}  // namespace ref_wave_fs

namespace {
template <class M>
void set_mat(M& m, const float* colmajor) {
  for (int k = 0; k < 16; ++k) m.m[k] = colmajor[k];
}
}  // namespace

extern "C" int32_t ref_particle_fragment(const ref_render_inputs* in, const float pp[3], float depth, float px,
                                         float py, const float point_coord[2], float out[4]) {
  using namespace ref_particle_fs;
  set_mat(P, in->P);
  set_mat(V, in->V);
  set_mat(PV, in->PV);
  eye_w = vec4(in->eye[0], in->eye[1], in->eye[2], 1.0f);
  pass = 0;
  time = 0.0f;
  skybox_tex = samplerCube{in->sky, in->sky_size};
  depth_tex = sampler2D{in->depth_image, in->w, in->h, 1};
  fbo_tex = sampler2D{};
  inData.particle_pos = vec3(pp[0], pp[1], pp[2]);
  inData.depth = depth;
  gl_FragCoord = vec4(px, py, 0.5f, 1.0f);
  gl_PointCoord = vec2(point_coord[0], point_coord[1]);
  glsl_discarded = false;
  glsl_init_globals();
  main();
  for (int c = 0; c < 4; ++c) out[c] = frag_color.e[c];
  return glsl_discarded ? 1 : 0;
}

extern "C" int32_t ref_wave_fragment(const ref_render_inputs* in, const float pw[3], const float nw[3], float v,
                                     float out[4]) {
  using namespace ref_wave_fs;
  eye_w = vec4(in->eye[0], in->eye[1], in->eye[2], 1.0f);
  skybox_tex = samplerCube{in->sky, in->sky_size};
  // the wave sample: a 2 x 2 texture of v read at a texel centre returns v
  const float tex[4] = {v, v, v, v};
  wave_tex = sampler2D{tex, 2, 2, 1};
  inData.tex_coord = vec2(0.25f, 0.25f);
  inData.pw = vec3(pw[0], pw[1], pw[2]);
  inData.nw = vec3(nw[0], nw[1], nw[2]);
  glsl_init_globals();
  main();
  for (int c = 0; c < 4; ++c) out[c] = fragcolor.e[c];
  return 0;
}
