"""The GLSL -> C++ rewrite that compiles the reference's shaders for the CPU
(oracle/ref_shaders/glsl_to_cpp.py), checked rule by rule on small shaders
written here, and end to end: a synthetic compute shader rewritten, compiled
against glsl.h in its float and double builds, dispatched, and compared with
the same arithmetic in numpy.  Needs no reference checkout and no GPU."""
from __future__ import annotations

import importlib.util
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
SHADERS = ROOT / "oracle" / "ref_shaders"


def _load():
    spec = importlib.util.spec_from_file_location("glsl_to_cpp", SHADERS / "glsl_to_cpp.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


g2c = _load()


def _squash(s: str) -> str:
    return " ".join(s.split())


def test_version_extension_and_local_size_are_dropped():
    out = g2c.transform("#version 450\n#extension GL_ARB_x : enable\nlayout(local_size_x = 64) in;\nvoid main() {}\n")
    assert "#version" not in out and "#extension" not in out and "local_size" not in out
    assert "void main() {}" in out


def test_comments_are_stripped_in_one_pass():
    # "//*" is a line comment (a block toggle), not the start of a block comment
    out = g2c.transform("//* toggle\nint a = 1;\n/* block // with a line marker */ int b = 2;\n//*/\nint c = 3;\n")
    assert "toggle" not in out and "block" not in out
    for decl in ("int a", "int b", "int c"):
        assert decl in out


@pytest.mark.parametrize("src, want", [
    ("x = 1.5;", "x = 1.5f;"),
    ("x = .5;", "x = .5f;"),
    ("x = 2.;", "x = 2.f;"),
    ("x = 1e5;", "x = 1e5f;"),
    ("x = 2.5E-3;", "x = 2.5E-3f;"),
    ("x = 1.0f;", "x = 1.0f;"),
    ("x = 1.0lf;", "x = 1.0;"),
    ("x = 3;", "x = 3;"),
    ("x = 3u;", "x = 3u;"),
    ("x = 0x1e5;", "x = 0x1e5;"),
    ("x = vec2(1.0, a1);", "x = vec2(1.0f, a1);"),
])
def test_float_literals_follow_glsl_typing(src, want):
    assert g2c._float_literals(src) == want


def test_parameter_qualifiers_become_references():
    out = g2c.transform("void f(inout vec3 a, out float b, in int c) { b = 1.0; }\n")
    assert "void f(vec3& a, float& b, int c)" in _squash(out)


def test_interface_blocks_become_globals():
    src = ("layout(std430, binding = 0) buffer Data { float vals[]; int n; };\n"
           "layout(std140, binding = 1) uniform Params { float bias; int count; } params;\n"
           "in vec3 pos_attrib;\nout vec4 color;\n")
    out = _squash(g2c.transform(src))
    assert "float* vals = nullptr;" in out and "int n;" in out
    assert "struct Params { float bias; int count; }; Params params;" in out
    assert "vec3 pos_attrib;" in out and "vec4 color;" in out
    assert "buffer" not in out and "layout" not in out and "uniform" not in out


def test_globals_split_into_constants_and_deferred_initialisers():
    src = ("#define N 4\nconst float A = 0.1;\nconst float B = A * 3.0;\nconst int K = N * 2;\n"
           "uniform float gain = 0.7;\nuniform float level;\nfloat scratch = B + 1.0;\n"
           "const float C = level * 2.0;\n")
    out = _squash(g2c.transform(src))
    assert "const glsl_cfloat A = GLSL_CONST(A, 0.1f);" in out
    assert "const glsl_cfloat B = GLSL_CONST(B, A * 3.0f);" in out
    assert "const int K = N * 2;" in out
    assert "glsl_cfloat gain = GLSL_CONST(gain, 0.7f);" in out
    # a non-const global and a const one that reads a uniform are initialised per dispatch
    assert "float scratch;" in out and "float C;" in out
    init = out[out.index("void glsl_init_globals()"):]
    assert "scratch = B + 1.0f;" in init and "C = level * 2.0f;" in init


SYNTHETIC = """#version 450
#extension GL_ARB_shading_language_420pack : enable
layout(local_size_x = 64) in;
//* a block toggle left on
const float C0 = 0.1;
const float C1 = C0 * 3.0;                     /* folded in float */
uniform float gain = 0.7;
layout(std430, binding = 0) buffer Data { float vals[]; };
layout(std140, binding = 1) uniform Params { float bias; int count; } params;
float scratch = C1 + 1e-3;

void accumulate(inout float acc, in float x, out float y)
{
    acc += x * C1;
    y = x + 2.5e1;
}

void main()
{
    uint i = gl_GlobalInvocationID.x;
    if (i >= uint(params.count)) return;
    float acc = params.bias;
    float y;
    accumulate(acc, vals[i], y);
    vals[i] = acc * gain + y + scratch + 1e2;
}
"""

HARNESS = r"""
#include "glsl.h"
#include <cstdio>
#include <vector>

#define RUN                                                         \
  void run(const double* in, int n, double bias) {                  \
    using S = decltype(vec4().x);                                   \
    std::vector<S> v(in, in + n);                                   \
    vals = v.data();                                                \
    params.bias = (S)bias;                                          \
    params.count = n;                                               \
    for (int k = 0; k < n + 3; ++k) {                               \
      gl_GlobalInvocationID = uvec3((unsigned)k, 0u, 0u);           \
      glsl_init_globals();                                          \
      main();                                                       \
    }                                                               \
    for (int k = 0; k < n; ++k) std::printf("%.17g\n", (double)v[k]); \
  }

#define GLSL_CONST(name, init) (init)
namespace t32 {
GLSL_PRELUDE(f32)
#include "synthetic.inc"
RUN
}  // namespace t32
#undef GLSL_CONST
#define GLSL_CONST(name, init) (t32::name)
namespace t64 {
GLSL_PRELUDE(f64)
#define float double
#include "synthetic.inc"
#undef float
RUN
}  // namespace t64

int main() {
  const double in[5] = {0.0, 1.0, -2.75, 3.3333333333333335, 1.0e-7};
  t32::run(in, 5, 0.625);
  t64::run(in, 5, 0.625);
  return 0;
}
"""


def _expected(x: np.ndarray, bias: float):
    f = np.float32
    c0 = f(0.1)
    c1 = f(c0 * f(3.0))
    gain = f(0.7)
    xs = x.astype(np.float32)
    scratch = f(c1 + f(1e-3))
    acc = f(bias) + xs * c1
    y = xs + f(25.0)
    out32 = ((acc * gain + y) + scratch) + f(100.0)
    # the double build: the float build's constants, double arithmetic
    d = np.float64
    c1d, gaind = d(c1), d(gain)
    scratch_d = c1d + d(f(1e-3))
    acc_d = d(bias) + x * c1d
    out64 = ((acc_d * gaind + (x + 25.0)) + scratch_d) + 100.0
    return out32, out64


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_synthetic_shader_runs_in_float_and_double(tmp_path):
    (tmp_path / "synthetic.inc").write_text(g2c.transform(SYNTHETIC))
    (tmp_path / "harness.cpp").write_text(HARNESS)
    exe = tmp_path / "harness"
    subprocess.run(["g++", "-std=c++20", "-O1", "-ffp-contract=off", "-fno-fast-math", f"-I{SHADERS}",
                    f"-I{tmp_path}", "-o", str(exe), str(tmp_path / "harness.cpp")], check=True,
                   capture_output=True, text=True)
    got = np.array([float(v) for v in subprocess.run([str(exe)], check=True, capture_output=True,
                                                     text=True).stdout.split()])
    x = np.array([0.0, 1.0, -2.75, 3.3333333333333335, 1.0e-7])
    want32, want64 = _expected(x, 0.625)
    # float build: every operation rounded to float, literals and constants included
    np.testing.assert_array_equal(got[:5].astype(np.float32), want32)
    # double build: the same constants, arithmetic in double (not the float result)
    np.testing.assert_array_equal(got[5:], want64)
    assert not np.array_equal(got[5:], want32.astype(np.float64))
