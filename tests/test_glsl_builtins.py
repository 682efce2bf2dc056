"""The GLSL built-ins of oracle/ref_shaders/glsl.h, which the reference's
shaders compile against for the CPU pins, checked against the GLSL 4.50 and
GL 4.5 core definitions restated in numpy: one rounding per operation in the
order the definitions write, in float for the float build and in double
for the double build.  A wrong built-in would move every pin built on it,
so each one the shaders use is compared bit for bit on seeded inputs,
edges included (clamped texture coordinates, NaN operands of max/min,
total internal reflection, every cube-map face, out-of-range texelFetch and
imageLoad).  Needs g++, not the reference or a GPU."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
SHADERS = ROOT / "oracle" / "ref_shaders"
N = 2000
TW, TH, T1, CS = 7, 5, 9, 4  # 2D texture w x h, 1D texture w, cube face size

HARNESS = r"""
#include "glsl.h"
#include <cstdio>
#include <cstdlib>
#include <vector>

constexpr int kN = @N@, kTW = @TW@, kTH = @TH@, kT1 = @T1@, kCS = @CS@;

template <class T> std::vector<T> slurp(const char* path, size_t n) {
  std::vector<T> v(n);
  FILE* f = std::fopen(path, "rb");
  if (!f || std::fread(v.data(), sizeof(T), n, f) != n) std::abort();
  std::fclose(f);
  return v;
}

#define RUN(NS, TAG)                                                                        \
  {                                                                                         \
    using namespace glsl::NS;                                                               \
    using S = scalar;                                                                       \
    auto in = slurp<double>("in.bin", (size_t)kN * 14);                                      \
    auto tex = slurp<float>("tex2d.bin", (size_t)kTW * kTH * 4);                              \
    auto tex1 = slurp<float>("tex1d.bin", (size_t)kT1 * 4);                                \
    glsl::sampler2D t2{tex.data(), kTW, kTH, 4};                                              \
    glsl::sampler1D t1{tex1.data(), kT1, 4};                                               \
    auto cube = slurp<uint8_t>("cube.bin", (size_t)6 * kCS * kCS * 4);                      \
    glsl::samplerCube tc{cube.data(), kCS};                                                 \
    std::vector<S> img((size_t)kTW * kTH * 4);                                              \
    for (size_t e = 0; e < img.size(); ++e) img[e] = (S)tex[e];                             \
    glsl::image2D im{img.data(), kTW, kTH, sizeof(S) == sizeof(double)};                    \
    FILE* o = std::fopen(TAG ".bin", "wb");                                                 \
    auto put = [&](S v) { double d = (double)v; std::fwrite(&d, sizeof d, 1, o); };        \
    for (int k = 0; k < kN; ++k) {                                                         \
      const double* q = &in[(size_t)k * 14];                                                \
      const S a = (S)q[0], b = (S)q[1], c = (S)q[2];                                        \
      const vec3 u((S)q[3], (S)q[4], (S)q[5]), v((S)q[6], (S)q[7], (S)q[8]);                \
      put(smoothstep(a, b, c));                                                             \
      put(mix(a, b, c));                                                                    \
      put(fract(a));                                                                        \
      put(sign(a));                                                                         \
      put(clamp(a, b, c));                                                                  \
      put(max(a, b));                                                                       \
      put(min(a, b));                                                                       \
      put(length(u));                                                                       \
      const vec3 nu = normalize(u), rf = reflect(u, nu), rr = refract(nu, normalize(v), c); \
      const vec3 cr = cross(u, v);                                                          \
      put(nu.x); put(nu.y); put(nu.z);                                                      \
      put(rf.x); put(rf.y); put(rf.z);                                                      \
      put(rr.x); put(rr.y); put(rr.z);                                                      \
      put(cr.x); put(cr.y); put(cr.z);                                                      \
      put(dot(u, v));                                                                       \
      const vec4 s2 = texture(t2, vec2((S)q[9], (S)q[10]));                                 \
      const vec4 s1 = texture(t1, (S)q[11]);                                                \
      const vec4 f2 = texelFetch(t2, glsl::ivec2((int)q[12] - 2, (int)q[13] - 2), 0);       \
      const vec4 sc = texture(tc, u);                                                       \
      const vec4 il = imageLoad(im, glsl::ivec2((int)q[12] - 2, (int)q[13] - 2));           \
      for (int e = 0; e < 4; ++e) {                                                         \
        put(s2.e[e]); put(s1.e[e]); put(f2.e[e]); put(sc.e[e]); put(il.e[e]);               \
      }                                                                                     \
    }                                                                                       \
    std::fclose(o);                                                                         \
  }

int main() {
  RUN(f32, "f32")
  RUN(f64, "f64")
  return 0;
}
"""

OUTS = ["smoothstep", "mix", "fract", "sign", "clamp", "max", "min", "length",
        "nx", "ny", "nz", "rfx", "rfy", "rfz", "rrx", "rry", "rrz", "crx", "cry", "crz", "dot"] + \
       [f"{kind}{e}" for e in range(4) for kind in ("tex2d", "tex1d", "fetch", "cube", "iload")]


def _inputs():
    rng = np.random.default_rng(2024)
    q = np.empty((N, 14))
    q[:, 0] = rng.uniform(-3, 3, N)
    q[:, 1] = q[:, 0] + rng.uniform(0.01, 4, N)  # e1 > e0 for smoothstep, hi >= lo ...
    q[:, 2] = rng.uniform(-2, 3, N)
    q[:, 3:9] = rng.uniform(-4, 4, (N, 6))
    q[:, 9:11] = rng.uniform(-0.3, 1.3, (N, 2))  # outside [0, 1]: clamped to the edge texels
    q[:, 11] = rng.uniform(-0.3, 1.3, N)
    q[:8, 0] = [0.0, -0.0, 2.0, -2.0, 1.5, -1.5, 3.0, -3.0]  # exact floors, signed zeros
    q[8, 0], q[9, 1] = np.nan, np.nan  # max / min with a NaN operand
    q[10:20, 2] = np.linspace(1.2, 3.0, 10)  # eta > 1: total internal reflection for grazing rays
    # texel coordinates for texelFetch: -2 .. TW + 1 (and TH + 1) after the harness's -2 offset
    q[:, 12] = np.floor(rng.uniform(0, TW + 4, N))
    q[:, 13] = np.floor(rng.uniform(0, TH + 4, N))
    tex2 = rng.uniform(0, 1, (TH, TW, 4)).astype(np.float32)
    tex1 = rng.uniform(0, 1, (T1, 4)).astype(np.float32)
    cube = rng.integers(0, 256, (6, CS, CS, 4), dtype=np.uint8)
    q[20:26, 3:6] = [[1, 0.5, -0.25], [-1, 0.25, 0.5], [0.5, 1, 0.25], [0.25, -1, -0.5], [0.5, 0.25, 1],
                     [-0.25, 0.5, -1]]  # one direction into each cube face
    return q, tex2, tex1, cube


def _spec(q, tex2, tex1, cube, T):
    """The GLSL / GL definitions in numpy at scalar type T, one rounding per
    operation in the definitions' order."""
    one, zero, two, half = T(1), T(0), T(2), T(0.5)
    a, b, c = q[:, 0].astype(T), q[:, 1].astype(T), q[:, 2].astype(T)
    u, v = q[:, 3:6].astype(T), q[:, 6:9].astype(T)
    with np.errstate(all="ignore"):
        def glmax(x, y):  # y if x < y, else x
            return np.where(x < y, y, x)

        def glmin(x, y):  # y if y < x, else x
            return np.where(y < x, y, x)

        def clamp(x, lo, hi):
            return glmin(glmax(x, lo), hi)

        def dot(p, r):
            return (p[:, 0] * r[:, 0] + p[:, 1] * r[:, 1]) + p[:, 2] * r[:, 2]

        def normalize(p):
            ln = np.sqrt(dot(p, p))
            return p / ln[:, None]

        t = clamp((c - a) / (b - a), zero, one)
        out = {"smoothstep": t * t * (T(3) - two * t),
               "mix": a * (one - c) + b * c,
               "fract": a - np.floor(a),
               "sign": np.where(a > 0, one, np.where(a < 0, -one, zero)),
               "clamp": clamp(a, b, c),
               "max": glmax(a, b), "min": glmin(a, b),
               "length": np.sqrt(dot(u, u)),
               "dot": dot(u, v)}
        nu = normalize(u)
        rf = u - (two * dot(nu, u))[:, None] * nu
        nv = normalize(v)
        d = dot(nv, nu)
        k = one - c * c * (one - d * d)
        rr = c[:, None] * nu - (c * d + np.sqrt(np.where(k < 0, zero, k)))[:, None] * nv
        rr[k < 0] = zero
        cr = np.stack([u[:, 1] * v[:, 2] - v[:, 1] * u[:, 2], u[:, 2] * v[:, 0] - v[:, 2] * u[:, 0],
                       u[:, 0] * v[:, 1] - v[:, 0] * u[:, 1]], 1)
        for i, ax in enumerate("xyz"):
            out["n" + ax], out["rf" + ax], out["rr" + ax], out["cr" + ax] = nu[:, i], rf[:, i], rr[:, i], cr[:, i]

        # GL 4.5 core 8.14.2 with CLAMP_TO_EDGE: u' = s w - 1/2, i0 = floor(u'), alpha = frac(u')
        def axis(s, n):
            us = s * T(n) - half
            fi = np.floor(us)
            al = us - fi
            i0 = fi.astype(np.int64)
            return np.clip(i0, 0, n - 1), np.clip(i0 + 1, 0, n - 1), al

        x0, x1, al = axis(q[:, 9].astype(T), TW)
        y0, y1, be = axis(q[:, 10].astype(T), TH)
        t2 = tex2.astype(T)
        s2 = (((((one - al) * (one - be))[:, None] * t2[y0, x0] + (al * (one - be))[:, None] * t2[y0, x1])
               + ((one - al) * be)[:, None] * t2[y1, x0]) + (al * be)[:, None] * t2[y1, x1])
        z0, z1, ga = axis(q[:, 11].astype(T), T1)
        t1 = tex1.astype(T)
        s1 = (one - ga)[:, None] * t1[z0] + ga[:, None] * t1[z1]
        fx, fy = q[:, 12].astype(int) - 2, q[:, 13].astype(int) - 2
        inside = (fx >= 0) & (fy >= 0) & (fx < TW) & (fy < TH)
        f2 = np.zeros((N, 4), T)
        f2[inside] = t2[fy[inside], fx[inside]]
        # GL 4.5 core 8.13, table 8.19: the major axis picks the face, (s, t) = ((sc / |ma|) + 1) / 2,
        # ((tc / |ma|) + 1) / 2, then GL_LINEAR inside the face, coordinates clamped to its edge
        rx, ry, rz = u[:, 0], u[:, 1], u[:, 2]
        ax, ay, az = np.abs(rx), np.abs(ry), np.abs(rz)
        xm = (ax >= ay) & (ax >= az)
        ym = ~xm & (ay >= az)
        zm = ~xm & ~ym
        face = np.where(xm, np.where(rx >= 0, 0, 1), np.where(ym, np.where(ry >= 0, 2, 3), np.where(rz >= 0, 4, 5)))
        sc = np.where(xm, np.where(rx >= 0, -rz, rz), np.where(ym, rx, np.where(rz >= 0, rx, -rx)))
        tc = np.where(xm, -ry, np.where(ym, np.where(ry >= 0, rz, -rz), -ry))
        ma = np.where(xm, ax, np.where(ym, ay, az))
        cs = half * (sc / ma + one)
        ct = half * (tc / ma + one)
        cx0, cx1, ca = axis(cs, CS)
        cy0, cy1, cb = axis(ct, CS)
        texel = (cube.astype(np.float32) / np.float32(255)).astype(T)
        fsel = lambda yy, xx: texel[face, yy, xx]
        sc4 = (((((one - ca) * (one - cb))[:, None] * fsel(cy0, cx0) + (ca * (one - cb))[:, None] * fsel(cy0, cx1))
                + ((one - ca) * cb)[:, None] * fsel(cy1, cx0)) + (ca * cb)[:, None] * fsel(cy1, cx1))
        il = np.zeros((N, 4), T)  # imageLoad: zero out of range (GLSL 4.50, 8.12)
        il[inside] = t2[fy[inside], fx[inside]]
        for e in range(4):
            out[f"tex2d{e}"], out[f"tex1d{e}"], out[f"fetch{e}"] = s2[:, e], s1[:, e], f2[:, e]
            out[f"cube{e}"], out[f"iload{e}"] = sc4[:, e], il[:, e]
    return out


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    d = tmp_path_factory.mktemp("glsl_builtins")
    q, tex2, tex1, cube = _inputs()
    q.tofile(d / "in.bin")
    cube.tofile(d / "cube.bin")
    tex2.tofile(d / "tex2d.bin")
    tex1.tofile(d / "tex1d.bin")
    src = (HARNESS.replace("@N@", str(N)).replace("@TW@", str(TW)).replace("@TH@", str(TH))
           .replace("@T1@", str(T1)).replace("@CS@", str(CS)))
    (d / "h.cpp").write_text(src)
    subprocess.run(["g++", "-std=c++20", "-O1", "-ffp-contract=off", "-fno-fast-math", f"-I{SHADERS}",
                    "-o", str(d / "h"), str(d / "h.cpp")],
                   check=True, capture_output=True, text=True)
    subprocess.run([str(d / "h")], check=True, cwd=d)
    got = {}
    for tag in ("f32", "f64"):
        raw = np.fromfile(d / f"{tag}.bin", np.float64).reshape(N, len(OUTS))
        got[tag] = {name: raw[:, i] for i, name in enumerate(OUTS)}
    return q, tex2, tex1, cube, got


@pytest.mark.parametrize("tag,T", [("f32", np.float32), ("f64", np.float64)])
@pytest.mark.parametrize("name", OUTS)
def test_builtin_equals_its_definition(results, tag, T, name):
    q, tex2, tex1, cube, got = results
    want = _spec(q, tex2, tex1, cube, T)[name].astype(np.float64)
    np.testing.assert_array_equal(got[tag][name], want, err_msg=f"{name} ({tag})")


def test_edge_cases_are_exercised(results):
    q, tex2, tex1, cube, got = results
    g = got["f32"]
    assert np.isnan(g["max"][8]) and g["max"][9] == np.float32(q[9, 0])  # max(NaN, y) = NaN; max(x, NaN) = x
    assert np.isnan(g["min"][8]) and g["min"][9] == np.float32(q[9, 0])
    assert np.any((g["rrx"] == 0) & (g["rry"] == 0) & (g["rrz"] == 0))  # total internal reflection
    assert np.any(np.all(np.stack([g[f"fetch{e}"] for e in range(4)]) == 0, axis=0))  # out-of-range fetch
    uv = q[:, 9:11]
    assert np.any(uv < 0) and np.any(uv > 1)  # clamped texture coordinates
