"""Rewrite a GLSL compute shader's declarations so that its source compiles
as C++ against glsl.h.  TEST INFRASTRUCTURE ONLY (the oracle's check against
the reference's own shader code); the output goes to oracle/_ref/gen/ and is
never committed.

Only declarations are rewritten; every function body compiles as written:
  1. the `#version` line is dropped;
  2. the work-group size declaration `layout(local_size_x = ...) in;` is
     dropped (the dispatch loop supplies gl_GlobalInvocationID);
  3. interface blocks `uniform NAME { ... };` and `buffer NAME { ... };`
     become their members as globals; a runtime-sized array `T a[];` becomes
     a pointer `T* a;` that the dispatch binds;
  4. the remaining `layout(...)` qualifiers and the qualifiers `uniform`,
     `readonly`, `writeonly`, `restrict`, `coherent` are dropped (a
     uniform's initialiser, its default value, stays);
  5. a parameter `inout T x` becomes `T& x`;
  6. an unsuffixed floating literal gets the suffix `f` (a GLSL literal
     without `lf` is a float);
  7. a global whose initializer is not a constant (it reads a uniform or
     calls a function), and every global that is not `const` but has an
     initializer (invocation-private storage in GLSL; uniforms excepted), is
     declared without it; the initialisations move, in source order, into
     `void glsl_init_globals()`, which the dispatch calls after binding the
     uniforms (once per dispatch, or before each invocation for shaders that
     write such globals).

Usage: python glsl_to_cpp.py SHADER.glsl OUT.inc
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

QUALIFIERS = ("readonly", "writeonly", "restrict", "coherent")
UNIFORM_MARK = "GLSL_UNIFORM"
TYPE_NAMES = {"float", "int", "uint", "bool", "vec2", "vec3", "vec4", "ivec2", "ivec3", "ivec4", "uvec3", "mat4"}


def _drop_version(src: str) -> str:
    return re.sub(r"^\s*#version[^\n]*\n", "", src, count=1, flags=re.M)


def _drop_local_size(src: str) -> str:
    return re.sub(r"layout\s*\([^)]*local_size[^)]*\)\s*in\s*;", "", src)


def _blocks(src: str) -> str:
    pat = re.compile(r"(?:layout\s*\([^)]*\)\s*)?\b(uniform|buffer)\s+(\w+)\s*\{(.*?)\}\s*(\w*)\s*;", re.S)

    def repl(m: re.Match) -> str:
        if m.group(4):
            raise SystemExit(f"instance-named interface block {m.group(2)} is not handled")
        body = m.group(3)
        body = re.sub(r"(\w+)\s+(\w+)\s*\[\s*\]\s*;", r"\1* \2 = nullptr;", body)
        return body

    return pat.sub(repl, src)


def _qualifiers(src: str) -> str:
    src = re.sub(r"layout\s*\([^)]*\)", "", src)
    # a uniform's initialiser is its default value, set once at link time:
    # marked so that rule 7 leaves it in place
    src = re.sub(r"\buniform\b", UNIFORM_MARK, src)
    for q in QUALIFIERS:
        src = re.sub(rf"\b{q}\b", "", src)
    return src


def _inout(src: str) -> str:
    return re.sub(r"\binout\s+(\w+)\s+(\w+)", r"\1& \2", src)


def _float_literals(src: str) -> str:
    out = []
    for line in src.split("\n"):
        code, sep, comment = line.partition("//")
        code = re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][+-]?\d+)?(?![\w.])", r"\1\2f", code)
        out.append(code + sep + comment)
    return "\n".join(out)


def _macro_names(src: str) -> set[str]:
    return set(re.findall(r"^\s*#define\s+(\w+)", src, re.M))


def _deferred_globals(src: str) -> tuple[str, list[str]]:
    """Top-level `[const] T name = init;` statements: keep constant ones,
    defer the rest (rule 7)."""
    macros = _macro_names(src)
    inits: list[str] = []
    out: list[str] = []
    depth = 0
    i = 0
    decl = re.compile(r"(const\s+)?(\w+)\s+(\w+)\s*=\s*([^;{}]+);")
    while i < len(src):
        c = src[i]
        if depth == 0 and (c.isalpha() or c == "_") and (i == 0 or not (src[i - 1].isalnum() or src[i - 1] == "_")):
            m = decl.match(src, i)
            line_start = src.rfind("\n", 0, i) + 1
            if m and src[line_start:i].strip() == "" and m.group(2) not in ("return", "else"):
                is_const, typ, name, init = m.group(1), m.group(2), m.group(3), m.group(4)
                idents = set(re.findall(r"\b[A-Za-z_]\w*\b", init)) - TYPE_NAMES - macros
                idents = {w for w in idents if not re.fullmatch(r"\d+\w*", w)}
                if is_const and not idents:
                    out.append(m.group(0))
                else:
                    out.append(f"{typ} {name};")
                    inits.append(f"  {name} = {init.strip()};")
                i = m.end()
                continue
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
        out.append(c)
        i += 1
    return "".join(out), inits


def transform(src: str) -> str:
    src = _drop_version(src)
    src = _drop_local_size(src)
    src = _blocks(src)
    src = _qualifiers(src)
    src = _inout(src)
    src = _float_literals(src)
    src, inits = _deferred_globals(src)
    src = re.sub(rf"{UNIFORM_MARK}\s*", "", src)
    return src + "\nvoid glsl_init_globals() {\n" + "\n".join(inits) + "\n}\n"


def main() -> None:
    if len(sys.argv) != 3:
        sys.exit("usage: glsl_to_cpp.py SHADER.glsl OUT.inc")
    src = Path(sys.argv[1]).read_text()
    out = Path(sys.argv[2])
    out.parent.mkdir(parents=True, exist_ok=True)
    out.write_text(f"// generated from {Path(sys.argv[1]).name} by glsl_to_cpp.py: do not commit\n" + transform(src))


if __name__ == "__main__":
    main()
