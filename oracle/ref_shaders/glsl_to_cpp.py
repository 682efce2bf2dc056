"""Rewrite a GLSL compute shader's declarations so that its source compiles
as C++ against glsl.h.  TEST INFRASTRUCTURE ONLY (the oracle's check against
the reference's own shader code); the output goes to oracle/_ref/gen/ and is
never committed.

Only declarations are rewritten; every function body compiles as written:
  1. the `#version` and `#extension` lines and the comments are dropped;
  2. the work-group size declaration `layout(local_size_x = ...) in;` is
     dropped (the dispatch loop supplies gl_GlobalInvocationID);
  3. interface blocks `uniform NAME { ... };` and `buffer NAME { ... };`
     become their members as globals (an instance-named block, also a
     stage's `in` / `out` block, `... } inst;` becomes a struct NAME and its
     instance); a runtime-sized array `T a[];` becomes a pointer `T* a;` that
     the dispatch binds; a global stage input or output `in T x;` /
     `out T x;` loses its qualifier;
  4. the remaining `layout(...)` qualifiers and the qualifiers `uniform`,
     `readonly`, `writeonly`, `restrict`, `coherent` are dropped (a
     uniform's initialiser, its default value, stays);
  5. a parameter `inout T x` or `out T x` becomes `T& x`, `in T x` becomes
     `T x`;
  6. an unsuffixed floating literal (`1.5`, `.5`, `2.`, `1e5`, `2.5e-3`)
     gets the suffix `f` (a GLSL literal without `lf` is a float); one with
     `lf` loses the suffix (a C++ double);
  7. a global whose initializer is not a constant (it reads a uniform or
     calls a function other than a constructor or a pure math built-in; a
     constant reads only literals, macros and earlier constants), and every
     global that is not `const` but has an initializer (invocation-private
     storage in GLSL; uniforms excepted), is declared without it; the
     initialisations move, in source order, into
     `void glsl_init_globals()`, which the dispatch calls after binding the
     uniforms (once per dispatch, or before each invocation for shaders that
     write such globals);
  8. a global `const float` with a constant initializer, and a `float`
     uniform's default value, become `glsl_cfloat NAME = GLSL_CONST(NAME,
     init)`: the compiler folds a shader's constants, and the GL sets a
     uniform's default, in float.  The float build evaluates the
     initializer; the double build (glsl_cfloat = double) takes the value the
     float build folded, so its constants are the shader's float values and
     only its run-time arithmetic is in double.

Usage: python glsl_to_cpp.py SHADER.glsl OUT.inc
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

QUALIFIERS = ("readonly", "writeonly", "restrict", "coherent")
UNIFORM_MARK = "GLSL_UNIFORM"
CONST_FLOAT = "glsl_cfloat"
TYPE_NAMES = {"float", "int", "uint", "bool", "vec2", "vec3", "vec4", "ivec2", "ivec3", "ivec4", "uvec3", "mat4"}
PURE_BUILTINS = {"sqrt", "pow", "exp", "sin", "cos", "abs", "min", "max", "floor"}


def _drop_version(src: str) -> str:
    src = re.sub(r"^\s*#version[^\n]*\n", "", src, count=1, flags=re.M)
    return re.sub(r"^\s*#extension[^\n]*\n", "", src, flags=re.M)


def _drop_local_size(src: str) -> str:
    return re.sub(r"layout\s*\([^)]*local_size[^)]*\)\s*in\s*;", "", src)


def _blocks(src: str) -> str:
    pat = re.compile(r"(?:layout\s*\([^)]*\)\s*)?\b(uniform|buffer|in|out)\s+(\w+)\s*\{(.*?)\}\s*(\w*)\s*;", re.S)

    def repl(m: re.Match) -> str:
        body = re.sub(r"(\w+)\s+(\w+)\s*\[\s*\]\s*;", r"\1* \2 = nullptr;", m.group(3))
        if m.group(4):  # an instance-named block: a struct and its instance
            return f"struct {m.group(2)} {{{body}}};\n{m.group(2)} {m.group(4)};"
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


def _strip_comments(src: str) -> str:
    # one left-to-right pass, so a line comment that holds "/*" or "*/"
    # (the "//*" block toggles) stays a line comment
    return re.sub(r"//[^\n]*|/\*.*?\*/", lambda m: "" if m.group(0).startswith("//") else " ", src, flags=re.S)


def _io_qualifiers(src: str) -> str:
    # a global `in T x;` / `out T x;` (stage inputs and outputs) loses the qualifier
    return re.sub(r"(?m)^(\s*)(?:in|out)\s+(?=\w+\s+\w+\s*;)", r"\1", src)


def _param_qualifiers(src: str) -> str:
    # in a parameter list: `inout T x` / `out T x` -> `T& x`, `in T x` -> `T x`
    src = re.sub(r"(?<=[(,])(\s*)(?:inout|out)\s+(\w+)\s+(\w+)", r"\1\2& \3", src)
    return re.sub(r"(?<=[(,])(\s*)in\s+(\w+)\s+(\w+)", r"\1\2 \3", src)


_FLOAT_LITERAL = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(lf|LF)?(?![\w.])")


def _float_literals(src: str) -> str:
    # GLSL's floating literals: digits with a point, an exponent, or both.
    # Unsuffixed ones are float (suffix f); `lf` ones are double (no suffix
    # in C++).  Suffixed float literals, integers and hex are left alone.
    return _FLOAT_LITERAL.sub(lambda m: m.group(1) if m.group(2) else m.group(1) + "f", src)


def _macro_names(src: str) -> set[str]:
    return set(re.findall(r"^\s*#define\s+(\w+)", src, re.M))


def _deferred_globals(src: str) -> tuple[str, list[str]]:
    """Top-level `[const] T name = init;` statements: keep constant ones,
    defer the rest (rule 7)."""
    constant = _macro_names(src) | TYPE_NAMES | PURE_BUILTINS
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
                idents = set(re.findall(r"\b[A-Za-z_]\w*\b", init)) - constant
                if is_const and not idents:
                    if typ == "float":  # rule 8
                        out.append(f"const {CONST_FLOAT} {name} = GLSL_CONST({name}, {init.strip()});")
                    else:
                        out.append(f"const {typ} {name} = {init.strip()};")
                    constant.add(name)
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
    src = _strip_comments(src)
    src = _drop_local_size(src)
    src = _blocks(src)
    src = _qualifiers(src)
    src = _io_qualifiers(src)
    src = _param_qualifiers(src)
    src = _float_literals(src)
    src, inits = _deferred_globals(src)
    # rule 8 for a float uniform's default value
    src = re.sub(rf"{UNIFORM_MARK}\s+float\s+(\w+)\s*=\s*([^;]+);",
                 lambda m: f"{CONST_FLOAT} {m.group(1)} = GLSL_CONST({m.group(1)}, {m.group(2).strip()});", src)
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
