"""Recipe: compile the reference's own shader code as C++ (TEST INFRASTRUCTURE).

Copies the path-tracing shader functions out of the reference tree (where
they lie, never into the repository), rewrites the few GLSL forms C++ lacks,
and compiles them with the GLSL shim (glsl_shim.h) and the harness
(glslref.cpp) into oracle/_ref/libglslref.so.  The tests then run the
reference's own ray-gen / closest-hit / any-hit / miss / shadow / tone-map
code beside the oracle's restatement on the same inputs.

Reference location: $HELIOS_REFERENCE, else the reference checkout at
/root/reference; without it build() returns None and the pinning tests skip.
Outputs go to oracle/_ref/ only (git-ignored).

Text rewrites (each GLSL form -> the C++ form with the same meaning):
  * `in T x` -> `T x`; `out T x` / `inout T x` -> `T& x` (parameter lists only);
  * float literals `1.0` -> `1.0f` (GLSL literals are single precision);
  * constructor calls `vec3(a, b, c)` -> `vec3{a, b, c}` (left-to-right
    argument evaluation, as GLSL defines);
  * swizzles `.xyz .rgb .xy .yz .zw .yzw` -> accessor calls, `.r .g .b .a`
    -> `.x .y .z .w`;
  * M_PI / INFINITY are undefined before the shader's own #defines.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
OUT = os.path.join(ORACLE, "_ref")
GEN = os.path.join(OUT, "glsl_gen")
LIB = os.path.join(OUT, "libglslref.so")

SHADER_DIR = os.path.join("src", "engine", "shader")

# (file, items) — items: "defines", "structs", "functions" (all) or a list of names.
PIECES = {
    # include order of the shaders: common.glsl includes random.glsl first
    "common_gen.inc": [("random.glsl", ["structs", "functions"]),
                       ("common.glsl", ["defines", "structs", "functions"]),
                       ("sampling.glsl", ["functions"]),
                       ("brdf.glsl", ["functions"])],
    "rchit_gen.inc": [("path_trace_rchit.glsl", ["functions"])],
    "rgen_gen.inc": [("path_trace_rgen.glsl", ["structs", "functions"])],
    "rmiss_gen.inc": [("path_trace_rmiss.glsl", ["functions"])],
    "rahit_gen.inc": [("path_trace_rahit.glsl", ["functions"])],
    "shadow_rchit_gen.inc": [("path_trace_shadow.rchit", ["functions"])],
    "shadow_rmiss_gen.inc": [("path_trace_shadow.rmiss", ["functions"])],
    "tonemap_gen.inc": [("tone_map.frag", ["defines", "functions"])],
}

CTORS = ("vec2", "vec3", "vec4", "uvec2", "uvec3", "uvec4", "ivec2", "ivec4", "mat3", "mat4")


def reference_root():
    ref = os.environ.get("HELIOS_REFERENCE", "/root/reference")
    return ref if os.path.isdir(os.path.join(ref, SHADER_DIR)) else None


def _match(text, i, open_c, close_c):
    """Index just past the bracket that closes the one at text[i]."""
    depth = 0
    while i < len(text):
        c = text[i]
        if c == open_c:
            depth += 1
        elif c == close_c:
            depth -= 1
            if depth == 0:
                return i + 1
        i += 1
    raise ValueError("unbalanced %s%s" % (open_c, close_c))


def _strip_comments(src):
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def top_items(src):
    """Top-level #defines, structs and function definitions, in source order."""
    src = _strip_comments(src)
    items = []
    for m in re.finditer(r"^#define\s+(\w+)[^\n]*", src, re.M):
        if not m.group(1).endswith("_GLSL"):
            items.append(("defines", m.group(1), m.start(), m.group(0)))
    for m in re.finditer(r"^struct\s+(\w+)\s*\{", src, re.M):
        end = _match(src, m.end() - 1, "{", "}")
        end = src.index(";", end) + 1
        items.append(("structs", m.group(1), m.start(), src[m.start():end]))
    for m in re.finditer(r"^(\w+)\s+(\w+)\s*\(([^)]*)\)\s*\{", src, re.M):
        if m.group(1) in ("struct", "layout", "return"):
            continue
        end = _match(src, m.end() - 1, "{", "}")
        items.append(("functions", m.group(2), m.start(), src[m.start():end]))
    items.sort(key=lambda it: it[2])
    return items


def _params(header):
    def fix(p):
        p = p.strip()
        p = re.sub(r"^in\s+", "", p)
        m = re.match(r"^(out|inout)\s+(\w+)\s+(\w+)$", p)
        return "%s& %s" % (m.group(2), m.group(3)) if m else p
    head, rest = header.split("(", 1)
    args = rest.rsplit(")", 1)[0]
    fixed = ", ".join(fix(a) for a in args.split(",")) if args.strip() else ""
    return "%s(%s)" % (head, fixed)


def _braces(text):
    out, i = [], 0
    pat = re.compile(r"\b(%s)\(" % "|".join(CTORS))
    while True:
        m = pat.search(text, i)
        if not m:
            out.append(text[i:])
            return "".join(out)
        open_at = m.end() - 1
        close = _match(text, open_at, "(", ")")
        inner = _braces(text[open_at + 1:close - 1])
        out.append(text[i:m.start()] + m.group(1) + "{" + inner + "}")
        i = close


def to_cpp(kind, text):
    if kind == "functions":
        hdr_end = text.index("{")
        text = _params(text[:hdr_end].rstrip()) + "\n" + text[hdr_end:]
    text = re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][+-]?\d+)?(?![\w.])", r"\1\2f", text)
    text = _braces(text)
    text = re.sub(r"\.(xyz|rgb|yzw|xy|yz|zw)\b", r".\1()", text)
    for a, b in (("r", "x"), ("g", "y"), ("b", "z"), ("a", "w")):
        text = re.sub(r"\.%s\b" % a, "." + b, text)
    if kind == "defines":
        name = text.split()[1]
        text = "#undef %s\n%s" % (name, text)
    return text


# Push-constant blocks, emitted as plain structs: (file, block name).
BLOCKS = [("path_trace_rgen.glsl", "PathTraceConsts"), ("tone_map.frag", "PushConstants")]


def push_constant_struct(src, name):
    src = _strip_comments(src)
    m = re.search(r"uniform\s+%s\s*\{" % name, src)
    end = _match(src, m.end() - 1, "{", "}")
    return "struct %s %s;" % (name, src[m.end() - 1:end])


def generate(ref):
    os.makedirs(GEN, exist_ok=True)
    shaders = os.path.join(ref, SHADER_DIR)
    blocks = ["// Generated by oracle/glslref/build.py from the reference's shaders; not committed."]
    for fname, name in BLOCKS:
        blocks.append(push_constant_struct(open(os.path.join(shaders, fname)).read(), name))
    with open(os.path.join(GEN, "consts_gen.inc"), "w") as f:
        f.write("\n".join(blocks) + "\n")
    for out_name, parts in PIECES.items():
        chunks = ["// Generated by oracle/glslref/build.py from the reference's shaders; not committed."]
        for fname, wanted in parts:
            src = open(os.path.join(shaders, fname)).read()
            chunks.append("// ---- %s" % fname)
            for kind, name, _, text in top_items(src):
                if kind in wanted or name in wanted:
                    chunks.append(to_cpp(kind, text))
        with open(os.path.join(GEN, out_name), "w") as f:
            f.write("\n".join(chunks) + "\n")


def build(force=False):
    """Generates and compiles oracle/_ref/libglslref.so; None without the reference."""
    ref = reference_root()
    if ref is None:
        return None
    deps = [os.path.join(HERE, f) for f in ("glslref.cpp", "glsl_shim.h", "build.py")]
    deps += [os.path.join(ORACLE, f) for f in ("oracle.cpp", "oracle_core.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    generate(ref)
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-Wno-unused-variable", "-Wno-unused-but-set-variable", "-I", GEN, "-I", HERE,
           "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "glslref.cpp"), "-o", LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("glslref build failed:\n%s%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    out = build(force="--force" in sys.argv)
    print(out or "reference tree not found: nothing built")
