"""ORACLE — test infrastructure only.  Recipe for `oracle/_ref/libref_glsl.so`: the reference's own shader
source, compiled for the host as C++20 against the GLSL-compatibility layer in this directory.

It reads reina-vk's `shaders/raytrace/*.glsl`, `shaders/postprocessing/**/*.glsl` and `polyglot/*.h` where
they lie (the directory in REINA_REFERENCE_DIR, by default /root/reference), applies only mechanical,
meaning-preserving rewrites, writes the results under `oracle/_ref/src/` (build output, not committed) and
compiles one translation unit per shader stage, each in its own namespace:

  * `#version` / `#extension` lines dropped; the polyglot headers' `#ifdef __cplusplus` block (glm types)
    dropped, the GLSL types of glsl_compat.h are used instead;
  * `layout(...)` resource declarations become host stand-ins (glsl_runtime.h): buffer-block members become
    `Field<T>` / `View<T>` at their scalar-layout byte offsets, storage images `Image2D`, the texture array
    `SamplerArray`, push-constant blocks a reference into the push-constant bytes, ray payloads and hit
    attributes thread-local variables, `accelerationStructureEXT` a dummy integer;
  * `inout T x` / `out T x` parameters become `T& x`;
  * floating-point literals get an `f` suffix (GLSL literals are float; C++ would read double);
  * the swizzles `.xyz`, `.xy`, `.rgb` become calls (`.xyz()`);
  * a declaration whose initializer calls a function of the same name (`vec3 fSubsurface = fSubsurface(...)`,
    `ivec2 imageSize = imageSize(...)`: legal GLSL, where the new name is not yet in scope) calls it through
    the stage's namespace;
  * multi-argument vector constructors are written as braced initializers, so that their arguments are
    evaluated left to right as GLSL requires (C++ leaves a call's argument order unspecified);
  * `traceRayEXT(...)` calls a per-stage function that hands the payload declared at that location to the
    host trace (glsl::trace_ray).

Nothing in the shader arithmetic is changed.  Run: python oracle/glsl/build_ref.py [--force]
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE = HERE.parent
OUT = ORACLE / "_ref"
SRC = OUT / "src"
LIB = OUT / "libref_glsl.so"
FLAGS = ["-O2", "-std=c++20", "-fPIC", "-pthread", "-ffp-contract=off", "-fno-fast-math", "-w"]


def reference_dir() -> Path:
    return Path(os.environ.get("REINA_REFERENCE_DIR", "/root/reference"))


# stage files: (stage id, path under shaders/, kind)
STAGES = [
    ("raygen", "raytrace/raytrace.rgen.glsl", "raygen"),
    ("lambertian", "raytrace/lambertian.rchit.glsl", "hit"),
    ("metal", "raytrace/metal.rchit.glsl", "hit"),
    ("dielectric", "raytrace/dielectric.rchit.glsl", "hit"),
    ("disney", "raytrace/disney.rchit.glsl", "hit"),
    ("miss", "raytrace/raytrace.rmiss.glsl", "miss"),
    ("shadow_miss", "raytrace/shadow.rmiss.glsl", "miss"),
    ("blur_x", "postprocessing/bloom/blurX.comp.glsl", "compute"),
    ("blur_y", "postprocessing/bloom/blurY.comp.glsl", "compute"),
    ("combine", "postprocessing/bloom/combine.comp.glsl", "compute"),
    ("tonemap", "postprocessing/tonemap/tonemapping.comp.glsl", "compute"),
]
# SBT record of each closest-hit stage (the material index, src/tools/vktools.cpp:483) and miss index
HIT_RECORD = {"lambertian": 0, "metal": 1, "dielectric": 2, "disney": 3}
MISS_INDEX = {"miss": 0, "shadow_miss": 1}

# scalar-layout sizes of the types that appear in buffer blocks
SIZES = {"uint": 4, "int": 4, "float": 4, "bool": 4, "vec2": 8, "vec3": 12, "vec4": 16, "mat3": 36, "mat4": 64,
         "mat4x4": 64, "InstanceProperties": 120, "InstanceData": 112}

FLOAT_LIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)(?![\w.])")


def strip_comments(text: str) -> str:
    text = re.sub(r"/\*.*?\*/", lambda m: "\n" * m.group(0).count("\n"), text, flags=re.S)
    return re.sub(r"//[^\n]*", "", text)


class Translation:
    def __init__(self):
        self.payloads: dict[int, str] = {}      # rayPayloadEXT: location -> variable
        self.payload_in: str | None = None      # rayPayloadInEXT variable
        self.attribs: str | None = None         # hitAttributeEXT variable


def translate_layouts(text: str, tr: Translation) -> str:
    def binding_of(q: str) -> int:
        m = re.search(r"binding\s*=\s*(\d+)", q)
        return int(m.group(1)) if m else -1

    def repl(m: re.Match) -> str:
        qual, decl, block = m.group(1), m.group(2).strip(), m.group(3)
        if re.fullmatch(r"local_size_x.*", qual.strip()) or decl == "in":
            return ""
        if "push_constant" in qual:
            inner = block.strip()[1:-1].strip().rstrip(";").split()
            return f"static {inner[0]}& {inner[1]} = glsl::push_constants<{inner[0]}>();"
        loc = re.search(r"location\s*=\s*(\d+)", qual)
        if decl.startswith("rayPayloadEXT"):
            _, ty, name = decl.split()
            tr.payloads[int(loc.group(1))] = name
            return f"static thread_local {ty} {name}{{}};"
        if decl.startswith("rayPayloadInEXT"):
            _, ty, name = decl.split()
            tr.payload_in = name
            return f"static thread_local {ty} {name}{{}};"
        b = binding_of(qual)
        if "accelerationStructureEXT" in decl:
            name = decl.split()[-1]
            return f"static int {name} = {b};"
        if "image2D" in decl:
            name = decl.split()[-1]
            return f"static const glsl::Image2D {name}({b});"
        if "sampler2D" in decl:
            name = decl.split()[-1].replace("[]", "")
            return f"static const glsl::SamplerArray {name}({b});"
        if decl.split()[-2:-1] == ["buffer"] or decl.startswith("buffer") or " buffer " in f" {decl} ":
            out, off = [], 0
            for mem in [x.strip() for x in block.strip()[1:-1].split(";") if x.strip()]:
                ty, name = mem.split()
                if name.endswith("[]"):
                    out.append(f"static const glsl::View<{ty}> {name[:-2]}({b}, {off});")
                else:
                    out.append(f"static const glsl::Field<{ty}> {name}({b}, {off});")
                    off += SIZES[ty]
            return "\n".join(out)
        raise ValueError(f"unhandled layout declaration: layout({qual}) {decl} {block or ''}")

    pat = re.compile(r"layout\s*\(([^)]*)\)\s*([A-Za-z_][\w\s\[\]]*?)\s*(\{[^}]*\})?\s*;", re.S)
    return pat.sub(repl, text)


def braced_constructors(text: str) -> str:
    """Multi-argument vector constructors as braced initializers: GLSL evaluates call arguments in order,
    left to right (GLSL 4.60, 6.1.1), and C++ evaluates a braced initializer's clauses in order but leaves
    the order of function-call arguments unspecified (vec3(random(s), random(s), random(s)) draws three
    numbers whose order matters)."""
    out, i = [], 0
    pat = re.compile(r"\b(vec2|vec3|vec4|ivec2|ivec3)\(")
    while True:
        m = pat.search(text, i)
        if not m:
            out.append(text[i:])
            return "".join(out)
        start = m.end() - 1
        depth, j, top_comma = 0, start, False
        while True:
            c = text[j]
            if c in "([{":
                depth += 1
            elif c in ")]}":
                depth -= 1
                if depth == 0:
                    break
            elif c == "," and depth == 1:
                top_comma = True
            j += 1
        inner = braced_constructors(text[start + 1:j])
        out.append(text[i:m.start()])
        out.append(f"{m.group(1)}{{{inner}}}" if top_comma else f"{m.group(1)}({inner})")
        i = j + 1


def translate_glsl(text: str, ns: str, tr: Translation) -> str:
    text = strip_comments(text)
    text = re.sub(r"^\s*#\s*(version|extension)[^\n]*", "", text, flags=re.M)
    text = translate_layouts(text, tr)
    m = re.search(r"hitAttributeEXT\s+(\w+)\s+(\w+)\s*;", text)
    if m:
        tr.attribs = m.group(2)
        text = text.replace(m.group(0), f"static thread_local {m.group(1)} {m.group(2)};")
    text = re.sub(r"\b(?:inout|out)\s+(\w+)\s+(\w+)", r"\1& \2", text)
    text = FLOAT_LIT.sub(lambda m: m.group(1) + "f", text)
    text = re.sub(r"\.(xyz|xy|rgb)\b(?!\s*\()", r".\1()", text)
    text = re.sub(r"\b(\w+)\s+(\w+)\s*=\s*\2\s*\(", lambda m: f"{m.group(1)} {m.group(2)} = {ns}::{m.group(2)}(", text)
    text = re.sub(r"\btraceRayEXT\s*\(", "glsl_trace_(", text)
    return braced_constructors(text)


def translate_polyglot(text: str) -> str:
    return re.sub(r"#ifdef __cplusplus.*?#endif[^\n]*", "", text, flags=re.S)


def stage_unit(stage: str, rel: str, kind: str, tr: Translation) -> str:
    ns = f"ref_{stage}"
    lines = ['#include "glsl_runtime.h"', f"namespace {ns} {{", "using namespace glsl;",
             "static void glsl_trace_(int, uint, uint, uint, uint, uint, vec3, float, vec3, float, int);",
             f'#include "{Path(rel).name}"']
    cases = "".join(f"    case {loc}: glsl::trace_ray(flags, sbt_offset, miss, o, tmin, d, tmax, &{v}, sizeof({v})); return;\n"
                    for loc, v in sorted(tr.payloads.items()))
    lines.append("static void glsl_trace_(int, uint flags, uint, uint sbt_offset, uint, uint miss, vec3 o, float tmin, "
                 "vec3 d, float tmax, int loc) {\n  switch (loc) {\n" + cases + "    default: glsl::note_out_of_range(-4);\n  }\n}")
    kat = HERE / f"ref_kat_{stage}.inc"
    if kat.exists():
        lines.append(f'#include "{kat.name}"')
    lines.append(f"}}  // namespace {ns}")
    if kind in ("hit", "miss"):
        body = []
        if tr.payload_in:
            body.append(f"    memcpy(&{ns}::{tr.payload_in}, payload, sizeof({ns}::{tr.payload_in}));")
        if tr.attribs:
            body.append(f"    {ns}::{tr.attribs} = glsl::rt().attribs;")
        body.append(f"    {ns}::main();")
        if tr.payload_in:
            body.append(f"    memcpy(payload, &{ns}::{tr.payload_in}, sizeof({ns}::{tr.payload_in}));")
        lines.append(f"void ref_stage_{stage}(void* payload, unsigned long long) {{\n" + "\n".join(body) + "\n}")
    else:
        lines.append(f"void ref_stage_{stage}() {{ {ns}::main(); }}")
    return "\n".join(lines) + "\n"


def stages_unit() -> str:
    decl, reg = [], []
    for stage, _, kind in STAGES:
        if kind in ("hit", "miss"):
            decl.append(f"void ref_stage_{stage}(void*, unsigned long long);")
            if kind == "hit":
                reg.append(f"    glsl::register_hit_stage({HIT_RECORD[stage]}, ref_stage_{stage});")
            else:
                reg.append(f"    glsl::register_miss_stage({MISS_INDEX[stage]}, ref_stage_{stage});")
    kat_decl, kat_calls = [], []
    for stage, _, _ in STAGES:
        if (HERE / f"ref_kat_{stage}.inc").exists():
            kat_decl.append(f"namespace ref_{stage} {{ bool kat(int kind, const float* r, double* o); }}")
            kat_calls.append(f"        if (ref_{stage}::kat(kind, r, o)) continue;")
    return ("#include \"glsl_runtime.h\"\n" + "\n".join(decl) + "\n" + "\n".join(kat_decl) +
            "\nvoid ref_register_stages() {\n" + "\n".join(reg) + "\n}\n"
            "extern \"C\" void ref_kat_dispatch(int kind, const float* records, unsigned long long n, double* out) {\n"
            "    for (unsigned long long i = 0; i < n; ++i) {\n        const float* r = records + 40 * i;\n"
            "        double* o = out + 8 * i;\n        for (int k = 0; k < 8; ++k) o[k] = 0.0;\n" + "\n".join(kat_calls) +
            "\n    }\n}\n")


def include_closure(path: Path) -> list[Path]:
    """`path` and the .glsl files it includes, directly or through other includes (same directory)."""
    seen, todo = [], [path]
    while todo:
        f = todo.pop()
        if f in seen:
            continue
        seen.append(f)
        for m in re.finditer(r'#include\s+"([^"]+\.glsl)"', strip_comments(f.read_text())):
            todo.append(f.parent / m.group(1))
    return seen


def build(force: bool = False) -> Path:
    ref = reference_dir()
    shaders, poly = ref / "shaders", ref / "polyglot"
    if not shaders.is_dir() or not poly.is_dir():
        raise FileNotFoundError(f"reference shaders not found under {ref} (set REINA_REFERENCE_DIR)")
    inputs = sorted(shaders.rglob("*.glsl")) + sorted(poly.glob("*.h"))
    own = sorted(HERE.glob("*.h")) + sorted(HERE.glob("*.cpp")) + sorted(HERE.glob("*.inc")) + [Path(__file__)]
    newest = max(p.stat().st_mtime for p in inputs + own)
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    SRC.mkdir(parents=True, exist_ok=True)
    for h in poly.glob("*.h"):
        (SRC / h.name).write_text(translate_polyglot(h.read_text()))
    units = []
    for stage, rel, kind in STAGES:
        tr = Translation()
        # the stage file and the shader headers it includes, each translated into this stage's own copy
        # (payload and attribute declarations are collected from exactly these files)
        for f in include_closure(shaders / rel):
            t = translate_glsl(f.read_text(), f"ref_{stage}", tr)
            t = re.sub(r'#include\s+"([^"]+\.glsl)"', lambda m: f'#include "{stage}__{m.group(1)}"', t)
            (SRC / f"{stage}__{f.name}").write_text(t)
        unit = SRC / f"stage_{stage}.cpp"
        unit.write_text(stage_unit(stage, f"{stage}__{Path(rel).name}", kind, tr))
        units.append(unit)
    (SRC / "ref_stages.cpp").write_text(stages_unit())
    units += [SRC / "ref_stages.cpp", HERE / "glsl_runtime.cpp"]
    objs = []
    procs = []
    for u in units:
        o = SRC / (u.stem + ".o")
        objs.append(o)
        procs.append((u, subprocess.Popen(["g++", *FLAGS, "-c", f"-I{HERE}", f"-I{SRC}", str(u), "-o", str(o)],
                                          stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)))
    for u, p in procs:
        out, err = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"compile of {u.name} failed:\n{err[-6000:]}")
    res = subprocess.run(["g++", "-shared", "-pthread", "-o", str(LIB), *map(str, objs)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
