"""Translate the reference's ray-tracing shaders into host C++ (test infrastructure).

Reads the GLSL source of Asuna's hot path where it lies in the reference tree
and writes mechanically rewritten copies into ``oracle/_ref/gen/`` (git-ignored,
never committed).  ``oracle/ref_harness.cpp`` includes them and provides the
ray-tracing built-ins (traceRayEXT, gl_* variables, descriptor bindings), so
the reference's own shading, sampling and accumulation code runs on the CPU.
It is the pin of the CPU restatement in ``oracle/asuna_oracle.cpp``.

Rewrites (all mechanical, no logic changes):
  * drop ``#version`` / ``#extension`` lines and the single-line ``layout(...)``
    / payload / hit-attribute declarations (the harness defines those globals);
  * ``#include`` of a GLSL file -> the translated file; of ``shared/*.h`` ->
    dropped (the harness includes them at global scope);
  * ``inout T x`` / ``out T x`` -> ``T& x``; ``in T x`` -> ``T x``;
  * rvalue swizzles ``.xy .xyz .rg .rgb .rgba .r`` -> accessor calls;
  * unsuffixed floating literals get an ``f`` suffix (GLSL literals are float);
  * the macro ``INFINITY`` is renamed (it clashes with C's);
  * ``vec2(rand(s), rand(s))`` -> brace initialisation, because C++ does not
    order function arguments and GLSL evaluates them left to right;
  * stage bodies (rgen / rmiss / rchit) are wrapped in their own namespaces;
  * utils/sun_and_sky.glsl's ``M_PI`` (its own 3.1415926535f, defined only
    where the name is free) is renamed, as the host's <cmath> defines M_PI as
    a double;
  * raytrace.projective.rgen clears ``mRec.channel[i]`` for i < 9 although the
    array has 8 entries (an out-of-bounds write on the GPU); the loop bound is
    reduced to 8 so host C++ stays defined.

The reference's ``src/shared/*.h`` headers (the device-ABI structs the
shaders and the harness include) are copied beside the translation, so the
generated tree compiles where the reference checkout is absent (the GPU
host): ``oracle/build_oracle.py`` builds from it there.

Usage: python oracle/gen_ref.py [--ref <reference checkout>] [--out oracle/_ref/gen]
The checkout defaults to $ASUNA_REFERENCE, else ``baseline/_ref`` in this
repository, else the path the build container mounts it at (find_ref_tree).
"""
import argparse
import os
import re
import shutil
import sys

_REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# where the build container mounts the reference checkout (read-only)
_MOUNTED_CHECKOUT = "/root/reference"
MANIFEST = "GENERATED_FROM"


def find_ref_tree():
    """The reference checkout holding src/shaders, or None."""
    for cand in (os.environ.get("ASUNA_REFERENCE"), os.path.join(_REPO, "baseline", "_ref"), _MOUNTED_CHECKOUT):
        if cand and os.path.isdir(os.path.join(cand, "src", "shaders")):
            return cand
    return None

SHADERS = {
    # file (relative to src/shaders) -> stage namespace (None = shared utility)
    "utils/structs.glsl": None,
    "utils/math.glsl": None,
    "utils/sun_and_sky.glsl": None,
    "utils/sample_light.glsl": None,
    "utils/rchit_layouts.glsl": None,
    "raytrace.projective.rgen": "stage_rgen",
    "raytrace.default.rmiss": "stage_miss",
    "raytrace.shadow.rmiss": "stage_shadow",
    "bxdf/raytrace.brdf_lambertian.rchit": "stage_lambertian",
    "bxdf/raytrace.brdf_rough_plastic.rchit": "stage_rough_plastic",
    "bxdf/raytrace.bsdf_dielectric.rchit": "stage_dielectric",
    "bxdf/raytrace.brdf_emissive.rchit": "stage_emissive",
    "bxdf/raytrace.brdf_plastic.rchit": "stage_plastic",
    "bxdf/raytrace.brdf_mirror.rchit": "stage_mirror",
    "bxdf/raytrace.brdf_conductor.rchit": "stage_conductor",
    "bxdf/raytrace.brdf_rough_conductor.rchit": "stage_rough_conductor",
    "bxdf/raytrace.brdf_phong.rchit": "stage_phong",
    "bxdf/raytrace.brdf_pbr_metalness_roughness.rchit": "stage_pbr",
    "bxdf/raytrace.brdf_disney.rchit": "stage_disney",
    "bxdf/raytrace.brdf_kang18.rchit": "stage_kang18",
    # the post pass (oracle/post_harness.cpp)
    "utils/tonemapping.glsl": None,
    "utils/random.glsl": None,
    "post.idle.frag": "stage_post",
}

FLOAT_LIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")
SWIZZLE = re.compile(r"\.(xyz|xy|rgba|rgb|rg|r)\b")
DROP_LINE = re.compile(r"^\s*(#version|#extension|layout\s*\(|hitAttributeEXT)")


def out_name(rel):
    return os.path.basename(rel) + ".h"


def translate(text, rel, stage):
    lines = []
    body_start = 0
    for line in text.splitlines():
        if DROP_LINE.match(line):
            if line.lstrip().startswith("layout") and not line.rstrip().endswith(";"):
                raise SystemExit(f"{rel}: multi-line layout declaration not handled: {line!r}")
            lines.append("// [dropped] " + line.strip())
            continue
        m = re.match(r'^\s*#include\s+"([^"]+)"', line)
        if m:
            inc = m.group(1)
            base = os.path.basename(inc)
            if "/shared/" in inc or inc.startswith("shared/"):
                lines.append(f"// [shared header at global scope] {inc}")
            else:
                lines.append(f'#include "{base}.h"')
            body_start = len(lines)
            continue
        lines.append(line)
    src = "\n".join(lines)
    # code-level rewrites (comments are rewritten too, harmlessly)
    src = re.sub(r"\b(inout|out)\s+(\w+)\s+(\w+)", r"\2& \3", src)
    src = re.sub(r"\bin\s+(?=(const\s+)?\w+\s+\w+\s*[,)\[])", "", src)
    src = SWIZZLE.sub(lambda m: "." + m.group(1) + "()", src)
    src = FLOAT_LIT.sub(lambda m: m.group(1) + "f", src)
    src = re.sub(r"\bINFINITY\b", "GLSL_INFINITY", src)
    src = re.sub(r"\bM_PI\b", "GLSL_SKY_PI", src)
    src = src.replace("vec2(rand(seed), rand(seed))", "vec2{rand(seed), rand(seed)}")
    src = src.replace("vec3(rand(seed), rand(seed), rand(seed))", "vec3{rand(seed), rand(seed), rand(seed)}")
    src = src.replace("vec2(rand(prev), rand(prev))", "vec2{rand(prev), rand(prev)}")
    if rel == "post.idle.frag":
        # a GLSL array constructor; the output's and the input's .g/.b/.a
        # components (not accessor-rewritten above) name the harness's fields
        if "float[7](1, 2, 4, 8, 16, 32, 64)" not in src:
            raise SystemExit("post.idle.frag: the scale array constructor not found")
        src = src.replace("float[7](1, 2, 4, 8, 16, 32, 64)", "{1, 2, 4, 8, 16, 32, 64}")
        for a, b in ((r"\bfragColor\.g\b", "fragColor.c.y"), (r"\bfragColor\.b\b", "fragColor.c.z"),
                     (r"\bhdr\.g\b", "hdr.y"), (r"\bhdr\.b\b", "hdr.z"), (r"\bhdr\.a\b", "hdr.w")):
            src, k = re.subn(a, b, src)
            if not k:
                raise SystemExit(f"post.idle.frag: {a} not found")
    if rel == "raytrace.projective.rgen":
        new = src.replace("for (int i = 0; i < NUM_OUTPUT_IMAGES; i++)\n      payload.mRec.channel[i]",
                          "for (int i = 0; i < NUM_OUTPUT_IMAGES - 1; i++)\n      payload.mRec.channel[i]")
        if new == src:
            raise SystemExit("rgen: channel-clear loop not found")
        src = new
    # no other call may take two side-effecting rand() arguments
    for ln in src.splitlines():
        if ln.count("rand(") + ln.count("rand2(") >= 2 and "{rand(seed)" not in ln and "{rand(prev)" not in ln \
                and not ln.strip().startswith("//"):
            raise SystemExit(f"{rel}: multiple RNG draws in one expression: {ln.strip()}")
    if stage:
        out = src.splitlines()
        out.insert(body_start, f"namespace {stage} {{")
        out.append(f"}}  // namespace {stage}")
        src = "\n".join(out)
    header = f"// Generated by oracle/gen_ref.py from the reference's src/shaders/{rel}; do not commit.\n"
    return header + src + "\n"


def main(argv=None):
    ap = argparse.ArgumentParser()
    here = os.path.dirname(os.path.abspath(__file__))
    ap.add_argument("--ref", default=None)
    ap.add_argument("--out", default=os.path.join(here, "_ref", "gen"))
    a = ap.parse_args(argv)
    if a.ref is None:
        a.ref = find_ref_tree()
    if a.ref is None:
        print("reference checkout not found ($ASUNA_REFERENCE, baseline/_ref)", file=sys.stderr)
        return 2
    shaders = os.path.join(a.ref, "src", "shaders")
    if not os.path.isdir(shaders):
        print(f"reference shaders not found under {shaders}", file=sys.stderr)
        return 2
    os.makedirs(a.out, exist_ok=True)
    for rel, stage in SHADERS.items():
        with open(os.path.join(shaders, rel)) as f:
            txt = f.read()
        with open(os.path.join(a.out, out_name(rel)), "w") as f:
            f.write(translate(txt, rel, stage))
    shared_in, shared_out = os.path.join(a.ref, "src", "shared"), os.path.join(a.out, "shared")
    os.makedirs(shared_out, exist_ok=True)
    for name in sorted(os.listdir(shared_in)):
        if name.endswith(".h"):
            shutil.copyfile(os.path.join(shared_in, name), os.path.join(shared_out, name))
    with open(os.path.join(a.out, MANIFEST), "w") as f:
        f.write(os.path.abspath(a.ref) + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
