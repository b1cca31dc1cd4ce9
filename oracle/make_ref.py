"""Build the reference-shader CPU library ``oracle/_ref/libref_ibl.so``.

TEST INFRASTRUCTURE ONLY.  Reads the reference's own compute shaders
(Shaders/IBL_Precompute/GenIrradianceMap.comp, PreFilterEnvMap.comp and
Shaders/SSRGlossyConvolve.comp) from the reference checkout, applies a purely
mechanical GLSL -> C++ rewrite and compiles the result against
``oracle/glsl_compat.hpp``:

* drop ``#version``, ``layout(local_size...) in;``, ``//`` comments and the
  ``#include <Bindless/...>`` line (the compat header defines the heap macros);
* ``layout(...) uniform [writeonly] T name;`` -> ``T name;``;
* the push-constant block -> a ``struct`` with a global instance;
* top-level mutable globals (``uvec2 seed;``) -> ``thread_local``;
* ``in T x`` -> ``T x`` and ``out T x`` -> ``T& x`` in parameter lists;
* swizzles ``.xz .yx .xy .rgb`` -> accessor calls;
* float literals get an ``f`` suffix (GLSL literals are single precision);
* ``vec2(rng(), rng())`` -> ``ALTHEA_XI()``, a left-to-right sequenced
  ``vec2{rng(), rng()}`` (C++ leaves constructor-argument order unspecified;
  GLSL evaluates arguments left to right), or the Hammersley source for the
  ``hammersley`` variant;
* ``#define MAX_SAMPLES 10000`` -> a run-time sample count;
* ``main`` -> ``shader_main``, plus a driver that sets
  ``gl_GlobalInvocationID`` for each texel (for SSRGlossyConvolve: for every
  invocation of the reference's dispatch, Src/ReflectionBuffer.cpp:266-268).

Outputs go only to ``oracle/_ref/`` (git-ignored): the generated ``.cpp``
files and the shared library.  The generated sources are kept there so that a
machine without the reference checkout can still compile them
(``python oracle/make_ref.py --compile-only``).
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_ROOT = os.environ.get("ALTHEA_REFERENCE_ROOT", "/root/reference")
SHADER_DIR = os.path.join(REF_ROOT, "Shaders", "IBL_Precompute")

FLOAT_LIT = re.compile(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][+-]?\d+)?(?![\w.])")


def transform(src: str) -> str:
    out = []
    for line in src.splitlines():
        code = line.split("//", 1)[0].rstrip()
        s = code.strip()
        if not s:
            continue
        if s.startswith("#version") or s.startswith("#include <Bindless/"):
            continue
        if re.match(r"layout\s*\(\s*local_size", s):
            continue
        m = re.match(r"layout\s*\([^)]*\)\s*uniform\s+(?:writeonly\s+|readonly\s+)?(\w+)\s+(\w+)\s*;", s)
        if m:
            out.append(f"{m.group(1)} {m.group(2)};")
            continue
        m = re.match(r"layout\s*\(\s*push_constant\s*\)\s*uniform\s+(\w+)\s*\{", s)
        if m:
            out.append(f"struct {m.group(1)} {{")
            continue
        if s.startswith("#define MAX_SAMPLES"):
            out.append("#define MAX_SAMPLES (glslc_max_samples)")
            continue
        if re.match(r"^(uvec2|vec2|vec3|float|int|uint)\s+\w+\s*;$", code):
            code = "thread_local " + code
        code = re.sub(r"([(,]\s*)in\s+(\w+)\s+", r"\1\2 ", code)
        code = re.sub(r"([(,]\s*)out\s+(\w+)\s+", r"\1\2& ", code)
        code = re.sub(r"\.(xz|yx|xy|rgb)\b", r".\1()", code)
        code = code.replace("vec2(rng(), rng())", "ALTHEA_XI()")
        code = re.sub(r"\bvoid\s+main\s*\(", "void shader_main(", code)
        if not code.lstrip().startswith("#include"):
            code = FLOAT_LIT.sub(lambda m: m.group(0) + "f", code)
        out.append(code)
    return "\n".join(out) + "\n"


DRIVER = r"""
// ---- driver (generated) ----------------------------------------------------
extern "C" void {fn}(const float* chain, int w, int h, int levels, float* out,
                     int ow, int oh, {extra_params} const int* xy, int n,
                     int nthreads) {{
  glslc::g_res.chain = chain;
  glslc::g_res.w = w;
  glslc::g_res.h = h;
  glslc::g_res.levels = levels;
  glslc::g_res.out = out;
  glslc::g_res.ow = ow;
  glslc::g_res.oh = oh;
{set_push}
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nt)
  for (int i = 0; i < n; ++i) {{
    glslc::gl_GlobalInvocationID.x = (uint32_t)xy[2 * i];
    glslc::gl_GlobalInvocationID.y = (uint32_t)xy[2 * i + 1];
    glslc::gl_GlobalInvocationID.z = 0;
    glslc::g_sample_index = 0;
    shader_main();
  }}
}}
"""


def make_unit(shader_file: str, ns: str, xi: str, fn: str, prefilter: bool) -> str:
    with open(os.path.join(SHADER_DIR, shader_file), "r", encoding="utf-8") as f:
        body = transform(f.read())
    if prefilter:
        extra = "float roughness, int samples,"
        setp = ("  pushConstants.envMapWidth = (float)w;\n"
                "  pushConstants.envMapHeight = (float)h;\n"
                "  pushConstants.width = (float)ow;\n"
                "  pushConstants.height = (float)oh;\n"
                "  pushConstants.roughness = roughness;\n"
                "  glslc_max_samples = samples;\n"
                "  glslc::g_sample_count = samples;")
    else:
        extra = ""
        # GenIrradianceMap's push constants carry the env size: the reference
        # dispatches it at env size (Src/ImageBasedLighting.cpp:328-343).
        setp = ("  pushConstants.width = (float)w;\n"
                "  pushConstants.height = (float)h;")
    drv = DRIVER.format(fn=fn, extra_params=extra, set_push=setp)
    return (
        "// GENERATED by oracle/make_ref.py from " + shader_file + " -- do not edit.\n"
        "#include <omp.h>\n#include \"../glsl_compat.hpp\"\n"
        f"namespace {ns} {{\nGLSLC_USING\nstatic int glslc_max_samples = 0;\n"
        f"#define ALTHEA_XI() {xi}\n" + body + drv + "}\n#undef ALTHEA_XI\n#undef PI\n#undef MAX_SAMPLES\n"
    )


SSR_DRIVER = r"""
// ---- driver (generated) ----------------------------------------------------
// One vkCmdDispatch of the convolution pass: texture heap slot 0 = level l-1,
// image heap slot 0 = level l, push constants as the caller sets them.
extern "C" void ref_ssr_dispatch(const uint16_t* src, int sw, int sh, uint16_t* dst, int dw,
                                 int dh, unsigned width, unsigned height, float dirx, float diry,
                                 float roughness, int nthreads) {
  glslc::g_heap_tex[0].src = src;
  glslc::g_heap_tex[0].w = sw;
  glslc::g_heap_tex[0].h = sh;
  glslc::g_heap_img[0].dst = dst;
  glslc::g_heap_img[0].w = dw;
  glslc::g_heap_img[0].h = dh;
  pushConstants.srcMipTexHandle = 0;
  pushConstants.targetMipImgHandle = 0;
  pushConstants.width = width;
  pushConstants.height = height;
  pushConstants.direction = vec2(dirx, diry);
  pushConstants.roughness = roughness;
  const unsigned gx = (width - 1) / 16 + 1, gy = (height - 1) / 16 + 1;
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long long i = 0; i < (long long)gx * 16 * gy * 16; ++i) {
    glslc::gl_GlobalInvocationID.x = (uint32_t)(i % (gx * 16));
    glslc::gl_GlobalInvocationID.y = (uint32_t)(i / (gx * 16));
    glslc::gl_GlobalInvocationID.z = 0;
    shader_main();
  }
}
"""


def make_ssr_unit() -> str:
    path = os.path.join(REF_ROOT, "Shaders", "SSRGlossyConvolve.comp")
    with open(path, "r", encoding="utf-8") as f:
        body = transform(f.read())
    return (
        "// GENERATED by oracle/make_ref.py from SSRGlossyConvolve.comp -- do not edit.\n"
        "#include <omp.h>\n#include \"../glsl_compat.hpp\"\n"
        "namespace ref_ssr {\nGLSLC_USING\n" + body + SSR_DRIVER + "}\n"
    )


UNITS = [
    ("PreFilterEnvMap.comp", "ref_prefilter_hash", "vec2{rng(), rng()}", "ref_prefilter_hash", True),
    ("PreFilterEnvMap.comp", "ref_prefilter_hammersley", "glslc::hammersley_next()", "ref_prefilter_hammersley", True),
    ("GenIrradianceMap.comp", "ref_irradiance", "vec2{rng(), rng()}", "ref_irradiance_raw", False),
]


def generate() -> None:
    os.makedirs(OUT, exist_ok=True)
    for shader, ns, xi, fn, pre in UNITS:
        with open(os.path.join(OUT, ns + ".cpp"), "w", encoding="utf-8") as f:
            f.write(make_unit(shader, ns, xi, fn, pre))
    with open(os.path.join(OUT, "ref_ssr.cpp"), "w", encoding="utf-8") as f:
        f.write(make_ssr_unit())


def compile_lib() -> str:
    srcs = [os.path.join(OUT, ns + ".cpp") for _, ns, _, _, _ in UNITS]
    if os.path.exists(os.path.join(OUT, "ref_ssr.cpp")):
        srcs.append(os.path.join(OUT, "ref_ssr.cpp"))
    srcs.append(os.path.join(HERE, "ref_support.cpp"))
    lib = os.path.join(OUT, "libref_ibl.so")
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", lib] + srcs
    subprocess.check_call(cmd)
    return lib


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--compile-only", action="store_true",
                    help="compile previously generated sources (no reference checkout needed)")
    args = ap.parse_args()
    if not args.compile_only:
        if not os.path.isdir(SHADER_DIR):
            print(f"reference shaders not found at {SHADER_DIR}", file=sys.stderr)
            return 1
        generate()
    print(compile_lib())
    return 0


if __name__ == "__main__":
    sys.exit(main())
