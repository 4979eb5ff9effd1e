#!/usr/bin/env python3
"""Build oracle/_ref/libsvo_ref.so from the reference's own GLSL shader source.

TEST INFRASTRUCTURE ONLY.  The reference (AdamYuan/SparseVoxelOctree) runs its hot path as Vulkan
shaders; Vulkan is not available here, but the compute, march, camera and diffuse shaders are plain
GLSL arithmetic.  This recipe reads them where they lie in the reference checkout, rewrites the
handful of GLSL-only constructs into C++ that oracle/ref_shim/glsl_shim.hpp understands, writes the
result to oracle/_ref/ (git-ignored, never committed) and compiles it with g++ together with
oracle/ref_shim/harness.cpp.  Nothing is copied into the repository.

Rewrites (each keeps the shader's meaning):
  * drop #version / #extension lines and the layout(...) declarations of buffers, uniforms, push
    constants, specialisation constants, workgroup sizes and stage interfaces (the shim declares
    globals with the same names that the harness binds);
  * `out T x` parameters become `T &x`, `in` qualifiers are dropped;
  * unsuffixed floating literals get an `f` suffix (GLSL literals are float, C++ ones double);
  * rvalue swizzles `.xy/.xyz/.yzx/.zxy/.zw` become calls `._xy()` ...; compound-assigned ones stay;
  * `discard;` throws glsl_discard; `void main()` becomes `void <shader>_main()`;
  * the march's private `uint stack[]` becomes thread_local; each file goes into its own namespace.

Usage: python oracle/build_ref.py [--reference DIR]   (default: $SVO_REFERENCE or /root/reference)
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

SHADERS = [
    # (file, namespace, main-function name or None)
    ("octree_init_node.comp", "ref_init", "init_main"),
    ("octree_tag_node.comp", "ref_tag", "tag_main"),
    ("octree_alloc_node.comp", "ref_alloc", "alloc_main"),
    ("octree_modify_arg.comp", "ref_modify", "modify_main"),
    ("octree.glsl", "ref_octree", None),
    ("camera.glsl", "ref_camera", None),
    ("util.glsl", "ref_util", None),
    ("diffuse.glsl", "ref_diffuse", None),
    ("voxelizer.geom", "ref_vgeom", "geom_main"),
    ("voxelizer_conservative.geom", "ref_vgeom_cons", "geom_main"),
    ("voxelizer.frag", "ref_vfrag", "frag_main"),
    ("sobol.glsl", "ref_sobol", None),
    ("sobol.comp", "ref_sobolc", "sobol_main"),
    ("mis.glsl", "ref_mis", None),
    ("environment_map.glsl", "ref_envmap", None),
    ("path_tracer.comp", "ref_pt", "pt_main"),
]

# Per-file rewrites on top of transform(): environment_map.glsl is compiled with its sampling half
# enabled (path_tracer.comp defines ENVIRONMENT_MAP_ENABLE_SAMPLE before including it) and its
# image-size global becomes an expression evaluated at use; sobol.comp's workgroup-shared variable
# becomes a static and its direction-number table writable (a harness may run the shader with other
# numbers); isnan maps to the shim's.
FILE_FIXUPS = {
    "environment_map.glsl": [(r"ivec2\s+env_map_dim\s*=[^;]*;", "#define env_map_dim textureSize(uEnvironmentMap, 0)"),
                             (r"#ifndef ENVIRONMENT_MAP_ENABLE_SAMPLE", "#define ENVIRONMENT_MAP_ENABLE_SAMPLE 1\n#ifndef ENVIRONMENT_MAP_ENABLE_SAMPLE")],
    "sobol.comp": [(r"^shared\s+", "static "), (r"^const\s+uint\s+kMatrices", "uint kMatrices")],
    "path_tracer.comp": [(r"\bisnan\(", "glsl_isnan(")],
}

# EnvironmentMap::weigh_hdr_image and generate_alias_table (src/EnvironmentMap.cpp), compiled from their
# place in the reference against stubs of the few library names they use.
ENVMAP_PRELUDE = """// generated by oracle/build_ref.py from the reference's src/EnvironmentMap.cpp; do not commit
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>
namespace spdlog { template <class... A> inline void info(A &&...) {} }
namespace glm {
using std::sin;
template <class T> inline T clamp(T x, T lo, T hi) { return std::min(std::max(x, lo), hi); }
}
struct EnvironmentMap {
	struct HdrImg { uint32_t m_width, m_height; float *m_data; };
	struct AliasPair { uint32_t m_prob, m_alias; };
	static std::vector<double> weigh_hdr_image(const HdrImg *img);
	static void generate_alias_table(std::vector<double> *weights_ptr, AliasPair *alias_table);
};
"""

FLOAT_LIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")
SWIZZLE = re.compile(r"\.(xyz|yzx|zxy|xy|zw)\b(?!\s*[-+*/]?=(?!=))")


def transform(src: str, namespace: str, main_name: str | None) -> str:
    s = src
    s = re.sub(r"^\s*#\s*(version|extension)\b.*$", "", s, flags=re.M)
    # buffer / uniform blocks (possibly multi-line)
    s = re.sub(r"layout\s*\([^)]*\)\s*(?:readonly\s+|writeonly\s+)*(?:buffer|uniform)\s+\w+\s*\{.*?\}\s*;", "",
               s, flags=re.S)
    # remaining layout(...) declarations: specialisation constants, samplers, interfaces, local size
    s = re.sub(r"^\s*layout\s*\([^)]*\)[^;{]*;", "", s, flags=re.M)
    s = re.sub(r'#include\s+"(\w+)\.glsl"', r'#include "gen_\1.hpp"', s)
    s = re.sub(r"\bout\s+(\w+)\s+(\w+)", r"\1 &\2", s)
    s = re.sub(r"\bin\s+const\b", "const", s)
    s = re.sub(r"\bin\s+(\w+\s+\w+)", r"\1", s)
    s = FLOAT_LIT.sub(lambda m: m.group(1) + "f", s)
    s = SWIZZLE.sub(lambda m: "._" + m.group(1) + "()", s)
    s = re.sub(r"\bdiscard\s*;", "throw glsl_discard{};", s)
    s = re.sub(r"^uint\s+stack\[", "thread_local uint stack[", s, flags=re.M)
    if main_name:
        s = re.sub(r"\bvoid\s+main\s*\(\s*\)", f"void {main_name}()", s)
    # includes must stay outside the namespace
    includes = re.findall(r'^#include "gen_\w+\.hpp"$', s, flags=re.M)
    s = re.sub(r'^#include "gen_\w+\.hpp"$', "", s, flags=re.M)
    head = "\n".join(includes)
    return f"// generated by oracle/build_ref.py from the reference's shader source; do not commit\n" \
           f"#pragma once\n#include \"../ref_shim/glsl_shim.hpp\"\n{head}\nnamespace {namespace} {{\n" \
           f"{s}\n}} // namespace {namespace}\n"


# Where the reference checkout is read from: $SVO_REFERENCE, else the checkout's location in the build
# container (this recipe is the one file that names it; the GPU machine has no checkout and builds nothing here).
DEFAULT_REFERENCE = os.environ.get("SVO_REFERENCE") or "/root/reference"


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=DEFAULT_REFERENCE)
    args = ap.parse_args()
    shader_dir = os.path.join(args.reference, "shader")
    if not os.path.isdir(shader_dir):
        print(f"reference shader directory not found: {shader_dir}", file=sys.stderr)
        return 2
    os.makedirs(OUT, exist_ok=True)
    for fname, ns, main_name in SHADERS:
        with open(os.path.join(shader_dir, fname)) as f:
            src = f.read()
        stem = fname.replace(".", "_")
        if fname.endswith(".glsl"):
            stem = fname[: -len(".glsl")]
        for pat, rep in FILE_FIXUPS.get(fname, []):
            src = re.sub(pat, rep, src, flags=re.M)
        with open(os.path.join(OUT, f"gen_{stem}.hpp"), "w") as f:
            f.write(transform(src, ns, main_name))
    with open(os.path.join(args.reference, "src", "EnvironmentMap.cpp")) as f:
        cpp = f.read()
    begin, end = cpp.index("inline static float luminance"), cpp.index("void EnvironmentMap::create_images")
    with open(os.path.join(OUT, "gen_envmap_cpp.hpp"), "w") as f:
        f.write(ENVMAP_PRELUDE + cpp[begin:end])
    # two builds: GLSL's sin / cos / atan / acos as libm, and as the engine's restatements
    for lib_name, defs in (("libsvo_ref.so", []), ("libsvo_ref_etrig.so", ["-DSHIM_ENGINE_TRIG"])):
        cmd = ["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-w", *defs,
               "-I", OUT, "-o", os.path.join(OUT, lib_name), os.path.join(HERE, "ref_shim", "harness.cpp"),
               "-lpthread"]
        subprocess.run(cmd, check=True)
        print(os.path.join(OUT, lib_name))
    return 0


if __name__ == "__main__":
    sys.exit(main())
