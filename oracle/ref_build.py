"""Builds oracle/_ref/libref_setup.so: the reference's own quad-setup functions compiled as C++.

The reference's hot path exists only as GLSL compute shaders, and no graphics stack is available
to run them. Its setup arithmetic, though, is written as straight-line GLSL functions over vector
types; with the GLSL-in-C++ shim (oracle/glsl_shim.h) they compile as plain C++. This recipe reads
them where they lie in the reference tree (nothing is copied into the repository), extracts:

* from data/shaders/quad_setup.glsl: vertexLoad, vertexClipMask, computeClippedAABB,
  computeAABB, processInputQuad, storeQuad, storeTri, addVisibleQuad, addVisibleTri, its
  #define lines and its `shared` declarations;
* from data/shaders/shared/funcs.glsl: encodeNormalUint, encodeAABB28;
* from data/shaders/shared/definitions.glsl: the INST_*, REJECTION_TYPE_* and STORAGE_* macros;
* from data/shaders/shared/structures.glsl: the InstanceData, Lighting, Frustum and
  LucidConfig structs;
* from data/shaders/bin_counter.glsl: scanlineStep, countSmallQuadBins, loadScanlineParamsBin,
  countLargeTriBins, with the ScanlineParams loaders of shared/scanline.glsl and decodeAABB28;
* from data/shaders/raster_low.glsl: scratchBlockRowOffset, generateRowTris, with rasterBinStep
  and the block / half-block macros of shared/raster.glsl;
* from data/shaders/shared/shading.glsl: getTriangleParams, getTriangleVertexColors,
  getTriangleVertexNormals, getTriangleVertexTexCoords, shadeSample, the ReductionContext struct
  with its RC_* macros, swap, initReduceSamples, reduceSample, finishReduceSamples; with
  decodeRGBA8, encodeRGBA8, SRGBToLinear, linearToSRGB, finalShading, the swap helpers and
  SATURATE of shared/funcs.glsl (GLSL's pow is implementation-defined: the harness routes it
  to the oracle's refPow, the one pow both the oracle and the CUDA path use; textureGrad is a
  stub that the tests never reach: their scenes carry no textures);

applies mechanical GLSL-to-C++ rewrites (float literals stay single precision, swizzles become
accessor calls, out / inout parameters references, int() / uint() of floats the GPU's saturating
truncation, `shared` becomes `static`), writes the result to oracle/_ref/ref_setup_gen.inc and
compiles oracle/ref_setup_harness.cpp (which drives the functions exactly as the shader's main()
does, one invocation at a time) into oracle/_ref/libref_setup.so.

Only this container has the reference tree; elsewhere build() returns None and the tests that
use the library skip. Outputs go to oracle/_ref/ only (git-ignored).
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libref_setup.so")
GEN = os.path.join(OUT_DIR, "ref_setup_gen.inc")
REF_ROOT = "/root/reference"
SHADERS = os.path.join(REF_ROOT, "data", "shaders")

SETUP_FUNCS = ["vertexLoad", "vertexClipMask", "computeClippedAABB", "computeAABB", "processInputQuad",
               "storeQuad", "storeTri", "addVisibleQuad", "addVisibleTri"]
FUNCS_FUNCS = ["encodeNormalUint", "encodeAABB28", "decodeAABB28"]
STRUCTS = ["InstanceData", "Lighting", "Frustum", "LucidConfig"]
SCANLINE_FUNCS = ["loadScanlineParamsRow", "loadScanlineParamsBin"]
COUNTER_FUNCS = ["scanlineStep", "countSmallQuadBins", "loadScanlineParamsBin", "countLargeTriBins"]
RASTER_FUNCS = ["rasterBinStep"]
RASTER_LOW_FUNCS = ["scratchBlockRowOffset", "generateRowTris"]
COLOR_FUNCS = ["decodeNormalUint", "decodeRGBA8", "encodeRGBA8", "linearToSRGB", "SRGBToLinear", "finalShading"]
SHADING_FUNCS = ["getTriangleParams", "getTriangleVertexColors", "getTriangleVertexNormals",
                 "getTriangleVertexTexCoords", "shadeSample"]
REDUCE_FUNCS = ["initReduceSamples", "reduceSample", "finishReduceSamples"]


def _read(*parts):
    with open(os.path.join(SHADERS, *parts), encoding="latin-1") as f:
        return f.read()


def _block(text, start):
    """Text from `start` through the brace that closes the first '{' after it."""
    i = text.index("{", start)
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
            if depth == 0:
                return text[start:j + 1]
    raise ValueError("unbalanced braces")


def _function(text, name):
    m = re.search(r"^[A-Za-z_][\w]*\s+" + name + r"\s*\(", text, re.M)
    if not m:
        raise ValueError(f"function {name} not found")
    return _block(text, m.start())


def _struct(text, name):
    m = re.search(r"^struct\s+" + name + r"\s*\{", text, re.M)
    if not m:
        raise ValueError(f"struct {name} not found")
    return _block(text, m.start()) + ";"


FLOAT_LIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][-+]?\d+)?)(?![\w.])")
SWIZZLE = re.compile(r"\.(xyz|xzw|xy|zw|rgb)\b(?!\s*\()")
COMPONENT = re.compile(r"\.([rgba])\b(?!\s*\()")
OUT_PARAM = re.compile(r"\b(?:in\s+out|inout|out)\s+(\w+)\s+(\w+)")


def _to_cpp(src):
    src = FLOAT_LIT.sub(r"\1f", src)      # GLSL float literals are single precision
    src = SWIZZLE.sub(r".\1()", src)       # swizzles: accessor calls of the shim's vector types
    src = COMPONENT.sub(lambda m: "." + "xyzw"["rgba".index(m.group(1))], src)  # .r/.g/.b/.a
    src = OUT_PARAM.sub(r"\1& \2", src)    # out / inout parameters: references
    src = re.sub(r"\buvec4\(aabb\)", "toUvec4(aabb)", src)
    src = re.sub(r"\bint\(", "toInt(", src)    # int() / uint() of floats: the GPU's truncation
    src = re.sub(r"\buint\(", "toUint(", src)
    return src


def _defines(text, pattern, exclude=()):
    out = []
    for line in text.splitlines():
        m = re.match(r"#define\s+(\w+)", line)
        if m and re.match(pattern, m.group(1)) and m.group(1) not in exclude and not line.rstrip().endswith("\\"):
            out.append(line)
    return out


def generate():
    setup = _read("quad_setup.glsl")
    funcs = _read("shared", "funcs.glsl")
    defs = _read("shared", "definitions.glsl")
    structs = _read("shared", "structures.glsl")
    out = ["// generated by oracle/ref_build.py from the reference's shader sources; not committed"]
    for line in defs.splitlines():
        if re.match(r"#define\s+(INST_|REJECTION_TYPE_|STORAGE_|STATS_COUNT)", line):
            out.append(line)
    for line in setup.splitlines():
        if re.match(r"#define\s+(MAX_INSTANCE_QUADS|LSIZE|MAX_PACKET_SIZE)\b", line):
            out.append(line)
    for name in STRUCTS:
        out.append(_to_cpp(_struct(structs, name)))
    # the shader's buffers and uniform block, defined by the harness
    out.append("extern LucidConfig u_config;\nextern float* g_verts;\nextern vec2* g_tex_coords;\n"
               "extern uint* g_colors;\nextern uint* g_normals;\nextern uint* g_quad_aabbs;\n"
               "extern uvec4* g_uvec4_storage;\nextern uint* g_normals_storage;\n"
               "extern InstanceData* g_instances;\nextern int* s_bins;\nextern uvec2* g_scratch_64;\n"
               "extern ivec2 s_bin_pos;")
    for line in setup.splitlines():
        if line.startswith("shared "):
            out.append("static " + line[len("shared "):])
    for name in FUNCS_FUNCS:
        out.append(_to_cpp(_function(funcs, name)))
    for name in SETUP_FUNCS:
        out.append(_to_cpp(_function(setup, name)))
    # bin counter (bin_counter.glsl) with the scanline loaders (shared/scanline.glsl)
    scan = _read("shared", "scanline.glsl")
    counter = _read("bin_counter.glsl")
    out.append(_to_cpp(_struct(scan, "ScanlineParams")))
    for name in SCANLINE_FUNCS:
        out.append(_to_cpp(_function(scan, name)))
    for name in COUNTER_FUNCS:
        out.append(_to_cpp(_function(counter, name)))
    # row spans of the low-level raster (raster_low.glsl with shared/raster.glsl)
    raster = _read("shared", "raster.glsl")
    low = _read("raster_low.glsl")
    out += _defines(raster, r"(BIN_MASK|BLOCK_|HBLOCK_|NUM_BLOCKS|NUM_HBLOCKS)")
    out += _defines(low, r"(MAX_BLOCK_|WORKGROUP_SCRATCH_)")
    for line in low.splitlines():
        if line.startswith("shared uint s_block_row_tri_count"):
            out.append("static " + line[len("shared "):])
    for name in RASTER_FUNCS:
        out.append(_to_cpp(_function(raster, name)))
    for name in RASTER_LOW_FUNCS:
        out.append(_to_cpp(_function(low, name)))
    # shading and the 3-deep reduction window (shared/shading.glsl with shared/funcs.glsl)
    shading = _read("shared", "shading.glsl")
    for line in funcs.splitlines():
        if re.match(r"#define\s+SATURATE\b", line):
            out.append(line)
    for m in re.finditer(r"^void swap\(inout (float|uint|int) a, inout \1 b\)", funcs, re.M):
        out.append(_to_cpp(_block(funcs, m.start())))
    for name in COLOR_FUNCS:
        out.append(_to_cpp(_function(funcs, name)))
    out.append("extern uint* g_instance_colors;\nextern vec4* g_instance_uv_rects;\n"
               "extern sampler2D opaque_texture, transparent_texture;\nextern uint s_stats[STATS_COUNT];")
    for name in SHADING_FUNCS:
        out.append(_to_cpp(_function(shading, name)))
    i0 = shading.index("#define RC_COLOR_SIZE")
    i1 = shading.index("struct ReductionContext")
    out.append(shading[i0:i1].strip())
    out.append(_to_cpp(_struct(shading, "ReductionContext")))
    m = re.search(r"^void swap\(inout ReductionContext", shading, re.M)
    out.append(_to_cpp(_block(shading, m.start())))
    for name in REDUCE_FUNCS:
        out.append(_to_cpp(_function(shading, name)))
    return "\n\n".join(out) + "\n"


def available():
    return os.path.isdir(SHADERS)


def build(force=False):
    """Builds the library when the reference tree is present; returns its path, or None."""
    if not available():
        return None
    srcs = [os.path.join(HERE, "ref_setup_harness.cpp"), os.path.join(HERE, "glsl_shim.h"), __file__]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(s) <= os.path.getmtime(LIB) for s in srcs):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    with open(GEN, "w") as f:
        f.write(generate())
    cmd = ["g++", "-O2", "-std=c++20", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-I", OUT_DIR, "-I", HERE, "-I", os.path.join(HERE, "..", "include"), "-o", LIB + ".tmp",
           os.path.join(HERE, "ref_setup_harness.cpp")]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
