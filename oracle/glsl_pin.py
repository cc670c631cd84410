"""The reference's own shader text, compiled as C++ for the CPU.  TEST INFRASTRUCTURE ONLY.

The reference's voxel path is GLSL run through Vulkan, which no machine here can run.  Its arithmetic does not need
a GPU, though: this script takes the functions the oracle restates out of the reference's own files, verbatim, and
compiles them under a small GLSL vocabulary (oracle/glsl_shim.h) into oracle/_ref/libf184glsl.so:

  Shader/math.inc            PI, hemisphereSample_cos
  Shader/Lighting/indirect.frag
                             lambertBrdf, HitState, make_coord_space, unpackColor565, unpackNormal565, getIndirect,
                             second_bounce and main()'s four rays with their second bounces (up to `indirect *= 0.25`)
  Pipelang/Internal/main.lua VoxelGS's dominant-axis choice, VoxelPS's RGB565 albedo and normal packing

Three mechanical translations of GLSL into C++, and nothing else, are applied to the text:
  1. float literals get an `f` suffix (a GLSL float literal is single precision; a C++ one is double);
  2. `inout T name` parameters become `T& name` (the reference never aliases them, so copy-in/copy-out and a
     reference agree);
  3. `state.brdf * getIndirect(...)` is spelled `lr_mul{state.brdf, getIndirect(...)}`: GLSL reads the left operand
     before the call that rewrites `state`, C++ leaves the order of the operands of `*` open, and a braced list is
     evaluated left to right.
The noise the shader draws (hash, blugausnoise2) is supplied by the harness (the same numbers the restatement uses),
and the volume, shadow map, matrices and sun are set through ref_march_setup.  Only built where the reference tree
is present (F184_REFERENCE, default /root/reference); tests skip without it.

    python oracle/glsl_pin.py      # writes oracle/_ref/glsl_pin.cpp and builds oracle/_ref/libf184glsl.so
"""
import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("F184_REFERENCE", "/root/reference")
OUT_DIR = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT_DIR, "glsl_pin.cpp")
LIB = os.path.join(OUT_DIR, "libf184glsl.so")


def _read(rel):
    with open(os.path.join(REF_ROOT, rel)) as f:
        return f.read()


def _line_of(text, pos):
    return text.count("\n", 0, pos) + 1


def _function(text, name, rel):
    """The definition of GLSL function `name` (return type through its closing brace) and its line range."""
    m = re.search(r"^[ \t]*\w+[ \t]+%s[ \t]*\([^)]*\)[ \t\r\n]*\{" % re.escape(name), text, re.M)
    if not m:
        raise RuntimeError("%s: function %s not found" % (rel, name))
    depth, i = 0, m.end() - 1
    while True:
        c = text[i]
        depth += c == "{"
        depth -= c == "}"
        i += 1
        if depth == 0:
            break
    return text[m.start():i], (_line_of(text, m.start()), _line_of(text, i))


def _struct(text, name, rel):
    m = re.search(r"^struct[ \t]+%s[ \t]*\{.*?\};" % re.escape(name), text, re.M | re.S)
    if not m:
        raise RuntimeError("%s: struct %s not found" % (rel, name))
    return m.group(0), (_line_of(text, m.start()), _line_of(text, m.end()))


def _between(text, start, end, rel, include_end=True):
    a = text.find(start)
    if a < 0:
        raise RuntimeError("%s: %r not found" % (rel, start))
    b = text.find(end, a)
    if b < 0:
        raise RuntimeError("%s: %r not found after %r" % (rel, end, start))
    if include_end:
        b += len(end)
    return text[a:b], (_line_of(text, a), _line_of(text, b))


FLOAT_LIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?)(?![\w.])")


def glsl_to_cpp(code):
    code = FLOAT_LIT.sub(r"\1f", code)
    code = re.sub(r"\binout[ \t]+(\w+)[ \t]+(\w+)", r"\1& \2", code)
    code = re.sub(r"(\bstate\.brdf)[ \t]*\*[ \t]*(getIndirect\([^;]*\));", r"lr_mul{\1, \2};", code)
    return code


def extract():
    pieces = []  # (citation, code)
    math_inc = _read("Shader/math.inc")
    m = re.search(r"^const float PI = [^;]*;", math_inc, re.M)
    if not m:
        raise RuntimeError("Shader/math.inc: PI not found")
    pieces.append(("Shader/math.inc:%d" % _line_of(math_inc, m.start()), m.group(0)))
    code, (a, b) = _function(math_inc, "hemisphereSample_cos", "Shader/math.inc")
    pieces.append(("Shader/math.inc:%d-%d" % (a, b), code))
    frag_rel = "Shader/Lighting/indirect.frag"
    frag = _read(frag_rel)
    for kind, name in (("f", "lambertBrdf"), ("s", "HitState"), ("f", "make_coord_space"), ("f", "unpackColor565"),
                       ("f", "unpackNormal565"), ("f", "getIndirect")):
        code, (a, b) = (_function if kind == "f" else _struct)(frag, name, frag_rel)
        pieces.append(("%s:%d-%d" % (frag_rel, a, b), code))
    m = re.search(r"^const bool second_bounce = [^;]*;", frag, re.M)
    if not m:
        raise RuntimeError("%s: second_bounce not found" % frag_rel)
    pieces.append(("%s:%d" % (frag_rel, _line_of(frag, m.start())), m.group(0)))
    main_body, (a, b) = _between(frag, "HitState state;", "indirect *= 0.25;", frag_rel)
    pieces.append(("%s:%d-%d" % (frag_rel, a, b),
                   "vec3 ref_pixel(vec3 wpos, vec3 wnorm) {\n    " + main_body +
                   "\n    return indirect;\n}"))
    lua_rel = "Pipelang/Internal/main.lua"
    lua = _read(lua_rel)
    gs, _ = _between(lua, "function VoxelGS()", "EndPrimitive();", lua_rel)
    gs_at = lua.find("function VoxelGS()")
    axis, (a, b) = _between(gs, "vec3 faceNormal = cross(", "for(i = 0; i < gl_in.length(); i++)", lua_rel,
                            include_end=False)
    a += _line_of(lua, gs_at) - 1
    b += _line_of(lua, gs_at) - 2
    pieces.append(("%s:%d-%d" % (lua_rel, a, b),
                   "uint ref_dominant_axis(const vec3 viewPos[3]) {\n    uint iOrientation = 0u;\n    " + axis +
                   "\n    return iOrientation;\n}"))
    ps, _ = _between(lua, "function VoxelPS()", "imageStore(", lua_rel)
    ps_at = lua.find("function VoxelPS()")
    pack, (a, b) = _between(ps, "uint packedColor =", "uint(iNormal.b * 16 + 15);", lua_rel)
    a += _line_of(lua, ps_at) - 1
    b += _line_of(lua, ps_at) - 1
    pieces.append(("%s:%d-%d" % (lua_rel, a, b),
                   "void ref_pack565(const vec4 BaseColor, const vec3 iNormal, uint out2[2]) {\n    " + pack +
                   "\n    out2[0] = packedColor;\n    out2[1] = packedNormal;\n}"))
    return pieces


PRELUDE = r'''// GENERATED by oracle/glsl_pin.py from the reference's shader sources (test infrastructure, not committed).
#include <cstdint>
#include "glsl_shim.h"
using namespace glsl;

namespace ref {
// the fragment's interface (indirect.frag:5-41), set by ref_march_setup
vec2 inUV, resolution;
uint frameCount = 0u;
float iiTime = 0.0f;
sampler s;
texture2D t_shadow;
uimage3D voxels;
mat4 InvModelView, ShadowView, ShadowProj, VoxelView, VoxelProj;
struct SunBlock { vec3 luminance; vec3 position; } sun;

// The shader's noise, supplied by the harness: hash(vec2(randSeed)) names the ray (getIndirect calls it first),
// then blugausnoise2 returns that ray's rands.x and rands.y in turn.
const float* g_rands = nullptr;  // [seed][2]
int g_seed = 0, g_next = 0;
float hash(vec2 p) {
    g_seed = int(p.x);
    g_next = 0;
    return 0.0f;
}
float blugausnoise2(vec2) { return g_rands[g_seed * 2 + (g_next++ & 1)]; }

struct lr_mul {  // a * b with a read before b is evaluated (braced lists evaluate left to right)
    vec3 a, b;
    operator vec3() const { return a * b; }
};
inline vec3& operator+=(vec3& x, const lr_mul& m) { return x += vec3(m); }
'''

EPILOGUE = r'''
}  // namespace ref

extern "C" {
void ref_hemisphere_sample_cos(float u, float v, float out[3]) {
    const glsl::vec3 d = ref::hemisphereSample_cos(u, v);
    out[0] = d.x, out[1] = d.y, out[2] = d.z;
}
void ref_make_coord_space(const float n[3], float out[9]) {  // rows: x, y, z axes
    const glsl::mat3 m = ref::make_coord_space(glsl::vec3(n[0], n[1], n[2]));
    for (int i = 0; i < 3; ++i) out[i * 3] = m.c[i].x, out[i * 3 + 1] = m.c[i].y, out[i * 3 + 2] = m.c[i].z;
}
void ref_unpack_color565(uint32_t x, float out[3]) {
    const glsl::vec3 c = ref::unpackColor565(x);
    out[0] = c.x, out[1] = c.y, out[2] = c.z;
}
void ref_unpack_normal565(uint32_t x, float out[3]) {
    const glsl::vec3 c = ref::unpackNormal565(x);
    out[0] = c.x, out[1] = c.y, out[2] = c.z;
}
uint32_t ref_dominant_axis(const float v[9]) {
    const glsl::vec3 p[3] = {glsl::vec3(v[0], v[1], v[2]), glsl::vec3(v[3], v[4], v[5]), glsl::vec3(v[6], v[7], v[8])};
    return ref::ref_dominant_axis(p);
}
void ref_pack565(const float rgba[4], const float n[3], uint32_t out[2]) {
    ref::ref_pack565(glsl::vec4(rgba[0], rgba[1], rgba[2], rgba[3]), glsl::vec3(n[0], n[1], n[2]), out);
}
// voxels: size^3 RG16UI packed r | g << 16; shadow: res x res R32F; matrices row-major 4x4 (as tc::Matrix4)
void ref_march_setup(const uint32_t* vol, int size, const float* shadow, int res, const float voxel_proj[16],
                     const float voxel_view[16], const float shadow_proj[16], const float shadow_view[16],
                     const float lum[3], const float dir[3], uint32_t frame_count) {
    ref::voxels.texels = vol, ref::voxels.size = size;
    ref::t_shadow.texels = shadow, ref::t_shadow.width = res, ref::t_shadow.height = res;
    const float* src[4] = {voxel_proj, voxel_view, shadow_proj, shadow_view};
    glsl::mat4* dst[4] = {&ref::VoxelProj, &ref::VoxelView, &ref::ShadowProj, &ref::ShadowView};
    for (int k = 0; k < 4; ++k)
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) dst[k]->m[c][r] = src[k][r * 4 + c];
    ref::sun.luminance = glsl::vec3(lum[0], lum[1], lum[2]);
    ref::sun.position = glsl::vec3(dir[0], dir[1], dir[2]);
    ref::frameCount = frame_count;
}
// n points: wpos, wnorm (3 floats each), rands [n][8][2] -> out [n][3] (main()'s indirect before the temporal blend)
void ref_march_points(const float* wpos, const float* wnorm, const float* rands, uint64_t n, float* out) {
    for (uint64_t i = 0; i < n; ++i) {
        ref::g_rands = rands + i * 16;
        const glsl::vec3 o = ref::ref_pixel(glsl::vec3(wpos[i * 3], wpos[i * 3 + 1], wpos[i * 3 + 2]),
                                            glsl::vec3(wnorm[i * 3], wnorm[i * 3 + 1], wnorm[i * 3 + 2]));
        out[i * 3] = o.x, out[i * 3 + 1] = o.y, out[i * 3 + 2] = o.z;
    }
}
}
'''


def build(force=False):
    """Extract, generate and compile; returns the library path, or None where the reference tree is absent."""
    if not os.path.isdir(REF_ROOT):
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [__file__, os.path.join(HERE, "glsl_shim.h")]
    if os.path.exists(LIB) and not force and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    parts = [PRELUDE]
    for cite, code in extract():
        parts.append("\n// ---- %s (verbatim, then the literal / inout / operand-order translations) ----\n" % cite)
        parts.append(glsl_to_cpp(code))
        parts.append("\n")
    parts.append(EPILOGUE)
    with open(SRC, "w") as f:
        f.write("".join(parts))
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-w", "-I", HERE,
           SRC, "-o", LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("glsl pin build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(force=True))
