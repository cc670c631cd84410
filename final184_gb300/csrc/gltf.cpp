// gltf.cpp -- glTF 2.0 scenes as world-space triangle lists (f184gi_gltf_load).
//
// Stands in for the reference's importer (Foreground/SceneGraph/glTFSceneImporter.cpp:200-440), which reads the
// file with tinygltf (a third-party submodule, absent from the reference tree, version not pinned there), walks
// the default scene's node tree (matrix, or translation * rotation * scale, composed with the parent:
// glTFSceneImporter.cpp:355-385) and keeps each mesh primitive with its material.  This loader follows the
// Khronos glTF 2.0 specification for the same walk and flattens it into what the voxelizer consumes: triangles in
// world space, one RGBA8 albedo and one roughness per triangle, and one object per (node, primitive) instance.
//   - .glb (binary container) or .gltf (JSON); buffers from the GLB chunk, a base64 data URI or a file next to
//     the .gltf;
//   - POSITION accessors of FP32 VEC3; indices of u8/u16/u32 or none; modes 4 (triangles), 5 (strip), 6 (fan);
//     points and lines are skipped; sparse accessors are refused;
//   - material: pbrMetallicRoughness.baseColorFactor (default white) and roughnessFactor (default 1) -- the
//     glTF names; the reference asks tinygltf for the older "baseColor"/"roughness" keys and falls back to the
//     same defaults (glTFSceneImporter.cpp:181-196); textures are not sampled.
// Light: the reference's sun (App/MainBehaviour.cpp:40-44: colour (1.1, 0.93, 0.81) x 4, node rotated by the
// Euler angles (-75, -30, 50) degrees, shining along its -Z).  Camera: outside the bounds, looking at the centre.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "gi_internal.h"

namespace f184 {
namespace {

// ---------------- JSON ----------------
struct JVal {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<JVal> arr;
    std::vector<std::pair<std::string, JVal>> obj;
    const JVal* get(const char* key) const {
        if (kind != Obj) return nullptr;
        for (const auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    double num_or(const char* key, double d) const {
        const JVal* v = get(key);
        return v && v->kind == Num ? v->num : d;
    }
    int64_t int_or(const char* key, int64_t d) const {
        const JVal* v = get(key);
        return v && v->kind == Num ? int64_t(v->num) : d;
    }
};

struct JParser {
    const char* p;
    const char* end;
    std::string err;
    int depth = 0;
    void ws() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
    }
    bool fail(const char* m) {
        if (err.empty()) err = m;
        return false;
    }
    bool lit(const char* s) {
        size_t n = std::strlen(s);
        if (size_t(end - p) < n || std::strncmp(p, s, n) != 0) return fail("bad literal");
        p += n;
        return true;
    }
    static void utf8(std::string& o, uint32_t c) {
        if (c < 0x80) {
            o += char(c);
        } else if (c < 0x800) {
            o += char(0xC0 | (c >> 6)), o += char(0x80 | (c & 0x3F));
        } else if (c < 0x10000) {
            o += char(0xE0 | (c >> 12)), o += char(0x80 | ((c >> 6) & 0x3F)), o += char(0x80 | (c & 0x3F));
        } else {
            o += char(0xF0 | (c >> 18)), o += char(0x80 | ((c >> 12) & 0x3F)), o += char(0x80 | ((c >> 6) & 0x3F)),
                o += char(0x80 | (c & 0x3F));
        }
    }
    bool hex4(uint32_t& c) {
        if (end - p < 4) return fail("bad \\u escape");
        c = 0;
        for (int i = 0; i < 4; ++i) {
            char h = *p++;
            c <<= 4;
            if (h >= '0' && h <= '9') c |= uint32_t(h - '0');
            else if (h >= 'a' && h <= 'f') c |= uint32_t(h - 'a' + 10);
            else if (h >= 'A' && h <= 'F') c |= uint32_t(h - 'A' + 10);
            else return fail("bad \\u escape");
        }
        return true;
    }
    bool string(std::string& o) {
        if (p >= end || *p != '"') return fail("expected a string");
        ++p;
        while (p < end && *p != '"') {
            char c = *p++;
            if (c != '\\') {
                o += c;
                continue;
            }
            if (p >= end) return fail("bad escape");
            char e = *p++;
            switch (e) {
                case '"': o += '"'; break;
                case '\\': o += '\\'; break;
                case '/': o += '/'; break;
                case 'b': o += '\b'; break;
                case 'f': o += '\f'; break;
                case 'n': o += '\n'; break;
                case 'r': o += '\r'; break;
                case 't': o += '\t'; break;
                case 'u': {
                    uint32_t c1;
                    if (!hex4(c1)) return false;
                    if (c1 >= 0xD800 && c1 < 0xDC00 && end - p >= 6 && p[0] == '\\' && p[1] == 'u') {
                        p += 2;
                        uint32_t c2;
                        if (!hex4(c2)) return false;
                        c1 = 0x10000 + ((c1 - 0xD800) << 10) + (c2 - 0xDC00);
                    }
                    utf8(o, c1);
                    break;
                }
                default: return fail("bad escape");
            }
        }
        if (p >= end) return fail("unterminated string");
        ++p;
        return true;
    }
    bool value(JVal& v) {
        if (++depth > 256) return fail("nesting too deep");
        ws();
        if (p >= end) return fail("unexpected end");
        bool ok = true;
        if (*p == '{') {
            v.kind = JVal::Obj;
            ++p;
            ws();
            if (p < end && *p == '}') {
                ++p;
            } else {
                while (ok) {
                    ws();
                    std::pair<std::string, JVal> kv;
                    if (!string(kv.first)) return false;
                    ws();
                    if (p >= end || *p != ':') return fail("expected ':'");
                    ++p;
                    if (!value(kv.second)) return false;
                    v.obj.push_back(std::move(kv));
                    ws();
                    if (p < end && *p == ',') {
                        ++p;
                    } else if (p < end && *p == '}') {
                        ++p;
                        break;
                    } else {
                        return fail("expected ',' or '}'");
                    }
                }
            }
        } else if (*p == '[') {
            v.kind = JVal::Arr;
            ++p;
            ws();
            if (p < end && *p == ']') {
                ++p;
            } else {
                while (true) {
                    JVal e;
                    if (!value(e)) return false;
                    v.arr.push_back(std::move(e));
                    ws();
                    if (p < end && *p == ',') {
                        ++p;
                    } else if (p < end && *p == ']') {
                        ++p;
                        break;
                    } else {
                        return fail("expected ',' or ']'");
                    }
                }
            }
        } else if (*p == '"') {
            v.kind = JVal::Str;
            ok = string(v.str);
        } else if (*p == 't') {
            v.kind = JVal::Bool, v.b = true;
            ok = lit("true");
        } else if (*p == 'f') {
            v.kind = JVal::Bool;
            ok = lit("false");
        } else if (*p == 'n') {
            ok = lit("null");
        } else {
            char* q = nullptr;
            std::string tok;
            const char* s = p;
            while (p < end && (std::strchr("+-.eE", *p) || (*p >= '0' && *p <= '9'))) ++p;
            tok.assign(s, p);
            if (tok.empty()) return fail("unexpected character");
            v.kind = JVal::Num;
            v.num = std::strtod(tok.c_str(), &q);
            if (!q || *q != '\0') return fail("bad number");
        }
        --depth;
        return ok;
    }
};

// ---------------- glTF ----------------
constexpr uint32_t kGlbMagic = 0x46546C67u, kChunkJson = 0x4E4F534Au, kChunkBin = 0x004E4942u;

bool read_file(const std::string& path, std::vector<unsigned char>& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    f.seekg(0, std::ios::end);
    std::streamoff n = f.tellg();
    if (n < 0) return false;
    f.seekg(0);
    out.resize(size_t(n));
    if (n > 0) f.read(reinterpret_cast<char*>(out.data()), n);
    return bool(f) || n == 0;
}

bool base64(const std::string& s, size_t start, std::vector<unsigned char>& out) {
    auto val = [](char c) -> int {
        if (c >= 'A' && c <= 'Z') return c - 'A';
        if (c >= 'a' && c <= 'z') return c - 'a' + 26;
        if (c >= '0' && c <= '9') return c - '0' + 52;
        if (c == '+' || c == '-') return 62;
        if (c == '/' || c == '_') return 63;
        return -1;
    };
    uint32_t acc = 0;
    int bits = 0;
    for (size_t i = start; i < s.size(); ++i) {
        char c = s[i];
        if (c == '=') break;
        int v = val(c);
        if (v < 0) {
            if (c == '\n' || c == '\r' || c == ' ') continue;
            return false;
        }
        acc = (acc << 6) | uint32_t(v);
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back(static_cast<unsigned char>((acc >> bits) & 0xFFu));
        }
    }
    return true;
}

struct Mat4 {  // column-major 4x4 (glTF's convention), FP64
    double m[16];
    static Mat4 identity() {
        Mat4 r{};
        r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0;
        return r;
    }
    Mat4 operator*(const Mat4& b) const {
        Mat4 r{};
        for (int c = 0; c < 4; ++c)
            for (int rr = 0; rr < 4; ++rr) {
                double s = 0.0;
                for (int k = 0; k < 4; ++k) s += m[k * 4 + rr] * b.m[c * 4 + k];
                r.m[c * 4 + rr] = s;
            }
        return r;
    }
};

// local transform of a node: its matrix, else T * R * S (rotation quaternion x, y, z, w)
Mat4 node_local(const JVal& n) {
    const JVal* mat = n.get("matrix");
    if (mat && mat->kind == JVal::Arr && mat->arr.size() == 16) {
        Mat4 r;
        for (int i = 0; i < 16; ++i) r.m[i] = mat->arr[i].num;
        return r;
    }
    double t[3] = {0, 0, 0}, q[4] = {0, 0, 0, 1}, s[3] = {1, 1, 1};
    if (const JVal* v = n.get("translation"))
        for (size_t i = 0; i < 3 && i < v->arr.size(); ++i) t[i] = v->arr[i].num;
    if (const JVal* v = n.get("rotation"))
        for (size_t i = 0; i < 4 && i < v->arr.size(); ++i) q[i] = v->arr[i].num;
    if (const JVal* v = n.get("scale"))
        for (size_t i = 0; i < 3 && i < v->arr.size(); ++i) s[i] = v->arr[i].num;
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    const double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w),
                         2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
                         2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)};  // row-major
    Mat4 r = Mat4::identity();
    for (int rr = 0; rr < 3; ++rr)
        for (int c = 0; c < 3; ++c) r.m[c * 4 + rr] = R[rr * 3 + c] * s[c];
    for (int rr = 0; rr < 3; ++rr) r.m[12 + rr] = t[rr];
    return r;
}

struct Loader {
    JVal doc;
    std::string dir;
    std::vector<unsigned char> glb_bin;
    bool has_glb_bin = false;
    std::vector<std::vector<unsigned char>> buffers;
    std::vector<float> xyz;
    std::vector<uint32_t> albedo;
    std::vector<float> rough;
    std::vector<uint32_t> first, count;
    std::string err;

    bool fail(const std::string& m) {
        if (err.empty()) err = m;
        return false;
    }
    const JVal* arr(const char* key) const {
        const JVal* v = doc.get(key);
        return v && v->kind == JVal::Arr ? v : nullptr;
    }
    bool load_buffers() {
        const JVal* bs = arr("buffers");
        if (!bs) return true;
        for (size_t i = 0; i < bs->arr.size(); ++i) {
            const JVal& b = bs->arr[i];
            std::vector<unsigned char> data;
            const JVal* uri = b.get("uri");
            if (!uri) {
                if (i != 0 || !has_glb_bin) return fail("buffer " + std::to_string(i) + " has no data");
                data = glb_bin;
            } else if (uri->str.compare(0, 5, "data:") == 0) {
                size_t comma = uri->str.find(',');
                if (comma == std::string::npos || uri->str.find(";base64") == std::string::npos ||
                    !base64(uri->str, comma + 1, data))
                    return fail("buffer " + std::to_string(i) + ": unsupported data URI");
            } else {
                if (!read_file(dir + uri->str, data)) return fail("cannot read buffer file " + uri->str);
            }
            const int64_t len = b.int_or("byteLength", -1);
            if (len < 0 || size_t(len) > data.size()) return fail("buffer " + std::to_string(i) + " is short");
            data.resize(size_t(len));
            buffers.push_back(std::move(data));
        }
        return true;
    }
    // element i, component c of an accessor, as double; false when out of range
    struct Acc {
        const unsigned char* base = nullptr;
        size_t stride = 0, count = 0, comps = 0, csize = 0;
        int ctype = 0;
        bool normalized = false;
        double get(size_t i, size_t c) const {
            const unsigned char* e = base + i * stride + c * csize;
            switch (ctype) {
                case 5120: { int8_t v; std::memcpy(&v, e, 1); return normalized ? std::max(v / 127.0, -1.0) : v; }
                case 5121: return normalized ? e[0] / 255.0 : e[0];
                case 5122: { int16_t v; std::memcpy(&v, e, 2); return normalized ? std::max(v / 32767.0, -1.0) : v; }
                case 5123: { uint16_t v; std::memcpy(&v, e, 2); return normalized ? v / 65535.0 : v; }
                case 5125: { uint32_t v; std::memcpy(&v, e, 4); return v; }
                default: { float v; std::memcpy(&v, e, 4); return v; }
            }
        }
    };
    bool accessor(int64_t idx, Acc& a) {
        const JVal* as = arr("accessors");
        if (!as || idx < 0 || size_t(idx) >= as->arr.size()) return fail("bad accessor index");
        const JVal& A = as->arr[size_t(idx)];
        if (A.get("sparse")) return fail("sparse accessors are not supported");
        const std::string type = A.get("type") ? A.get("type")->str : "";
        a.comps = type == "SCALAR" ? 1 : type == "VEC2" ? 2 : type == "VEC3" ? 3 : type == "VEC4" ? 4 : 0;
        a.ctype = int(A.int_or("componentType", 0));
        a.csize = (a.ctype == 5120 || a.ctype == 5121) ? 1 : (a.ctype == 5122 || a.ctype == 5123) ? 2 : 4;
        if (!a.comps || !(a.ctype == 5120 || a.ctype == 5121 || a.ctype == 5122 || a.ctype == 5123 ||
                          a.ctype == 5125 || a.ctype == 5126))
            return fail("unsupported accessor type");
        a.normalized = A.get("normalized") && A.get("normalized")->b;
        const int64_t cnt = A.int_or("count", -1);
        if (cnt < 0) return fail("accessor without a count");
        a.count = size_t(cnt);
        const int64_t bv = A.int_or("bufferView", -1);
        if (bv < 0) return fail("accessors without a buffer view are not supported");
        const JVal* bvs = arr("bufferViews");
        if (!bvs || size_t(bv) >= bvs->arr.size()) return fail("bad buffer view index");
        const JVal& V = bvs->arr[size_t(bv)];
        const int64_t buf = V.int_or("buffer", -1);
        if (buf < 0 || size_t(buf) >= buffers.size()) return fail("bad buffer index");
        const int64_t voff = V.int_or("byteOffset", 0), vlen = V.int_or("byteLength", -1);
        const int64_t aoff = A.int_or("byteOffset", 0);
        const size_t elem = a.comps * a.csize;
        const int64_t vstride = V.int_or("byteStride", 0);
        a.stride = vstride > 0 ? size_t(vstride) : elem;
        if (voff < 0 || vlen < 0 || aoff < 0 || size_t(voff + vlen) > buffers[size_t(buf)].size())
            return fail("buffer view out of range");
        if (a.count && size_t(aoff) + (a.count - 1) * a.stride + elem > size_t(vlen))
            return fail("accessor out of range");
        a.base = buffers[size_t(buf)].data() + voff + aoff;
        return true;
    }
    void material(int64_t idx, uint32_t& rgba, float& r) {
        rgba = 0xFFFFFFFFu;
        r = 1.0f;
        const JVal* ms = arr("materials");
        if (!ms || idx < 0 || size_t(idx) >= ms->arr.size()) return;
        const JVal* pbr = ms->arr[size_t(idx)].get("pbrMetallicRoughness");
        if (!pbr) return;
        if (const JVal* bc = pbr->get("baseColorFactor")) {
            rgba = 0;
            for (size_t c = 0; c < 4 && c < bc->arr.size(); ++c) {
                const double v = std::min(1.0, std::max(0.0, bc->arr[c].num));
                rgba |= uint32_t(std::lround(v * 255.0)) << (8 * c);
            }
        }
        r = float(pbr->num_or("roughnessFactor", 1.0));
    }
    bool primitive(const JVal& prim, const Mat4& M) {
        const int64_t mode = prim.int_or("mode", 4);
        if (mode < 4 || mode > 6) return true;  // points and lines carry no surface
        const JVal* attrs = prim.get("attributes");
        const JVal* pos = attrs ? attrs->get("POSITION") : nullptr;
        if (!pos) return true;
        Acc P;
        if (!accessor(int64_t(pos->num), P)) return false;
        if (P.comps != 3 || P.ctype != 5126) return fail("POSITION must be FP32 VEC3");
        std::vector<uint32_t> idx;
        const int64_t ii = prim.int_or("indices", -1);
        if (ii >= 0) {
            Acc I;
            if (!accessor(ii, I)) return false;
            if (I.comps != 1 || !(I.ctype == 5121 || I.ctype == 5123 || I.ctype == 5125))
                return fail("indices must be unsigned scalars");
            idx.resize(I.count);
            for (size_t k = 0; k < I.count; ++k) {
                idx[k] = uint32_t(I.get(k, 0));
                if (idx[k] >= P.count) return fail("index out of range");
            }
        } else {
            idx.resize(P.count);
            for (size_t k = 0; k < P.count; ++k) idx[k] = uint32_t(k);
        }
        std::vector<float> world(P.count * 3);
        for (size_t v = 0; v < P.count; ++v) {
            const double x = P.get(v, 0), y = P.get(v, 1), z = P.get(v, 2);
            for (int r = 0; r < 3; ++r)
                world[v * 3 + r] = float(M.m[r] * x + M.m[4 + r] * y + M.m[8 + r] * z + M.m[12 + r]);
        }
        uint32_t rgba;
        float rg;
        material(prim.int_or("material", -1), rgba, rg);
        const uint32_t f0 = uint32_t(albedo.size());
        auto emit = [&](uint32_t a, uint32_t b, uint32_t c) {
            for (uint32_t v : {a, b, c})
                for (int k = 0; k < 3; ++k) xyz.push_back(world[size_t(v) * 3 + k]);
            albedo.push_back(rgba);
            rough.push_back(rg);
        };
        const size_t n = idx.size();
        if (mode == 4) {
            for (size_t k = 0; k + 2 < n; k += 3) emit(idx[k], idx[k + 1], idx[k + 2]);
        } else if (mode == 5) {  // strip: every other triangle reversed to keep the winding
            for (size_t k = 0; k + 2 < n; ++k)
                if (k % 2 == 0) emit(idx[k], idx[k + 1], idx[k + 2]);
                else emit(idx[k + 1], idx[k], idx[k + 2]);
        } else {  // fan
            for (size_t k = 1; k + 1 < n; ++k) emit(idx[0], idx[k], idx[k + 1]);
        }
        const uint32_t cnt = uint32_t(albedo.size()) - f0;
        if (cnt) first.push_back(f0), count.push_back(cnt);
        return true;
    }
    bool visit(int64_t ni, const Mat4& parent, int depth) {
        const JVal* ns = arr("nodes");
        if (!ns || ni < 0 || size_t(ni) >= ns->arr.size()) return fail("bad node index");
        if (depth > 64) return fail("node tree too deep (or cyclic)");
        const JVal& n = ns->arr[size_t(ni)];
        const Mat4 M = parent * node_local(n);
        const int64_t mi = n.int_or("mesh", -1);
        if (mi >= 0) {
            const JVal* ms = arr("meshes");
            if (!ms || size_t(mi) >= ms->arr.size()) return fail("bad mesh index");
            const JVal* prims = ms->arr[size_t(mi)].get("primitives");
            if (prims)
                for (const JVal& p : prims->arr)
                    if (!primitive(p, M)) return false;
        }
        if (const JVal* ch = n.get("children"))
            for (const JVal& c : ch->arr)
                if (!visit(int64_t(c.num), M, depth + 1)) return false;
        return true;
    }
};

// the reference sun's direction of travel: its node is rotated by the Euler angles (-75, -30, 50) degrees --
// the product of the rotations about Y, X and Z, in that order, q = qY qX qZ -- and shines along its -Z
struct Quat {
    double w, x, y, z;
};
Quat qmul(const Quat& a, const Quat& b) {
    return Quat{a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z, a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
                a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x, a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w};
}
Quat axis_quat(int axis, double deg) {
    const double h = deg * M_PI / 360.0;
    Quat q{std::cos(h), 0.0, 0.0, 0.0};
    (axis == 0 ? q.x : axis == 1 ? q.y : q.z) = std::sin(h);
    return q;
}
void reference_sun(float dir[3]) {
    const Quat q = qmul(qmul(axis_quat(1, -30.0), axis_quat(0, -75.0)), axis_quat(2, 50.0));
    const Quat v{0.0, 0.0, 0.0, -1.0};
    const Quat r = qmul(qmul(q, v), Quat{q.w, -q.x, -q.y, -q.z});
    dir[0] = float(r.x), dir[1] = float(r.y), dir[2] = float(r.z);
}

}  // namespace
}  // namespace f184

using namespace f184;

extern "C" void f184gi_reference_sun_direction(float dir[3]) { reference_sun(dir); }

extern "C" int f184gi_gltf_load(const char* path, f184gi_scene** out) {
    if (!path || !out) return fail(F184GI_ERR_INVALID, "gltf_load: null argument");
    *out = nullptr;
    std::vector<unsigned char> file;
    if (!read_file(path, file)) return fail(F184GI_ERR_NOTFOUND, std::string("gltf_load: cannot read ") + path);
    Loader L;
    std::string sp(path);
    size_t slash = sp.find_last_of("/\\");
    L.dir = slash == std::string::npos ? std::string() : sp.substr(0, slash + 1);
    const char* json_begin = reinterpret_cast<const char*>(file.data());
    const char* json_end = json_begin + file.size();
    uint32_t magic = 0;
    if (file.size() >= 4) std::memcpy(&magic, file.data(), 4);
    if (magic == kGlbMagic) {  // header (magic, version, length), then chunks (length, type, data)
        uint32_t hdr[3];
        if (file.size() < 20) return fail(F184GI_ERR_INVALID, "gltf_load: truncated GLB header");
        std::memcpy(hdr, file.data(), 12);
        if (hdr[1] != 2 || hdr[2] > file.size()) return fail(F184GI_ERR_INVALID, "gltf_load: unsupported GLB header");
        json_begin = json_end = nullptr;
        size_t off = 12;
        while (off + 8 <= hdr[2]) {
            uint32_t ch[2];
            std::memcpy(ch, file.data() + off, 8);
            off += 8;
            if (off + ch[0] > hdr[2]) return fail(F184GI_ERR_INVALID, "gltf_load: truncated GLB chunk");
            if (ch[1] == kChunkJson && !json_begin) {
                json_begin = reinterpret_cast<const char*>(file.data() + off);
                json_end = json_begin + ch[0];
            } else if (ch[1] == kChunkBin && !L.has_glb_bin) {
                L.glb_bin.assign(file.data() + off, file.data() + off + ch[0]);
                L.has_glb_bin = true;
            }
            off += (ch[0] + 3) & ~size_t(3);
        }
        if (!json_begin) return fail(F184GI_ERR_INVALID, "gltf_load: GLB without a JSON chunk");
    }
    JParser jp{json_begin, json_end, {}};
    if (!jp.value(L.doc) || L.doc.kind != JVal::Obj)
        return fail(F184GI_ERR_INVALID, "gltf_load: JSON: " + (jp.err.empty() ? std::string("not an object") : jp.err));
    if (!L.load_buffers()) return fail(F184GI_ERR_INVALID, "gltf_load: " + L.err);
    const JVal* scenes = L.arr("scenes");
    const int64_t si = L.doc.int_or("scene", 0);
    if (scenes && si >= 0 && size_t(si) < scenes->arr.size()) {
        if (const JVal* roots = scenes->arr[size_t(si)].get("nodes"))
            for (const JVal& r : roots->arr)
                if (!L.visit(int64_t(r.num), Mat4::identity(), 0)) return fail(F184GI_ERR_INVALID, "gltf_load: " + L.err);
    }
    if (L.albedo.empty()) return fail(F184GI_ERR_INVALID, "gltf_load: the default scene has no triangles");
    f184gi_scene* s = static_cast<f184gi_scene*>(std::calloc(1, sizeof(f184gi_scene)));
    if (!s) return fail(F184GI_ERR_OOM, "gltf_load: host allocation failed");
    s->ntris = L.albedo.size();
    s->nobjects = uint32_t(L.first.size());
    s->tri_xyz = static_cast<float*>(std::malloc(L.xyz.size() * 4));
    s->albedo = static_cast<uint32_t*>(std::malloc(L.albedo.size() * 4));
    s->roughness = static_cast<float*>(std::malloc(L.rough.size() * 4));
    s->object_first = static_cast<uint32_t*>(std::malloc(L.first.size() * 4 + 4));
    s->object_count = static_cast<uint32_t*>(std::malloc(L.count.size() * 4 + 4));
    if (!s->tri_xyz || !s->albedo || !s->roughness || !s->object_first || !s->object_count) {
        f184gi_scene_free(s);
        return fail(F184GI_ERR_OOM, "gltf_load: host allocation failed");
    }
    std::memcpy(s->tri_xyz, L.xyz.data(), L.xyz.size() * 4);
    std::memcpy(s->albedo, L.albedo.data(), L.albedo.size() * 4);
    std::memcpy(s->roughness, L.rough.data(), L.rough.size() * 4);
    std::memcpy(s->object_first, L.first.data(), L.first.size() * 4);
    std::memcpy(s->object_count, L.count.data(), L.count.size() * 4);
    float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
    for (size_t k = 0; k < L.xyz.size(); ++k) mn[k % 3] = std::min(mn[k % 3], L.xyz[k]), mx[k % 3] = std::max(mx[k % 3], L.xyz[k]);
    s->bounds.min = {mn[0], mn[1], mn[2]};
    s->bounds.max = {mx[0], mx[1], mx[2]};
    s->light.luminance[0] = 1.1f * 4.0f;
    s->light.luminance[1] = 0.93f * 4.0f;
    s->light.luminance[2] = 0.81f * 4.0f;
    reference_sun(s->light.direction);
    float ext = 0.0f;
    for (int a = 0; a < 3; ++a) {
        s->target[a] = 0.5f * (mn[a] + mx[a]);
        ext = std::max(ext, mx[a] - mn[a]);
    }
    s->eye[0] = s->target[0];
    s->eye[1] = s->target[1] + 0.25f * ext;
    s->eye[2] = mx[2] + 0.75f * ext;
    *out = s;
    return F184GI_OK;
}
