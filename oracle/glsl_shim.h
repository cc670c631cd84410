// glsl_shim.h -- just enough GLSL 4.50 vocabulary for C++ to compile the reference's shader functions verbatim.
// TEST INFRASTRUCTURE ONLY (the reference pin built by oracle/glsl_pin.py).
//
// Types, constructors, swizzles (read and assign), component-wise operators and the built-ins the extracted
// functions use, with GLSL's single-precision semantics: every operation is one FP32 operation rounded on its
// own (the pin is compiled with -ffp-contract=off; float literals get GLSL's single-precision meaning from the
// extraction script).  Where GLSL leaves the evaluation open, the shim fixes it:
//   - mat * vec sums the columns in order, ((c0 x + c1 y) + c2 z) + c3 w, per component;
//   - normalize(v) = v / length(v), length(v) = sqrt(dot(v, v)), dot sums left to right;
//   - pow, sin, cos, sqrt are the C library's float functions.
// Texture and image reads go through handles the harness fills.  Anonymous structs inside unions (the swizzle
// overlays) are a GNU extension that g++ accepts.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>

namespace glsl {

typedef unsigned int uint;

struct vec2;
struct vec3;

// Swizzle proxies: a view of the N floats of a vector that reads as (and assigns from) the picked components.
template <int N, int A, int B>
struct Sw2 {
    float d[N];
    operator vec2() const;
    Sw2& operator=(const vec2& v);
};
template <int N, int A, int B, int C>
struct Sw3 {
    float d[N];
    operator vec3() const;
    Sw3& operator=(const vec3& v);
};

struct vec2 {
    union {
        struct { float x, y; };
        struct { float r, g; };
        struct { float s, t; };
    };
    vec2() : x(0.f), y(0.f) {}
    explicit vec2(float v) : x(v), y(v) {}
    vec2(float a, float b) : x(a), y(b) {}
};

struct vec3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
        Sw2<3, 0, 1> xy;
        Sw2<3, 0, 1> rg;
        Sw3<3, 0, 1, 2> xyz;
        Sw3<3, 0, 1, 2> rgb;
    };
    vec3() : x(0.f), y(0.f), z(0.f) {}
    explicit vec3(float v) : x(v), y(v), z(v) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const vec2& v, float c) : x(v.x), y(v.y), z(c) {}
    vec3(const vec3& v) : x(v.x), y(v.y), z(v.z) {}
    vec3& operator=(const vec3& v) {
        x = v.x, y = v.y, z = v.z;
        return *this;
    }
};

struct vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        Sw2<4, 0, 1> xy;
        Sw2<4, 0, 1> st;
        Sw2<4, 0, 1> rg;
        Sw3<4, 0, 1, 2> xyz;
        Sw3<4, 0, 1, 2> rgb;
    };
    vec4() : x(0.f), y(0.f), z(0.f), w(0.f) {}
    explicit vec4(float v) : x(v), y(v), z(v), w(v) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec4(const vec4& v) : x(v.x), y(v.y), z(v.z), w(v.w) {}
    vec4& operator=(const vec4& v) {
        x = v.x, y = v.y, z = v.z, w = v.w;
        return *this;
    }
};

template <int N, int A, int B>
Sw2<N, A, B>::operator vec2() const { return vec2(d[A], d[B]); }
template <int N, int A, int B>
Sw2<N, A, B>& Sw2<N, A, B>::operator=(const vec2& v) {
    d[A] = v.x, d[B] = v.y;
    return *this;
}
template <int N, int A, int B, int C>
Sw3<N, A, B, C>::operator vec3() const { return vec3(d[A], d[B], d[C]); }
template <int N, int A, int B, int C>
Sw3<N, A, B, C>& Sw3<N, A, B, C>::operator=(const vec3& v) {
    d[A] = v.x, d[B] = v.y, d[C] = v.z;
    return *this;
}

struct ivec2 {
    int x, y;
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const vec2& v) : x(int(v.x)), y(int(v.y)) {}
};
struct ivec3 {
    int x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit ivec3(const vec3& v) : x(int(v.x)), y(int(v.y)), z(int(v.z)) {}
};
inline bool operator!=(const ivec3& a, const ivec3& b) { return a.x != b.x || a.y != b.y || a.z != b.z; }
inline bool operator==(const ivec3& a, const ivec3& b) { return !(a != b); }

struct uvec2 {
    union {
        struct { uint x, y; };
        struct { uint r, g; };
    };
    uvec2() : x(0u), y(0u) {}
    uvec2(uint a, uint b) : x(a), y(b) {}
};
struct SwU2 {
    uint d[4];
    operator uvec2() const { return uvec2(d[0], d[1]); }
};
struct uvec4 {
    union {
        struct { uint x, y, z, w; };
        struct { uint r, g, b, a; };
        SwU2 rg;
    };
    uvec4() : x(0u), y(0u), z(0u), w(0u) {}
    uvec4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
};

// ---- component-wise arithmetic ----
inline vec2 operator+(const vec2& a, const vec2& b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator+(const vec2& a, float s) { return vec2(a.x + s, a.y + s); }
inline vec2 operator*(const vec2& a, const vec2& b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator*(const vec2& a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator-(const vec2& a) { return vec2(-a.x, -a.y); }

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3& operator+=(vec3& a, const vec3& b) { return a = a + b; }
inline vec3& operator*=(vec3& a, float s) { return a = a * s; }
inline vec4& operator/=(vec4& a, float s) {
    a.x = a.x / s, a.y = a.y / s, a.z = a.z / s, a.w = a.w / s;
    return a;
}

struct mat3 {  // column-major, as GLSL: c[i] is column i
    vec3 c[3];
    mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a, c[1] = b, c[2] = d; }
};
inline vec3 operator*(const mat3& m, const vec3& v) {
    return vec3((m.c[0].x * v.x + m.c[1].x * v.y) + m.c[2].x * v.z, (m.c[0].y * v.x + m.c[1].y * v.y) + m.c[2].y * v.z,
                (m.c[0].z * v.x + m.c[1].z * v.y) + m.c[2].z * v.z);
}

struct mat4 {  // column-major: m[col][row]; default identity
    float m[4][4];
    mat4() {
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) m[i][j] = i == j ? 1.f : 0.f;
    }
};
inline vec4 operator*(const mat4& M, const vec4& v) {
    float o[4];
    for (int r = 0; r < 4; ++r) o[r] = ((M.m[0][r] * v.x + M.m[1][r] * v.y) + M.m[2][r] * v.z) + M.m[3][r] * v.w;
    return vec4(o[0], o[1], o[2], o[3]);
}
inline mat4 operator*(const mat4& A, const mat4& B) {
    mat4 C;
    for (int col = 0; col < 4; ++col) {
        const vec4 o = A * vec4(B.m[col][0], B.m[col][1], B.m[col][2], B.m[col][3]);
        C.m[col][0] = o.x, C.m[col][1] = o.y, C.m[col][2] = o.z, C.m[col][3] = o.w;
    }
    return C;
}

// ---- built-ins ----
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(const vec3& v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(const vec3& v) { return v / length(v); }
inline vec3 abs(const vec3& v) { return vec3(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }
inline float abs(float v) { return std::fabs(v); }
inline float sqrt(float v) { return std::sqrt(v); }
inline float cos(float v) { return std::cos(v); }
inline float sin(float v) { return std::sin(v); }
inline vec3 pow(const vec3& a, const vec3& e) { return vec3(std::pow(a.x, e.x), std::pow(a.y, e.y), std::pow(a.z, e.z)); }
inline float max(float a, float b) { return a > b ? a : b; }
inline float min(float a, float b) { return a < b ? a : b; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float step(float edge, float x) { return x < edge ? 0.0f : 1.0f; }
inline float smoothstep(float e0, float e1, float x) {
    const float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// ---- resources: the harness points these at its volume and shadow map ----
struct texture2D {
    const float* texels = nullptr;  // R32F, row-major
    int width = 0, height = 0;
};
struct sampler {};
struct sampler2D {
    const texture2D* t;
    sampler2D(const texture2D& tex, const sampler&) : t(&tex) {}
};
inline vec4 texelFetch(const sampler2D& s, const ivec2& p, int) {  // out of range reads zero (robust access)
    if (p.x < 0 || p.y < 0 || p.x >= s.t->width || p.y >= s.t->height) return vec4(0.f);
    return vec4(s.t->texels[size_t(p.y) * size_t(s.t->width) + size_t(p.x)], 0.f, 0.f, 1.f);
}
struct uimage3D {
    const uint32_t* texels = nullptr;  // RG16UI packed as r | g << 16, x fastest
    int size = 0;
};
inline uvec4 imageLoad(const uimage3D& im, const ivec3& p) {
    if (p.x < 0 || p.y < 0 || p.z < 0 || p.x >= im.size || p.y >= im.size || p.z >= im.size) return uvec4(0, 0, 0, 0);
    const uint32_t v = im.texels[(size_t(p.z) * size_t(im.size) + size_t(p.y)) * size_t(im.size) + size_t(p.x)];
    return uvec4(v & 0xffffu, v >> 16, 0u, 1u);
}

}  // namespace glsl
