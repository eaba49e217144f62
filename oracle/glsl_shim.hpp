// glsl_shim.hpp — just enough of GLSL 4.10 for the reference's vertex shader
// source to compile as C++.  Test infrastructure only: used by
// oracle/build_ref.py to build oracle/_ref from the shader where it lies.
//
// Built-ins follow the GLSL 4.10 definitions (mix = x*(1-a) + y*a,
// mod = x - y*floor(x/y), normalize = v/length(v), cross as in the spec,
// sin/cos = the C library's float functions) and texture() does GL_LINEAR on
// the base level with GL_REPEAT / GL_MIRRORED_REPEAT texel wrap.  These are
// the same definitions oracle/reference_mode.c uses, in the same operation
// order, so both compile (with -ffp-contract=off) to the same results.
#pragma once
#include <math.h>
#include <stdint.h>

typedef unsigned int uint;

struct vec2;
struct vec3;
struct vec4;

template <int A, int B>
struct swz2 {
    float e[4];
    operator vec2() const;
};
template <int A, int B, int C>
struct swz3 {
    float e[4];
    operator vec3() const;
};

struct vec2 {
    union {
        struct { float x, y; };
        struct { float s, t; };
    };
    vec2() { x = 0.0f; y = 0.0f; }
    vec2(float a, float b) { x = a; y = b; }
};

struct vec3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
    };
    vec3() { x = 0.0f; y = 0.0f; z = 0.0f; }
    vec3(float a, float b, float c) { x = a; y = b; z = c; }
    vec3& operator+=(const vec3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    vec3& operator*=(float s) { x = x * s; y = y * s; z = z * s; return *this; }
};

struct vec4 {
    union {
        float e[4];
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        struct { float s, t, p, q; };
        swz2<0, 2> xz;
        swz2<0, 1> xy;
        swz3<0, 1, 2> xyz;
    };
    vec4() { x = 0.0f; y = 0.0f; z = 0.0f; w = 0.0f; }
    vec4(float a, float b, float c, float d) { x = a; y = b; z = c; w = d; }
    vec4(const vec3& v, float d) { x = v.x; y = v.y; z = v.z; w = d; }
};

template <int A, int B>
swz2<A, B>::operator vec2() const { return vec2(e[A], e[B]); }
template <int A, int B, int C>
swz3<A, B, C>::operator vec3() const { return vec3(e[A], e[B], e[C]); }

// column-major 4x4, m[c][r]
struct mat4 {
    float m[4][4];
};

inline vec2 operator+(const vec2& a, const vec2& b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(const vec2& a, const vec2& b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator*(float s, const vec2& v) { return vec2(s * v.x, s * v.y); }
inline vec2 operator/(const vec2& v, float s) { return vec2(v.x / s, v.y / s); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(float s, const vec3& v) { return vec3(s * v.x, s * v.y, s * v.z); }
inline vec4 operator-(const vec4& a, const vec4& b) { return vec4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline vec4 operator*(const mat4& M, const vec4& v) {
    return vec4(M.m[0][0] * v.x + M.m[1][0] * v.y + M.m[2][0] * v.z + M.m[3][0] * v.w,
                M.m[0][1] * v.x + M.m[1][1] * v.y + M.m[2][1] * v.z + M.m[3][1] * v.w,
                M.m[0][2] * v.x + M.m[1][2] * v.y + M.m[2][2] * v.z + M.m[3][2] * v.w,
                M.m[0][3] * v.x + M.m[1][3] * v.y + M.m[2][3] * v.z + M.m[3][3] * v.w);
}

inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline vec4 mix(const vec4& x, const vec4& y, float a) {
    return vec4(mix(x.x, y.x, a), mix(x.y, y.y, a), mix(x.z, y.z, a), mix(x.w, y.w, a));
}
inline float mod(float x, float y) { return x - y * floorf(x / y); }
inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline vec3 normalize(const vec3& v) {
    float l = sqrtf(dot(v, v));
    return vec3(v.x / l, v.y / l, v.z / l);
}

// sampler2D over an R channel in [0, 1]; texture() returns (r, r, r, 1) like
// the RGBA expansion of a grey image.
struct sampler2D {
    const float* texels;
    uint32_t width, height;
    uint32_t wrap;  // 0 repeat, 1 mirrored repeat
};

inline int64_t glsl_shim_wrap(int64_t i, int64_t n, uint32_t mode) {
    if (mode == 1) {
        int64_t m = i % (2 * n);
        if (m < 0) m += 2 * n;
        int64_t a = m - n;
        return n - 1 - (a >= 0 ? a : -(1 + a));
    }
    int64_t m = i % n;
    return m < 0 ? m + n : m;
}

inline vec4 texture(const sampler2D& smp, const vec2& st) {
    if (!smp.texels) return vec4(0.0f, 0.0f, 0.0f, 0.0f);
    float u = st.x * (float)smp.width - 0.5f;
    float v = st.y * (float)smp.height - 0.5f;
    float fi = floorf(u), fj = floorf(v);
    float a = u - fi, b = v - fj;
    int64_t i0 = (int64_t)fi, j0 = (int64_t)fj;
    int64_t ia = glsl_shim_wrap(i0, smp.width, smp.wrap), ib = glsl_shim_wrap(i0 + 1, smp.width, smp.wrap);
    int64_t ja = glsl_shim_wrap(j0, smp.height, smp.wrap), jb = glsl_shim_wrap(j0 + 1, smp.height, smp.wrap);
    float t00 = smp.texels[ja * smp.width + ia], t10 = smp.texels[ja * smp.width + ib];
    float t01 = smp.texels[jb * smp.width + ia], t11 = smp.texels[jb * smp.width + ib];
    float g = (1.0f - b) * ((1.0f - a) * t00 + a * t10) + b * ((1.0f - a) * t01 + a * t11);
    return vec4(g, g, g, 1.0f);
}

// vertex-stage built-ins
static int gl_VertexID;
static vec4 gl_Position;

// storage qualifiers and the entry point
#define uniform
#define in
#define out
#define main wt_glsl_vertex_main
