// glsl_frag_shim.hpp — just enough of GLSL 4.10 for the reference's water
// fragment shader source (assets/shaders/water-grid.frag) to compile as C++.
// Test infrastructure only: used by oracle/build.py to build oracle/_ref from
// the shader where it lies.
//
// Built-ins follow the GLSL 4.10 definitions: mix = x*(1-a) + y*a,
// clamp = min(max(x, lo), hi), length = sqrt(dot(v, v)),
// reflect(I, N) = I - 2*dot(N, I)*N, pow = the C library's powf.  Samplers
// follow the reference's sampler state (src/render-engine.cpp:86-206):
// CLAMP_TO_EDGE everywhere, GL_NEAREST for the depth texture, GL_LINEAR for
// the RGBA8 colour textures and the cube map (face chosen by the major axis of
// the direction, OpenGL 4.1 table 3.19, no seamless filtering).  These are the
// same definitions oracle/water.c uses, in the same operation order, so both
// compile (with -ffp-contract=off) to the same results.
#pragma once
#include <stdint.h>

// The C library's float functions, declared here rather than through
// <math.h>: in C++ that header also brings the std::pow overloads, which
// would compute pow(float, int) in double instead of GLSL's float pow.
extern "C" {
float sqrtf(float);
float powf(float, float);
float floorf(float);
float fabsf(float);
float fminf(float, float);
float fmaxf(float, float);
}

#include "wt_oracle.h"

typedef unsigned int uint;

struct vec2;
struct vec3;

template <int A, int B>
struct fswz2 {
    float e[4];
    operator vec2() const;
};
template <int A, int B, int C>
struct fswz3 {
    float e[4];
    operator vec3() const;
    fswz3& operator=(const vec3& v);
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
};

struct vec4 {
    union {
        float e[4];
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        fswz2<0, 1> xy;
        fswz3<0, 1, 2> rgb;
    };
    vec4() { x = 0.0f; y = 0.0f; z = 0.0f; w = 0.0f; }
    vec4(float p, float q, float u, float v) { x = p; y = q; z = u; w = v; }
    vec4(const vec3& c, float d) { x = c.x; y = c.y; z = c.z; w = d; }
    vec4(const vec4& o) { x = o.x; y = o.y; z = o.z; w = o.w; }
    vec4& operator=(const vec4& o) { x = o.x; y = o.y; z = o.z; w = o.w; return *this; }
};

template <int A, int B>
fswz2<A, B>::operator vec2() const { return vec2(e[A], e[B]); }
template <int A, int B, int C>
fswz3<A, B, C>::operator vec3() const { return vec3(e[A], e[B], e[C]); }
template <int A, int B, int C>
fswz3<A, B, C>& fswz3<A, B, C>::operator=(const vec3& v) {
    e[A] = v.x;
    e[B] = v.y;
    e[C] = v.z;
    return *this;
}

inline vec2 operator+(const vec2& a, const vec2& b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator/(const vec2& a, const vec2& b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator/(const vec2& v, float s) { return vec2(v.x / s, v.y / s); }
inline vec2 operator*(float s, const vec2& v) { return vec2(s * v.x, s * v.y); }
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(float s, const vec3& v) { return vec3(s * v.x, s * v.y, s * v.z); }
inline vec3 operator*(const vec3& v, float s) { return vec3(v.x * s, v.y * s, v.z * s); }
inline vec3 operator/(const vec3& v, float s) { return vec3(v.x / s, v.y / s, v.z / s); }

inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(const vec3& v) { return sqrtf(dot(v, v)); }
inline vec3 reflect(const vec3& I, const vec3& N) { return I - (2.0f * dot(N, I)) * N; }
inline float clamp(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
inline vec2 clamp(const vec2& v, const vec2& lo, const vec2& hi) {
    return vec2(clamp(v.x, lo.x, hi.x), clamp(v.y, lo.y, hi.y));
}
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline vec2 mix(const vec2& x, const vec2& y, float a) { return vec2(mix(x.x, y.x, a), mix(x.y, y.y, a)); }
inline vec3 mix(const vec3& x, const vec3& y, float a) {
    return vec3(mix(x.x, y.x, a), mix(x.y, y.y, a), mix(x.z, y.z, a));
}
inline float pow(float x, float y) { return powf(x, y); }
inline float pow(float x, int y) { return powf(x, (float)y); }

// 2D textures: depth (float, GL_NEAREST) or RGBA8 (GL_LINEAR); clamp to edge.
struct sampler2D {
    const float* depth;
    const uint8_t* rgba8;
    uint32_t width, height;
};

inline uint32_t wtfs_clampi(int64_t i, uint32_t n) { return (uint32_t)(i < 0 ? 0 : (i >= (int64_t)n ? n - 1 : i)); }

inline vec4 wtfs_bilinear_rgba8(const uint8_t* px, uint32_t w, uint32_t h, float s, float t) {
    float u = s * (float)w - 0.5f;
    float v = t * (float)h - 0.5f;
    float fi = floorf(u), fj = floorf(v);
    float a = u - fi, b = v - fj;
    uint32_t i0 = wtfs_clampi((int64_t)fi, w), i1 = wtfs_clampi((int64_t)fi + 1, w);
    uint32_t j0 = wtfs_clampi((int64_t)fj, h), j1 = wtfs_clampi((int64_t)fj + 1, h);
    vec4 o;
    for (int c = 0; c < 4; ++c) {
        float t00 = (float)px[4 * ((size_t)j0 * w + i0) + c] / 255.0f;
        float t10 = (float)px[4 * ((size_t)j0 * w + i1) + c] / 255.0f;
        float t01 = (float)px[4 * ((size_t)j1 * w + i0) + c] / 255.0f;
        float t11 = (float)px[4 * ((size_t)j1 * w + i1) + c] / 255.0f;
        o.e[c] = (1.0f - b) * ((1.0f - a) * t00 + a * t10) + b * ((1.0f - a) * t01 + a * t11);
    }
    return o;
}

inline vec4 texture(const sampler2D& smp, const vec2& st) {
    if (smp.depth) {
        uint32_t i = wtfs_clampi((int64_t)floorf(st.x * (float)smp.width), smp.width);
        uint32_t j = wtfs_clampi((int64_t)floorf(st.y * (float)smp.height), smp.height);
        float d = smp.depth[(size_t)j * smp.width + i];
        return vec4(d, d, d, 1.0f);
    }
    if (!smp.rgba8) return vec4(0.0f, 0.0f, 0.0f, 0.0f);
    return wtfs_bilinear_rgba8(smp.rgba8, smp.width, smp.height, st.x, st.y);
}

// Cube map: six RGBA8 faces (+X, -X, +Y, -Y, +Z, -Z) of size x size.
struct samplerCube {
    const uint8_t* faces;
    uint32_t size;
};

inline vec4 texture(const samplerCube& smp, const vec3& r) {
    float ax = fabsf(r.x), ay = fabsf(r.y), az = fabsf(r.z);
    int face;
    float sc, tc, ma;
    if (ax >= ay && ax >= az) {
        face = r.x >= 0.0f ? 0 : 1;
        sc = r.x >= 0.0f ? -r.z : r.z;
        tc = -r.y;
        ma = ax;
    } else if (ay >= az) {
        face = r.y >= 0.0f ? 2 : 3;
        sc = r.x;
        tc = r.y >= 0.0f ? r.z : -r.z;
        ma = ay;
    } else {
        face = r.z >= 0.0f ? 4 : 5;
        sc = r.z >= 0.0f ? r.x : -r.x;
        tc = -r.y;
        ma = az;
    }
    float s = (sc / ma + 1.0f) / 2.0f;
    float t = (tc / ma + 1.0f) / 2.0f;
    return wtfs_bilinear_rgba8(smp.faces + (size_t)face * smp.size * smp.size * 4, smp.size, smp.size, s, t);
}

// fragment-stage built-in
static vec4 gl_FragCoord;

// storage qualifiers and the entry point
#define uniform
#define in
#define out
#define main wt_glsl_fragment_main
