/*
 * glsl_compat.h — the GLSL 4.60 subset the reference's GRIS shaders use, as C++20,
 * so that the reference's own shader sources (src/shader/*.glsl) compile with g++ and
 * run on the CPU as the pinning reference for the oracle.
 *
 * TEST INFRASTRUCTURE (oracle). Nothing outside tests/, smoke() and bench.py's
 * cpu_baseline leg may use it.
 *
 * Compiled with: -std=c++20 -fsingle-precision-constant (GLSL float literals are
 * binary32) -ffp-contract=off (no fused multiply-add, as on the CUDA side with
 * --fmad=false) -ftrivial-auto-var-init=zero (GLSL locals that the shaders read before
 * writing get the defined value 0).
 *
 * Everything lives in namespace glsl, so the shader code (included inside that namespace)
 * finds these functions before the C library's.
 *
 * Semantics this header fixes where GLSL leaves them to the implementation:
 *   - dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z; normalize(v) = v * (1 / sqrt(dot(v,v)));
 *     mat*vec sums columns left to right; mix(x,y,a) = x*(1-a) + y*a (the GLSL spec form).
 *   - max/min follow IEEE maxNum/minNum (a NaN operand yields the other operand).
 *   - sin/cos/tan/pow are the deterministic functions of oracle/detmath.h.
 *   - inverse(mat3) is the adjugate divided by the determinant.
 *   - texture(sampler2D, uv) is bilinear with REPEAT addressing and 8-bit sub-texel
 *     weights (the fixed-point weights hardware samplers use; this also makes a lookup
 *     at a texel centre return that texel exactly).
 *   - texelFetch and imageLoad outside the image and buffer reads past the end return zeros, writes
 *     past the end are dropped (Vulkan robust access).
 */
#ifndef GRIS_GLSL_COMPAT_H
#define GRIS_GLSL_COMPAT_H

#include <stdint.h>
#include <string.h>
#include "../detmath.h"

namespace glsl {

typedef unsigned int uint;

struct vec2; struct vec3; struct vec4; struct uvec2; struct ivec2; struct uvec4; struct ivec4;

static inline float glsl_sqrt(float x) { return __builtin_sqrtf(x); }

struct uvec2 {
    uint x, y;
    uvec2() = default;
    uvec2(uint a, uint b) : x(a), y(b) {}
    explicit uvec2(uint s) : x(s), y(s) {}
    explicit uvec2(const vec2& v);
    explicit uvec2(const ivec2& v);
    uvec2& xy() { return *this; }
    const uvec2& xy() const { return *this; }
};
struct ivec2 {
    int x, y;
    ivec2() = default;
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(int s) : x(s), y(s) {}
    explicit ivec2(const vec2& v);
    explicit ivec2(const uvec2& v) : x((int)v.x), y((int)v.y) {}
};
struct uvec4 {
    uint x, y, z, w;
    uvec4() = default;
    uvec4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
};

struct vec2 {
    float x, y;
    vec2() = default;
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    explicit vec2(const uvec2& v) : x((float)v.x), y((float)v.y) {}
    explicit vec2(const ivec2& v) : x((float)v.x), y((float)v.y) {}
    explicit vec2(const vec3& v);
    vec2& xy() { return *this; }
};
inline uvec2::uvec2(const vec2& v) : x((uint)v.x), y((uint)v.y) {}
inline ivec2::ivec2(const vec2& v) : x((int)v.x), y((int)v.y) {}
inline uvec2::uvec2(const ivec2& v) : x((uint)v.x), y((uint)v.y) {}

struct vec3 {
    float x, y, z;
    vec3() = default;
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    vec3(const vec2& v, float c) : x(v.x), y(v.y), z(c) {}
    explicit vec3(const vec4& v);
    vec2& xy() { return *reinterpret_cast<vec2*>(&x); }
    vec2& yz() { return *reinterpret_cast<vec2*>(&y); }
    const vec2& xy() const { return *reinterpret_cast<const vec2*>(&x); }
    const vec2& yz() const { return *reinterpret_cast<const vec2*>(&y); }
};
inline vec2::vec2(const vec3& v) : x(v.x), y(v.y) {}

struct vec4 {
    float x, y, z, w;
    vec4() = default;
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec4(const vec2& a, const vec2& b) : x(a.x), y(a.y), z(b.x), w(b.y) {}
    vec2& xy() { return *reinterpret_cast<vec2*>(&x); }
    vec2& zw() { return *reinterpret_cast<vec2*>(&z); }
    vec3& xyz() { return *reinterpret_cast<vec3*>(&x); }
    vec3& yzw() { return *reinterpret_cast<vec3*>(&y); }
    vec3& rgb() { return *reinterpret_cast<vec3*>(&x); }
    const vec2& xy() const { return *reinterpret_cast<const vec2*>(&x); }
    const vec2& zw() const { return *reinterpret_cast<const vec2*>(&z); }
    const vec3& xyz() const { return *reinterpret_cast<const vec3*>(&x); }
    const vec3& yzw() const { return *reinterpret_cast<const vec3*>(&y); }
    const vec3& rgb() const { return *reinterpret_cast<const vec3*>(&x); }
};
inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

/* ---- arithmetic: component-wise, each component one IEEE operation ---- */
#define GLSL_VEC2_OP(OP) \
    inline vec2 operator OP(const vec2& a, const vec2& b) { return vec2(a.x OP b.x, a.y OP b.y); } \
    inline vec2 operator OP(const vec2& a, float b) { return vec2(a.x OP b, a.y OP b); } \
    inline vec2 operator OP(float a, const vec2& b) { return vec2(a OP b.x, a OP b.y); } \
    inline vec2& operator OP##=(vec2& a, const vec2& b) { a = a OP b; return a; } \
    inline vec2& operator OP##=(vec2& a, float b) { a = a OP b; return a; }
#define GLSL_VEC3_OP(OP) \
    inline vec3 operator OP(const vec3& a, const vec3& b) { return vec3(a.x OP b.x, a.y OP b.y, a.z OP b.z); } \
    inline vec3 operator OP(const vec3& a, float b) { return vec3(a.x OP b, a.y OP b, a.z OP b); } \
    inline vec3 operator OP(float a, const vec3& b) { return vec3(a OP b.x, a OP b.y, a OP b.z); } \
    inline vec3& operator OP##=(vec3& a, const vec3& b) { a = a OP b; return a; } \
    inline vec3& operator OP##=(vec3& a, float b) { a = a OP b; return a; }
#define GLSL_VEC4_OP(OP) \
    inline vec4 operator OP(const vec4& a, const vec4& b) { return vec4(a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w); } \
    inline vec4 operator OP(const vec4& a, float b) { return vec4(a.x OP b, a.y OP b, a.z OP b, a.w OP b); } \
    inline vec4 operator OP(float a, const vec4& b) { return vec4(a OP b.x, a OP b.y, a OP b.z, a OP b.w); } \
    inline vec4& operator OP##=(vec4& a, const vec4& b) { a = a OP b; return a; } \
    inline vec4& operator OP##=(vec4& a, float b) { a = a OP b; return a; }
GLSL_VEC2_OP(+) GLSL_VEC2_OP(-) GLSL_VEC2_OP(*) GLSL_VEC2_OP(/)
GLSL_VEC3_OP(+) GLSL_VEC3_OP(-) GLSL_VEC3_OP(*) GLSL_VEC3_OP(/)
GLSL_VEC4_OP(+) GLSL_VEC4_OP(-) GLSL_VEC4_OP(*) GLSL_VEC4_OP(/)
inline ivec2 operator-(const ivec2& a, int b) { return ivec2(a.x - b, a.y - b); }
inline vec2 operator-(const vec2& a) { return vec2(-a.x, -a.y); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec4 operator-(const vec4& a) { return vec4(-a.x, -a.y, -a.z, -a.w); }

/* ---- matrices (column-major, as GLSL and the reference's host glm) ---- */
struct mat3 {
    vec3 c[3];
    mat3() = default;
    mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a; c[1] = b; c[2] = d; }
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};
struct mat4 {
    vec4 c[4];
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
inline vec3 operator*(const mat3& m, const vec3& v) { return ((m.c[0] * v.x + m.c[1] * v.y) + m.c[2] * v.z); }
inline vec4 operator*(const mat4& m, const vec4& v) { return (((m.c[0] * v.x + m.c[1] * v.y) + m.c[2] * v.z) + m.c[3] * v.w); }

/* ---- built-in functions ---- */
inline float abs(float x) { return __builtin_fabsf(x); }
inline vec3 abs(const vec3& v) { return vec3(abs(v.x), abs(v.y), abs(v.z)); }
inline float max(float a, float b) { return __builtin_fmaxf(a, b); }
inline float min(float a, float b) { return __builtin_fminf(a, b); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline vec3 clamp(const vec3& x, const vec3& lo, const vec3& hi) { return min(max(x, lo), hi); }
inline vec4 clamp(const vec4& x, float lo, float hi) { return vec4(clamp(x.x, lo, hi), clamp(x.y, lo, hi), clamp(x.z, lo, hi), clamp(x.w, lo, hi)); }
inline float sqrt(float x) { return glsl_sqrt(x); }
inline float floor(float x) { return __builtin_floorf(x); }
inline float sin(float x) { return oracle_det_sinf(x); }
inline float cos(float x) { return oracle_det_cosf(x); }
inline float tan(float x) { return oracle_det_tanf(x); }
/* asin / atan appear only in helpers the GRIS path never calls (angleBetween,
 * sphereToPlane); they are defined so the shader library compiles. */
inline float asin(float x) { return __builtin_asinf(x); }
inline float atan(float y, float x) { return __builtin_atan2f(y, x); }
inline float radians(float deg) { return deg * 0.01745329251994329577f; }
/* pow is implementation-defined in GLSL: here the deterministic oracle_det_powf of detmath.h */
inline float pow(float x, float y) { return oracle_det_powf(x, y); }
inline vec3 pow(const vec3& x, const vec3& y) { return vec3(pow(x.x, y.x), pow(x.y, y.y), pow(x.z, y.z)); }
inline bool isnan(float x) { return __builtin_isnan(x); }
inline bool isinf(float x) { return __builtin_isinf(x); }
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(const vec3& x, const vec3& y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(const vec3& x, const vec3& y, const vec3& a) { return x * (1.0f - a) + y * a; }
inline vec4 mix(const vec4& x, const vec4& y, float a) { return x * (1.0f - a) + y * a; }
inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(const vec2& v) { return sqrt(dot(v, v)); }
inline float length(const vec3& v) { return sqrt(dot(v, v)); }
inline float distance(const vec3& a, const vec3& b) { return length(a - b); }
inline vec3 normalize(const vec3& v) { return v * (1.0f / sqrt(dot(v, v))); }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline vec3 reflect(const vec3& i, const vec3& n) { return i - n * (2.0f * dot(n, i)); }
inline mat3 inverse(const mat3& m) {
    vec3 r0 = cross(m.c[1], m.c[2]);
    vec3 r1 = cross(m.c[2], m.c[0]);
    vec3 r2 = cross(m.c[0], m.c[1]);
    float invDet = 1.0f / dot(m.c[0], r0);
    /* rows of the inverse are r0, r1, r2 (scaled); store as columns */
    return mat3(vec3(r0.x * invDet, r1.x * invDet, r2.x * invDet),
                vec3(r0.y * invDet, r1.y * invDet, r2.y * invDet),
                vec3(r0.z * invDet, r1.z * invDet, r2.z * invDet));
}
inline uint floatBitsToUint(float f) { uint u; memcpy(&u, &f, 4); return u; }
inline float uintBitsToFloat(uint u) { float f; memcpy(&f, &u, 4); return f; }
inline uvec2 floatBitsToUint(const vec2& v) { return uvec2(floatBitsToUint(v.x), floatBitsToUint(v.y)); }
inline vec2 uintBitsToFloat(const uvec2& v) { return vec2(uintBitsToFloat(v.x), uintBitsToFloat(v.y)); }
inline uint packUnorm1(float c) { return (uint)floor(clamp(c, 0.0f, 1.0f) * 255.0f + 0.5f); }
inline uint packUnorm4x8(const vec4& v) {
    return packUnorm1(v.x) | (packUnorm1(v.y) << 8) | (packUnorm1(v.z) << 16) | (packUnorm1(v.w) << 24);
}
inline vec4 unpackUnorm4x8(uint p) {
    return vec4((float)(p & 0xffu) / 255.0f, (float)((p >> 8) & 0xffu) / 255.0f,
                (float)((p >> 16) & 0xffu) / 255.0f, (float)(p >> 24) / 255.0f);
}
/* packSnorm2x16 / unpackSnorm2x16 belong to helpers the GRIS path never calls. */
inline uint packSnorm2x16(const vec2& v) {
    int a = (int)floor(clamp(v.x, -1.0f, 1.0f) * 32767.0f + 0.5f);
    int b = (int)floor(clamp(v.y, -1.0f, 1.0f) * 32767.0f + 0.5f);
    return ((uint)a & 0xffffu) | (((uint)b & 0xffffu) << 16);
}
inline vec2 unpackSnorm2x16(uint p) {
    float a = (float)(int16_t)(p & 0xffffu) / 32767.0f, b = (float)(int16_t)(p >> 16) / 32767.0f;
    return vec2(clamp(a, -1.0f, 1.0f), clamp(b, -1.0f, 1.0f));
}
#define nonuniformEXT(x) (x)

/* ---- storage buffers with robust (zero) out-of-range access ---- */
template <typename T> struct GBuf {
    T* data = nullptr;
    uint64_t n = 0;
    T& operator[](uint64_t i) {
        if (i < n) return data[i];
        static thread_local T dummy;
        memset((void*)&dummy, 0, sizeof(T));
        return dummy;
    }
};

/* ---- images and samplers ---- */
struct sampler2D {             /* float texels, `ch` channels each (4: RGBA32F, 2: RG16F decoded) */
    const float* data = nullptr;
    int w = 0, h = 0, ch = 4;
};
struct usampler2D {            /* RG32UI */
    const uint* data = nullptr;
    int w = 0, h = 0;
};
struct image2D { float* data = nullptr; int w = 0, h = 0; };   /* RGBA32F */
struct accelerationStructureEXT { int unused = 0; };

inline vec4 glsl_texel(const sampler2D& s, int x, int y) {
    if (x < 0 || y < 0 || x >= s.w || y >= s.h || !s.data) return vec4(0.0f);
    const float* p = s.data + ((size_t)y * s.w + x) * s.ch;
    return s.ch == 4 ? vec4(p[0], p[1], p[2], p[3]) : vec4(p[0], p[1], 0.0f, 1.0f);
}
inline vec4 texelFetch(const sampler2D& s, const ivec2& p, int) { return glsl_texel(s, p.x, p.y); }
inline uvec4 texelFetch(const usampler2D& s, const ivec2& p, int) {
    if (p.x < 0 || p.y < 0 || p.x >= s.w || p.y >= s.h || !s.data) return uvec4(0, 0, 0, 0);
    const uint* q = s.data + ((size_t)p.y * s.w + p.x) * 2;
    return uvec4(q[0], q[1], 0, 1);
}
inline ivec2 textureSize(const sampler2D& s, int) { return ivec2(s.w, s.h); }
inline vec4 imageLoad(const image2D& im, const ivec2& p) {
    if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h || !im.data) return vec4(0.0f);
    const float* q = im.data + ((size_t)p.y * im.w + p.x) * 4;
    return vec4(q[0], q[1], q[2], q[3]);
}
inline int glsl_wrap(int i, int n) { int r = i % n; return r < 0 ? r + n : r; }
inline vec4 texture(const sampler2D& s, const vec2& uv) {
    float x = uv.x * (float)s.w - 0.5f;
    float y = uv.y * (float)s.h - 0.5f;
    float x0 = floor(x), y0 = floor(y);
    float qx = floor((x - x0) * 256.0f + 0.5f);
    float qy = floor((y - y0) * 256.0f + 0.5f);
    int ix = (int)x0, iy = (int)y0;
    if (qx >= 256.0f) { ix += 1; qx = 0.0f; }
    if (qy >= 256.0f) { iy += 1; qy = 0.0f; }
    float wx = qx * 0.00390625f, wy = qy * 0.00390625f;
    int i0 = glsl_wrap(ix, s.w), i1 = glsl_wrap(ix + 1, s.w);
    int j0 = glsl_wrap(iy, s.h), j1 = glsl_wrap(iy + 1, s.h);
    vec4 top = mix(glsl_texel(s, i0, j0), glsl_texel(s, i1, j0), wx);
    vec4 bot = mix(glsl_texel(s, i0, j1), glsl_texel(s, i1, j1), wx);
    return mix(top, bot, wy);
}

/* Ray flags used by the shaders (values of GL_EXT_ray_tracing). */
const uint gl_RayFlagsNoneEXT = 0u;
const uint gl_RayFlagsOpaqueEXT = 1u;
const uint gl_RayFlagsTerminateOnFirstHitEXT = 4u;
const uint gl_RayFlagsSkipClosestHitShaderEXT = 8u;

}  /* namespace glsl */

#endif
