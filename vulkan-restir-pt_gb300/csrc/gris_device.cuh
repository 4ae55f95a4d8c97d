/*
 * gris_device.cuh — device-side restatement of the reference's GRIS shading library.
 *
 * Every function states the reference function it implements (file:line, under src/shader/).
 * Floating-point expressions keep the reference's evaluation order operation by operation
 * (this translation unit is compiled with --fmad=false and IEEE division/sqrt), built-ins
 * follow the project definitions (dot = (x*x' + y*y') + z*z', normalize = v * (1/|v|),
 * mix(x,y,a) = x*(1-a) + y*a, max/min = IEEE maxNum/minNum, sin/cos/tan from detmath.h,
 * inverse(mat3) = adjugate / determinant), and GLSL locals that the shaders read before
 * writing start at zero. Buffer reads past the end return zeros (robust access).
 */
#ifndef GRISRT_GRIS_DEVICE_CUH
#define GRISRT_GRIS_DEVICE_CUH

#include <stdint.h>

#include "../../include/grisrt.h"
#include "bvh_traverse.h"
#include "detmath.h"

namespace grisrt {

#define GD __device__ __forceinline__

/* ---------------------------------------------------------------- constants (math.glsl:4-5,
 * ray_layouts.glsl:9-13, gris_reservoir.glsl:8-19, material.glsl:6-20, camera.glsl:6-7) */
constexpr float kPi = 0x1.921fb6p+1f;
constexpr float kPiInv = 0x1.45f306p-2f;   /* 1.0f / kPi, correctly rounded */
constexpr float kMinRayDistance = 1e-4f;
constexpr float kMaxRayDistance = 1e7f;
constexpr uint32_t kInvalidHit = 0xffffffffu;
constexpr uint32_t kSpecialHit = 0xfffffffeu;
constexpr float kDistanceThreshold = 0.01f;
constexpr uint32_t kShiftReconnection = 0u;
constexpr uint32_t kRcLightSampled = 0u, kRcLightScattered = 1u, kRcSurface = 2u;
constexpr uint32_t kDiffuse = 1u << 0, kGlossy = 1u << 1, kSpecular = 1u << 2, kReflection = 1u << 4,
                   kTransmission = 1u << 5, kInvalidBSDFSample = 0x80000000u;
constexpr uint32_t kLambert = 1u, kMetallicWorkflow = 2u, kMetal = 3u, kDielectric = 4u, kFake = 6u;
constexpr uint32_t kCameraClearFlag = 0x80000000u;
constexpr uint32_t kCameraFrameIndexMask = 0x7fffffffu;

/* ---------------------------------------------------------------- vectors */
struct V2 { float x, y; };
struct V3 { float x, y, z; };
GD V2 v2(float x, float y) { V2 r; r.x = x; r.y = y; return r; }
GD V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
GD V3 v3s(float s) { return v3(s, s, s); }
GD V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
GD V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
GD V3 operator*(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
GD V3 operator/(V3 a, V3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
GD V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
GD V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
GD V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
GD V3 operator+(V3 a, float s) { return v3(a.x + s, a.y + s, a.z + s); }
GD V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
GD float dot3(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
GD float dot2(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
GD V3 cross3(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
GD float length3(V3 v) { return sqrtf(dot3(v, v)); }
GD float distance3(V3 a, V3 b) { return length3(a - b); }
GD V3 normalize3(V3 v) { return v * (1.0f / sqrtf(dot3(v, v))); }
GD float absDot(V3 a, V3 b) { return fabsf(dot3(a, b)); }
GD float satDot(V3 a, V3 b) { return fmaxf(dot3(a, b), 0.0f); }
GD float square(float x) { return x * x; }
GD V3 mix3(V3 x, V3 y, float a) { return x * (1.0f - a) + y * a; }
GD V3 mix3v(V3 x, V3 y, V3 a) { return x * (v3s(1.0f) - a) + y * a; }
GD float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
GD V3 reflect3(V3 i, V3 n) { return i - n * (2.0f * dot3(n, i)); }
GD bool isnan3(V3 c) { return isnan(c.x) || isnan(c.y) || isnan(c.z); }

/* ---------------------------------------------------------------- data records */
struct Isec { float bx, by; uint32_t inst, tri; };                    /* layouts.glsl:90-94 */
struct Surf { V3 pos, norm, albedo; uint32_t matIndex; bool isLight; };  /* ray_layouts.glsl:20-26 */
struct Mat { V3 baseColor; uint32_t type, textureIdx; float metallic, roughness, ior; };
struct PathSample {                                                     /* layouts.glsl:132-147 */
    Isec rcIsec;
    V3 rcLi; uint32_t rcRng;
    V3 rcWi; uint32_t flags;
    float pad0, pad1, rcPrevSamplePdf, rcJacobian;
    V3 F; uint32_t primaryRng;
};
struct Resv { PathSample s; float sampleCount, resampleWeight, contribWeight, pad0; };  /* :149-156 */
struct BsdfSample { V3 wi; float pdf; V3 bsdf; uint32_t type; };        /* material.glsl:24-29 */
struct RcData { Isec rcPrevIsec; V3 rcPrevWo; V3 rcPrevThroughput; };   /* layouts.glsl:158-164 */
struct Ray3 { V3 ori, dir; };

GD Isec isec_zero() { Isec r; r.bx = 0.0f; r.by = 0.0f; r.inst = 0u; r.tri = 0u; return r; }
GD Surf surf_zero() { Surf s; s.pos = v3s(0.0f); s.norm = v3s(0.0f); s.albedo = v3s(0.0f); s.matIndex = 0u; s.isLight = false; return s; }
GD PathSample ps_zero() {
    PathSample p;
    p.rcIsec = isec_zero(); p.rcLi = v3s(0.0f); p.rcRng = 0u; p.rcWi = v3s(0.0f); p.flags = 0u;
    p.pad0 = 0.0f; p.pad1 = 0.0f; p.rcPrevSamplePdf = 0.0f; p.rcJacobian = 0.0f; p.F = v3s(0.0f); p.primaryRng = 0u;
    return p;
}
GD Resv resv_zero() { Resv r; r.s = ps_zero(); r.sampleCount = 0.0f; r.resampleWeight = 0.0f; r.contribWeight = 0.0f; r.pad0 = 0.0f; return r; }
GD BsdfSample bs_zero() { BsdfSample b; b.wi = v3s(0.0f); b.pdf = 0.0f; b.bsdf = v3s(0.0f); b.type = 0u; return b; }

/* ---------------------------------------------------------------- scene view */
struct DevScene {
    const GrisMeshVertex* vertices; uint64_t nVertices;
    const uint32_t* indices; uint64_t nIndices;
    const GrisObjectInstance* instances; uint64_t nInstances;
    const GrisMaterial* materials; uint64_t nMaterials;
    const int32_t* matIndices; uint64_t nMatIndices;
    const GrisTriangleLight* lights; uint64_t nLights;
    const GrisLightTableEntry* table; uint64_t nTable;
    const uint32_t* nodes;
    const float* tris;
};

GD float ldf(const float* p) { return __ldg(p); }
GD uint32_t ldu(const uint32_t* p) { return __ldg(p); }

GD Mat load_material(const DevScene& sc, uint32_t i) {
    Mat m;
    if (i < sc.nMaterials) {
        const float4* p = reinterpret_cast<const float4*>(sc.materials + i);
        float4 a = __ldg(p), b = __ldg(p + 1);
        m.baseColor = v3(a.x, a.y, a.z); m.type = __float_as_uint(a.w);
        m.textureIdx = __float_as_uint(b.x); m.metallic = b.y; m.roughness = b.z; m.ior = b.w;
    } else {
        m.baseColor = v3s(0.0f); m.type = 0u; m.textureIdx = 0u; m.metallic = 0.0f; m.roughness = 0.0f; m.ior = 0.0f;
    }
    return m;
}
GD GrisLightTableEntry load_table(const DevScene& sc, uint64_t i) {
    GrisLightTableEntry e;
    if (i < sc.nTable) { e.prob = ldf(&sc.table[i].prob); e.failId = ldu(&sc.table[i].failId); }
    else { e.prob = 0.0f; e.failId = 0u; }
    return e;
}
struct Light { V3 v0, v1, v2, n, radiance; float area; };
GD Light load_light(const DevScene& sc, uint64_t i) {
    Light L;
    if (i < sc.nLights) {
        const float4* p = reinterpret_cast<const float4*>(sc.lights + i);
        float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
        L.v0 = v3(a.x, a.y, a.z); L.v1 = v3(b.x, b.y, b.z); L.v2 = v3(c.x, c.y, c.z);
        L.n = v3(a.w, b.w, c.w); L.radiance = v3(d.x, d.y, d.z); L.area = d.w;
    } else {
        L.v0 = L.v1 = L.v2 = L.n = L.radiance = v3s(0.0f); L.area = 0.0f;
    }
    return L;
}

/* ---------------------------------------------------------------- math.glsl */
GD float luminance(V3 c) { return (c.x * 0.299f + c.y * 0.587f) + c.z * 0.114f; }       /* :171-173 */
GD bool isBlack(V3 c) { return luminance(c) < 1e-5f; }                                   /* :175-177 */
GD V3 clampColor(V3 c) {                                                                 /* :187-192 */
    if (isnan3(c)) return v3s(0.0f);
    return v3(fminf(fmaxf(c.x, 0.0f), 1e4f), fminf(fmaxf(c.y, 0.0f), 1e4f), fminf(fmaxf(c.z, 0.0f), 1e4f));
}
GD uint32_t hash2(uint32_t seed) {                                                       /* :227-234 */
    seed = (seed ^ 61u) ^ (seed >> 16u);
    seed *= 9u;
    seed = seed ^ (seed >> 4u);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15u);
    return seed;
}
GD uint32_t makeSeed(uint32_t rnd, uint32_t index) { return hash2(rnd) + hash2(index); }  /* :240-242 */
GD uint32_t makeSeed2(uint32_t seed, uint32_t ix, uint32_t iy) {                         /* :244-246 */
    return makeSeed((seed + ix) ^ (iy - 1u), iy * (ix - 2u));
}
GD float sample1f(uint32_t& rng) { rng = hash2(rng); return (float)rng / 4294967296.0f; }  /* :248-254 */
GD V2 sample2f(uint32_t& rng) { float a = sample1f(rng); float b = sample1f(rng); return v2(a, b); }
GD V3 sample3f(uint32_t& rng) { V2 a = sample2f(rng); float b = sample1f(rng); return v3(a.x, a.y, b); }
struct V4 { float x, y, z, w; };
GD V4 sample4f(uint32_t& rng) { V2 a = sample2f(rng); V2 b = sample2f(rng); V4 r; r.x = a.x; r.y = a.y; r.z = b.x; r.w = b.y; return r; }
GD float MISWeight(float f, float g) { return (f * f) / (f * f + g * g); }               /* :268-270 */
GD V2 toConcentricDisk(V2 v) {                                                           /* :23-39 */
    if (v.x == 0.0f && v.y == 0.0f) return v2(0.0f, 0.0f);
    v = v2(v.x * 2.0f - 1.0f, v.y * 2.0f - 1.0f);
    float phi, r;
    if (v.x * v.x > v.y * v.y) { r = v.x; phi = kPi * v.y / v.x * 0.25f; }
    else { r = v.y; phi = kPi * 0.5f - kPi * v.x / v.y * 0.25f; }
    float s, c;
    gris_det_sincosf(phi, &s, &c);
    return v2(r * c, r * s);
}
struct M3 { V3 c0, c1, c2; };
GD V3 m3mul(const M3& m, V3 v) { return (m.c0 * v.x + m.c1 * v.y) + m.c2 * v.z; }
GD M3 matLocalToWorld(V3 n) {                                                            /* :69-78 */
    V3 t = fabsf(n.z) > 0.999f ? v3(0.0f, 1.0f, 0.0f) : v3(0.0f, 0.0f, 1.0f);
    V3 b = normalize3(cross3(n, t));
    t = cross3(b, n);
    M3 m; m.c0 = t; m.c1 = b; m.c2 = n; return m;
}
GD M3 inverse3(const M3& m) {
    V3 r0 = cross3(m.c1, m.c2), r1 = cross3(m.c2, m.c0), r2 = cross3(m.c0, m.c1);
    float invDet = 1.0f / dot3(m.c0, r0);
    M3 o;
    o.c0 = v3(r0.x * invDet, r1.x * invDet, r2.x * invDet);
    o.c1 = v3(r0.y * invDet, r1.y * invDet, r2.y * invDet);
    o.c2 = v3(r0.z * invDet, r1.z * invDet, r2.z * invDet);
    return o;
}
GD V3 sampleCosineWeightedHemisphere(V3 n, V2 u) {                                      /* :85-89 */
    V2 uv = toConcentricDisk(u);
    float z = sqrtf(1.0f - dot2(uv, uv));
    return normalize3(m3mul(matLocalToWorld(n), v3(uv.x, uv.y, z)));
}
GD V2 uvToBary(V2 uv) { float r = sqrtf(uv.y); return v2(1.0f - r, uv.x * r); }       /* :117-120 */

/* ---------------------------------------------------------------- material.glsl */
GD float pow5(float x) { float x2 = x * x; return x2 * x2 * x; }
GD float fresnelSchlickF(float cosTheta, float ior) {                                   /* :31-34 */
    float f0 = fabsf(1.0f - ior) / (1.0f + ior);
    return mixf(f0, 1.0f, pow5(1.0f - cosTheta));
}
GD V3 fresnelSchlickV(float cosTheta, V3 f0) { return mix3(f0, v3s(1.0f), pow5(1.0f - cosTheta)); }  /* :36-38 */
GD float schlickG(float cosTheta, float alpha) {                                        /* :59-62 */
    float a = alpha * 0.5f;
    return cosTheta / (cosTheta * (1.0f - a) + a);
}
GD float smithG(float cosWo, float cosWi, float alpha) { return schlickG(fabsf(cosWo), alpha) * schlickG(fabsf(cosWi), alpha); }
GD float GTR2Distrib(float cosTheta, float alpha) {                                     /* :68-77 */
    if (cosTheta < 1e-6f) return 0.0f;
    float aa = alpha * alpha;
    float nom = aa;
    float denom = cosTheta * cosTheta * (aa - 1.0f) + 1.0f;
    denom = denom * denom * kPi;
    return nom / denom;
}
GD float GTR2Pdf(V3 n, V3 m, V3 wo, float alpha) {                                     /* :79-82 */
    return GTR2Distrib(dot3(n, m), alpha) * schlickG(dot3(n, wo), alpha) * absDot(m, wo) / absDot(n, wo);
}
GD V3 GTR2Sample(V3 n, V3 wo, float alpha, V2 r) {                                      /* :84-101 */
    M3 transMat = matLocalToWorld(n);
    M3 transInv = inverse3(transMat);
    V3 vh = normalize3(m3mul(transInv, wo) * v3(alpha, alpha, 1.0f));
    float lenSq = vh.x * vh.x + vh.y * vh.y;
    V3 t = lenSq > 0.0f ? v3(-vh.y, vh.x, 0.0f) / sqrtf(lenSq) : v3(1.0f, 0.0f, 0.0f);
    V3 b = cross3(vh, t);
    V2 p = toConcentricDisk(r);
    float s = 0.5f * (vh.z + 1.0f);
    p.y = (1.0f - s) * sqrtf(1.0f - p.x * p.x) + s * p.y;
    V3 wh = t * p.x + b * p.y + vh * sqrtf(fmaxf(0.0f, 1.0f - dot2(p, p)));
    wh = v3(wh.x * alpha, wh.y * alpha, fmaxf(0.0f, wh.z));
    return normalize3(m3mul(transMat, wh));
}
GD bool isGTR2Connectible(float roughness) { return roughness > 0.05f; }                /* :103-105 */
GD bool isGTR2Delta(float roughness) { return roughness < 0.01f; }                      /* :107-109 */
GD bool refractDir(V3 n, V3 wi, float ior, V3& wt) {                                    /* :111-128 */
    float cosIn = dot3(n, wi);
    if (cosIn < 0.0f) ior = 1.0f / ior;
    float sin2In = fmaxf(0.0f, 1.0f - cosIn * cosIn);
    float sin2Tr = sin2In / (ior * ior);
    if (sin2Tr >= 1.0f) return false;
    float cosTr = sqrtf(1.0f - sin2Tr);
    if (cosIn < 0.0f) cosTr = -cosTr;
    wt = normalize3(-wi / ior + n * (cosIn / ior - cosTr));
    return true;
}
GD V3 metallicWorkflowBSDF(const Mat& mat, V3 albedo, V3 n, V3 wo, V3 wi) {            /* :170-186 */
    float alpha = square(mat.roughness);
    V3 wh = normalize3(wo + wi);
    float cosO = dot3(n, wo);
    float cosI = dot3(n, wi);
    if (cosI * cosO < 1e-7f) return v3s(0.0f);
    V3 f = fresnelSchlickV(dot3(wh, wo), mix3(v3s(0.08f), albedo, mat.metallic));
    float g = smithG(cosO, cosI, alpha);
    float d = GTR2Distrib(dot3(n, wh), alpha);
    return mix3v(albedo * kPiInv * (1.0f - mat.metallic), v3s(g * d / (4.0f * cosI * cosO)), f);
}
GD float metallicWorkflowPdf(const Mat& mat, V3 n, V3 wo, V3 wi) {                      /* :188-196 */
    V3 wh = normalize3(wo + wi);
    return mixf(satDot(n, wi) * kPiInv, GTR2Pdf(n, wh, wo, square(mat.roughness)) / (4.0f * absDot(wh, wo)),
                1.0f / (2.0f - mat.metallic));
}
GD V3 metalBSDF(const Mat& mat, V3 albedo, V3 n, V3 wo, V3 wi) {                       /* :223-243 */
    if (isGTR2Delta(mat.roughness)) return v3s(0.0f);
    float alpha = square(mat.roughness);
    V3 wh = normalize3(wo + wi);
    float cosO = dot3(n, wo);
    float cosI = dot3(n, wi);
    if (cosI * cosO < 1e-7f) return v3s(0.0f);
    float f = fresnelSchlickF(absDot(wh, wo), mat.ior);
    float g = smithG(cosO, cosI, alpha);
    float d = GTR2Distrib(dot3(n, wh), alpha);
    return albedo * f * g * d / (4.0f * cosI * cosO);
}
GD float metalPdf(const Mat& mat, V3 n, V3 wo, V3 wi) {                                 /* :245-251 */
    if (isGTR2Delta(mat.roughness)) return 0.0f;
    V3 wh = normalize3(wo + wi);
    return GTR2Pdf(n, wh, wo, square(mat.roughness)) / (4.0f * absDot(wh, wo));
}
GD V3 evalBSDF(const Mat& mat, V3 albedo, V3 n, V3 wo, V3 wi) {                        /* :286-299 */
    switch (mat.type) {
    case kLambert: return albedo * kPiInv;
    case kMetallicWorkflow: return metallicWorkflowBSDF(mat, albedo, n, wo, wi);
    case kMetal: return metalBSDF(mat, albedo, n, wo, wi);
    default: return v3s(0.0f);
    }
}
GD float evalPdf(const Mat& mat, V3 n, V3 wo, V3 wi) {                                  /* :301-314 */
    switch (mat.type) {
    case kLambert: return absDot(n, wi) * kPiInv;
    case kMetallicWorkflow: return metallicWorkflowPdf(mat, n, wo, wi);
    case kMetal: return metalPdf(mat, n, wo, wi);
    default: return 0.0f;
    }
}
/* sampleBSDF (:316-330) with lambert/dielectric/metallicWorkflow/metal/fake (:138-284). On the
 * invalid paths `s` keeps the fields the reference leaves unwritten. */
GD bool sampleBSDF(const Mat& mat, V3 albedo, V3 n, V3 wo, V3 r, BsdfSample& s) {
    switch (mat.type) {
    case kLambert:
        s.wi = sampleCosineWeightedHemisphere(n, v2(r.x, r.y));
        s.pdf = absDot(n, s.wi) * kPiInv;
        s.bsdf = albedo * kPiInv;
        s.type = kDiffuse | kReflection;
        return true;
    case kMetallicWorkflow: {
        float alpha = square(mat.roughness);
        s.type = kReflection;
        if (r.z > (1.0f / (2.0f - mat.metallic))) {
            s.wi = sampleCosineWeightedHemisphere(n, v2(r.x, r.y));
            s.type |= kDiffuse;
        } else {
            V3 wh = GTR2Sample(n, wo, alpha, v2(r.x, r.y));
            s.wi = -reflect3(wo, wh);
            s.type |= isGTR2Delta(mat.roughness) ? kSpecular : kGlossy;
        }
        if (dot3(n, s.wi) < 0.0f) { s.type = kInvalidBSDFSample; return false; }
        s.bsdf = metallicWorkflowBSDF(mat, albedo, n, wo, s.wi);
        s.pdf = metallicWorkflowPdf(mat, n, wo, s.wi);
        return true;
    }
    case kMetal: {
        float alpha = square(mat.roughness);
        bool isDelta = isGTR2Delta(mat.roughness);
        if (isDelta) s.wi = -reflect3(wo, n);
        else { V3 wh = GTR2Sample(n, wo, alpha, v2(r.x, r.y)); s.wi = -reflect3(wo, wh); }
        if (dot3(n, s.wi) < 0.0f) { s.type = kInvalidBSDFSample; return false; }
        s.bsdf = isDelta ? albedo * fresnelSchlickF(absDot(n, wo), mat.ior) : metalBSDF(mat, albedo, n, wo, s.wi);
        s.pdf = isDelta ? 1.0f : metalPdf(mat, n, wo, s.wi);
        s.type = kReflection | (isDelta ? kSpecular : kGlossy);
        return true;
    }
    case kDielectric: {
        float pdfReflect = fresnelSchlickF(dot3(n, wo), mat.ior);
        s.bsdf = albedo;
        if (r.z < pdfReflect) {
            s.wi = reflect3(-wo, n);
            s.type = kSpecular | kReflection;
            s.pdf = 1.0f;
        } else {
            V3 wt;
            if (!refractDir(n, wo, mat.ior, wt)) { s.type = kInvalidBSDFSample; return false; }
            s.wi = wt;
            float ior = mat.ior;
            if (dot3(n, wo) < 0.0f) ior = 1.0f / ior;
            s.bsdf = s.bsdf / (ior * ior);
            s.type = kSpecular | kTransmission;
            s.pdf = 1.0f;
        }
        return true;
    }
    case kFake:
        s.wi = -wo; s.bsdf = albedo; s.pdf = 1.0f; s.type = kSpecular | kTransmission;
        return true;
    default:
        return false;
    }
}
GD bool isBSDFDelta(const Mat& mat) {                                                    /* :332-345 */
    switch (mat.type) {
    case kLambert: return false;
    case kMetallicWorkflow: return isGTR2Delta(mat.roughness) && mat.metallic > 0.9f;
    case kMetal: return isGTR2Delta(mat.roughness);
    default: return true;
    }
}
GD bool isBSDFConnectible(const Mat& mat) {                                              /* :347-360 */
    switch (mat.type) {
    case kLambert: return true;
    case kMetallicWorkflow: return isGTR2Connectible(mat.roughness) || mat.metallic < 0.9f;
    case kMetal: return isGTR2Connectible(mat.roughness);
    default: return false;
    }
}
GD bool isSampleTypeDelta(uint32_t type) { return (type & kSpecular) == kSpecular; }     /* :362-364 */

/* ---------------------------------------------------------------- light_sampling.glsl */
GD V3 sampleTriangleLight(const Light& light, V3 ref, V3& wi, float& dist, float& pdf, float& jacobian, V2& bary, V2 r) {
    bary = uvToBary(r);                                                                  /* :6-23 */
    V3 pos = light.v0 * (1.0f - bary.x - bary.y) + light.v1 * bary.x + light.v2 * bary.y;
    dist = distance3(ref, pos);
    wi = (pos - ref) / dist;
    jacobian = absDot(light.n, wi) / square(dist);
    pdf = 1.0f / jacobian / light.area;
    if (dot3(light.n, wi) > 0.0f) return v3s(0.0f);
    return light.radiance;
}
GD V3 sampleLightByPower(const DevScene& sc, V3 ref, V3& wi, float& dist, float& pdf, float& jacobian, V2& bary,
                         uint32_t& id, V4 r) {                                            /* :25-37 */
    GrisLightTableEntry t0 = load_table(sc, 0);
    float sumPower = t0.prob;
    uint32_t numLights = t0.failId;
    id = (uint32_t)((float)numLights * r.x);
    GrisLightTableEntry e = load_table(sc, (uint64_t)id + 1u);
    id = (r.y < e.prob) ? id : e.failId - 1u;
    Light light = load_light(sc, id);
    V3 radiance = sampleTriangleLight(light, ref, wi, dist, pdf, jacobian, bary, v2(r.z, r.w));
    pdf *= luminance(light.radiance) * light.area / sumPower;
    return radiance;
}

/* ---------------------------------------------------------------- surfaces (ray_layouts.glsl:50-104) */
GD V3 m4mul_point(const float* m, V3 p, float w) {   /* mat4 * vec4(p, w), xyz; m column-major */
    V3 c0 = v3(m[0], m[1], m[2]), c1 = v3(m[4], m[5], m[6]), c2 = v3(m[8], m[9], m[10]), c3 = v3(m[12], m[13], m[14]);
    return ((c0 * p.x + c1 * p.y) + c2 * p.z) + c3 * w;
}
GD void load_mat4(const float* src, float* dst) {
    const float4* p = reinterpret_cast<const float4*>(src);
    for (int i = 0; i < 4; i++) { float4 v = __ldg(p + i); dst[4 * i] = v.x; dst[4 * i + 1] = v.y; dst[4 * i + 2] = v.z; dst[4 * i + 3] = v.w; }
}
GD void load_vertex(const DevScene& sc, uint64_t vi, V3& pos, V3& norm) {
    if (vi < sc.nVertices) {
        const float4* p = reinterpret_cast<const float4*>(sc.vertices + vi);
        float4 a = __ldg(p), b = __ldg(p + 1);
        pos = v3(a.x, a.y, a.z); norm = v3(b.x, b.y, b.z);
    } else { pos = v3s(0.0f); norm = v3s(0.0f); }
}
GD uint32_t load_index(const DevScene& sc, uint64_t i) { return i < sc.nIndices ? ldu(sc.indices + i) : 0u; }

/* loadSurfaceInfo(Intersection, out SurfaceInfo) — a light hit leaves matIndex as it was. */
GD void loadSurfaceInfo(const DevScene& sc, const Isec& isec, Surf& info) {
    V3 b = v3(1.0f - isec.bx - isec.by, isec.bx, isec.by);
    if (isec.inst == 0u) {
        Light L = load_light(sc, isec.tri);
        info.pos = L.v0 * b.x + L.v1 * b.y + L.v2 * b.z;
        info.norm = L.n;
        info.albedo = L.radiance;
        info.isLight = true;
        return;
    }
    uint64_t k = (uint64_t)isec.inst - 1u;
    float T[16], TI[16];
    uint32_t indexOffset = 0u;
    if (k < sc.nInstances) {
        const GrisObjectInstance* I = sc.instances + k;
        load_mat4(I->transform, T);
        load_mat4(I->transformInvT, TI);
        indexOffset = ldu(&I->indexOffset);
    } else {
        for (int i = 0; i < 16; i++) { T[i] = 0.0f; TI[i] = 0.0f; }
    }
    uint64_t mi = (uint64_t)(indexOffset / 3u + isec.tri);
    info.matIndex = (uint32_t)(mi < sc.nMatIndices ? (int32_t)ldu(reinterpret_cast<const uint32_t*>(sc.matIndices + mi)) : 0);
    uint64_t base = (uint64_t)(indexOffset + isec.tri * 3u);
    V3 p0, p1, p2, n0, n1, n2;
    load_vertex(sc, load_index(sc, base + 0), p0, n0);
    load_vertex(sc, load_index(sc, base + 1), p1, n1);
    load_vertex(sc, load_index(sc, base + 2), p2, n2);
    V3 pos = p0 * b.x + p1 * b.y + p2 * b.z;
    V3 norm = n0 * b.x + n1 * b.y + n2 * b.z;
    info.pos = m4mul_point(T, pos, 1.0f);
    info.norm = normalize3(m4mul_point(TI, norm, 1.0f));
    info.albedo = load_material(sc, info.matIndex).baseColor;   /* textureIdx must be invalid (checked at upload) */
    info.isLight = false;
}

/* ---------------------------------------------------------------- camera.glsl:28-42 */
/* aspect = w / h and tanHalfFov = tan(FOV / 2) are the per-frame constants of the ray
 * (computed on the host by make_cam with the same binary32 operations as the shader's). */
struct CamD {
    V3 pos, front, right, up;
    float FOV;
    uint32_t w, h, frameIndex, seed;
    float aspect, tanHalfFov;
};
/* The shader adds (1 / size) * 0 to uv before mapping to [-1, 1]; that term is +0 and changes no
 * result (x + 0 = x, and -0 maps to -1 as +0 does), so it is left out. */
GD Ray3 pinholeCameraSampleRay(const CamD& cam, V2 uv) {
    V2 ndc = v2(uv.x * 2.0f - 1.0f, uv.y * 2.0f - 1.0f);
    const float aspect = cam.aspect, tanFOV = cam.tanHalfFov;
    V3 pFocus = v3(ndc.x * aspect * tanFOV, ndc.y * 1.0f * tanFOV, 1.0f);
    V3 dir = normalize3(pFocus);
    dir = normalize3(cam.right * dir.x + cam.up * dir.y + cam.front * dir.z);
    Ray3 r; r.ori = cam.pos; r.dir = dir;
    return r;
}

/* ---------------------------------------------------------------- G-buffer views */
struct GBufView {
    const float4* depthNormal;
    const uint2* albedoMatId;
    int w, h;
};
GD float4 texel4(const float4* t, int w, int h, int x, int y) {
    if (x < 0 || y < 0 || x >= w || y >= h) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    return __ldg(t + (size_t)y * w + x);
}
GD int wrapi(int i, int n) { int r = i % n; return r < 0 ? r + n : r; }
GD float4 mix4(float4 a, float4 b, float t) {
    float u = 1.0f - t;
    return make_float4(a.x * u + b.x * t, a.y * u + b.y * t, a.z * u + b.z * t, a.w * u + b.w * t);
}
/* texture(sampler2D, uv): bilinear, REPEAT, 8-bit sub-texel weights. */
GD float4 texture_bilinear(const float4* t, int w, int h, V2 uv) {
    float x = uv.x * (float)w - 0.5f;
    float y = uv.y * (float)h - 0.5f;
    float x0 = floorf(x), y0 = floorf(y);
    float qx = floorf((x - x0) * 256.0f + 0.5f);
    float qy = floorf((y - y0) * 256.0f + 0.5f);
    int ix = (int)x0, iy = (int)y0;
    if (qx >= 256.0f) { ix += 1; qx = 0.0f; }
    if (qy >= 256.0f) { iy += 1; qy = 0.0f; }
    float wx = qx * 0.00390625f, wy = qy * 0.00390625f;
    int i0 = wrapi(ix, w), i1 = wrapi(ix + 1, w), j0 = wrapi(iy, h), j1 = wrapi(iy + 1, h);
    float4 top = mix4(texel4(t, w, h, i0, j0), texel4(t, w, h, i1, j0), wx);
    float4 bot = mix4(texel4(t, w, h, i0, j1), texel4(t, w, h, i1, j1), wx);
    return mix4(top, bot, wy);
}
GD uint2 fetch_am(const uint2* t, int w, int h, int x, int y) {
    if (x < 0 || y < 0 || x >= w || y >= h) return make_uint2(0u, 0u);
    return __ldg(t + (size_t)y * w + x);
}
GD V3 unpackAlbedo(uint32_t p) {
    return v3((float)(p & 0xffu) / 255.0f, (float)((p >> 8) & 0xffu) / 255.0f, (float)((p >> 16) & 0xffu) / 255.0f);
}
/* unpackGBuffer (gbuffer_util.glsl:24-35) */
GD bool unpackGBuffer(float4 dn, uint2 am, float& depth, V3& normal, V3& albedo, int& matMeshId) {
    depth = dn.x;
    if (depth == 0.0f) return false;
    normal = v3(dn.y, dn.z, dn.w);
    albedo = unpackAlbedo(am.x);
    matMeshId = (int)am.y;
    return true;
}

/* ---------------------------------------------------------------- reservoirs (gris_reservoir.glsl) */
GD void setRcVertexId(uint32_t& f, uint32_t id) { f = (f & 0xffffff00u) | (id & 0xffu); }
GD void setPathLength(uint32_t& f, uint32_t l) { f = (f & 0xffff00ffu) | ((l & 0xffu) << 8); }
GD void setRcVertexType(uint32_t& f, uint32_t t) { f = (f & 0xff00ffffu) | ((t & 0xffu) << 16); }
GD uint32_t rcVertexId(uint32_t f) { return f & 0xffu; }
GD uint32_t rcVertexType(uint32_t f) { return (f >> 16) & 0xffu; }
GD void pathSampleReset(PathSample& p) {                                                 /* :61-69 */
    p.rcIsec.inst = kInvalidHit; p.rcLi = v3s(0.0f); p.rcWi = v3s(0.0f);
    p.rcPrevSamplePdf = 0.0f; p.rcJacobian = 0.0f; p.flags = 0u; p.F = v3s(0.0f);
}
GD void resvReset(Resv& r) { r.s.rcIsec.inst = kInvalidHit; r.sampleCount = 0.0f; r.resampleWeight = 0.0f; }  /* :75-79 */
GD bool resvIsValid(const Resv& r) { return !isnan(r.resampleWeight) && r.resampleWeight >= 0.0f; }   /* :93-95 */
GD void resvResetIfInvalid(Resv& r) { if (!resvIsValid(r)) resvReset(r); }
GD bool resvMerge(Resv& r, const Resv& rhs, float rnd) {                                  /* :114-123 */
    r.sampleCount += rhs.sampleCount;
    r.resampleWeight += rhs.resampleWeight;
    if (rnd * r.resampleWeight < rhs.resampleWeight) { r.s = rhs.s; return true; }
    return false;
}
GD void resvCap(Resv& r, float cap) {                                                     /* :131-136 */
    if (r.sampleCount > cap) { r.resampleWeight *= cap / r.sampleCount; r.sampleCount = cap; }
}

GD Resv load_resv(const GrisReservoir* buf, uint64_t i, uint64_t n) {
    Resv r;
    if (i >= n) return resv_zero();
    const uint4* p = reinterpret_cast<const uint4*>(buf + i);
    uint4 a = p[0], b = p[1], c = p[2], d = p[3], e = p[4], f = p[5];
    r.s.rcIsec.bx = __uint_as_float(a.x); r.s.rcIsec.by = __uint_as_float(a.y); r.s.rcIsec.inst = a.z; r.s.rcIsec.tri = a.w;
    r.s.rcLi = v3(__uint_as_float(b.x), __uint_as_float(b.y), __uint_as_float(b.z)); r.s.rcRng = b.w;
    r.s.rcWi = v3(__uint_as_float(c.x), __uint_as_float(c.y), __uint_as_float(c.z)); r.s.flags = c.w;
    r.s.pad0 = __uint_as_float(d.x); r.s.pad1 = __uint_as_float(d.y);
    r.s.rcPrevSamplePdf = __uint_as_float(d.z); r.s.rcJacobian = __uint_as_float(d.w);
    r.s.F = v3(__uint_as_float(e.x), __uint_as_float(e.y), __uint_as_float(e.z)); r.s.primaryRng = e.w;
    r.sampleCount = __uint_as_float(f.x); r.resampleWeight = __uint_as_float(f.y);
    r.contribWeight = __uint_as_float(f.z); r.pad0 = __uint_as_float(f.w);
    return r;
}
GD void store_resv(GrisReservoir* buf, uint64_t i, const Resv& r) {
    uint4* p = reinterpret_cast<uint4*>(buf + i);
    p[0] = make_uint4(__float_as_uint(r.s.rcIsec.bx), __float_as_uint(r.s.rcIsec.by), r.s.rcIsec.inst, r.s.rcIsec.tri);
    p[1] = make_uint4(__float_as_uint(r.s.rcLi.x), __float_as_uint(r.s.rcLi.y), __float_as_uint(r.s.rcLi.z), r.s.rcRng);
    p[2] = make_uint4(__float_as_uint(r.s.rcWi.x), __float_as_uint(r.s.rcWi.y), __float_as_uint(r.s.rcWi.z), r.s.flags);
    p[3] = make_uint4(__float_as_uint(r.s.pad0), __float_as_uint(r.s.pad1), __float_as_uint(r.s.rcPrevSamplePdf),
                      __float_as_uint(r.s.rcJacobian));
    p[4] = make_uint4(__float_as_uint(r.s.F.x), __float_as_uint(r.s.F.y), __float_as_uint(r.s.F.z), r.s.primaryRng);
    p[5] = make_uint4(__float_as_uint(r.sampleCount), __float_as_uint(r.resampleWeight), __float_as_uint(r.contribWeight),
                      __float_as_uint(r.pad0));
}

}  // namespace grisrt

#endif
