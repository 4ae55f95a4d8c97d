/*
 * gris_oracle.cpp — CPU restatement of the reference's ReSTIR PT (GRIS) path.
 *
 * TEST INFRASTRUCTURE: the oracle. Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference legs may load it, and only as the checker or the timed CPU
 * baseline. It is never part of the product path.
 *
 * Pinning: this restatement is checked bit for bit against the reference's own shader
 * code compiled as C++ (oracle/_ref, built by oracle/ref/make_ref.py from the reference
 * sources) on the synthetic scenes, and against golden fixtures generated from it
 * (tests/golden). The light alias table is additionally checked against the reference's
 * src/util/AliasTable.h compiled directly.
 *
 * Definitions where the reference is implementation-defined (the same in the compiled
 * reference harness and the CUDA kernels): ray queries are exact Moller-Trumbore (cross and dot
 * products fused, one rounding per fma) over
 * world-space triangles (closest hit = smallest t, then smallest (instance, triangle));
 * the G-buffer is a primary ray per pixel centre that ignores the light instance;
 * texture() is bilinear / repeat / 8-bit sub-texel weights; robust (zero) out-of-range
 * reads; sin/cos/tan from detmath.h; reads of locals before their first write see 0.
 *
 * Build: g++ -O2 -std=c++17 -ffp-contract=off -fopenmp -shared -fPIC (oracle/build_oracle.py).
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include <omp.h>

#include "detmath.h"

namespace oracle {

/* ------------------------------------------------------------------ vectors */
struct F2 { float x, y; };
struct F3 {
    float x, y, z;
    F3() : x(0), y(0), z(0) {}
    F3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit F3(float s) : x(s), y(s), z(s) {}
};
static inline F3 operator+(const F3& a, const F3& b) { return F3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline F3 operator-(const F3& a, const F3& b) { return F3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline F3 operator*(const F3& a, const F3& b) { return F3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline F3 operator*(const F3& a, float s) { return F3(a.x * s, a.y * s, a.z * s); }
static inline F3 operator/(const F3& a, float s) { return F3(a.x / s, a.y / s, a.z / s); }
static inline F3 operator-(const F3& a) { return F3(-a.x, -a.y, -a.z); }
static inline float dot(const F3& a, const F3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline F3 cross(const F3& a, const F3& b) { return F3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline float len(const F3& v) { return sqrtf(dot(v, v)); }
static inline F3 unit(const F3& v) { return v * (1.0f / sqrtf(dot(v, v))); }
static inline float fmx(float a, float b) { return fmaxf(a, b); }
static inline float fmn(float a, float b) { return fminf(a, b); }
static inline bool anyNan(const F3& c) { return std::isnan(c.x) || std::isnan(c.y) || std::isnan(c.z); }
static inline F3 lerp3(const F3& x, const F3& y, float a) { return x * (1.0f - a) + y * a; }

static const float PI = 3.14159265358979323846f;
static const float INV_PI = 0x1.45f306p-2f;
static const float RAY_TMIN = 1e-4f, RAY_TMAX = 1e7f;
static const uint32_t NO_HIT = 0xffffffffu, PRIMARY_HIT = 0xfffffffeu;

/* ------------------------------------------------------------------ reference layouts */
struct Material { float base[3]; uint32_t type, tex; float metallic, roughness, ior; };
struct Vertex { float pos[3]; float u; float nrm[3]; float v; };
struct Instance { float M[16], Minv[16], MinvT[16]; float radiance[3], pad; uint32_t indexOffset, indexCount, matIndex; float pad2; };
struct TriLight { float v0[3], nx, v1[3], ny, v2[3], nz, rad[3], area; };
struct TableEntry { float prob; uint32_t failId; };
struct Camera {
    float view[16], proj[16], projView[16], lastProjView[16];
    float pos[3], fov, angle[3], nearZ, front[3], farZ, right[3], lensRadius, up[3], focalDist;
    uint32_t film[2], frameIndex, seed;
};
struct Hit { float bx, by; uint32_t inst, tri; };
struct PathSample {
    Hit rc; float rcLi[3]; uint32_t rcRng; float rcWi[3]; uint32_t flags;
    float pad[2]; float rcPrevSamplePdf, rcJacobian; float F[3]; uint32_t primaryRng;
};
struct Reservoir { PathSample s; float M, W, contribWeight, pad0; };
struct Settings {
    uint32_t shift; float rrScale; uint32_t temporal, spatial, cap, maxDepth, neighbours; float radius;
    float envReserved[3];   /* must be 0 */
    uint32_t misWeights;    /* extension: 1 = pairwise generalised balance heuristic in the reuse passes */
};
static_assert(sizeof(Camera) == 352 && sizeof(Reservoir) == 96 && sizeof(Instance) == 224, "layouts");

static inline F3 ld3(const float* p) { return F3(p[0], p[1], p[2]); }
static inline void st3(float* p, const F3& v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }

/* ------------------------------------------------------------------ scene */
struct Tri { F3 v0, e1, e2; uint32_t inst, tri; };
struct Node { float lo[3], hi[3]; int32_t left; uint32_t first, count; };

struct Scene {
    std::vector<Vertex> vertices;
    std::vector<uint32_t> indices;
    std::vector<Instance> instances;
    std::vector<Material> materials;
    std::vector<int32_t> matIndices;
    std::vector<TriLight> lights;
    std::vector<TableEntry> table;
    std::vector<Tri> tris;
    std::vector<Node> bvh;
    std::vector<uint32_t> order;
    int useBvh = 0;
};
static Scene g;
static unsigned long long g_counts[4];
static int g_row0 = 0, g_row1 = 1 << 30;   /* rows processed by the passes (a bounded CPU sample) */

template <typename T> static inline T at(const std::vector<T>& v, uint64_t i) {
    if (i < v.size()) return v[i];
    T z; memset((void*)&z, 0, sizeof(T)); return z;
}

/* ------------------------------------------------------------------ ray queries (semantics in the file header) */
/* cross and dot products with one rounding per fused step: a*b - c*d = fma(a, b, -(c*d)),
 * a.b = fma(a.z, b.z, fma(a.y, b.y, a.x*b.x)) */
static inline F3 crossF(const F3& a, const F3& b) {
    return F3(fmaf(a.y, b.z, -(a.z * b.y)), fmaf(a.z, b.x, -(a.x * b.z)), fmaf(a.x, b.y, -(a.y * b.x)));
}
static inline float dotF(const F3& a, const F3& b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
static inline bool hitTriangle(const Tri& T, const F3& o, const F3& d, float tmin, float tmax, float& t, float& u, float& v) {
    F3 pv = crossF(d, T.e2);
    float det = dotF(T.e1, pv);
    if (det == 0.0f) return false;
    float inv = 1.0f / det;
    F3 tv = o - T.v0;
    u = dotF(tv, pv) * inv;
    if (!(u >= 0.0f) || !(u <= 1.0f)) return false;
    F3 qv = crossF(tv, T.e1);
    v = dotF(d, qv) * inv;
    if (!(v >= 0.0f) || !(u + v <= 1.0f)) return false;
    t = dotF(T.e2, qv) * inv;
    if (!(t >= tmin) || !(t <= tmax)) return false;
    return true;
}

struct Best { float t; unsigned long long key; float u, v; bool found; };
static inline void consider(const Tri& T, const F3& o, const F3& d, float tmin, Best& b) {
    float t, u, v;
    if (!hitTriangle(T, o, d, tmin, b.t, t, u, v)) return;
    unsigned long long key = ((unsigned long long)T.inst << 32) | T.tri;
    if (t < b.t || key < b.key) { b.t = t; b.key = key; b.u = u; b.v = v; b.found = true; }
}

static inline bool boxHit(const Node& n, const F3& o, const F3& inv, float tmin, float tmax) {
    float t0 = tmin, t1 = tmax;
    const float oo[3] = {o.x, o.y, o.z}, ii[3] = {inv.x, inv.y, inv.z};
    for (int a = 0; a < 3; a++) {
        float ta = (n.lo[a] - oo[a]) * ii[a], tb = (n.hi[a] - oo[a]) * ii[a];
        t0 = fmx(t0, fmn(ta, tb));
        t1 = fmn(t1, fmx(ta, tb));
    }
    return t0 <= t1;
}

static bool traceQuery(const F3& o, const F3& d, float tmin, float tmax, bool any, bool skipLights, Hit* out, float* tOut) {
    Best b; b.t = tmax; b.key = ~0ull; b.u = b.v = 0.0f; b.found = false;
    if (!g.useBvh || g.bvh.empty()) {
        for (const Tri& T : g.tris) {
            if (skipLights && T.inst == 0) continue;
            if (any) { float t, u, v; if (hitTriangle(T, o, d, tmin, tmax, t, u, v)) return true; continue; }
            consider(T, o, d, tmin, b);
        }
    } else {
        F3 inv(1.0f / (fabsf(d.x) > 1e-30f ? d.x : copysignf(1e-30f, d.x)),
               1.0f / (fabsf(d.y) > 1e-30f ? d.y : copysignf(1e-30f, d.y)),
               1.0f / (fabsf(d.z) > 1e-30f ? d.z : copysignf(1e-30f, d.z)));
        uint32_t stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp) {
            const Node& n = g.bvh[stack[--sp]];
            if (!boxHit(n, o, inv, tmin, b.t)) continue;
            if (n.count) {
                for (uint32_t i = 0; i < n.count; i++) {
                    const Tri& T = g.tris[g.order[n.first + i]];
                    if (skipLights && T.inst == 0) continue;
                    if (any) { float t, u, v; if (hitTriangle(T, o, d, tmin, tmax, t, u, v)) return true; continue; }
                    consider(T, o, d, tmin, b);
                }
            } else {
                stack[sp++] = (uint32_t)n.left;
                stack[sp++] = (uint32_t)n.left + 1;
            }
        }
    }
    if (any) return false;
    if (b.found && out) { out->bx = b.u; out->by = b.v; out->inst = (uint32_t)(b.key >> 32); out->tri = (uint32_t)b.key; }
    if (tOut) *tOut = b.found ? b.t : -1.0f;
    return b.found;
}

/* A plain binary BVH (median splits, boxes padded outward) used to time the CPU baseline;
 * with exact triangle tests it returns the same hits as the brute-force loop. */
static void buildBvh() {
    g.bvh.clear();
    g.order.resize(g.tris.size());
    for (size_t i = 0; i < g.tris.size(); i++) g.order[i] = (uint32_t)i;
    if (g.tris.empty()) return;
    std::vector<float> cen(g.tris.size() * 3);
    for (size_t i = 0; i < g.tris.size(); i++) {
        const Tri& T = g.tris[i];
        F3 a = T.v0, b = T.v0 + T.e1, c = T.v0 + T.e2;
        cen[i * 3] = (a.x + b.x + c.x) / 3.0f; cen[i * 3 + 1] = (a.y + b.y + c.y) / 3.0f; cen[i * 3 + 2] = (a.z + b.z + c.z) / 3.0f;
    }
    struct Job { uint32_t node, first, count; };
    std::vector<Job> jobs;
    g.bvh.push_back(Node());
    jobs.push_back({0, 0, (uint32_t)g.tris.size()});
    while (!jobs.empty()) {
        Job j = jobs.back(); jobs.pop_back();
        Node n;
        for (int a = 0; a < 3; a++) { n.lo[a] = INFINITY; n.hi[a] = -INFINITY; }
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t i = j.first; i < j.first + j.count; i++) {
            const Tri& T = g.tris[g.order[i]];
            F3 p[3] = {T.v0, T.v0 + T.e1, T.v0 + T.e2};
            for (int k = 0; k < 3; k++) {
                const float q[3] = {p[k].x, p[k].y, p[k].z};
                for (int a = 0; a < 3; a++) { n.lo[a] = fminf(n.lo[a], q[a]); n.hi[a] = fmaxf(n.hi[a], q[a]); }
            }
            for (int a = 0; a < 3; a++) { clo[a] = fminf(clo[a], cen[g.order[i] * 3 + a]); chi[a] = fmaxf(chi[a], cen[g.order[i] * 3 + a]); }
        }
        for (int a = 0; a < 3; a++) {
            float pad = 1e-4f * (n.hi[a] - n.lo[a]) + 1e-5f * fmaxf(fabsf(n.lo[a]), fabsf(n.hi[a])) + 1e-30f;
            n.lo[a] -= pad; n.hi[a] += pad;
        }
        if (j.count <= 4) { n.left = -1; n.first = j.first; n.count = j.count; g.bvh[j.node] = n; continue; }
        int axis = 0;
        for (int a = 1; a < 3; a++) if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
        uint32_t mid = j.first + j.count / 2;
        std::nth_element(g.order.begin() + j.first, g.order.begin() + mid, g.order.begin() + j.first + j.count,
                         [&](uint32_t x, uint32_t y) { return cen[x * 3 + axis] < cen[y * 3 + axis]; });
        n.left = (int32_t)g.bvh.size(); n.first = 0; n.count = 0;
        g.bvh[j.node] = n;
        g.bvh.push_back(Node()); g.bvh.push_back(Node());
        jobs.push_back({(uint32_t)n.left, j.first, mid - j.first});
        jobs.push_back({(uint32_t)n.left + 1, mid, j.first + j.count - mid});
    }
}

/* ------------------------------------------------------------------ RNG, sampling (math.glsl) */
static inline uint32_t hashU(uint32_t s) {                    /* hash2, math.glsl:227-234 */
    s = (s ^ 61u) ^ (s >> 16u);
    s *= 9u;
    s = s ^ (s >> 4u);
    s *= 0x27d4eb2du;
    return s ^ (s >> 15u);
}
static inline uint32_t pixelSeed(uint32_t seed, uint32_t x, uint32_t y) {   /* makeSeed, math.glsl:240-246 */
    return hashU((seed + x) ^ (y - 1u)) + hashU(y * (x - 2u));
}
static inline float rnd(uint32_t& st) { st = hashU(st); return (float)st / 4294967296.0f; }   /* sample1f, :252-254 */
static inline float lum(const F3& c) { return (c.x * 0.299f + c.y * 0.587f) + c.z * 0.114f; }
static inline float mis(float f, float g2) { return (f * f) / (f * f + g2 * g2); }

static F2 concentric(F2 v) {                                   /* toConcentricDisk, math.glsl:23-39 */
    if (v.x == 0.0f && v.y == 0.0f) return F2{0.0f, 0.0f};
    float x = v.x * 2.0f - 1.0f, y = v.y * 2.0f - 1.0f, r, phi;
    if (x * x > y * y) { r = x; phi = PI * y / x * 0.25f; }
    else { r = y; phi = PI * 0.5f - PI * x / y * 0.25f; }
    float s, c;
    oracle_det_sincosf(phi, &s, &c);
    return F2{r * c, r * s};
}
struct Frame3 { F3 t, b, n; };
static Frame3 frameOf(const F3& n) {                          /* matLocalToWorld, math.glsl:69-78 */
    F3 t = fabsf(n.z) > 0.999f ? F3(0.0f, 1.0f, 0.0f) : F3(0.0f, 0.0f, 1.0f);
    F3 b = unit(cross(n, t));
    return Frame3{cross(b, n), b, n};
}
static inline F3 apply(const Frame3& f, const F3& v) { return (f.t * v.x + f.b * v.y) + f.n * v.z; }
static F3 cosineHemisphere(const F3& n, F2 u) {                /* math.glsl:85-89 */
    F2 d = concentric(u);
    float z = sqrtf(1.0f - (d.x * d.x + d.y * d.y));
    return unit(apply(frameOf(n), F3(d.x, d.y, z)));
}

/* ------------------------------------------------------------------ BSDFs (material.glsl) */
enum : uint32_t { DIFFUSE = 1, GLOSSY = 2, SPECULAR = 4, REFLECTION = 16, TRANSMISSION = 32, BAD_SAMPLE = 0x80000000u };
enum : uint32_t { LAMBERT = 1, METALLIC_WF = 2, METAL = 3, DIELECTRIC = 4, FAKE = 6 };
struct Lobe { F3 wi; float pdf; F3 f; uint32_t type; };

static inline float p5(float x) { float x2 = x * x; return x2 * x2 * x; }
static inline float schlickScalar(float c, float ior) { float f0 = fabsf(1.0f - ior) / (1.0f + ior); float t = p5(1.0f - c); return f0 * (1.0f - t) + 1.0f * t; }
static inline F3 schlickColor(float c, const F3& f0) { return lerp3(f0, F3(1.0f), p5(1.0f - c)); }
static inline float gSchlick(float c, float alpha) { float a = alpha * 0.5f; return c / (c * (1.0f - a) + a); }
static inline float gSmith(float co, float ci, float alpha) { return gSchlick(fabsf(co), alpha) * gSchlick(fabsf(ci), alpha); }
static inline float dGTR2(float c, float alpha) {
    if (c < 1e-6f) return 0.0f;
    float aa = alpha * alpha;
    float den = c * c * (aa - 1.0f) + 1.0f;
    den = den * den * PI;
    return aa / den;
}
static inline float pdfGTR2(const F3& n, const F3& m, const F3& wo, float alpha) {
    return dGTR2(dot(n, m), alpha) * gSchlick(dot(n, wo), alpha) * fabsf(dot(m, wo)) / fabsf(dot(n, wo));
}
static F3 sampleGTR2(const F3& n, const F3& wo, float alpha, F2 r) {   /* GTR2Sample, material.glsl:84-101 */
    Frame3 f = frameOf(n);
    /* inverse(mat3(t, b, n)): rows cross(b,n), cross(n,t), cross(t,b) over det */
    F3 r0 = cross(f.b, f.n), r1 = cross(f.n, f.t), r2 = cross(f.t, f.b);
    float id = 1.0f / dot(f.t, r0);
    F3 c0(r0.x * id, r1.x * id, r2.x * id), c1(r0.y * id, r1.y * id, r2.y * id), c2(r0.z * id, r1.z * id, r2.z * id);
    F3 local = (c0 * wo.x + c1 * wo.y) + c2 * wo.z;
    F3 vh = unit(local * F3(alpha, alpha, 1.0f));
    float l2 = vh.x * vh.x + vh.y * vh.y;
    F3 t1 = l2 > 0.0f ? F3(-vh.y, vh.x, 0.0f) / sqrtf(l2) : F3(1.0f, 0.0f, 0.0f);
    F3 t2 = cross(vh, t1);
    F2 p = concentric(r);
    float s = 0.5f * (vh.z + 1.0f);
    p.y = (1.0f - s) * sqrtf(1.0f - p.x * p.x) + s * p.y;
    F3 h = t1 * p.x + t2 * p.y + vh * sqrtf(fmx(0.0f, 1.0f - (p.x * p.x + p.y * p.y)));
    h = F3(h.x * alpha, h.y * alpha, fmx(0.0f, h.z));
    return unit(apply(f, h));
}
static inline F3 mirror(const F3& i, const F3& n) { return i - n * (2.0f * dot(n, i)); }

static F3 fMetallic(const Material& m, const F3& alb, const F3& n, const F3& wo, const F3& wi) {
    float alpha = m.roughness * m.roughness;
    F3 h = unit(wo + wi);
    float co = dot(n, wo), ci = dot(n, wi);
    if (ci * co < 1e-7f) return F3(0.0f);
    F3 F = schlickColor(dot(h, wo), lerp3(F3(0.08f), alb, m.metallic));
    float G = gSmith(co, ci, alpha), D = dGTR2(dot(n, h), alpha);
    F3 diff = alb * INV_PI * (1.0f - m.metallic), spec(G * D / (4.0f * ci * co));
    return diff * (F3(1.0f) - F) + spec * F;
}
static float pdfMetallic(const Material& m, const F3& n, const F3& wo, const F3& wi) {
    F3 h = unit(wo + wi);
    float a = fmx(dot(n, wi), 0.0f) * INV_PI;
    float b = pdfGTR2(n, h, wo, m.roughness * m.roughness) / (4.0f * fabsf(dot(h, wo)));
    float t = 1.0f / (2.0f - m.metallic);
    return a * (1.0f - t) + b * t;
}
static F3 fMetal(const Material& m, const F3& alb, const F3& n, const F3& wo, const F3& wi) {
    if (m.roughness < 0.01f) return F3(0.0f);
    float alpha = m.roughness * m.roughness;
    F3 h = unit(wo + wi);
    float co = dot(n, wo), ci = dot(n, wi);
    if (ci * co < 1e-7f) return F3(0.0f);
    float F = schlickScalar(fabsf(dot(h, wo)), m.ior);
    float G = gSmith(co, ci, alpha), D = dGTR2(dot(n, h), alpha);
    return alb * F * G * D / (4.0f * ci * co);
}
static float pdfMetal(const Material& m, const F3& n, const F3& wo, const F3& wi) {
    if (m.roughness < 0.01f) return 0.0f;
    F3 h = unit(wo + wi);
    return pdfGTR2(n, h, wo, m.roughness * m.roughness) / (4.0f * fabsf(dot(h, wo)));
}
static F3 bsdfEval(const Material& m, const F3& alb, const F3& n, const F3& wo, const F3& wi) {
    if (m.type == LAMBERT) return alb * INV_PI;
    if (m.type == METALLIC_WF) return fMetallic(m, alb, n, wo, wi);
    if (m.type == METAL) return fMetal(m, alb, n, wo, wi);
    return F3(0.0f);
}
static float bsdfPdf(const Material& m, const F3& n, const F3& wo, const F3& wi) {
    if (m.type == LAMBERT) return fabsf(dot(n, wi)) * INV_PI;
    if (m.type == METALLIC_WF) return pdfMetallic(m, n, wo, wi);
    if (m.type == METAL) return pdfMetal(m, n, wo, wi);
    return 0.0f;
}
static bool bsdfSample(const Material& m, const F3& alb, const F3& n, const F3& wo, const F3& r, Lobe& s) {
    if (m.type == LAMBERT) {
        s.wi = cosineHemisphere(n, F2{r.x, r.y});
        s.pdf = fabsf(dot(n, s.wi)) * INV_PI;
        s.f = alb * INV_PI;
        s.type = DIFFUSE | REFLECTION;
        return true;
    }
    if (m.type == METALLIC_WF) {
        float alpha = m.roughness * m.roughness;
        s.type = REFLECTION;
        if (r.z > (1.0f / (2.0f - m.metallic))) { s.wi = cosineHemisphere(n, F2{r.x, r.y}); s.type |= DIFFUSE; }
        else { s.wi = -mirror(wo, sampleGTR2(n, wo, alpha, F2{r.x, r.y})); s.type |= (m.roughness < 0.01f) ? SPECULAR : GLOSSY; }
        if (dot(n, s.wi) < 0.0f) { s.type = BAD_SAMPLE; return false; }
        s.f = fMetallic(m, alb, n, wo, s.wi);
        s.pdf = pdfMetallic(m, n, wo, s.wi);
        return true;
    }
    if (m.type == METAL) {
        bool delta = m.roughness < 0.01f;
        s.wi = delta ? -mirror(wo, n) : -mirror(wo, sampleGTR2(n, wo, m.roughness * m.roughness, F2{r.x, r.y}));
        if (dot(n, s.wi) < 0.0f) { s.type = BAD_SAMPLE; return false; }
        s.f = delta ? alb * schlickScalar(fabsf(dot(n, wo)), m.ior) : fMetal(m, alb, n, wo, s.wi);
        s.pdf = delta ? 1.0f : pdfMetal(m, n, wo, s.wi);
        s.type = REFLECTION | (delta ? SPECULAR : GLOSSY);
        return true;
    }
    if (m.type == DIELECTRIC) {
        float pr = schlickScalar(dot(n, wo), m.ior);
        s.f = alb;
        if (r.z < pr) { s.wi = mirror(-wo, n); s.type = SPECULAR | REFLECTION; s.pdf = 1.0f; return true; }
        float ci = dot(n, wo), ior = m.ior;
        if (ci < 0.0f) ior = 1.0f / ior;
        float s2i = fmx(0.0f, 1.0f - ci * ci), s2t = s2i / (ior * ior);
        if (s2t >= 1.0f) { s.type = BAD_SAMPLE; return false; }
        float ct = sqrtf(1.0f - s2t);
        if (ci < 0.0f) ct = -ct;
        s.wi = unit(-wo / ior + n * (ci / ior - ct));
        float ior2 = m.ior;
        if (dot(n, wo) < 0.0f) ior2 = 1.0f / ior2;
        s.f = s.f / (ior2 * ior2);
        s.type = SPECULAR | TRANSMISSION;
        s.pdf = 1.0f;
        return true;
    }
    if (m.type == FAKE) { s.wi = -wo; s.f = alb; s.pdf = 1.0f; s.type = SPECULAR | TRANSMISSION; return true; }
    return false;
}
static inline bool deltaBsdf(const Material& m) {
    if (m.type == LAMBERT) return false;
    if (m.type == METALLIC_WF) return m.roughness < 0.01f && m.metallic > 0.9f;
    if (m.type == METAL) return m.roughness < 0.01f;
    return true;
}
static inline bool connectibleBsdf(const Material& m) {
    if (m.type == LAMBERT) return true;
    if (m.type == METALLIC_WF) return m.roughness > 0.05f || m.metallic < 0.9f;
    if (m.type == METAL) return m.roughness > 0.05f;
    return false;
}

/* ------------------------------------------------------------------ surfaces, lights, camera */
struct Surface { F3 p, n, albedo; uint32_t mat; bool light; };

static inline F3 xformPoint(const float* M, const F3& p) {
    F3 c0(M[0], M[1], M[2]), c1(M[4], M[5], M[6]), c2(M[8], M[9], M[10]), c3(M[12], M[13], M[14]);
    return ((c0 * p.x + c1 * p.y) + c2 * p.z) + c3 * 1.0f;
}

/* loadSurfaceInfo (ray_layouts.glsl:50-104); a light hit keeps s.mat. */
static void fetchSurface(const Hit& h, Surface& s) {
    F3 b(1.0f - h.bx - h.by, h.bx, h.by);
    if (h.inst == 0) {
        TriLight L = at(g.lights, h.tri);
        s.p = ld3(L.v0) * b.x + ld3(L.v1) * b.y + ld3(L.v2) * b.z;
        s.n = F3(L.nx, L.ny, L.nz);
        s.albedo = ld3(L.rad);
        s.light = true;
        return;
    }
    Instance I = at(g.instances, (uint64_t)h.inst - 1u);
    s.mat = (uint32_t)at(g.matIndices, (uint64_t)(uint32_t)(I.indexOffset / 3u + h.tri));
    uint32_t base = I.indexOffset + h.tri * 3u;
    Vertex a = at(g.vertices, at(g.indices, base)), bb = at(g.vertices, at(g.indices, base + 1u)),
           c = at(g.vertices, at(g.indices, base + 2u));
    F3 p = ld3(a.pos) * b.x + ld3(bb.pos) * b.y + ld3(c.pos) * b.z;
    F3 n = ld3(a.nrm) * b.x + ld3(bb.nrm) * b.y + ld3(c.nrm) * b.z;
    s.p = xformPoint(I.M, p);
    s.n = unit(xformPoint(I.MinvT, n));
    s.albedo = ld3(at(g.materials, s.mat).base);
    s.light = false;
}

/* sampleLightByPower + sampleTriangleLight (light_sampling.glsl:6-37) */
static F3 sampleLight(const F3& ref, const float r[4], F3& wi, float& dist, float& pdf, float& jac, F2& bary, uint32_t& id) {
    TableEntry t0 = at(g.table, 0);
    id = (uint32_t)((float)t0.failId * r[0]);
    TableEntry e = at(g.table, (uint64_t)id + 1u);
    id = (r[1] < e.prob) ? id : e.failId - 1u;
    TriLight L = at(g.lights, id);
    float sq = sqrtf(r[3]);
    bary = F2{1.0f - sq, r[2] * sq};
    F3 pos = ld3(L.v0) * (1.0f - bary.x - bary.y) + ld3(L.v1) * bary.x + ld3(L.v2) * bary.y;
    dist = len(ref - pos);
    F3 n(L.nx, L.ny, L.nz);
    wi = (pos - ref) / dist;
    jac = fabsf(dot(n, wi)) / (dist * dist);
    pdf = 1.0f / jac / L.area;
    F3 radiance = dot(n, wi) > 0.0f ? F3(0.0f) : ld3(L.rad);
    pdf *= lum(ld3(L.rad)) * L.area / t0.prob;
    return radiance;
}

struct Ray { F3 o, d; };
static Ray cameraRay(const Camera& c, F2 uv) {                 /* pinholeCameraSampleRay, camera.glsl:28-42 */
    float tx = 1.0f / (float)c.film[0], ty = 1.0f / (float)c.film[1];
    float bx = uv.x + tx * 0.0f, by = uv.y + ty * 0.0f;
    float nx = bx * 2.0f - 1.0f, ny = by * 2.0f - 1.0f;
    float aspect = (float)c.film[0] / (float)c.film[1];
    float tf = oracle_det_tanf(c.fov * 0.5f * 0.01745329251994329577f);
    F3 d = unit(F3(nx * aspect * tf, ny * 1.0f * tf, 1.0f));
    d = unit(ld3(c.right) * d.x + ld3(c.up) * d.y + ld3(c.front) * d.z);
    return Ray{ld3(c.pos), d};
}

/* ------------------------------------------------------------------ G-buffer access */
struct GBuf { const float* dn; const uint32_t* am; int w, h; };
static inline void texelDN(const GBuf& b, int x, int y, float o[4]) {
    if (x < 0 || y < 0 || x >= b.w || y >= b.h) { o[0] = o[1] = o[2] = o[3] = 0.0f; return; }
    const float* p = b.dn + ((size_t)y * b.w + x) * 4;
    o[0] = p[0]; o[1] = p[1]; o[2] = p[2]; o[3] = p[3];
}
static inline int wrapIdx(int i, int n) { int r = i % n; return r < 0 ? r + n : r; }
static void sampleDN(const GBuf& b, F2 uv, float out[4]) {     /* texture(): bilinear / repeat / 8-bit weights */
    float x = uv.x * (float)b.w - 0.5f, y = uv.y * (float)b.h - 0.5f;
    float fx = floorf(x), fy = floorf(y);
    float qx = floorf((x - fx) * 256.0f + 0.5f), qy = floorf((y - fy) * 256.0f + 0.5f);
    int ix = (int)fx, iy = (int)fy;
    if (qx >= 256.0f) { ix += 1; qx = 0.0f; }
    if (qy >= 256.0f) { iy += 1; qy = 0.0f; }
    float wx = qx * 0.00390625f, wy = qy * 0.00390625f;
    float a[4], bb[4], c[4], d[4];
    texelDN(b, wrapIdx(ix, b.w), wrapIdx(iy, b.h), a);
    texelDN(b, wrapIdx(ix + 1, b.w), wrapIdx(iy, b.h), bb);
    texelDN(b, wrapIdx(ix, b.w), wrapIdx(iy + 1, b.h), c);
    texelDN(b, wrapIdx(ix + 1, b.w), wrapIdx(iy + 1, b.h), d);
    for (int k = 0; k < 4; k++) {
        float top = a[k] * (1.0f - wx) + bb[k] * wx;
        float bot = c[k] * (1.0f - wx) + d[k] * wx;
        out[k] = top * (1.0f - wy) + bot * wy;
    }
}
static inline void fetchAM(const GBuf& b, int x, int y, uint32_t o[2]) {
    if (x < 0 || y < 0 || x >= b.w || y >= b.h) { o[0] = o[1] = 0; return; }
    o[0] = b.am[((size_t)y * b.w + x) * 2]; o[1] = b.am[((size_t)y * b.w + x) * 2 + 1];
}
/* unpackGBuffer (gbuffer_util.glsl:24-35) */
static bool decodeGBuffer(const float dn[4], const uint32_t am[2], float& depth, F3& n, F3& albedo, int& matMesh) {
    depth = dn[0];
    if (depth == 0.0f) return false;
    n = F3(dn[1], dn[2], dn[3]);
    albedo = F3((float)(am[0] & 0xffu) / 255.0f, (float)((am[0] >> 8) & 0xffu) / 255.0f, (float)((am[0] >> 16) & 0xffu) / 255.0f);
    matMesh = (int)am[1];
    return true;
}

static uint16_t toHalf(float f) {                               /* IEEE binary16, round to nearest even */
    uint32_t x; memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u, ex = (x >> 23) & 0xffu, mant = x & 0x7fffffu;
    if (ex == 0xffu) return (uint16_t)(sign | 0x7c00u | (mant ? (0x200u | (mant >> 13)) : 0u));
    int e = (int)ex - 112;
    if (e >= 31) return (uint16_t)(sign | 0x7c00u);
    if (e <= 0) {
        if (e < -10) return (uint16_t)sign;
        mant |= 0x800000u;
        int sh = 14 - e;
        uint32_t hm = mant >> sh, rem = mant & ((1u << sh) - 1u), half = 1u << (sh - 1);
        if (rem > half || (rem == half && (hm & 1u))) hm++;
        return (uint16_t)(sign | hm);
    }
    uint32_t hm = mant >> 13, rem = mant & 0x1fffu, h = sign | ((uint32_t)e << 10) | hm;
    if (rem > 0x1000u || (rem == 0x1000u && (hm & 1u))) h++;
    return (uint16_t)h;
}
static float fromHalf(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16, ex = (h >> 10) & 0x1fu, mant = h & 0x3ffu, x;
    if (ex == 0) {
        if (mant == 0) x = sign;
        else { int e = -1; do { mant <<= 1; e++; } while (!(mant & 0x400u)); x = sign | ((uint32_t)(112 - e) << 23) | ((mant & 0x3ffu) << 13); }
    } else if (ex == 31) x = sign | 0x7f800000u | (mant << 13);
    else x = sign | ((ex + 112) << 23) | (mant << 13);
    float f; memcpy(&f, &x, 4); return f;
}

/* ------------------------------------------------------------------ reservoirs (gris_reservoir.glsl) */
static inline uint32_t rcId(uint32_t f) { return f & 0xffu; }
static inline uint32_t rcType(uint32_t f) { return (f >> 16) & 0xffu; }
static inline void setField(uint32_t& f, int shift, uint32_t v) { f = (f & ~(0xffu << shift)) | ((v & 0xffu) << shift); }
static inline bool usable(const Reservoir& r) { return !std::isnan(r.W) && r.W >= 0.0f; }
static inline void clearResv(Reservoir& r) { r.s.rc.inst = NO_HIT; r.M = 0.0f; r.W = 0.0f; }

struct Pass {
    Camera cam, prev;
    Settings set;
    GBuf cur, old;
    std::vector<float> motion;
    Reservoir *self, *previous, *temp;
    uint64_t n;
    int W, H;
};

/* replay of the source path's random numbers from the destination primary hit up to the
 * vertex before the reconnection vertex (traceReplayPathForHybridShift, gris_retrace.glsl:42-136) */
struct Replay { Hit prevHit; F3 prevWo, prevThroughput; };
static void replay(const Pass& P, Hit hit, Surface surf, Ray ray, uint32_t flags, uint32_t rng, Replay& out) {
    F3 thr(1.0f), wo = -ray.d;
    Material mat = at(g.materials, surf.mat);
    Lobe s; memset(&s, 0, sizeof(s));
    out.prevThroughput = F3(0.0f);
    out.prevHit.inst = NO_HIT;
    uint32_t target = rcId(flags);
    if (target == 1u) { out.prevHit = hit; out.prevWo = wo; out.prevThroughput = thr; return; }
    for (int bounce = 0; bounce < (int)P.set.maxDepth; bounce++) {
        if (bounce > 0) {
            __atomic_fetch_add(&g_counts[0], 1ull, __ATOMIC_RELAXED);
            if (!traceQuery(ray.o, ray.d, RAY_TMIN, RAY_TMAX, false, false, &hit, nullptr)) break;
            fetchSurface(hit, surf);
            mat = at(g.materials, surf.mat);
        }
        bool conn = connectibleBsdf(mat);
        rnd(rng);
        if (surf.light) break;
        if ((uint32_t)bounce == target - 1u) {
            if (conn) { out.prevHit = hit; out.prevWo = wo; out.prevThroughput = thr; }
            break;
        }
        for (int k = 0; k < 5; k++) rnd(rng);   /* the light sample (4) and the reservoir draw (1) of the path tracer */
        if (bounce > 4) {
            float term = fmx(1.0f - lum(thr) * P.set.rrScale, 0.0f);
            if (rnd(rng) < term) break;
            thr = thr / (1.0f - term);
        }
        float r3[3];
        for (int k = 0; k < 3; k++) r3[k] = rnd(rng);
        if (!bsdfSample(mat, surf.albedo, surf.n, wo, F3(r3[0], r3[1], r3[2]), s) || s.pdf < 1e-6f) break;
        float cosT = (s.type & SPECULAR) == SPECULAR ? 1.0f : fabsf(dot(surf.n, s.wi));
        thr = thr * (s.f * cosT / s.pdf);
        wo = -s.wi;
        ray.d = s.wi;
        ray.o = surf.p + ray.d * 1e-4f;
    }
}

static inline bool visible(const F3& a, const F3& b) {         /* traceVisibility, ray_query.glsl:29-39 */
    __atomic_fetch_add(&g_counts[1], 1ull, __ATOMIC_RELAXED);
    return !traceQuery(a, unit(b - a), RAY_TMIN, len(b - a) - RAY_TMIN, true, false, nullptr, nullptr);
}

/* The shift of the hybrid mapping (gris_retrace.glsl:138-224): replay of the source's prefix from
 * the destination's primary vertex, reconnection with one visibility ray, and the shifted sample
 * (its F, Jacobian and pdf at the destination). srcPHat: the target of the unshifted sample. */
struct Shifted { bool valid; float dstPHat, srcPHat; PathSample out; };
static Shifted shiftSample(const Pass& P, const Surface& dstSurf, const Hit& dstHit, const Ray& primary, PathSample ps) {
    Replay rd; memset(&rd, 0, sizeof(rd));
    Surface prevS; memset(&prevS, 0, sizeof(prevS));
    Surface rcS; memset(&rcS, 0, sizeof(rcS));
    Material rcMat, prevMat; memset(&rcMat, 0, sizeof(rcMat)); memset(&prevMat, 0, sizeof(prevMat));
    F3 wi, Li;
    bool ok = false;
    float dstJac = 0.0f, jac = 0.0f, pHat = 0.0f, dstPdf = 0.0f;
    if (ps.rc.inst != NO_HIT) {
        replay(P, dstHit, dstSurf, primary, ps.flags, ps.primaryRng, rd);
        if (rd.prevHit.inst != NO_HIT) {
            if (rd.prevHit.inst == PRIMARY_HIT) prevS = dstSurf; else fetchSurface(rd.prevHit, prevS);
            fetchSurface(ps.rc, rcS);
            rcMat = at(g.materials, rcS.mat);
            prevMat = at(g.materials, prevS.mat);
            float dist = len(prevS.p - rcS.p);
            wi = unit(rcS.p - prevS.p);
            float cosT = -dot(rcS.n, wi);
            dstJac = fabsf(cosT) / (dist * dist);
            jac = dstJac / ps.rcJacobian;
            if (dist > 0.01f && cosT > 0.0f && !std::isnan(jac) && ps.rcJacobian > 0.0f && connectibleBsdf(prevMat))
                ok = visible(prevS.p, rcS.p);
        }
    }
    Shifted r;
    r.valid = ok;
    r.dstPHat = 0.0f;
    r.srcPHat = lum(ld3(ps.F));
    if (ok) {
        uint32_t type = rcType(ps.flags);
        if (!std::isnan(ps.rcPrevSamplePdf) && ps.rcPrevSamplePdf > 1e-6f) {
            Li = ld3(ps.rcLi);
            F3 rcWi = ld3(ps.rcWi);
            if (type == 2u && len(rcWi) > 0.5f) Li = Li * (bsdfEval(rcMat, rcS.albedo, rcS.n, -wi, rcWi) * fmx(dot(rcS.n, rcWi), 0.0f));
            Li = Li * (bsdfEval(prevMat, prevS.albedo, prevS.n, rd.prevWo, wi) * fmx(dot(prevS.n, wi), 0.0f));
            Li = Li * rd.prevThroughput;
            Li = Li / ps.rcPrevSamplePdf;
            if (!(lum(Li) < 1e-5f) && !anyNan(Li)) pHat = lum(Li * jac);
            if (type == 0u) dstPdf = lum(rcS.albedo) / at(g.table, 0).prob / dstJac;
            else dstPdf = bsdfPdf(prevMat, prevS.n, rd.prevWo, wi);
        } else {
            Li = F3(0.0f);
        }
        ps.rcJacobian = dstJac;
        ps.rcPrevSamplePdf = (dstPdf < 1e-6f || std::isnan(dstPdf)) ? 0.0f : dstPdf;
        st3(ps.F, Li);
        r.dstPHat = pHat;
    }
    r.out = ps;
    return r;
}

/* GRISReservoirReuseAndMerge (gris_retrace.glsl:138-236): the shift, the source weight scaled by
 * the ratio of the targets, the merge (M adds up), the M cap. */
static void shiftAndMerge(const Pass& P, Reservoir& dst, const Surface& dstSurf, const Hit& dstHit, const Ray& primary,
                          Reservoir src, uint32_t& rng) {
    Shifted sh = shiftSample(P, dstSurf, dstHit, primary, src.s);
    if (sh.valid) {
        src.s = sh.out;
        src.W *= sh.dstPHat / sh.srcPHat;
    } else {
        src.W = 0.0f;
    }
    if (usable(src)) {
        float r = rnd(rng);
        dst.M += src.M;
        dst.W += src.W;
        if (r * dst.W < src.W) dst.s = src.s;
    }
    float cap = (float)P.set.cap;
    if (dst.M > cap) { dst.W *= cap / dst.M; dst.M = cap; }
}

/* Pairwise generalised balance heuristic (GrisSettings.misWeights = 1, an extension of the
 * reference): the canonical reservoir c and k reused reservoirs i; pair i weighs technique i
 * against a 1/k share of the canonical one, m_i(y) = M_i p_i(y) / (M_i p_i(y) + (M_c / k) p_c(y)),
 * with p_i the target of y shifted into i's pixel times that shift's Jacobian. A reused sample's
 * weight comes from its forward shift; the canonical sample's from the backward shift of it into
 * every reused pixel (pBack). The merged reservoir keeps the reference's representation
 * (resampleWeight = sum w * M, M = sum of the Ms). */
struct Pairwise {
    float Mc, pc, Rc, k, mcSum, wSum, M;
    PathSample canon, sel;
    void begin(const Reservoir& c, float kk) {
        Mc = c.M; pc = lum(ld3(c.s.F)); Rc = c.W; k = kk;
        mcSum = 0.0f; wSum = 0.0f; M = Mc;
        canon = c.s; sel = c.s;
    }
    void add(const Reservoir& src, const Shifted& fw, float pBack, float u) {
        const float Mi = src.M;
        if (pc > 0.0f) {
            float a = (Mc / k) * pc, b = Mi * pBack;
            mcSum += a / (a + b);
        }
        float w = 0.0f;
        if (fw.valid && fw.dstPHat > 0.0f && fw.srcPHat > 0.0f && Mi > 0.0f)
            w = (1.0f / k) * fw.dstPHat * src.W / (Mi * fw.srcPHat + (Mc / k) * fw.dstPHat);
        if (!(w >= 0.0f) || std::isinf(w)) w = 0.0f;
        wSum += w;
        if (u * wSum < w) sel = fw.out;
        M += Mi;
    }
    void skip() { if (pc > 0.0f) mcSum += 1.0f; }
    Reservoir finish(float u, float cap) {
        float wc = (pc > 0.0f && Mc > 0.0f) ? (mcSum / k) * Rc / Mc : 0.0f;
        if (!(wc >= 0.0f) || std::isinf(wc)) wc = 0.0f;
        float total = wSum + wc;
        Reservoir out; memset(&out, 0, sizeof(out));
        clearResv(out);
        out.s = (u * total < wc) ? canon : sel;
        out.M = M;
        out.W = total * M;
        if (out.M > cap) { out.W *= cap / out.M; out.M = cap; }
        return out;
    }
};

/* ------------------------------------------------------------------ passes */
static inline F2 pixelUV(int x, int y, int W, int H) { return F2{((float)x + 0.5f) / (float)W, ((float)y + 0.5f) / (float)H}; }

/* tracePath (gris_path_trace.glsl:45-306) */
static void pathTracePixel(Pass& P, int x, int y) {
    F2 uv = pixelUV(x, y, P.W, P.H);
    float dn[4]; uint32_t am[2];
    sampleDN(P.cur, uv, dn);
    fetchAM(P.cur, x, y, am);
    float depth; F3 nrm, alb; int matMesh;
    if (!decodeGBuffer(dn, am, depth, nrm, alb, matMesh)) return;
    Ray ray = cameraRay(P.cam, F2{uv.x, 1.0f - uv.y});
    uint32_t rng = pixelSeed(P.cam.seed, (uint32_t)x, (uint32_t)y);

    F3 thr(1.0f), rcThr(0.0f), wo = -ray.d, lastPos(0.0f);
    bool lastConn = false;
    uint32_t state = 0, lastState = 0;
    Surface surf; surf.p = ray.o + ray.d * (depth - 1e-4f); surf.n = nrm; surf.albedo = alb; surf.mat = 0; surf.light = false;
    Material mat = at(g.materials, (uint32_t)(matMesh >> 16));
    Lobe s; memset(&s, 0, sizeof(s));
    Hit hit; memset(&hit, 0, sizeof(hit));
    PathSample cand; memset(&cand, 0, sizeof(cand));
    cand.rc.inst = NO_HIT;
    cand.primaryRng = rng;
    PathSample chosen; memset(&chosen, 0, sizeof(chosen));
    float chosenW = 0.0f, wsum = 0.0f;
    auto stream = [&](float w, float r) { wsum += w; if (r * wsum < w) { chosenW = w; chosen = cand; } };

    for (int bounce = 0; bounce < (int)P.set.maxDepth; bounce++) {
        if (bounce > 0) {
            __atomic_fetch_add(&g_counts[0], 1ull, __ATOMIC_RELAXED);
            if (!traceQuery(ray.o, ray.d, RAY_TMIN, RAY_TMAX, false, false, &hit, nullptr)) break;
            fetchSurface(hit, surf);
            mat = at(g.materials, surf.mat);
        }
        setField(cand.flags, 8, (uint32_t)bounce + 1u);
        float cosPrev = dot(ray.d, surf.n);
        float dPrev = len(lastPos - surf.p);
        float gJac = fabsf(cosPrev) / (dPrev * dPrev);
        bool conn = surf.light || connectibleBsdf(mat);
        lastState = state;
        state = state == 2u ? 2u : (conn ? state + 1u : 0u);
        if (P.set.shift == 0u && bounce == 1 && !surf.light) { state = 2u; lastState = 1u; }
        float rResv = rnd(rng);
        if (surf.light) {
            if (bounce > 1 && cosPrev < 0.0f) {
                float w = 1.0f;
                float lightPdf = lum(surf.albedo) / at(g.table, 0).prob / gJac;
                if ((s.type & SPECULAR) != SPECULAR) w = mis(s.pdf, lightPdf);
                F3 Le = surf.albedo * w;
                if (state == 2u && lastState == 2u) {
                    st3(cand.rcLi, ld3(cand.rcLi) + Le * rcThr);
                    st3(cand.F, ld3(cand.F) + Le * thr);
                } else if (state == 2u && lastState == 1u && lastConn && dPrev > 0.01f) {
                    cand.rc = hit; cand.rcRng = rng; cand.rcPrevSamplePdf = s.pdf; cand.rcJacobian = gJac;
                    st3(cand.rcLi, Le); st3(cand.rcWi, F3(0.0f)); st3(cand.F, Le * thr);
                    setField(cand.flags, 0, (uint32_t)bounce);
                    setField(cand.flags, 16, 1u);
                    stream(lum(ld3(cand.F)), rResv);
                }
            }
            break;
        }
        bool reconnectable = conn && lastConn && dPrev > 0.01f;
        if (state == 2u && lastState == 1u && (reconnectable || P.set.shift == 0u)) {
            cand.rc = hit; cand.rcRng = rng; cand.rcPrevSamplePdf = s.pdf; cand.rcJacobian = gJac;
            setField(cand.flags, 0, (uint32_t)bounce);
            setField(cand.flags, 16, 2u);
            rcThr = F3(1.0f);
        }
        float rl[4];
        for (int k = 0; k < 4; k++) rl[k] = rnd(rng);
        rResv = rnd(rng);
        if (bounce > 0 && !deltaBsdf(mat)) {
            F3 ldir; F2 lbary; float ldist, lpdf, ljac; uint32_t lid;
            F3 Le = sampleLight(surf.p, rl, ldir, ldist, lpdf, ljac, lbary, lid);
            __atomic_fetch_add(&g_counts[1], 1ull, __ATOMIC_RELAXED);
            bool blocked = traceQuery(surf.p, ldir, RAY_TMIN, ldist - RAY_TMIN, true, false, nullptr, nullptr);
            if (!blocked && lpdf > 1e-6f) {
                float w = mis(lpdf, fabsf(dot(surf.n, ldir)) * INV_PI);
                F3 f = bsdfEval(mat, surf.albedo, surf.n, wo, ldir) * fmx(dot(surf.n, ldir), 0.0f);
                F3 wLe = Le / lpdf * w;
                if (state == 2u && lastState == 2u) {
                    st3(cand.rcLi, ld3(cand.rcLi) + wLe * f * rcThr);
                    st3(cand.F, ld3(cand.F) + wLe * f * thr);
                } else if (state == 2u && lastState == 1u) {
                    st3(cand.rcLi, wLe); st3(cand.rcWi, ldir); st3(cand.F, wLe * f * thr);
                    stream(lum(ld3(cand.F)), rResv);
                } else if (state == 1u && conn && ldist > 0.01f) {
                    cand.rc.bx = lbary.x; cand.rc.by = lbary.y; cand.rc.inst = 0u; cand.rc.tri = lid;
                    cand.rcRng = rng; cand.rcPrevSamplePdf = lpdf; cand.rcJacobian = ljac;
                    st3(cand.rcLi, Le * w); st3(cand.rcWi, F3(0.0f)); st3(cand.F, wLe * f * thr);
                    setField(cand.flags, 0, (uint32_t)bounce + 1u);
                    setField(cand.flags, 16, 0u);
                    stream(lum(ld3(cand.F)), rResv);
                }
            }
        }
        if (bounce > 4) {
            float term = fmx(1.0f - lum(thr) * P.set.rrScale, 0.0f);
            if (rnd(rng) < term) break;
            thr = thr / (1.0f - term);
            rcThr = rcThr / (1.0f - term);
        }
        float r3[3];
        for (int k = 0; k < 3; k++) r3[k] = rnd(rng);
        if (!bsdfSample(mat, surf.albedo, surf.n, wo, F3(r3[0], r3[1], r3[2]), s) || s.pdf < 1e-6f) break;
        float cosT = (s.type & SPECULAR) == SPECULAR ? 1.0f : fabsf(dot(surf.n, s.wi));
        F3 sc = s.f * cosT / s.pdf;
        thr = thr * sc;
        if (state == 2u && lastState == 2u) rcThr = rcThr * sc;
        else if (state == 2u && lastState == 1u) {
            st3(cand.rcLi, F3(0.0f)); st3(cand.rcWi, s.wi); st3(cand.F, F3(0.0f));
            rcThr = rcThr / s.pdf;
        }
        lastPos = surf.p;
        wo = -s.wi;
        ray.d = s.wi;
        ray.o = surf.p + ray.d * 1e-4f;
        lastConn = conn;
    }
    if (state == 2u && lastState == 2u) stream(lum(ld3(cand.F)), rnd(rng));

    Reservoir out; memset(&out, 0, sizeof(out));
    out.s = chosen;
    if (wsum > 0.0f && chosenW > 0.0f) {
        st3(out.s.F, ld3(out.s.F) * (wsum / chosenW));
        st3(out.s.rcLi, ld3(out.s.rcLi) * (wsum / chosenW));
        out.W = lum(ld3(out.s.F));
    } else {
        out.s.rc.inst = NO_HIT;
        st3(out.s.F, F3(0.0f));
    }
    out.M = 1.0f;
    P.self[(size_t)y * P.W + x] = out;
}

static inline Reservoir readResv(const Reservoir* buf, uint64_t i, uint64_t n) {
    if (i < n) return buf[i];
    Reservoir z; memset(&z, 0, sizeof(z)); return z;
}

/* temporalReuse (gris_resample_temporal.glsl:11-83) */
static void temporalPixel(Pass& P, int x, int y) {
    F2 uv = pixelUV(x, y, P.W, P.H);
    float dn[4]; uint32_t am[2];
    sampleDN(P.cur, uv, dn);
    fetchAM(P.cur, x, y, am);
    float depth; F3 nrm, alb; int matMesh;
    if (!decodeGBuffer(dn, am, depth, nrm, alb, matMesh)) return;
    size_t i = (size_t)y * P.W + x;
    F2 mv{P.motion[i * 2], P.motion[i * 2 + 1]};
    Ray ray = cameraRay(P.cam, F2{uv.x, 1.0f - uv.y});
    uint32_t resvRng = ~(pixelSeed(P.cam.seed, (uint32_t)x, (uint32_t)y) ^ 1u);
    F3 pos = ray.o + ray.d * (depth - 1e-4f);
    Reservoir r = P.self[i];
    Hit primary; primary.bx = uv.x; primary.by = uv.y; primary.inst = PRIMARY_HIT; primary.tri = 0;
    if (P.set.temporal && (P.cam.frameIndex & 0x80000000u) == 0u) {
        Surface ds; ds.p = pos; ds.n = nrm; ds.albedo = alb; ds.mat = (uint32_t)(matMesh >> 16); ds.light = false;
        F2 puv{uv.x + mv.x, uv.y + mv.y};
        if (!(puv.x < 0.0f || puv.y < 0.0f || puv.x > 1.0f || puv.y > 1.0f)) {
            int px = (int)(puv.x * (float)P.cam.film[0]), py = (int)(puv.y * (float)P.cam.film[1]);
            float pdn[4]; uint32_t pam[2];
            sampleDN(P.old, puv, pdn);
            fetchAM(P.old, px, py, pam);
            float pdepth; F3 pn, palb; int pmm;
            if (decodeGBuffer(pdn, pam, pdepth, pn, palb, pmm)) {
                Ray pr = cameraRay(P.prev, F2{puv.x, 1.0f - puv.y});
                F3 ppos = pr.o + pr.d * (pdepth - 1e-4f);
                if (!(pmm != matMesh || dot(pn, nrm) < 0.95f || len(pos - ppos) > 0.5f)) {
                    Reservoir src = readResv(P.previous, (uint64_t)(P.cam.film[0] * (uint32_t)py + (uint32_t)px), P.n);
                    if (usable(src) && P.set.misWeights) {
                        /* pairwise: the backward shift of the canonical sample into the previous pixel */
                        Surface ps; ps.p = ppos; ps.n = pn; ps.albedo = palb; ps.mat = (uint32_t)(pmm >> 16); ps.light = false;
                        Hit ph; ph.bx = puv.x; ph.by = puv.y; ph.inst = PRIMARY_HIT; ph.tri = 0;
                        Pairwise pw;
                        pw.begin(r, 1.0f);
                        Shifted fw = shiftSample(P, ds, primary, ray, src.s);
                        float pBack = 0.0f;
                        if (pw.pc > 0.0f) {
                            Shifted bw = shiftSample(P, ps, ph, pr, r.s);
                            if (bw.valid) pBack = bw.dstPHat;
                        }
                        float u0 = rnd(resvRng);
                        pw.add(src, fw, pBack, u0);
                        float u1 = rnd(resvRng);
                        r = pw.finish(u1, (float)P.set.cap);
                    } else if (usable(src)) {
                        shiftAndMerge(P, r, ds, primary, ray, src, resvRng);
                    }
                }
            }
        }
    }
    if (!usable(r)) clearResv(r);
    P.temp[i] = r;
}

/* spatialReuse + final shading (gris_resample_spatial.glsl:11-135); returns the pixel colour */
static F3 spatialPixel(Pass& P, int x, int y) {
    F2 uv = pixelUV(x, y, P.W, P.H);
    float dn[4]; uint32_t am[2];
    sampleDN(P.cur, uv, dn);
    fetchAM(P.cur, x, y, am);
    float depth; F3 nrm, alb; int matMesh;
    if (!decodeGBuffer(dn, am, depth, nrm, alb, matMesh)) return F3(0.0f);
    uint32_t rng = pixelSeed(P.cam.seed, (uint32_t)x, (uint32_t)y) ^ 2u;
    Ray ray = cameraRay(P.cam, F2{uv.x, 1.0f - uv.y});
    F3 pos = ray.o + ray.d * (depth - 1e-4f);
    size_t i = (size_t)y * P.W + x;
    Reservoir r = P.temp[i];
    Hit primary; primary.bx = uv.x; primary.by = uv.y; primary.inst = PRIMARY_HIT; primary.tri = 0;
    Surface ds; ds.p = pos; ds.n = nrm; ds.albedo = alb; ds.mat = (uint32_t)(matMesh >> 16); ds.light = false;
    if (P.set.spatial) {
        const bool pairwise = P.set.misWeights != 0u && P.set.neighbours > 0u;
        Pairwise pw;
        if (pairwise) pw.begin(r, (float)P.set.neighbours);
        float tx = 1.0f / (float)P.W, ty = 1.0f / (float)P.H;
        for (uint32_t k = 0; k < P.set.neighbours; k++) {
            float r0 = rnd(rng), r1 = rnd(rng);
            F2 d = concentric(F2{r0, r1});
            F2 nb{uv.x + d.x * P.set.radius * tx, uv.y + d.y * P.set.radius * ty};
            if (nb.x < 0.0f || nb.y < 0.0f || nb.x > 1.0f || nb.y > 1.0f) { if (pairwise) pw.skip(); continue; }
            int px = (int)(nb.x * (float)P.cam.film[0]), py = (int)(nb.y * (float)P.cam.film[1]);
            float ndn[4]; uint32_t nam[2];
            sampleDN(P.cur, nb, ndn);
            fetchAM(P.cur, px, py, nam);
            float ndepth; F3 nn, nalb; int nmm;
            if (!decodeGBuffer(ndn, nam, ndepth, nn, nalb, nmm)) { if (pairwise) pw.skip(); continue; }
            Ray nr = cameraRay(P.cam, F2{nb.x, 1.0f - nb.y});
            F3 npos = nr.o + nr.d * (ndepth - 1e-4f);
            if (dot(nn, nrm) < 0.9f || len(pos - npos) > 0.4f) { if (pairwise) pw.skip(); continue; }
            Reservoir src = readResv(P.temp, (uint64_t)(P.cam.film[0] * (uint32_t)py + (uint32_t)px), P.n);
            if (pairwise) {
                if (!usable(src)) { pw.skip(); continue; }
                Surface ns; ns.p = npos; ns.n = nn; ns.albedo = nalb; ns.mat = (uint32_t)(nmm >> 16); ns.light = false;
                Hit nh; nh.bx = nb.x; nh.by = nb.y; nh.inst = PRIMARY_HIT; nh.tri = 0;
                Shifted fw = shiftSample(P, ds, primary, ray, src.s);
                float pBack = 0.0f;
                if (pw.pc > 0.0f) {
                    Shifted bw = shiftSample(P, ns, nh, nr, pw.canon);
                    if (bw.valid) pBack = bw.dstPHat;
                }
                pw.add(src, fw, pBack, rnd(rng));
                continue;
            }
            if (usable(src)) shiftAndMerge(P, r, ds, primary, ray, src, rng);
        }
        if (pairwise) r = pw.finish(rnd(rng), (float)P.set.cap);
    }
    if (!usable(r)) clearResv(r);
    P.self[i] = r;
    F3 color(0.0f);
    if (usable(r) && r.M > 0.0f && r.s.rc.inst != NO_HIT) {
        Replay rd; memset(&rd, 0, sizeof(rd));
        replay(P, primary, ds, ray, r.s.flags, r.s.primaryRng, rd);
        if (rd.prevHit.inst != NO_HIT) {
            Surface prevS, rcS;
            memset(&prevS, 0, sizeof(prevS)); memset(&rcS, 0, sizeof(rcS));
            if (rd.prevHit.inst == PRIMARY_HIT) prevS = ds; else fetchSurface(rd.prevHit, prevS);
            fetchSurface(r.s.rc, rcS);
            Material rcMat = at(g.materials, rcS.mat), prevMat = at(g.materials, prevS.mat);
            F3 Li = ld3(r.s.rcLi), rcWi = ld3(r.s.rcWi);
            F3 wi = unit(rcS.p - prevS.p);
            if (rcType(r.s.flags) == 2u && len(rcWi) > 0.5f) Li = Li * (bsdfEval(rcMat, rcS.albedo, rcS.n, -wi, rcWi) * fmx(dot(rcS.n, rcWi), 0.0f));
            Li = Li * (bsdfEval(prevMat, prevS.albedo, prevS.n, rd.prevWo, wi) * fmx(dot(prevS.n, wi), 0.0f));
            Li = Li * rd.prevThroughput;
            Li = Li / r.s.rcPrevSamplePdf;
            if (!(lum(Li) < 1e-5f) && !anyNan(Li)) color = Li / lum(Li) * r.W / r.M;
        }
    }
    if (anyNan(color)) return F3(0.0f);
    return F3(fmn(fmx(color.x, 0.0f), 1e4f), fmn(fmx(color.y, 0.0f), 1e4f), fmn(fmx(color.z, 0.0f), 1e4f));
}

/* ================================================================== ReSTIR DI
 * Direct lighting at the primary vertex (TestReSTIR::render, src/TestReSTIR.cpp:9-35):
 * candidates (di_path_gen.glsl:9-62 with sampleLi, di_reservoir.glsl:78-174), temporal reuse
 * (di_temporal.glsl:36-90) and spatial reuse + shading (di_spatial.glsl:36-121). */
struct DISample { Hit isec; float Li[3]; float pad0; float jac, pdf; uint32_t rng, isLight; };   /* layouts.glsl:96-106 */
struct DIResv { DISample s; uint32_t M; float W, contrib, weight; };                           /* :108-115 */
struct DISettings { uint32_t shift, mode, temporal, spatial; };                                 /* TestReSTIR.h:12-17 */
static_assert(sizeof(DIResv) == 64, "DIReservoir layout");
enum : uint32_t { DI_LIGHT = 0, DI_BSDF = 1, DI_RECONNECT = 0, DI_REPLAY = 1 };
static const uint32_t DI_CAP = 40, DI_NEIGHBOURS = 10;
static const float DI_RADIUS = 20.0f;

static inline bool diUsable(const DIResv& r) { return !std::isnan(r.W); }                   /* di_reservoir.glsl:40-42 */
static inline void diClear(DIResv& r) { r.M = 0u; r.W = 0.0f; r.contrib = 0.0f; }          /* :34-38 */
static inline void diAdd(DIResv& r, const DISample& s, float w, float u) {                  /* :50-58 */
    r.W += w;
    r.M++;
    if (u * r.W < w) { r.s = s; r.weight = w; }
}
static inline void diMerge(DIResv& r, const DIResv& rhs, float u) {                         /* :60-68 */
    r.W += rhs.W;
    r.M += rhs.M;
    if (u * r.W < rhs.W) { r.s = rhs.s; r.weight = rhs.weight; }
}
static inline void diCap(DIResv& r, uint32_t cap) {                                         /* :70-75 */
    if (r.M > cap) { r.W *= (float)cap / (float)r.M; r.M = cap; }
}

/* sampleLi (di_reservoir.glsl:78-174): one light sample and/or one BSDF sample streamed into
 * `resv` (draws from resvRng), then the chosen sample's Li scaled by W / w, M = 1. */
static void diSampleLi(const Surface& surf, const Material& mat, const F3& wo, uint32_t rng, uint32_t& resvRng, DIResv& resv,
                       uint32_t mode) {
    DISample ps; memset(&ps, 0, sizeof(ps));
    ps.rng = rng;
    float lr[4], sr[3];
    for (int k = 0; k < 4; k++) lr[k] = rnd(rng);
    for (int k = 0; k < 3; k++) sr[k] = rnd(rng);
    if (mode != DI_BSDF && !deltaBsdf(mat)) {
        F3 wi; float dist, pdf, jac; F2 bary; uint32_t id;
        F3 Le = sampleLight(surf.p, lr, wi, dist, pdf, jac, bary, id);
        __atomic_fetch_add(&g_counts[1], 1ull, __ATOMIC_RELAXED);
        bool shadowed = traceQuery(surf.p, wi, RAY_TMIN, dist - RAY_TMIN, true, false, nullptr, nullptr);
        if (!shadowed && pdf > 1e-6f) {
            float w = mis(pdf, bsdfPdf(mat, surf.n, wo, wi));
            if (mode == DI_LIGHT) w = 1.0f;
            F3 contrib = Le * bsdfEval(mat, surf.albedo, surf.n, wo, wi) * fmx(dot(surf.n, wi), 0.0f) / pdf * w;
            float sw = lum(contrib);
            if (std::isnan(sw) || sw < 0.0f) sw = 0.0f;
            ps.isec.bx = bary.x; ps.isec.by = bary.y; ps.isec.inst = 0u; ps.isec.tri = id;
            st3(ps.Li, Le * w);
            ps.jac = jac; ps.pdf = pdf; ps.isLight = 1u;
            diAdd(resv, ps, sw, rnd(resvRng));
        }
    }
    ps.isLight = 0u;
    Lobe s; memset(&s, 0, sizeof(s));
    if (mode != DI_LIGHT && bsdfSample(mat, surf.albedo, surf.n, wo, F3(sr[0], sr[1], sr[2]), s) && s.pdf > 1e-6f) {
        __atomic_fetch_add(&g_counts[0], 1ull, __ATOMIC_RELAXED);
        Hit h;
        if (traceQuery(surf.p, s.wi, RAY_TMIN, RAY_TMAX, false, false, &h, nullptr)) {
            Surface hit; memset(&hit, 0, sizeof(hit));
            fetchSurface(h, hit);
            float cosT = -dot(s.wi, hit.n);
            if (hit.light && cosT > 0.0f) {
                float dist = len(hit.p - surf.p);
                float lightPdf = lum(hit.albedo) / at(g.table, 0).prob * dist * dist / fabsf(cosT);
                float w = mis(s.pdf, lightPdf);
                bool delta = (s.type & SPECULAR) == SPECULAR;
                if (mode == DI_BSDF || delta) w = 1.0f;
                float cosTerm = delta ? 1.0f : fmx(dot(surf.n, s.wi), 0.0f);
                F3 contrib = hit.albedo * s.f * cosTerm / s.pdf * w;
                ps.isec = h;
                st3(ps.Li, hit.albedo * w);
                ps.jac = fabsf(cosT) / (dist * dist); ps.pdf = s.pdf; ps.isLight = 0u;
                diAdd(resv, ps, lum(contrib), rnd(resvRng));   /* unclamped weight, as the reference */
            }
        }
    }
    if (!diUsable(resv)) diClear(resv);
    if (resv.M > 0u && resv.s.isec.inst != NO_HIT && resv.weight > 0.0f) {
        st3(resv.s.Li, ld3(resv.s.Li) * (resv.W / resv.weight));
        resv.weight = resv.W;
    } else {
        resv.s.isec.inst = NO_HIT;
        resv.weight = 0.0f;
        resv.W = 0.0f;
    }
    resv.M = 1u;
}

struct DIPass {
    Camera cam, prev;
    DISettings set;
    GBuf cur, old;
    std::vector<float> motion;
    DIResv *self, *previous, *temp;
    uint64_t n;
    int W, H;
};

static inline DIResv readDI(const DIResv* buf, uint64_t i, uint64_t n) {
    if (i < n) return buf[i];
    DIResv z; memset(&z, 0, sizeof(z)); return z;
}

/* randomReplay (di_reservoir.glsl:176-209): the source's candidates drawn again at the
 * destination from the source's seed; the reservoir draws come from the merge stream. */
static void diReplay(DIResv& dst, const Surface& ds, const DIResv& src, const F3& wo, uint32_t& rng, uint32_t mode) {
    Material mat = at(g.materials, ds.mat);
    DIResv rr; memset(&rr, 0, sizeof(rr));
    diClear(rr);
    diSampleLi(ds, mat, wo, src.s.rng, rng, rr, mode);
    if (rr.s.isec.inst != NO_HIT) {
        Surface rs; memset(&rs, 0, sizeof(rs));
        fetchSurface(rr.s.isec, rs);
        F3 wi = unit(rs.p - ds.p);
        F3 Li = ld3(rr.s.Li) * bsdfEval(mat, ds.albedo, ds.n, wo, wi) * fmx(dot(ds.n, wi), 0.0f) / rr.s.pdf;
        float pHat = lum(Li * 1.0f);
        rr.W = src.W * pHat / src.weight;
        rr.M = src.M;
    } else {
        rr.W = 0.0f;
    }
    if (diUsable(rr)) diMerge(dst, rr, rnd(rng));
}

/* reconnection (di_reservoir.glsl:211-287): the source's light vertex seen from the destination. */
static void diReconnect(DIResv& dst, const Surface& ds, DIResv src, const F3& wo, uint32_t& rng) {
    Material mat = at(g.materials, ds.mat);
    DISample ss = src.s;
    Surface rc; memset(&rc, 0, sizeof(rc));
    fetchSurface(ss.isec, rc);
    float dist = len(rc.p - ds.p);
    F3 wi = unit(rc.p - ds.p);
    float cosT = -dot(rc.n, wi);
    float dstJac = fabsf(cosT) / (dist * dist);
    float jac = dstJac / ss.jac;
    bool ok = false;
    float pHat = 0.0f, dstPdf = 0.0f;
    if (ss.isec.inst != NO_HIT && dist > 1e-4f) {
        if (cosT > 0.0f && !std::isnan(jac) && ss.jac > 0.0f) {
            if (visible(ds.p, rc.p)) {
                ok = true;
                if (!std::isnan(ss.pdf) && ss.pdf > 1e-6f) {
                    F3 Li = ld3(src.s.Li) * bsdfEval(mat, ds.albedo, ds.n, wo, wi) * fmx(dot(ds.n, wi), 0.0f) / ss.pdf;
                    pHat = lum(Li * jac);
                }
                if (ss.isLight) dstPdf = lum(rc.albedo) / at(g.table, 0).prob / dstJac;
                else dstPdf = bsdfPdf(mat, ds.n, wo, wi);
            }
        }
    }
    if (ok) {
        ss.jac = dstJac;
        ss.pdf = dstPdf;
        if (ss.pdf < 1e-6f || std::isnan(ss.pdf)) ss.pdf = 0.0f;
        src.s = ss;
        src.W *= pHat / src.weight;
        if (std::isnan(src.W)) src.W = 0.0f;
    } else {
        src.W = 0.0f;
    }
    if (diUsable(src)) diMerge(dst, src, rnd(rng));
}

static void diReuse(const DIPass& P, DIResv& dst, const Surface& ds, const DIResv& src, const F3& wo, uint32_t& rng) {
    if (P.set.shift == DI_RECONNECT) diReconnect(dst, ds, src, wo, rng);           /* di_reservoir.glsl:289-296 */
    else if (P.set.shift == DI_REPLAY) diReplay(dst, ds, src, wo, rng, P.set.mode);
}

/* generatePath (di_path_gen.glsl:9-40): candidates at the primary vertex; the returned colour
 * is never stored (di_path_gen.comp:14-26). */
static void diGenPixel(DIPass& P, int x, int y) {
    F2 uv = pixelUV(x, y, P.W, P.H);
    float dn[4]; uint32_t am[2];
    sampleDN(P.cur, uv, dn);
    fetchAM(P.cur, x, y, am);
    float depth; F3 nrm, alb; int matMesh;
    if (!decodeGBuffer(dn, am, depth, nrm, alb, matMesh)) return;
    Ray ray = cameraRay(P.cam, F2{uv.x, 1.0f - uv.y});
    uint32_t rng = pixelSeed(P.cam.seed, (uint32_t)x, (uint32_t)y);
    uint32_t resvRng = ~rng;
    Surface s; s.p = ray.o + ray.d * (depth - 1e-4f); s.n = nrm; s.albedo = alb; s.mat = (uint32_t)(matMesh >> 16); s.light = false;
    DIResv r; memset(&r, 0, sizeof(r));
    diClear(r);
    diSampleLi(s, at(g.materials, s.mat), -ray.d, rng, resvRng, r, P.set.mode);
    P.self[(size_t)y * P.W + x] = r;
}

/* The final-sample visibility test of both reuse passes (di_temporal.glsl:76-85, di_spatial.glsl:84-93). */
static inline void diOcclude(DIResv& r, const F3& pos) {
    if (diUsable(r) && r.s.isec.inst != NO_HIT) {
        Surface s; memset(&s, 0, sizeof(s));
        fetchSurface(r.s.isec, s);
        if (!visible(pos, s.p)) r.W = 0.0f;
    }
}

/* temporalReuse + findPreviousReservoir (di_temporal.glsl:9-90) */
static void diTemporalPixel(DIPass& P, int x, int y) {
    F2 uv = pixelUV(x, y, P.W, P.H);
    float dn[4]; uint32_t am[2];
    sampleDN(P.cur, uv, dn);
    fetchAM(P.cur, x, y, am);
    float depth; F3 nrm, alb; int matMesh;
    if (!decodeGBuffer(dn, am, depth, nrm, alb, matMesh)) return;
    size_t i = (size_t)y * P.W + x;
    F2 mv{P.motion[i * 2], P.motion[i * 2 + 1]};
    Ray ray = cameraRay(P.cam, F2{uv.x, 1.0f - uv.y});
    uint32_t resvRng = ~(pixelSeed(P.cam.seed, (uint32_t)x, (uint32_t)y) ^ 1u);
    F3 pos = ray.o + ray.d * (depth - 1e-4f);
    DIResv r = P.self[i];
    if (P.set.temporal) {
        Surface ds; ds.p = pos; ds.n = nrm; ds.albedo = alb; ds.mat = (uint32_t)(matMesh >> 16); ds.light = false;
        F2 puv{uv.x + mv.x, uv.y + mv.y};
        if ((P.cam.frameIndex & 0x80000000u) == 0u && !(puv.x < 0.0f || puv.y < 0.0f || puv.x > 1.0f || puv.y > 1.0f)) {
            int px = (int)(puv.x * (float)P.cam.film[0]), py = (int)(puv.y * (float)P.cam.film[1]);
            float pdn[4]; uint32_t pam[2];
            sampleDN(P.old, puv, pdn);
            fetchAM(P.old, px, py, pam);
            float pdepth; F3 pn, palb; int pmm;
            if (decodeGBuffer(pdn, pam, pdepth, pn, palb, pmm)) {
                Ray pr = cameraRay(P.prev, F2{puv.x, 1.0f - puv.y});
                F3 ppos = pr.o + pr.d * (pdepth - 1e-4f);
                if (!(pmm != matMesh || dot(pn, nrm) < 0.95f || len(pos - ppos) > 0.5f)) {
                    DIResv src = readDI(P.previous, (uint64_t)(P.cam.film[0] * (uint32_t)py + (uint32_t)px), P.n);
                    if (diUsable(src)) diReuse(P, r, ds, src, -ray.d, resvRng);
                }
            }
        }
        diOcclude(r, pos);
    }
    diCap(r, DI_CAP);
    if (!diUsable(r)) diClear(r);
    P.temp[i] = r;
}

/* spatialReuse + findNeighborReservoir (di_spatial.glsl:9-121); returns the pixel colour */
static F3 diSpatialPixel(DIPass& P, int x, int y) {
    F2 uv = pixelUV(x, y, P.W, P.H);
    float dn[4]; uint32_t am[2];
    sampleDN(P.cur, uv, dn);
    fetchAM(P.cur, x, y, am);
    float depth; F3 nrm, alb; int matMesh;
    if (!decodeGBuffer(dn, am, depth, nrm, alb, matMesh)) return F3(0.0f);
    uint32_t rng = pixelSeed(P.cam.seed, (uint32_t)x, (uint32_t)y) ^ 2u;
    Ray ray = cameraRay(P.cam, F2{uv.x, 1.0f - uv.y});
    F3 pos = ray.o + ray.d * (depth - 1e-4f), wo = -ray.d;
    size_t i = (size_t)y * P.W + x;
    DIResv r = P.temp[i];
    Surface ds; ds.p = pos; ds.n = nrm; ds.albedo = alb; ds.mat = (uint32_t)(matMesh >> 16); ds.light = false;
    if (P.set.spatial) {
        float tx = 1.0f / (float)P.W, ty = 1.0f / (float)P.H;
        for (uint32_t k = 0; k < DI_NEIGHBOURS; k++) {
            float r0 = rnd(rng), r1 = rnd(rng);
            F2 d = concentric(F2{r0, r1});
            F2 nb{uv.x + d.x * DI_RADIUS * tx, uv.y + d.y * DI_RADIUS * ty};
            if (nb.x < 0.0f || nb.y < 0.0f || nb.x > 1.0f || nb.y > 1.0f) continue;
            int px = (int)(nb.x * (float)P.cam.film[0]), py = (int)(nb.y * (float)P.cam.film[1]);
            float ndn[4]; uint32_t nam[2];
            sampleDN(P.cur, nb, ndn);
            fetchAM(P.cur, px, py, nam);
            float ndepth; F3 nn, nalb; int nmm;
            if (!decodeGBuffer(ndn, nam, ndepth, nn, nalb, nmm)) continue;
            Ray nr = cameraRay(P.cam, F2{nb.x, 1.0f - nb.y});
            F3 npos = nr.o + nr.d * (ndepth - 1e-4f);
            if (dot(nn, nrm) < 0.9f || len(pos - npos) > 0.4f) continue;
            DIResv src = readDI(P.temp, (uint64_t)(P.cam.film[0] * (uint32_t)py + (uint32_t)px), P.n);
            if (diUsable(src)) diReuse(P, r, ds, src, wo, rng);
        }
        diOcclude(r, pos);
    }
    diCap(r, DI_CAP);
    if (!diUsable(r)) diClear(r);
    P.self[i] = r;
    F3 color(0.0f);
    if (diUsable(r) && r.s.isec.inst != NO_HIT) {
        Surface ls; memset(&ls, 0, sizeof(ls));
        fetchSurface(r.s.isec, ls);
        F3 wi = unit(ls.p - pos);
        if (r.M > 0u) {
            Material mat = at(g.materials, ds.mat);
            F3 Li = ld3(r.s.Li) * bsdfEval(mat, alb, nrm, wo, wi) * fmx(dot(nrm, wi), 0.0f) / r.s.pdf;
            if (!(lum(Li) < 1e-5f)) color = Li / lum(Li) * r.W / (float)r.M;
        }
    }
    if (anyNan(color)) return F3(0.0f);
    return F3(fmn(fmx(color.x, 0.0f), 1e4f), fmn(fmx(color.y, 0.0f), 1e4f), fmn(fmx(color.z, 0.0f), 1e4f));
}

}  // namespace oracle

using namespace oracle;

extern "C" {

int oracle_sizeof(int which) {
    switch (which) {
    case 0: return (int)sizeof(Camera);
    case 1: return (int)sizeof(Reservoir);
    case 2: return (int)sizeof(Material);
    case 3: return (int)sizeof(Vertex);
    case 4: return (int)sizeof(Instance);
    case 5: return (int)sizeof(TriLight);
    case 6: return (int)sizeof(TableEntry);
    }
    return -1;
}

int oracle_scene_set(void* vertices, unsigned long long nv, void* indices, unsigned long long ni, void* instances,
                     unsigned long long ninst, void* materials, unsigned long long nmat, void* matIndices,
                     unsigned long long nmi, void* lights, unsigned long long nl, void* table, unsigned long long nt) {
    g.vertices.assign((Vertex*)vertices, (Vertex*)vertices + nv);
    g.indices.assign((uint32_t*)indices, (uint32_t*)indices + ni);
    g.instances.assign((Instance*)instances, (Instance*)instances + ninst);
    g.materials.assign((Material*)materials, (Material*)materials + nmat);
    g.matIndices.assign((int32_t*)matIndices, (int32_t*)matIndices + nmi);
    g.lights.assign((TriLight*)lights, (TriLight*)lights + nl);
    g.table.assign((TableEntry*)table, (TableEntry*)table + nt);
    g.tris.clear();
    for (uint32_t i = 0; i < (uint32_t)nl; i++) {
        Tri T; T.v0 = ld3(g.lights[i].v0); T.e1 = ld3(g.lights[i].v1) - T.v0; T.e2 = ld3(g.lights[i].v2) - T.v0;
        T.inst = 0; T.tri = i;
        g.tris.push_back(T);
    }
    for (uint32_t k = 0; k < (uint32_t)ninst; k++) {
        const Instance& I = g.instances[k];
        for (uint32_t t = 0; t < I.indexCount / 3u; t++) {
            F3 w[3];
            for (uint32_t j = 0; j < 3; j++) w[j] = xformPoint(I.M, ld3(at(g.vertices, at(g.indices, I.indexOffset + t * 3u + j)).pos));
            Tri T; T.v0 = w[0]; T.e1 = w[1] - w[0]; T.e2 = w[2] - w[0]; T.inst = k + 1u; T.tri = t;
            g.tris.push_back(T);
        }
    }
    buildBvh();
    return (int)g.tris.size();
}

void oracle_set_traversal(int useBvh) { g.useBvh = useBvh; }

/* Keeps several scenes resident: slot `slot` becomes the current scene (empty until
 * oracle_scene_set fills it); the previous current scene stays in its own slot. */
static std::vector<Scene> g_slots(1);
static int g_slot = 0;
int oracle_scene_select(int slot) {
    if (slot < 0 || slot >= 4096) return -1;
    if (slot == g_slot) return 0;
    if ((size_t)slot >= g_slots.size()) g_slots.resize((size_t)slot + 1);
    int useBvh = g.useBvh;
    std::swap(g, g_slots[(size_t)g_slot]);
    std::swap(g, g_slots[(size_t)slot]);
    g.useBvh = useBvh;
    g_slot = slot;
    return 0;
}

/* Restricts the G-buffer and the three passes to rows [y0, y1) (a bounded sample of a frame). */
void oracle_set_rows(int y0, int y1) { g_row0 = y0; g_row1 = y1; }

int oracle_threads(void) {
    int n = 1;
#pragma omp parallel
#pragma omp single
    n = omp_get_num_threads();
    return n;
}

void oracle_counters(unsigned long long* out, int reset) {
    for (int i = 0; i < 4; i++) { out[i] = g_counts[i]; if (reset) g_counts[i] = 0; }
}

void oracle_trace(const float* rays, unsigned long long n, int anyHit, float* tuv, uint32_t* inst, uint32_t* tri) {
#pragma omp parallel for schedule(dynamic, 64)
    for (long long i = 0; i < (long long)n; i++) {
        const float* r = rays + i * 8;
        Hit h; float t;
        F3 o(r[0], r[1], r[2]), d(r[4], r[5], r[6]);
        tuv[i * 4 + 1] = tuv[i * 4 + 2] = tuv[i * 4 + 3] = 0.0f;
        if (anyHit) {
            bool b = traceQuery(o, d, r[3], r[7], true, false, nullptr, nullptr);
            tuv[i * 4] = b ? 1.0f : -1.0f; inst[i] = b ? 0u : NO_HIT; tri[i] = b ? 0u : NO_HIT;
            continue;
        }
        if (traceQuery(o, d, r[3], r[7], false, false, &h, &t)) {
            tuv[i * 4] = t; tuv[i * 4 + 1] = h.bx; tuv[i * 4 + 2] = h.by; inst[i] = h.inst; tri[i] = h.tri;
        } else { tuv[i * 4] = -1.0f; inst[i] = NO_HIT; tri[i] = NO_HIT; }
    }
}

/* G-buffer (GBuffer.vert:16-28 / GBuffer.frag:21-54 restated as a ray cast without the lights) */
void oracle_gbuffer(const void* camera, uint32_t W, uint32_t H, float* dn, uint32_t* am, uint16_t* mv) {
    Camera cam; memcpy(&cam, camera, sizeof(cam));
    int y0 = std::max(0, g_row0), y1 = std::min((int)H, g_row1);
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = y0; y < y1; y++)
        for (int x = 0; x < (int)W; x++) {
            size_t p = (size_t)y * W + x;
            F2 uv = pixelUV(x, y, (int)W, (int)H);
            Ray ray = cameraRay(cam, F2{uv.x, 1.0f - uv.y});
            __atomic_fetch_add(&g_counts[2], 1ull, __ATOMIC_RELAXED);
            Hit h;
            if (!traceQuery(ray.o, ray.d, RAY_TMIN, RAY_TMAX, false, true, &h, nullptr)) {
                memset(dn + p * 4, 0, 16); am[p * 2] = am[p * 2 + 1] = 0; mv[p * 2] = mv[p * 2 + 1] = 0;
                continue;
            }
            uint32_t k = h.inst - 1u;
            Instance I = at(g.instances, k);
            F3 b(1.0f - h.bx - h.by, h.bx, h.by);
            F3 P3[3], N3[3];
            for (uint32_t j = 0; j < 3; j++) {
                Vertex v = at(g.vertices, at(g.indices, I.indexOffset + h.tri * 3u + j));
                P3[j] = xformPoint(I.M, ld3(v.pos));
                F3 c0(I.MinvT[0], I.MinvT[1], I.MinvT[2]), c1(I.MinvT[4], I.MinvT[5], I.MinvT[6]), c2(I.MinvT[8], I.MinvT[9], I.MinvT[10]);
                N3[j] = unit((c0 * v.nrm[0] + c1 * v.nrm[1]) + c2 * v.nrm[2]);
            }
            F3 pos = (P3[0] * b.x + P3[1] * b.y) + P3[2] * b.z;
            F3 nor = unit((N3[0] * b.x + N3[1] * b.y) + N3[2] * b.z);
            uint32_t mat = (uint32_t)at(g.matIndices, (uint64_t)(uint32_t)(I.indexOffset / 3u + h.tri));
            F3 alb = ld3(at(g.materials, mat).base);
            const float* M = cam.lastProjView;
            float lx = ((M[0] * pos.x + M[4] * pos.y) + M[8] * pos.z) + M[12] * 1.0f;
            float ly = ((M[1] * pos.x + M[5] * pos.y) + M[9] * pos.z) + M[13] * 1.0f;
            float lw = ((M[3] * pos.x + M[7] * pos.y) + M[11] * pos.z) + M[15] * 1.0f;
            lx = lx / lw * 0.5f + 0.5f;
            ly = ly / lw * 0.5f + 0.5f;
            dn[p * 4] = len(ld3(cam.pos) - pos); dn[p * 4 + 1] = nor.x; dn[p * 4 + 2] = nor.y; dn[p * 4 + 3] = nor.z;
            auto q = [](float c) { return (uint32_t)floorf(fminf(fmaxf(c, 0.0f), 1.0f) * 255.0f + 0.5f); };
            am[p * 2] = q(alb.x) | (q(alb.y) << 8) | (q(alb.z) << 16) | (q(1.0f) << 24);
            am[p * 2 + 1] = (mat << 16) | k;
            mv[p * 2] = toHalf(lx - ((float)x + 0.5f) / (float)W);
            mv[p * 2 + 1] = toHalf(ly - ((float)y + 0.5f) / (float)H);
        }
}

/* GRISReSTIR::render (src/GRISReSTIR.cpp:9-53): passes bit 0 path trace, 1 temporal, 2 spatial */
void oracle_gris_frame(const void* camera, const void* prevCamera, const void* settings, const float* dnCur,
                       const float* dnPrev, const uint32_t* amCur, const uint32_t* amPrev, const uint16_t* motion,
                       void* resvThis, void* resvPrev, void* resvTemp, float* output, int passes) {
    Pass P;
    memcpy(&P.cam, camera, sizeof(Camera));
    memcpy(&P.prev, prevCamera, sizeof(Camera));
    memcpy(&P.set, settings, sizeof(Settings));
    P.W = (int)P.cam.film[0]; P.H = (int)P.cam.film[1];
    P.n = (uint64_t)P.W * P.H;
    P.cur = GBuf{dnCur, amCur, P.W, P.H};
    P.old = GBuf{dnPrev, amPrev, P.W, P.H};
    P.motion.resize(P.n * 2);
    for (uint64_t i = 0; i < P.n * 2; i++) P.motion[i] = fromHalf(motion[i]);
    P.self = (Reservoir*)resvThis; P.previous = (Reservoir*)resvPrev; P.temp = (Reservoir*)resvTemp;
    int y0 = std::max(0, g_row0), y1 = std::min(P.H, g_row1);
    if (passes & 1) {
#pragma omp parallel for schedule(dynamic, 2)
        for (int y = y0; y < y1; y++) for (int x = 0; x < P.W; x++) pathTracePixel(P, x, y);
    }
    if (passes & 2) {
#pragma omp parallel for schedule(dynamic, 2)
        for (int y = y0; y < y1; y++) for (int x = 0; x < P.W; x++) temporalPixel(P, x, y);
    }
    if (passes & 4) {
        float n = (float)(P.cam.frameIndex & 0x7fffffffu);
#pragma omp parallel for schedule(dynamic, 2)
        for (int y = y0; y < y1; y++)
            for (int x = 0; x < P.W; x++) {
                F3 c = spatialPixel(P, x, y);
                float* o = output + ((size_t)y * P.W + x) * 4;
                F3 acc = (F3(o[0], o[1], o[2]) * n + c) / (n + 1.0f);
                o[0] = acc.x; o[1] = acc.y; o[2] = acc.z; o[3] = 1.0f;
            }
    }
}

/* TestReSTIR::render (src/TestReSTIR.cpp:9-35): passes bit 0 candidates, 1 temporal, 2 spatial +
 * running mean into the direct output (di_spatial.comp:14-27). */
void oracle_di_frame(const void* camera, const void* prevCamera, const void* settings, const float* dnCur,
                     const float* dnPrev, const uint32_t* amCur, const uint32_t* amPrev, const uint16_t* motion,
                     void* resvThis, void* resvPrev, void* resvTemp, float* output, int passes) {
    DIPass P;
    memcpy(&P.cam, camera, sizeof(Camera));
    memcpy(&P.prev, prevCamera, sizeof(Camera));
    memcpy(&P.set, settings, sizeof(DISettings));
    P.W = (int)P.cam.film[0]; P.H = (int)P.cam.film[1];
    P.n = (uint64_t)P.W * P.H;
    P.cur = GBuf{dnCur, amCur, P.W, P.H};
    P.old = GBuf{dnPrev, amPrev, P.W, P.H};
    P.motion.resize(P.n * 2);
    for (uint64_t i = 0; i < P.n * 2; i++) P.motion[i] = fromHalf(motion[i]);
    P.self = (DIResv*)resvThis; P.previous = (DIResv*)resvPrev; P.temp = (DIResv*)resvTemp;
    int y0 = std::max(0, g_row0), y1 = std::min(P.H, g_row1);
    if (passes & 1) {
#pragma omp parallel for schedule(dynamic, 2)
        for (int y = y0; y < y1; y++) for (int x = 0; x < P.W; x++) diGenPixel(P, x, y);
    }
    if (passes & 2) {
#pragma omp parallel for schedule(dynamic, 2)
        for (int y = y0; y < y1; y++) for (int x = 0; x < P.W; x++) diTemporalPixel(P, x, y);
    }
    if (passes & 4) {
        float n = (float)(P.cam.frameIndex & 0x7fffffffu);
#pragma omp parallel for schedule(dynamic, 2)
        for (int y = y0; y < y1; y++)
            for (int x = 0; x < P.W; x++) {
                F3 c = diSpatialPixel(P, x, y);
                float* o = output + ((size_t)y * P.W + x) * 4;
                F3 acc = (F3(o[0], o[1], o[2]) * n + c) / (n + 1.0f);
                o[0] = acc.x; o[1] = acc.y; o[2] = acc.z; o[3] = 1.0f;
            }
    }
}

/* The presentation pass (post_proc.frag:16-44, push constant PostProcessFrag.h:7-12) at pixel
 * centres of a full-screen quad; settings: {toneMapping, correctGamma, noDirect, noIndirect}.
 * Writes the fragment colour (float4) and its B8G8R8A8_UNORM conversion (R, G, B, A bytes). */
static inline float oraFilmicCurve(float c) {
    return (c * (c * 0.22f + 0.03f) + 0.002f) / (c * (c * 0.22f + 0.3f) + 0.06f) - 1.0f / 30.0f;
}
static inline float oraTonemap(float c, uint32_t mode) {
    if (mode == 0u) return c;
    if (mode == 1u) return oraFilmicCurve(c * 1.6f) / oraFilmicCurve(11.2f);
    return (c * (c * 2.51f + 0.03f)) / (c * (c * 2.43f + 0.59f) + 0.14f);
}
static inline uint8_t oraUnorm8(float c) {
    if (!(c > 0.0f)) return 0;
    if (c >= 1.0f) return 255;
    return (uint8_t)floorf(c * 255.0f + 0.5f);
}
void oracle_post(uint32_t W, uint32_t H, const float* direct, const float* indirect, const uint32_t* settings,
                 float* color, uint8_t* rgba8) {
    for (uint32_t y = 0; y < H; y++)
        for (uint32_t x = 0; x < W; x++) {
            float u = ((float)x + 0.5f) / (float)W, v = ((float)y + 0.5f) / (float)H;
            uint32_t cx = (uint32_t)((float)(W - 1u) * u), cy = (uint32_t)((float)(H - 1u) * v);
            size_t src = (size_t)cy * W + cx, dst = (size_t)y * W + x;
            float c[3] = {0.0f, 0.0f, 0.0f};
            for (int k = 0; k < 3; k++) {
                if (settings[2] == 0u) c[k] = c[k] + direct[src * 4 + k];
                if (settings[3] == 0u) c[k] = c[k] + indirect[src * 4 + k];
                c[k] = oraTonemap(c[k], settings[0]);
                if (settings[1] != 0u) c[k] = oracle_det_powf(c[k], 1.0f / 2.2f);
            }
            if (color) {   /* NaN channels as the canonical quiet NaN */
                for (int k = 0; k < 3; k++) color[dst * 4 + k] = std::isnan(c[k]) ? oracle_dm_float(0x7fc00000u) : c[k];
                color[dst * 4 + 3] = 1.0f;
            }
            if (rgba8) {
                rgba8[dst * 4] = oraUnorm8(c[0]); rgba8[dst * 4 + 1] = oraUnorm8(c[1]);
                rgba8[dst * 4 + 2] = oraUnorm8(c[2]); rgba8[dst * 4 + 3] = 255;
            }
        }
}

uint16_t oracle_f16(float f) { return toHalf(f); }

}  /* extern "C" */
