/*
 * converged_fp64.cpp — FP64 CPU oracle of the converged image the GRIS path converges to.
 *
 * TEST INFRASTRUCTURE: the oracle. Only tests/ and bench.py's baseline legs may load it, and
 * only as the checker. It is never part of the product path.
 *
 * What it computes: per pixel, the mean over `spp` independent paths of one of two estimators,
 * in double precision throughout (vectors, BSDFs, light sampling, ray-triangle tests, sums):
 *
 *   estimator 0 ("gris")  the sum of the candidate contributions that the path tracer of
 *                         gris_path_trace.glsl:45-306 feeds its reservoir stream (addStream),
 *                         i.e. the expectation of the canonical GRIS sample's F * sumW / w — what
 *                         ReSTIR PT's output converges to. Contributions at vertices before the
 *                         first reconnectible pair are not candidates there and are not summed.
 *   estimator 1 ("full")  every NEE and BSDF-sampled light-hit contribution of the same path
 *                         (the indirect illumination of gi_naive.glsl:28-149: NEE on non-delta
 *                         vertices with bounce > 0, light hits with bounce > 1), with the MIS
 *                         weights of gris_path_trace.glsl (NEE: power heuristic against
 *                         cos/pi, gris_path_trace.glsl:193; light hits: against the light pdf).
 *                         gi_naive.glsl:113 overrides its NEE weight with 1.0; that variant is
 *                         estimator 2 (it counts the NEE-reachable light twice).
 *
 * Both follow the reference's sampling procedures (cosine hemisphere, the GTR2 visible-normal
 * sampler of material.glsl:84-101 with its Schlick-G1 pdf, the metallic-workflow lobe choice,
 * light selection through the alias table, Russian roulette after bounce 4 with rrScale), so the
 * estimands are those of the reference's FP32 estimator; only the random numbers (a 64-bit
 * counter-based generator per pixel and sample) and the precision differ. Each sample is
 * clamped as clampColor (math.glsl:187-192) before it is summed.
 *
 * The primary vertex comes from the same G-buffer the GRIS passes read (depth, shading normal,
 * 8-bit albedo, material id), so the estimand is conditioned on the same primary surfaces.
 * Supported materials: Lambert (type 1) and MetallicWorkflow (type 2).
 *
 * Traversal: a binary BVH (median split) over world-space triangles in double precision;
 * closest hit = smallest t; shadow rays hit anything in [1e-4, dist - 1e-4], lights included.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include <omp.h>

namespace fp64 {

struct D3 {
    double x, y, z;
    D3() : x(0), y(0), z(0) {}
    D3(double a, double b, double c) : x(a), y(b), z(c) {}
    explicit D3(double s) : x(s), y(s), z(s) {}
};
static inline D3 operator+(const D3& a, const D3& b) { return D3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline D3 operator-(const D3& a, const D3& b) { return D3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline D3 operator*(const D3& a, const D3& b) { return D3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline D3 operator*(const D3& a, double s) { return D3(a.x * s, a.y * s, a.z * s); }
static inline D3 operator/(const D3& a, double s) { return D3(a.x / s, a.y / s, a.z / s); }
static inline D3 operator-(const D3& a) { return D3(-a.x, -a.y, -a.z); }
static inline double dot(const D3& a, const D3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline D3 cross(const D3& a, const D3& b) { return D3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline double length(const D3& v) { return sqrt(dot(v, v)); }
static inline D3 normalize(const D3& v) { return v / length(v); }
static inline double lum(const D3& c) { return c.x * 0.299 + c.y * 0.587 + c.z * 0.114; }
static inline D3 lerp(const D3& a, const D3& b, double t) { return a * (1.0 - t) + b * t; }
static inline double mis(double f, double g) { return f * f / (f * f + g * g); }   /* MISWeight, math.glsl */
static const double kPi = 3.14159265358979323846;

/* scene layouts (the C-ABI's) */
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
struct Settings { uint32_t shift; float rrScale; uint32_t temporal, spatial, cap, maxDepth, neighbours; float radius; };
static_assert(sizeof(Camera) == 352 && sizeof(Instance) == 224 && sizeof(Material) == 32, "layouts");

static inline D3 ld(const float* p) { return D3(p[0], p[1], p[2]); }
static inline D3 xform(const float* M, const D3& p) {   /* column-major 4x4 times (p, 1) */
    return D3(M[0] * p.x + M[4] * p.y + M[8] * p.z + M[12], M[1] * p.x + M[5] * p.y + M[9] * p.z + M[13],
              M[2] * p.x + M[6] * p.y + M[10] * p.z + M[14]);
}

struct Tri { D3 v0, e1, e2; uint32_t inst, tri; };
struct Node { D3 lo, hi; int left, right; uint32_t first, count; };

struct Scene {
    std::vector<Material> materials;
    std::vector<int32_t> matIndices;
    std::vector<Vertex> vertices;
    std::vector<uint32_t> indices;
    std::vector<Instance> instances;
    std::vector<TriLight> lights;
    std::vector<TableEntry> table;
    std::vector<Tri> tris;
    std::vector<Node> nodes;
};
static Scene S;

static void build(std::vector<uint32_t>& idx, uint32_t begin, uint32_t end, std::vector<D3>& cen) {
    Node n;
    n.lo = D3(1e300); n.hi = D3(-1e300);
    D3 clo(1e300), chi(-1e300);
    for (uint32_t i = begin; i < end; i++) {
        const Tri& T = S.tris[idx[i]];
        D3 p[3] = {T.v0, T.v0 + T.e1, T.v0 + T.e2};
        for (auto& q : p) {
            n.lo = D3(std::min(n.lo.x, q.x), std::min(n.lo.y, q.y), std::min(n.lo.z, q.z));
            n.hi = D3(std::max(n.hi.x, q.x), std::max(n.hi.y, q.y), std::max(n.hi.z, q.z));
        }
        const D3& c = cen[idx[i]];
        clo = D3(std::min(clo.x, c.x), std::min(clo.y, c.y), std::min(clo.z, c.z));
        chi = D3(std::max(chi.x, c.x), std::max(chi.y, c.y), std::max(chi.z, c.z));
    }
    int self = (int)S.nodes.size();
    S.nodes.push_back(n);
    if (end - begin <= 4) {
        S.nodes[self].left = S.nodes[self].right = -1;
        S.nodes[self].first = begin; S.nodes[self].count = end - begin;
        return;
    }
    D3 ext = chi - clo;
    int axis = ext.x > ext.y ? (ext.x > ext.z ? 0 : 2) : (ext.y > ext.z ? 1 : 2);
    uint32_t mid = (begin + end) / 2;
    auto key = [&](uint32_t t) { const D3& c = cen[t]; return axis == 0 ? c.x : axis == 1 ? c.y : c.z; };
    std::nth_element(idx.begin() + begin, idx.begin() + mid, idx.begin() + end,
                     [&](uint32_t a, uint32_t b) { return key(a) < key(b) || (key(a) == key(b) && a < b); });
    build(idx, begin, mid, cen);
    int l = self + 1;
    int r = (int)S.nodes.size();
    build(idx, mid, end, cen);
    S.nodes[self].left = l; S.nodes[self].right = r; S.nodes[self].count = 0;
}

static void build_bvh() {
    S.nodes.clear();
    if (S.tris.empty()) return;
    std::vector<uint32_t> idx(S.tris.size());
    std::vector<D3> cen(S.tris.size());
    for (uint32_t i = 0; i < idx.size(); i++) {
        idx[i] = i;
        const Tri& T = S.tris[i];
        cen[i] = T.v0 + (T.e1 + T.e2) / 3.0;
    }
    build(idx, 0, (uint32_t)idx.size(), cen);
    std::vector<Tri> sorted(S.tris.size());
    for (uint32_t i = 0; i < idx.size(); i++) sorted[i] = S.tris[idx[i]];
    S.tris.swap(sorted);
}

static inline bool box_hit(const Node& n, const D3& o, const D3& inv, double tmax) {
    double t0 = 0.0, t1 = tmax;
    const double lo[3] = {n.lo.x, n.lo.y, n.lo.z}, hi[3] = {n.hi.x, n.hi.y, n.hi.z};
    const double oo[3] = {o.x, o.y, o.z}, ii[3] = {inv.x, inv.y, inv.z};
    for (int a = 0; a < 3; a++) {
        double ta = (lo[a] - oo[a]) * ii[a], tb = (hi[a] - oo[a]) * ii[a];
        if (ta > tb) std::swap(ta, tb);
        t0 = std::max(t0, ta); t1 = std::min(t1, tb);
        if (t0 > t1 * (1.0 + 1e-12) + 1e-12) return false;
    }
    return true;
}

struct Hit { double t, u, v; uint32_t inst, tri; bool found; };

/* Moller-Trumbore, two-sided; t in [tmin, tmax] */
static bool trace(const D3& o, const D3& d, double tmin, double tmax, bool any, Hit* out) {
    if (S.nodes.empty()) return false;
    D3 inv(1.0 / d.x, 1.0 / d.y, 1.0 / d.z);
    Hit best; best.found = false; best.t = tmax;
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const Node& n = S.nodes[stack[--sp]];
        if (!box_hit(n, o, inv, best.t)) continue;
        if (n.left < 0) {
            for (uint32_t i = n.first; i < n.first + n.count; i++) {
                const Tri& T = S.tris[i];
                D3 p = cross(d, T.e2);
                double det = dot(T.e1, p);
                if (det == 0.0) continue;
                double id = 1.0 / det;
                D3 s = o - T.v0;
                double u = dot(s, p) * id;
                if (u < 0.0 || u > 1.0) continue;
                D3 q = cross(s, T.e1);
                double v = dot(d, q) * id;
                if (v < 0.0 || u + v > 1.0) continue;
                double t = dot(T.e2, q) * id;
                if (t < tmin || t > best.t) continue;
                if (any) return true;
                if (t < best.t || !best.found || (T.inst < best.inst || (T.inst == best.inst && T.tri < best.tri))) {
                    best.t = t; best.u = u; best.v = v; best.inst = T.inst; best.tri = T.tri; best.found = true;
                }
            }
        } else if (sp + 2 <= 128) {
            stack[sp++] = n.left;
            stack[sp++] = n.right;
        }
    }
    if (out) *out = best;
    return best.found;
}

struct Surface { D3 p, n, albedo; uint32_t mat; bool light; };

static void surface(const Hit& h, Surface& s) {
    double b0 = 1.0 - h.u - h.v, b1 = h.u, b2 = h.v;
    if (h.inst == 0) {
        const TriLight& L = S.lights[h.tri];
        s.p = ld(L.v0) * b0 + ld(L.v1) * b1 + ld(L.v2) * b2;
        s.n = D3(L.nx, L.ny, L.nz);
        s.albedo = ld(L.rad);
        s.light = true;
        return;
    }
    const Instance& I = S.instances[h.inst - 1];
    s.mat = (uint32_t)S.matIndices[I.indexOffset / 3u + h.tri];
    uint32_t base = I.indexOffset + h.tri * 3u;
    const Vertex& a = S.vertices[S.indices[base]];
    const Vertex& b = S.vertices[S.indices[base + 1]];
    const Vertex& c = S.vertices[S.indices[base + 2]];
    s.p = xform(I.M, ld(a.pos) * b0 + ld(b.pos) * b1 + ld(c.pos) * b2);
    s.n = normalize(xform(I.MinvT, ld(a.nrm) * b0 + ld(b.nrm) * b1 + ld(c.nrm) * b2));
    s.albedo = ld(S.materials[s.mat].base);
    s.light = false;
}

/* ---------------------------------------------------------------- sampling (material.glsl, math.glsl) */
struct Frame { D3 t, b, n; };
static Frame frame_of(const D3& n) {
    D3 t = fabs(n.z) > 0.999 ? D3(0, 1, 0) : D3(0, 0, 1);
    D3 b = normalize(cross(n, t));
    return Frame{cross(b, n), b, n};
}
static inline D3 to_world(const Frame& f, const D3& v) { return f.t * v.x + f.b * v.y + f.n * v.z; }
static inline D3 to_local(const Frame& f, const D3& v) { return D3(dot(v, f.t), dot(v, f.b), dot(v, f.n)); }
static void concentric(double u0, double u1, double& x, double& y) {
    if (u0 == 0.0 && u1 == 0.0) { x = y = 0.0; return; }
    double a = u0 * 2.0 - 1.0, b = u1 * 2.0 - 1.0, r, phi;
    if (a * a > b * b) { r = a; phi = kPi * b / a * 0.25; }
    else { r = b; phi = kPi * 0.5 - kPi * a / b * 0.25; }
    x = r * cos(phi); y = r * sin(phi);
}
static D3 cosine_hemisphere(const D3& n, double u0, double u1) {
    double x, y;
    concentric(u0, u1, x, y);
    return normalize(to_world(frame_of(n), D3(x, y, sqrt(std::max(0.0, 1.0 - x * x - y * y)))));
}
static inline double g_schlick(double c, double alpha) { double a = alpha * 0.5; return c / (c * (1.0 - a) + a); }
static inline double d_gtr2(double c, double alpha) {
    if (c < 1e-6) return 0.0;
    double aa = alpha * alpha, den = c * c * (aa - 1.0) + 1.0;
    return aa / (den * den * kPi);
}
static inline double pdf_gtr2(const D3& n, const D3& m, const D3& wo, double alpha) {
    return d_gtr2(dot(n, m), alpha) * g_schlick(dot(n, wo), alpha) * fabs(dot(m, wo)) / fabs(dot(n, wo));
}
/* visible-normal sample of GTR2 (material.glsl:84-101) */
static D3 sample_gtr2(const D3& n, const D3& wo, double alpha, double u0, double u1) {
    Frame f = frame_of(n);
    D3 local = to_local(f, wo);
    D3 vh = normalize(D3(local.x * alpha, local.y * alpha, local.z));
    double l2 = vh.x * vh.x + vh.y * vh.y;
    D3 t1 = l2 > 0.0 ? D3(-vh.y, vh.x, 0.0) / sqrt(l2) : D3(1, 0, 0);
    D3 t2 = cross(vh, t1);
    double px, py;
    concentric(u0, u1, px, py);
    double s = 0.5 * (vh.z + 1.0);
    py = (1.0 - s) * sqrt(std::max(0.0, 1.0 - px * px)) + s * py;
    D3 h = t1 * px + t2 * py + vh * sqrt(std::max(0.0, 1.0 - px * px - py * py));
    h = D3(h.x * alpha, h.y * alpha, std::max(0.0, h.z));
    return normalize(to_world(f, h));
}
static inline D3 reflect(const D3& i, const D3& n) { return i - n * (2.0 * dot(n, i)); }
static inline double pow5(double x) { double x2 = x * x; return x2 * x2 * x; }

static D3 f_metallic(const Material& m, const D3& alb, const D3& n, const D3& wo, const D3& wi) {
    double alpha = (double)m.roughness * m.roughness;
    D3 h = normalize(wo + wi);
    double co = dot(n, wo), ci = dot(n, wi);
    if (ci * co < 1e-7) return D3(0.0);
    D3 F = lerp(lerp(D3(0.08), alb, m.metallic), D3(1.0), pow5(1.0 - dot(h, wo)));
    double G = g_schlick(fabs(co), alpha) * g_schlick(fabs(ci), alpha), Dd = d_gtr2(dot(n, h), alpha);
    D3 diff = alb / kPi * (1.0 - m.metallic);
    double spec = G * Dd / (4.0 * ci * co);
    return diff * (D3(1.0) - F) + F * spec;
}
static double pdf_metallic(const Material& m, const D3& n, const D3& wo, const D3& wi) {
    D3 h = normalize(wo + wi);
    double a = std::max(dot(n, wi), 0.0) / kPi;
    double b = pdf_gtr2(n, h, wo, (double)m.roughness * m.roughness) / (4.0 * fabs(dot(h, wo)));
    double t = 1.0 / (2.0 - m.metallic);
    return a * (1.0 - t) + b * t;
}
static D3 bsdf(const Material& m, const D3& alb, const D3& n, const D3& wo, const D3& wi) {
    if (m.type == 1) return alb / kPi;
    return f_metallic(m, alb, n, wo, wi);
}
struct Sample { D3 wi, f; double pdf; bool delta; };
static bool sample_bsdf(const Material& m, const D3& alb, const D3& n, const D3& wo, double u0, double u1, double u2,
                        Sample& s) {
    s.delta = false;
    if (m.type == 1) {
        s.wi = cosine_hemisphere(n, u0, u1);
        s.pdf = fabs(dot(n, s.wi)) / kPi;
        s.f = alb / kPi;
        return true;
    }
    double alpha = (double)m.roughness * m.roughness;
    if (u2 > 1.0 / (2.0 - m.metallic)) s.wi = cosine_hemisphere(n, u0, u1);
    else { s.wi = -reflect(wo, sample_gtr2(n, wo, alpha, u0, u1)); s.delta = m.roughness < 0.01f; }
    if (dot(n, s.wi) < 0.0) return false;
    s.f = f_metallic(m, alb, n, wo, s.wi);
    s.pdf = pdf_metallic(m, n, wo, s.wi);
    return true;
}
static inline bool is_delta(const Material& m) { return m.type == 2 && m.roughness < 0.01f && m.metallic > 0.9f; }
static inline bool connectible(const Material& m) { return m.type == 1 || m.roughness > 0.05f || m.metallic < 0.9f; }

/* sampleLightByPower + sampleTriangleLight (light_sampling.glsl:6-37) */
static D3 sample_light(const D3& ref, const double r[4], D3& wi, double& dist, double& pdf) {
    const TableEntry& t0 = S.table[0];
    uint32_t id = (uint32_t)((double)t0.failId * r[0]);
    if (id >= t0.failId) id = t0.failId - 1;
    const TableEntry& e = S.table[id + 1];
    id = r[1] < (double)e.prob ? id : e.failId - 1u;
    const TriLight& L = S.lights[id];
    double sq = sqrt(r[3]), bx = 1.0 - sq, by = r[2] * sq;
    D3 pos = ld(L.v0) * (1.0 - bx - by) + ld(L.v1) * bx + ld(L.v2) * by;
    dist = length(ref - pos);
    D3 n(L.nx, L.ny, L.nz);
    wi = (pos - ref) / dist;
    double jac = fabs(dot(n, wi)) / (dist * dist);
    pdf = 1.0 / jac / (double)L.area * (lum(ld(L.rad)) * (double)L.area / (double)t0.prob);
    return dot(n, wi) > 0.0 ? D3(0.0) : ld(L.rad);
}

/* ---------------------------------------------------------------- random numbers */
struct Rng {
    uint64_t s;
    double next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    }
};

static inline D3 clamp_color(const D3& c) {                    /* clampColor, math.glsl:187-192 */
    if (std::isnan(c.x) || std::isnan(c.y) || std::isnan(c.z)) return D3(0.0);
    return D3(std::min(std::max(c.x, 0.0), 1e4), std::min(std::max(c.y, 0.0), 1e4), std::min(std::max(c.z, 0.0), 1e4));
}

/* One path from the pixel's primary surface; returns the estimator's value. */
static D3 path(const Settings& set, const D3& camPos, const D3& primaryDir, double depth, const D3& nrm, const D3& alb,
               uint32_t matId, Rng& rng, int estimator) {
    const double kDist = 0.01;   /* DistanceThreshold */
    D3 dir = primaryDir, orig = camPos;
    D3 thr(1.0), wo = -dir, lastPos(0.0);
    Surface surf;
    surf.p = orig + dir * (depth - 1e-4);
    surf.n = nrm; surf.albedo = alb; surf.mat = matId; surf.light = false;
    Material mat = S.materials[matId];
    Sample s; s.pdf = 0.0; s.delta = false;
    bool lastConn = false;
    uint32_t state = 0, lastState = 0;
    D3 candF(0.0), sumCand(0.0), sumAll(0.0);
    for (int bounce = 0; bounce < (int)set.maxDepth; bounce++) {
        if (bounce > 0) {
            Hit h;
            if (!trace(orig, dir, 1e-4, 1e7, false, &h)) break;
            surface(h, surf);
            if (!surf.light) mat = S.materials[surf.mat];
        }
        double cosPrev = dot(dir, surf.n);
        double dPrev = length(lastPos - surf.p);
        double gJac = fabs(cosPrev) / (dPrev * dPrev);
        bool conn = surf.light || connectible(mat);
        lastState = state;
        state = state == 2u ? 2u : (conn ? state + 1u : 0u);
        if (set.shift == 0u && bounce == 1 && !surf.light) { state = 2u; lastState = 1u; }
        if (surf.light) {
            if (bounce > 1 && cosPrev < 0.0) {
                double w = 1.0;
                double lightPdf = lum(surf.albedo) / (double)S.table[0].prob / gJac;
                if (!s.delta) w = mis(s.pdf, lightPdf);
                D3 c = surf.albedo * w * thr;
                sumAll = sumAll + c;
                if (state == 2u && lastState == 2u) candF = candF + c;
                else if (state == 2u && lastState == 1u && lastConn && dPrev > kDist) { candF = c; sumCand = sumCand + candF; }
            }
            break;
        }
        double rl[4] = {rng.next(), rng.next(), rng.next(), rng.next()};
        if (bounce > 0 && !is_delta(mat)) {
            D3 ldir; double ldist, lpdf;
            D3 Le = sample_light(surf.p, rl, ldir, ldist, lpdf);
            bool blocked = trace(surf.p, ldir, 1e-4, ldist - 1e-4, true, nullptr);
            if (!blocked && lpdf > 1e-6) {
                double w = estimator == 2 ? 1.0 : mis(lpdf, fabs(dot(surf.n, ldir)) / kPi);
                D3 c = Le / lpdf * w * bsdf(mat, surf.albedo, surf.n, wo, ldir) * std::max(dot(surf.n, ldir), 0.0) * thr;
                sumAll = sumAll + c;
                if (state == 2u && lastState == 2u) candF = candF + c;
                else if (state == 2u && lastState == 1u) { candF = c; sumCand = sumCand + candF; }
                else if (state == 1u && conn && ldist > kDist) { candF = c; sumCand = sumCand + candF; }
            }
        }
        if (bounce > 4) {
            double term = std::max(1.0 - lum(thr) * (double)set.rrScale, 0.0);
            if (rng.next() < term) break;
            thr = thr / (1.0 - term);
        }
        double u0 = rng.next(), u1 = rng.next(), u2 = rng.next();
        if (!sample_bsdf(mat, surf.albedo, surf.n, wo, u0, u1, u2, s) || s.pdf < 1e-6) break;
        double cosT = s.delta ? 1.0 : fabs(dot(surf.n, s.wi));
        thr = thr * (s.f * (cosT / s.pdf));
        if (state == 2u && lastState == 1u) candF = D3(0.0);
        lastPos = surf.p;
        wo = -s.wi;
        dir = s.wi;
        orig = surf.p + dir * 1e-4;
        lastConn = conn;
    }
    if (state == 2u && lastState == 2u) sumCand = sumCand + candF;
    return clamp_color(estimator == 0 ? sumCand : sumAll);
}

}  // namespace fp64

using namespace fp64;

extern "C" {

/* Same arrays as oracle_scene_set; returns the triangle count, or -2 for an unsupported material. */
int fp64_scene_set(void* vertices, unsigned long long nv, void* indices, unsigned long long ni, void* instances,
                   unsigned long long ninst, void* materials, unsigned long long nmat, void* matIndices,
                   unsigned long long nmi, void* lights, unsigned long long nl, void* table, unsigned long long nt) {
    S = Scene();
    S.vertices.assign((Vertex*)vertices, (Vertex*)vertices + nv);
    S.indices.assign((uint32_t*)indices, (uint32_t*)indices + ni);
    S.instances.assign((Instance*)instances, (Instance*)instances + ninst);
    S.materials.assign((Material*)materials, (Material*)materials + nmat);
    S.matIndices.assign((int32_t*)matIndices, (int32_t*)matIndices + nmi);
    S.lights.assign((TriLight*)lights, (TriLight*)lights + nl);
    S.table.assign((TableEntry*)table, (TableEntry*)table + nt);
    for (const Material& m : S.materials)
        if (m.type != 1 && m.type != 2) return -2;
    for (uint32_t i = 0; i < (uint32_t)nl; i++) {
        const TriLight& L = S.lights[i];
        Tri T; T.v0 = ld(L.v0); T.e1 = ld(L.v1) - T.v0; T.e2 = ld(L.v2) - T.v0; T.inst = 0; T.tri = i;
        S.tris.push_back(T);
    }
    for (uint32_t k = 0; k < (uint32_t)ninst; k++) {
        const Instance& I = S.instances[k];
        for (uint32_t t = 0; t < I.indexCount / 3u; t++) {
            D3 w[3];
            for (uint32_t j = 0; j < 3; j++) w[j] = xform(I.M, ld(S.vertices[S.indices[I.indexOffset + t * 3u + j]].pos));
            Tri T; T.v0 = w[0]; T.e1 = w[1] - w[0]; T.e2 = w[2] - w[0]; T.inst = k + 1u; T.tri = t;
            S.tris.push_back(T);
        }
    }
    build_bvh();
    return (int)S.tris.size();
}

/* Accumulates `spp` paths (sample indices [sppBegin, sppBegin + spp)) of each pixel of the
 * rectangle [x0,x1) x [y0,y1) of a W x H frame, from the G-buffer (dn: float4 per pixel, am: uint2
 * per pixel) of `camera`; sum and sumSq (3 doubles per rectangle pixel, row-major) are added to. */
void fp64_render(const void* camera, const void* settings, uint32_t W, uint32_t H, const float* dn, const uint32_t* am,
                 int x0, int y0, int x1, int y1, unsigned long long sppBegin, unsigned long long spp,
                 unsigned long long seed, int estimator, double* sum, double* sumSq) {
    Camera cam;
    memcpy(&cam, camera, sizeof(cam));
    Settings set;
    memcpy(&set, settings, sizeof(set));
    const int rw = x1 - x0, rh = y1 - y0;
    const double aspect = (double)cam.film[0] / (double)cam.film[1];
    const double tf = tan((double)cam.fov * 0.5 * kPi / 180.0);
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < rw * rh; i++) {
        int x = x0 + i % rw, y = y0 + i / rw;
        size_t p = (size_t)y * W + x;
        double depth = dn[p * 4];
        if (depth == 0.0) continue;
        D3 nrm(dn[p * 4 + 1], dn[p * 4 + 2], dn[p * 4 + 3]);
        uint32_t a0 = am[p * 2];
        D3 alb((double)(float)((a0 & 0xffu) / 255.0f), (double)(float)(((a0 >> 8) & 0xffu) / 255.0f),
               (double)(float)(((a0 >> 16) & 0xffu) / 255.0f));
        uint32_t matId = am[p * 2 + 1] >> 16;
        /* pinholeCameraSampleRay (camera.glsl:28-42) through the pixel centre, uv.y flipped */
        double u = ((double)x + 0.5) / W, v = 1.0 - ((double)y + 0.5) / H;
        D3 d = normalize(D3((u * 2.0 - 1.0) * aspect * tf, (v * 2.0 - 1.0) * tf, 1.0));
        D3 dir = normalize(ld(cam.right) * d.x + ld(cam.up) * d.y + ld(cam.front) * d.z);
        D3 acc(0.0), acc2(0.0);
        for (unsigned long long k = sppBegin; k < sppBegin + spp; k++) {
            Rng rng{seed * 0x2545f4914f6cdd1dull ^ ((uint64_t)p * 0x9e3779b97f4a7c15ull) ^ (k * 0xd1b54a32d192ed03ull)};
            rng.next();
            D3 c = path(set, ld(cam.pos), dir, depth, nrm, alb, matId, rng, estimator);
            acc = acc + c;
            acc2 = acc2 + c * c;
        }
        double* o = sum + (size_t)i * 3;
        o[0] += acc.x; o[1] += acc.y; o[2] += acc.z;
        if (sumSq) {
            double* q = sumSq + (size_t)i * 3;
            q[0] += acc2.x; q[1] += acc2.y; q[2] += acc2.z;
        }
    }
}

}  // extern "C"
