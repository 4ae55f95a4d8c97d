/*
 * host_scene.cpp — host helpers of grisrt: the light alias table, camera set-up and the
 * synthetic scenes that stand in for the reference's XML scenes (none ship with it).
 *
 * All arithmetic here is plain IEEE (compiled with -ffp-contract=off) with the
 * deterministic transcendental functions of detmath.h, so a scene and a camera built on an
 * x86-64 host and on an aarch64 host are byte-identical.
 */
#include <ctype.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/grisrt.h"
#include "detmath.h"
#include "grisrt_internal.h"

namespace grisrt {

/* ------------------------------------------------------------------ small vector math */
struct H3 { float x, y, z; };
static inline H3 h3(float x, float y, float z) { H3 r = {x, y, z}; return r; }
static inline H3 operator+(H3 a, H3 b) { return h3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline H3 operator-(H3 a, H3 b) { return h3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline H3 operator*(H3 a, float s) { return h3(a.x * s, a.y * s, a.z * s); }
static inline float hdot(H3 a, H3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline H3 hcross(H3 a, H3 b) { return h3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline H3 hnorm(H3 v) { return v * (1.0f / sqrtf(hdot(v, v))); }
static inline float hlen(H3 v) { return sqrtf(hdot(v, v)); }

/* column-major 4x4, m[c*4 + r] */
struct M4 { float m[16]; };
static M4 m4_identity() { M4 r; memset(r.m, 0, sizeof(r.m)); r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0f; return r; }
static M4 m4_mul(const M4& a, const M4& b) {
    M4 r;
    for (int c = 0; c < 4; c++)
        for (int row = 0; row < 4; row++) {
            float s = a.m[0 * 4 + row] * b.m[c * 4 + 0];
            s = s + a.m[1 * 4 + row] * b.m[c * 4 + 1];
            s = s + a.m[2 * 4 + row] * b.m[c * 4 + 2];
            s = s + a.m[3 * 4 + row] * b.m[c * 4 + 3];
            r.m[c * 4 + row] = s;
        }
    return r;
}
static M4 m4_transpose(const M4& a) {
    M4 r;
    for (int c = 0; c < 4; c++) for (int row = 0; row < 4; row++) r.m[c * 4 + row] = a.m[row * 4 + c];
    return r;
}
/* Inverse of an affine transform [A t; 0 1] (all instance transforms here are affine). */
static M4 m4_affine_inverse(const M4& a) {
    double A[3][3], inv[3][3];
    for (int r = 0; r < 3; r++) for (int c = 0; c < 3; c++) A[r][c] = a.m[c * 4 + r];
    double det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) - A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
                 A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
    inv[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) / det;
    inv[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) / det;
    inv[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) / det;
    inv[1][0] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) / det;
    inv[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) / det;
    inv[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / det;
    inv[2][0] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) / det;
    inv[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) / det;
    inv[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) / det;
    M4 r = m4_identity();
    for (int row = 0; row < 3; row++) {
        double t = 0.0;
        for (int c = 0; c < 3; c++) { r.m[c * 4 + row] = (float)inv[row][c]; t -= inv[row][c] * a.m[12 + c]; }
        r.m[12 + row] = (float)t;
    }
    return r;
}
static M4 m4_translate_scale_rotz(H3 t, float scale, float rotz) {
    float s, c;
    gris_det_sincosf(rotz, &s, &c);
    M4 r = m4_identity();
    r.m[0] = c * scale; r.m[1] = s * scale;
    r.m[4] = -s * scale; r.m[5] = c * scale;
    r.m[10] = scale;
    r.m[12] = t.x; r.m[13] = t.y; r.m[14] = t.z;
    return r;
}

}  // namespace grisrt

using namespace grisrt;

/* ------------------------------------------------------------------ alias table */
/* reference: DiscreteSampler1D<float>::build (src/util/AliasTable.h:26-71): normalise the
 * distribution to mean 1, then pair "small" and "large" entries from two stacks (LIFO),
 * entry i+1 = {probability of keeping i, 1-based id of the alias}; entry 0 = {sum, n}. */
extern "C" int grisBuildLightTable(const float* distribution, uint32_t n, GrisLightTableEntry* out) {
    if (!distribution || !out || n == 0) return GRIS_ERR_INVALID_ARGUMENT;
    std::vector<float> d(distribution, distribution + n);
    float sumAll = 0.0f;
    for (uint32_t i = 0; i < n; i++) sumAll += d[i];
    float sumInv = (float)n / sumAll;
    for (uint32_t i = 0; i < n; i++) d[i] *= sumInv;
    struct E { float prob; uint32_t id; };
    std::vector<E> large(n * 2), small(n * 2);
    int nl = 0, ns = 0;
    for (uint32_t i = 0; i < n; i++) {
        E e = {d[i], i + 1};
        if (d[i] > 1.0f) large[nl++] = e; else small[ns++] = e;
    }
    while (nl && ns) {
        E g = large[--nl];
        E l = small[--ns];
        out[l.id].prob = l.prob; out[l.id].failId = g.id;
        g.prob -= (1.0f - l.prob);
        if (g.prob > 1.0f) large[nl++] = g; else small[ns++] = g;
    }
    for (int i = nl - 1; i >= 0; i--) { out[large[i].id].prob = large[i].prob; out[large[i].id].failId = large[i].id; }
    for (int i = ns - 1; i >= 0; i--) { out[small[i].id].prob = small[i].prob; out[small[i].id].failId = small[i].id; }
    out[0].prob = sumAll; out[0].failId = n;
    return GRIS_OK;
}

/* ------------------------------------------------------------------ camera */
static const float kDegToRad = 0.01745329251994329577f;

/* reference: Camera::update (src/Camera.cpp:78-98) with glm::lookAt / glm::perspective
 * (right-handed, depth 0..1) and the Vulkan y flip proj[1][1] *= -1. angle.z is used as
 * radians there (glm::rotate without glm::radians) and is kept so. */
static void camera_update(GrisCamera* cam) {
    float ax = cam->angle[0] * kDegToRad, ay = cam->angle[1] * kDegToRad;
    float sx, cx, sy, cy;
    gris_det_sincosf(ax, &sx, &cx);
    gris_det_sincosf(ay, &sy, &cy);
    H3 look = h3(sx * cy, cx * cy, sy);
    H3 front = hnorm(look);
    H3 right = hnorm(hcross(front, h3(0.0f, 0.0f, 1.0f)));
    /* rotate `right` about `front` by angle.z (Rodrigues; glm::rotate builds the same matrix) */
    float sr, cr;
    gris_det_sincosf(cam->angle[2], &sr, &cr);
    H3 k = front;
    H3 rr = right * cr + hcross(k, right) * sr + k * (hdot(k, right) * (1.0f - cr));
    right = hnorm(rr);
    H3 up = hnorm(hcross(right, front));
    H3 pos = h3(cam->pos[0], cam->pos[1], cam->pos[2]);
    /* view = lookAt(pos, pos + look, up) */
    H3 f = hnorm(look);
    H3 s = hnorm(hcross(f, up));
    H3 u = hcross(s, f);
    M4 view = m4_identity();
    view.m[0] = s.x; view.m[4] = s.y; view.m[8] = s.z;
    view.m[1] = u.x; view.m[5] = u.y; view.m[9] = u.z;
    view.m[2] = -f.x; view.m[6] = -f.y; view.m[10] = -f.z;
    view.m[12] = -hdot(s, pos); view.m[13] = -hdot(u, pos); view.m[14] = hdot(f, pos);
    float aspect = (float)cam->filmSize[0] / (float)cam->filmSize[1];
    float tanHalf = gris_det_tanf(cam->FOV * kDegToRad * 0.5f);
    M4 proj;
    memset(proj.m, 0, sizeof(proj.m));
    proj.m[0] = 1.0f / (aspect * tanHalf);
    proj.m[5] = 1.0f / tanHalf;
    proj.m[10] = cam->farZ / (cam->nearZ - cam->farZ);
    proj.m[11] = -1.0f;
    proj.m[14] = -(cam->farZ * cam->nearZ) / (cam->farZ - cam->nearZ);
    proj.m[5] *= -1.0f;
    M4 pv = m4_mul(proj, view);
    memcpy(cam->view, view.m, 64);
    memcpy(cam->proj, proj.m, 64);
    memcpy(cam->projView, pv.m, 64);
    memcpy(cam->lastProjView, pv.m, 64);
    cam->front[0] = front.x; cam->front[1] = front.y; cam->front[2] = front.z;
    cam->right[0] = right.x; cam->right[1] = right.y; cam->right[2] = right.z;
    cam->up[0] = up.x; cam->up[1] = up.y; cam->up[2] = up.z;
    cam->frameIndex = 0;
}

extern "C" int grisCameraSetup(GrisCamera* cam, const float pos[3], const float angle[3], float fovDeg,
                               uint32_t width, uint32_t height) {
    if (!cam || !pos || !angle || width == 0 || height == 0) return GRIS_ERR_INVALID_ARGUMENT;
    memset(cam, 0, sizeof(*cam));
    for (int i = 0; i < 3; i++) { cam->pos[i] = pos[i]; cam->angle[i] = angle[i]; }
    cam->FOV = std::min(std::max(fovDeg, 0.1f), 90.0f);   /* Camera::setFOV clamp (Camera.cpp:30-34) */
    cam->nearZ = 1e-3f; cam->farZ = 1e3f;                 /* Camera.h:56,59 */
    cam->focalDist = 1.0f;
    cam->filmSize[0] = width; cam->filmSize[1] = height;
    cam->seed = 0;
    camera_update(cam);
    return GRIS_OK;
}

/* Role of Camera::setDir (src/Camera.cpp:36-45): yaw/pitch from a direction, then update().
 * The yaw is taken with atan2 so that update()'s front = (sin yaw cos pitch, cos yaw cos pitch,
 * sin pitch) points at the target (setDir's asin form assumes a different yaw origin). The
 * angles are computed once in double and handed to every consumer as floats. */
extern "C" int grisCameraLookAt(GrisCamera* cam, const float pos[3], const float target[3], float fovDeg,
                                uint32_t width, uint32_t height) {
    if (!cam || !pos || !target) return GRIS_ERR_INVALID_ARGUMENT;
    H3 dir = hnorm(h3(target[0] - pos[0], target[1] - pos[1], target[2] - pos[2]));
    float pitch = (float)(asin((double)dir.z) * 57.29577951308232);
    float yaw = (float)(atan2((double)dir.x, (double)dir.y) * 57.29577951308232);
    float angle[3] = {yaw, pitch, 0.0f};
    return grisCameraSetup(cam, pos, angle, fovDeg, width, height);
}

/* ------------------------------------------------------------------ synthetic scenes */
struct GrisHostScene {
    int kind = 0;
    uint64_t seed = 0;
    std::vector<GrisMeshVertex> vertices;
    std::vector<uint32_t> indices;
    std::vector<GrisObjectInstance> instances;
    std::vector<GrisMaterial> materials;
    std::vector<int32_t> materialIndices;
    std::vector<GrisTriangleLight> lights;
    std::vector<GrisLightTableEntry> table;
    float center[3] = {0, 0, 0};
    float orbitRadius = 1.0f, orbitHeight = 0.0f, fov = 60.0f;
    float camPos[3] = {0, 0, 0}, camAngle[3] = {0, 0, 0};
    /* scenes loaded from a scene file */
    bool camLookAt = false;
    float camTarget[3] = {0, 0, 0};
    uint32_t filmW = 0, filmH = 0;
};

namespace {

struct Rng {   /* splitmix64 */
    uint64_t s;
    uint64_t next() { uint64_t z = (s += 0x9e3779b97f4a7c15ull); z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
                      z = (z ^ (z >> 27)) * 0x94d049bb133111ebull; return z ^ (z >> 31); }
    float uniform() { return (float)(next() >> 40) * (1.0f / 16777216.0f); }   /* [0,1) */
};

GrisMaterial make_material(uint32_t type, H3 color, float metallic, float roughness) {
    GrisMaterial m;
    m.baseColor[0] = color.x; m.baseColor[1] = color.y; m.baseColor[2] = color.z;
    m.type = type; m.textureIdx = 0xffffffffu; m.metallic = metallic; m.roughness = roughness; m.ior = 1.5f;
    return m;
}

void set_instance(GrisObjectInstance& inst, const M4& T, uint32_t indexOffset, uint32_t indexCount, uint32_t matIndex) {
    memset(&inst, 0, sizeof(inst));
    M4 inv = m4_affine_inverse(T);
    M4 invT = m4_transpose(inv);
    memcpy(inst.transform, T.m, 64);
    memcpy(inst.transformInv, inv.m, 64);
    memcpy(inst.transformInvT, invT.m, 64);
    inst.indexOffset = indexOffset; inst.indexCount = indexCount; inst.matIndex = matIndex;
}

/* Adds a quad (a, b, c, d counter-clockwise seen from the side `n` points to) to the mesh. */
void add_quad(GrisHostScene& s, H3 a, H3 b, H3 c, H3 d, H3 n, int32_t mat) {
    uint32_t base = (uint32_t)s.vertices.size();
    H3 p[4] = {a, b, c, d};
    for (int i = 0; i < 4; i++) {
        GrisMeshVertex v;
        v.pos[0] = p[i].x; v.pos[1] = p[i].y; v.pos[2] = p[i].z;
        v.norm[0] = n.x; v.norm[1] = n.y; v.norm[2] = n.z;
        v.uvx = (i == 1 || i == 2) ? 1.0f : 0.0f; v.uvy = (i >= 2) ? 1.0f : 0.0f;
        s.vertices.push_back(v);
    }
    uint32_t idx[6] = {base, base + 1, base + 2, base, base + 2, base + 3};
    for (uint32_t i : idx) s.indices.push_back(i);
    s.materialIndices.push_back(mat);
    s.materialIndices.push_back(mat);
}

/* reference: the light build of Scene::loadModels (src/Scene.cpp:208-291): world-space
 * triangles, n = normalize(cross(v1-v0, v2-v0)), area = |cross|/2, radiance = power / total
 * area of the light mesh (here the radiance is given directly). */
void add_quad_light(GrisHostScene& s, H3 a, H3 b, H3 c, H3 d, H3 radiance) {
    H3 tri[2][3] = {{a, b, c}, {a, c, d}};
    for (auto& t : tri) {
        GrisTriangleLight L;
        memset(&L, 0, sizeof(L));
        H3 n = hcross(t[1] - t[0], t[2] - t[0]);
        L.area = 0.5f * hlen(n);
        n = hnorm(n);
        L.v0[0] = t[0].x; L.v0[1] = t[0].y; L.v0[2] = t[0].z;
        L.v1[0] = t[1].x; L.v1[1] = t[1].y; L.v1[2] = t[1].z;
        L.v2[0] = t[2].x; L.v2[1] = t[2].y; L.v2[2] = t[2].z;
        L.nx = n.x; L.ny = n.y; L.nz = n.z;
        L.radiance[0] = radiance.x; L.radiance[1] = radiance.y; L.radiance[2] = radiance.z;
        s.lights.push_back(L);
    }
}

/* reference: Scene::buildLightDataStructure (src/Scene.cpp:309-322): distribution = luminance(radiance * area). */
void build_light_table(GrisHostScene& s) {
    std::vector<float> power(s.lights.size());
    for (size_t i = 0; i < s.lights.size(); i++) {
        const GrisTriangleLight& L = s.lights[i];
        float r = L.radiance[0] * L.area, g = L.radiance[1] * L.area, b = L.radiance[2] * L.area;
        power[i] = (r * 0.299f + g * 0.587f) + b * 0.114f;
    }
    s.table.resize(s.lights.size() + 1);
    grisBuildLightTable(power.data(), (uint32_t)power.size(), s.table.data());
}

/* Closed room [-1,1]^3 (6 quads, normals inward) + a rotated block (6 quads, normals outward),
 * ceiling light of 1/16 of the ceiling area just under the ceiling, radiance 15. */
void build_box(GrisHostScene& s) {
    Rng rng{s.seed * 0x2545f4914f6cdd1dull + 1};
    for (int q = 0; q < 12; q++) {
        float r = 0.2f + 0.6f * rng.uniform(), g = 0.2f + 0.6f * rng.uniform(), b = 0.2f + 0.6f * rng.uniform();
        s.materials.push_back(make_material(1u, h3(r, g, b), 0.0f, 1.0f));
    }
    /* room: instance 0 (identity) */
    H3 P[8];
    for (int i = 0; i < 8; i++) P[i] = h3((i & 1) ? 1.0f : -1.0f, (i & 2) ? 1.0f : -1.0f, (i & 4) ? 1.0f : -1.0f);
    add_quad(s, P[0], P[1], P[3], P[2], h3(0, 0, 1), 0);     /* floor z=-1, normal +z */
    add_quad(s, P[4], P[6], P[7], P[5], h3(0, 0, -1), 1);    /* ceiling */
    add_quad(s, P[0], P[4], P[5], P[1], h3(0, 1, 0), 2);     /* y=-1 */
    add_quad(s, P[2], P[3], P[7], P[6], h3(0, -1, 0), 3);    /* y=+1 (back wall) */
    add_quad(s, P[0], P[2], P[6], P[4], h3(1, 0, 0), 4);     /* x=-1 */
    add_quad(s, P[1], P[5], P[7], P[3], h3(-1, 0, 0), 5);    /* x=+1 */
    uint32_t roomCount = (uint32_t)s.indices.size();
    /* block: unit cube [-0.5,0.5]^3 mesh, placed by instance 1 */
    uint32_t blockOffset = (uint32_t)s.indices.size();
    for (int i = 0; i < 8; i++) P[i] = h3((i & 1) ? 0.5f : -0.5f, (i & 2) ? 0.5f : -0.5f, (i & 4) ? 0.5f : -0.5f);
    add_quad(s, P[0], P[2], P[3], P[1], h3(0, 0, -1), 6);
    add_quad(s, P[4], P[5], P[7], P[6], h3(0, 0, 1), 7);
    add_quad(s, P[0], P[1], P[5], P[4], h3(0, -1, 0), 8);
    add_quad(s, P[2], P[6], P[7], P[3], h3(0, 1, 0), 9);
    add_quad(s, P[0], P[4], P[6], P[2], h3(-1, 0, 0), 10);
    add_quad(s, P[1], P[3], P[7], P[5], h3(1, 0, 0), 11);
    uint32_t blockCount = (uint32_t)s.indices.size() - blockOffset;
    s.instances.resize(2);
    set_instance(s.instances[0], m4_identity(), 0, roomCount, 0);
    M4 bt = m4_translate_scale_rotz(h3(0.3f, 0.25f, -0.6f), 0.8f, 0.4f);
    set_instance(s.instances[1], bt, blockOffset, blockCount, 6);
    /* ceiling light: 0.5 x 0.5 (1/16 of the 2 x 2 ceiling), facing down */
    float z = 0.999f, h = 0.25f;
    add_quad_light(s, h3(-h, -h, z), h3(-h, h, z), h3(h, h, z), h3(h, -h, z), h3(15.0f, 15.0f, 15.0f));
    build_light_table(s);
    s.camPos[0] = 0.0f; s.camPos[1] = -0.92f; s.camPos[2] = 0.05f;
    s.camAngle[0] = 0.0f; s.camAngle[1] = -4.0f; s.camAngle[2] = 0.0f;
    s.fov = 70.0f;
    s.orbitRadius = 0.0f;
}

/* value noise on an integer lattice (hash of the cell corners), smooth-step interpolated */
float lattice(uint64_t seed, int ix, int iy) {
    uint64_t h = seed ^ ((uint64_t)(uint32_t)ix * 0x9e3779b97f4a7c15ull) ^ ((uint64_t)(uint32_t)iy * 0xc2b2ae3d27d4eb4full);
    Rng r{h};
    return r.uniform() * 2.0f - 1.0f;
}
float value_noise(uint64_t seed, float x, float y) {
    float fx = floorf(x), fy = floorf(y);
    int ix = (int)fx, iy = (int)fy;
    float tx = x - fx, ty = y - fy;
    tx = tx * tx * (3.0f - 2.0f * tx);
    ty = ty * ty * (3.0f - 2.0f * ty);
    float a = lattice(seed, ix, iy), b = lattice(seed, ix + 1, iy);
    float c = lattice(seed, ix, iy + 1), d = lattice(seed, ix + 1, iy + 1);
    float top = a + (b - a) * tx, bot = c + (d - c) * tx;
    return top + (bot - top) * ty;
}
float fbm(uint64_t seed, float x, float y) {
    float sum = 0.0f, amp = 0.5f, freq = 1.0f;
    for (int o = 0; o < 6; o++) {
        sum += amp * value_noise(seed + (uint64_t)o * 7919u, x * freq, y * freq);
        amp *= 0.5f; freq *= 2.0f;
    }
    return sum;
}

/* Icosphere of the given subdivision level (unit radius, outward normals). */
void icosphere(int level, std::vector<H3>& V, std::vector<uint32_t>& F) {
    const float t = 1.6180339887498949f;
    H3 base[12] = {h3(-1, t, 0), h3(1, t, 0), h3(-1, -t, 0), h3(1, -t, 0), h3(0, -1, t), h3(0, 1, t),
                   h3(0, -1, -t), h3(0, 1, -t), h3(t, 0, -1), h3(t, 0, 1), h3(-t, 0, -1), h3(-t, 0, 1)};
    uint32_t faces[60] = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6, 7, 1, 8,
                          3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1};
    V.clear(); F.assign(faces, faces + 60);
    for (H3 p : base) V.push_back(hnorm(p));
    for (int l = 0; l < level; l++) {
        std::vector<uint32_t> nf;
        std::vector<std::pair<uint64_t, uint32_t>> cache;
        auto mid = [&](uint32_t a, uint32_t b) {
            uint64_t key = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
            for (auto& e : cache) if (e.first == key) return e.second;
            V.push_back(hnorm((V[a] + V[b]) * 0.5f));
            cache.push_back({key, (uint32_t)V.size() - 1});
            return (uint32_t)V.size() - 1;
        };
        for (size_t f = 0; f < F.size(); f += 3) {
            uint32_t a = F[f], b = F[f + 1], c = F[f + 2];
            uint32_t ab = mid(a, b), bc = mid(b, c), ca = mid(c, a);
            uint32_t add[12] = {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca};
            nf.insert(nf.end(), add, add + 12);
        }
        F.swap(nf);
    }
}

/* kind 3: the box room of kind 0 furnished with `spheres` instanced level-2 icospheres (320
 * triangles each) resting at random places inside it, Lambertian or GGX. */
void build_box_spheres(GrisHostScene& s, uint32_t spheres) {
    build_box(s);
    Rng rng{s.seed * 0x9e3779b97f4a7c15ull + 3};
    std::vector<H3> SV; std::vector<uint32_t> SF;
    icosphere(2, SV, SF);
    uint32_t sBase = (uint32_t)s.vertices.size();
    for (H3 p : SV) {
        GrisMeshVertex v;
        v.pos[0] = p.x; v.pos[1] = p.y; v.pos[2] = p.z;
        v.norm[0] = p.x; v.norm[1] = p.y; v.norm[2] = p.z;
        v.uvx = 0.0f; v.uvy = 0.0f;
        s.vertices.push_back(v);
    }
    for (uint32_t k = 0; k < spheres; k++) {
        float radius = 0.02f + 0.1f * rng.uniform();
        float px = -0.9f + 1.8f * rng.uniform();
        float py = -0.9f + 1.8f * rng.uniform();
        float pz = -1.0f + radius + 1.4f * rng.uniform();
        float cr = 0.2f + 0.75f * rng.uniform();
        float cg = 0.2f + 0.75f * rng.uniform();
        float cb = 0.2f + 0.75f * rng.uniform();
        float rough = 0.05f + 0.95f * rng.uniform();
        float metal = rng.uniform() < 0.3f ? 1.0f : 0.0f;
        uint32_t type = rng.uniform() < 0.5f ? 1u : 2u;
        uint32_t mat = (uint32_t)s.materials.size();
        s.materials.push_back(make_material(type, h3(cr, cg, cb), metal, rough));
        uint32_t off = (uint32_t)s.indices.size();
        for (uint32_t f : SF) s.indices.push_back(sBase + f);
        for (size_t f = 0; f < SF.size() / 3; f++) s.materialIndices.push_back((int32_t)mat);
        s.instances.emplace_back();
        float rot = 6.2831853f * rng.uniform();
        set_instance(s.instances.back(), m4_translate_scale_rotz(h3(px, py, pz), radius, rot), off, (uint32_t)SF.size(), mat);
    }
}

/* kind 1 / 2: heightfield + instanced icospheres + 4 quad lights. */
void build_terrain(GrisHostScene& s, uint32_t gridN, uint32_t spheres, bool glossy) {
    Rng rng{s.seed * 0x9e3779b97f4a7c15ull + 7};
    const float L = 50.0f, amp = 6.0f;
    if (gridN < 2) gridN = 2;
    /* terrain material 0 */
    s.materials.push_back(make_material(2u, h3(0.45f, 0.42f, 0.35f), 0.0f, glossy ? 0.25f : 0.8f));
    uint32_t tOffset = 0;
    std::vector<float> hgt((size_t)gridN * gridN);
    auto hx = [&](uint32_t i) { return -L + 2.0f * L * (float)i / (float)(gridN - 1); };
    for (uint32_t j = 0; j < gridN; j++)
        for (uint32_t i = 0; i < gridN; i++)
            hgt[(size_t)j * gridN + i] = amp * fbm(s.seed + 17u, hx(i) * 0.035f + 3.1f, hx(j) * 0.035f - 1.7f);
    float cell = 2.0f * L / (float)(gridN - 1);
    for (uint32_t j = 0; j < gridN; j++)
        for (uint32_t i = 0; i < gridN; i++) {
            uint32_t i0 = i > 0 ? i - 1 : i, i1 = i + 1 < gridN ? i + 1 : i;
            uint32_t j0 = j > 0 ? j - 1 : j, j1 = j + 1 < gridN ? j + 1 : j;
            float dx = (hgt[(size_t)j * gridN + i1] - hgt[(size_t)j * gridN + i0]) / ((float)(i1 - i0) * cell);
            float dy = (hgt[(size_t)j1 * gridN + i] - hgt[(size_t)j0 * gridN + i]) / ((float)(j1 - j0) * cell);
            H3 n = hnorm(h3(-dx, -dy, 1.0f));
            GrisMeshVertex v;
            v.pos[0] = hx(i); v.pos[1] = hx(j); v.pos[2] = hgt[(size_t)j * gridN + i];
            v.norm[0] = n.x; v.norm[1] = n.y; v.norm[2] = n.z;
            v.uvx = (float)i / (float)(gridN - 1); v.uvy = (float)j / (float)(gridN - 1);
            s.vertices.push_back(v);
        }
    for (uint32_t j = 0; j + 1 < gridN; j++)
        for (uint32_t i = 0; i + 1 < gridN; i++) {
            uint32_t a = j * gridN + i, b = a + 1, c = a + gridN + 1, d = a + gridN;
            uint32_t q[6] = {a, b, c, a, c, d};
            s.indices.insert(s.indices.end(), q, q + 6);
            s.materialIndices.push_back(0);
            s.materialIndices.push_back(0);
        }
    uint32_t tCount = (uint32_t)s.indices.size();
    s.instances.emplace_back();
    set_instance(s.instances.back(), m4_identity(), tOffset, tCount, 0);
    /* icosphere mesh shared by every sphere instance; each instance gets its own index range
     * (same vertices) so its triangles can carry its own material index */
    std::vector<H3> SV; std::vector<uint32_t> SF;
    icosphere(2, SV, SF);
    uint32_t sBase = (uint32_t)s.vertices.size();
    for (H3 p : SV) {
        GrisMeshVertex v;
        v.pos[0] = p.x; v.pos[1] = p.y; v.pos[2] = p.z;
        v.norm[0] = p.x; v.norm[1] = p.y; v.norm[2] = p.z;
        v.uvx = 0.0f; v.uvy = 0.0f;
        s.vertices.push_back(v);
    }
    for (uint32_t k = 0; k < spheres; k++) {
        float radius = (float)(0.1 * gris_det_exp((double)rng.uniform() * 2.995732273553991));   /* 0.1 * 20^u */
        float px = -L * 0.9f + 1.8f * L * rng.uniform(), py = -L * 0.9f + 1.8f * L * rng.uniform();
        /* terrain height under the centre (nearest grid vertex) */
        uint32_t gi = (uint32_t)((px + L) / cell + 0.5f), gj = (uint32_t)((py + L) / cell + 0.5f);
        if (gi >= gridN) gi = gridN - 1;
        if (gj >= gridN) gj = gridN - 1;
        float pz = hgt[(size_t)gj * gridN + gi] + radius * 0.7f;
        /* one draw per statement: the order of evaluation of function arguments is unspecified */
        float cr = 0.2f + 0.75f * rng.uniform();
        float cg = 0.2f + 0.75f * rng.uniform();
        float cb = 0.2f + 0.75f * rng.uniform();
        H3 col = h3(cr, cg, cb);
        float rough, metal;
        if (glossy) { rough = 0.02f + 0.28f * rng.uniform(); metal = rng.uniform() < 0.7f ? 1.0f : 0.0f; }
        else { rough = 0.05f + 0.95f * rng.uniform(); metal = rng.uniform() < 0.3f ? 1.0f : 0.0f; }
        uint32_t mat = (uint32_t)s.materials.size();
        s.materials.push_back(make_material(2u, col, metal, rough));
        uint32_t off = (uint32_t)s.indices.size();
        for (uint32_t f : SF) s.indices.push_back(sBase + f);
        for (size_t f = 0; f < SF.size() / 3; f++) s.materialIndices.push_back((int32_t)mat);
        s.instances.emplace_back();
        float rot = 6.2831853f * rng.uniform();
        set_instance(s.instances.back(), m4_translate_scale_rotz(h3(px, py, pz), radius, rot), off, (uint32_t)SF.size(), mat);
    }
    /* four 8 x 8 quad lights at height 22: facing down; in the glossy variant facing up under a
     * white Lambertian bounce panel, so no light reaches the ground directly and the energy
     * arrives after 2+ bounces */
    H3 lightPos[4] = {h3(-20, -20, 22), h3(20, -20, 22), h3(20, 20, 22), h3(-20, 20, 22)};
    H3 lightCol[4] = {h3(40, 36, 30), h3(30, 34, 40), h3(40, 40, 40), h3(36, 30, 40)};
    for (int l = 0; l < 4; l++) {
        H3 c = lightPos[l];
        float h = 4.0f;
        if (!glossy) {
            add_quad_light(s, h3(c.x - h, c.y - h, c.z), h3(c.x - h, c.y + h, c.z), h3(c.x + h, c.y + h, c.z),
                           h3(c.x + h, c.y - h, c.z), lightCol[l]);
            continue;
        }
        add_quad_light(s, h3(c.x - h, c.y - h, c.z), h3(c.x + h, c.y - h, c.z), h3(c.x + h, c.y + h, c.z),
                       h3(c.x - h, c.y + h, c.z), lightCol[l] * 4.0f);
        uint32_t mat = (uint32_t)s.materials.size();
        s.materials.push_back(make_material(1u, h3(0.85f, 0.85f, 0.85f), 0.0f, 1.0f));
        uint32_t off = (uint32_t)s.indices.size();
        float ph = 12.0f, pz = c.z + 4.0f;
        add_quad(s, h3(c.x - ph, c.y - ph, pz), h3(c.x - ph, c.y + ph, pz), h3(c.x + ph, c.y + ph, pz),
                 h3(c.x + ph, c.y - ph, pz), h3(0, 0, -1), (int32_t)mat);
        s.instances.emplace_back();
        set_instance(s.instances.back(), m4_identity(), off, 6, mat);
    }
    build_light_table(s);
    s.center[0] = 0.0f; s.center[1] = 0.0f; s.center[2] = 0.0f;
    s.orbitRadius = 38.0f; s.orbitHeight = 14.0f; s.fov = 60.0f;
}

}  // namespace

extern "C" int grisHostSceneCreate(int kind, uint64_t seed, uint32_t gridN, uint32_t spheres, GrisHostScene** out) {
    if (!out || kind < 0 || kind > 3) return GRIS_ERR_INVALID_ARGUMENT;
    GrisHostScene* s = new GrisHostScene();
    s->kind = kind; s->seed = seed;
    if (kind == 0) build_box(*s);
    else if (kind == 3) build_box_spheres(*s, spheres);
    else build_terrain(*s, gridN ? gridN : 512, spheres, kind == 2);
    *out = s;
    return GRIS_OK;
}

extern "C" int grisHostSceneDesc(const GrisHostScene* s, GrisSceneDesc* d) {
    if (!s || !d) return GRIS_ERR_INVALID_ARGUMENT;
    d->vertices = s->vertices.data(); d->vertexCount = s->vertices.size();
    d->indices = s->indices.data(); d->indexCount = s->indices.size();
    d->instances = s->instances.data(); d->instanceCount = s->instances.size();
    d->materials = s->materials.data(); d->materialCount = s->materials.size();
    d->materialIndices = s->materialIndices.data(); d->materialIndexCount = s->materialIndices.size();
    d->lights = s->lights.data(); d->lightCount = s->lights.size();
    d->lightTable = s->table.data(); d->lightTableCount = s->table.size();
    return GRIS_OK;
}

/* Camera of frame `frame` of `frames`: the box scene's fixed camera, or a quarter orbit
 * around the terrain centre for the terrain scenes. */
extern "C" int grisHostSceneCamera(const GrisHostScene* s, uint32_t frame, uint32_t frames, uint32_t width,
                                   uint32_t height, GrisCamera* out) {
    if (!s || !out) return GRIS_ERR_INVALID_ARGUMENT;
    if (s->camLookAt) return grisCameraLookAt(out, s->camPos, s->camTarget, s->fov, width, height);
    if (s->orbitRadius <= 0.0f) return grisCameraSetup(out, s->camPos, s->camAngle, s->fov, width, height);
    float a = 0.7853982f + 1.5707964f * (float)frame / (float)(frames > 1 ? frames : 1);
    float sa, ca;
    gris_det_sincosf(a, &sa, &ca);
    float pos[3] = {s->center[0] + s->orbitRadius * ca, s->center[1] + s->orbitRadius * sa, s->center[2] + s->orbitHeight};
    float tgt[3] = {s->center[0], s->center[1], s->center[2] - 2.0f};
    return grisCameraLookAt(out, pos, tgt, s->fov, width, height);
}

extern "C" int grisHostSceneDestroy(GrisHostScene* s) {
    delete s;
    return GRIS_OK;
}

/* ------------------------------------------------------------------ scene files */
/* The reference's scene description (src/Scene.cpp:131-303, src/Material.cpp:5-70): an XML
 * document <scene> with <integrator><size width height/></integrator>, <camera> (<position
 * value="x y z"/>, <angle value="yaw pitch roll"/> or <lookAt value="x y z"/>, <fov value/>),
 * and <modelInstances> whose children name a mesh file (path relative to the scene file), a
 * <transform translate scale rotate/> (model matrix as src/Model.cpp:11-21: translate, rotate
 * rot.x about z, rot.y + 90 degrees about x, rot.z about y, scale (s.x, s.z, s.y)), for
 * type="light" a <radiance value/> (the light's power, spread over its world-space area) and an
 * optional flip="true", and otherwise an optional <material type=...> overriding the mesh's
 * materials (lambertian, metalWorkflow, metal, dielectric, thinDielectric, fake; "default"
 * keeps the mesh file's) with <baseColor value/>, <metallic/>, <roughness/>, <ior/>.
 * Meshes are Wavefront OBJ (+ MTL diffuse colours), read by a small loader standing in for the
 * reference's assimp import: polygons fan-triangulated, a vertex per face corner, texture v
 * flipped, missing normals generated (objects: the mean of the unit face normals at each
 * position; lights: flat). Image textures are rejected (the GRIS kernels read base colours). */
namespace {

struct XmlNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<XmlNode> kids;
    const char* attr(const char* k) const {
        for (auto& a : attrs) if (a.first == k) return a.second.c_str();
        return nullptr;
    }
    const XmlNode* child(const char* k) const {
        for (auto& c : kids) if (c.name == k) return &c;
        return nullptr;
    }
};

struct XmlParser {
    const std::string& t;
    size_t i = 0;
    std::string err;
    explicit XmlParser(const std::string& text) : t(text) {}
    void ws() { while (i < t.size() && isspace((unsigned char)t[i])) i++; }
    bool starts(const char* p) const { return t.compare(i, strlen(p), p) == 0; }
    bool skip_misc() {   /* comments, processing instructions, doctype, text */
        for (;;) {
            while (i < t.size() && t[i] != '<') i++;
            if (i >= t.size()) return false;
            if (starts("<!--")) { size_t e = t.find("-->", i); if (e == std::string::npos) return false; i = e + 3; continue; }
            if (starts("<?") || starts("<!")) { size_t e = t.find('>', i); if (e == std::string::npos) return false; i = e + 1; continue; }
            return true;
        }
    }
    static std::string unescape(const std::string& v) {
        std::string r;
        for (size_t k = 0; k < v.size(); k++) {
            if (v[k] == '&') {
                static const char* ent[][2] = {{"&amp;", "&"}, {"&lt;", "<"}, {"&gt;", ">"}, {"&quot;", "\""}, {"&apos;", "'"}};
                bool done = false;
                for (auto& e : ent)
                    if (v.compare(k, strlen(e[0]), e[0]) == 0) { r += e[1]; k += strlen(e[0]) - 1; done = true; break; }
                if (!done) r += v[k];
            } else {
                r += v[k];
            }
        }
        return r;
    }
    bool element(XmlNode& n, int depth) {
        if (depth > 64) { err = "nesting too deep"; return false; }
        if (!skip_misc() || t[i] != '<') { err = "expected an element"; return false; }
        i++;
        size_t b = i;
        while (i < t.size() && !isspace((unsigned char)t[i]) && t[i] != '>' && t[i] != '/') i++;
        n.name = t.substr(b, i - b);
        for (;;) {
            ws();
            if (i >= t.size()) { err = "unterminated tag"; return false; }
            if (t[i] == '/') { if (i + 1 < t.size() && t[i + 1] == '>') { i += 2; return true; } err = "bad tag end"; return false; }
            if (t[i] == '>') { i++; break; }
            size_t k = i;
            while (i < t.size() && t[i] != '=' && !isspace((unsigned char)t[i])) i++;
            std::string key = t.substr(k, i - k);
            ws();
            if (i >= t.size() || t[i] != '=') { err = "attribute without value"; return false; }
            i++;
            ws();
            if (i >= t.size() || (t[i] != '"' && t[i] != '\'')) { err = "unquoted attribute"; return false; }
            char q = t[i++];
            size_t e = t.find(q, i);
            if (e == std::string::npos) { err = "unterminated attribute"; return false; }
            n.attrs.push_back({key, unescape(t.substr(i, e - i))});
            i = e + 1;
        }
        for (;;) {
            if (!skip_misc()) { err = "unterminated element " + n.name; return false; }
            if (starts("</")) {
                size_t e = t.find('>', i);
                if (e == std::string::npos) { err = "bad closing tag"; return false; }
                i = e + 1;
                return true;
            }
            n.kids.emplace_back();
            if (!element(n.kids.back(), depth + 1)) return false;
        }
    }
};

bool read_file(const std::string& path, std::string& out) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return false;
    char buf[65536];
    size_t n;
    while ((n = fread(buf, 1, sizeof(buf), f)) > 0) out.append(buf, n);
    fclose(f);
    return true;
}

std::string dir_of(const std::string& p) {
    size_t k = p.find_last_of('/');
    return k == std::string::npos ? std::string(".") : p.substr(0, k);
}

bool parse_floats(const char* v, float* out, int n) {
    if (!v) return false;
    const char* p = v;
    for (int k = 0; k < n; k++) {
        char* e = nullptr;
        double d = strtod(p, &e);
        if (e == p) return false;
        out[k] = (float)d;
        p = e;
    }
    return true;
}

struct ObjMesh {            /* one material group of an OBJ file, a vertex per face corner */
    std::vector<GrisMeshVertex> verts;
    int material = -1;      /* index into ObjModel::materials, or -1 */
};
struct ObjModel {
    std::vector<ObjMesh> meshes;
    std::vector<H3> materials;   /* MTL diffuse colours */
};

bool load_mtl(const std::string& path, std::vector<std::string>& names, std::vector<H3>& kd) {
    std::string text;
    if (!read_file(path, text)) return false;
    size_t pos = 0;
    while (pos < text.size()) {
        size_t e = text.find('\n', pos);
        std::string line = text.substr(pos, e == std::string::npos ? std::string::npos : e - pos);
        pos = e == std::string::npos ? text.size() : e + 1;
        char word[64] = {0};
        if (sscanf(line.c_str(), "%63s", word) != 1) continue;
        if (!strcmp(word, "newmtl")) {
            char name[256] = {0};
            sscanf(line.c_str(), "%*s %255s", name);
            names.push_back(name);
            kd.push_back(h3(0.6f, 0.6f, 0.6f));
        } else if (!strcmp(word, "Kd") && !kd.empty()) {
            float c[3];
            if (sscanf(line.c_str(), "%*s %f %f %f", &c[0], &c[1], &c[2]) == 3) kd.back() = h3(c[0], c[1], c[2]);
        }
    }
    return true;
}

bool load_obj(const std::string& path, bool light, ObjModel& m, std::string& err) {
    std::string text;
    if (!read_file(path, text)) { err = "cannot read " + path; return false; }
    std::vector<H3> P, N;
    std::vector<float> UV;
    std::vector<std::string> mtlNames;
    std::vector<H3> mtlKd;
    int current = -1;
    m.meshes.emplace_back();
    std::vector<std::vector<int>> hasN(1);
    size_t pos = 0;
    while (pos < text.size()) {
        size_t e = text.find('\n', pos);
        std::string line = text.substr(pos, e == std::string::npos ? std::string::npos : e - pos);
        pos = e == std::string::npos ? text.size() : e + 1;
        const char* c = line.c_str();
        while (*c == ' ' || *c == '\t') c++;
        if (c[0] == 'v' && (c[1] == ' ' || c[1] == '\t')) {
            float v[3] = {0, 0, 0};
            sscanf(c + 1, "%f %f %f", &v[0], &v[1], &v[2]);
            P.push_back(h3(v[0], v[1], v[2]));
        } else if (c[0] == 'v' && c[1] == 'n') {
            float v[3] = {0, 0, 0};
            sscanf(c + 2, "%f %f %f", &v[0], &v[1], &v[2]);
            N.push_back(h3(v[0], v[1], v[2]));
        } else if (c[0] == 'v' && c[1] == 't') {
            float v[2] = {0, 0};
            sscanf(c + 2, "%f %f", &v[0], &v[1]);
            UV.push_back(v[0]); UV.push_back(v[1]);
        } else if (!strncmp(c, "mtllib", 6)) {
            char name[512] = {0};
            if (sscanf(c + 6, "%511s", name) == 1) load_mtl(dir_of(path) + "/" + name, mtlNames, mtlKd);
        } else if (!strncmp(c, "usemtl", 6)) {
            char name[256] = {0};
            sscanf(c + 6, "%255s", name);
            int idx = -1;
            for (size_t k = 0; k < mtlNames.size(); k++) if (mtlNames[k] == name) idx = (int)k;
            if (idx != current) {
                current = idx;
                if (!m.meshes.back().verts.empty()) { m.meshes.emplace_back(); hasN.emplace_back(); }
                m.meshes.back().material = idx;
            }
        } else if (c[0] == 'f' && (c[1] == ' ' || c[1] == '\t')) {
            struct Corner { int p, t, n; };
            std::vector<Corner> poly;
            const char* q = c + 1;
            for (;;) {
                while (*q == ' ' || *q == '\t') q++;
                if (!*q || *q == '\r') break;
                Corner k = {0, 0, 0};
                char* endp = nullptr;
                k.p = (int)strtol(q, &endp, 10);
                q = endp;
                if (*q == '/') {
                    q++;
                    if (*q != '/') { k.t = (int)strtol(q, &endp, 10); q = endp; }
                    if (*q == '/') { q++; k.n = (int)strtol(q, &endp, 10); q = endp; }
                }
                while (*q && *q != ' ' && *q != '\t') q++;
                auto fix = [](int i, size_t n) { return i < 0 ? (int)n + i : i - 1; };   /* 1-based or negative */
                k.p = fix(k.p, P.size());
                k.t = k.t ? fix(k.t, UV.size() / 2) : -1;
                k.n = k.n ? fix(k.n, N.size()) : -1;
                if (k.p < 0 || k.p >= (int)P.size() || k.t >= (int)(UV.size() / 2) || k.n >= (int)N.size()) {
                    err = path + ": face index out of range";
                    return false;
                }
                poly.push_back(k);
            }
            for (size_t j = 1; j + 1 < poly.size(); j++) {
                const Corner tri[3] = {poly[0], poly[j], poly[j + 1]};
                H3 fn = hcross(P[tri[1].p] - P[tri[0].p], P[tri[2].p] - P[tri[0].p]);
                float fl = hlen(fn);
                fn = fl > 0.0f ? fn * (1.0f / fl) : h3(0, 0, 1);
                for (const Corner& k : tri) {
                    GrisMeshVertex v;
                    v.pos[0] = P[k.p].x; v.pos[1] = P[k.p].y; v.pos[2] = P[k.p].z;
                    H3 n = k.n >= 0 ? N[k.n] : fn;
                    v.norm[0] = n.x; v.norm[1] = n.y; v.norm[2] = n.z;
                    v.uvx = k.t >= 0 ? UV[2 * k.t] : 0.0f;
                    v.uvy = k.t >= 0 ? 1.0f - UV[2 * k.t + 1] : 0.0f;
                    m.meshes.back().verts.push_back(v);
                    hasN.back().push_back(k.n >= 0 ? 1 : 0);
                }
            }
        }
    }
    if (m.meshes.back().verts.empty() && m.meshes.size() > 1) { m.meshes.pop_back(); hasN.pop_back(); }
    if (!light) {
        /* smooth normals where the file has none: the mean of the unit face normals at each position */
        for (size_t mi = 0; mi < m.meshes.size(); mi++) {
            auto& V = m.meshes[mi].verts;
            std::map<std::tuple<float, float, float>, H3> acc;
            for (size_t k = 0; k < V.size(); k++) {
                if (hasN[mi][k]) continue;
                auto key = std::make_tuple(V[k].pos[0], V[k].pos[1], V[k].pos[2]);
                H3 n = h3(V[k].norm[0], V[k].norm[1], V[k].norm[2]);
                auto it = acc.find(key);
                acc[key] = it == acc.end() ? n : it->second + n;
            }
            for (size_t k = 0; k < V.size(); k++) {
                if (hasN[mi][k]) continue;
                H3 n = acc[std::make_tuple(V[k].pos[0], V[k].pos[1], V[k].pos[2])];
                float l = hlen(n);
                if (l > 0.0f) { n = n * (1.0f / l); V[k].norm[0] = n.x; V[k].norm[1] = n.y; V[k].norm[2] = n.z; }
            }
        }
    }
    m.materials = mtlKd;
    return true;
}

M4 m4_rot(float deg, int axis) {
    float s, c;
    gris_det_sincosf(deg * 0.017453292519943295f, &s, &c);
    M4 r = m4_identity();
    int a = (axis + 1) % 3, b = (axis + 2) % 3;   /* rotation in the (a, b) plane, counter-clockwise */
    r.m[a * 4 + a] = c; r.m[b * 4 + a] = -s;
    r.m[a * 4 + b] = s; r.m[b * 4 + b] = c;
    return r;
}

}  // namespace

namespace grisrt {
/* reference: ModelInstance::modelMatrix (src/Model.cpp:11-21) */
M4 model_matrix(const float pos[3], const float scale[3], const float rot[3]) {
    M4 t = m4_identity();
    t.m[12] = pos[0]; t.m[13] = pos[1]; t.m[14] = pos[2];
    M4 m = m4_mul(t, m4_rot(rot[0], 2));
    m = m4_mul(m, m4_rot(rot[1] + 90.0f, 0));
    m = m4_mul(m, m4_rot(rot[2], 1));
    M4 sc = m4_identity();
    sc.m[0] = scale[0]; sc.m[5] = scale[2]; sc.m[10] = scale[1];
    return m4_mul(m, sc);
}
}  // namespace grisrt

static int xml_fail(char* errBuf, size_t errLen, const std::string& msg) {
    if (errBuf && errLen) {
        strncpy(errBuf, msg.c_str(), errLen - 1);
        errBuf[errLen - 1] = 0;
    }
    return GRIS_ERR_INVALID_ARGUMENT;
}

extern "C" int grisHostSceneLoad(const char* path, GrisHostScene** out, char* errBuf, size_t errLen) {
    if (!path || !out) return xml_fail(errBuf, errLen, "null argument");
    *out = nullptr;
    std::string text;
    if (!read_file(path, text)) return xml_fail(errBuf, errLen, std::string("cannot read ") + path);
    XmlParser xp(text);
    XmlNode root;
    if (!xp.element(root, 0)) return xml_fail(errBuf, errLen, std::string(path) + ": " + xp.err);
    if (root.name != "scene") return xml_fail(errBuf, errLen, std::string(path) + ": the root element is not <scene>");
    std::unique_ptr<GrisHostScene> s(new GrisHostScene());
    s->kind = -1;
    s->orbitRadius = 0.0f;
    const std::string base = dir_of(path);
    if (const XmlNode* integ = root.child("integrator"))
        if (const XmlNode* size = integ->child("size")) {
            const char* w = size->attr("width");
            const char* h = size->attr("height");
            s->filmW = w ? (uint32_t)atoi(w) : 0;
            s->filmH = h ? (uint32_t)atoi(h) : 0;
        }
    if (const XmlNode* cam = root.child("camera")) {
        const XmlNode* p = cam->child("position");
        if (p) parse_floats(p->attr("value"), s->camPos, 3);
        if (const XmlNode* a = cam->child("angle")) parse_floats(a->attr("value"), s->camAngle, 3);
        else if (const XmlNode* l = cam->child("lookAt")) { s->camLookAt = parse_floats(l->attr("value"), s->camTarget, 3); }
        if (const XmlNode* f = cam->child("fov")) parse_floats(f->attr("value"), &s->fov, 1);
    }
    /* materials[0]: the default (magenta) material of an empty resource (src/Resource.cpp:36-40) */
    s->materials.push_back(make_material(1u, h3(1.0f, 0.0f, 1.0f), 0.0f, 1.0f));
    std::vector<float> lightPower;
    const XmlNode* models = root.child("modelInstances");
    if (models) for (const XmlNode& mi : models->kids) {
        const char* rel = mi.attr("path");
        if (!rel) return xml_fail(errBuf, errLen, "a model instance without a path");
        const bool isLight = mi.attr("type") && !strcmp(mi.attr("type"), "light");
        ObjModel obj;
        std::string err;
        if (!load_obj(base + "/" + rel, isLight, obj, err)) return xml_fail(errBuf, errLen, err);
        float pos[3] = {0, 0, 0}, scale[3] = {1, 1, 1}, rot[3] = {0, 0, 0};
        if (const XmlNode* tr = mi.child("transform")) {
            if (tr->attr("translate")) parse_floats(tr->attr("translate"), pos, 3);
            if (tr->attr("scale")) parse_floats(tr->attr("scale"), scale, 3);
            if (tr->attr("rotate")) parse_floats(tr->attr("rotate"), rot, 3);
        }
        M4 M = model_matrix(pos, scale, rot);
        if (isLight) {
            float power[3] = {0, 0, 0};
            if (const XmlNode* r = mi.child("radiance")) parse_floats(r->attr("value"), power, 3);
            const bool flip = mi.attr("flip") && !strcmp(mi.attr("flip"), "true");
            size_t first = s->lights.size();
            float area = 0.0f;   /* summed serially, in triangle order */
            for (const ObjMesh& mesh : obj.meshes)
                for (size_t k = 0; k + 2 < mesh.verts.size(); k += 3) {
                    H3 w[3];
                    for (int j = 0; j < 3; j++) {
                        const float* p = mesh.verts[k + j].pos;
                        w[j] = h3(((M.m[0] * p[0] + M.m[4] * p[1]) + M.m[8] * p[2]) + M.m[12],
                                  ((M.m[1] * p[0] + M.m[5] * p[1]) + M.m[9] * p[2]) + M.m[13],
                                  ((M.m[2] * p[0] + M.m[6] * p[1]) + M.m[10] * p[2]) + M.m[14]);
                    }
                    GrisTriangleLight L;
                    memset(&L, 0, sizeof(L));
                    H3 n = hcross(w[1] - w[0], w[2] - w[0]);
                    L.area = 0.5f * hlen(n);
                    n = hnorm(n);
                    if (flip) n = n * -1.0f;
                    L.v0[0] = w[0].x; L.v0[1] = w[0].y; L.v0[2] = w[0].z;
                    L.v1[0] = w[1].x; L.v1[1] = w[1].y; L.v1[2] = w[1].z;
                    L.v2[0] = w[2].x; L.v2[1] = w[2].y; L.v2[2] = w[2].z;
                    L.nx = n.x; L.ny = n.y; L.nz = n.z;
                    area += L.area;
                    s->lights.push_back(L);
                }
            for (size_t k = first; k < s->lights.size(); k++)
                for (int c = 0; c < 3; c++) s->lights[k].radiance[c] = power[c] / area;
            continue;
        }
        /* materials of this model: the MTL colours (or the default), overridden by <material> */
        std::vector<uint32_t> matOf(obj.meshes.size());
        const XmlNode* mat = mi.child("material");
        const char* mtype = mat ? mat->attr("type") : nullptr;
        const bool override = mtype && strcmp(mtype, "default") != 0;
        for (size_t k = 0; k < obj.meshes.size(); k++) {
            GrisMaterial g = make_material(1u, h3(1.0f, 1.0f, 1.0f), 0.0f, 1.0f);
            int src = obj.meshes[k].material;
            if (src >= 0 && src < (int)obj.materials.size()) {
                g.baseColor[0] = obj.materials[src].x; g.baseColor[1] = obj.materials[src].y; g.baseColor[2] = obj.materials[src].z;
            }
            if (override) {
                static const char* names[] = {"principled", "lambertian", "metalWorkflow", "metal", "dielectric", "thinDielectric", "fake"};
                int type = -1;
                for (int t = 0; t < 7; t++) if (!strcmp(mtype, names[t])) type = t;
                if (type < 1) return xml_fail(errBuf, errLen, std::string("unsupported material type ") + mtype);
                g.type = (uint32_t)type;
                g.metallic = 0.0f; g.roughness = 1.0f; g.ior = 1.5f;
                if (const XmlNode* c = mat->child("metallic")) parse_floats(c->attr("value"), &g.metallic, 1);
                if (const XmlNode* c = mat->child("roughness")) parse_floats(c->attr("value"), &g.roughness, 1);
                if (const XmlNode* c = mat->child("ior")) parse_floats(c->attr("value"), &g.ior, 1);
                if (const XmlNode* bc = mat->child("baseColor")) {
                    if (bc->attr("image")) return xml_fail(errBuf, errLen, "image textures are not supported");
                    if (bc->attr("value")) parse_floats(bc->attr("value"), g.baseColor, 3);
                    else { g.baseColor[0] = g.baseColor[1] = g.baseColor[2] = 1.0f; }
                }
            }
            matOf[k] = (uint32_t)s->materials.size();
            s->materials.push_back(g);
        }
        uint32_t indexOffset = (uint32_t)s->indices.size();
        for (size_t k = 0; k < obj.meshes.size(); k++) {
            const ObjMesh& mesh = obj.meshes[k];
            uint32_t vbase = (uint32_t)s->vertices.size();
            for (const GrisMeshVertex& v : mesh.verts) s->vertices.push_back(v);
            for (uint32_t j = 0; j < (uint32_t)mesh.verts.size(); j++) s->indices.push_back(vbase + j);
            for (size_t f = 0; f < mesh.verts.size() / 3; f++) s->materialIndices.push_back((int32_t)matOf[k]);
        }
        uint32_t indexCount = (uint32_t)s->indices.size() - indexOffset;
        s->instances.emplace_back();
        set_instance(s->instances.back(), M, indexOffset, indexCount, obj.meshes.empty() ? 0u : matOf[0]);
    }
    if (s->lights.empty()) return xml_fail(errBuf, errLen, "the scene has no light");
    build_light_table(*s);
    *out = s.release();
    return GRIS_OK;
}

extern "C" int grisHostSceneFilmSize(const GrisHostScene* s, uint32_t* width, uint32_t* height) {
    if (!s || !width || !height) return GRIS_ERR_INVALID_ARGUMENT;
    *width = s->filmW;
    *height = s->filmH;
    return GRIS_OK;
}
