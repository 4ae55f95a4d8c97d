/*
 * di_kernels.cu — the ReSTIR DI pass (direct lighting at the primary vertex) on sm_103a.
 *
 *   k_di_candidates  di_path_gen.comp / generatePath (di_path_gen.glsl:9-40) with sampleLi
 *                    (di_reservoir.glsl:78-174)
 *   k_di_temporal    di_temporal.comp / temporalReuse (di_temporal.glsl:9-90)
 *   k_di_spatial     di_spatial.comp / spatialReuse + final shading + running mean
 *                    (di_spatial.glsl:9-121, di_spatial.comp:14-27)
 * with the two shifts of DIReservoirReuseAndMerge (reconnection, random replay;
 * di_reservoir.glsl:176-296) shared by the reuse kernels, in the order of TestReSTIR::render
 * (src/TestReSTIR.cpp:9-35).
 *
 * One thread per pixel of a 16 x 8 tile, as the GRIS kernels; reservoirs are 64 B (four 16-byte
 * words per pixel, read and written as uint4). Traversal is the 8-wide BVH walk shared with the
 * GRIS kernels (ray_query.cuh), called out of line from the several query sites of a kernel.
 * The kernels ask for 8 resident blocks of 128 threads per SM (at most 64 registers): measured at
 * 1080p with one shift per neighbour in order, the spatial pass ran in 4.53 ms that way, 4.81 ms
 * at 5 blocks, 4.60 at 10 and 5.91 ms at its natural 160 registers (3 blocks); the latency of the
 * walks is hidden by more warps rather than by registers, despite the spills. Its reconnection
 * loop now runs in three phases with the warp's visibility queries pooled (3.12 ms).
 */
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "gris_device.cuh"
#include "gris_kernels.h"
#include "grisrt_internal.h"
#include "ray_query.cuh"

namespace grisrt {

static_assert(sizeof(GrisDIReservoir) == 64, "DIReservoir is 64 B");

struct DISample { Isec isec; V3 Li; float pad0; float jac, pdf; uint32_t rng, isLight; };   /* layouts.glsl:96-106 */
struct DIResv { DISample s; uint32_t M; float W, contrib, weight; };                        /* :108-115 */

struct DICtx {
    DevScene sc;
    CamD cam, prev;
    GrisDISettings set;
    GrisDIBindings b;
    unsigned long long* counters;
    int countWork;
};

constexpr uint32_t kDICap = 40;              /* DIReservoirCapSample(resv, 40), di_temporal.glsl:87 / di_spatial.glsl:95 */
constexpr uint32_t kDINeighbours = 10;       /* ResampleNum, di_spatial.glsl:62 */
constexpr float kDIRadius = 20.0f;           /* ResampleRadius, di_spatial.glsl:63 */

GD DIResv di_zero() {
    DIResv r;
    r.s.isec = isec_zero(); r.s.Li = v3s(0.0f); r.s.pad0 = 0.0f; r.s.jac = 0.0f; r.s.pdf = 0.0f;
    r.s.rng = 0u; r.s.isLight = 0u;
    r.M = 0u; r.W = 0.0f; r.contrib = 0.0f; r.weight = 0.0f;
    return r;
}
GD bool di_usable(const DIResv& r) { return !isnan(r.W); }                                    /* di_reservoir.glsl:40-42 */
GD void di_clear(DIResv& r) { r.M = 0u; r.W = 0.0f; r.contrib = 0.0f; }                       /* :34-38 */
GD void di_add(DIResv& r, const DISample& s, float w, float u) {                              /* :50-58 */
    r.W += w;
    r.M++;
    if (u * r.W < w) { r.s = s; r.weight = w; }
}
GD void di_merge(DIResv& r, const DIResv& rhs, float u) {                                     /* :60-68 */
    r.W += rhs.W;
    r.M += rhs.M;
    if (u * r.W < rhs.W) { r.s = rhs.s; r.weight = rhs.weight; }
}
GD void di_cap(DIResv& r, uint32_t cap) {                                                      /* :70-75 */
    if (r.M > cap) { r.W *= (float)cap / (float)r.M; r.M = cap; }
}

GD DIResv load_di(const GrisDIReservoir* buf, uint64_t i, uint64_t n) {
    if (i >= n) return di_zero();
    const uint4* p = reinterpret_cast<const uint4*>(buf + i);
    uint4 a = p[0], b = p[1], c = p[2], d = p[3];
    DIResv r;
    r.s.isec.bx = __uint_as_float(a.x); r.s.isec.by = __uint_as_float(a.y); r.s.isec.inst = a.z; r.s.isec.tri = a.w;
    r.s.Li = v3(__uint_as_float(b.x), __uint_as_float(b.y), __uint_as_float(b.z)); r.s.pad0 = __uint_as_float(b.w);
    r.s.jac = __uint_as_float(c.x); r.s.pdf = __uint_as_float(c.y); r.s.rng = c.z; r.s.isLight = c.w;
    r.M = d.x; r.W = __uint_as_float(d.y); r.contrib = __uint_as_float(d.z); r.weight = __uint_as_float(d.w);
    return r;
}
GD void store_di(GrisDIReservoir* buf, uint64_t i, const DIResv& r) {
    uint4* p = reinterpret_cast<uint4*>(buf + i);
    p[0] = make_uint4(__float_as_uint(r.s.isec.bx), __float_as_uint(r.s.isec.by), r.s.isec.inst, r.s.isec.tri);
    p[1] = make_uint4(__float_as_uint(r.s.Li.x), __float_as_uint(r.s.Li.y), __float_as_uint(r.s.Li.z), __float_as_uint(r.s.pad0));
    p[2] = make_uint4(__float_as_uint(r.s.jac), __float_as_uint(r.s.pdf), r.s.rng, r.s.isLight);
    p[3] = make_uint4(r.M, __float_as_uint(r.W), __float_as_uint(r.contrib), __float_as_uint(r.weight));
}

/* sampleLi (di_reservoir.glsl:78-174): the light and / or BSDF candidate streamed into `resv`
 * (one draw of resvRng per candidate), then the chosen sample's Li scaled by W / w and M = 1.
 * The candidates' own colour sum is never used by the pass and is not formed. */
/* The candidates' two ray queries, answered on the spot (DITraceInline) or by the walks of the
 * candidates pass in three launches (DITraceQueue / DITraceAnswer, below). */
struct DITraceInline {
    RayCount& rc;
    int& err;
    GD bool shadow(const DICtx& P, V3 o, V3 d, float tmax) { return traceShadowCall(P.sc, o, kMinRayDistance, d, tmax, rc, err); }
    GD Isec closest(const DICtx& P, V3 o, V3 d) { return traceClosestHitCall(P.sc, o, d, kMinRayDistance, kMaxRayDistance, rc, err); }
};

template <class Tracer>
GD void di_sample_li(const DICtx& P, const Surf& surf, const Mat& mat, V3 wo, uint32_t rng, uint32_t& resvRng,
                     DIResv& resv, Tracer& tracer) {
    DISample ps = di_zero().s;
    ps.rng = rng;
    V4 lr = sample4f(rng);
    V3 sr = sample3f(rng);
    if (P.set.sampleType != GRIS_DI_SAMPLE_BSDF && !isBSDFDelta(mat)) {
        V3 wi = v3s(0.0f); float dist = 0.0f, pdf = 0.0f, jac = 0.0f; V2 bary = v2(0.0f, 0.0f); uint32_t id = 0u;
        V3 Le = sampleLightByPower(P.sc, surf.pos, wi, dist, pdf, jac, bary, id, lr);
        bool shadowed = tracer.shadow(P, surf.pos, wi, dist - kMinRayDistance);
        if (!shadowed && pdf > 1e-6f) {
            float w = MISWeight(pdf, evalPdf(mat, surf.norm, wo, wi));
            if (P.set.sampleType == GRIS_DI_SAMPLE_LIGHT) w = 1.0f;
            V3 contrib = Le * evalBSDF(mat, surf.albedo, surf.norm, wo, wi) * satDot(surf.norm, wi) / pdf * w;
            float sw = luminance(contrib);
            if (isnan(sw) || sw < 0.0f) sw = 0.0f;
            ps.isec.bx = bary.x; ps.isec.by = bary.y; ps.isec.inst = 0u; ps.isec.tri = id;
            ps.Li = Le * w;
            ps.jac = jac; ps.pdf = pdf; ps.isLight = 1u;
            di_add(resv, ps, sw, sample1f(resvRng));
        }
    }
    ps.isLight = 0u;
    BsdfSample s = bs_zero();
    if (P.set.sampleType != GRIS_DI_SAMPLE_LIGHT && sampleBSDF(mat, surf.albedo, surf.norm, wo, sr, s) && s.pdf > 1e-6f) {
        Isec isec = tracer.closest(P, surf.pos, s.wi);
        if (isec.inst != kInvalidHit) {
            Surf hit = surf_zero();
            loadSurfaceInfo(P.sc, isec, hit);
            float cosT = -dot3(s.wi, hit.norm);
            if (hit.isLight && cosT > 0.0f) {
                float dist = length3(hit.pos - surf.pos);
                float lightPdf = luminance(hit.albedo) / load_table(P.sc, 0).prob * dist * dist / fabsf(cosT);
                float w = MISWeight(s.pdf, lightPdf);
                bool delta = isSampleTypeDelta(s.type);
                if (P.set.sampleType == GRIS_DI_SAMPLE_BSDF || delta) w = 1.0f;
                float cosTerm = delta ? 1.0f : satDot(surf.norm, s.wi);
                V3 contrib = hit.albedo * s.bsdf * cosTerm / s.pdf * w;
                ps.isec = isec;
                ps.Li = hit.albedo * w;
                ps.jac = fabsf(cosT) / square(dist); ps.pdf = s.pdf; ps.isLight = 0u;
                di_add(resv, ps, luminance(contrib), sample1f(resvRng));   /* unclamped, as the reference */
            }
        }
    }
    if (!di_usable(resv)) di_clear(resv);
    if (resv.M > 0u && resv.s.isec.inst != kInvalidHit && resv.weight > 0.0f) {
        resv.s.Li = resv.s.Li * (resv.W / resv.weight);
        resv.weight = resv.W;
    } else {
        resv.s.isec.inst = kInvalidHit;
        resv.weight = 0.0f;
        resv.W = 0.0f;
    }
    resv.M = 1u;
}

/* randomReplay (di_reservoir.glsl:176-209): the source's candidates drawn again at the
 * destination from the source's seed; their reservoir draws come from the merge stream. */
GD void di_replay(const DICtx& P, DIResv& dst, const Surf& ds, const DIResv& src, V3 wo, uint32_t& rng, RayCount& rc,
                  int& err) {
    Mat mat = load_material(P.sc, ds.matIndex);
    DIResv rr = di_zero();
    di_clear(rr);
    DITraceInline tracer{rc, err};
    di_sample_li(P, ds, mat, wo, src.s.rng, rng, rr, tracer);
    if (rr.s.isec.inst != kInvalidHit) {
        Surf rs = surf_zero();
        loadSurfaceInfo(P.sc, rr.s.isec, rs);
        V3 wi = normalize3(rs.pos - ds.pos);
        V3 Li = rr.s.Li * evalBSDF(mat, ds.albedo, ds.norm, wo, wi) * satDot(ds.norm, wi) / rr.s.pdf;
        float pHat = luminance(Li * 1.0f);
        rr.W = src.W * pHat / src.weight;
        rr.M = src.M;
    } else {
        rr.W = 0.0f;
    }
    if (di_usable(rr)) di_merge(dst, rr, sample1f(rng));
}

/* reconnection (di_reservoir.glsl:211-287): the source's light vertex seen from the destination
 * (one visibility ray), Jacobian (|cos| / d^2)_dst / jacobian_src. */
/* the reconnection's visibility query, answered on the spot */
struct DIVisInline {
    RayCount& rc;
    int& err;
    GD bool visible(const DICtx& P, V3 from, V3 to) { return traceVisibility(P.sc, from, to, rc, err); }
};

template <class Vis>
GD void di_reconnect(const DICtx& P, DIResv& dst, const Surf& ds, DIResv src, V3 wo, uint32_t& rng, Vis& vis) {
    Mat mat = load_material(P.sc, ds.matIndex);
    DISample ss = src.s;
    Surf lv = surf_zero();
    loadSurfaceInfo(P.sc, ss.isec, lv);
    float dist = distance3(lv.pos, ds.pos);
    V3 wi = normalize3(lv.pos - ds.pos);
    float cosT = -dot3(lv.norm, wi);
    float dstJac = fabsf(cosT) / square(dist);
    float jac = dstJac / ss.jac;
    bool ok = false;
    float pHat = 0.0f, dstPdf = 0.0f;
    if (ss.isec.inst != kInvalidHit && dist > 1e-4f) {
        if (cosT > 0.0f && !isnan(jac) && ss.jac > 0.0f) {
            if (vis.visible(P, ds.pos, lv.pos)) {
                ok = true;
                if (!isnan(ss.pdf) && ss.pdf > 1e-6f) {
                    V3 Li = src.s.Li * evalBSDF(mat, ds.albedo, ds.norm, wo, wi) * satDot(ds.norm, wi) / ss.pdf;
                    pHat = luminance(Li * jac);
                }
                if (ss.isLight) dstPdf = luminance(lv.albedo) / load_table(P.sc, 0).prob / dstJac;
                else dstPdf = evalPdf(mat, ds.norm, wo, wi);
            }
        }
    }
    if (ok) {
        ss.jac = dstJac;
        ss.pdf = dstPdf;
        if (ss.pdf < 1e-6f || isnan(ss.pdf)) ss.pdf = 0.0f;
        src.s = ss;
        src.W *= pHat / src.weight;
        if (isnan(src.W)) src.W = 0.0f;
    } else {
        src.W = 0.0f;
    }
    if (di_usable(src)) di_merge(dst, src, sample1f(rng));
}

/* DIReservoirReuseAndMerge (di_reservoir.glsl:289-296) */
GD void di_reuse(const DICtx& P, DIResv& dst, const Surf& ds, const DIResv& src, V3 wo, uint32_t& rng, RayCount& rc,
                 int& err) {
    if (P.set.shiftType == GRIS_DI_SHIFT_RECONNECTION) {
        DIVisInline vis{rc, err};
        di_reconnect(P, dst, ds, src, wo, rng, vis);
    } else if (P.set.shiftType == GRIS_DI_SHIFT_REPLAY) {
        di_replay(P, dst, ds, src, wo, rng, rc, err);
    }
}

/* The final sample's visibility in both reuse passes (di_temporal.glsl:76-85, di_spatial.glsl:84-93). */
GD void di_occlude(const DICtx& P, DIResv& r, V3 pos, RayCount& rc, int& err) {
    if (di_usable(r) && r.s.isec.inst != kInvalidHit) {
        Surf s = surf_zero();
        loadSurfaceInfo(P.sc, r.s.isec, s);
        if (!traceVisibility(P.sc, pos, s.pos, rc, err)) r.W = 0.0f;
    }
}

/* The pixel's primary vertex from the G-buffer (unpackGBuffer + camera ray, as every DI shader). */
struct DIPixel {
    V2 uv;
    Ray3 ray;
    Surf surf;
    int matMeshId;
};
GD bool di_pixel(const DICtx& P, uint32_t ix, uint32_t iy, DIPixel& px) {
    const int W = (int)P.b.width, H = (int)P.b.height;
    px.uv = v2(((float)ix + 0.5f) / (float)W, ((float)iy + 0.5f) / (float)H);
    float depth = 0.0f; V3 norm = v3s(0.0f), albedo = v3s(0.0f); int mm = 0;
    float4 dn = texture_bilinear(reinterpret_cast<const float4*>(P.b.depthNormal), W, H, px.uv);
    uint2 am = fetch_am(reinterpret_cast<const uint2*>(P.b.albedoMatId), W, H, (int)ix, (int)iy);
    if (!unpackGBuffer(dn, am, depth, norm, albedo, mm)) return false;
    px.ray = pinholeCameraSampleRay(P.cam, v2(px.uv.x, 1.0f - px.uv.y));
    px.surf.pos = px.ray.ori + px.ray.dir * (depth - 1e-4f);
    px.surf.norm = norm; px.surf.albedo = albedo; px.surf.matIndex = (uint32_t)(mm >> 16); px.surf.isLight = false;
    px.matMeshId = mm;
    return true;
}

/* resident blocks of 128 threads per SM asked of the compiler for the DI kernels that walk their
 * queries inline (the temporal pass, the spatial pass's finish with the final occlusion test).
 * At 1080p: 8 blocks (64 registers; their spills stay in L1) 188.1 frames/s, 7 blocks 186.7,
 * 6 blocks 184.1. */
#ifndef GRIS_DI_INLINE_WALK_BLOCKS
#define GRIS_DI_INLINE_WALK_BLOCKS 8
#endif

/* ------------------------------------------------------------------ kernels */
__global__ void __launch_bounds__(128, 8) k_di_candidates(DICtx P) {
    RayCount rc = ray_count();
    int err = 0;
    uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    DIPixel px;
    if (x < P.b.width && y < P.b.height && di_pixel(P, x, y, px)) {
        uint32_t rng = makeSeed2(P.cam.seed, x, y);
        uint32_t resvRng = ~rng;
        DIResv r = di_zero();
        di_clear(r);
        DITraceInline tracer{rc, err};
        di_sample_li(P, px.surf, load_material(P.sc, px.surf.matIndex), -px.ray.dir, rng, resvRng, r, tracer);
        store_di(P.b.reservoirThis, (uint64_t)y * P.b.width + x, r);
    }
    flush_counts(P.counters, rc, err, 4, P.countWork);
}

/* findPreviousReservoir (di_temporal.glsl:9-34) + temporalReuse (:36-90) */
/* The temporal neighbour of pixel (x, y) (di_temporal.glsl:36-74: reprojection, the previous
 * G-buffer's checks): true with its reservoir in src when it is found and usable. */
GD bool di_temporal_source(const DICtx& P, uint32_t x, uint32_t y, const DIPixel& px, DIResv& src) {
    const int W = (int)P.b.width, H = (int)P.b.height;
    const uint64_t n = (uint64_t)W * (uint64_t)H, idx = (uint64_t)y * W + x;
    float2 motion = __half22float2(reinterpret_cast<const __half2*>(P.b.motion)[idx]);
    V2 puv = v2(px.uv.x + motion.x, px.uv.y + motion.y);
    if ((P.cam.frameIndex & kCameraClearFlag) != 0u || puv.x < 0.0f || puv.y < 0.0f || puv.x > 1.0f || puv.y > 1.0f)
        return false;
    int qx = (int)(puv.x * (float)P.cam.w), qy = (int)(puv.y * (float)P.cam.h);
    float pdepth = 0.0f; V3 pn = v3s(0.0f), palb = v3s(0.0f); int pmm = 0;
    float4 pdn = texture_bilinear(reinterpret_cast<const float4*>(P.b.depthNormalPrev), W, H, puv);
    uint2 pam = fetch_am(reinterpret_cast<const uint2*>(P.b.albedoMatIdPrev), W, H, qx, qy);
    if (!unpackGBuffer(pdn, pam, pdepth, pn, palb, pmm)) return false;
    Ray3 pray = pinholeCameraSampleRay(P.prev, v2(puv.x, 1.0f - puv.y));
    V3 ppos = pray.ori + pray.dir * (pdepth - 1e-4f);
    if (pmm != px.matMeshId || dot3(pn, px.surf.norm) < 0.95f || distance3(px.surf.pos, ppos) > 0.5f) return false;
    src = load_di(P.b.reservoirPrev, (uint64_t)((uint32_t)P.cam.w * (uint32_t)qy + (uint32_t)qx), n);
    return di_usable(src);
}

__global__ void __launch_bounds__(128, GRIS_DI_INLINE_WALK_BLOCKS) k_di_temporal(DICtx P) {
    RayCount rc = ray_count();
    int err = 0;
    uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    DIPixel px;
    if (x < P.b.width && y < P.b.height && di_pixel(P, x, y, px)) {
        const int W = (int)P.b.width, H = (int)P.b.height;
        const uint64_t n = (uint64_t)W * (uint64_t)H, idx = (uint64_t)y * W + x;
        uint32_t resvRng = ~(makeSeed2(P.cam.seed, x, y) ^ 1u);
        DIResv r = load_di(P.b.reservoirThis, idx, n);
        if (P.set.temporalReuse) {
            DIResv src;
            if (di_temporal_source(P, x, y, px, src)) di_reuse(P, r, px.surf, src, -px.ray.dir, resvRng, rc, err);
            di_occlude(P, r, px.surf.pos, rc, err);
        }
        di_cap(r, kDICap);
        if (!di_usable(r)) di_clear(r);
        store_di(P.b.reservoirTemp, idx, r);
    }
    flush_counts(P.counters, rc, err, 5, P.countWork);
}

/* The spatial pass's neighbour loop under the reconnection shift (di_spatial.glsl:60-82 with
 * di_reservoir.glsl:211-287), in three phases with the reference's results and draw order:
 *   1. di_spatial_shift: every neighbour's gather, gates and shift up to its visibility query,
 *      with the merge's draw taken where the reference takes it (one per neighbour reaching the
 *      shift: a shifted reservoir is always usable, its W being 0 when the shift fails);
 *   2. di_pooled_visibility: the warp's queries pooled and walked 32 at a time, one per lane
 *      whichever pixel posted it (a warp walks ceil(queries / 32) times instead of once per
 *      neighbour index with the lanes whose neighbour needs no query idle);
 *   3. di_spatial_merge: the merges in neighbour order with the verdicts, and the chosen
 *      neighbour's reservoir read again for its sample. */
struct DINeighbour {
    float Wv, u, jac, pdf;   /* W if visible; merge draw; Jacobian and pdf at the destination */
    uint32_t M, q;           /* source M; source pixel */
    V3 to;                   /* the light vertex the query looks at */
};
GD void di_spatial_shift(const DICtx& P, const DIPixel& px, V3 wo, uint32_t& rng, DINeighbour* nb, uint32_t& m,
                         uint32_t& queries) {
    const int W = (int)P.b.width, H = (int)P.b.height;
    const uint64_t n = (uint64_t)W * (uint64_t)H;
    const Surf& ds = px.surf;
    const Mat mat = load_material(P.sc, ds.matIndex);
    const float tx = 1.0f / (float)W, ty = 1.0f / (float)H;
    m = 0; queries = 0;
    for (uint32_t k = 0; k < kDINeighbours; k++) {
        V2 d = toConcentricDisk(sample2f(rng));
        V2 uv = v2(px.uv.x + d.x * kDIRadius * tx, px.uv.y + d.y * kDIRadius * ty);
        if (uv.x < 0.0f || uv.y < 0.0f || uv.x > 1.0f || uv.y > 1.0f) continue;
        int qx = (int)(uv.x * (float)P.cam.w), qy = (int)(uv.y * (float)P.cam.h);
        float ndepth = 0.0f; V3 nn = v3s(0.0f), nalb = v3s(0.0f); int nmm = 0;
        float4 ndn = texture_bilinear(reinterpret_cast<const float4*>(P.b.depthNormal), W, H, uv);
        uint2 nam = fetch_am(reinterpret_cast<const uint2*>(P.b.albedoMatId), W, H, qx, qy);
        if (!unpackGBuffer(ndn, nam, ndepth, nn, nalb, nmm)) continue;
        Ray3 nr = pinholeCameraSampleRay(P.cam, v2(uv.x, 1.0f - uv.y));
        V3 npos = nr.ori + nr.dir * (ndepth - 1e-4f);
        if (dot3(nn, ds.norm) < 0.9f || distance3(ds.pos, npos) > 0.4f) continue;
        const uint32_t q = (uint32_t)P.cam.w * (uint32_t)qy + (uint32_t)qx;
        DIResv src = load_di(P.b.reservoirTemp, (uint64_t)q, n);
        if (!di_usable(src)) continue;
        Surf lv = surf_zero();
        loadSurfaceInfo(P.sc, src.s.isec, lv);
        float dist = distance3(lv.pos, ds.pos);
        V3 wi = normalize3(lv.pos - ds.pos);
        float cosT = -dot3(lv.norm, wi);
        float dstJac = fabsf(cosT) / square(dist);
        float jac = dstJac / src.s.jac;
        bool query = src.s.isec.inst != kInvalidHit && dist > 1e-4f && cosT > 0.0f && !isnan(jac) && src.s.jac > 0.0f;
        float pHat = 0.0f, dstPdf = 0.0f, Wv = 0.0f;
        if (query) {
            if (!isnan(src.s.pdf) && src.s.pdf > 1e-6f) {
                V3 Li = src.s.Li * evalBSDF(mat, ds.albedo, ds.norm, wo, wi) * satDot(ds.norm, wi) / src.s.pdf;
                pHat = luminance(Li * jac);
            }
            if (src.s.isLight) dstPdf = luminance(lv.albedo) / load_table(P.sc, 0).prob / dstJac;
            else dstPdf = evalPdf(mat, ds.norm, wo, wi);
            if (dstPdf < 1e-6f || isnan(dstPdf)) dstPdf = 0.0f;
            Wv = src.W * (pHat / src.weight);
            if (isnan(Wv)) Wv = 0.0f;
            queries |= 1u << m;
        }
        nb[m].Wv = Wv; nb[m].u = sample1f(rng); nb[m].jac = dstJac; nb[m].pdf = dstPdf;
        nb[m].M = src.M; nb[m].q = q; nb[m].to = lv.pos;
        m++;
    }
}

/* Called by every lane of the warp (lanes without a pixel post no query): each lane posts its
 * queries (from its pixel's position to a light vertex) in a per-warp list in shared memory, at
 * the exclusive prefix of the lanes' query counts; the warp walks the list 32 entries per round
 * and sets the verdict bits in the posting lane's word. Returns the lane's verdicts by query bit. */
constexpr uint32_t kDIWarps = 4;   /* 128 threads per block */
GD uint32_t di_pooled_visibility(const DICtx& P, V3 from, const DINeighbour* nb, uint32_t queries, RayCount& rc,
                                 int& err) {
    __shared__ float4 sFrom[kDIWarps][32];
    __shared__ float4 sTo[kDIWarps][32];
    __shared__ uint32_t sVerdict[kDIWarps][32];
    const uint32_t t = threadIdx.y * blockDim.x + threadIdx.x, w = t >> 5, lane = t & 31u;
    const uint32_t c = (uint32_t)__popc(queries);
    uint32_t incl = c;
    for (uint32_t d = 1; d < 32; d <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
    }
    const uint32_t first = incl - c, total = __shfl_sync(0xffffffffu, incl, 31);
    sFrom[w][lane] = make_float4(from.x, from.y, from.z, 0.0f);
    sVerdict[w][lane] = 0u;
    for (uint32_t base = 0; base < total; base += 32) {
        __syncwarp();
        if (first < base + 32 && first + c > base) {
            uint32_t g = first;
            for (uint32_t pending = queries; pending; pending &= pending - 1u, g++) {
                if (g < base || g >= base + 32) continue;
                const uint32_t i = (uint32_t)__ffs(pending) - 1u;
                sTo[w][g - base] = make_float4(nb[i].to.x, nb[i].to.y, nb[i].to.z, __uint_as_float((lane << 4) | i));
            }
        }
        __syncwarp();
        if (base + lane < total) {
            const float4 q = sTo[w][lane];
            const uint32_t tag = __float_as_uint(q.w), owner = tag >> 4;
            const float4 f = sFrom[w][owner];
            if (traceVisibility(P.sc, v3(f.x, f.y, f.z), v3(q.x, q.y, q.z), rc, err))
                atomicOr(&sVerdict[w][owner], 1u << (tag & 15u));
        }
    }
    __syncwarp();
    return sVerdict[w][lane];
}

GD void di_spatial_merge(const DICtx& P, const DINeighbour* nb, uint32_t m, uint32_t visible, DIResv& r) {
    const uint64_t n = (uint64_t)P.b.width * (uint64_t)P.b.height;
    int sel = -1;
    for (uint32_t i = 0; i < m; i++) {
        const float w = (visible >> i) & 1u ? nb[i].Wv : 0.0f;
        r.W += w;
        r.M += nb[i].M;
        if (nb[i].u * r.W < w) sel = (int)i;
    }
    if (sel >= 0) {
        DIResv src = load_di(P.b.reservoirTemp, (uint64_t)nb[sel].q, n);
        r.s = src.s;
        r.weight = src.weight;
        if ((visible >> sel) & 1u) { r.s.jac = nb[sel].jac; r.s.pdf = nb[sel].pdf; }
    }
}

/* findNeighborReservoir (di_spatial.glsl:9-34) + spatialReuse (:36-121) + the running mean of
 * di_spatial.comp:21-26 (a background pixel accumulates black). Every lane of a warp reaches the
 * pooled visibility phase (the block is 16 x 8, whole warps, lanes outside the image included). */
__global__ void __launch_bounds__(128, 8) k_di_spatial(DICtx P) {
    RayCount rc = ray_count();
    int err = 0;
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const int W = (int)P.b.width, H = (int)P.b.height;
    const uint64_t n = (uint64_t)W * (uint64_t)H, idx = (uint64_t)y * W + x;
    const bool inside = x < P.b.width && y < P.b.height;
    const bool phased = P.set.spatialReuse && P.set.shiftType == GRIS_DI_SHIFT_RECONNECTION;
    DIPixel px;
    const bool fg = inside && di_pixel(P, x, y, px);
    uint32_t rng = 0u;
    V3 wo = v3s(0.0f), from = v3s(0.0f);
    DIResv r = di_zero();
    DINeighbour nb[kDINeighbours];
    uint32_t m = 0, queries = 0, visible = 0;
    if (fg) {
        rng = makeSeed2(P.cam.seed, x, y) ^ 2u;
        wo = -px.ray.dir;
        from = px.surf.pos;
        r = load_di(P.b.reservoirTemp, idx, n);
        if (phased) di_spatial_shift(P, px, wo, rng, nb, m, queries);
    }
    if (phased) visible = di_pooled_visibility(P, from, nb, queries, rc, err);
    V3 color = v3s(0.0f);
    if (fg) {
        if (phased) {
            di_spatial_merge(P, nb, m, visible, r);
            di_occlude(P, r, px.surf.pos, rc, err);
        } else if (P.set.spatialReuse) {
            float tx = 1.0f / (float)W, ty = 1.0f / (float)H;
            for (uint32_t k = 0; k < kDINeighbours; k++) {
                V2 d = toConcentricDisk(sample2f(rng));
                V2 nuv = v2(px.uv.x + d.x * kDIRadius * tx, px.uv.y + d.y * kDIRadius * ty);
                if (nuv.x < 0.0f || nuv.y < 0.0f || nuv.x > 1.0f || nuv.y > 1.0f) continue;
                int qx = (int)(nuv.x * (float)P.cam.w), qy = (int)(nuv.y * (float)P.cam.h);
                float ndepth = 0.0f; V3 nn = v3s(0.0f), nalb = v3s(0.0f); int nmm = 0;
                float4 ndn = texture_bilinear(reinterpret_cast<const float4*>(P.b.depthNormal), W, H, nuv);
                uint2 nam = fetch_am(reinterpret_cast<const uint2*>(P.b.albedoMatId), W, H, qx, qy);
                if (!unpackGBuffer(ndn, nam, ndepth, nn, nalb, nmm)) continue;
                Ray3 nr = pinholeCameraSampleRay(P.cam, v2(nuv.x, 1.0f - nuv.y));
                V3 npos = nr.ori + nr.dir * (ndepth - 1e-4f);
                if (dot3(nn, px.surf.norm) < 0.9f || distance3(px.surf.pos, npos) > 0.4f) continue;
                DIResv src = load_di(P.b.reservoirTemp, (uint64_t)((uint32_t)P.cam.w * (uint32_t)qy + (uint32_t)qx), n);
                if (di_usable(src)) di_reuse(P, r, px.surf, src, wo, rng, rc, err);
            }
            di_occlude(P, r, px.surf.pos, rc, err);
        }
        di_cap(r, kDICap);
        if (!di_usable(r)) di_clear(r);
        store_di(P.b.reservoirThis, idx, r);
        if (di_usable(r) && r.s.isec.inst != kInvalidHit) {
            Surf ls = surf_zero();
            loadSurfaceInfo(P.sc, r.s.isec, ls);
            V3 wi = normalize3(ls.pos - px.surf.pos);
            if (r.M > 0u) {
                Mat mat = load_material(P.sc, px.surf.matIndex);
                V3 Li = r.s.Li * evalBSDF(mat, px.surf.albedo, px.surf.norm, wo, wi) * satDot(px.surf.norm, wi) / r.s.pdf;
                if (!isBlack(Li)) color = Li / luminance(Li) * r.W / (float)r.M;
            }
        }
        color = clampColor(color);
    }
    if (inside) {
        float frameCount = (float)(P.cam.frameIndex & kCameraFrameIndexMask);
        float4* out = reinterpret_cast<float4*>(P.b.directOutput) + idx;
        float4 o = *out;
        V3 acc = (v3(o.x, o.y, o.z) * frameCount + color) / (frameCount + 1.0f);
        *out = make_float4(acc.x, acc.y, acc.z, 1.0f);
    }
    flush_counts(P.counters, rc, err, 6, P.countWork);
}

/* ------------------------------------------------------------------ spatial pass in three launches */
/* With the reconnection shift the spatial pass runs as prepare (per pixel: the ten neighbours'
 * shifts up to their visibility queries, di_spatial_shift, each neighbour's record kept in slot k
 * of pixel p at k * P + p and its query appended to a queue of slots), the refilling any-hit walk
 * of that queue (a visible segment sets its slot's verdict) and finish (the merges in neighbour
 * order with the verdicts, the final occlusion test, the cap and the running mean): the
 * operations of k_di_spatial in the same order, each query answered as traceVisibility answers
 * it. A warp's queries no longer wait for the longest walk among them. */
struct DISplit {
    float4* from;        /* per pixel: its primary vertex */
    uint32_t* mq;        /* per pixel: neighbour records | query bits << 8 */
    float4* recA;        /* per slot: W if visible, merge draw, Jacobian, pdf */
    uint2* recB;         /* per slot: source M, source pixel */
    float4* recTo;       /* per slot: the light vertex the query looks at */
    uint8_t* vis;        /* per slot: 1 = visible */
    uint32_t* queue;     /* query slots */
    uint32_t* counts;    /* [0] queries, [1] the walk's cursor */
    uint64_t P;          /* pixels */
};

__global__ void __launch_bounds__(128, 8) k_di_spatial_prepare(DICtx P, DISplit S) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    const uint64_t idx = (uint64_t)y * P.b.width + x;
    uint32_t queries = 0u;
    if (x < P.b.width && y < P.b.height) {
        DIPixel px;
        uint32_t m = 0u;
        if (di_pixel(P, x, y, px)) {
            uint32_t rng = makeSeed2(P.cam.seed, x, y) ^ 2u;
            DINeighbour nb[kDINeighbours];
            di_spatial_shift(P, px, -px.ray.dir, rng, nb, m, queries);
            S.from[idx] = make_float4(px.surf.pos.x, px.surf.pos.y, px.surf.pos.z, 0.0f);
            for (uint32_t i = 0; i < m; i++) {
                const uint64_t s = (uint64_t)i * S.P + idx;
                S.recA[s] = make_float4(nb[i].Wv, nb[i].u, nb[i].jac, nb[i].pdf);
                S.recB[s] = make_uint2(nb[i].M, nb[i].q);
                S.recTo[s] = make_float4(nb[i].to.x, nb[i].to.y, nb[i].to.z, 0.0f);
                S.vis[s] = 0u;
            }
        }
        S.mq[idx] = m | (queries << 8);
    }
    /* the lane's queries at the warp's exclusive prefix, one atomic per warp */
    const uint32_t lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31u;
    const uint32_t c = (uint32_t)__popc(queries);
    uint32_t incl = c;
    for (uint32_t d = 1; d < 32; d <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    uint32_t base = 0u;
    if (lane == 31u && total) base = atomicAdd(S.counts, total);
    base = __shfl_sync(0xffffffffu, base, 31);
    uint32_t at = base + incl - c;
    for (uint32_t pending = queries; pending; pending &= pending - 1u)
        S.queue[at++] = (uint32_t)((uint64_t)(__ffs(pending) - 1) * S.P + idx);
}

constexpr int kDIWalkShared = 8;   /* walk stack entries in shared memory (after two in registers) */
constexpr int kDIWalkTris = 2;     /* leaf triangles tested per step */

__global__ void __launch_bounds__(128, 7) k_di_visibility(DICtx P, DISplit S) {
    const uint32_t n = S.counts[0];
    uint32_t* cursor = S.counts + 1;
    const uint32_t lane = threadIdx.x & 31u;
    RayCount rc = ray_count();
    int err = 0;
    GrisTraversal<true> tr;
    __shared__ uint32_t sStack[2 * kDIWalkShared * 128];
    GrisShortStack<kDIWalkShared> stack;
    stack.bind(sStack, threadIdx.x, 128u);
    uint32_t slot = 0u;
    bool active = false, more = true;
    while (true) {
        const unsigned idle = __ballot_sync(0xffffffffu, !active);
        if (more && __popc(idle) >= 8) {
            const uint32_t take = (uint32_t)__popc(idle), leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(cursor, take);
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!active) {
                const uint32_t i = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (i < n) {
                    slot = S.queue[i];
                    const float4 f = S.from[slot % S.P], t = S.recTo[slot];
                    /* traceVisibility's segment: from the pixel to the light vertex */
                    const V3 from = v3(f.x, f.y, f.z), to = v3(t.x, t.y, t.z);
                    const V3 d = normalize3(to - from);
                    stack.reset();
                    tr.init(from.x, from.y, from.z, d.x, d.y, d.z, kMinRayDistance,
                            distance3(to, from) - kMinRayDistance);
                    active = true;
                }
            }
            if (base + take >= n) more = false;
        }
        if (__ballot_sync(0xffffffffu, active) == 0u) {
            if (!more) break;
            continue;
        }
        if (active && !tr.template step<kDIWalkTris>(P.sc.nodes, P.sc.tris, false, &err, stack)) {
            GrisRayHit h;
            tr.result(&h, &rc.work);
            rc.shadow++;
            if (!tr.found) S.vis[slot] = 1u;
            active = false;
        }
    }
    flush_counts(P.counters, rc, err, 6, P.countWork);
}

__global__ void __launch_bounds__(128, GRIS_DI_INLINE_WALK_BLOCKS) k_di_spatial_finish(DICtx P, DISplit S) {
    RayCount rc = ray_count();
    int err = 0;
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= P.b.width || y >= P.b.height) return;
    const int W = (int)P.b.width, H = (int)P.b.height;
    const uint64_t n = (uint64_t)W * (uint64_t)H, idx = (uint64_t)y * W + x;
    DIPixel px;
    V3 color = v3s(0.0f);
    if (di_pixel(P, x, y, px)) {
        const V3 wo = -px.ray.dir;
        DIResv r = load_di(P.b.reservoirTemp, idx, n);
        const uint32_t mq = S.mq[idx], m = mq & 0xffu, queries = mq >> 8;
        DINeighbour nb[kDINeighbours];
        uint32_t visible = 0u;
        for (uint32_t i = 0; i < m; i++) {
            const uint64_t s = (uint64_t)i * S.P + idx;
            const float4 a = S.recA[s];
            const uint2 b = S.recB[s];
            nb[i].Wv = a.x; nb[i].u = a.y; nb[i].jac = a.z; nb[i].pdf = a.w;
            nb[i].M = b.x; nb[i].q = b.y;
            if (((queries >> i) & 1u) && S.vis[s]) visible |= 1u << i;
        }
        di_spatial_merge(P, nb, m, visible, r);
        di_occlude(P, r, px.surf.pos, rc, err);
        di_cap(r, kDICap);
        if (!di_usable(r)) di_clear(r);
        store_di(P.b.reservoirThis, idx, r);
        if (di_usable(r) && r.s.isec.inst != kInvalidHit) {
            Surf ls = surf_zero();
            loadSurfaceInfo(P.sc, r.s.isec, ls);
            V3 wi = normalize3(ls.pos - px.surf.pos);
            if (r.M > 0u) {
                Mat mat = load_material(P.sc, px.surf.matIndex);
                V3 Li = r.s.Li * evalBSDF(mat, px.surf.albedo, px.surf.norm, wo, wi) * satDot(px.surf.norm, wi) / r.s.pdf;
                if (!isBlack(Li)) color = Li / luminance(Li) * r.W / (float)r.M;
            }
        }
        color = clampColor(color);
    }
    float frameCount = (float)(P.cam.frameIndex & kCameraFrameIndexMask);
    float4* out = reinterpret_cast<float4*>(P.b.directOutput) + idx;
    float4 o = *out;
    V3 acc = (v3(o.x, o.y, o.z) * frameCount + color) / (frameCount + 1.0f);
    *out = make_float4(acc.x, acc.y, acc.z, 1.0f);
    flush_counts(P.counters, rc, err, 6, P.countWork);
}

/* The candidates pass in three launches: prepare (per pixel the light and BSDF samples, their
 * shadow and closest-hit queries appended to two queues), the resident walks of the two queues,
 * and finish (the same samples drawn again, the walks' answers in place of the inline queries,
 * the candidate stream as before). */
struct DICandidates {
    float4* qS;          /* shadow queries: origin | tmax, direction | pixel */
    float4* qC;          /* closest-hit queries: origin | 0, direction | pixel */
    uint8_t* blocked;    /* per pixel: the shadow query's answer */
    Isec* hit;           /* per pixel: the closest-hit query's answer */
    uint32_t* counts;    /* [0] shadow queries, [1] cursor, [2] closest-hit queries, [3] cursor */
};
struct DITraceQueue {
    bool wantS = false, wantC = false;
    float4 s0, s1, c0, c1;
    uint32_t pix;
    GD bool shadow(const DICtx&, V3 o, V3 d, float tmax) {
        wantS = true;
        s0 = make_float4(o.x, o.y, o.z, tmax); s1 = make_float4(d.x, d.y, d.z, __uint_as_float(pix));
        return true;   /* the prepare pass draws the same numbers whatever the answer */
    }
    GD Isec closest(const DICtx&, V3 o, V3 d) {
        wantC = true;
        c0 = make_float4(o.x, o.y, o.z, 0.0f); c1 = make_float4(d.x, d.y, d.z, __uint_as_float(pix));
        Isec r; r.bx = 0.0f; r.by = 0.0f; r.inst = kInvalidHit; r.tri = 0u;
        return r;
    }
};
struct DITraceAnswer {
    const DICandidates& Q;
    uint32_t pix;
    GD bool shadow(const DICtx&, V3, V3, float) { return Q.blocked[pix] != 0u; }
    GD Isec closest(const DICtx&, V3, V3) { return Q.hit[pix]; }
};

/* appends `want` lanes' records to a queue, one atomic per warp (all lanes call) */
GD void di_push(float4* q, uint32_t* count, bool want, float4 a, float4 b) {
    const unsigned m = __ballot_sync(0xffffffffu, want);
    if (!m) return;
    const uint32_t lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31u, leader = (uint32_t)__ffs(m) - 1u;
    uint32_t base = 0u;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (want) {
        const uint32_t i = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
        q[2 * (uint64_t)i] = a;
        q[2 * (uint64_t)i + 1] = b;
    }
}

__global__ void __launch_bounds__(128, 8) k_di_candidates_prepare(DICtx P, DICandidates Q) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    DITraceQueue tr;
    tr.pix = y * P.b.width + x;
    DIPixel px;
    if (x < P.b.width && y < P.b.height && di_pixel(P, x, y, px)) {
        uint32_t rng = makeSeed2(P.cam.seed, x, y);
        uint32_t resvRng = ~rng;
        DIResv r = di_zero();
        di_clear(r);
        di_sample_li(P, px.surf, load_material(P.sc, px.surf.matIndex), -px.ray.dir, rng, resvRng, r, tr);
    }
    di_push(Q.qS, Q.counts + 0, tr.wantS, tr.s0, tr.s1);
    di_push(Q.qC, Q.counts + 2, tr.wantC, tr.c0, tr.c1);
}

/* the resident walk of a candidates queue (ANY: shadow queries; else closest hits) */
template <bool ANY>
__global__ void __launch_bounds__(128, 7) k_di_candidates_walk(DICtx P, DICandidates Q) {
    const uint32_t n = Q.counts[ANY ? 0 : 2];
    uint32_t* cursor = Q.counts + (ANY ? 1 : 3);
    const float4* q = ANY ? Q.qS : Q.qC;
    const uint32_t lane = threadIdx.x & 31u;
    RayCount rc = ray_count();
    int err = 0;
    GrisTraversal<ANY> tr;
    __shared__ uint32_t sStack[2 * kDIWalkShared * 128];
    GrisShortStack<kDIWalkShared> stack;
    stack.bind(sStack, threadIdx.x, 128u);
    uint32_t pix = 0u;
    bool active = false, more = true;
    while (true) {
        const unsigned idle = __ballot_sync(0xffffffffu, !active);
        if (more && __popc(idle) >= 8) {
            const uint32_t take = (uint32_t)__popc(idle), leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(cursor, take);
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!active) {
                const uint32_t i = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (i < n) {
                    const float4 a = q[2 * (uint64_t)i], b = q[2 * (uint64_t)i + 1];
                    pix = __float_as_uint(b.w);
                    stack.reset();
                    tr.init(a.x, a.y, a.z, b.x, b.y, b.z, kMinRayDistance, ANY ? a.w : kMaxRayDistance);
                    active = true;
                }
            }
            if (base + take >= n) more = false;
        }
        if (__ballot_sync(0xffffffffu, active) == 0u) {
            if (!more) break;
            continue;
        }
        if (active && !tr.template step<(ANY ? kDIWalkTris : 0)>(P.sc.nodes, P.sc.tris, false, &err, stack)) {
            GrisRayHit h;
            tr.result(&h, &rc.work);
            if (ANY) {
                rc.shadow++;
                Q.blocked[pix] = tr.found ? 1u : 0u;
            } else {
                rc.closest++;
                Isec r;
                if (tr.found) { r.bx = h.u; r.by = h.v; r.inst = h.inst; r.tri = h.tri; }
                else { r.bx = 0.0f; r.by = 0.0f; r.inst = kInvalidHit; r.tri = 0u; }
                Q.hit[pix] = r;
            }
            active = false;
        }
    }
    flush_counts(P.counters, rc, err, 4, P.countWork);
}

__global__ void __launch_bounds__(128, 8) k_di_candidates_finish(DICtx P, DICandidates Q) {
    uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    DIPixel px;
    if (x < P.b.width && y < P.b.height && di_pixel(P, x, y, px)) {
        uint32_t rng = makeSeed2(P.cam.seed, x, y);
        uint32_t resvRng = ~rng;
        DIResv r = di_zero();
        di_clear(r);
        DITraceAnswer tr{Q, y * P.b.width + x};
        di_sample_li(P, px.surf, load_material(P.sc, px.surf.matIndex), -px.ray.dir, rng, resvRng, r, tr);
        store_di(P.b.reservoirThis, (uint64_t)y * P.b.width + x, r);
    }
}

size_t di_split_bytes_per_pixel() {
    return sizeof(float4) + sizeof(uint32_t) +
           kDINeighbours * (sizeof(float4) + sizeof(uint2) + sizeof(float4) + 1 + sizeof(uint32_t));
}

cudaError_t launch_di(const DeviceSceneView& scene, const GrisDIBindings& b, const GrisCamera& cam,
                      const GrisCamera& prevCam, const GrisDISettings& set, int passes, unsigned long long* counters,
                      int countWork, KernelTimer* timer, cudaStream_t stream, void* split, uint64_t splitPixels,
                      const DISide* side) {
    DICtx P;
    P.sc = to_dev(scene);
    P.cam = make_cam(cam);
    P.prev = make_cam(prevCam);
    P.set = set;
    P.b = b;
    P.counters = counters;
    P.countWork = countWork;
    dim3 block(16, 8), grid((b.width + 15) / 16, (b.height + 7) / 8);
    const uint64_t npx = (uint64_t)b.width * b.height;
    const bool haveSplit = split && splitPixels >= npx;
    const int gridWalk = current_sm_count() * 16;
    /* the spatial pass's carving of the scratch: per pixel from, mq; per slot recA, recTo, recB,
     * vis, queue (slot k of pixel p at k * P + p) */
    DISplit S;
    memset(&S, 0, sizeof(S));
    if (haveSplit) {
        unsigned char* c = reinterpret_cast<unsigned char*>(split);
        const uint64_t slots = (uint64_t)kDINeighbours * npx;
        S.counts = reinterpret_cast<uint32_t*>(c); c += 256;
        S.from = reinterpret_cast<float4*>(c); c += npx * sizeof(float4);
        S.recA = reinterpret_cast<float4*>(c); c += slots * sizeof(float4);
        S.recTo = reinterpret_cast<float4*>(c); c += slots * sizeof(float4);
        S.recB = reinterpret_cast<uint2*>(c); c += slots * sizeof(uint2);
        S.mq = reinterpret_cast<uint32_t*>(c); c += npx * sizeof(uint32_t);
        S.queue = reinterpret_cast<uint32_t*>(c); c += slots * sizeof(uint32_t);
        S.vis = reinterpret_cast<uint8_t*>(c);
        S.P = npx;
    }
    if (passes & 1) {
        if (timer) timer->mark(GRIS_SLOT_DI_CANDIDATES, true, stream);
        if (haveSplit) {
            /* the scratch as two queues of 32-byte queries, the answers per pixel */
            DICandidates Q;
            unsigned char* c = reinterpret_cast<unsigned char*>(split);
            Q.counts = reinterpret_cast<uint32_t*>(c); c += 256;
            Q.qS = reinterpret_cast<float4*>(c); c += npx * 2 * sizeof(float4);
            Q.qC = reinterpret_cast<float4*>(c); c += npx * 2 * sizeof(float4);
            Q.hit = reinterpret_cast<Isec*>(c); c += npx * sizeof(Isec);
            Q.blocked = reinterpret_cast<uint8_t*>(c);
            cudaError_t e = cudaMemsetAsync(Q.counts, 0, 4 * sizeof(uint32_t), stream);
            if (e != cudaSuccess) return e;
            k_di_candidates_prepare<<<grid, block, 0, stream>>>(P, Q);
            /* the two walks share nothing but the ray counters (atomics): the shadow queries on
             * the side stream beside the closest-hit queries, joined before the finish kernel */
            const bool fork = side != nullptr && side->aux != nullptr && timer == nullptr;
            if (fork) {
                if ((e = cudaEventRecord(side->evFork, stream)) != cudaSuccess) return e;
                if ((e = cudaStreamWaitEvent(side->aux, side->evFork, 0)) != cudaSuccess) return e;
                k_di_candidates_walk<true><<<gridWalk, 128, 0, side->aux>>>(P, Q);
                if ((e = cudaEventRecord(side->evJoin, side->aux)) != cudaSuccess) return e;
            } else {
                k_di_candidates_walk<true><<<gridWalk, 128, 0, stream>>>(P, Q);
            }
            k_di_candidates_walk<false><<<gridWalk, 128, 0, stream>>>(P, Q);
            if (fork && (e = cudaStreamWaitEvent(stream, side->evJoin, 0)) != cudaSuccess) return e;
            k_di_candidates_finish<<<grid, block, 0, stream>>>(P, Q);
        } else {
            k_di_candidates<<<grid, block, 0, stream>>>(P);
        }
        if (timer) timer->mark(GRIS_SLOT_DI_CANDIDATES, false, stream);
    }
    if (passes & 2) {
        if (timer) timer->mark(GRIS_SLOT_DI_TEMPORAL, true, stream);
        k_di_temporal<<<grid, block, 0, stream>>>(P);
        if (timer) timer->mark(GRIS_SLOT_DI_TEMPORAL, false, stream);
    }
    if (passes & 4) {
        if (timer) timer->mark(GRIS_SLOT_DI_SPATIAL, true, stream);
        const bool phased = set.spatialReuse && set.shiftType == GRIS_DI_SHIFT_RECONNECTION;
        if (phased && haveSplit) {
            cudaError_t e = cudaMemsetAsync(S.counts, 0, 2 * sizeof(uint32_t), stream);
            if (e != cudaSuccess) return e;
            k_di_spatial_prepare<<<grid, block, 0, stream>>>(P, S);
            k_di_visibility<<<gridWalk, 128, 0, stream>>>(P, S);
            k_di_spatial_finish<<<grid, block, 0, stream>>>(P, S);
        } else {
            k_di_spatial<<<grid, block, 0, stream>>>(P);
        }
        if (timer) timer->mark(GRIS_SLOT_DI_SPATIAL, false, stream);
    }
    return cudaGetLastError();
}

}  // namespace grisrt
