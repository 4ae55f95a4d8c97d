/*
 * gris_kernels.cu — the GRIS hot path on sm_103a.
 *
 *   k_gbuffer      GBuffer.vert/.frag (raster) as one primary ray per pixel over the BVH
 *   k_path_trace   gris_path_trace.comp / tracePath (gris_path_trace.glsl:45-306)
 *   k_temporal     gris_resample_temporal.comp / temporalReuse (gris_resample_temporal.glsl:36-83)
 *   k_spatial      gris_resample_spatial.comp / spatialReuse + final shading + running mean
 *                  (gris_resample_spatial.glsl:36-135, gris_resample_spatial.comp:14-28)
 * with the hybrid shift traceReplayPathForHybridShift / GRISReservoirReuseAndMerge
 * (gris_retrace.glsl:42-236) shared by the two reuse kernels.
 *
 * One thread per pixel, 16 x 8 pixel tiles; traversal is the 8-wide BVH walk of
 * bvh_traverse.h. Ray counts are accumulated per thread and added once per warp.
 *
 * Batches (k_batch_gbuffer, k_batch_pass) run the same tasks for many views per launch. Their
 * path tracer can also run as a wavefront, one launch per stage and bounce level over compacted
 * queues: k_wave_begin, then per level the closest hits (k_wave_extend, or k_wave_trace_refill
 * for full levels + k_wave_trace_coop, one ray per warp, for levels under 8,192 rays),
 * k_wave_shade, the shadow queries (k_wave_shadow, or the same refilling / one-ray-per-warp
 * pair) and k_wave_post; k_gwave_* are the guided stages.
 */
#include <cuda_fp16.h>
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "gris_device.cuh"
#include "gris_kernels.h"
#include "ray_query.cuh"
#include "guide.cuh"
#include "guide_kernels.h"
#include "grisrt_internal.h"

namespace grisrt {

struct PassCtx {
    DevScene sc;
    CamD cam, prev;
    GrisSettings set;
    GrisPassBindings b;
    unsigned long long* counters;
    int countWork;
    /* guided batches: the network's raw outputs at every pixel's primary vertex (indexed by the
     * batch's path id = pixelBase + pixel), and the probability of drawing from the guide */
    const float* gPrim;
    const float* gPrimPrev;   /* the previous frame's, for shifts into the previous frame's pixels */
    float gMix;
    uint32_t pixelBase;
};

/* ------------------------------------------------------------------ path sampling */
struct Stream { PathSample ps; float weight, sumWeight; uint32_t sampleCount; };       /* gris_path_trace.glsl:10-23 */
GD void addStream(Stream& r, const PathSample& ps, float weight, float rnd) {           /* :25-33 */
    r.sumWeight += weight;
    if (rnd * r.sumWeight < weight) { r.weight = weight; r.ps = ps; r.sampleCount++; }
}
GD uint32_t nextRcVertexSampleState(uint32_t state, bool connectible) {                 /* :35-43 */
    if (state == 2u) return 2u;
    if (!connectible) return 0u;
    return state + (connectible ? 1u : 0u);
}

/* ------------------------------------------------------------------ guided sampling */
/* Whether the guide may draw at a vertex of this material (Lambert, or metallic-workflow rough
 * enough that the BSDF sampler never returns a specular-typed sample). */
GD bool guide_material(const Mat& m) { return m.type == 1u || (m.type == 2u && m.roughness >= 0.01f); }

/* One-sample MIS of the guide mixture (probability mix) and the BSDF sampler: s.pdf is the
 * mixture pdf of the direction, pdfBsdf the BSDF's own pdf of it. Draws sample1f + sample3f. */
GD bool guided_sample(const guide::Lobes& L, float mix, const Mat& mat, V3 albedo, V3 n, V3 wo, uint32_t& rng,
                      BsdfSample& s, float& pdfBsdf) {
    float u = sample1f(rng);
    V3 r = sample3f(rng);
    if (u < mix) {
        float d[3];
        guide::lobes_sample(L, r.x, r.y, r.z, d);
        s.wi = v3(d[0], d[1], d[2]);
        if (dot3(n, s.wi) <= 0.0f) return false;   /* no reflection there: a zero sample */
        s.bsdf = evalBSDF(mat, albedo, n, wo, s.wi);
        pdfBsdf = evalPdf(mat, n, wo, s.wi);
        s.type = kReflection | (mat.type == 1u ? kDiffuse : kGlossy);
    } else {
        if (!sampleBSDF(mat, albedo, n, wo, r, s)) return false;
        pdfBsdf = s.pdf;
    }
    s.pdf = mix * guide::lobes_pdf(L, s.wi.x, s.wi.y, s.wi.z) + (1.0f - mix) * pdfBsdf;
    return s.pdf >= 1e-6f;
}

/* The mixture at the primary vertex of pixel `idx` of the view (guided batches): false where
 * the primary vertex is not guided. */
GD bool primary_lobes(const PassCtx& P, uint64_t idx, const Mat& mat, guide::Lobes& L, bool previousFrame = false) {
    const float* g = previousFrame ? P.gPrimPrev : P.gPrim;
    if (!g || !guide_material(mat) || P.set.maxDepth < 2u) return false;
    guide::make_lobes(g + ((uint64_t)P.pixelBase + idx) * guide::kRaw, L);
    return true;
}


/* tracePath (gris_path_trace.glsl:45-306) as a state machine: begin() is the prologue up to the
 * bounce loop, step() one iteration of the loop (false where the reference breaks), end() the
 * epilogue that writes the canonical reservoir. Driving begin / step until false or maxDepth /
 * end performs exactly the reference's sequence of operations for the pixel.
 * kAcc (the converged-image estimators) also sums, per path, the candidate contributions given
 * to the reservoir stream (accCand) and every NEE / light-hit contribution (accAll).
 * kGuide (guided batches, implies kAcc): shade() leaves post() to the caller (kPost), and post()
 * draws the direction from the guide mixture or the BSDF (one-sample MIS) where the caller
 * passes the vertex's mixture; light hits then weigh the BSDF strategy by the BSDF's own pdf of
 * the sampled direction (pdfHit), so the estimand stays the unguided one. */
template <bool kAcc, bool kGuide = false>
struct PathTracerT {
    static constexpr bool kAccumulate = kAcc || kGuide;
    static constexpr bool kGuided = kGuide;
    uint32_t ix, iy;
    int bounce;
    uint32_t rng;
    V3 throughput, rcThroughput, wo, lastPos;
    bool isLastVertexConnectible;
    uint32_t sampleState, lastSampleState;
    Surf surf;
    Mat mat;
    BsdfSample s;
    Isec isec;
    PathSample pathSample;
    Stream stream;
    Ray3 ray;
    /* carried from shade() to post() of the same bounce */
    bool isThisVertexConnectible, nee;
    float resvRandSample;
    V3 lightRadiance, lightDir;
    V2 lightBary;
    float lightDist, lightPdf, lightJacobian;
    uint32_t lightId;
    V3 accCand, accAll;
    float pdfHit;        /* kGuide: the BSDF pdf of the last sampled direction */
    V3 thrSampled;       /* kGuide: the throughput at the last sampling, before its BSDF factor */
    uint32_t rec;        /* kGuide: this path holds a training record */

    GD void candidate() {
        addStream(stream, pathSample, luminance(pathSample.F), resvRandSample);
        if constexpr (kAccumulate) accCand = accCand + pathSample.F;
    }

    GD bool begin(const PassCtx& P, uint32_t px, uint32_t py) { return begin(P, px, py, P.cam.seed); }
    GD bool begin(const PassCtx& P, uint32_t px, uint32_t py, uint32_t frameSeed) {
        const DevScene& sc = P.sc;
        const int W = (int)P.b.width, H = (int)P.b.height;
        ix = px; iy = py;
        V2 uv = v2(((float)ix + 0.5f) / (float)W, ((float)iy + 0.5f) / (float)H);
        float depth = 0.0f; V3 norm = v3s(0.0f), albedo = v3s(0.0f); int matMeshId = 0;
        float4 dn = texture_bilinear(reinterpret_cast<const float4*>(P.b.depthNormal), W, H, uv);
        uint2 am = fetch_am(reinterpret_cast<const uint2*>(P.b.albedoMatId), W, H, (int)ix, (int)iy);
        if (!unpackGBuffer(dn, am, depth, norm, albedo, matMeshId)) return false;
        int matId = matMeshId >> 16;
        ray = pinholeCameraSampleRay(P.cam, v2(uv.x, 1.0f - uv.y));
        rng = makeSeed2(frameSeed, ix, iy);
        if constexpr (kAccumulate) { accCand = v3s(0.0f); accAll = v3s(0.0f); }
        if constexpr (kGuide) { pdfHit = 0.0f; thrSampled = v3s(0.0f); rec = 0u; }
        throughput = v3s(1.0f);
        rcThroughput = v3s(0.0f);
        wo = -ray.dir;
        lastPos = v3s(0.0f);
        isLastVertexConnectible = false;
        sampleState = 0u; lastSampleState = 0u;
        surf = surf_zero();
        surf.pos = ray.ori + ray.dir * (depth - 1e-4f);
        surf.norm = norm;
        surf.albedo = albedo;
        surf.isLight = false;
        mat = load_material(sc, (uint32_t)matId);
        s = bs_zero();
        isec = isec_zero();
        pathSample = ps_zero();
        pathSampleReset(pathSample);
        pathSample.primaryRng = rng;
        stream.ps = ps_zero(); stream.weight = 0.0f; stream.sumWeight = 0.0f; stream.sampleCount = 0u;
        bounce = 0;
        return true;
    }

    /* One iteration of the bounce loop (gris_path_trace.glsl:91-258) in two parts around the
     * NEE shadow query. shade() takes the closest hit of `ray` (bounce > 0) and runs up to the
     * light sample: kShadow asks the caller for the shadow query (surf.pos along lightDir, up to
     * lightDist - MinRayDistance) and then post(shadowed); kNext / kEnd report a vertex without
     * NEE whose post() already ran (continue / the reference breaks). */
    static constexpr int kEnd = 0, kShadow = 1, kNext = 2, kPost = 3;
    GD int shade(const PassCtx& P, const Isec& hit) {
        const DevScene& sc = P.sc;
        if (bounce > 0) {
            isec = hit;
            if (isec.inst == kInvalidHit) return kEnd;
            loadSurfaceInfo(sc, isec, surf);
            mat = load_material(sc, surf.matIndex);
        }
        setPathLength(pathSample.flags, (uint32_t)bounce + 1u);

        float cosPrevWi = dot3(ray.dir, surf.norm);
        float distToPrev = distance3(lastPos, surf.pos);
        float geometryJacobian = fabsf(cosPrevWi) / square(distToPrev);

        isThisVertexConnectible = surf.isLight || isBSDFConnectible(mat);

        lastSampleState = sampleState;
        sampleState = nextRcVertexSampleState(sampleState, isThisVertexConnectible);

        if (P.set.shiftType == kShiftReconnection && bounce == 1 && !surf.isLight) {
            sampleState = 2u;
            lastSampleState = 1u;
        }
        resvRandSample = sample1f(rng);

        if (surf.isLight) {
            if (bounce > 1 && cosPrevWi < 0.0f) {
                float weight = 1.0f;
                float sumPower = load_table(sc, 0).prob;
                float lightPdf = luminance(surf.albedo) / sumPower / geometryJacobian;
                if (!isSampleTypeDelta(s.type)) weight = MISWeight(kGuide ? pdfHit : s.pdf, lightPdf);
                V3 weightedLi = surf.albedo * weight;
                if constexpr (kAccumulate) accAll = accAll + weightedLi * throughput;
                if (sampleState == 2u && lastSampleState == 2u) {
                    pathSample.rcLi = pathSample.rcLi + weightedLi * rcThroughput;
                    pathSample.F = pathSample.F + weightedLi * throughput;
                } else if ((sampleState == 2u && lastSampleState == 1u) && isLastVertexConnectible &&
                           distToPrev > kDistanceThreshold) {
                    pathSample.rcIsec = isec;
                    pathSample.rcRng = rng;
                    pathSample.rcPrevSamplePdf = s.pdf;
                    pathSample.rcJacobian = geometryJacobian;
                    pathSample.rcLi = weightedLi;
                    pathSample.rcWi = v3s(0.0f);
                    pathSample.F = weightedLi * throughput;
                    setRcVertexId(pathSample.flags, (uint32_t)bounce);
                    setRcVertexType(pathSample.flags, kRcLightScattered);
                    candidate();
                }
                        }
            return kEnd;
        }

        bool connectible = isThisVertexConnectible && isLastVertexConnectible && distToPrev > kDistanceThreshold;

        if ((sampleState == 2u && lastSampleState == 1u) && (connectible || P.set.shiftType == kShiftReconnection)) {
            pathSample.rcIsec = isec;
            pathSample.rcRng = rng;
            pathSample.rcPrevSamplePdf = s.pdf;
            pathSample.rcJacobian = geometryJacobian;
            setRcVertexId(pathSample.flags, (uint32_t)bounce);
            setRcVertexType(pathSample.flags, kRcSurface);
            rcThroughput = v3s(1.0f);
        }

        V4 lightRandSample = sample4f(rng);
        resvRandSample = sample1f(rng);

        nee = bounce > 0 && !isBSDFDelta(mat);
        if (nee) {
            lightRadiance = sampleLightByPower(sc, surf.pos, lightDir, lightDist, lightPdf, lightJacobian, lightBary,
                                               lightId, lightRandSample);
            return kShadow;
        }
        if constexpr (kGuide) return kPost;
        return post(P, false) ? kNext : kEnd;
    }

    /* The ray post() continues the path with, computed ahead of it from the state shade() leaves
     * (unguided paths): Russian roulette and the BSDF sample draw the same numbers in post() and
     * read nothing the shadow query's answer changes (throughput, the material, the surface, wo),
     * so the next bounce's closest hit can be traced while the shadow query is. false: post()
     * will end the path. */
    GD bool next_ray(const PassCtx& P, V3& o, V3& d) const {
        uint32_t r = rng;
        if (bounce > 4) {
            float pdfTerminate = fmaxf(1.0f - luminance(throughput) * P.set.rrScale, 0.0f);
            if (sample1f(r) < pdfTerminate) return false;
        }
        BsdfSample s2;
        if (!sampleBSDF(mat, surf.albedo, surf.norm, wo, sample3f(r), s2) || s2.pdf < 1e-6f) return false;
        d = s2.wi;
        o = surf.pos + d * 1e-4f;
        return true;
    }

    /* second part: the NEE contribution (when shade() sampled a light), Russian roulette, BSDF
     * sampling; true = the path continues */
    GD bool post(const PassCtx& P, bool shadowed, const guide::Lobes* L = nullptr, float mix = 0.0f) {
        if (nee) {
            if (!shadowed && lightPdf > 1e-6f) {
                float bsdfPdf = absDot(surf.norm, lightDir) * kPiInv;
                float weight = MISWeight(lightPdf, bsdfPdf);
                V3 scatterTerm = evalBSDF(mat, surf.albedo, surf.norm, wo, lightDir) * satDot(surf.norm, lightDir);
                V3 weightedLi = lightRadiance / lightPdf * weight;
                if constexpr (kAccumulate) accAll = accAll + weightedLi * scatterTerm * throughput;
                if (sampleState == 2u && lastSampleState == 2u) {
                    pathSample.rcLi = pathSample.rcLi + weightedLi * scatterTerm * rcThroughput;
                    pathSample.F = pathSample.F + weightedLi * scatterTerm * throughput;
                } else if (sampleState == 2u && lastSampleState == 1u) {
                    pathSample.rcLi = weightedLi;
                    pathSample.rcWi = lightDir;
                    pathSample.F = weightedLi * scatterTerm * throughput;
                    candidate();
                } else if ((sampleState == 1u) && isThisVertexConnectible && lightDist > kDistanceThreshold) {
                    pathSample.rcIsec.bx = lightBary.x; pathSample.rcIsec.by = lightBary.y;
                    pathSample.rcIsec.inst = 0u; pathSample.rcIsec.tri = lightId;
                    pathSample.rcRng = rng;
                    pathSample.rcPrevSamplePdf = lightPdf;
                    pathSample.rcJacobian = lightJacobian;
                    pathSample.rcLi = lightRadiance * weight;
                    pathSample.rcWi = v3s(0.0f);
                    pathSample.F = weightedLi * scatterTerm * throughput;
                    setRcVertexId(pathSample.flags, (uint32_t)bounce + 1u);
                    setRcVertexType(pathSample.flags, kRcLightSampled);
                    candidate();
                }
            }
        }

        if (bounce > 4) {
            float pdfTerminate = fmaxf(1.0f - luminance(throughput) * P.set.rrScale, 0.0f);
            if (sample1f(rng) < pdfTerminate) return false;
            throughput = throughput / (1.0f - pdfTerminate);
            rcThroughput = rcThroughput / (1.0f - pdfTerminate);
        }

        if constexpr (kGuide) {
            thrSampled = throughput;
            if (L) {
                if (!guided_sample(*L, mix, mat, surf.albedo, surf.norm, wo, rng, s, pdfHit)) return false;
            } else {
                if (!sampleBSDF(mat, surf.albedo, surf.norm, wo, sample3f(rng), s) || s.pdf < 1e-6f) return false;
                pdfHit = s.pdf;
            }
        } else {
            if (!sampleBSDF(mat, surf.albedo, surf.norm, wo, sample3f(rng), s) || s.pdf < 1e-6f) return false;
        }

        float cosTheta = isSampleTypeDelta(s.type) ? 1.0f : absDot(surf.norm, s.wi);
        V3 scatterTerm = s.bsdf * cosTheta / s.pdf;
        throughput = throughput * scatterTerm;

        if (sampleState == 2u && lastSampleState == 2u) {
            rcThroughput = rcThroughput * scatterTerm;
        } else if (sampleState == 2u && lastSampleState == 1u) {
            pathSample.rcLi = v3s(0.0f);
            pathSample.rcWi = s.wi;
            pathSample.F = v3s(0.0f);
            rcThroughput = rcThroughput / s.pdf;
        }

        lastPos = surf.pos;
        wo = -s.wi;
        ray.dir = s.wi;
        ray.ori = surf.pos + ray.dir * 1e-4f;
        isLastVertexConnectible = isThisVertexConnectible;
        return true;
    }


    /* the whole iteration with the ray queries inline (grid and persistent forms) */
    GD bool step(const PassCtx& P, RayCount& rc, int& err) {
        Isec hit = isec_zero();
        if (bounce > 0) hit = traceClosestHit(P.sc, ray.ori, ray.dir, kMinRayDistance, kMaxRayDistance, rc, err);
        int r = shade(P, hit);
        if (r != kShadow) return r == kNext;
        bool shadowed = traceShadow(P.sc, surf.pos, kMinRayDistance, lightDir, lightDist - kMinRayDistance, rc, err);
        return post(P, shadowed);
    }

    /* the converged-image estimators' epilogue: the last candidate, without the stream */
    GD void finish() {
        if (sampleState == 2u && lastSampleState == 2u) accCand = accCand + pathSample.F;
    }

    /* after the loop (gris_path_trace.glsl:260-278) */
    GD void end(const PassCtx& P) {
        const int W = (int)P.b.width;
        Resv resv = resv_zero();
        resvReset(resv);
        if (sampleState == 2u && lastSampleState == 2u) addStream(stream, pathSample, luminance(pathSample.F), sample1f(rng));

        pathSample = stream.ps;
        if (stream.sumWeight > 0.0f && stream.weight > 0.0f) {
            pathSample.F = pathSample.F * (stream.sumWeight / stream.weight);
            pathSample.rcLi = pathSample.rcLi * (stream.sumWeight / stream.weight);
            resv.resampleWeight = luminance(pathSample.F);
        } else {
            pathSample.rcIsec.inst = kInvalidHit;
            pathSample.F = v3s(0.0f);
        }
        resv.s = pathSample;
        resv.sampleCount = 1.0f;
        store_resv(P.b.reservoirThis, (uint64_t)iy * (uint64_t)W + ix, resv);
    }
};
using PathTracer = PathTracerT<false>;

/* ------------------------------------------------------------------ hybrid shift (gris_retrace.glsl) */
/* traceReplayPathForHybridShift (:42-136) */
/* evalBSDF as one out-of-line copy (arguments by value) for the reuse passes, which evaluate the
 * BSDF at four sites: inlined there, the kernels' code outgrew the instruction cache (1080p C2:
 * spatial 2.67 -> 2.41 ms, temporal 0.98 -> 0.96 ms out of line). */
static __device__ __noinline__ V3 evalBSDFCall(Mat mat, V3 albedo, V3 n, V3 wo, V3 wi) { return evalBSDF(mat, albedo, n, wo, wi); }

GD void traceReplay(const PassCtx& P, Isec isec, Surf surf, Ray3 ray, uint32_t targetFlags, uint32_t rng, RcData& rcData,
                    RayCount& rc, int& err, const guide::Lobes* L = nullptr) {
    const DevScene& sc = P.sc;
    V3 throughput = v3s(1.0f);
    V3 wo = -ray.dir;
    Mat mat = load_material(sc, surf.matIndex);
    BsdfSample s = bs_zero();
    rcData.rcPrevThroughput = v3s(0.0f);
    rcData.rcPrevIsec.inst = kInvalidHit;
    uint32_t targetId = rcVertexId(targetFlags);
    if (targetId == 1u) {
        rcData.rcPrevIsec = isec;
        rcData.rcPrevWo = wo;
        rcData.rcPrevThroughput = throughput;
        return;
    }
    const int maxDepth = (int)P.set.maxDepth;
    for (int bounce = 0; bounce < maxDepth; bounce++) {
        if (bounce > 0) {
            isec = traceClosestHitCall(sc, ray.ori, ray.dir, kMinRayDistance, kMaxRayDistance, rc, err);
            if (isec.inst == kInvalidHit) break;
            loadSurfaceInfo(sc, isec, surf);
            mat = load_material(sc, surf.matIndex);
        }
        bool isThisVertexConnectible = isBSDFConnectible(mat);
        float resvRandSample = sample1f(rng);
        (void)resvRandSample;
        if (surf.isLight) break;
        if ((uint32_t)bounce == targetId - 1u) {
            if (isThisVertexConnectible) {
                rcData.rcPrevIsec = isec;
                rcData.rcPrevWo = wo;
                rcData.rcPrevThroughput = throughput;
            }
            break;
        }
        V4 lightRandSample = sample4f(rng);
        (void)lightRandSample;
        resvRandSample = sample1f(rng);
        if (bounce > 4) {
            float pdfTerminate = fmaxf(1.0f - luminance(throughput) * P.set.rrScale, 0.0f);
            if (sample1f(rng) < pdfTerminate) break;
            throughput = throughput / (1.0f - pdfTerminate);
        }
        if (L && bounce == 0) {
            /* a guided batch draws the primary vertex's direction from the destination pixel's mixture */
            float pdfBsdf;
            if (!guided_sample(*L, P.gMix, mat, surf.albedo, surf.norm, wo, rng, s, pdfBsdf)) break;
        } else if (!sampleBSDF(mat, surf.albedo, surf.norm, wo, sample3f(rng), s) || s.pdf < 1e-6f) {
            break;
        }
        float cosTheta = isSampleTypeDelta(s.type) ? 1.0f : absDot(surf.norm, s.wi);
        V3 scatterTerm = s.bsdf * cosTheta / s.pdf;
        throughput = throughput * scatterTerm;
        wo = -s.wi;
        ray.dir = s.wi;
        ray.ori = surf.pos + ray.dir * 1e-4f;
    }
}

/* The shift of a path sample into a destination pixel's domain (gris_retrace.glsl:138-219):
 * prefix replay from the destination's primary vertex, reconnection, visibility. On success
 * `out` is the shifted sample (F, rcJacobian and rcPrevSamplePdf of the destination) and
 * dstPHat = luminance(F * jacobian); srcPHat = luminance(src.F). */
struct Shift {
    bool valid;
    float dstPHat, srcPHat;
    PathSample out;
};
GD Shift shiftToDomain(const PassCtx& P, const Surf& dstPrimarySurf, const Isec& dstPrimaryIsec, const Ray3& primaryRay,
                       const PathSample& srcIn, RayCount& rc, int& err, const guide::Lobes* L = nullptr) {
    const DevScene& sc = P.sc;
    PathSample srcSample = srcIn;
    RcData dstRcData;
    dstRcData.rcPrevIsec = isec_zero(); dstRcData.rcPrevWo = v3s(0.0f); dstRcData.rcPrevThroughput = v3s(0.0f);
    Surf rcPrevSurf = surf_zero(), rcSurf = surf_zero();
    Mat rcMat = load_material(sc, 0xffffffffu), rcPrevMat = rcMat;
    V3 wi = v3s(0.0f);
    V3 Li = v3s(0.0f);
    bool srcSampleValid = false;
    float dstJacobian = 0.0f, jacobian = 0.0f, dist = 0.0f, dstPHat = 0.0f, dstSamplePdf = 0.0f;

    if (srcSample.rcIsec.inst != kInvalidHit) {
        traceReplay(P, dstPrimaryIsec, dstPrimarySurf, primaryRay, srcSample.flags, srcSample.primaryRng, dstRcData, rc, err,
                    L);
        if (dstRcData.rcPrevIsec.inst != kInvalidHit) {
            if (dstRcData.rcPrevIsec.inst == kSpecialHit) rcPrevSurf = dstPrimarySurf;
            else loadSurfaceInfo(sc, dstRcData.rcPrevIsec, rcPrevSurf);
            loadSurfaceInfo(sc, srcSample.rcIsec, rcSurf);
            rcMat = load_material(sc, rcSurf.matIndex);
            rcPrevMat = load_material(sc, rcPrevSurf.matIndex);
            dist = distance3(rcPrevSurf.pos, rcSurf.pos);
            wi = normalize3(rcSurf.pos - rcPrevSurf.pos);
            float cosTheta = -dot3(rcSurf.norm, wi);
            dstJacobian = fabsf(cosTheta) / square(dist);
            jacobian = dstJacobian / srcSample.rcJacobian;
            if (dist > kDistanceThreshold && cosTheta > 0.0f && !isnan(jacobian) && srcSample.rcJacobian > 0.0f &&
                isBSDFConnectible(rcPrevMat)) {
                if (traceVisibility(sc, rcPrevSurf.pos, rcSurf.pos, rc, err)) srcSampleValid = true;
            }
        }
    }

    Shift r;
    r.valid = srcSampleValid;
    r.dstPHat = 0.0f;
    r.srcPHat = luminance(srcSample.F);
    if (srcSampleValid) {
        uint32_t rcType = rcVertexType(srcSample.flags);
        if (!isnan(srcSample.rcPrevSamplePdf) && srcSample.rcPrevSamplePdf > 1e-6f) {
            Li = srcSample.rcLi;
            if (rcType == kRcSurface && length3(srcSample.rcWi) > 0.5f) {
                Li = Li * (evalBSDFCall(rcMat, rcSurf.albedo, rcSurf.norm, -wi, srcSample.rcWi) * satDot(rcSurf.norm, srcSample.rcWi));
            }
            Li = Li * (evalBSDFCall(rcPrevMat, rcPrevSurf.albedo, rcPrevSurf.norm, dstRcData.rcPrevWo, wi) * satDot(rcPrevSurf.norm, wi));
            Li = Li * dstRcData.rcPrevThroughput;
            Li = Li / srcSample.rcPrevSamplePdf;
            if (!isBlack(Li) && !isnan3(Li)) dstPHat = luminance(Li * jacobian);
            if (rcType == kRcLightSampled) {
                float sumPower = load_table(sc, 0).prob;
                dstSamplePdf = luminance(rcSurf.albedo) / sumPower / dstJacobian;
            } else {
                dstSamplePdf = evalPdf(rcPrevMat, rcPrevSurf.norm, dstRcData.rcPrevWo, wi);
                if (L && dstRcData.rcPrevIsec.inst == kSpecialHit)   /* the destination's primary vertex is guided */
                    dstSamplePdf = P.gMix * guide::lobes_pdf(*L, wi.x, wi.y, wi.z) + (1.0f - P.gMix) * dstSamplePdf;
            }
        }
        srcSample.rcJacobian = dstJacobian;
        srcSample.rcPrevSamplePdf = dstSamplePdf;
        srcSample.F = Li;
        if (srcSample.rcPrevSamplePdf < 1e-6f || isnan(srcSample.rcPrevSamplePdf)) srcSample.rcPrevSamplePdf = 0.0f;
        r.dstPHat = dstPHat;
    }
    r.out = srcSample;
    return r;
}

/* GRISReservoirReuseAndMerge (:138-236): the shift (as shiftToDomain, written out here: this
 * form keeps the reuse kernels' register footprint), the source weight scaled by the ratio of
 * the targets, the merge (M adds up: the M-proportional weights of the reference), the M cap. */
GD void reuseAndMerge(const PassCtx& P, Resv& dstResv, const Surf& dstPrimarySurf, const Isec& dstPrimaryIsec,
                      const Ray3& primaryRay, Resv srcResv, uint32_t& rng, RayCount& rc, int& err,
                      const guide::Lobes* L = nullptr) {
    const DevScene& sc = P.sc;
    PathSample srcSample = srcResv.s;
    RcData dstRcData;
    dstRcData.rcPrevIsec = isec_zero(); dstRcData.rcPrevWo = v3s(0.0f); dstRcData.rcPrevThroughput = v3s(0.0f);
    Surf rcPrevSurf = surf_zero(), rcSurf = surf_zero();
    Mat rcMat = load_material(sc, 0xffffffffu), rcPrevMat = rcMat;
    V3 wi = v3s(0.0f);
    V3 Li = v3s(0.0f);
    bool srcSampleValid = false;
    float dstJacobian = 0.0f, jacobian = 0.0f, dist = 0.0f, dstPHat = 0.0f, dstSamplePdf = 0.0f;

    if (srcSample.rcIsec.inst != kInvalidHit) {
        traceReplay(P, dstPrimaryIsec, dstPrimarySurf, primaryRay, srcSample.flags, srcSample.primaryRng, dstRcData, rc, err,
                    L);
        if (dstRcData.rcPrevIsec.inst != kInvalidHit) {
            if (dstRcData.rcPrevIsec.inst == kSpecialHit) rcPrevSurf = dstPrimarySurf;
            else loadSurfaceInfo(sc, dstRcData.rcPrevIsec, rcPrevSurf);
            loadSurfaceInfo(sc, srcSample.rcIsec, rcSurf);
            rcMat = load_material(sc, rcSurf.matIndex);
            rcPrevMat = load_material(sc, rcPrevSurf.matIndex);
            dist = distance3(rcPrevSurf.pos, rcSurf.pos);
            wi = normalize3(rcSurf.pos - rcPrevSurf.pos);
            float cosTheta = -dot3(rcSurf.norm, wi);
            dstJacobian = fabsf(cosTheta) / square(dist);
            jacobian = dstJacobian / srcSample.rcJacobian;
            if (dist > kDistanceThreshold && cosTheta > 0.0f && !isnan(jacobian) && srcSample.rcJacobian > 0.0f &&
                isBSDFConnectible(rcPrevMat)) {
                if (traceVisibility(sc, rcPrevSurf.pos, rcSurf.pos, rc, err)) srcSampleValid = true;
            }
        }
    }

    if (srcSampleValid) {
        uint32_t rcType = rcVertexType(srcSample.flags);
        if (!isnan(srcSample.rcPrevSamplePdf) && srcSample.rcPrevSamplePdf > 1e-6f) {
            Li = srcSample.rcLi;
            if (rcType == kRcSurface && length3(srcSample.rcWi) > 0.5f) {
                Li = Li * (evalBSDFCall(rcMat, rcSurf.albedo, rcSurf.norm, -wi, srcSample.rcWi) * satDot(rcSurf.norm, srcSample.rcWi));
            }
            Li = Li * (evalBSDFCall(rcPrevMat, rcPrevSurf.albedo, rcPrevSurf.norm, dstRcData.rcPrevWo, wi) * satDot(rcPrevSurf.norm, wi));
            Li = Li * dstRcData.rcPrevThroughput;
            Li = Li / srcSample.rcPrevSamplePdf;
            if (!isBlack(Li) && !isnan3(Li)) dstPHat = luminance(Li * jacobian);
            if (rcType == kRcLightSampled) {
                float sumPower = load_table(sc, 0).prob;
                dstSamplePdf = luminance(rcSurf.albedo) / sumPower / dstJacobian;
            } else {
                dstSamplePdf = evalPdf(rcPrevMat, rcPrevSurf.norm, dstRcData.rcPrevWo, wi);
                if (L && dstRcData.rcPrevIsec.inst == kSpecialHit)   /* the destination's primary vertex is guided */
                    dstSamplePdf = P.gMix * guide::lobes_pdf(*L, wi.x, wi.y, wi.z) + (1.0f - P.gMix) * dstSamplePdf;
            }
        }
        float srcPHat = luminance(srcSample.F);
        srcSample.rcJacobian = dstJacobian;
        srcSample.rcPrevSamplePdf = dstSamplePdf;
        srcSample.F = Li;
        if (srcSample.rcPrevSamplePdf < 1e-6f || isnan(srcSample.rcPrevSamplePdf)) srcSample.rcPrevSamplePdf = 0.0f;
        srcResv.s = srcSample;
        srcResv.resampleWeight *= dstPHat / srcPHat;
    } else {
        srcResv.resampleWeight = 0.0f;
    }
    if (resvIsValid(srcResv)) resvMerge(dstResv, srcResv, sample1f(rng));
    resvCap(dstResv, (float)P.set.cap);
}

/* The shift of reservoir `src` into the destination pixel up to its reconnection's visibility
 * query (reuseAndMerge, gris_retrace.glsl:138-219, without the query): the prefix replay, the
 * reconnection's Jacobian and gates, and what the sample becomes if the query finds the segment
 * visible — its resampling weight (src.resampleWeight * dstPHat / srcPHat), Jacobian, pdf and F —
 * with the query's endpoints. Returns kShiftNoQuery when the shift fails before the query (the
 * source then merges with weight 0), kShiftQuery when the query decides between that weight and
 * 0, kShiftQueryBadWeight when the weight if visible is not a valid weight (NaN or negative: a
 * visible segment then merges nothing, an occluded one merges with weight 0). */
constexpr int kShiftNoQuery = 0, kShiftQuery = 1, kShiftQueryBadWeight = 2;
struct ShiftPending {
    float rw, jac, pdf;
    V3 F, from, to;
};
GD int shift_until_query(const PassCtx& P, const Surf& dst, const Isec& dstIsec, const Ray3& ray, const Resv& src,
                         const guide::Lobes* Lp, ShiftPending& q, RayCount& rc, int& err) {
    const DevScene& sc = P.sc;
    const PathSample& s = src.s;
    RcData rd;
    rd.rcPrevIsec = isec_zero(); rd.rcPrevWo = v3s(0.0f); rd.rcPrevThroughput = v3s(0.0f);
    Surf rcPrevSurf = surf_zero(), rcSurf = surf_zero();
    q.rw = 0.0f; q.jac = 0.0f; q.pdf = 0.0f; q.F = v3s(0.0f);
    bool query = false;
    float dstJacobian = 0.0f, jacobian = 0.0f;
    V3 wi = v3s(0.0f);
    Mat rcMat = load_material(sc, 0xffffffffu), rcPrevMat = rcMat;
    if (s.rcIsec.inst != kInvalidHit) {
        traceReplay(P, dstIsec, dst, ray, s.flags, s.primaryRng, rd, rc, err, Lp);
        if (rd.rcPrevIsec.inst != kInvalidHit) {
            if (rd.rcPrevIsec.inst == kSpecialHit) rcPrevSurf = dst;
            else loadSurfaceInfo(sc, rd.rcPrevIsec, rcPrevSurf);
            loadSurfaceInfo(sc, s.rcIsec, rcSurf);
            rcMat = load_material(sc, rcSurf.matIndex);
            rcPrevMat = load_material(sc, rcPrevSurf.matIndex);
            float dist = distance3(rcPrevSurf.pos, rcSurf.pos);
            wi = normalize3(rcSurf.pos - rcPrevSurf.pos);
            float cosTheta = -dot3(rcSurf.norm, wi);
            dstJacobian = fabsf(cosTheta) / square(dist);
            jacobian = dstJacobian / s.rcJacobian;
            query = dist > kDistanceThreshold && cosTheta > 0.0f && !isnan(jacobian) && s.rcJacobian > 0.0f &&
                    isBSDFConnectible(rcPrevMat);
        }
    }
    if (!query) return kShiftNoQuery;
    V3 Li = v3s(0.0f);
    float dstPHat = 0.0f, dstSamplePdf = 0.0f;
    uint32_t rcType = rcVertexType(s.flags);
    if (!isnan(s.rcPrevSamplePdf) && s.rcPrevSamplePdf > 1e-6f) {
        Li = s.rcLi;
        if (rcType == kRcSurface && length3(s.rcWi) > 0.5f) {
            Li = Li * (evalBSDFCall(rcMat, rcSurf.albedo, rcSurf.norm, -wi, s.rcWi) * satDot(rcSurf.norm, s.rcWi));
        }
        Li = Li * (evalBSDFCall(rcPrevMat, rcPrevSurf.albedo, rcPrevSurf.norm, rd.rcPrevWo, wi) * satDot(rcPrevSurf.norm, wi));
        Li = Li * rd.rcPrevThroughput;
        Li = Li / s.rcPrevSamplePdf;
        if (!isBlack(Li) && !isnan3(Li)) dstPHat = luminance(Li * jacobian);
        if (rcType == kRcLightSampled) {
            float sumPower = load_table(sc, 0).prob;
            dstSamplePdf = luminance(rcSurf.albedo) / sumPower / dstJacobian;
        } else {
            dstSamplePdf = evalPdf(rcPrevMat, rcPrevSurf.norm, rd.rcPrevWo, wi);
            if (Lp && rd.rcPrevIsec.inst == kSpecialHit)
                dstSamplePdf = P.gMix * guide::lobes_pdf(*Lp, wi.x, wi.y, wi.z) + (1.0f - P.gMix) * dstSamplePdf;
        }
    }
    float srcPHat = luminance(s.F);
    q.rw = src.resampleWeight * (dstPHat / srcPHat);
    q.jac = dstJacobian;
    q.pdf = (dstSamplePdf < 1e-6f || isnan(dstSamplePdf)) ? 0.0f : dstSamplePdf;
    q.F = Li;
    q.from = rcPrevSurf.pos;
    q.to = rcSurf.pos;
    return (!isnan(q.rw) && q.rw >= 0.0f) ? kShiftQuery : kShiftQueryBadWeight;
}

/* Pairwise generalised balance heuristic (GrisSettings.misWeights = 1). The canonical reservoir
 * c (M_c, sample x_c) and k reused reservoirs i (M_i, x_i): pair i weighs technique i against
 * a 1/k share of the canonical one, m_i(y) = M_i p_i(y) / (M_i p_i(y) + (M_c/k) p_c(y)), where
 * p_i(y) is i's target at the shift of y into i's pixel times the shift's Jacobian. For a
 * reused sample y_i = T(x_i) that is M_i pHat_i(x_i) / (M_i pHat_i(x_i) + (M_c/k) dstPHat) (the
 * forward shift's numbers); the canonical sample gets (1/k) sum over the pairs of the
 * complementary weight, which needs the shift of x_c into each reused pixel (backward shift).
 * Resampling weights w = m * target * unbiased contribution weight (= resampleWeight / M of the
 * source); the merged reservoir keeps the reference's representation (resampleWeight = sum w *
 * M, M = sum of the Ms), so the final shading is unchanged. */
struct PairwiseMerge {
    float Mc, pc, Rc;      /* canonical: M, target of its own sample, resampleWeight */
    float k, mcSum, wSum, M;
    PathSample canon, sel;
    GD void begin(const Resv& canonical, float kNeighbours) {
        Mc = canonical.sampleCount;
        pc = luminance(canonical.s.F);
        Rc = canonical.resampleWeight;
        k = kNeighbours;
        mcSum = 0.0f; wSum = 0.0f; M = Mc;
        canon = canonical.s;
        sel = canonical.s;
    }
    /* a reused reservoir: its forward shift, and the target of the canonical sample shifted into
     * its pixel times that shift's Jacobian (pBack, 0 if the shift failed) */
    GD void add(const Resv& src, const Shift& fw, float pBack, float rnd) {
        const float Mi = src.sampleCount;
        if (pc > 0.0f) {
            float a = (Mc / k) * pc, b = Mi * pBack;
            mcSum += a / (a + b);
        }
        float w = 0.0f;
        if (fw.valid && fw.dstPHat > 0.0f && fw.srcPHat > 0.0f && Mi > 0.0f)
            w = (1.0f / k) * fw.dstPHat * src.resampleWeight / (Mi * fw.srcPHat + (Mc / k) * fw.dstPHat);
        if (!(w >= 0.0f) || isinf(w)) w = 0.0f;
        wSum += w;
        if (rnd * wSum < w) sel = fw.out;
        M += Mi;
    }
    /* a reused slot without a reservoir: its pair gives the canonical sample the full weight */
    GD void skip() { if (pc > 0.0f) mcSum += 1.0f; }
    /* the canonical candidate last, then the merged reservoir */
    GD Resv finish(float rnd, float cap) {
        float wc = (pc > 0.0f && Mc > 0.0f) ? (mcSum / k) * Rc / Mc : 0.0f;
        if (!(wc >= 0.0f) || isinf(wc)) wc = 0.0f;
        float total = wSum + wc;
        Resv out = resv_zero();
        resvReset(out);
        out.s = (rnd * total < wc) ? canon : sel;
        out.sampleCount = M;
        out.resampleWeight = total * M;
        resvCap(out, cap);
        return out;
    }
};

/* ------------------------------------------------------------------ temporal reuse */
/* temporalReuse (gris_resample_temporal.glsl:36-83): begin() finds the previous reservoir
 * (findPreviousReservoir, :11-34) and finishes the pixel when there is nothing to merge;
 * step() shifts and merges it and writes the temporary reservoir. */
template <bool kGuide, bool kPair = false>
struct TemporalTaskT {
    uint64_t idx;
    Resv resv, src;
    Surf dst;
    Isec dstIsec;
    Ray3 ray;
    uint32_t resvRng;
    /* the previous frame's pixel (pairwise weights: the shift of the canonical sample into it) */
    Surf prevSurf;
    Isec prevIsec;
    Ray3 prevRay;
    uint32_t pidx;
    /* deferred (set by the caller): begin() reads nothing of this frame's path tracing — the
     * current reservoir is neither loaded nor copied; copy reports a pixel whose current
     * reservoir goes to the temporary one unmerged (the three-launch form's finish kernel copies
     * it), so that the pass's shifts and queries can run beside the path tracer */
    bool deferred = false, copy = false;

    GD void finish(const PassCtx& P) {
        if (deferred) { copy = true; return; }
        resvResetIfInvalid(resv);
        store_resv(P.b.reservoirTemp, idx, resv);
    }

    GD bool begin(const PassCtx& P, uint32_t ix, uint32_t iy, RayCount&, int&) {
        const int W = (int)P.b.width, H = (int)P.b.height;
        const uint64_t n = (uint64_t)W * (uint64_t)H;
        V2 uv = v2(((float)ix + 0.5f) / (float)W, ((float)iy + 0.5f) / (float)H);
        float depth = 0.0f; V3 norm = v3s(0.0f), albedo = v3s(0.0f); int matMeshId = 0;
        float4 dn = texture_bilinear(reinterpret_cast<const float4*>(P.b.depthNormal), W, H, uv);
        uint2 am = fetch_am(reinterpret_cast<const uint2*>(P.b.albedoMatId), W, H, (int)ix, (int)iy);
        if (!unpackGBuffer(dn, am, depth, norm, albedo, matMeshId)) return false;
        const __half2* mv = reinterpret_cast<const __half2*>(P.b.motion);
        float2 motion = __half22float2(mv[(uint64_t)iy * W + ix]);
        int matId = matMeshId >> 16;
        ray = pinholeCameraSampleRay(P.cam, v2(uv.x, 1.0f - uv.y));
        uint32_t rng = makeSeed2(P.cam.seed, ix, iy) ^ 1u;
        resvRng = ~rng;
        V3 pos = ray.ori + ray.dir * (depth - 1e-4f);
        idx = (uint64_t)iy * W + ix;
        if (!deferred) resv = load_resv(P.b.reservoirThis, idx, n);
        dstIsec.bx = uv.x; dstIsec.by = uv.y; dstIsec.inst = kSpecialHit; dstIsec.tri = 0u;
        if (P.set.temporalReuse) {
            src = resv_zero();
            resvReset(src);
            dst.pos = pos; dst.norm = norm; dst.albedo = albedo; dst.matIndex = (uint32_t)matId; dst.isLight = false;
            if ((P.cam.frameIndex & kCameraClearFlag) == 0u) {
                V2 puv = v2(uv.x + motion.x, uv.y + motion.y);
                bool found = false;
                if (!(puv.x < 0.0f || puv.y < 0.0f || puv.x > 1.0f || puv.y > 1.0f)) {
                    int px = (int)(puv.x * (float)P.cam.w), py = (int)(puv.y * (float)P.cam.h);
                    float depthPrev = 0.0f; V3 normalPrev = v3s(0.0f), albedoPrev = v3s(0.0f); int matMeshIdPrev = 0;
                    float4 pdn = texture_bilinear(reinterpret_cast<const float4*>(P.b.depthNormalPrev), W, H, puv);
                    uint2 pam = fetch_am(reinterpret_cast<const uint2*>(P.b.albedoMatIdPrev), W, H, px, py);
                    if (unpackGBuffer(pdn, pam, depthPrev, normalPrev, albedoPrev, matMeshIdPrev)) {
                        Ray3 pray = pinholeCameraSampleRay(P.prev, v2(puv.x, 1.0f - puv.y));
                        V3 posPrev = pray.ori + pray.dir * (depthPrev - 1e-4f);
                        if (!(matMeshIdPrev != matMeshId || dot3(normalPrev, norm) < 0.95f || distance3(pos, posPrev) > 0.5f)) {
                            pidx = (uint32_t)P.cam.w * (uint32_t)py + (uint32_t)px;
                            src = load_resv(P.b.reservoirPrev, pidx, n);
                            found = true;
                            if (kPair && P.set.misWeights) {
                                prevSurf.pos = posPrev; prevSurf.norm = normalPrev; prevSurf.albedo = albedoPrev;
                                prevSurf.matIndex = (uint32_t)(matMeshIdPrev >> 16); prevSurf.isLight = false;
                                prevIsec.bx = puv.x; prevIsec.by = puv.y; prevIsec.inst = kSpecialHit; prevIsec.tri = 0u;
                                prevRay = pray;
                            }
                        }
                    }
                }
                if (found && resvIsValid(src)) return true;
            }
        }
        finish(P);
        return false;
    }

    GD bool step(const PassCtx& P, RayCount& rc, int& err) {
        const guide::Lobes* Lp = nullptr;
        guide::Lobes L;
        if constexpr (kGuide) {
            if (primary_lobes(P, idx, load_material(P.sc, dst.matIndex), L)) Lp = &L;
        }
        if (!(kPair && P.set.misWeights)) {
            reuseAndMerge(P, resv, dst, dstIsec, ray, src, resvRng, rc, err, Lp);
        } else {
            PairwiseMerge pm;
            pm.begin(resv, 1.0f);
            Shift fw = shiftToDomain(P, dst, dstIsec, ray, src.s, rc, err, Lp);
            float pBack = 0.0f;
            if (pm.pc > 0.0f) {
                const guide::Lobes* Lq = nullptr;
                guide::Lobes Lprev;
                if constexpr (kGuide) {
                    if (primary_lobes(P, pidx, load_material(P.sc, prevSurf.matIndex), Lprev, true)) Lq = &Lprev;
                }
                Shift bw = shiftToDomain(P, prevSurf, prevIsec, prevRay, resv.s, rc, err, Lq);
                if (bw.valid) pBack = bw.dstPHat;
            }
            pm.add(src, fw, pBack, sample1f(resvRng));
            resv = pm.finish(sample1f(resvRng), (float)P.set.cap);
        }
        finish(P);
        return false;
    }
};
using TemporalTask = TemporalTaskT<false>;

/* ------------------------------------------------------------------ spatial reuse + final shading */
/* spatialReuse (gris_resample_spatial.glsl:36-135) + the running mean of
 * gris_resample_spatial.comp:21-27. begin() reads the pixel (a background pixel only updates the
 * running mean); each step() handles one neighbour (findNeighborReservoir, :11-34, then the shift
 * and merge); the last step writes the reservoir, shades and accumulates. */
template <bool kGuide, bool kPair = false>
struct SpatialTaskT {
    PairwiseMerge pm;   /* pairwise weights (misWeights = 1) */
    uint32_t ix, iy, i, rng;
    uint64_t idx;
    Resv resv;
    Surf dst;
    Isec dstIsec;
    Ray3 ray;

    GD static void accumulate(const PassCtx& P, uint32_t x, uint32_t y, V3 color) {
        float frameCount = (float)(P.cam.frameIndex & kCameraFrameIndexMask);
        float4* out = reinterpret_cast<float4*>(P.b.output) + (uint64_t)y * P.b.width + x;
        float4 o = *out;
        V3 acc = v3(o.x, o.y, o.z);
        acc = (acc * frameCount + color) / (frameCount + 1.0f);
        *out = make_float4(acc.x, acc.y, acc.z, 1.0f);
    }

    GD bool begin(const PassCtx& P, uint32_t px, uint32_t py, RayCount&, int&) {
        const int W = (int)P.b.width, H = (int)P.b.height;
        ix = px; iy = py;
        V2 uv = v2(((float)ix + 0.5f) / (float)W, ((float)iy + 0.5f) / (float)H);
        float depth = 0.0f; V3 norm = v3s(0.0f), albedo = v3s(0.0f); int matMeshId = 0;
        float4 dn = texture_bilinear(reinterpret_cast<const float4*>(P.b.depthNormal), W, H, uv);
        uint2 am = fetch_am(reinterpret_cast<const uint2*>(P.b.albedoMatId), W, H, (int)ix, (int)iy);
        if (!unpackGBuffer(dn, am, depth, norm, albedo, matMeshId)) {
            accumulate(P, ix, iy, v3s(0.0f));
            return false;
        }
        rng = makeSeed2(P.cam.seed, ix, iy) ^ 2u;
        ray = pinholeCameraSampleRay(P.cam, v2(uv.x, 1.0f - uv.y));
        V3 pos = ray.ori + ray.dir * (depth - 1e-4f);
        int matId = matMeshId >> 16;
        idx = (uint64_t)iy * W + ix;
        resv = load_resv(P.b.reservoirTemp, idx, (uint64_t)W * (uint64_t)H);
        dstIsec.bx = uv.x; dstIsec.by = uv.y; dstIsec.inst = kSpecialHit; dstIsec.tri = 0u;
        dst.pos = pos; dst.norm = norm; dst.albedo = albedo; dst.matIndex = (uint32_t)matId; dst.isLight = false;
        i = 0;
        if (kPair && P.set.misWeights && P.set.spatialReuse && P.set.spatialNeighbors > 0u) pm.begin(resv, (float)P.set.spatialNeighbors);
        return true;
    }

    /* The neighbours under the reference's weights (misWeights = 0) in chunks of kChunk, each in
     * three phases with the results and draw order of one step() per neighbour:
     *   1. per neighbour: the gather and gates, the source reservoir, the replay and the shift up
     *      to its visibility query (target, pdf, Jacobian, weight if visible), and the merge's
     *      draw where reuseAndMerge takes it — always, unless the weight if visible is not a
     *      valid weight, in which case the query is answered on the spot, as it decides the draw;
     *   2. the lane's pending queries back to back (a warp walks max-over-lanes of the query
     *      counts rather than one walk per neighbour index, most lanes having no query);
     *   3. the merges and M caps in neighbour order with the verdicts. */
    static constexpr uint32_t kChunk = 4;
    struct Pending {
        float rw, rnd, jac, pdf;   /* weight if visible; merge draw; the shifted sample's Jacobian and pdf */
        float M;                   /* the source's sample count */
        V3 F, from, to;            /* the shifted sample's F; the query's endpoints */
        uint32_t nidx, state;      /* source pixel; kMerge | kQuery | kVisible */
    };
    static constexpr uint32_t kMerge = 1u, kQuery = 2u, kVisible = 4u;

    GD void reuse_phased(const PassCtx& P, RayCount& rc, int& err) {
        const DevScene& sc = P.sc;
        const int W = (int)P.b.width, H = (int)P.b.height;
        const uint64_t n = (uint64_t)W * (uint64_t)H;
        const float tx = 1.0f / (float)W, ty = 1.0f / (float)H;
        const V2 uv = v2(dstIsec.bx, dstIsec.by);
        const guide::Lobes* Lp = nullptr;
        guide::Lobes L;
        if constexpr (kGuide) {
            if (primary_lobes(P, idx, load_material(sc, dst.matIndex), L)) Lp = &L;
        }
        for (uint32_t base = 0; base < P.set.spatialNeighbors; base += kChunk) {
            const uint32_t end = min(P.set.spatialNeighbors, base + kChunk);
            Pending e[kChunk];
            uint32_t m = 0, queries = 0;
            for (uint32_t k = base; k < end; k++) {
                V2 d = toConcentricDisk(sample2f(rng));
                V2 nb = v2(uv.x + d.x * P.set.spatialRadius * tx, uv.y + d.y * P.set.spatialRadius * ty);
                if (nb.x < 0.0f || nb.y < 0.0f || nb.x > 1.0f || nb.y > 1.0f) continue;
                int px = (int)(nb.x * (float)P.cam.w), py = (int)(nb.y * (float)P.cam.h);
                float depthN = 0.0f; V3 normalN = v3s(0.0f), albedoN = v3s(0.0f); int matMeshIdN = 0;
                float4 ndn = texture_bilinear(reinterpret_cast<const float4*>(P.b.depthNormal), W, H, nb);
                uint2 nam = fetch_am(reinterpret_cast<const uint2*>(P.b.albedoMatId), W, H, px, py);
                if (!unpackGBuffer(ndn, nam, depthN, normalN, albedoN, matMeshIdN)) continue;
                Ray3 nray = pinholeCameraSampleRay(P.cam, v2(nb.x, 1.0f - nb.y));
                V3 posN = nray.ori + nray.dir * (depthN - 1e-4f);
                if (dot3(normalN, dst.norm) < 0.9f || distance3(dst.pos, posN) > 0.4f) continue;
                const uint32_t nidx = (uint32_t)P.cam.w * (uint32_t)py + (uint32_t)px;
                const Resv src = load_resv(P.b.reservoirTemp, nidx, n);
                if (!resvIsValid(src)) continue;
                /* reuseAndMerge up to the visibility query */
                const PathSample& s = src.s;
                RcData rd;
                rd.rcPrevIsec = isec_zero(); rd.rcPrevWo = v3s(0.0f); rd.rcPrevThroughput = v3s(0.0f);
                Surf rcPrevSurf = surf_zero(), rcSurf = surf_zero();
                Pending& q = e[m];
                q.rw = 0.0f; q.jac = 0.0f; q.pdf = 0.0f; q.F = v3s(0.0f); q.nidx = nidx; q.state = 0u;
                q.M = src.sampleCount;
                bool query = false;
                float dstJacobian = 0.0f, jacobian = 0.0f;
                V3 wi = v3s(0.0f);
                Mat rcMat = load_material(sc, 0xffffffffu), rcPrevMat = rcMat;
                if (s.rcIsec.inst != kInvalidHit) {
                    traceReplay(P, dstIsec, dst, ray, s.flags, s.primaryRng, rd, rc, err, Lp);
                    if (rd.rcPrevIsec.inst != kInvalidHit) {
                        if (rd.rcPrevIsec.inst == kSpecialHit) rcPrevSurf = dst;
                        else loadSurfaceInfo(sc, rd.rcPrevIsec, rcPrevSurf);
                        loadSurfaceInfo(sc, s.rcIsec, rcSurf);
                        rcMat = load_material(sc, rcSurf.matIndex);
                        rcPrevMat = load_material(sc, rcPrevSurf.matIndex);
                        float dist = distance3(rcPrevSurf.pos, rcSurf.pos);
                        wi = normalize3(rcSurf.pos - rcPrevSurf.pos);
                        float cosTheta = -dot3(rcSurf.norm, wi);
                        dstJacobian = fabsf(cosTheta) / square(dist);
                        jacobian = dstJacobian / s.rcJacobian;
                        query = dist > kDistanceThreshold && cosTheta > 0.0f && !isnan(jacobian) && s.rcJacobian > 0.0f &&
                                isBSDFConnectible(rcPrevMat);
                    }
                }
                bool merge = true;
                if (query) {
                    V3 Li = v3s(0.0f);
                    float dstPHat = 0.0f, dstSamplePdf = 0.0f;
                    uint32_t rcType = rcVertexType(s.flags);
                    if (!isnan(s.rcPrevSamplePdf) && s.rcPrevSamplePdf > 1e-6f) {
                        Li = s.rcLi;
                        if (rcType == kRcSurface && length3(s.rcWi) > 0.5f) {
                            Li = Li * (evalBSDFCall(rcMat, rcSurf.albedo, rcSurf.norm, -wi, s.rcWi) * satDot(rcSurf.norm, s.rcWi));
                        }
                        Li = Li * (evalBSDFCall(rcPrevMat, rcPrevSurf.albedo, rcPrevSurf.norm, rd.rcPrevWo, wi) * satDot(rcPrevSurf.norm, wi));
                        Li = Li * rd.rcPrevThroughput;
                        Li = Li / s.rcPrevSamplePdf;
                        if (!isBlack(Li) && !isnan3(Li)) dstPHat = luminance(Li * jacobian);
                        if (rcType == kRcLightSampled) {
                            float sumPower = load_table(sc, 0).prob;
                            dstSamplePdf = luminance(rcSurf.albedo) / sumPower / dstJacobian;
                        } else {
                            dstSamplePdf = evalPdf(rcPrevMat, rcPrevSurf.norm, rd.rcPrevWo, wi);
                            if (Lp && rd.rcPrevIsec.inst == kSpecialHit)
                                dstSamplePdf = P.gMix * guide::lobes_pdf(*Lp, wi.x, wi.y, wi.z) + (1.0f - P.gMix) * dstSamplePdf;
                        }
                    }
                    float srcPHat = luminance(s.F);
                    q.rw = src.resampleWeight * (dstPHat / srcPHat);
                    q.jac = dstJacobian;
                    q.pdf = (dstSamplePdf < 1e-6f || isnan(dstSamplePdf)) ? 0.0f : dstSamplePdf;
                    q.F = Li;
                    q.from = rcPrevSurf.pos; q.to = rcSurf.pos;
                    if (!isnan(q.rw) && q.rw >= 0.0f) {
                        q.state = kQuery;
                        queries |= 1u << m;
                    } else {   /* visible: an invalid weight, no merge and no draw; occluded: weight 0, merged */
                        bool vis = traceVisibility(sc, q.from, q.to, rc, err);
                        merge = !vis;
                    }
                }
                if (merge) { q.state |= kMerge; q.rnd = sample1f(rng); }
                m++;
            }
            for (uint32_t pending = queries; pending; pending &= pending - 1u) {
                const uint32_t j = (uint32_t)__ffs(pending) - 1u;
                if (traceVisibility(sc, e[j].from, e[j].to, rc, err)) e[j].state |= kVisible;
            }
            int sel = -1;
            for (uint32_t j = 0; j < m; j++) {
                if (e[j].state & kMerge) {
                    const float w = (e[j].state & kVisible) ? e[j].rw : 0.0f;
                    resv.sampleCount += e[j].M;
                    resv.resampleWeight += w;
                    if (e[j].rnd * resv.resampleWeight < w) sel = (int)j;
                }
                resvCap(resv, (float)P.set.cap);
            }
            if (sel >= 0) {
                Resv src = load_resv(P.b.reservoirTemp, e[sel].nidx, n);
                resv.s = src.s;
                if (e[sel].state & kVisible) {
                    resv.s.rcJacobian = e[sel].jac;
                    resv.s.rcPrevSamplePdf = e[sel].pdf;
                    resv.s.F = e[sel].F;
                }
            }
        }
    }

    GD bool step(const PassCtx& P, RayCount& rc, int& err) {
        const DevScene& sc = P.sc;
        const int W = (int)P.b.width, H = (int)P.b.height;
        const uint64_t n = (uint64_t)W * (uint64_t)H;
        if (P.set.spatialReuse && i < P.set.spatialNeighbors && !(kPair && P.set.misWeights != 0u)) {
            reuse_phased(P, rc, err);
            i = P.set.spatialNeighbors;
            return true;
        }
        if (P.set.spatialReuse && i < P.set.spatialNeighbors) {
            i++;
            const float resampleRadius = P.set.spatialRadius;
            float tx = 1.0f / (float)W, ty = 1.0f / (float)H;
            V2 uv = v2(dstIsec.bx, dstIsec.by);
            V2 d = toConcentricDisk(sample2f(rng));
            V2 nb = v2(uv.x + d.x * resampleRadius * tx, uv.y + d.y * resampleRadius * ty);
            const bool pairwise = kPair && P.set.misWeights != 0u;
            if (nb.x < 0.0f || nb.y < 0.0f || nb.x > 1.0f || nb.y > 1.0f) { if (pairwise) pm.skip(); return true; }
            int px = (int)(nb.x * (float)P.cam.w), py = (int)(nb.y * (float)P.cam.h);
            float depthN = 0.0f; V3 normalN = v3s(0.0f), albedoN = v3s(0.0f); int matMeshIdN = 0;
            float4 ndn = texture_bilinear(reinterpret_cast<const float4*>(P.b.depthNormal), W, H, nb);
            uint2 nam = fetch_am(reinterpret_cast<const uint2*>(P.b.albedoMatId), W, H, px, py);
            if (!unpackGBuffer(ndn, nam, depthN, normalN, albedoN, matMeshIdN)) { if (pairwise) pm.skip(); return true; }
            Ray3 nray = pinholeCameraSampleRay(P.cam, v2(nb.x, 1.0f - nb.y));
            V3 posN = nray.ori + nray.dir * (depthN - 1e-4f);
            if (dot3(normalN, dst.norm) < 0.9f || distance3(dst.pos, posN) > 0.4f) { if (pairwise) pm.skip(); return true; }
            uint32_t nidx = (uint32_t)P.cam.w * (uint32_t)py + (uint32_t)px;
            Resv neighborResv = load_resv(P.b.reservoirTemp, nidx, n);
            if (pairwise) {
                if (!resvIsValid(neighborResv)) { pm.skip(); return true; }
                const guide::Lobes* Lp = nullptr;
                const guide::Lobes* Lq = nullptr;
                guide::Lobes L, Ln;
                Surf nbSurf;
                nbSurf.pos = posN; nbSurf.norm = normalN; nbSurf.albedo = albedoN;
                nbSurf.matIndex = (uint32_t)(matMeshIdN >> 16); nbSurf.isLight = false;
                if constexpr (kGuide) {
                    if (primary_lobes(P, idx, load_material(sc, dst.matIndex), L)) Lp = &L;
                    if (primary_lobes(P, nidx, load_material(sc, nbSurf.matIndex), Ln)) Lq = &Ln;
                }
                Shift fw = shiftToDomain(P, dst, dstIsec, ray, neighborResv.s, rc, err, Lp);
                float pBack = 0.0f;
                if (pm.pc > 0.0f) {
                    Isec nbIsec;
                    nbIsec.bx = nb.x; nbIsec.by = nb.y; nbIsec.inst = kSpecialHit; nbIsec.tri = 0u;
                    Shift bw = shiftToDomain(P, nbSurf, nbIsec, nray, pm.canon, rc, err, Lq);
                    if (bw.valid) pBack = bw.dstPHat;
                }
                pm.add(neighborResv, fw, pBack, sample1f(rng));
                return true;
            }
            if (resvIsValid(neighborResv)) {
                const guide::Lobes* Lp = nullptr;
                guide::Lobes L;
                if constexpr (kGuide) {
                    if (primary_lobes(P, idx, load_material(sc, dst.matIndex), L)) Lp = &L;
                }
                reuseAndMerge(P, resv, dst, dstIsec, ray, neighborResv, rng, rc, err, Lp);
            }
            return true;
        }
        if (kPair && P.set.misWeights && P.set.spatialReuse && P.set.spatialNeighbors > 0u) resv = pm.finish(sample1f(rng), (float)P.set.cap);
        shade_final(P, rc, err);
        return false;
    }

    /* After the neighbours: the pixel's reservoir is stored, its sample replayed and shaded
     * (gris_resample_spatial.glsl:88-133) and the result added to the running mean. */
    GD void shade_final(const PassCtx& P, RayCount& rc, int& err) {
        const DevScene& sc = P.sc;
        resvResetIfInvalid(resv);
        store_resv(P.b.reservoirThis, idx, resv);
        V3 radiance = v3s(0.0f);
        if (resvIsValid(resv) && resv.sampleCount > 0.0f) {
            PathSample pathSample = resv.s;
            if (pathSample.rcIsec.inst != kInvalidHit) {
                RcData rcData;
                rcData.rcPrevIsec = isec_zero(); rcData.rcPrevWo = v3s(0.0f); rcData.rcPrevThroughput = v3s(0.0f);
                const guide::Lobes* Lp = nullptr;
                guide::Lobes L;
                if constexpr (kGuide) {
                    if (primary_lobes(P, idx, load_material(sc, dst.matIndex), L)) Lp = &L;
                }
                traceReplay(P, dstIsec, dst, ray, pathSample.flags, pathSample.primaryRng, rcData, rc, err, Lp);
                if (rcData.rcPrevIsec.inst != kInvalidHit) {
                    Surf rcPrevSurf = surf_zero(), rcSurf = surf_zero();
                    if (rcData.rcPrevIsec.inst == kSpecialHit) rcPrevSurf = dst;
                    else loadSurfaceInfo(sc, rcData.rcPrevIsec, rcPrevSurf);
                    loadSurfaceInfo(sc, pathSample.rcIsec, rcSurf);
                    Mat rcMat = load_material(sc, rcSurf.matIndex);
                    Mat rcPrevMat = load_material(sc, rcPrevSurf.matIndex);
                    V3 Li = pathSample.rcLi;
                    uint32_t rcType = rcVertexType(pathSample.flags);
                    V3 wi = normalize3(rcSurf.pos - rcPrevSurf.pos);
                    if (rcType == kRcSurface && length3(pathSample.rcWi) > 0.5f)
                        Li = Li * (evalBSDFCall(rcMat, rcSurf.albedo, rcSurf.norm, -wi, pathSample.rcWi) * satDot(rcSurf.norm, pathSample.rcWi));
                    Li = Li * (evalBSDFCall(rcPrevMat, rcPrevSurf.albedo, rcPrevSurf.norm, rcData.rcPrevWo, wi) * satDot(rcPrevSurf.norm, wi));
                    Li = Li * rcData.rcPrevThroughput;
                    Li = Li / pathSample.rcPrevSamplePdf;
                    if (!isBlack(Li) && !isnan3(Li)) radiance = Li / luminance(Li) * resv.resampleWeight / resv.sampleCount;
                }
            }
        }
        accumulate(P, ix, iy, clampColor(radiance));
    }
};
using SpatialTask = SpatialTaskT<false>;

struct PathTask {
    PathTracer t;
    GD bool begin(const PassCtx& P, uint32_t x, uint32_t y, RayCount&, int&) { return t.begin(P, x, y); }
    GD bool step(const PassCtx& P, RayCount& rc, int& err) {
        if (!t.step(P, rc, err) || ++t.bounce >= (int)P.set.maxDepth) {
            t.end(P);
            return false;
        }
        return true;
    }
};

/* ------------------------------------------------------------------ launch forms */
/* Grid form: one thread per pixel of a 16 x 8 tile. */
template <typename Task>
GD void run_grid(const PassCtx& P, RayCount& rc, int& err) {
    uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= P.b.width || y >= P.b.height) return;
    Task t;
    if (t.begin(P, x, y, rc, err))
        while (t.step(P, rc, err)) {}
}

/* Persistent form: warps take 16 x 16 pixel tiles from a global cursor (one atomic per tile);
 * whenever lanes are idle (path ended, background pixel) they take the tile's next pixels, so a
 * warp's lanes stay busy while they run paths of different lengths. Per-pixel arithmetic is the
 * same as in the grid form; only the assignment of pixels to lanes differs. */
constexpr uint32_t kTileSide = 16;
constexpr uint32_t kTilePixels = kTileSide * kTileSide;

template <typename Task>
GD void run_persistent(const PassCtx& P, unsigned int* cursor, RayCount& rc, int& err) {
    const uint32_t W = P.b.width, H = P.b.height;
    const uint32_t tilesX = (W + kTileSide - 1) / kTileSide;
    const uint32_t numTiles = tilesX * ((H + kTileSide - 1) / kTileSide);
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned lanesBelow = (1u << lane) - 1u;
    uint32_t tile = 0, next = kTilePixels;   /* warp-uniform; next == kTilePixels: no current tile */
    bool active = false, more = true;
    Task t;
    while (true) {
        unsigned idle = __ballot_sync(0xffffffffu, !active);
        while (idle && more) {
            if (next >= kTilePixels) {
                unsigned int v = 0;
                if (lane == 0) v = atomicAdd(cursor, 1u);
                tile = __shfl_sync(0xffffffffu, v, 0);
                next = 0;
                if (tile >= numTiles) { more = false; break; }
            }
            uint32_t n = min((uint32_t)__popc(idle), kTilePixels - next);
            uint32_t rank = (uint32_t)__popc(idle & lanesBelow);
            if (!active && rank < n) {
                uint32_t k = next + rank;
                uint32_t px = (tile % tilesX) * kTileSide + (k % kTileSide);
                uint32_t py = (tile / tilesX) * kTileSide + (k / kTileSide);
                if (px < W && py < H) active = t.begin(P, px, py, rc, err);
            }
            next += n;
            idle = __ballot_sync(0xffffffffu, !active);
        }
        if (__ballot_sync(0xffffffffu, active) == 0u) break;
        if (active) active = t.step(P, rc, err);
    }
}

/* ------------------------------------------------------------------ kernels */
/* Resident blocks per SM requested from the compiler for the grid form: the reuse passes run
 * faster at 8 blocks (64 registers) despite their spills (1080p C2: temporal + spatial 3.65 ms at
 * 8 blocks, 3.79 at 6, 4.04 at 5); the path tracer at its natural occupancy. */
template <int KERNEL> struct GridMinBlocks { static constexpr int value = KERNEL == 1 ? 1 : 8; };

template <typename Task, int KERNEL>
__global__ void __launch_bounds__(128, GridMinBlocks<KERNEL>::value) k_pass_grid(PassCtx P) {
    RayCount rc = ray_count();
    int err = 0;
    run_grid<Task>(P, rc, err);
    flush_counts(P.counters, rc, err, KERNEL, P.countWork);
}

template <typename Task, int KERNEL>
__global__ void __launch_bounds__(128) k_pass_persistent(PassCtx P) {
    RayCount rc = ray_count();
    int err = 0;
    run_persistent<Task>(P, reinterpret_cast<unsigned int*>(P.counters + 24) + KERNEL, rc, err);
    flush_counts(P.counters, rc, err, KERNEL, P.countWork);
}

/* G-buffer (GBuffer.vert:16-28, GBuffer.frag:21-54) by primary rays that ignore instance 0. */
struct GBufCtx {
    DevScene sc;
    CamD cam;
    float lastProjView[16];
    GrisGBufferBindings b;
    unsigned long long* counters;
    int countWork;
};

GD uint32_t packUnorm1(float c) { return (uint32_t)floorf(fminf(fmaxf(c, 0.0f), 1.0f) * 255.0f + 0.5f); }

/* One pixel of the G-buffer; returns 1 (a primary ray was cast). */
GD uint32_t gbuffer_pixel(const GBufCtx& G, uint32_t x, uint32_t y, int& err, GrisWork& work) {
    const DevScene& sc = G.sc;
    uint64_t p = (uint64_t)y * G.b.width + x;
    V2 uv = v2(((float)x + 0.5f) / (float)G.b.width, ((float)y + 0.5f) / (float)G.b.height);
    Ray3 ray = pinholeCameraSampleRay(G.cam, v2(uv.x, 1.0f - uv.y));
    GrisRayHit h;
    bool hit = gris_bvh_trace<false>(sc.nodes, sc.tris, ray.ori.x, ray.ori.y, ray.ori.z, ray.dir.x, ray.dir.y,
                                      ray.dir.z, kMinRayDistance, kMaxRayDistance, true, &h, &err, &work);
    float4* dnOut = reinterpret_cast<float4*>(G.b.depthNormal) + p;
    uint2* amOut = reinterpret_cast<uint2*>(G.b.albedoMatId) + p;
    __half2* mvOut = reinterpret_cast<__half2*>(G.b.motion) + p;
    if (!hit) {
        *dnOut = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        *amOut = make_uint2(0u, 0u);
        *mvOut = __halves2half2(__ushort_as_half(0), __ushort_as_half(0));
        return 1u;
    }
    uint64_t k = (uint64_t)h.inst - 1u;
    float T[16], TI[16];
    uint32_t indexOffset = 0u;
    if (k < sc.nInstances) {
        load_mat4(sc.instances[k].transform, T);
        load_mat4(sc.instances[k].transformInvT, TI);
        indexOffset = ldu(&sc.instances[k].indexOffset);
    } else {
        for (int i = 0; i < 16; i++) { T[i] = 0.0f; TI[i] = 0.0f; }
    }
    V3 b = v3(1.0f - h.u - h.v, h.u, h.v);
    V3 Pj[3], Nj[3];
    for (int j = 0; j < 3; j++) {
        V3 vp, vn;
        load_vertex(sc, load_index(sc, (uint64_t)(indexOffset + h.tri * 3u + (uint32_t)j)), vp, vn);
        Pj[j] = m4mul_point(T, vp, 1.0f);
        V3 c0 = v3(TI[0], TI[1], TI[2]), c1 = v3(TI[4], TI[5], TI[6]), c2 = v3(TI[8], TI[9], TI[10]);
        Nj[j] = normalize3((c0 * vn.x + c1 * vn.y) + c2 * vn.z);
    }
    V3 pos = (Pj[0] * b.x + Pj[1] * b.y) + Pj[2] * b.z;
    V3 nor = normalize3((Nj[0] * b.x + Nj[1] * b.y) + Nj[2] * b.z);
    uint64_t mi = (uint64_t)(indexOffset / 3u + h.tri);
    uint32_t matIndex = (uint32_t)(mi < sc.nMatIndices ? (int32_t)ldu(reinterpret_cast<const uint32_t*>(sc.matIndices + mi)) : 0);
    V3 albedo = load_material(sc, matIndex).baseColor;
    const float* M = G.lastProjView;
    float lx = ((M[0] * pos.x + M[4] * pos.y) + M[8] * pos.z) + M[12] * 1.0f;
    float ly = ((M[1] * pos.x + M[5] * pos.y) + M[9] * pos.z) + M[13] * 1.0f;
    float lw = ((M[3] * pos.x + M[7] * pos.y) + M[11] * pos.z) + M[15] * 1.0f;
    lx = lx / lw; ly = ly / lw;
    lx = lx * 0.5f + 0.5f; ly = ly * 0.5f + 0.5f;
    float tx = ((float)x + 0.5f) / (float)G.b.width, ty = ((float)y + 0.5f) / (float)G.b.height;
    float mx = lx - tx, my = ly - ty;
    *dnOut = make_float4(length3(G.cam.pos - pos), nor.x, nor.y, nor.z);
    uint32_t packed = packUnorm1(albedo.x) | (packUnorm1(albedo.y) << 8) | (packUnorm1(albedo.z) << 16) | (packUnorm1(1.0f) << 24);
    *amOut = make_uint2(packed, (matIndex << 16) | (uint32_t)k);
    *mvOut = __halves2half2(__float2half_rn(mx), __float2half_rn(my));
    return 1u;
}

GD void flush_gbuffer_counts(unsigned long long* counters, uint32_t primary, int err, const GrisWork& work, int countWork) {
    unsigned int c = __reduce_add_sync(0xffffffffu, primary);
    unsigned int e = __reduce_or_sync(0xffffffffu, (unsigned)err);
    unsigned long long nodes = 0, tris = 0;
    if (countWork) {
        nodes = __reduce_add_sync(0xffffffffu, work.nodes);
        tris = __reduce_add_sync(0xffffffffu, work.tris);
    }
    if (((threadIdx.y * blockDim.x + threadIdx.x) & 31u) == 0u) {
        if (c) atomicAdd(counters + GRIS_COUNTER_PRIMARY, (unsigned long long)c);
        if (e) atomicOr(counters + GRIS_COUNTER_ERROR, (unsigned long long)e);
        if (countWork) {
            atomicAdd(counters + 8, nodes);
            atomicAdd(counters + 9, tris);
            atomicAdd(counters + 16, (unsigned long long)c);
        }
    }
}

/* resident blocks of 128 threads per SM asked of the compiler for the batch G-buffer kernel
 * (0: no request). At C2: 7 blocks (72 registers) 0.546 ms per frame, none (80 registers, 6
 * blocks) 0.583 ms, 8 blocks (64 registers, spills) 0.591 ms. The single-view kernel k_gbuffer
 * (the DI frame's G-buffer) measured slower with 7 (0.551 against 0.530 ms) and keeps none. */
#ifndef GRIS_GBUFFER_MIN_BLOCKS
#define GRIS_GBUFFER_MIN_BLOCKS 7
#endif

__global__ void __launch_bounds__(128) k_gbuffer(GBufCtx G) {
    uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    int err = 0;
    uint32_t primary = 0;
    GrisWork work; work.nodes = 0u; work.tris = 0u;
    if (x < G.b.width && y < G.b.height) primary = gbuffer_pixel(G, x, y, err, work);
    flush_gbuffer_counts(G.counters, primary, err, work, G.countWork);
}

/* One whole walk with the resident kernels' stack, here with a single shared-memory entry, so that
 * walks of depth 4 and more already use all three of its tiers (registers, shared memory, the
 * local-memory overflow). */
template <bool ANY>
GD bool debug_walk_short_stack(const uint32_t* nodes, const float* tris, const float* r, uint32_t* slab, GrisRayHit* h,
                               int* err) {
    GrisTraversal<ANY> w;
    GrisShortStack<1> stack;
    stack.bind(slab, threadIdx.x, blockDim.x);
    w.init(r[0], r[1], r[2], r[4], r[5], r[6], r[3], r[7]);
    while (w.step(nodes, tris, false, err, stack)) {}
    w.result(h, nullptr);
    return w.found;
}

/* Builder check: one ray per thread, walked with the short stack of the resident traversal
 * kernels (k_wave_trace_refill, k_reuse_visibility) in a small configuration. */
__global__ void __launch_bounds__(128) k_debug_trace(const uint32_t* nodes, const float* tris, const float* rays, uint64_t n,
                                                     int anyHit, float* hitTUV, uint32_t* hitInst, uint32_t* hitTri,
                                                     unsigned long long* counters) {
    __shared__ uint32_t slab[2 * 1 * 128];
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = rays + i * 8;
    GrisRayHit h;
    int err = 0;
    bool hit = anyHit ? debug_walk_short_stack<true>(nodes, tris, r, slab, &h, &err)
                      : debug_walk_short_stack<false>(nodes, tris, r, slab, &h, &err);
    if (hit) { hitTUV[i * 4] = h.t; hitTUV[i * 4 + 1] = h.u; hitTUV[i * 4 + 2] = h.v; hitTUV[i * 4 + 3] = 0.0f; hitInst[i] = h.inst; hitTri[i] = h.tri; }
    else { hitTUV[i * 4] = -1.0f; hitTUV[i * 4 + 1] = 0.0f; hitTUV[i * 4 + 2] = 0.0f; hitTUV[i * 4 + 3] = 0.0f; hitInst[i] = GRIS_INVALID_HIT; hitTri[i] = GRIS_INVALID_HIT; }
    if (err) atomicOr(counters + GRIS_COUNTER_ERROR, 1ull);
}

/* ------------------------------------------------------------------ launchers */
cudaError_t launch_gbuffer(const DeviceSceneView& scene, const GrisGBufferBindings& b, const GrisCamera& cam,
                           unsigned long long* counters, int countWork, KernelTimer* timer, cudaStream_t stream) {
    GBufCtx G;
    G.countWork = countWork;
    G.sc = to_dev(scene);
    G.cam = make_cam(cam);
    for (int i = 0; i < 16; i++) G.lastProjView[i] = cam.lastProjView[i];
    G.b = b;
    G.counters = counters;
    dim3 block(16, 8), grid((b.width + 15) / 16, (b.height + 7) / 8);
    if (timer) timer->mark(0, true, stream);
    k_gbuffer<<<grid, block, 0, stream>>>(G);
    if (timer) timer->mark(0, false, stream);
    return cudaGetLastError();
}

cudaError_t launch_gris(const DeviceSceneView& scene, const GrisPassBindings& b, const GrisCamera& cam,
                        const GrisCamera& prevCam, const GrisSettings& set, int passes, unsigned long long* counters,
                        int countWork, KernelTimer* timer, cudaStream_t stream, int launchMode) {
    PassCtx P;
    P.countWork = countWork;
    P.sc = to_dev(scene);
    P.cam = make_cam(cam);
    P.prev = make_cam(prevCam);
    P.set = set;
    P.b = b;
    P.counters = counters;
    dim3 block(16, 8), grid((b.width + 15) / 16, (b.height + 7) / 8);
    bool persistent = launchMode == GRIS_LAUNCH_PERSISTENT;
    int blocksPT = 0, blocksT = 0, blocksS = 0;
    if (persistent) {
        /* SM count and resident blocks per SM of each persistent kernel, per device */
        const int smCount = current_sm_count();
        int occ[3];
        occ[0] = once_per_device(kDeviceKeyOccPath, []() {
            int o = 0;
            return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_pass_persistent<PathTask, 1>, 128, 0) == cudaSuccess ? o : -1;
        });
        occ[1] = once_per_device(kDeviceKeyOccTemporal, []() {
            int o = 0;
            return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_pass_persistent<TemporalTask, 2>, 128, 0) == cudaSuccess ? o : -1;
        });
        occ[2] = once_per_device(kDeviceKeyOccSpatial, []() {
            int o = 0;
            return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_pass_persistent<SpatialTask, 3>, 128, 0) == cudaSuccess ? o : -1;
        });
        blocksPT = smCount * (occ[0] > 0 ? occ[0] : 1);
        blocksT = smCount * (occ[1] > 0 ? occ[1] : 1);
        blocksS = smCount * (occ[2] > 0 ? occ[2] : 1);
        cudaError_t e = cudaMemsetAsync(counters + 24, 0, 2 * sizeof(unsigned long long), stream);
        if (e != cudaSuccess) return e;
    }
    if (passes & 1) {
        if (timer) timer->mark(1, true, stream);
        if (persistent) k_pass_persistent<PathTask, 1><<<blocksPT, 128, 0, stream>>>(P);
        else k_pass_grid<PathTask, 1><<<grid, block, 0, stream>>>(P);
        if (timer) timer->mark(1, false, stream);
    }
    if (passes & 2) {
        if (timer) timer->mark(2, true, stream);
        if (set.misWeights) k_pass_grid<TemporalTaskT<false, true>, 2><<<grid, block, 0, stream>>>(P);
        else if (persistent) k_pass_persistent<TemporalTask, 2><<<blocksT, 128, 0, stream>>>(P);
        else k_pass_grid<TemporalTask, 2><<<grid, block, 0, stream>>>(P);
        if (timer) timer->mark(2, false, stream);
    }
    if (passes & 4) {
        if (timer) timer->mark(3, true, stream);
        if (set.misWeights) k_pass_grid<SpatialTaskT<false, true>, 3><<<grid, block, 0, stream>>>(P);
        else if (persistent) k_pass_persistent<SpatialTask, 3><<<blocksS, 128, 0, stream>>>(P);
        else k_pass_grid<SpatialTask, 3><<<grid, block, 0, stream>>>(P);
        if (timer) timer->mark(3, false, stream);
    }
    return cudaGetLastError();
}

/* ------------------------------------------------------------------ converged image */
/* Seed of sample s of a pixel's sequence: a hash of the frame seed and the sample index, so
 * the samples are streams of makeSeed like the frames of the renderer. */
GD uint32_t sample_seed(uint32_t frameSeed, uint32_t s) { return hash2(frameSeed ^ hash2(s * 0x9e3779b9u + 0x7f4a7c15u)); }

/* `sppN` independent paths per pixel (samples [spp0, spp0 + sppN)) of the path tracer from the
 * pixel's G-buffer surface; each path's estimate (estimator 0: the sum of its reservoir
 * candidates; 1: every NEE and light-hit contribution) is clamped as clampColor and added in
 * FP64 to sum (and its square to sumSq). One thread per pixel: no two threads touch one pixel. */
__global__ void __launch_bounds__(128) k_converged(PassCtx P, double* sum, double* sumSq, uint32_t spp0, uint32_t sppN,
                                                   int estimator) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= P.b.width || y >= P.b.height) return;
    RayCount rc = ray_count();
    int err = 0;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, q0 = 0.0, q1 = 0.0, q2 = 0.0;
    for (uint32_t s = spp0; s < spp0 + sppN; s++) {
        PathTracerT<true> t;
        if (!t.begin(P, x, y, sample_seed(P.cam.seed, s))) break;   /* background: the same for every sample */
        while (t.step(P, rc, err) && ++t.bounce < (int)P.set.maxDepth) {}
        t.finish();
        V3 c = clampColor(estimator == 0 ? t.accCand : t.accAll);
        a0 += (double)c.x; a1 += (double)c.y; a2 += (double)c.z;
        q0 += (double)c.x * (double)c.x; q1 += (double)c.y * (double)c.y; q2 += (double)c.z * (double)c.z;
    }
    const size_t i = ((size_t)y * P.b.width + x) * 3;
    sum[i] += a0; sum[i + 1] += a1; sum[i + 2] += a2;
    if (sumSq) { sumSq[i] += q0; sumSq[i + 1] += q1; sumSq[i + 2] += q2; }
    if (err) atomicOr(P.counters + GRIS_COUNTER_ERROR, (unsigned long long)err);
}

cudaError_t launch_converged(const DeviceSceneView& scene, const GrisConvergedBindings& b, const GrisCamera& cam,
                             const GrisSettings& set, uint32_t sppBegin, uint32_t sppCount, int estimator,
                             unsigned long long* counters, cudaStream_t stream) {
    PassCtx P;
    P.countWork = 0;
    P.sc = to_dev(scene);
    P.cam = make_cam(cam);
    P.prev = P.cam;
    P.set = set;
    memset(&P.b, 0, sizeof(P.b));
    P.b.width = b.width; P.b.height = b.height;
    P.b.depthNormal = b.depthNormal;
    P.b.albedoMatId = b.albedoMatId;
    P.counters = counters;
    dim3 block(16, 8), grid((b.width + 15) / 16, (b.height + 7) / 8);
    /* about 2^23 paths per launch keeps every launch short */
    const uint64_t px = (uint64_t)b.width * b.height;
    uint32_t chunk = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(sppCount, (1ull << 23) / std::max<uint64_t>(1, px)));
    for (uint32_t s = 0; s < sppCount; s += chunk) {
        uint32_t n = std::min(chunk, sppCount - s);
        k_converged<<<grid, block, 0, stream>>>(P, b.sum, b.sumSq, sppBegin + s, n, estimator);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

/* relMSE = mean over pixels and channels of (img - ref)^2 / (ref^2 + eps), MSE = mean of
 * (img - ref)^2, ref = refSum * refScale; FP64 sums in a fixed order (grid-stride per thread,
 * then a fixed shuffle and block tree, then one block over the partials): deterministic. */
constexpr int kReduceBlocks = 304, kReduceThreads = 256;
__global__ void __launch_bounds__(kReduceThreads) k_relmse_partial(const float4* img, const double* refSum, double refScale,
                                                                   uint64_t n, double eps, double* partial) {
    double rel = 0.0, sq = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        float4 v = img[i];
        const double c[3] = {(double)v.x, (double)v.y, (double)v.z};
        for (int k = 0; k < 3; k++) {
            double r = refSum[i * 3 + k] * refScale, d = c[k] - r;
            rel += d * d / (r * r + eps);
            sq += d * d;
        }
    }
    __shared__ double sr[kReduceThreads / 32], ss[kReduceThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        rel += __shfl_down_sync(0xffffffffu, rel, o);
        sq += __shfl_down_sync(0xffffffffu, sq, o);
    }
    if ((threadIdx.x & 31) == 0) { sr[threadIdx.x >> 5] = rel; ss[threadIdx.x >> 5] = sq; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < kReduceThreads / 32; w++) { a += sr[w]; b += ss[w]; }
        partial[2 * blockIdx.x] = a;
        partial[2 * blockIdx.x + 1] = b;
    }
}
__global__ void k_relmse_final(const double* partial, int blocks, uint64_t n, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double a = 0.0, b = 0.0;
    for (int i = 0; i < blocks; i++) { a += partial[2 * i]; b += partial[2 * i + 1]; }
    out[0] = n ? a / (3.0 * (double)n) : 0.0;
    out[1] = n ? b / (3.0 * (double)n) : 0.0;
}

cudaError_t launch_relmse(const float* image, const double* refSum, double refScale, uint64_t pixels, double eps,
                          double* scratch, cudaStream_t stream) {
    k_relmse_partial<<<kReduceBlocks, kReduceThreads, 0, stream>>>(reinterpret_cast<const float4*>(image), refSum,
                                                                    refScale, pixels, eps, scratch + 2);
    k_relmse_final<<<1, 32, 0, stream>>>(scratch + 2, kReduceBlocks, pixels, scratch);
    return cudaGetLastError();
}
size_t relmse_scratch_doubles() { return 2 + 2 * (size_t)kReduceBlocks; }

cudaError_t launch_debug_trace(const uint32_t* nodes, const float* tris, const float* rays, uint64_t n, int anyHit,
                               float* hitTUV, uint32_t* hitInst, uint32_t* hitTri, unsigned long long* counters,
                               cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    k_debug_trace<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(nodes, tris, rays, n, anyHit, hitTUV, hitInst, hitTri, counters);
    return cudaGetLastError();
}

}  // namespace grisrt

/* ==================================================================================================
 * Batches: many views (each with its own scene, size, cameras and settings) in one launch per
 * pass, and the wavefront form of the path tracer with per-bounce compacted queues.
 * ================================================================================================== */
namespace grisrt {

/* One view of a batch, as the kernels read it from the device view table. */
struct ViewEntry {
    PassCtx P;
    GBufCtx G;
    uint32_t tileBase;   /* first 16 x 8 tile of the view in the batch's tile space */
    uint32_t tilesX;
    uint32_t pixelBase;  /* first path id of the view */
    uint32_t pad;
    float boxMin[3], boxInv[3];   /* the scene box (guide inputs: position in [0,1]^3) */
};

size_t view_entry_bytes() { return sizeof(ViewEntry); }

GD int find_view_by_tile(const ViewEntry* V, int n, uint32_t tile) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (V[mid].tileBase <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}
GD int find_view_by_pixel(const ViewEntry* V, int n, uint32_t id) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (V[mid].pixelBase <= id) lo = mid; else hi = mid - 1;
    }
    return lo;
}

/* G-buffer, temporal and spatial passes over every view: one 16 x 8 block per tile. */
__global__ void __launch_bounds__(128, GRIS_GBUFFER_MIN_BLOCKS) k_batch_gbuffer(const ViewEntry* __restrict__ V, int n) {
    int v = find_view_by_tile(V, n, blockIdx.x);
    const GBufCtx& G = V[v].G;
    uint32_t t = blockIdx.x - V[v].tileBase;
    uint32_t x = (t % V[v].tilesX) * 16u + threadIdx.x, y = (t / V[v].tilesX) * 8u + threadIdx.y;
    int err = 0;
    uint32_t primary = 0;
    GrisWork work; work.nodes = 0u; work.tris = 0u;
    if (x < G.b.width && y < G.b.height) primary = gbuffer_pixel(G, x, y, err, work);
    flush_gbuffer_counts(G.counters, primary, err, work, G.countWork);
}

template <typename Task, int KERNEL>
__global__ void __launch_bounds__(128, GridMinBlocks<KERNEL>::value) k_batch_pass(const ViewEntry* __restrict__ V, int n) {
    int v = find_view_by_tile(V, n, blockIdx.x);
    const PassCtx& P = V[v].P;
    uint32_t t = blockIdx.x - V[v].tileBase;
    uint32_t x = (t % V[v].tilesX) * 16u + threadIdx.x, y = (t / V[v].tilesX) * 8u + threadIdx.y;
    RayCount rc = ray_count();
    int err = 0;
    if (x < P.b.width && y < P.b.height) {
        Task task;
        if (task.begin(P, x, y, rc, err))
            while (task.step(P, rc, err)) {}
    }
    flush_counts(P.counters, rc, err, KERNEL, P.countWork);
}

/* ------------------------------------------------------------------ wavefront path tracer */
/* Path state between kernels, per path id: the loop-carried members of PathTracer (17 x 16 B)
 * and the part of a bounce carried from shade() to post() across the shadow query (6 x 16 B). */
struct WaveRec { uint4 w[16]; };
struct NeeRec { uint4 w[6]; };
static_assert(sizeof(WaveRec) == kWaveStateBytes && sizeof(NeeRec) == kWaveNeeBytes, "wavefront record sizes");

GD uint4 u4f(float a, float b, float c, float d) {
    return make_uint4(__float_as_uint(a), __float_as_uint(b), __float_as_uint(c), __float_as_uint(d));
}
/* The two path samples of a wavefront record in 9 words: their pad fields, always 0 in the path
 * tracer, are left out (18 32-bit fields each). */
GD void ps_put18(const PathSample& p, uint32_t* u) {
    u[0] = __float_as_uint(p.rcIsec.bx); u[1] = __float_as_uint(p.rcIsec.by); u[2] = p.rcIsec.inst; u[3] = p.rcIsec.tri;
    u[4] = __float_as_uint(p.rcLi.x); u[5] = __float_as_uint(p.rcLi.y); u[6] = __float_as_uint(p.rcLi.z); u[7] = p.rcRng;
    u[8] = __float_as_uint(p.rcWi.x); u[9] = __float_as_uint(p.rcWi.y); u[10] = __float_as_uint(p.rcWi.z); u[11] = p.flags;
    u[12] = __float_as_uint(p.rcPrevSamplePdf); u[13] = __float_as_uint(p.rcJacobian);
    u[14] = __float_as_uint(p.F.x); u[15] = __float_as_uint(p.F.y); u[16] = __float_as_uint(p.F.z); u[17] = p.primaryRng;
}
GD void ps_get18(PathSample& p, const uint32_t* u) {
    p.rcIsec.bx = __uint_as_float(u[0]); p.rcIsec.by = __uint_as_float(u[1]); p.rcIsec.inst = u[2]; p.rcIsec.tri = u[3];
    p.rcLi = v3(__uint_as_float(u[4]), __uint_as_float(u[5]), __uint_as_float(u[6])); p.rcRng = u[7];
    p.rcWi = v3(__uint_as_float(u[8]), __uint_as_float(u[9]), __uint_as_float(u[10])); p.flags = u[11];
    p.pad0 = 0.0f; p.pad1 = 0.0f;
    p.rcPrevSamplePdf = __uint_as_float(u[12]); p.rcJacobian = __uint_as_float(u[13]);
    p.F = v3(__uint_as_float(u[14]), __uint_as_float(u[15]), __uint_as_float(u[16])); p.primaryRng = u[17];
}

/* A path's wavefront record (256 bytes, 8 whole sectors): [0..5] the tracer's scalars and ray,
 * [6..14] the path sample and the stream's sample, [15] the accumulating / guided tracers' extra
 * state (zero for the plain tracer, which does not read it). */
template <class T>
GD void save_wave(WaveRec* __restrict__ dst, const T& t) {
    uint4 w[16];
    w[0] = make_uint4(t.rng, t.sampleState | (t.lastSampleState << 8) | ((t.isLastVertexConnectible ? 1u : 0u) << 16),
                      t.surf.matIndex, t.s.type);
    w[1] = u4f(t.throughput.x, t.throughput.y, t.throughput.z, t.s.pdf);
    w[2] = u4f(t.rcThroughput.x, t.rcThroughput.y, t.rcThroughput.z, t.stream.weight);
    w[3] = u4f(t.lastPos.x, t.lastPos.y, t.lastPos.z, t.stream.sumWeight);
    w[4] = make_uint4(__float_as_uint(t.ray.ori.x), __float_as_uint(t.ray.ori.y), __float_as_uint(t.ray.ori.z), t.stream.sampleCount);
    float pdfHit = 0.0f;
    if constexpr (T::kGuided) pdfHit = t.pdfHit;
    w[5] = u4f(t.ray.dir.x, t.ray.dir.y, t.ray.dir.z, pdfHit);
    uint32_t u[36];
    ps_put18(t.pathSample, u);
    ps_put18(t.stream.ps, u + 18);
#pragma unroll
    for (int i = 0; i < 9; i++) w[6 + i] = make_uint4(u[4 * i], u[4 * i + 1], u[4 * i + 2], u[4 * i + 3]);
    w[15] = make_uint4(0u, 0u, 0u, 0u);
    if constexpr (T::kAccumulate) w[15] = make_uint4(__float_as_uint(t.accAll.x), __float_as_uint(t.accAll.y),
                                                     __float_as_uint(t.accAll.z), 0u);
    if constexpr (T::kGuided) w[15].w = t.rec;
    /* all 16 words, so that every 32-byte sector of the record is written whole (a partly written
     * sector costs the L2 a read-merge when it goes to DRAM) */
#pragma unroll
    for (int i = 0; i < 16; i++) dst->w[i] = w[i];
}
template <class T>
GD void load_wave(const WaveRec* __restrict__ src, T& t) {
    uint4 w[16];
#pragma unroll
    for (int i = 0; i < 15; i++) w[i] = src->w[i];
    if constexpr (T::kAccumulate) {
        w[15] = src->w[15];
        t.accAll = v3(__uint_as_float(w[15].x), __uint_as_float(w[15].y), __uint_as_float(w[15].z));
        t.accCand = v3s(0.0f);
    }
    if constexpr (T::kGuided) { t.rec = w[15].w; t.pdfHit = __uint_as_float(w[5].w); t.thrSampled = v3s(0.0f); }
    t.rng = w[0].x;
    t.sampleState = w[0].y & 0xffu; t.lastSampleState = (w[0].y >> 8) & 0xffu; t.isLastVertexConnectible = (w[0].y >> 16) & 1u;
    t.surf.matIndex = w[0].z; t.s.type = w[0].w;
    t.throughput = v3(__uint_as_float(w[1].x), __uint_as_float(w[1].y), __uint_as_float(w[1].z)); t.s.pdf = __uint_as_float(w[1].w);
    t.rcThroughput = v3(__uint_as_float(w[2].x), __uint_as_float(w[2].y), __uint_as_float(w[2].z)); t.stream.weight = __uint_as_float(w[2].w);
    t.lastPos = v3(__uint_as_float(w[3].x), __uint_as_float(w[3].y), __uint_as_float(w[3].z)); t.stream.sumWeight = __uint_as_float(w[3].w);
    t.ray.ori = v3(__uint_as_float(w[4].x), __uint_as_float(w[4].y), __uint_as_float(w[4].z)); t.stream.sampleCount = w[4].w;
    t.ray.dir = v3(__uint_as_float(w[5].x), __uint_as_float(w[5].y), __uint_as_float(w[5].z));
    uint32_t u[36];
#pragma unroll
    for (int i = 0; i < 9; i++) { u[4 * i] = w[6 + i].x; u[4 * i + 1] = w[6 + i].y; u[4 * i + 2] = w[6 + i].z; u[4 * i + 3] = w[6 + i].w; }
    ps_get18(t.pathSample, u);
    ps_get18(t.stream.ps, u + 18);
    t.wo = -t.ray.dir;   /* wo = -ray.dir holds at every bounce boundary */
    t.s.wi = v3s(0.0f); t.s.bsdf = v3s(0.0f);
    t.surf.isLight = false;
}
/* extra: bit 2 = the path's next ray is queued already (set by shade(), checked by post()) */
template <class T>
GD void save_nee(NeeRec* __restrict__ dst, const T& t, uint32_t extra = 0u) {
    dst->w[0] = make_uint4(__float_as_uint(t.surf.pos.x), __float_as_uint(t.surf.pos.y), __float_as_uint(t.surf.pos.z),
                           __float_as_uint(t.resvRandSample));
    dst->w[1] = make_uint4(__float_as_uint(t.surf.norm.x), __float_as_uint(t.surf.norm.y), __float_as_uint(t.surf.norm.z),
                           (t.isThisVertexConnectible ? 1u : 0u) | (t.nee ? 2u : 0u) | extra);
    dst->w[2] = make_uint4(__float_as_uint(t.surf.albedo.x), __float_as_uint(t.surf.albedo.y), __float_as_uint(t.surf.albedo.z), t.lightId);
    dst->w[3] = u4f(t.lightRadiance.x, t.lightRadiance.y, t.lightRadiance.z, t.lightDist);
    dst->w[4] = u4f(t.lightDir.x, t.lightDir.y, t.lightDir.z, t.lightPdf);
    dst->w[5] = u4f(t.lightBary.x, t.lightBary.y, t.lightJacobian, 0.0f);
}
template <class T>
GD void load_nee(const NeeRec* __restrict__ src, T& t) {
    uint4 w[6];
    for (int i = 0; i < 6; i++) w[i] = src->w[i];
    t.surf.pos = v3(__uint_as_float(w[0].x), __uint_as_float(w[0].y), __uint_as_float(w[0].z)); t.resvRandSample = __uint_as_float(w[0].w);
    t.surf.norm = v3(__uint_as_float(w[1].x), __uint_as_float(w[1].y), __uint_as_float(w[1].z));
    t.isThisVertexConnectible = (w[1].w & 1u) != 0u;
    t.nee = (w[1].w & 2u) != 0u;
    t.surf.albedo = v3(__uint_as_float(w[2].x), __uint_as_float(w[2].y), __uint_as_float(w[2].z)); t.lightId = w[2].w;
    t.lightRadiance = v3(__uint_as_float(w[3].x), __uint_as_float(w[3].y), __uint_as_float(w[3].z)); t.lightDist = __uint_as_float(w[3].w);
    t.lightDir = v3(__uint_as_float(w[4].x), __uint_as_float(w[4].y), __uint_as_float(w[4].z)); t.lightPdf = __uint_as_float(w[4].w);
    t.lightBary = v2(__uint_as_float(w[5].x), __uint_as_float(w[5].y)); t.lightJacobian = __uint_as_float(w[5].z);
}

struct WaveCtx {
    const ViewEntry* V;
    int nViews;
    uint32_t totalPixels;
    WaveRec* state;
    NeeRec* nee;
    Isec* hit;
    unsigned char* blocked;
    uint32_t* queue[2];
    uint32_t* shadowQueue;
    uint4* ray;         /* per path: the next closest-hit ray, origin.xyz | dir.xyz (2 x uint4) */
    uint32_t* counts;   /* [level] paths, [256 + level] shadow queries, [512 + level] post() calls and
                           [768 + level] guided vertices of the level (guided batches) */
    unsigned long long* counters;
    int countWork;
    /* guided batches */
    uint32_t* postQueue;
    float* gFeat;        /* per guided vertex (queue order): position in [0,1]^3, normal, wo */
    float* gOut;         /* per guided vertex: the network's 40 raw outputs */
    float* gRec;         /* per path: its training record (features 9, direction 3, throughput 3, sum 3) */
    float* gPrimFeat;    /* per path: the guide's inputs at its primary vertex */
    uint32_t* gFrame;    /* [0] guided vertices this frame, [1] record probability (float bits) */
    guide::GuideDevice guide;
    uint32_t frameSeed;
};

/* Appends `id` (for lanes with `push`) to a queue with one atomic per warp. */
GD void warp_push(uint32_t* queue, uint32_t* count, bool push, uint32_t id) {
    unsigned m = __ballot_sync(0xffffffffu, push);
    if (!m) return;
    uint32_t lane = threadIdx.x & 31u;
    uint32_t leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (push) queue[base + __popc(m & ((1u << lane) - 1u))] = id;
}

GD void path_coords(const WaveCtx& C, uint32_t id, int& v, uint32_t& x, uint32_t& y) {
    v = find_view_by_pixel(C.V, C.nViews, id);
    uint32_t px = id - C.V[v].pixelBase;
    x = px % C.V[v].P.b.width;
    y = px / C.V[v].P.b.width;
}

/* At the end of a guided path holding a training record: the record's sample weight
 * w = luminance((radiance gathered after the vertex) / (throughput at the vertex)) — the
 * one-sample estimate of f cos L_in / pdf for the sampled direction — and, when positive, the
 * record joins the frame's training batch. */
template <class T>
GD void guide_finish_record(const WaveCtx& C, const T& t, uint32_t id) {
    if constexpr (T::kGuided) {
        if (!t.rec) return;
        const float* r = C.gRec + (size_t)id * 18;
        const float acc[3] = {t.accAll.x, t.accAll.y, t.accAll.z};
        float li[3];
        for (int c = 0; c < 3; c++) {
            float thr = r[12 + c];
            li[c] = thr > 1e-20f ? (acc[c] - r[15 + c]) / thr : 0.0f;
        }
        float w = luminance(v3(li[0], li[1], li[2]));
        if (!(w > 0.0f)) return;
        w = fminf(w, 1e4f);
        uint32_t slot = atomicAdd(C.guide.tCount, 1u);
        if (slot >= C.guide.cap) return;
        for (int i = 0; i < 9; i++) C.guide.tFeat[(size_t)slot * 9 + i] = r[i];
        for (int i = 0; i < 3; i++) C.guide.tDir[(size_t)slot * 3 + i] = r[9 + i];
        C.guide.tWeight[slot] = w;
    }
}

GD void store_ray(const WaveCtx& C, uint32_t id, V3 o, V3 d) {
    C.ray[2 * (uint64_t)id] = u4f(o.x, o.y, o.z, 0.0f);
    C.ray[2 * (uint64_t)id + 1] = u4f(d.x, d.y, d.z, 0.0f);
}

/* After a bounce's post(): the next level (the state saved; with `queue`, the path's next ray
 * stored for the closest-hit walk and the path pushed by the caller) or the end of the path.
 * Returns whether the path continues. */
template <class T>
GD bool wave_continue(const WaveCtx& C, const PassCtx& P, T& t, uint32_t id, bool cont, int level, bool& push,
                      bool queue = true) {
    push = false;
    if (cont) {
        t.bounce++;
        if (t.bounce < (int)P.set.maxDepth) {
            save_wave(C.state + id, t);
            if (queue) {
                store_ray(C, id, t.ray.ori, t.ray.dir);
                push = true;
            }
            return true;
        }
    }
    t.end(P);
    guide_finish_record(C, t, id);
    return false;
}

/* level 0: begin() + the primary vertex for every pixel of every view */
__global__ void __launch_bounds__(128) k_wave_begin(WaveCtx C) {
    uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    bool push = false;
    RayCount rc = ray_count();
    if (id < C.totalPixels) {
        int v; uint32_t x, y;
        path_coords(C, id, v, x, y);
        const PassCtx& P = C.V[v].P;
        PathTracer t;
        if (t.begin(P, x, y)) {
            int r = t.shade(P, isec_zero());   /* no NEE at bounce 0 */
            wave_continue(C, P, t, id, r == PathTracer::kNext, 0, push);
        }
    }
    warp_push(C.queue[1], C.counts + 1, push, id);
}

/* closest hits of the level's paths */
__global__ void __launch_bounds__(128) k_wave_extend(WaveCtx C, int level) {
    const uint32_t n = C.counts[level];
    const uint32_t* q = C.queue[level & 1];
    RayCount rc = ray_count();
    int err = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i - threadIdx.x < n; i += gridDim.x * blockDim.x) {
        if (i < n) {
            uint32_t id = q[i];
            const uint4 a = C.ray[2 * (uint64_t)id], b = C.ray[2 * (uint64_t)id + 1];
            V3 o = v3(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z));
            V3 d = v3(__uint_as_float(b.x), __uint_as_float(b.y), __uint_as_float(b.z));
            int v = find_view_by_pixel(C.V, C.nViews, id);
            C.hit[id] = traceClosestHit(C.V[v].P.sc, o, d, kMinRayDistance, kMaxRayDistance, rc, err);
        }
    }
    flush_counts(C.counters, rc, err, 1, C.countWork, 0);
}

/* ---------------------------------------------------------------- sparse levels: one ray per warp */
/* A level with fewer rays than kCoopMaxRays lasts as long as its longest walk (a lane per ray, one
 * dependent node or triangle fetch after another). There the warp walks one ray at a time:
 * each round takes up to 4 nodes off the warp's stack, 8 lanes per node test one child box each
 * (the walker's own box test), the hit inner children are pushed, and the hit leaves' triangles
 * are tested 32 at a time (the walker's triangle test, tmax = the best t so far) and reduced over
 * the warp. The closest hit is the lexicographic minimum of (t, instanceIdx, triangleIdx) over
 * the accepted triangles, and an any-hit query asks only whether one exists, so the order of the
 * visits does not change a result: k_wave_trace_refill's results, bit for bit. */
/* entries of a resident walk's stack held in shared memory (after two in registers) */
#ifndef GRIS_WALK_SHARED_ENTRIES
#define GRIS_WALK_SHARED_ENTRIES 8
#endif
constexpr int kWalkSharedEntries = GRIS_WALK_SHARED_ENTRIES;
/* resident blocks of 128 threads per SM asked of the compiler for the resident traversal kernels
 * (0: no request) */
#ifndef GRIS_WALK_MIN_BLOCKS
#define GRIS_WALK_MIN_BLOCKS 7
#endif
constexpr int kWalkMinBlocks = GRIS_WALK_MIN_BLOCKS;
/* leaf triangles a resident walk tests per step (0: all of a node's at once), for closest-hit and
 * for any-hit walks. Measured at C2 (frames/s): any-hit 2 per step 147.3, 1 per step 140.7, all
 * 142.3; the closest-hit walks lose a little with fewer per step. */
#ifndef GRIS_WALK_TRIS_CLOSEST
#define GRIS_WALK_TRIS_CLOSEST 0
#endif
#ifndef GRIS_WALK_TRIS_ANY
#define GRIS_WALK_TRIS_ANY 2
#endif
constexpr int kWalkTrisClosest = GRIS_WALK_TRIS_CLOSEST, kWalkTrisAny = GRIS_WALK_TRIS_ANY;
/* prefetch the next node while a node's triangles are tested (1) or not (0) */
#ifndef GRIS_WALK_PREFETCH
#define GRIS_WALK_PREFETCH 0
#endif
constexpr bool kWalkPrefetch = GRIS_WALK_PREFETCH != 0;
/* idle lanes of a warp at which the resident walks take new rays (one atomic per refill) */
#ifndef GRIS_WALK_REFILL_IDLE
#define GRIS_WALK_REFILL_IDLE 8
#endif
constexpr int kWalkRefillIdle = GRIS_WALK_REFILL_IDLE;
/* preferred shared-memory carveout of the resident walks in percent (-1: the driver's choice);
 * 28% holds their 7 blocks of 8 KB and leaves the rest of the 256 KB to L1 (C2: 0.3% faster than
 * the driver's choice, 3% faster than 100%) */
#ifndef GRIS_WALK_CARVEOUT
#define GRIS_WALK_CARVEOUT 28
#endif
constexpr int kWalkCarveout = GRIS_WALK_CARVEOUT;

constexpr uint32_t kCoopMaxRays = 8192;
/* tiles of 16 x 8 pixels from which the spatial pass runs in two pipelined halves (below, a
 * frame's launches and stream joins cost more than the overlap saves) */
#ifndef GRIS_SPATIAL_HALVES_MIN_TILES
#define GRIS_SPATIAL_HALVES_MIN_TILES 2048
#endif
constexpr uint32_t kSpatialHalvesMinTiles = GRIS_SPATIAL_HALVES_MIN_TILES;
constexpr uint32_t kCoopStack = 1024;      /* node indices per warp (pushes are at most 32 per round) */
constexpr uint32_t kCoopTris = 96;         /* triangles per round: 4 nodes x 8 slots x 3 */
constexpr uint32_t kCoopMaxRounds = 1u << 20;

struct CoopHit { bool found; float t, u, v; uint32_t inst, tri; };

template <bool ANY>
GD CoopHit coop_walk(const uint32_t* __restrict__ nodes, const float* __restrict__ tris, float ox, float oy, float oz,
                     float dx, float dy, float dz, float tmin, float tmax, uint32_t* stack, uint32_t* triList,
                     RayCount& rc, int& err) {
    const uint32_t lane = threadIdx.x & 31u;
    const float tiny = 1e-30f;
    const float idx = 1.0f / ((dx > tiny || dx < -tiny) ? dx : (dx < 0.0f ? -tiny : tiny));
    const float idy = 1.0f / ((dy > tiny || dy < -tiny) ? dy : (dy < 0.0f ? -tiny : tiny));
    const float idz = 1.0f / ((dz > tiny || dz < -tiny) ? dz : (dz < 0.0f ? -tiny : tiny));
    const uint32_t oct = (dx < 0.0f ? 1u : 0u) | (dy < 0.0f ? 2u : 0u) | (dz < 0.0f ? 4u : 0u);
    CoopHit best;
    best.found = false; best.t = tmax; best.u = 0.0f; best.v = 0.0f; best.inst = kInvalidHit; best.tri = kInvalidHit;
    if (ox != ox || oy != oy || oz != oz || dx != dx || dy != dy || dz != dz) return best;   /* as GrisTraversal::init */
    uint32_t sp = 1u;
    if (lane == 0u) stack[0] = 0u;
    __syncwarp();
    for (uint32_t round = 0; sp > 0u; round++) {
        if (round >= kCoopMaxRounds) { err = 1; break; }
        const uint32_t p = min(sp, 4u), j = lane >> 3, s = lane & 7u;
        bool inner = false;
        uint32_t child = 0u, triCnt = 0u, triFirst = 0u;
        if (j < p) {
            const uint4* N = reinterpret_cast<const uint4*>(nodes + (uint64_t)stack[sp - 1u - j] * GRIS_NODE_WORDS);
            const uint4 w0 = __ldg(N + 0), w1 = __ldg(N + 1), w2 = __ldg(N + 2), w3 = __ldg(N + 3), w4 = __ldg(N + 4);
            const uint32_t W[20] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w, w2.x, w2.y,
                                    w2.z, w2.w, w3.x, w3.y, w3.z, w3.w, w4.x, w4.y, w4.z, w4.w};
            const uint32_t meta = gris_byte((s >> 2) ? W[7] : W[6], (int)(s & 3u));
            if (meta != 0u) {
                const uint32_t imask = W[3] >> 24;
                GrisNodeRay nr;
                gris_node_ray(W, ox, oy, oz, idx, idy, idz, oct, nr);
                if (gris_slot_hit(nr, (int)s, tmin, best.t)) {
                    if (imask & (1u << s)) { inner = true; child = W[4] + (uint32_t)__popc(imask & ((1u << s) - 1u)); }
                    else { triCnt = (meta >> 5) & 3u; triFirst = W[5] + (meta & 31u); }
                }
            }
        }
        if (lane == 0u) rc.work.nodes += p;
        __syncwarp();                                     /* the popped entries are read before pushes */
        sp -= p;
        const unsigned im = __ballot_sync(0xffffffffu, inner);
        const uint32_t nIn = (uint32_t)__popc(im);
        if (sp + nIn > kCoopStack) {
            err = 1;                                      /* not reached for trees the builder accepts */
        } else {
            if (inner) stack[sp + (uint32_t)__popc(im & ((1u << lane) - 1u))] = child;
            sp += nIn;
        }
        uint32_t incl = triCnt;
        for (uint32_t d = 1; d < 32; d <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) incl += v;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        for (uint32_t k = 0; k < triCnt; k++) triList[incl - triCnt + k] = triFirst + k;
        __syncwarp();
        for (uint32_t base = 0; base < total; base += 32u) {
            bool ok = false;
            float t = 0.0f, u = 0.0f, v = 0.0f;
            uint32_t inst = kInvalidHit, tri = kInvalidHit;
            if (base + lane < total) {
                const float4* T4 = reinterpret_cast<const float4*>(tris + (uint64_t)triList[base + lane] * GRIS_TRI_FLOATS);
                const float4 t0 = __ldg(T4 + 0), t1 = __ldg(T4 + 1), t2 = __ldg(T4 + 2);
                const float TT[12] = {t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z, t1.w, t2.x, t2.y, t2.z, t2.w};
                inst = gris_f2u(TT[3]); tri = gris_f2u(TT[7]);
                rc.work.tris++;
                ok = gris_tri_test(TT, ox, oy, oz, dx, dy, dz, tmin, best.t, &t, &u, &v);
            }
            if constexpr (ANY) {
                if (__any_sync(0xffffffffu, ok)) { best.found = true; break; }
                continue;
            } else {
            /* the warp's best accepted triangle by (t, instanceIdx, triangleIdx), in every lane */
            for (uint32_t off = 16; off > 0; off >>= 1) {
                const bool ok2 = __shfl_xor_sync(0xffffffffu, ok, off);
                const float t2_ = __shfl_xor_sync(0xffffffffu, t, off), u2 = __shfl_xor_sync(0xffffffffu, u, off),
                            v2 = __shfl_xor_sync(0xffffffffu, v, off);
                const uint32_t i2 = __shfl_xor_sync(0xffffffffu, inst, off), r2 = __shfl_xor_sync(0xffffffffu, tri, off);
                const bool take = ok2 && (!ok || t2_ < t || (t2_ == t && (i2 < inst || (i2 == inst && r2 < tri))));
                if (take) { ok = true; t = t2_; u = u2; v = v2; inst = i2; tri = r2; }
            }
            if (ok) {
                const bool keyLess = inst < best.inst || (inst == best.inst && tri < best.tri);
                if (t < best.t || (t == best.t && keyLess)) {
                    best.found = true; best.t = t; best.u = u; best.v = v; best.inst = inst; best.tri = tri;
                }
            }
            }
        }
        if (ANY && best.found) break;
        __syncwarp();                                     /* triList and the stack are rewritten next round */
    }
    return best;
}

template <bool ANY>
__global__ void __launch_bounds__(128) k_wave_trace_coop(WaveCtx C, int level) {
    const uint32_t n = ANY ? C.counts[256 + level] : C.counts[level];
    if (n >= kCoopMaxRays) return;                        /* k_wave_trace_refill takes the level */
    __shared__ uint32_t sStack[4][kCoopStack];
    __shared__ uint32_t sTris[4][kCoopTris];
    const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t* q = ANY ? C.shadowQueue : C.queue[level & 1];
    uint32_t* cursor = C.counts + (ANY ? 1280 : 1024) + level;
    RayCount rc = ray_count();
    int err = 0;
    while (true) {
        uint32_t i = 0u;
        if (lane == 0u) i = atomicAdd(cursor, 1u);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= n) break;
        const uint32_t id = q[i];
        const int v = find_view_by_pixel(C.V, C.nViews, id);
        float o[3], d[3], tmax;
        if (ANY) {
            const uint4* wv = C.nee[id].w;
            const uint4 a = wv[0], d4 = wv[4], r3 = wv[3];
            o[0] = __uint_as_float(a.x); o[1] = __uint_as_float(a.y); o[2] = __uint_as_float(a.z);
            d[0] = __uint_as_float(d4.x); d[1] = __uint_as_float(d4.y); d[2] = __uint_as_float(d4.z);
            tmax = __uint_as_float(r3.w) - kMinRayDistance;
        } else {
            const uint4 a = C.ray[2 * (uint64_t)id], b = C.ray[2 * (uint64_t)id + 1];
            o[0] = __uint_as_float(a.x); o[1] = __uint_as_float(a.y); o[2] = __uint_as_float(a.z);
            d[0] = __uint_as_float(b.x); d[1] = __uint_as_float(b.y); d[2] = __uint_as_float(b.z);
            tmax = kMaxRayDistance;
        }
        const CoopHit h = coop_walk<ANY>(C.V[v].P.sc.nodes, C.V[v].P.sc.tris, o[0], o[1], o[2], d[0], d[1], d[2],
                                         kMinRayDistance, tmax, sStack[w], sTris[w], rc, err);
        if (lane == 0u) {
            if (ANY) {
                rc.shadow++;
                C.blocked[id] = h.found ? 1 : 0;
            } else {
                rc.closest++;
                Isec r;
                if (h.found) { r.bx = h.u; r.by = h.v; r.inst = h.inst; r.tri = h.tri; }
                else { r.bx = 0.0f; r.by = 0.0f; r.inst = kInvalidHit; r.tri = 0u; }
                C.hit[id] = r;
            }
        }
        __syncwarp();
    }
    flush_counts(C.counters, rc, err, 1, C.countWork, ANY ? 1 : 0);
}

/* The level's closest hits (ANY = false, the path queue) or shadow queries (ANY = true, the
 * shadow queue), resident form: every lane walks its own ray step by step, and whenever a quarter
 * of a warp's lanes are idle the warp takes that many rays from the queue (one atomic on the
 * level's cursor), so lanes do not wait for the longest walk of their warp. Same walks, same
 * results as k_wave_extend / k_wave_shadow. */
template <bool ANY>
__global__ void __launch_bounds__(128, kWalkMinBlocks) k_wave_trace_refill(WaveCtx C, int level) {
    const uint32_t n = ANY ? C.counts[256 + level] : C.counts[level];
    if (n < kCoopMaxRays) return;                         /* k_wave_trace_coop takes a sparse level */
    const uint32_t* q = ANY ? C.shadowQueue : C.queue[level & 1];
    uint32_t* cursor = C.counts + (ANY ? 1280 : 1024) + level;
    const uint32_t lane = threadIdx.x & 31u;
    RayCount rc = ray_count();
    int err = 0;
    GrisTraversal<ANY> tr;
    __shared__ uint32_t sStack[2 * (kWalkSharedEntries > 0 ? kWalkSharedEntries : 1) * 128];
    GrisShortStack<kWalkSharedEntries> stack;
    stack.bind(sStack, threadIdx.x, 128u);
    const uint32_t* nodes = nullptr;
    const float* tris = nullptr;
    uint32_t id = 0;
    bool active = false, more = true;
    while (true) {
        unsigned idle = __ballot_sync(0xffffffffu, !active);
        if (more && __popc(idle) >= kWalkRefillIdle) {
            uint32_t take = (uint32_t)__popc(idle), leader = __ffs(idle) - 1, base = 0;
            if (lane == leader) base = atomicAdd(cursor, take);
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!active) {
                uint32_t i = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (i < n) {
                    id = q[i];
                    int v = find_view_by_pixel(C.V, C.nViews, id);
                    nodes = C.V[v].P.sc.nodes;
                    tris = C.V[v].P.sc.tris;
                    stack.reset();
                    if (ANY) {
                        const uint4* w = C.nee[id].w;
                        uint4 a = w[0], d4 = w[4], r3 = w[3];
                        float dist = __uint_as_float(r3.w);
                        tr.init(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z), __uint_as_float(d4.x),
                                __uint_as_float(d4.y), __uint_as_float(d4.z), kMinRayDistance, dist - kMinRayDistance);
                    } else {
                        const uint4 a = C.ray[2 * (uint64_t)id], b = C.ray[2 * (uint64_t)id + 1];
                        tr.init(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z), __uint_as_float(b.x),
                                __uint_as_float(b.y), __uint_as_float(b.z), kMinRayDistance, kMaxRayDistance);
                    }
                    active = true;
                }
            }
            if (base + take >= n) more = false;
        }
        if (__ballot_sync(0xffffffffu, active) == 0u) {
            if (!more) break;
            continue;
        }
        if (active && !tr.template step<(ANY ? kWalkTrisAny : kWalkTrisClosest), kWalkPrefetch>(nodes, tris, false, &err, stack)) {
            GrisRayHit h;
            tr.result(&h, &rc.work);
            if (ANY) {
                rc.shadow++;
                C.blocked[id] = tr.found ? 1 : 0;
            } else {
                rc.closest++;
                Isec r;
                if (tr.found) { r.bx = h.u; r.by = h.v; r.inst = h.inst; r.tri = h.tri; }
                else { r.bx = 0.0f; r.by = 0.0f; r.inst = kInvalidHit; r.tri = 0u; }
                C.hit[id] = r;
            }
            active = false;
        }
    }
    flush_counts(C.counters, rc, err, 1, C.countWork, ANY ? 1 : 0);
}

/* shade() of the level's paths: the end, the next level, or a shadow query */
/* resident blocks of 128 threads per SM asked of the compiler for the shading kernels (0: none) */
#ifndef GRIS_WAVE_SHADE_MIN_BLOCKS
#define GRIS_WAVE_SHADE_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(128, GRIS_WAVE_SHADE_MIN_BLOCKS) k_wave_shade(WaveCtx C, int level) {
    const uint32_t n = C.counts[level];
    const uint32_t* q = C.queue[level & 1];
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
        uint32_t i = i0 + threadIdx.x;
        bool pushNext = false, pushShadow = false;
        uint32_t id = 0;
        if (i < n) {
            id = q[i];
            int v; uint32_t x, y;
            path_coords(C, id, v, x, y);
            const PassCtx& P = C.V[v].P;
            PathTracer t;
            load_wave(C.state + id, t);
            t.ix = x; t.iy = y; t.bounce = level;
            t.mat = load_material(P.sc, t.surf.matIndex);
            int r = t.shade(P, C.hit[id]);
            if (r == PathTracer::kShadow) {
                /* the next bounce's ray now, so that its closest hit is traced while the shadow
                 * query is; post() continues the path with the same ray and checks the queueing */
                V3 o, d;
                pushNext = level + 1 < (int)P.set.maxDepth && t.next_ray(P, o, d);
                if (pushNext) store_ray(C, id, o, d);
                save_wave(C.state + id, t);
                save_nee(C.nee + id, t, pushNext ? 4u : 0u);
                pushShadow = true;
            } else {
                wave_continue(C, P, t, id, r == PathTracer::kNext, level, pushNext);
            }
        }
        warp_push(C.queue[(level + 1) & 1], C.counts + level + 1, pushNext, id);
        warp_push(C.shadowQueue, C.counts + 256 + level, pushShadow, id);
    }
}

/* the shadow queries of the level */
__global__ void __launch_bounds__(128) k_wave_shadow(WaveCtx C, int level) {
    const uint32_t n = C.counts[256 + level];
    RayCount rc = ray_count();
    int err = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i - threadIdx.x < n; i += gridDim.x * blockDim.x) {
        if (i < n) {
            uint32_t id = C.shadowQueue[i];
            const uint4* w = C.nee[id].w;
            uint4 a = w[0], d4 = w[4], r3 = w[3];
            V3 o = v3(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(a.z));
            V3 d = v3(__uint_as_float(d4.x), __uint_as_float(d4.y), __uint_as_float(d4.z));
            float dist = __uint_as_float(r3.w);
            int v = find_view_by_pixel(C.V, C.nViews, id);
            C.blocked[id] = traceShadow(C.V[v].P.sc, o, kMinRayDistance, d, dist - kMinRayDistance, rc, err) ? 1 : 0;
        }
    }
    flush_counts(C.counters, rc, err, 1, C.countWork, 1);
}

/* post() of the paths that made a shadow query */
/* post() of the level's NEE vertices. Their next rays were queued by shade() (next_ray): here
 * the path's state moves on to the next level or the path ends; a disagreement with shade()'s
 * queueing (not expected: both decisions read the same state and numbers) raises bit 3 of the
 * error word. */
__global__ void __launch_bounds__(128, GRIS_WAVE_SHADE_MIN_BLOCKS) k_wave_post(WaveCtx C, int level) {
    const uint32_t n = C.counts[256 + level];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t id = C.shadowQueue[i];
        int v; uint32_t x, y;
        path_coords(C, id, v, x, y);
        const PassCtx& P = C.V[v].P;
        PathTracer t;
        load_wave(C.state + id, t);
        load_nee(C.nee + id, t);
        const bool queued = (C.nee[id].w[1].w & 4u) != 0u;
        t.ix = x; t.iy = y; t.bounce = level;
        t.mat = load_material(P.sc, t.surf.matIndex);
        bool cont = t.post(P, C.blocked[id] != 0);
        bool unused;
        if (wave_continue(C, P, t, id, cont, level, unused, false) != queued)
            atomicOr(C.counters + GRIS_COUNTER_ERROR, 8ull);
    }
}

/* ------------------------------------------------------------------ reuse passes in three launches */
/* The temporal and spatial passes of a batch as prepare -> visibility walk -> finish (views
 * without pairwise weights; the per-pixel kernels k_batch_pass<TemporalTask / SpatialTask> stay
 * for the other forms). A reconnection's visibility query is the bulk of a reuse pass's time, and
 * inside a per-pixel kernel the few lanes that issue one leave the rest of their warp waiting:
 *   prepare  per pixel (and neighbour): the gathers, the gates, the prefix replay and the shift up
 *            to the visibility query (shift_until_query), the merge's random draw where the
 *            reference takes it; the query goes into a compacted queue, what the merge needs
 *            into per-slot records;
 *   walk     the queue by the refilling any-hit traversal (every lane busy until it is empty);
 *            a visible segment sets its slot's kRsVisible bit;
 *   finish   per pixel: the merges and M caps in neighbour order with the verdicts, the selected
 *            source sample (with the shifted Jacobian, pdf and F when visible), then the temporal
 *            reservoir, or the spatial reservoir, final shading and running mean.
 * Same operations on the same values in the same order as the per-pixel kernels: results bit for
 * bit identical, ray counts equal. Slot k of pixel p (batch pixel id) lives at k * R.P + p. */
constexpr uint8_t kRsEntry = 1u, kRsMerge = 2u, kRsQuery = 4u, kRsVisible = 8u, kRsBadWeight = 16u, kRsCopy = 32u,
                  kRsActive = 128u;

struct ReuseCtx {
    float4* pa;          /* weight if visible, source M, shifted Jacobian, shifted pdf */
    float4* pb;          /* shifted F, merge draw */
    uint32_t* pn;        /* source pixel (in the view) */
    uint8_t* ps;         /* kRs* bits; slot 0 also carries kRsActive for a non-background pixel */
    float4* q;           /* per query: origin + tmax, direction + slot */
    uint32_t* counts;    /* [0] temporal queries, [1] their cursor, [2] spatial queries, [3] their cursor */
    uint32_t P;          /* slot stride = pixels of the batch */
    uint64_t qCap;       /* queries the queue holds */
    uint32_t tile0;      /* first tile of the launch (the spatial pass runs in two halves of the tiles) */
};

/* Appends the visibility query of `q` (traceVisibility's ray: from -> to, tmin = MinRayDistance,
 * tmax = distance - MinRayDistance) for `slot`, one atomic per group of converged lanes. */
GD void reuse_push_query(const ReuseCtx& R, uint32_t* count, const ShiftPending& q, uint32_t slot, int& err) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    uint32_t base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(count, g.size());
    base = g.shfl(base, 0) + g.thread_rank();
    if ((uint64_t)base >= R.qCap) { err = 1; return; }   /* not reached: the queue holds a query per slot */
    const V3 d = normalize3(q.to - q.from);
    const float tmax = distance3(q.to, q.from) - kMinRayDistance;
    R.q[2 * (uint64_t)base] = make_float4(q.from.x, q.from.y, q.from.z, tmax);
    R.q[2 * (uint64_t)base + 1] = make_float4(d.x, d.y, d.z, __uint_as_float(slot));
}

/* resident blocks of 128 threads per SM asked of the compiler for the prepare / finish kernels */
#ifndef GRIS_REUSE_PREPARE_BLOCKS
#define GRIS_REUSE_PREPARE_BLOCKS 8
#endif
#ifndef GRIS_REUSE_FINISH_BLOCKS
#define GRIS_REUSE_FINISH_BLOCKS 8
#endif
constexpr int kReusePrepareBlocks = GRIS_REUSE_PREPARE_BLOCKS, kReuseFinishBlocks = GRIS_REUSE_FINISH_BLOCKS;

template <bool kGuide>
__global__ void __launch_bounds__(128, kReusePrepareBlocks) k_reuse_temporal_prepare(const ViewEntry* __restrict__ V, int n,
                                                                                     ReuseCtx R) {
    const int v = find_view_by_tile(V, n, blockIdx.x);
    const PassCtx& P = V[v].P;
    const uint32_t t = blockIdx.x - V[v].tileBase;
    const uint32_t x = (t % V[v].tilesX) * 16u + threadIdx.x, y = (t / V[v].tilesX) * 8u + threadIdx.y;
    RayCount rc = ray_count();
    int err = 0;
    if (x < P.b.width && y < P.b.height) {
        const uint32_t pix = V[v].pixelBase + y * P.b.width + x;
        TemporalTaskT<kGuide> task;
        task.deferred = true;
        uint8_t state = 0;
        if (task.begin(P, x, y, rc, err)) {   /* false: nothing to merge (copy: the finish kernel copies) */
            const guide::Lobes* Lp = nullptr;
            guide::Lobes L;
            if constexpr (kGuide) {
                if (primary_lobes(P, task.idx, load_material(P.sc, task.dst.matIndex), L)) Lp = &L;
            }
            ShiftPending q;
            const int kind = shift_until_query(P, task.dst, task.dstIsec, task.ray, task.src, Lp, q, rc, err);
            state = kRsEntry;
            if (kind != kShiftNoQuery) {
                state |= kRsQuery | (kind == kShiftQueryBadWeight ? kRsBadWeight : 0u);
                reuse_push_query(R, R.counts + 0, q, pix, err);
            }
            R.pa[pix] = make_float4(q.rw, task.src.sampleCount, q.jac, q.pdf);
            R.pb[pix] = make_float4(q.F.x, q.F.y, q.F.z, 0.0f);
            R.pn[pix] = task.pidx;
        } else if (task.copy) {
            state = kRsCopy;
        }
        R.ps[pix] = state;
    }
    flush_counts(P.counters, rc, err, 2, P.countWork);
}

/* reuseAndMerge's merge and cap with the verdict, then TemporalTaskT::finish */
__global__ void __launch_bounds__(128, kReuseFinishBlocks) k_reuse_temporal_finish(const ViewEntry* __restrict__ V, int n,
                                                                                    ReuseCtx R) {
    const int v = find_view_by_tile(V, n, blockIdx.x);
    const PassCtx& P = V[v].P;
    const uint32_t t = blockIdx.x - V[v].tileBase;
    const uint32_t x = (t % V[v].tilesX) * 16u + threadIdx.x, y = (t / V[v].tilesX) * 8u + threadIdx.y;
    if (x >= P.b.width || y >= P.b.height) return;
    const uint32_t pix = V[v].pixelBase + y * P.b.width + x;
    const uint8_t state = R.ps[pix];
    if (!(state & (kRsEntry | kRsCopy))) return;
    const uint64_t idx = (uint64_t)y * P.b.width + x, npx = (uint64_t)P.b.width * P.b.height;
    Resv resv = load_resv(P.b.reservoirThis, idx, npx);
    if (!(state & kRsEntry)) {               /* no temporal neighbour: the current reservoir as is */
        resvResetIfInvalid(resv);
        store_resv(P.b.reservoirTemp, idx, resv);
        return;
    }
    const float4 a = R.pa[pix];
    const bool visible = (state & kRsVisible) != 0u;
    const float w = visible ? a.x : 0.0f;   /* the source's weight: 0 unless the segment is visible */
    if (!isnan(w) && w >= 0.0f) {           /* resvIsValid(srcResv): merge */
        uint32_t resvRng = ~(makeSeed2(P.cam.seed, x, y) ^ 1u);
        const float rnd = sample1f(resvRng);
        resv.sampleCount += a.y;
        resv.resampleWeight += w;
        if (rnd * resv.resampleWeight < w) {
            resv.s = load_resv(P.b.reservoirPrev, R.pn[pix], npx).s;
            if (visible) {
                const float4 b = R.pb[pix];
                resv.s.rcJacobian = a.z;
                resv.s.rcPrevSamplePdf = a.w;
                resv.s.F = v3(b.x, b.y, b.z);
            }
        }
    }
    resvCap(resv, (float)P.set.cap);
    resvResetIfInvalid(resv);
    store_resv(P.b.reservoirTemp, idx, resv);
}

template <bool kGuide>
__global__ void __launch_bounds__(128, kReusePrepareBlocks) k_reuse_spatial_prepare(const ViewEntry* __restrict__ V, int n,
                                                                                    ReuseCtx R) {
    const uint32_t tb = blockIdx.x + R.tile0;
    const int v = find_view_by_tile(V, n, tb);
    const PassCtx& P = V[v].P;
    const uint32_t t = tb - V[v].tileBase;
    const uint32_t x = (t % V[v].tilesX) * 16u + threadIdx.x, y = (t / V[v].tilesX) * 8u + threadIdx.y;
    RayCount rc = ray_count();
    int err = 0;
    if (x < P.b.width && y < P.b.height) {
        const uint32_t pix = V[v].pixelBase + y * P.b.width + x;
        SpatialTaskT<kGuide> task;
        const bool active = task.begin(P, x, y, rc, err);   /* false: background, its running mean is updated */
        R.ps[pix] = active ? kRsActive : 0u;
        if (active && P.set.spatialReuse) {
            const DevScene& sc = P.sc;
            const int W = (int)P.b.width, H = (int)P.b.height;
            const uint64_t npx = (uint64_t)W * (uint64_t)H;
            const float tx = 1.0f / (float)W, ty = 1.0f / (float)H;
            const V2 uv = v2(task.dstIsec.bx, task.dstIsec.by);
            const guide::Lobes* Lp = nullptr;
            guide::Lobes L;
            if constexpr (kGuide) {
                if (primary_lobes(P, task.idx, load_material(sc, task.dst.matIndex), L)) Lp = &L;
            }
            for (uint32_t k = 0; k < P.set.spatialNeighbors; k++) {
                const uint32_t slot = k * R.P + pix;
                uint8_t st = 0;
                /* findNeighborReservoir (gris_resample_spatial.glsl:11-34) */
                const V2 d = toConcentricDisk(sample2f(task.rng));
                const V2 nb = v2(uv.x + d.x * P.set.spatialRadius * tx, uv.y + d.y * P.set.spatialRadius * ty);
                bool found = !(nb.x < 0.0f || nb.y < 0.0f || nb.x > 1.0f || nb.y > 1.0f);
                uint32_t nidx = 0;
                Resv src;
                if (found) {
                    const int px = (int)(nb.x * (float)P.cam.w), py = (int)(nb.y * (float)P.cam.h);
                    float depthN = 0.0f; V3 normalN = v3s(0.0f), albedoN = v3s(0.0f); int matMeshIdN = 0;
                    const float4 ndn = texture_bilinear(reinterpret_cast<const float4*>(P.b.depthNormal), W, H, nb);
                    const uint2 nam = fetch_am(reinterpret_cast<const uint2*>(P.b.albedoMatId), W, H, px, py);
                    found = unpackGBuffer(ndn, nam, depthN, normalN, albedoN, matMeshIdN);
                    if (found) {
                        const Ray3 nray = pinholeCameraSampleRay(P.cam, v2(nb.x, 1.0f - nb.y));
                        const V3 posN = nray.ori + nray.dir * (depthN - 1e-4f);
                        found = !(dot3(normalN, task.dst.norm) < 0.9f || distance3(task.dst.pos, posN) > 0.4f);
                        nidx = (uint32_t)P.cam.w * (uint32_t)py + (uint32_t)px;
                    }
                }
                if (found) {
                    src = load_resv(P.b.reservoirTemp, nidx, npx);
                    found = resvIsValid(src);
                }
                if (found) {
                    ShiftPending q;
                    const int kind = shift_until_query(P, task.dst, task.dstIsec, task.ray, src, Lp, q, rc, err);
                    bool merge = true;
                    st = kRsEntry;
                    if (kind == kShiftQuery) {
                        st |= kRsQuery;
                        reuse_push_query(R, R.counts + 2, q, slot, err);
                    } else if (kind == kShiftQueryBadWeight) {
                        /* the verdict decides whether the merge (and its draw) happens: answered here */
                        merge = !traceVisibility(sc, q.from, q.to, rc, err);
                    }
                    float rnd = 0.0f;
                    if (merge) { st |= kRsMerge; rnd = sample1f(task.rng); }
                    R.pa[slot] = make_float4(q.rw, src.sampleCount, q.jac, q.pdf);
                    R.pb[slot] = make_float4(q.F.x, q.F.y, q.F.z, rnd);
                    R.pn[slot] = nidx;
                }
                R.ps[slot] = k == 0u ? (uint8_t)(st | kRsActive) : st;
            }
        }
    }
    flush_counts(P.counters, rc, err, 3, P.countWork);
}

/* the merges and caps in neighbour order with the verdicts (SpatialTaskT::reuse_phased's last
 * phase), then SpatialTaskT::shade_final */
template <bool kGuide>
__global__ void __launch_bounds__(128, kReuseFinishBlocks) k_reuse_spatial_finish(const ViewEntry* __restrict__ V, int n,
                                                                                   ReuseCtx R) {
    const uint32_t tb = blockIdx.x + R.tile0;
    const int v = find_view_by_tile(V, n, tb);
    const PassCtx& P = V[v].P;
    const uint32_t t = tb - V[v].tileBase;
    const uint32_t x = (t % V[v].tilesX) * 16u + threadIdx.x, y = (t / V[v].tilesX) * 8u + threadIdx.y;
    RayCount rc = ray_count();
    int err = 0;
    if (x < P.b.width && y < P.b.height) {
        const uint32_t pix = V[v].pixelBase + y * P.b.width + x;
        if (R.ps[pix] & kRsActive) {
            SpatialTaskT<kGuide> task;
            task.begin(P, x, y, rc, err);   /* the pixel's surface, ray and temporary reservoir */
            if (P.set.spatialReuse) {
                int sel = -1;
                float4 sa = make_float4(0.0f, 0.0f, 0.0f, 0.0f), sb = sa;
                bool svis = false;
                for (uint32_t k = 0; k < P.set.spatialNeighbors; k++) {
                    const uint32_t slot = k * R.P + pix;
                    const uint8_t st = R.ps[slot];
                    if (!(st & kRsEntry)) continue;
                    if (st & kRsMerge) {
                        const float4 a = R.pa[slot], b = R.pb[slot];
                        const bool vis = (st & kRsVisible) != 0u;
                        const float w = vis ? a.x : 0.0f;
                        task.resv.sampleCount += a.y;
                        task.resv.resampleWeight += w;
                        if (b.w * task.resv.resampleWeight < w) { sel = (int)k; sa = a; sb = b; svis = vis; }
                    }
                    resvCap(task.resv, (float)P.set.cap);
                }
                if (sel >= 0) {
                    const uint64_t npx = (uint64_t)P.b.width * P.b.height;
                    task.resv.s = load_resv(P.b.reservoirTemp, R.pn[(uint32_t)sel * R.P + pix], npx).s;
                    if (svis) {
                        task.resv.s.rcJacobian = sa.z;
                        task.resv.s.rcPrevSamplePdf = sa.w;
                        task.resv.s.F = v3(sb.x, sb.y, sb.z);
                    }
                }
            }
            task.shade_final(P, rc, err);
        }
    }
    flush_counts(P.counters, rc, err, 3, P.countWork);
}

/* The pass's visibility queries, resident form of k_wave_trace_refill<true>: every lane walks its
 * own query step by step, and whenever a quarter of a warp's lanes are idle the warp takes that
 * many queries from the queue. KERNEL: the pass whose counters the walks add to (2 temporal,
 * 3 spatial); which = 0 temporal queue, 1 spatial queue. */
template <int KERNEL>
__global__ void __launch_bounds__(128, kWalkMinBlocks) k_reuse_visibility(const ViewEntry* __restrict__ V, int nViews, ReuseCtx R,
                                                                          int which) {
    const uint32_t n = R.counts[2 * which];
    uint32_t* cursor = R.counts + 2 * which + 1;
    const uint32_t lane = threadIdx.x & 31u;
    RayCount rc = ray_count();
    int err = 0;
    GrisTraversal<true> tr;
    __shared__ uint32_t sStack[2 * (kWalkSharedEntries > 0 ? kWalkSharedEntries : 1) * 128];
    GrisShortStack<kWalkSharedEntries> stack;
    stack.bind(sStack, threadIdx.x, 128u);
    const uint32_t* nodes = nullptr;
    const float* tris = nullptr;
    uint32_t slot = 0;
    bool active = false, more = n > 0u;
    while (true) {
        unsigned idle = __ballot_sync(0xffffffffu, !active);
        if (more && __popc(idle) >= kWalkRefillIdle) {
            const uint32_t take = (uint32_t)__popc(idle), leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(cursor, take);
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!active) {
                const uint32_t i = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (i < n) {
                    const float4 a = R.q[2 * (uint64_t)i], b = R.q[2 * (uint64_t)i + 1];
                    slot = __float_as_uint(b.w);
                    const int v = find_view_by_pixel(V, nViews, slot % R.P);
                    nodes = V[v].P.sc.nodes;
                    tris = V[v].P.sc.tris;
                    stack.reset();
                    tr.init(a.x, a.y, a.z, b.x, b.y, b.z, kMinRayDistance, a.w);
                    active = true;
                }
            }
            if (base + take >= n) more = false;
        }
        if (__ballot_sync(0xffffffffu, active) == 0u) {
            if (!more) break;
            continue;
        }
        if (active && !tr.template step<kWalkTrisAny, kWalkPrefetch>(nodes, tris, false, &err, stack)) {
            GrisRayHit h;
            tr.result(&h, &rc.work);
            rc.shadow++;
            if (!tr.found) R.ps[slot] |= kRsVisible;
            active = false;
        }
    }
    flush_counts(V[0].P.counters, rc, err, KERNEL, V[0].P.countWork, KERNEL);
}

/* ------------------------------------------------------------------ guided wavefront */
using GuidedTracer = PathTracerT<true, true>;

/* Vertices whose outgoing direction the guide may draw: after the path's reconnection vertex
 * (a surface), which the hybrid shift never replays, on Lambert or rough metallic-workflow
 * surfaces, when the direction will be traced. */
GD bool guide_eligible(const GuidedTracer& t, const PassCtx& P) {
    return t.sampleState == 2u && rcVertexType(t.pathSample.flags) == kRcSurface && !t.surf.isLight &&
           (t.mat.type == 1u || (t.mat.type == 2u && t.mat.roughness >= 0.01f)) && t.bounce + 1 < (int)P.set.maxDepth;
}

/* A slot per lane with `take` from a counter, one atomic per warp. */
GD uint32_t warp_alloc(uint32_t* count, bool take) {
    unsigned m = __ballot_sync(0xffffffffu, take);
    if (!m) return 0u;
    uint32_t lane = threadIdx.x & 31u, leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

/* frame start: the probability of keeping a guided vertex as a training record, from the
 * previous frame's count of guided vertices, so that about `cap` records are gathered */
__global__ void k_guide_frame_begin(uint32_t* frame, uint32_t* tCount, uint32_t cap) {
    uint32_t e = frame[0];
    float p = e > 0u ? fminf(1.0f, 1.25f * (float)cap / (float)e) : 1.0f;
    frame[1] = __float_as_uint(p);
    frame[0] = 0u;
    frame[2] += 1u;
    *tCount = 0u;
}

/* The guide's inputs at every pixel's primary vertex (zeros for the background), for one
 * inference over the whole batch before the path tracer. */
__global__ void __launch_bounds__(128) k_guide_primary_features(WaveCtx C, float* feat) {
    uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= C.totalPixels) return;
    int v; uint32_t x, y;
    path_coords(C, id, v, x, y);
    const ViewEntry& V = C.V[v];
    const PassCtx& P = V.P;
    const int W = (int)P.b.width, H = (int)P.b.height;
    V2 uv = v2(((float)x + 0.5f) / (float)W, ((float)y + 0.5f) / (float)H);
    float depth = 0.0f; V3 norm = v3s(0.0f), albedo = v3s(0.0f); int matMeshId = 0;
    float4 dn = texture_bilinear(reinterpret_cast<const float4*>(P.b.depthNormal), W, H, uv);
    uint2 am = fetch_am(reinterpret_cast<const uint2*>(P.b.albedoMatId), W, H, (int)x, (int)y);
    float f[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (unpackGBuffer(dn, am, depth, norm, albedo, matMeshId)) {
        Ray3 ray = pinholeCameraSampleRay(P.cam, v2(uv.x, 1.0f - uv.y));
        V3 pos = ray.ori + ray.dir * (depth - 1e-4f);
        f[0] = fminf(fmaxf((pos.x - V.boxMin[0]) * V.boxInv[0], 0.0f), 1.0f);
        f[1] = fminf(fmaxf((pos.y - V.boxMin[1]) * V.boxInv[1], 0.0f), 1.0f);
        f[2] = fminf(fmaxf((pos.z - V.boxMin[2]) * V.boxInv[2], 0.0f), 1.0f);
        f[3] = norm.x; f[4] = norm.y; f[5] = norm.z;
        f[6] = -ray.dir.x; f[7] = -ray.dir.y; f[8] = -ray.dir.z;
    }
    for (int k = 0; k < 9; k++) feat[(size_t)id * 9 + k] = f[k];
}

/* Keeps the guided vertex just sampled as the path's training record with the frame's record
 * probability (a hash of the frame, the path and the level). */
GD void guide_maybe_record(const WaveCtx& C, GuidedTracer& t, uint32_t id, int level, const float* feat, float pKeep,
                           uint32_t frame) {
    uint32_t h = hash2(frame * 0x9e3779b9u ^ hash2(id * 0x85ebca6bu + (uint32_t)level));
    if ((float)(h >> 8) * (1.0f / 16777216.0f) >= pKeep) return;
    float* r = C.gRec + (size_t)id * 18;
    for (int k = 0; k < 9; k++) r[k] = feat[k];
    r[9] = t.s.wi.x; r[10] = t.s.wi.y; r[11] = t.s.wi.z;
    r[12] = t.thrSampled.x; r[13] = t.thrSampled.y; r[14] = t.thrSampled.z;
    r[15] = t.accAll.x; r[16] = t.accAll.y; r[17] = t.accAll.z;
    t.rec = 1u;
}

/* level 0 of a guided batch: the primary vertex's direction is drawn from the pixel's mixture
 * (the hybrid shift replays that draw with the destination pixel's mixture) */
__global__ void __launch_bounds__(128) k_gwave_begin(WaveCtx C) {
    uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
    bool push = false, guided = false;
    if (id < C.totalPixels) {
        int v; uint32_t x, y;
        path_coords(C, id, v, x, y);
        const PassCtx& P = C.V[v].P;
        GuidedTracer t;
        if (t.begin(P, x, y)) {
            int r = t.shade(P, isec_zero());   /* no NEE at bounce 0 */
            bool cont = false;
            if (r == GuidedTracer::kPost) {
                guide::Lobes L;
                guided = primary_lobes(P, (uint64_t)y * P.b.width + x, t.mat, L);
                cont = t.post(P, false, guided ? &L : nullptr, P.gMix);
                if (cont && guided)
                    guide_maybe_record(C, t, id, 0, C.gPrimFeat + (size_t)id * 9, __uint_as_float(C.gFrame[1]), C.gFrame[2]);
            }
            wave_continue(C, P, t, id, cont, 0, push);
        }
    }
    unsigned m = __ballot_sync(0xffffffffu, guided);
    if (m && (threadIdx.x & 31u) == (uint32_t)(__ffs(m) - 1)) atomicAdd(C.gFrame, (uint32_t)__popc(m));
    warp_push(C.queue[1], C.counts + 1, push, id);
}

/* shade() of the level's paths: the end, or a post() call (after a shadow query for NEE
 * vertices), with the guide's inputs written for eligible vertices */
__global__ void __launch_bounds__(128) k_gwave_shade(WaveCtx C, int level) {
    const uint32_t n = C.counts[level];
    const uint32_t* q = C.queue[level & 1];
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
        uint32_t i = i0 + threadIdx.x;
        bool pushPost = false, pushShadow = false, pushGuide = false;
        uint32_t id = 0;
        float feat[9];
        if (i < n) {
            id = q[i];
            int v; uint32_t x, y;
            path_coords(C, id, v, x, y);
            const PassCtx& P = C.V[v].P;
            GuidedTracer t;
            load_wave(C.state + id, t);
            t.ix = x; t.iy = y; t.bounce = level;
            t.mat = load_material(P.sc, t.surf.matIndex);
            int r = t.shade(P, C.hit[id]);
            if (r == GuidedTracer::kShadow || r == GuidedTracer::kPost) {
                pushGuide = guide_eligible(t, P);
                if (pushGuide) {
                    const ViewEntry& V = C.V[v];
                    feat[0] = fminf(fmaxf((t.surf.pos.x - V.boxMin[0]) * V.boxInv[0], 0.0f), 1.0f);
                    feat[1] = fminf(fmaxf((t.surf.pos.y - V.boxMin[1]) * V.boxInv[1], 0.0f), 1.0f);
                    feat[2] = fminf(fmaxf((t.surf.pos.z - V.boxMin[2]) * V.boxInv[2], 0.0f), 1.0f);
                    feat[3] = t.surf.norm.x; feat[4] = t.surf.norm.y; feat[5] = t.surf.norm.z;
                    feat[6] = t.wo.x; feat[7] = t.wo.y; feat[8] = t.wo.z;
                }
                save_wave(C.state + id, t);
                save_nee(C.nee + id, t);
                pushPost = true;
                pushShadow = r == GuidedTracer::kShadow;
            } else {
                bool unused;
                wave_continue(C, P, t, id, false, level, unused);
            }
        }
        uint32_t slot = warp_alloc(C.counts + 768 + level, pushGuide);
        if (pushGuide) {
            for (int k = 0; k < 9; k++) C.gFeat[(size_t)slot * 9 + k] = feat[k];
        }
        if (pushPost) reinterpret_cast<uint32_t*>(&C.nee[id].w[5])[3] = pushGuide ? slot + 1u : 0u;
        warp_push(C.postQueue, C.counts + 512 + level, pushPost, id);
        warp_push(C.shadowQueue, C.counts + 256 + level, pushShadow, id);
    }
}

/* post() of the level's paths, with the guide mixture at guided vertices; a guided vertex is
 * kept as its path's training record with the frame's record probability */
__global__ void __launch_bounds__(128) k_gwave_post(WaveCtx C, int level) {
    const uint32_t n = C.counts[512 + level];
    const float pKeep = __uint_as_float(C.gFrame[1]);
    const uint32_t frame = C.gFrame[2];
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
        uint32_t i = i0 + threadIdx.x;
        bool push = false, guided = false;
        uint32_t id = 0;
        if (i < n) {
            id = C.postQueue[i];
            int v; uint32_t x, y;
            path_coords(C, id, v, x, y);
            const PassCtx& P = C.V[v].P;
            GuidedTracer t;
            load_wave(C.state + id, t);
            load_nee(C.nee + id, t);
            t.ix = x; t.iy = y; t.bounce = level;
            t.mat = load_material(P.sc, t.surf.matIndex);
            const uint32_t slot1 = reinterpret_cast<const uint32_t*>(&C.nee[id].w[5])[3];
            guide::Lobes L;
            if (slot1) guide::make_lobes(C.gOut + (size_t)(slot1 - 1u) * guide::kRaw, L);
            guided = slot1 != 0u;
            bool blocked = t.nee ? C.blocked[id] != 0 : false;
            bool cont = t.post(P, blocked, guided ? &L : nullptr, C.guide.mix);
            if (cont && guided) guide_maybe_record(C, t, id, level, C.gFeat + (size_t)(slot1 - 1u) * 9, pKeep, frame);
            wave_continue(C, P, t, id, cont, level, push);
        }
        unsigned m = __ballot_sync(0xffffffffu, guided);
        if (m && (threadIdx.x & 31u) == (uint32_t)(__ffs(m) - 1)) atomicAdd(C.gFrame, (uint32_t)__popc(m));
        warp_push(C.queue[(level + 1) & 1], C.counts + level + 1, push, id);
    }
}

cudaError_t wave_streams_create(WaveBuffers& wb) {
    cudaError_t e = cudaStreamCreateWithFlags(&wb.aux, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&wb.aux2, cudaStreamNonBlocking);
    for (cudaEvent_t* ev : {&wb.evFork, &wb.evJoin, &wb.evTemporal, &wb.evTemporalDone})
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    return e;
}

void wave_streams_destroy(WaveBuffers& wb) {
    for (cudaStream_t* s : {&wb.aux, &wb.aux2})
        if (*s) { cudaStreamSynchronize(*s); cudaStreamDestroy(*s); *s = nullptr; }
    for (cudaEvent_t* ev : {&wb.evFork, &wb.evJoin, &wb.evTemporal, &wb.evTemporalDone})
        if (*ev) { cudaEventDestroy(*ev); *ev = nullptr; }
}


static size_t reuse_up(size_t n) { return (n + 255) & ~(size_t)255; }
size_t reuse_bytes(uint64_t pixels, uint32_t slots) {
    const size_t s = (size_t)pixels * slots;
    return 2 * reuse_up(s * 16) + reuse_up(s * 4) + reuse_up(s) + reuse_up(s * 32) + 256;
}
void reuse_carve(ReuseBuffers& r, void* block, uint64_t pixels, uint32_t slots) {
    const size_t s = (size_t)pixels * slots;
    char* p = (char*)block;
    r.block = block;
    r.pa = p; p += reuse_up(s * 16);
    r.pb = p; p += reuse_up(s * 16);
    r.pn = (uint32_t*)p; p += reuse_up(s * 4);
    r.ps = (unsigned char*)p; p += reuse_up(s);
    r.q = p; p += reuse_up(s * 32);
    r.counts = (uint32_t*)p;
    r.slots = slots;
    r.capacity = pixels;
}

BatchShape fill_view_table(const BatchView* views, int n, void* hViews, unsigned long long* counters, int countWork,
                           const float* gPrim, float gMix) {
    BatchShape sh;
    sh.n = n; sh.tiles = 0; sh.pixels = 0; sh.maxDepth = 0;
    ViewEntry* H = reinterpret_cast<ViewEntry*>(hViews);
    for (int i = 0; i < n; i++) {
        const BatchView& bv = views[i];
        ViewEntry& e = H[i];
        memset(&e, 0, sizeof(e));
        e.P.countWork = countWork;
        e.P.sc = to_dev(bv.scene);
        e.P.cam = make_cam(bv.cam);
        e.P.prev = make_cam(bv.prev);
        e.P.set = bv.set;
        e.P.b = bv.b;
        e.P.counters = counters;
        e.P.gPrim = gPrim;
        e.P.gMix = gMix;
        e.P.pixelBase = sh.pixels;
        e.G.sc = e.P.sc;
        e.G.cam = e.P.cam;
        for (int k = 0; k < 16; k++) e.G.lastProjView[k] = bv.cam.lastProjView[k];
        e.G.b = bv.gb;
        e.G.counters = counters;
        e.G.countWork = countWork;
        for (int c = 0; c < 3; c++) {
            float ext = bv.scene.boxMax[c] - bv.scene.boxMin[c];
            e.boxMin[c] = bv.scene.boxMin[c];
            e.boxInv[c] = ext > 0.0f ? 1.0f / ext : 0.0f;
        }
        e.tilesX = (bv.b.width + 15) / 16;
        e.tileBase = sh.tiles;
        e.pixelBase = sh.pixels;
        sh.tiles += e.tilesX * ((bv.b.height + 7) / 8);
        sh.pixels += bv.b.width * bv.b.height;
        if ((int)bv.set.maxDepth > sh.maxDepth) sh.maxDepth = (int)bv.set.maxDepth;
        if (bv.set.misWeights) sh.pairwise = true;
        if (bv.set.spatialNeighbors > sh.maxNeighbours) sh.maxNeighbours = bv.set.spatialNeighbors;
    }
    return sh;
}

cudaError_t enqueue_batch(const BatchShape& sh, void* dViews, const void* hViews, const WaveBuffers& wb,
                          unsigned long long* counters, int countWork, KernelTimer* timer, cudaStream_t stream,
                          int pathForm, int passes, const WaveLaunch& wl, const guide::GuideDevice* guide) {
    const int n = sh.n;
    if (guide && (pathForm != GRIS_PATH_WAVEFRONT || !wb.postQueue)) return cudaErrorInvalidValue;
    if (n <= 0 || n > 4096) return cudaErrorInvalidValue;
    if ((uint64_t)sh.pixels > wb.capacity && pathForm == GRIS_PATH_WAVEFRONT && (passes & 1)) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemcpyAsync(dViews, hViews, sizeof(ViewEntry) * (size_t)n, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return e;
    const ViewEntry* V = reinterpret_cast<const ViewEntry*>(dViews);
    const uint32_t tiles = sh.tiles, pixels = sh.pixels;
    dim3 blk(16, 8);
    if (passes & 8) {
        if (timer) timer->mark(0, true, stream);
        k_batch_gbuffer<<<tiles, blk, 0, stream>>>(V, n);
        if (timer) timer->mark(0, false, stream);
    }
    /* the three-launch form of the reuse passes where its buffers fit the frame */
    const bool split = wb.reuse.slots > 0u && !sh.pairwise && sh.maxNeighbours <= wb.reuse.slots &&
                       (uint64_t)sh.pixels <= wb.reuse.capacity && (passes & 6);
    ReuseCtx R;
    memset(&R, 0, sizeof(R));
    if (split) {
        R.pa = reinterpret_cast<float4*>(wb.reuse.pa);
        R.pb = reinterpret_cast<float4*>(wb.reuse.pb);
        R.pn = wb.reuse.pn;
        R.ps = wb.reuse.ps;
        R.q = reinterpret_cast<float4*>(wb.reuse.q);
        R.counts = wb.reuse.counts;
        R.P = pixels;
        R.qCap = (uint64_t)pixels * wb.reuse.slots;
        e = cudaMemsetAsync(wb.reuse.counts, 0, 4 * sizeof(uint32_t), stream);
        if (e != cudaSuccess) return e;
    }
    const int gridVis = current_sm_count() * (wl.traceBlocksPerSM > 0 ? wl.traceBlocksPerSM : 16);
    if (kWalkCarveout >= 0) {
        /* the resident walks' preferred shared-memory carveout (percent of the maximum): what is
         * not shared memory is L1, which caches the nodes and triangles */
        once_per_device(kDeviceKeyWalkCarveout, []() {
            cudaError_t c = cudaFuncSetAttribute(k_wave_trace_refill<false>, cudaFuncAttributePreferredSharedMemoryCarveout, kWalkCarveout);
            if (c == cudaSuccess) c = cudaFuncSetAttribute(k_wave_trace_refill<true>, cudaFuncAttributePreferredSharedMemoryCarveout, kWalkCarveout);
            if (c == cudaSuccess) c = cudaFuncSetAttribute(k_reuse_visibility<2>, cudaFuncAttributePreferredSharedMemoryCarveout, kWalkCarveout);
            if (c == cudaSuccess) c = cudaFuncSetAttribute(k_reuse_visibility<3>, cudaFuncAttributePreferredSharedMemoryCarveout, kWalkCarveout);
            return c == cudaSuccess ? 1 : -1;
        });
    }
    /* The temporal pass's prepare kernel and its visibility walk read the G-buffers, the
     * previous frame's reservoirs and, in a guided batch, the guide's mixture at the primary
     * vertices — nothing of this frame's path tracing (the current reservoir is merged, or
     * copied, by the finish kernel): with a side stream they run beside the path tracer (from
     * the G-buffer on, or from the primary vertices' inference on in a guided batch), joined
     * before the finish kernel. */
    const bool earlyTemporal = split && (passes & 2) && wb.aux2 != nullptr && timer == nullptr &&
                               (!guide || (passes & 1));
    auto early_temporal = [&]() -> cudaError_t {
        cudaError_t x = cudaEventRecord(wb.evTemporal, stream);
        if (x == cudaSuccess) x = cudaStreamWaitEvent(wb.aux2, wb.evTemporal, 0);
        if (x != cudaSuccess) return x;
        if (guide) k_reuse_temporal_prepare<true><<<tiles, blk, 0, wb.aux2>>>(V, n, R);
        else k_reuse_temporal_prepare<false><<<tiles, blk, 0, wb.aux2>>>(V, n, R);
        k_reuse_visibility<2><<<gridVis, 128, 0, wb.aux2>>>(V, n, R, 0);
        return cudaEventRecord(wb.evTemporalDone, wb.aux2);
    };
    if (earlyTemporal && !guide && (e = early_temporal()) != cudaSuccess) return e;
    if (passes & 1) {
        if (timer) timer->mark(1, true, stream);
        if (pathForm == GRIS_PATH_WAVEFRONT) {
            WaveCtx C;
            C.V = V; C.nViews = n; C.totalPixels = pixels;
            C.state = reinterpret_cast<WaveRec*>(wb.state);
            C.nee = reinterpret_cast<NeeRec*>(wb.nee);
            C.hit = reinterpret_cast<Isec*>(wb.hit);
            C.blocked = wb.blocked;
            C.queue[0] = wb.queue[0]; C.queue[1] = wb.queue[1];
            C.shadowQueue = wb.shadowQueue;
            C.ray = reinterpret_cast<uint4*>(wb.ray);
            C.counts = wb.counts;
            C.counters = counters;
            C.countWork = countWork;
            C.postQueue = wb.postQueue;
            C.gFeat = wb.gFeat; C.gOut = wb.gOut; C.gRec = wb.gRec; C.gFrame = wb.gFrame; C.gPrimFeat = wb.gPrimFeat;
            if (guide) C.guide = *guide; else memset(&C.guide, 0, sizeof(C.guide));
            C.frameSeed = 0u;
            e = cudaMemsetAsync(wb.counts, 0, 1536 * sizeof(uint32_t), stream);
            if (e != cudaSuccess) return e;
            const int sm = current_sm_count();
            const int gridShade = sm * (wl.shadeBlocksPerSM > 0 ? wl.shadeBlocksPerSM : 8);
            const int gridTrace = sm * (wl.traceBlocksPerSM > 0 ? wl.traceBlocksPerSM : 16);
            const int gridCoop = sm * 4;   /* sparse levels: 4 blocks of 4 warps per SM, 17.9 KB shared each */
            /* timer slots 4..8: begin, extend, shade, shadow, post */
            auto mark = [&](int slot, bool begin) { if (timer) timer->mark(slot, begin, stream); };
            if (guide) {
                /* guided: every path continues through post(); guided vertices get the network's
                 * mixture between the shading and post() (timer slot 9) */
                k_guide_frame_begin<<<1, 1, 0, stream>>>(wb.gFrame, guide->tCount, guide->cap);
                mark(9, true);
                k_guide_primary_features<<<(pixels + 127) / 128, 128, 0, stream>>>(C, wb.gPrimFeat);
                {
                    guide::FwdArgs fa;
                    fa.wPacked = guide->wPacked; fa.bias = guide->bias; fa.feat = wb.gPrimFeat;
                    fa.count = nullptr; fa.n = pixels; fa.out = wb.gPrimOut;
                    fa.tensorCores = guide->tensorCores; fa.err = counters + GRIS_COUNTER_ERROR;
                    e = guide::launch_forward(fa, stream);
                    if (e != cudaSuccess) return e;
                }
                mark(9, false);
                if (earlyTemporal && (e = early_temporal()) != cudaSuccess) return e;
                mark(4, true);
                k_gwave_begin<<<(pixels + 127) / 128, 128, 0, stream>>>(C);
                mark(4, false);
                for (int level = 1; level < sh.maxDepth; level++) {
                    mark(5, true);
                    if (wl.refill) { k_wave_trace_refill<false><<<gridTrace, 128, 0, stream>>>(C, level); k_wave_trace_coop<false><<<gridCoop, 128, 0, stream>>>(C, level); }
                    else k_wave_extend<<<gridTrace, 128, 0, stream>>>(C, level);
                    mark(5, false);
                    mark(6, true);
                    k_gwave_shade<<<gridShade, 128, 0, stream>>>(C, level);
                    mark(6, false);
                    /* the level's shadow queries beside the guide's inference (post() needs both);
                     * in order on one stream under the kernel timer */
                    const bool gfork = wb.aux != nullptr && timer == nullptr;
                    cudaStream_t ss = gfork ? wb.aux : stream;
                    if (gfork) {
                        if ((e = cudaEventRecord(wb.evFork, stream)) != cudaSuccess) return e;
                        if ((e = cudaStreamWaitEvent(wb.aux, wb.evFork, 0)) != cudaSuccess) return e;
                    }
                    mark(7, true);
                    if (wl.refill) { k_wave_trace_refill<true><<<gridTrace, 128, 0, ss>>>(C, level); k_wave_trace_coop<true><<<gridCoop, 128, 0, ss>>>(C, level); }
                    else k_wave_shadow<<<gridTrace, 128, 0, ss>>>(C, level);
                    mark(7, false);
                    mark(9, true);
                    guide::FwdArgs fa;
                    fa.wPacked = guide->wPacked; fa.bias = guide->bias; fa.feat = wb.gFeat;
                    fa.count = wb.counts + 768 + level; fa.n = (uint32_t)wb.capacity; fa.out = wb.gOut;
                    fa.tensorCores = guide->tensorCores; fa.err = counters + GRIS_COUNTER_ERROR;
                    e = guide::launch_forward(fa, stream);
                    if (e != cudaSuccess) return e;
                    mark(9, false);
                    if (gfork) {
                        if ((e = cudaEventRecord(wb.evJoin, wb.aux)) != cudaSuccess) return e;
                        if ((e = cudaStreamWaitEvent(stream, wb.evJoin, 0)) != cudaSuccess) return e;
                    }
                    mark(8, true);
                    k_gwave_post<<<gridShade, 128, 0, stream>>>(C, level);
                    mark(8, false);
                }
                if (timer) timer->mark(1, false, stream);
                goto reuse;
            }
            mark(4, true);
            k_wave_begin<<<(pixels + 127) / 128, 128, 0, stream>>>(C);
            mark(4, false);
            /* Level L's closest hits (queued by shade(L - 1), NEE vertices' next rays included)
             * run beside level L - 1's shadow queries and post() on a second stream (a fork and a
             * join in the captured graph); with a kernel timer everything runs in order on one
             * stream. */
            const bool fork = wb.aux != nullptr && timer == nullptr;
            auto shadow_post = [&](int lv, cudaStream_t s) {
                mark(7, true);
                if (wl.refill) { k_wave_trace_refill<true><<<gridTrace, 128, 0, s>>>(C, lv); k_wave_trace_coop<true><<<gridCoop, 128, 0, s>>>(C, lv); }
                else k_wave_shadow<<<gridTrace, 128, 0, s>>>(C, lv);
                mark(7, false);
                mark(8, true);
                k_wave_post<<<gridShade, 128, 0, s>>>(C, lv);
                mark(8, false);
            };
            for (int level = 1; level < sh.maxDepth; level++) {
                const bool prev = level > 1;
                if (prev && fork) {
                    if ((e = cudaEventRecord(wb.evFork, stream)) != cudaSuccess) return e;
                    if ((e = cudaStreamWaitEvent(wb.aux, wb.evFork, 0)) != cudaSuccess) return e;
                    shadow_post(level - 1, wb.aux);
                }
                mark(5, true);
                if (wl.refill) { k_wave_trace_refill<false><<<gridTrace, 128, 0, stream>>>(C, level); k_wave_trace_coop<false><<<gridCoop, 128, 0, stream>>>(C, level); }
                else k_wave_extend<<<gridTrace, 128, 0, stream>>>(C, level);
                mark(5, false);
                if (prev && fork) {
                    if ((e = cudaEventRecord(wb.evJoin, wb.aux)) != cudaSuccess) return e;
                    if ((e = cudaStreamWaitEvent(stream, wb.evJoin, 0)) != cudaSuccess) return e;
                } else if (prev) {
                    shadow_post(level - 1, stream);
                }
                mark(6, true);
                k_wave_shade<<<gridShade, 128, 0, stream>>>(C, level);
                mark(6, false);
            }
            if (sh.maxDepth > 1) shadow_post(sh.maxDepth - 1, stream);
        } else {
            k_batch_pass<PathTask, 1><<<tiles, blk, 0, stream>>>(V, n);
        }
        if (timer) timer->mark(1, false, stream);
    }
reuse:
    if (split && (passes & 2)) {
        if (timer) timer->mark(2, true, stream);
        if (earlyTemporal) {
            if ((e = cudaStreamWaitEvent(stream, wb.evTemporalDone, 0)) != cudaSuccess) return e;
        } else {
            if (guide) k_reuse_temporal_prepare<true><<<tiles, blk, 0, stream>>>(V, n, R);
            else k_reuse_temporal_prepare<false><<<tiles, blk, 0, stream>>>(V, n, R);
            if (timer) timer->mark(GRIS_SLOT_REUSE_VIS_TEMPORAL, true, stream);
            k_reuse_visibility<2><<<gridVis, 128, 0, stream>>>(V, n, R, 0);
            if (timer) timer->mark(GRIS_SLOT_REUSE_VIS_TEMPORAL, false, stream);
        }
        k_reuse_temporal_finish<<<tiles, blk, 0, stream>>>(V, n, R);
        if (timer) timer->mark(2, false, stream);
    }
    if (split && (passes & 4)) {
        if (timer) timer->mark(3, true, stream);
        auto prepare = [&](const ReuseCtx& r, uint32_t nt, cudaStream_t s) {
            if (guide) k_reuse_spatial_prepare<true><<<nt, blk, 0, s>>>(V, n, r);
            else k_reuse_spatial_prepare<false><<<nt, blk, 0, s>>>(V, n, r);
        };
        auto finish = [&](const ReuseCtx& r, uint32_t nt, cudaStream_t s) {
            if (guide) k_reuse_spatial_finish<true><<<nt, blk, 0, s>>>(V, n, r);
            else k_reuse_spatial_finish<false><<<nt, blk, 0, s>>>(V, n, r);
        };
        if (wb.aux2 != nullptr && timer == nullptr && tiles >= kSpatialHalvesMinTiles) {
            /* Two halves of the tiles, pipelined: the first half's walk and merges on the side
             * stream beside the second half's shifts and walk. Each half queues its queries in its
             * own part of the queue (counts [2..3] and [4..5]); a pixel's records and verdicts
             * belong to its half alone, and the shifts read only the temporal pass's output. */
            const uint32_t tA = tiles / 2;
            uint64_t pixA = 0;
            const ViewEntry* H = reinterpret_cast<const ViewEntry*>(hViews);
            for (int v = 0, t = 0; v < n && (uint32_t)t < tA; v++) {
                const uint32_t W = H[v].P.b.width, Hh = H[v].P.b.height, tx = H[v].tilesX;
                const uint32_t tv = tx * ((Hh + 7u) / 8u);
                for (uint32_t k = 0; k < tv && (uint32_t)t < tA; k++, t++) {
                    const uint32_t x0 = (k % tx) * 16u, y0 = (k / tx) * 8u;
                    pixA += (uint64_t)min(16u, W - x0) * min(8u, Hh - y0);
                }
            }
            ReuseCtx RA = R, RB = R;
            RA.qCap = pixA * wb.reuse.slots;
            RB.q = R.q + 2 * RA.qCap;
            RB.qCap = R.qCap - RA.qCap;
            RB.counts = R.counts + 2;
            RB.tile0 = tA;
            if ((e = cudaMemsetAsync(R.counts + 4, 0, 2 * sizeof(uint32_t), stream)) != cudaSuccess) return e;
            prepare(RA, tA, stream);
            if ((e = cudaEventRecord(wb.evTemporal, stream)) != cudaSuccess) return e;
            if ((e = cudaStreamWaitEvent(wb.aux2, wb.evTemporal, 0)) != cudaSuccess) return e;
            k_reuse_visibility<3><<<gridVis, 128, 0, wb.aux2>>>(V, n, RA, 1);
            finish(RA, tA, wb.aux2);
            if ((e = cudaEventRecord(wb.evTemporalDone, wb.aux2)) != cudaSuccess) return e;
            prepare(RB, tiles - tA, stream);
            k_reuse_visibility<3><<<gridVis, 128, 0, stream>>>(V, n, RB, 1);
            finish(RB, tiles - tA, stream);
            if ((e = cudaStreamWaitEvent(stream, wb.evTemporalDone, 0)) != cudaSuccess) return e;
        } else {
            prepare(R, tiles, stream);
            if (timer) timer->mark(GRIS_SLOT_REUSE_VIS_SPATIAL, true, stream);
            k_reuse_visibility<3><<<gridVis, 128, 0, stream>>>(V, n, R, 1);
            if (timer) timer->mark(GRIS_SLOT_REUSE_VIS_SPATIAL, false, stream);
            finish(R, tiles, stream);
        }
        if (timer) timer->mark(3, false, stream);
    }
    if (split) return cudaGetLastError();
    if (passes & 2) {
        if (timer) timer->mark(2, true, stream);
        if (guide && sh.pairwise) k_batch_pass<TemporalTaskT<true, true>, 2><<<tiles, blk, 0, stream>>>(V, n);
        else if (guide) k_batch_pass<TemporalTaskT<true>, 2><<<tiles, blk, 0, stream>>>(V, n);
        else if (sh.pairwise) k_batch_pass<TemporalTaskT<false, true>, 2><<<tiles, blk, 0, stream>>>(V, n);
        else k_batch_pass<TemporalTask, 2><<<tiles, blk, 0, stream>>>(V, n);
        if (timer) timer->mark(2, false, stream);
    }
    if (passes & 4) {
        if (timer) timer->mark(3, true, stream);
        if (guide && sh.pairwise) k_batch_pass<SpatialTaskT<true, true>, 3><<<tiles, blk, 0, stream>>>(V, n);
        else if (guide) k_batch_pass<SpatialTaskT<true>, 3><<<tiles, blk, 0, stream>>>(V, n);
        else if (sh.pairwise) k_batch_pass<SpatialTaskT<false, true>, 3><<<tiles, blk, 0, stream>>>(V, n);
        else k_batch_pass<SpatialTask, 3><<<tiles, blk, 0, stream>>>(V, n);
        if (timer) timer->mark(3, false, stream);
    }
    return cudaGetLastError();
}

cudaError_t launch_batch(const BatchView* views, int n, void* dViews, void* hViews, const WaveBuffers& wb,
                         unsigned long long* counters, int countWork, KernelTimer* timer, cudaStream_t stream,
                         int pathForm, int passes, const WaveLaunch& wl) {
    if (n <= 0 || n > 4096) return cudaErrorInvalidValue;
    BatchShape sh = fill_view_table(views, n, hViews, counters, countWork, nullptr, 0.0f);
    return enqueue_batch(sh, dViews, hViews, wb, counters, countWork, timer, stream, pathForm, passes, wl, nullptr);
}

}  // namespace grisrt
