/*
 * bvh_traverse.h — 8-wide compressed BVH layout and traversal (closest hit / any hit).
 *
 * Replaces the reference's hardware ray queries (src/shader/ray_query.glsl:6-70:
 * traceClosestHit, traceShadow) with a software walk of a compressed wide BVH in the form
 * published by Ylitie, Karras & Laine, "Efficient Incoherent Ray Traversal on GPUs Through
 * Compressed Wide BVHs", HPG 2017 — 80-byte nodes holding 8 child boxes quantised to 8 bits
 * per plane against a per-node origin and power-of-two scale, child slots ordered so that
 * visiting slot (position XOR ray octant) is approximately near-to-far.
 *
 * Node = 20 x u32:
 *   [0..2]  origin p (float)       [3] ex | ey<<8 | ez<<16 | imask<<24   (scale = 2^(e-127))
 *   [4]     first child node       [5] first triangle
 *   [6..7]  meta[8]: 0 empty; 0x80|rank (internal child, rank among internal slots);
 *           0x80 | count<<5 | offset (leaf child: `count` triangles from first+offset)
 *   [8..19] qlo_x[8] qlo_y[8] qlo_z[8] qhi_x[8] qhi_y[8] qhi_z[8] (bytes)
 * Triangle = 12 x f32: v0.xyz, instanceIdx | e1.xyz, triangleIdx | e2.xyz, 0  (e = v - v0).
 *
 * Hit semantics (the same everywhere in this project): Moller-Trumbore with its cross and dot
 * products fused (gris_tri_test), two-sided, hits with t in [tmin, tmax]; the closest hit is the smallest t, ties broken by the smaller
 * (instanceIdx, triangleIdx). Box tests only decide what is visited; boxes are padded and
 * rounded outward at build time so that every triangle the test would accept is reached.
 *
 * Box test of child slot s (gris_slot_hit): per axis the plane distances fma(q, scale/d,
 * (p - o)/d) of the slot's near and far planes, the near plane being qlo where d >= 0 and qhi
 * where d < 0. For qlo <= qhi and a finite scale/d (the builder caps the scale at 2^28, and
 * |1/d| <= 1e30) the fma is monotone in q, so near = min and far = max of the two plane
 * distances: the min/max form of the slab test, with six fewer operations per slot.
 */
#ifndef GRISRT_BVH_TRAVERSE_H
#define GRISRT_BVH_TRAVERSE_H

#include <stdint.h>

#ifdef __CUDACC__
#define GRIS_HD __host__ __device__ __forceinline__
#define GRIS_HDM __host__ __device__ __forceinline__
#else
#define GRIS_HD static inline
#define GRIS_HDM inline
#endif

#define GRIS_BVH_STACK 64
#define GRIS_NODE_WORDS 20
#define GRIS_TRI_FLOATS 12
#define GRIS_INVALID_HIT 0xffffffffu

struct GrisRayHit {
    float t, u, v;
    uint32_t inst, tri;
};

/* Work done by one or more traversals: nodes intersected, triangles tested. */
struct GrisWork {
    uint32_t nodes, tris;
};

GRIS_HD float gris_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return __builtin_fmaf(a, b, c);
#endif
}
GRIS_HD float gris_fmin(float a, float b) {
#ifdef __CUDA_ARCH__
    return fminf(a, b);
#else
    return __builtin_fminf(a, b);
#endif
}
GRIS_HD float gris_fmax(float a, float b) {
#ifdef __CUDA_ARCH__
    return fmaxf(a, b);
#else
    return __builtin_fmaxf(a, b);
#endif
}
GRIS_HD float gris_u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    union { uint32_t u; float f; } c; c.u = u; return c.f;
#endif
}
GRIS_HD uint32_t gris_f2u(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    union { uint32_t u; float f; } c; c.f = f; return c.u;
#endif
}
GRIS_HD int gris_popc(uint32_t x) {
#ifdef __CUDA_ARCH__
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
}
GRIS_HD int gris_ffs(uint32_t x) {   /* index of the lowest set bit; x != 0 */
#ifdef __CUDA_ARCH__
    return __ffs(x) - 1;
#else
    return __builtin_ctz(x);
#endif
}

/* The project's ray/triangle test. Every cross product a*b - c*d is fma(a, b, -(c*d)) and every
 * dot product a.x*b.x + a.y*b.y + a.z*b.z is fma(a.z, b.z, fma(a.y, b.y, a.x*b.x)): fused
 * operations written out (each rounded once, the same on the host and the device), the rest of
 * the sequence plain IEEE single precision. */
GRIS_HD bool gris_tri_test(const float* T, float ox, float oy, float oz, float dx, float dy, float dz,
                           float tmin, float tmax, float* tOut, float* uOut, float* vOut) {
    float e1x = T[4], e1y = T[5], e1z = T[6];
    float e2x = T[8], e2y = T[9], e2z = T[10];
    float pvx = gris_fma(dy, e2z, -(dz * e2y)), pvy = gris_fma(dz, e2x, -(dx * e2z)), pvz = gris_fma(dx, e2y, -(dy * e2x));
    float det = gris_fma(e1z, pvz, gris_fma(e1y, pvy, e1x * pvx));
    if (det == 0.0f) return false;
    float inv = 1.0f / det;
    float tvx = ox - T[0], tvy = oy - T[1], tvz = oz - T[2];
    float u = gris_fma(tvz, pvz, gris_fma(tvy, pvy, tvx * pvx)) * inv;
    if (!(u >= 0.0f) || !(u <= 1.0f)) return false;
    float qvx = gris_fma(tvy, e1z, -(tvz * e1y)), qvy = gris_fma(tvz, e1x, -(tvx * e1z)), qvz = gris_fma(tvx, e1y, -(tvy * e1x));
    float v = gris_fma(dz, qvz, gris_fma(dy, qvy, dx * qvx)) * inv;
    if (!(v >= 0.0f) || !(u + v <= 1.0f)) return false;
    float t = gris_fma(e2z, qvz, gris_fma(e2y, qvy, e2x * qvx)) * inv;
    if (!(t >= tmin) || !(t <= tmax)) return false;
    *tOut = t; *uOut = u; *vOut = v;
    return true;
}

GRIS_HD uint32_t gris_byte(uint32_t w, int i) { return (w >> (i * 8)) & 0xffu; }

/* Byte i of w as a float (exact). On the device the byte is placed in the low mantissa bits of
 * 2^23 by a byte permute and 2^23 subtracted: an integer and an add instead of a conversion. */
GRIS_HD float gris_qf(uint32_t w, int i) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u | (uint32_t)i)) - 8388608.0f;
#else
    return (float)gris_byte(w, i);
#endif
}

/* Three-operand max / min (one instruction on the device; the same value as the nested pair,
 * NaN operands ignored alike). */
GRIS_HD float gris_fmax3(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return gris_fmax(gris_fmax(a, b), c);
#endif
}
GRIS_HD float gris_fmin3(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
#else
    return gris_fmin(gris_fmin(a, b), c);
#endif
}

/* The near and far planes' bytes as floats: by byte permute (gris_qf) or by conversion, chosen per
 * plane kind (GRIS_BOX_CONVERT: bit 0 near planes, bit 1 far planes converted), to balance the
 * integer and conversion pipes. Both are exact. */
#ifndef GRIS_BOX_CONVERT
#define GRIS_BOX_CONVERT 2
#endif
GRIS_HD float gris_qf_near(uint32_t w, int i) {
    return (GRIS_BOX_CONVERT & 1) ? (float)gris_byte(w, i) : gris_qf(w, i);
}
GRIS_HD float gris_qf_far(uint32_t w, int i) {
    return (GRIS_BOX_CONVERT & 2) ? (float)gris_byte(w, i) : gris_qf(w, i);
}

/* A node's planes for one ray: the origin terms b = (p - o) / d, the scales a = scale / d and
 * the words of the near and far quantised planes per axis ([axis][word]). */
struct GrisNodeRay {
    float ax, ay, az, bx, by, bz;
    uint32_t nw[3][2], fw[3][2];
};

/* W: the node's 20 words; oct: bit a set where the direction's axis a is negative. */
GRIS_HD void gris_node_ray(const uint32_t* W, float ox, float oy, float oz, float idx, float idy, float idz,
                           uint32_t oct, GrisNodeRay& nr) {
    const float px = gris_u2f(W[0]), py = gris_u2f(W[1]), pz = gris_u2f(W[2]);
    const uint32_t e = W[3];
    const float sx = gris_u2f((e & 0xffu) << 23), sy = gris_u2f(((e >> 8) & 0xffu) << 23),
                sz = gris_u2f(((e >> 16) & 0xffu) << 23);
    nr.ax = sx * idx; nr.ay = sy * idy; nr.az = sz * idz;
    nr.bx = (px - ox) * idx; nr.by = (py - oy) * idy; nr.bz = (pz - oz) * idz;
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
    for (int a = 0; a < 3; a++) {
        const bool neg = (oct >> a) & 1u;
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
        for (int w = 0; w < 2; w++) {
            const uint32_t lo = W[8 + 2 * a + w], hi = W[14 + 2 * a + w];
            nr.nw[a][w] = neg ? hi : lo;
            nr.fw[a][w] = neg ? lo : hi;
        }
    }
}

/* The slab test of child slot s (0-7) against [tmin, tmax]. The words are chosen by selects, not
 * by an index, so that a slot known only at run time keeps nr in registers. */
GRIS_HD bool gris_slot_hit(const GrisNodeRay& nr, int s, float tmin, float tmax) {
    const bool w = (s >> 2) != 0;
    const int b = s & 3;
    const float nx = gris_fma(gris_qf_near(w ? nr.nw[0][1] : nr.nw[0][0], b), nr.ax, nr.bx);
    const float ny = gris_fma(gris_qf_near(w ? nr.nw[1][1] : nr.nw[1][0], b), nr.ay, nr.by);
    const float nz = gris_fma(gris_qf_near(w ? nr.nw[2][1] : nr.nw[2][0], b), nr.az, nr.bz);
    const float fx = gris_fma(gris_qf_far(w ? nr.fw[0][1] : nr.fw[0][0], b), nr.ax, nr.bx);
    const float fy = gris_fma(gris_qf_far(w ? nr.fw[1][1] : nr.fw[1][0], b), nr.ay, nr.by);
    const float fz = gris_fma(gris_qf_far(w ? nr.fw[2][1] : nr.fw[2][0], b), nr.az, nr.bz);
    const float tn = gris_fmax3(gris_fmax(nx, ny), nz, tmin);
    const float tf = gris_fmin3(gris_fmin(fx, fy), fz, tmax);
    return tn <= tf;
}

/*
 * The walk's stack of pending node groups. An entry is (first child node of a group, the group's
 * hit slots | the node's internal-child mask << 8). push() returns false when GRIS_BVH_STACK
 * entries are held, pop() when none is.
 *
 * GrisArrayStack holds every entry in one array: the host walk, and the device walks that run
 * outside the traversal kernels (per-thread local memory there).
 */
struct GrisArrayStack {
    uint32_t base[GRIS_BVH_STACK], bits[GRIS_BVH_STACK];
    int n;
    GRIS_HDM void reset() { n = 0; }
    GRIS_HDM bool push(uint32_t b, uint32_t m) {
        if (n >= GRIS_BVH_STACK) return false;
        base[n] = b; bits[n] = m; n++;
        return true;
    }
    GRIS_HDM bool pop(uint32_t& b, uint32_t& m) {
        if (n == 0) return false;
        n--; b = base[n]; m = bits[n];
        return true;
    }
    GRIS_HDM bool peek(uint32_t& b, uint32_t& m) const {
        if (n == 0) return false;
        b = base[n - 1]; m = bits[n - 1];
        return true;
    }
};

#ifdef __CUDACC__
/*
 * GrisShortStack (device): the top two entries in registers, the next kShared in the calling
 * thread's column of a shared-memory slab (entry i at sh[2 i stride] and sh[(2 i + 1) stride],
 * stride = the block's thread count, so a warp's same-depth accesses hit distinct banks), and
 * only deeper entries — rare: a wide BVH's walk seldom holds more than a few groups — in a
 * local-memory overflow array. A pop hands out the register top at once; the refill of the
 * second register from the slab is off the walk's critical path.
 */
template <int kShared>
struct GrisShortStack {
    uint32_t b0, m0, b1, m1;
    uint32_t* sh;
    uint32_t stride;
    int n;
    uint32_t lb[GRIS_BVH_STACK - 2 - kShared], lm[GRIS_BVH_STACK - 2 - kShared];
    __device__ __forceinline__ void bind(uint32_t* slab, uint32_t tid, uint32_t threads) {
        sh = slab + tid; stride = threads; n = 0;
    }
    __device__ __forceinline__ void reset() { n = 0; }
    __device__ __forceinline__ void store(int i, uint32_t b, uint32_t m) {
        if (i < kShared) { sh[(uint32_t)(2 * i) * stride] = b; sh[(uint32_t)(2 * i + 1) * stride] = m; }
        else { lb[i - kShared] = b; lm[i - kShared] = m; }
    }
    __device__ __forceinline__ void load(int i, uint32_t& b, uint32_t& m) const {
        if (i < kShared) { b = sh[(uint32_t)(2 * i) * stride]; m = sh[(uint32_t)(2 * i + 1) * stride]; }
        else { b = lb[i - kShared]; m = lm[i - kShared]; }
    }
    __device__ __forceinline__ bool push(uint32_t b, uint32_t m) {
        if (n >= GRIS_BVH_STACK) return false;
        if (n >= 2) store(n - 2, b1, m1);
        b1 = b0; m1 = m0; b0 = b; m0 = m; n++;
        return true;
    }
    __device__ __forceinline__ bool pop(uint32_t& b, uint32_t& m) {
        if (n == 0) return false;
        b = b0; m = m0; b0 = b1; m0 = m1;
        if (n >= 3) load(n - 3, b1, m1);
        n--;
        return true;
    }
    __device__ __forceinline__ bool peek(uint32_t& b, uint32_t& m) const {
        if (n == 0) return false;
        b = b0; m = m0;
        return true;
    }
};
#endif

/*
 * One ray's walk of the BVH as a resumable state machine: init() then step() until it returns
 * false (each step visits one node or pops one group). ANY: stop at the first accepted hit
 * (shadow rays). skipInst0: ignore the light instance (the G-buffer is rasterised without
 * lights). *err is set to 1 if the stack limit was reached (the builder guarantees it is not:
 * tree depth <= GRIS_BVH_STACK). Resumable so that a lane whose ray has finished can take the
 * next ray while the other lanes of its warp are still walking. The stack (GrisArrayStack or
 * GrisShortStack) is the caller's, reset by it before init(): kept outside the struct, the
 * struct's scalars stay in registers.
 */
template <bool ANY>
struct GrisTraversal {
    float ox, oy, oz, dx, dy, dz, idx, idy, idz, tmin;
    uint32_t oct;
    float bestT, bestU, bestV;
    uint32_t bestInst, bestTri;
    bool found;
    uint32_t grpBase, grpHits, grpImask, nodeIdx;
    uint32_t triBase, triHits;   /* the leaf triangles of the last node visited still to be tested */
    bool haveNode;
    uint32_t visits, tests;

    GRIS_HDM void init(float ox_, float oy_, float oz_, float dx_, float dy_, float dz_, float tmin_, float tmax_) {
        const float tiny = 1e-30f;
        ox = ox_; oy = oy_; oz = oz_; dx = dx_; dy = dy_; dz = dz_; tmin = tmin_;
        idx = 1.0f / ((dx > tiny || dx < -tiny) ? dx : (dx < 0.0f ? -tiny : tiny));
        idy = 1.0f / ((dy > tiny || dy < -tiny) ? dy : (dy < 0.0f ? -tiny : tiny));
        idz = 1.0f / ((dz > tiny || dz < -tiny) ? dz : (dz < 0.0f ? -tiny : tiny));
        oct = (dx < 0.0f ? 1u : 0u) | (dy < 0.0f ? 2u : 0u) | (dz < 0.0f ? 4u : 0u);
        bestT = tmax_;
        bestInst = GRIS_INVALID_HIT; bestTri = GRIS_INVALID_HIT;
        bestU = 0.0f; bestV = 0.0f;
        found = false;
        grpBase = 0; grpHits = 0; grpImask = 0;
        triBase = 0; triHits = 0;
        nodeIdx = 0;
        /* A ray with a NaN coordinate hits nothing (every triangle test compares a NaN), but the
         * box test's maxNum/minNum would pass every node on it: skip the walk, same result. */
        haveNode = !(ox != ox || oy != oy || oz != oz || dx != dx || dy != dy || dz != dz);
        visits = 0; tests = 0;
    }

    /* One leaf triangle of the last node visited (the lowest bit of triHits): the closest-hit
     * update, or for ANY the end of the walk on an accepted hit (true: the walk is over). */
    GRIS_HDM bool test_next_triangle(const float* __restrict__ tris, bool skipInst0) {
        const int b = gris_ffs(triHits);
        triHits &= triHits - 1u;
        const float* T = tris + (uint64_t)(triBase + (uint32_t)b) * GRIS_TRI_FLOATS;
#ifdef __CUDA_ARCH__
        float4 t0 = __ldg(reinterpret_cast<const float4*>(T) + 0);
        float4 t1 = __ldg(reinterpret_cast<const float4*>(T) + 1);
        float4 t2 = __ldg(reinterpret_cast<const float4*>(T) + 2);
        float TT[12] = {t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z, t1.w, t2.x, t2.y, t2.z, t2.w};
#else
        float TT[12];
        for (int i = 0; i < 12; i++) TT[i] = T[i];
#endif
        uint32_t inst = gris_f2u(TT[3]), tri = gris_f2u(TT[7]);
        if (skipInst0 && inst == 0u) return false;
        tests++;
        float t, u, v;
        if (!gris_tri_test(TT, ox, oy, oz, dx, dy, dz, tmin, bestT, &t, &u, &v)) return false;
        if (ANY) {
            bestT = t; bestU = u; bestV = v; bestInst = inst; bestTri = tri; found = true;
            return true;
        }
        /* t <= bestT here (the test used bestT as tmax) */
        bool keyLess = inst < bestInst || (inst == bestInst && tri < bestTri);
        bool better = t < bestT || (t == bestT && keyLess);
        if (better) {
            bestT = t; bestU = u; bestV = v; bestInst = inst; bestTri = tri; found = true;
        }
        return false;
    }

    /* Visits the node chosen last (nodeIdx): its child boxes; the hit leaves' triangles become
     * pending (triBase / triHits) and the hit inner children the current group (the previous
     * group, if any slots of it remain, pushed). false: the stack overflowed (*err = 1). */
    template <bool kPrefetch = false, class Stack>
    GRIS_HDM bool visit_node(const uint32_t* __restrict__ nodes, int* err, Stack& stack, bool prefetchOk) {
        const uint32_t* N = nodes + (uint64_t)nodeIdx * GRIS_NODE_WORDS;
#ifdef __CUDA_ARCH__
        uint4 w0 = __ldg(reinterpret_cast<const uint4*>(N) + 0);
        uint4 w1 = __ldg(reinterpret_cast<const uint4*>(N) + 1);
        uint4 w2 = __ldg(reinterpret_cast<const uint4*>(N) + 2);
        uint4 w3 = __ldg(reinterpret_cast<const uint4*>(N) + 3);
        uint4 w4 = __ldg(reinterpret_cast<const uint4*>(N) + 4);
        uint32_t W[20] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w, w2.x, w2.y,
                          w2.z, w2.w, w3.x, w3.y, w3.z, w3.w, w4.x, w4.y, w4.z, w4.w};
#else
        uint32_t W[20];
        for (int i = 0; i < 20; i++) W[i] = N[i];
#endif
        visits++;
        GrisNodeRay nr;
        gris_node_ray(W, ox, oy, oz, idx, idy, idz, oct, nr);
        const uint32_t imask = W[3] >> 24;
        uint32_t innerHits = 0, leafHits = 0;
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
        for (int s = 0; s < 8; s++) {
            uint32_t meta = gris_byte(W[6 + (s >> 2)], s & 3);
            if (meta == 0) continue;
            if (!gris_slot_hit(nr, s, tmin, bestT)) continue;
            if (imask & (1u << s)) innerHits |= 1u << (s ^ oct);
            else {
                uint32_t cnt = (meta >> 5) & 3u, off = meta & 31u;
                leafHits |= ((1u << cnt) - 1u) << off;
            }
        }
        triBase = W[5];
        triHits = leafHits;
        if (innerHits) {
            if (grpHits && !stack.push(grpBase, grpHits | (grpImask << 8))) { *err = 1; return false; }
            grpBase = W[4]; grpHits = innerHits; grpImask = imask;
        }
        haveNode = false;
#ifdef __CUDA_ARCH__
        if (kPrefetch && prefetchOk && triHits) {
            /* the node visited after this one's triangles is known already (the group's first
             * remaining slot, or the top group of the stack): fetch it towards L1 while the
             * triangles are tested */
            uint32_t nb = grpBase, nm = grpHits | (grpImask << 8);
            if (grpHits || stack.peek(nb, nm)) {
                const uint32_t sl = (uint32_t)gris_ffs(nm & 0xffu) ^ oct;
                const uint32_t nxt = nb + (uint32_t)gris_popc((nm >> 8) & ((1u << sl) - 1u));
                const char* p = reinterpret_cast<const char*>(nodes + (uint64_t)nxt * GRIS_NODE_WORDS);
                asm volatile("prefetch.global.L1 [%0];" :: "l"(p));
                asm volatile("prefetch.global.L1 [%0];" :: "l"(p + 4 * GRIS_NODE_WORDS - 1));
            }
        }
#endif
        return true;
    }

    /* Chooses the next node: the nearest remaining slot of the current group, else of the group
     * on top of the stack. false: none is left (the walk is over). */
    template <class Stack>
    GRIS_HDM bool choose_next(Stack& stack) {
        if (grpHits == 0) {
            uint32_t b, m;
            if (!stack.pop(b, m)) return false;
            grpBase = b; grpHits = m & 0xffu; grpImask = m >> 8;
        }
        int pos = gris_ffs(grpHits);
        grpHits &= grpHits - 1u;
        uint32_t slot = (uint32_t)pos ^ oct;
        nodeIdx = grpBase + (uint32_t)gris_popc(grpImask & ((1u << slot) - 1u));
        haveNode = true;
        return true;
    }

    /* false: the walk is over (found / best* hold the result). A step visits the node chosen by
     * the previous step (its child boxes; the hit leaves' triangles become pending), tests up to
     * kTris pending triangles (0: all of them), and once none is pending chooses the next node.
     * The order of the box and triangle tests, and so every result and count, is the same for
     * every kTris; a small kTris only spreads a node's triangles over several steps, so that the
     * lanes of a warp whose nodes hit few triangles do not wait for the lane whose node hit many. */
    template <int kTris = 0, bool kPrefetch = false, class Stack>
    GRIS_HDM bool step(const uint32_t* __restrict__ nodes, const float* __restrict__ tris, bool skipInst0, int* err,
                       Stack& stack) {
        if (haveNode && !visit_node<kPrefetch>(nodes, err, stack, kTris > 0)) return false;
        if (kTris == 0) {
            while (triHits)
                if (test_next_triangle(tris, skipInst0)) return false;
        } else {
            for (int k = 0; k < kTris && triHits; k++)
                if (test_next_triangle(tris, skipInst0)) return false;
            if (triHits) return true;
        }
        return choose_next(stack);
    }

    GRIS_HDM void result(GrisRayHit* hit, GrisWork* work) const {
        if (work) { work->nodes += visits; work->tris += tests; }
        if (found) { hit->t = bestT; hit->u = bestU; hit->v = bestV; hit->inst = bestInst; hit->tri = bestTri; }
    }
};

/* A whole walk in one call: returns true if a hit was found; `hit` receives the closest one
 * (any one for ANY). */
template <bool ANY>
GRIS_HD bool gris_bvh_trace(const uint32_t* __restrict__ nodes, const float* __restrict__ tris,
                            float ox, float oy, float oz, float dx, float dy, float dz,
                            float tmin, float tmax, bool skipInst0, GrisRayHit* hit, int* err,
                            GrisWork* work) {
    GrisTraversal<ANY> w;
    GrisArrayStack stack;
    stack.reset();
    w.init(ox, oy, oz, dx, dy, dz, tmin, tmax);
    while (w.step(nodes, tris, skipInst0, err, stack)) {}
    w.result(hit, work);
    return w.found;
}

#endif
