/*
 * bvh_build.cpp — host construction of the 8-wide compressed BVH (layout in bvh_traverse.h).
 *
 * Replaces the reference's BLAS/TLAS builds (src/Scene.cpp:448-547,
 * zvk/core/AccelerationStructure.cpp:84-139; hardware acceleration structures). Instances are
 * flattened into world space: GB300 has no ray-tracing cores and ample HBM, so one level
 * and no per-ray transform is the faster layout; every hit still reports the reference's
 * (instanceIdx, triangleIdx) pair, with instance 0 = the light triangles.
 *
 * Steps: (1) world-space triangles; (2) top-down binary BVH by binned SAH (16 bins, leaves of
 * at most 3 triangles, OpenMP tasks for large subtrees); (3) SAH-optimal collapse to 8-wide
 * nodes by dynamic programming over the binary tree (Ylitie et al. 2017, section 3.1): every
 * subtree's best use of 1..8 slots, a slot holding a leaf of at most 3 triangles or a wide
 * internal node; (4) order each node's children over 8 slots by a greedy octant assignment;
 * (5) quantise the child boxes to 8 bits per plane, padded and rounded outward, each bound
 * verified in float.
 */
#include <math.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <vector>

#include "bvh_traverse.h"
#include "grisrt_internal.h"

namespace grisrt {

void world_triangles(const GrisSceneDesc& d, std::vector<float>& v, std::vector<uint32_t>& ids) {
    uint64_t nl = d.lightCount, nObj = 0;
    std::vector<uint64_t> start(d.instanceCount + 1, 0);
    for (uint64_t k = 0; k < d.instanceCount; k++) {
        start[k] = nl + nObj;
        nObj += d.instances[k].indexCount / 3;
    }
    uint64_t n = nl + nObj;
    v.assign(n * 9, 0.0f);
    ids.assign(n * 2, 0u);
    for (uint64_t i = 0; i < nl; i++) {
        const GrisTriangleLight& L = d.lights[i];
        for (int c = 0; c < 3; c++) { v[i * 9 + c] = L.v0[c]; v[i * 9 + 3 + c] = L.v1[c]; v[i * 9 + 6 + c] = L.v2[c]; }
        ids[i * 2] = 0; ids[i * 2 + 1] = (uint32_t)i;
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t k = 0; k < (int64_t)d.instanceCount; k++) {
        const GrisObjectInstance& I = d.instances[k];
        const float* m = I.transform;
        uint64_t tcount = I.indexCount / 3;
        for (uint64_t t = 0; t < tcount; t++) {
            uint64_t o = (start[k] + t);
            for (int j = 0; j < 3; j++) {
                uint64_t ii = (uint64_t)I.indexOffset + t * 3 + (uint64_t)j;
                float px = 0.0f, py = 0.0f, pz = 0.0f;
                if (ii < d.indexCount && d.indices[ii] < d.vertexCount) {
                    const GrisMeshVertex& mv = d.vertices[d.indices[ii]];
                    px = mv.pos[0]; py = mv.pos[1]; pz = mv.pos[2];
                }
                for (int r = 0; r < 3; r++) {
                    float s = m[0 * 4 + r] * px + m[1 * 4 + r] * py;
                    s = s + m[2 * 4 + r] * pz;
                    s = s + m[3 * 4 + r] * 1.0f;
                    v[o * 9 + j * 3 + r] = s;
                }
            }
            ids[o * 2] = (uint32_t)k + 1u;
            ids[o * 2 + 1] = (uint32_t)t;
        }
    }
}

namespace {

struct Box {
    float lo[3], hi[3];
    void empty() { for (int a = 0; a < 3; a++) { lo[a] = INFINITY; hi[a] = -INFINITY; } }
    void grow(const Box& b) { for (int a = 0; a < 3; a++) { lo[a] = std::min(lo[a], b.lo[a]); hi[a] = std::max(hi[a], b.hi[a]); } }
    void growp(const float* p) { for (int a = 0; a < 3; a++) { lo[a] = std::min(lo[a], p[a]); hi[a] = std::max(hi[a], p[a]); } }
    float area() const {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (dx < 0.0f || dy < 0.0f || dz < 0.0f) return 0.0f;
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }
};

struct BNode {
    Box box;
    int32_t left = -1, right = -1;
    uint32_t first = 0, count = 0;   /* count > 0: leaf */
};

struct Binary {
    std::vector<Box> pbox;
    std::vector<float> cent;
    std::vector<uint32_t> idx;
    std::vector<BNode> nodes;
    std::atomic<uint32_t> used{1};
    static constexpr int kBins = 16;

    void make_leaf(uint32_t id, uint32_t first, uint32_t count) {
        nodes[id].left = nodes[id].right = -1;
        nodes[id].first = first;
        nodes[id].count = count;
    }

    void build(uint32_t id, uint32_t first, uint32_t count) {
        Box b, cb;
        b.empty(); cb.empty();
        for (uint32_t i = first; i < first + count; i++) {
            b.grow(pbox[idx[i]]);
            cb.growp(&cent[idx[i] * 3]);
        }
        nodes[id].box = b;
        if (count == 1) { make_leaf(id, first, count); return; }
        int bestAxis = -1, bestSplit = 0;
        float bestCost = INFINITY;
        for (int a = 0; a < 3; a++) {
            float ext = cb.hi[a] - cb.lo[a];
            if (!(ext > 0.0f)) continue;
            Box bb[kBins];
            uint32_t bc[kBins] = {0};
            for (int k = 0; k < kBins; k++) bb[k].empty();
            float scale = (float)kBins / ext;
            for (uint32_t i = first; i < first + count; i++) {
                int k = (int)((cent[idx[i] * 3 + a] - cb.lo[a]) * scale);
                k = std::min(std::max(k, 0), kBins - 1);
                bb[k].grow(pbox[idx[i]]);
                bc[k]++;
            }
            float rightArea[kBins];
            uint32_t rightCount[kBins];
            Box acc; acc.empty();
            uint32_t cnt = 0;
            for (int k = kBins - 1; k > 0; k--) {
                acc.grow(bb[k]); cnt += bc[k];
                rightArea[k] = acc.area(); rightCount[k] = cnt;
            }
            acc.empty(); cnt = 0;
            for (int k = 0; k < kBins - 1; k++) {
                acc.grow(bb[k]); cnt += bc[k];
                if (cnt == 0 || rightCount[k + 1] == 0) continue;
                float c = acc.area() * (float)cnt + rightArea[k + 1] * (float)rightCount[k + 1];
                if (c < bestCost) { bestCost = c; bestAxis = a; bestSplit = k + 1; }
            }
        }
        float area = b.area();
        if (count <= 3) {
            float splitCost = area > 0.0f ? 1.0f + bestCost / area : INFINITY;
            if (bestAxis < 0 || (float)count <= splitCost) { make_leaf(id, first, count); return; }
        }
        uint32_t mid;
        if (bestAxis >= 0) {
            float ext = cb.hi[bestAxis] - cb.lo[bestAxis];
            float scale = (float)kBins / ext;
            uint32_t* p = std::partition(&idx[first], &idx[first] + count, [&](uint32_t t) {
                int k = (int)((cent[t * 3 + bestAxis] - cb.lo[bestAxis]) * scale);
                k = std::min(std::max(k, 0), kBins - 1);
                return k < bestSplit;
            });
            mid = (uint32_t)(p - &idx[0]);
        } else {
            mid = first + count / 2;   /* all centroids coincide: split the range */
        }
        if (mid == first || mid == first + count) mid = first + count / 2;
        uint32_t l = used.fetch_add(2);
        nodes[id].left = (int32_t)l;
        nodes[id].right = (int32_t)(l + 1);
        nodes[id].count = 0;
        uint32_t nl = mid - first, nr = first + count - mid;
        if (count > 8192) {
#pragma omp task default(shared) firstprivate(l, first, nl)
            build(l, first, nl);
            build(l + 1, mid, nr);
#pragma omp taskwait
        } else {
            build(l, first, nl);
            build(l + 1, mid, nr);
        }
    }
};

struct Quant { uint32_t e; uint8_t lo[8], hi[8]; };

/* Quantises the padded child bounds of one axis against origin pf; false if a bound does not fit. */
bool quantise_axis(float pf, int e, const double* clo, const double* chi, const bool* valid, Quant& q) {
    if (e < -126 || e > 127) return false;
    float s = ldexpf(1.0f, e);
    for (int k = 0; k < 8; k++) {
        if (!valid[k]) { q.lo[k] = 0; q.hi[k] = 0; continue; }
        double ql = floor((clo[k] - (double)pf) / (double)s);
        double qh = ceil((chi[k] - (double)pf) / (double)s);
        if (ql < 0.0) ql = 0.0;
        if (qh > 255.0) return false;
        while (ql > 0.0 && (double)(pf + (float)ql * s) > clo[k]) ql -= 1.0;
        if ((double)(pf + (float)ql * s) > clo[k]) return false;
        while (qh <= 255.0 && (double)(pf + (float)qh * s) < chi[k]) qh += 1.0;
        if (qh > 255.0) return false;
        q.lo[k] = (uint8_t)ql;
        q.hi[k] = (uint8_t)qh;
    }
    q.e = (uint32_t)(e + 127);
    return true;
}

}  // namespace

bool build_bvh(const GrisSceneDesc& d, BvhHost& out, std::string& err) {
    auto t0 = std::chrono::steady_clock::now();
    std::vector<float> v;
    std::vector<uint32_t> ids;
    world_triangles(d, v, ids);
    uint64_t n = ids.size() / 2;
    if (n >= 0x7fffffffull) { err = "too many triangles"; return false; }
    out.triangleCount = n;
    out.nodes.assign(GRIS_NODE_WORDS, 0u);
    out.tris.clear();
    out.maxDepth = 1;
    if (n == 0) {   /* one empty node: every ray misses */
        out.buildSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return true;
    }
    Binary B;
    B.pbox.resize(n);
    B.cent.resize(n * 3);
    B.idx.resize(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        Box b; b.empty();
        for (int j = 0; j < 3; j++) b.growp(&v[i * 9 + j * 3]);
        B.pbox[i] = b;
        for (int a = 0; a < 3; a++) B.cent[i * 3 + a] = 0.5f * (b.lo[a] + b.hi[a]);
        B.idx[i] = (uint32_t)i;
    }
    B.nodes.resize(2 * n + 1);
#pragma omp parallel
#pragma omp single
    B.build(0, 0, (uint32_t)n);

    /* Every binary subtree's triangle range (contiguous: the builder partitions in place), then
     * the SAH-optimal collapse to 8-wide nodes (the dynamic programme of Ylitie, Karras & Laine
     * 2017, section 3.1, written from the paper): cost[n][j-1] = the least SAH cost of covering
     * subtree n with at most j slots of a wide node, where one slot holds either a leaf (a subtree
     * of at most 3 triangles: area x kTriCost x triangles) or a wide internal node (area x
     * kNodeCost + its own 8 slots distributed over the subtree); split[n][j-1] = how many of the j
     * slots the left child takes when the subtree is split (0: not split). Children have larger
     * indices than their parents, so a reverse sweep is bottom-up. */
    const uint32_t nb = B.used.load();
    std::vector<uint32_t> subFirst(nb), subCount(nb);
    for (int64_t id = (int64_t)nb - 1; id >= 0; id--) {
        const BNode& bn = B.nodes[id];
        if (bn.count > 0) { subFirst[id] = bn.first; subCount[id] = bn.count; }
        else { subFirst[id] = subFirst[bn.left]; subCount[id] = subCount[bn.left] + subCount[bn.right]; }
    }
    constexpr float kNodeCost = 1.0f, kTriCost = 0.5f;   /* a triangle test against a node visit */
    std::vector<std::array<float, 8>> cost(nb);
    std::vector<std::array<uint8_t, 8>> split(nb);
    std::vector<uint8_t> asLeaf(nb);   /* with one slot: a leaf (1) or a wide internal node (0) */
    for (int64_t id = (int64_t)nb - 1; id >= 0; id--) {
        const BNode& bn = B.nodes[id];
        const float area = bn.box.area();
        const float leafCost = subCount[id] <= 3u ? area * kTriCost * (float)subCount[id] : INFINITY;
        float dist[9];
        uint8_t arg[9];
        for (int j = 0; j <= 8; j++) { dist[j] = INFINITY; arg[j] = 0; }
        if (bn.count == 0) {
            for (int j = 2; j <= 8; j++)
                for (int k = 1; k < j; k++) {
                    const float c = cost[bn.left][k - 1] + cost[bn.right][j - k - 1];
                    if (c < dist[j]) { dist[j] = c; arg[j] = (uint8_t)k; }
                }
        }
        const float internalCost = area * kNodeCost + dist[8];
        asLeaf[id] = leafCost <= internalCost ? 1 : 0;
        cost[id][0] = std::min(leafCost, internalCost);
        split[id][0] = 0;
        for (int j = 2; j <= 8; j++) {
            if (dist[j] < cost[id][j - 2]) { cost[id][j - 1] = dist[j]; split[id][j - 1] = arg[j]; }
            else { cost[id][j - 1] = cost[id][j - 2]; split[id][j - 1] = 0; }
        }
    }
    /* the slots of the wide node rooted at binary node r: subtree c with j slots either splits
     * into its children (split[c][j-1] of them to the left) or, with one slot or none to gain,
     * takes one slot */
    struct Slot { int32_t bnode; bool leaf; };
    auto slots_of = [&](int32_t r, std::vector<Slot>& out) {
        out.clear();
        struct Item { int32_t c; int j; };
        Item st[16];
        int sp = 0;
        const BNode& rn = B.nodes[r];
        if (rn.count > 0) { out.push_back({r, true}); return; }
        /* the root's own 8 slots: the best distribution between its two children */
        float best = INFINITY;
        int bk = 1;
        for (int k = 1; k < 8; k++) {
            const float c = cost[rn.left][k - 1] + cost[rn.right][8 - k - 1];
            if (c < best) { best = c; bk = k; }
        }
        st[sp++] = {rn.right, 8 - bk};
        st[sp++] = {rn.left, bk};
        while (sp > 0) {
            Item it = st[--sp];
            int j = it.j;
            while (j > 1 && split[it.c][j - 1] == 0) j--;
            if (j == 1) { out.push_back({it.c, asLeaf[it.c] != 0}); continue; }
            const int k = split[it.c][j - 1];
            const BNode& cn = B.nodes[it.c];
            st[sp++] = {cn.right, j - k};
            st[sp++] = {cn.left, k};
        }
    };

    struct Task { uint32_t wide; int32_t bnode; uint32_t depth; };
    std::vector<Task> queue;
    queue.push_back({0, 0, 1});
    std::vector<Slot> slotList;
    for (size_t qi = 0; qi < queue.size(); qi++) {
        Task task = queue[qi];
        const BNode& bn = B.nodes[task.bnode];
        slots_of(task.bnode, slotList);
        std::vector<int32_t> ch;
        std::vector<bool> chLeaf;
        for (const Slot& sl : slotList) { ch.push_back(sl.bnode); chLeaf.push_back(sl.leaf); }
        /* slot order: slot s holds the child nearest along the diagonal of octant s */
        float pc[3];
        for (int a = 0; a < 3; a++) pc[a] = 0.5f * (bn.box.lo[a] + bn.box.hi[a]);
        int childAt[8];
        bool leafAt[8] = {false};
        bool slotUsed[8] = {false}, childUsed[8] = {false};
        for (int s = 0; s < 8; s++) childAt[s] = -1;
        for (size_t round = 0; round < ch.size(); round++) {
            float bestC = INFINITY;
            int bs = -1, bi = -1;
            for (int s = 0; s < 8; s++) {
                if (slotUsed[s]) continue;
                for (size_t i = 0; i < ch.size(); i++) {
                    if (childUsed[i]) continue;
                    const Box& cb = B.nodes[ch[i]].box;
                    float c = 0.0f;
                    for (int a = 0; a < 3; a++) {
                        float dir = (s >> a) & 1 ? -1.0f : 1.0f;
                        c += dir * (0.5f * (cb.lo[a] + cb.hi[a]) - pc[a]);
                    }
                    if (c < bestC) { bestC = c; bs = s; bi = (int)i; }
                }
            }
            slotUsed[bs] = true; childUsed[bi] = true; childAt[bs] = ch[bi]; leafAt[bs] = chLeaf[bi];
        }
        uint32_t* W = nullptr;
        uint32_t internalCount = 0, imask = 0;
        for (int s = 0; s < 8; s++)
            if (childAt[s] >= 0 && !leafAt[s]) { imask |= 1u << s; internalCount++; }
        uint32_t childBase = (uint32_t)(out.nodes.size() / GRIS_NODE_WORDS);
        uint8_t meta[8] = {0};
        uint32_t rank = 0;
        for (int s = 0; s < 8; s++) {
            if (childAt[s] < 0 || !(imask & (1u << s))) continue;
            meta[s] = (uint8_t)(0x80u | rank);
            queue.push_back({childBase + rank, childAt[s], task.depth + 1});
            out.maxDepth = std::max(out.maxDepth, task.depth + 1);
            rank++;
        }
        out.nodes.resize(out.nodes.size() + (size_t)internalCount * GRIS_NODE_WORDS, 0u);
        uint32_t triBase = (uint32_t)(out.tris.size() / GRIS_TRI_FLOATS);
        uint32_t triOff = 0;
        for (int s = 0; s < 8; s++) {
            if (childAt[s] < 0 || (imask & (1u << s))) continue;
            const uint32_t lfirst = subFirst[childAt[s]], lcount = subCount[childAt[s]];
            meta[s] = (uint8_t)(0x80u | (lcount << 5) | triOff);
            for (uint32_t i = 0; i < lcount; i++) {
                uint32_t t = B.idx[lfirst + i];
                const float* p = &v[(size_t)t * 9];
                float rec[12] = {p[0], p[1], p[2], 0.0f, p[3] - p[0], p[4] - p[1], p[5] - p[2], 0.0f,
                                 p[6] - p[0], p[7] - p[1], p[8] - p[2], 0.0f};
                uint32_t inst = ids[(size_t)t * 2], tri = ids[(size_t)t * 2 + 1];
                memcpy(&rec[3], &inst, 4);
                memcpy(&rec[7], &tri, 4);
                out.tris.insert(out.tris.end(), rec, rec + 12);
            }
            triOff += lcount;
        }
        /* quantised child boxes */
        double clo[3][8], chi[3][8];
        bool valid[8];
        double nodeLo[3] = {INFINITY, INFINITY, INFINITY}, nodeHi[3] = {-INFINITY, -INFINITY, -INFINITY};
        float maxExt = 0.0f;
        for (int a = 0; a < 3; a++) maxExt = std::max(maxExt, bn.box.hi[a] - bn.box.lo[a]);
        for (int s = 0; s < 8; s++) {
            valid[s] = childAt[s] >= 0;
            if (!valid[s]) continue;
            const Box& cb = B.nodes[childAt[s]].box;
            for (int a = 0; a < 3; a++) {
                double mag = std::max(fabs((double)cb.lo[a]), fabs((double)cb.hi[a]));
                double pad = 1e-5 * (double)maxExt + 1e-6 * mag + 1e-30;
                clo[a][s] = (double)cb.lo[a] - pad;
                chi[a][s] = (double)cb.hi[a] + pad;
                nodeLo[a] = std::min(nodeLo[a], clo[a][s]);
                nodeHi[a] = std::max(nodeHi[a], chi[a][s]);
            }
        }
        W = &out.nodes[(size_t)task.wide * GRIS_NODE_WORDS];
        uint32_t ew = 0;
        Quant q[3];
        for (int a = 0; a < 3; a++) {
            float pf = (float)nodeLo[a];
            if ((double)pf > nodeLo[a]) pf = nextafterf(pf, -INFINITY);
            double ext = nodeHi[a] - (double)pf;
            int e = ext > 0.0 ? (int)ceil(log2(ext / 255.0)) : -126;
            if (e < -126) e = -126;
            while (!quantise_axis(pf, e, clo[a], chi[a], valid, q[a])) {
                e++;
                /* scales up to 2^28 keep scale / |direction| finite for every ray (|1/d| <= 1e30),
                 * which the walk's near/far plane selection needs (boxes up to 6.8e10 wide) */
                if (e > 28) { err = "BVH quantisation failed (scene extent too large)"; return false; }
            }
            memcpy(&W[a], &pf, 4);
            ew |= q[a].e << (8 * a);
        }
        W[3] = ew | (imask << 24);
        W[4] = childBase;
        W[5] = triBase;
        W[6] = (uint32_t)meta[0] | ((uint32_t)meta[1] << 8) | ((uint32_t)meta[2] << 16) | ((uint32_t)meta[3] << 24);
        W[7] = (uint32_t)meta[4] | ((uint32_t)meta[5] << 8) | ((uint32_t)meta[6] << 16) | ((uint32_t)meta[7] << 24);
        for (int a = 0; a < 3; a++) {
            W[8 + 2 * a] = q[a].lo[0] | (q[a].lo[1] << 8) | (q[a].lo[2] << 16) | ((uint32_t)q[a].lo[3] << 24);
            W[9 + 2 * a] = q[a].lo[4] | (q[a].lo[5] << 8) | (q[a].lo[6] << 16) | ((uint32_t)q[a].lo[7] << 24);
            W[14 + 2 * a] = q[a].hi[0] | (q[a].hi[1] << 8) | (q[a].hi[2] << 16) | ((uint32_t)q[a].hi[3] << 24);
            W[15 + 2 * a] = q[a].hi[4] | (q[a].hi[5] << 8) | (q[a].hi[6] << 16) | ((uint32_t)q[a].hi[7] << 24);
        }
    }
    if (out.maxDepth > GRIS_BVH_STACK) { err = "BVH deeper than the traversal stack"; return false; }
    out.buildSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return true;
}

}  // namespace grisrt
