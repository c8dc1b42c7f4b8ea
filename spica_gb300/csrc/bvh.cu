// bvh.cu -- device build of the compressed 8-wide BVH.
//
// Replaces the reference's serial binary SAH build (accelerators/bvh.cc:150-237,
// BVHAccel::constructRec) with a data-parallel one on the GPU:
//   1. per-triangle bounds and centroid bounds              (k_prim_bounds)
//   2. 63-bit Morton codes of the centroids under a large-triangle bit, radix sort
//                                                            (k_morton + cub)
//   3. binary tree by parallel locally-ordered clustering   (k_leaf_bounds, k_ploc_*)
//      -- Meister and Bittner, "Parallel Locally-Ordered Clustering for Bounding
//         Volume Hierarchy Construction" (IEEE TVCG 2018): clusters start as the
//         triangles in code order; each round every cluster finds the neighbour
//         within kPlocRadius positions whose merged box has the least surface area,
//         mutual nearest neighbours merge into a new node, and the clusters are
//         compacted in order, until one is left
//   4. SAH-optimal choice of the wide tree, bottom-up over the clustering rounds
//      (k_dp_round) -- the dynamic programme of Ylitie, Karras and Laine,
//      "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs"
//      (HPG 2017): for every binary node, the least SAH cost of spreading 1..8
//      child slots over its subtree, where a node is a leaf (at most 3 triangles),
//      a wide node, or passes slots on to its two children
//   5. top-down collapse into 8-wide nodes, level by level  (k_collapse),
//      following those decisions
//      Children are placed in slots by a greedy octant assignment so that the
//      traversal's slot order s ^ (7 - octant) runs roughly front to back, their
//      boxes are quantised conservatively to 8 bits on the node's grid, and leaf
//      triangles are copied into leaf order as (v0, v1, v2) records.
// The triangle set, and so the closest hit of every ray, is the reference's; only
// the tree differs.  Its build is deterministic (no atomics decide structure).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cstdio>
#include <vector>

#include "bvh.cuh"

namespace spgpu {

namespace {

constexpr int kLeafMax = 3;   // triangles a wide-node leaf may hold

__device__ __forceinline__ void atomicMinFloat(float *a, float v) {
    if (v >= 0.0f) atomicMin(reinterpret_cast<int *>(a), __float_as_int(v));
    else atomicMax(reinterpret_cast<unsigned int *>(a), __float_as_uint(v));
}
__device__ __forceinline__ void atomicMaxFloat(float *a, float v) {
    if (v >= 0.0f) atomicMax(reinterpret_cast<int *>(a), __float_as_int(v));
    else atomicMin(reinterpret_cast<unsigned int *>(a), __float_as_uint(v));
}

// scene bounds [0..5] and centroid bounds [6..11]
__global__ void k_prim_bounds(const float *__restrict__ verts, int n, float *__restrict__ bounds) {
    float lo[6], hi[6];
    for (int k = 0; k < 6; k++) {
        lo[k] = 3.0e38f;
        hi[k] = -3.0e38f;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float *v = verts + 9 * static_cast<int64_t>(i);
        for (int a = 0; a < 3; a++) {
            const float mn = fminf(v[a], fminf(v[3 + a], v[6 + a]));
            const float mx = fmaxf(v[a], fmaxf(v[3 + a], v[6 + a]));
            lo[a] = fminf(lo[a], mn);
            hi[a] = fmaxf(hi[a], mx);
            const float c = 0.5f * (mn + mx);
            lo[3 + a] = fminf(lo[3 + a], c);
            hi[3 + a] = fmaxf(hi[3 + a], c);
        }
    }
    for (int k = 0; k < 6; k++) {
        for (int off = 16; off > 0; off >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], off));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], off));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int a = 0; a < 3; a++) {
            atomicMinFloat(&bounds[a], lo[a]);
            atomicMaxFloat(&bounds[3 + a], hi[a]);
            atomicMinFloat(&bounds[6 + a], lo[3 + a]);
            atomicMaxFloat(&bounds[9 + a], hi[3 + a]);
        }
    }
}

__device__ __forceinline__ uint64_t spread21(uint32_t x) {
    uint64_t v = x & 0x1FFFFFu;
    v = (v | (v << 32)) & 0x1F00000000FFFFull;
    v = (v | (v << 16)) & 0x1F0000FF0000FFull;
    v = (v | (v << 8)) & 0x100F00F00F00F00Full;
    v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// Sort key: bit 63 marks a large triangle (box diagonal above 1/8 of the scene's), bits
// 0-62 are the 63-bit Morton code of its box centre.  The size bit is the extended
// Morton code idea of Vinkler, Bittner and Havran ("Extended Morton codes for high
// performance bounding volume hierarchy construction", HPG 2017) reduced to one class:
// large triangles (a floor quad, room walls) sort after all others, so the clustering,
// which merges only within a window of this order, joins them with each other first and
// with the rest near the root, instead of leaving them deep among small ones where every
// ancestor's box would span them.
constexpr float kLargeTriangle = 1.0f / 8.0f;

__global__ void k_morton(const float *__restrict__ verts, int n, const float *__restrict__ bounds,
                         uint64_t *__restrict__ keys, uint32_t *__restrict__ vals) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *v = verts + 9 * static_cast<int64_t>(i);
    uint32_t q[3];
    float d2 = 0.0f, s2 = 0.0f;
    for (int a = 0; a < 3; a++) {
        const float mn = fminf(v[a], fminf(v[3 + a], v[6 + a])), mx = fmaxf(v[a], fmaxf(v[3 + a], v[6 + a]));
        const float c = 0.5f * (mn + mx);
        const float lo = bounds[6 + a], ext = bounds[9 + a] - bounds[6 + a];
        const float u = ext > 0.0f ? (c - lo) / ext : 0.5f;
        q[a] = static_cast<uint32_t>(fminf(fmaxf(u * 2097152.0f, 0.0f), 2097151.0f));
        d2 += (mx - mn) * (mx - mn);
        s2 += (bounds[3 + a] - bounds[a]) * (bounds[3 + a] - bounds[a]);
    }
    const uint64_t large = d2 > kLargeTriangle * kLargeTriangle * s2 ? 1ull << 63 : 0ull;
    keys[i] = large | (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
    vals[i] = static_cast<uint32_t>(i);
}

__device__ __forceinline__ float areaOf(float4 lo, float4 hi) {
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

// ---------------------------------------------------------------- clustering
constexpr int kPlocRadius = 32;   // neighbours searched on each side, in code order
constexpr int kPlocBlock = 256;

// leaves: node n-1+j is the j-th triangle in code order
// SAH weights of the wide tree: a wide-node visit, a triangle test.  Equal weights were
// measured best for this traversal (triangle weight 0.3 / 0.6 / 1.0 / 1.5: 884 / 892 /
// 900 / 887 M path samples/s on the 1080p render; the 1M-triangle microbench also peaks
// at 1.0)
constexpr float kCostNode = 1.0f, kCostTri = 1.0f;

// per binary node: cost[8 * node + j - 1] = least SAH cost of its subtree over j child
// slots; split[8 * node + j - 1] = slots given to the left child (0: the node itself
// takes one slot); split of j = 8 before that choice is the node's own split as a wide
// node (wideSplit); leaf[node]: the node itself is cheaper as a leaf than as a wide node
struct DpArgs {
    float *cost;
    uint8_t *split;
    uint8_t *wideSplit;
    uint8_t *leaf;
};

__global__ void k_leaf_bounds(const float *__restrict__ verts, const uint32_t *__restrict__ order, int n,
                              float4 *bmin, float4 *bmax, int *count, int *clusters, DpArgs D) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const float *v = verts + 9 * static_cast<int64_t>(order[j]);
    const int node = n - 1 + j;
    const float4 lo = make_float4(fminf(v[0], fminf(v[3], v[6])), fminf(v[1], fminf(v[4], v[7])),
                                  fminf(v[2], fminf(v[5], v[8])), 0.0f);
    const float4 hi = make_float4(fmaxf(v[0], fmaxf(v[3], v[6])), fmaxf(v[1], fmaxf(v[4], v[7])),
                                  fmaxf(v[2], fmaxf(v[5], v[8])), 0.0f);
    bmin[node] = lo;
    bmax[node] = hi;
    count[node] = 1;
    clusters[j] = node;
    const float2 dx = make_float2(hi.x - lo.x, hi.y - lo.y);
    const float c = kCostTri * 2.0f * (dx.x * dx.y + dx.y * (hi.z - lo.z) + (hi.z - lo.z) * dx.x);
    for (int k = 0; k < 8; k++) {
        D.cost[8 * static_cast<int64_t>(node) + k] = c;
        D.split[8 * static_cast<int64_t>(node) + k] = 0;
    }
    D.leaf[node] = 1;
}

// nearest neighbour of each cluster: least surface area of the merged box among the
// clusters within kPlocRadius positions (ties: the lower position); the window's boxes
// are staged in shared memory
__global__ void __launch_bounds__(kPlocBlock) k_ploc_nn(const int *__restrict__ clusters, int m,
                                                        const float4 *__restrict__ bmin,
                                                        const float4 *__restrict__ bmax, int *nn) {
    __shared__ float4 slo[kPlocBlock + 2 * kPlocRadius], shi[kPlocBlock + 2 * kPlocRadius];
    const int base = blockIdx.x * kPlocBlock - kPlocRadius;
    for (int k = threadIdx.x; k < kPlocBlock + 2 * kPlocRadius; k += kPlocBlock) {
        const int p = base + k;
        if (p >= 0 && p < m) {
            const int c = clusters[p];
            slo[k] = bmin[c];
            shi[k] = bmax[c];
        }
    }
    __syncthreads();
    const int i = blockIdx.x * kPlocBlock + threadIdx.x;
    if (i >= m) return;
    const int li = threadIdx.x + kPlocRadius;
    const float4 lo = slo[li], hi = shi[li];
    float best = 3.0e38f;
    int bestJ = -1;
    for (int d = -kPlocRadius; d <= kPlocRadius; d++) {
        const int j = i + d;
        if (d == 0 || j < 0 || j >= m) continue;
        const float4 a = slo[li + d], b = shi[li + d];
        const float area = areaOf(make_float4(fminf(lo.x, a.x), fminf(lo.y, a.y), fminf(lo.z, a.z), 0.0f),
                                  make_float4(fmaxf(hi.x, b.x), fmaxf(hi.y, b.y), fmaxf(hi.z, b.z), 0.0f));
        if (area < best) {
            best = area;
            bestJ = j;
        }
    }
    nn[i] = bestJ;
}

// a cluster leads a merge when it and its neighbour chose each other and it comes
// first; it survives the round unless it is the second of such a pair
__global__ void k_ploc_flags(const int *__restrict__ nn, int m, int *lead, int *keep) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int j = nn[i];
    const bool mutual = j >= 0 && nn[j] == i;
    lead[i] = mutual && i < j ? 1 : 0;
    keep[i] = mutual && i > j ? 0 : 1;
}

// merged nodes take ids top - leadOffset (descending, so the last merge, the root, is
// node 0); survivors are compacted in order
__global__ void k_ploc_merge(const int *__restrict__ clusters, int m, const int *__restrict__ nn,
                             const int *__restrict__ lead, const int *__restrict__ leadOff,
                             const int *__restrict__ keep, const int *__restrict__ keepOff, int top, int2 *child,
                             float4 *bmin, float4 *bmax, int *count, int *next) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || !keep[i]) return;
    int node = clusters[i];
    if (lead[i]) {
        const int a = node, b = clusters[nn[i]];
        const int id = top - leadOff[i];
        child[id] = make_int2(a, b);
        const float4 a0 = bmin[a], a1 = bmax[a], b0 = bmin[b], b1 = bmax[b];
        bmin[id] = make_float4(fminf(a0.x, b0.x), fminf(a0.y, b0.y), fminf(a0.z, b0.z), 0.0f);
        bmax[id] = make_float4(fmaxf(a1.x, b1.x), fmaxf(a1.y, b1.y), fmaxf(a1.z, b1.z), 0.0f);
        count[id] = count[a] + count[b];
        node = id;
    }
    next[keepOff[i]] = node;
}


// one clustering round's nodes (ids lo..hi; their children are from earlier rounds)
__global__ void k_dp_round(const int2 *__restrict__ child, const int *__restrict__ count,
                           const float4 *__restrict__ bmin, const float4 *__restrict__ bmax, int lo, int hi,
                           DpArgs D, int kLeafLimit) {
    const int id = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (id > hi) return;
    const int2 c = child[id];
    const float *CL = D.cost + 8 * static_cast<int64_t>(c.x), *CR = D.cost + 8 * static_cast<int64_t>(c.y);
    float S[9];
    uint8_t K[9];
    S[1] = 3.0e38f;
    K[1] = 0;
    for (int j = 2; j <= 8; j++) {
        float best = 3.0e38f;
        uint8_t bk = 1;
        for (int k = 1; k < j; k++) {
            const float v = CL[k - 1] + CR[j - k - 1];
            if (v < best) {
                best = v;
                bk = static_cast<uint8_t>(k);
            }
        }
        S[j] = best;
        K[j] = bk;
        if (j > 2 && S[j - 1] <= S[j]) {   // fewer slots may be cheaper: keep that split
            S[j] = S[j - 1];
            K[j] = K[j - 1];
        }
    }
    const float A = areaOf(bmin[id], bmax[id]);
    const float cInternal = kCostNode * A + S[8];
    const float cLeaf = count[id] <= kLeafLimit ? kCostTri * A * static_cast<float>(count[id]) : 3.0e38f;
    const bool asLeaf = cLeaf <= cInternal;
    const float C = asLeaf ? cLeaf : cInternal;
    float *out = D.cost + 8 * static_cast<int64_t>(id);
    uint8_t *sp = D.split + 8 * static_cast<int64_t>(id);
    out[0] = C;
    sp[0] = 0;
    for (int j = 2; j <= 8; j++) {
        const bool self = C <= S[j];
        out[j - 1] = self ? C : S[j];
        sp[j - 1] = self ? 0 : K[j];
    }
    D.wideSplit[id] = K[8];
    D.leaf[id] = asLeaf ? 1 : 0;
}

struct CollapseArgs {
    const float *verts;
    const uint32_t *order;
    const int *tri_mat;
    const int *tri_light;
    int n;
    const int2 *child;
    const int *count;   // triangles under each binary node
    DpArgs dp;
    const float4 *bmin;
    const float4 *bmax;
    WideNode *nodes;
    TriRecord *tris;
    int2 *slot_shade;
    int *counters;   // [0] wide nodes allocated, [1] triangles placed, [2] next-level items
};

// the triangles (code-order positions) under binary node b, at most kLeafMax of them,
// left subtree first
__device__ __forceinline__ int leafPrims(const CollapseArgs &A, int b, int *pos) {
    int stack[2 * kLeafMax], sp = 0, k = 0;
    stack[sp++] = b;
    while (sp > 0 && k < kLeafMax) {
        const int x = stack[--sp];
        if (x >= A.n - 1) {
            pos[k++] = x - (A.n - 1);
        } else if (sp + 2 <= 2 * kLeafMax) {
            const int2 c = A.child[x];
            stack[sp++] = c.y;
            stack[sp++] = c.x;
        }
    }
    return k;
}

// one thread per wide node of the current level; items are (binary node, wide node)
__global__ void k_collapse(CollapseArgs A, const int2 *__restrict__ items, int nitems, int2 *__restrict__ next) {
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= nitems) return;
    const int b = items[it].x, w = items[it].y;
    const bool rootLeaf = b >= A.n - 1;   // single-triangle scene
    int C[8];
    int nc = 0;
    if (rootLeaf) {
        C[nc++] = b;
    } else {
        // the 8 slots of wide node b, spread as the SAH programme decided: (node, slots)
        int stN[8], stJ[8], sp = 0;
        const int k0 = A.dp.wideSplit[b];
        stN[sp] = A.child[b].y;
        stJ[sp++] = 8 - k0;
        stN[sp] = A.child[b].x;
        stJ[sp++] = k0;
        while (sp > 0 && nc < 8) {
            const int x = stN[--sp], j = stJ[sp];
            const int k = (x < A.n - 1 && j > 1) ? A.dp.split[8 * static_cast<int64_t>(x) + j - 1] : 0;
            if (k == 0 || sp + 2 > 8) {
                C[nc++] = x;
            } else {
                const int2 cc = A.child[x];
                stN[sp] = cc.y;
                stJ[sp++] = j - k;
                stN[sp] = cc.x;
                stJ[sp++] = k;
            }
        }
    }
    // node box
    float3 lo = mk(3.0e38f, 3.0e38f, 3.0e38f), hi = mk(-3.0e38f, -3.0e38f, -3.0e38f);
    for (int k = 0; k < nc; k++) {
        lo = fminf3(lo, xyz(A.bmin[C[k]]));
        hi = fmaxf3(hi, xyz(A.bmax[C[k]]));
    }
    const float3 ctr = (lo + hi) * 0.5f;
    // greedy slot assignment: child whose centroid offset lies in octant o prefers slot o
    int slotOf[8];
    bool usedSlot[8] = {false, false, false, false, false, false, false, false};
    bool done[8] = {false, false, false, false, false, false, false, false};
    float cost[8][8];
    for (int k = 0; k < nc; k++) {
        const float3 c = (xyz(A.bmin[C[k]]) + xyz(A.bmax[C[k]])) * 0.5f - ctr;
        for (int s = 0; s < 8; s++) {
            const float3 sg = mk((s & 1) ? -1.0f : 1.0f, (s & 2) ? -1.0f : 1.0f, (s & 4) ? -1.0f : 1.0f);
            cost[k][s] = -dot(c, sg);
        }
    }
    for (int r = 0; r < nc; r++) {
        float bc = 3.0e38f;
        int bk = -1, bs = -1;
        for (int k = 0; k < nc; k++) {
            if (done[k]) continue;
            for (int s = 0; s < 8; s++) {
                if (usedSlot[s]) continue;
                if (cost[k][s] < bc) {
                    bc = cost[k][s];
                    bk = k;
                    bs = s;
                }
            }
        }
        done[bk] = true;
        usedSlot[bs] = true;
        slotOf[bk] = bs;
    }
    // classify children: internal (wide node) or leaf (<= 3 triangles)
    int slotChild[8];
    for (int s = 0; s < 8; s++) slotChild[s] = -1;
    for (int k = 0; k < nc; k++) slotChild[slotOf[k]] = C[k];
    uint32_t imask = 0;
    int nInt = 0, nTri = 0;
    for (int s = 0; s < 8; s++) {
        const int c = slotChild[s];
        if (c < 0) continue;
        const int count = A.count[c];
        if (c < A.n - 1 && (count > kLeafMax || !A.dp.leaf[c])) {
            imask |= 1u << s;
            nInt++;
        } else {
            nTri += count;
        }
    }
    const int childBase = nInt ? atomicAdd(&A.counters[0], nInt) : 0;
    const int triBase = nTri ? atomicAdd(&A.counters[1], nTri) : 0;
    const int itemBase = nInt ? atomicAdd(&A.counters[2], nInt) : 0;

    WideNode node;
    node.px = lo.x;
    node.py = lo.y;
    node.pz = lo.z;
    int e[3];
    const float ext[3] = {hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
    for (int a = 0; a < 3; a++) {
        int ex = -126;
        if (ext[a] > 0.0f) {
            frexpf(ext[a] / 255.0f, &ex);   // ext/255 = m 2^ex, m in [0.5, 1)
            ex = max(ex, -126);
            for (int g = 0; g < 4 && ldexpf(255.0f, ex) < ext[a]; g++) ex++;
        }
        e[a] = ex;
    }
    node.ex = static_cast<uint8_t>(e[0] + 127);
    node.ey = static_cast<uint8_t>(e[1] + 127);
    node.ez = static_cast<uint8_t>(e[2] + 127);
    node.imask = static_cast<uint8_t>(imask);
    node.child_base = static_cast<uint32_t>(childBase);
    node.tri_base = static_cast<uint32_t>(triBase);
    const double p[3] = {lo.x, lo.y, lo.z};
    int rank = 0, triOff = 0;
    for (int s = 0; s < 8; s++) {
        const int c = slotChild[s];
        if (c < 0) {
            node.meta[s] = 0;
            node.qlo_x[s] = node.qlo_y[s] = node.qlo_z[s] = 0;
            node.qhi_x[s] = node.qhi_y[s] = node.qhi_z[s] = 0;
            continue;
        }
        const float4 cl = A.bmin[c], ch = A.bmax[c];
        const double clo[3] = {cl.x, cl.y, cl.z}, chi[3] = {ch.x, ch.y, ch.z};
        uint8_t ql[3], qh[3];
        for (int a = 0; a < 3; a++) {
            const double sc = ldexp(1.0, e[a]);
            double l = floor((clo[a] - p[a]) / sc), h = ceil((chi[a] - p[a]) / sc);
            l = fmin(fmax(l, 0.0), 255.0);
            h = fmin(fmax(h, 0.0), 255.0);
            ql[a] = static_cast<uint8_t>(l);
            qh[a] = static_cast<uint8_t>(h);
        }
        node.qlo_x[s] = ql[0];
        node.qlo_y[s] = ql[1];
        node.qlo_z[s] = ql[2];
        node.qhi_x[s] = qh[0];
        node.qhi_y[s] = qh[1];
        node.qhi_z[s] = qh[2];
        if (imask & (1u << s)) {
            node.meta[s] = static_cast<uint8_t>(0x20 | (24 + s));
            next[itemBase + rank] = make_int2(c, childBase + rank);
            rank++;
        } else {
            int pos[kLeafMax];
            const int count = leafPrims(A, c, pos);
            node.meta[s] = static_cast<uint8_t>((((1u << count) - 1u) << 5) | static_cast<uint32_t>(triOff));
            for (int q = 0; q < count; q++) {
                const uint32_t prim = A.order[pos[q]];
                const float *v = A.verts + 9 * static_cast<int64_t>(prim);
                TriRecord r;
                r.v0 = make_float4(v[0], v[1], v[2], __int_as_float(static_cast<int>(prim)));
                r.v1 = make_float4(v[3], v[4], v[5], 0.0f);
                r.v2 = make_float4(v[6], v[7], v[8], 0.0f);
                A.tris[triBase + triOff + q] = r;
                A.slot_shade[triBase + triOff + q] =
                    make_int2(A.tri_mat ? A.tri_mat[prim] : 0, A.tri_light ? A.tri_light[prim] : -1);
            }
            triOff += count;
        }
    }
    A.nodes[w] = node;
}

template <class T>
T *dalloc(size_t n) {
    T *p = nullptr;
    if (cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) return nullptr;
    return p;
}

}  // namespace

void freeWideBVH(DeviceBVH *b) {
    cudaFree(b->nodes);
    cudaFree(b->tris);
    cudaFree(b->slot_shade);
    *b = DeviceBVH{};
}

int buildWideBVH(const float *d_verts, int n, const int *d_tri_mat, const int *d_tri_light, DeviceBVH *out,
                 cudaStream_t stream, char *err, size_t errlen) {
    freeWideBVH(out);
    if (n <= 0) {
        snprintf(err, errlen, "buildWideBVH: empty scene");
        return -2;
    }
    const int nNodes = 2 * n - 1;
    float *d_bounds = dalloc<float>(12);
    uint64_t *keys[2] = {dalloc<uint64_t>(n), dalloc<uint64_t>(n)};
    uint32_t *vals[2] = {dalloc<uint32_t>(n), dalloc<uint32_t>(n)};
    int2 *child = dalloc<int2>(n);
    int *count = dalloc<int>(nNodes);
    int *clusters[2] = {dalloc<int>(n), dalloc<int>(n)};
    int *nn = dalloc<int>(n), *lead = dalloc<int>(n), *keep = dalloc<int>(n);
    int *leadOff = dalloc<int>(n), *keepOff = dalloc<int>(n);
    float4 *bmin = dalloc<float4>(nNodes);
    float4 *bmax = dalloc<float4>(nNodes);
    DpArgs dp{dalloc<float>(8 * static_cast<size_t>(nNodes)), dalloc<uint8_t>(8 * static_cast<size_t>(nNodes)),
              dalloc<uint8_t>(n), dalloc<uint8_t>(nNodes)};
    int2 *items[2] = {dalloc<int2>(n), dalloc<int2>(n)};
    int *counters = dalloc<int>(4);
    out->nodes = dalloc<WideNode>(n);
    out->tris = dalloc<TriRecord>(n);
    out->slot_shade = dalloc<int2>(n);
    int rc = 0;
    void *tmp = nullptr, *scanTmp = nullptr;
    size_t tmpBytes = 0, scanBytes = 0;
    auto fail = [&](const char *what, cudaError_t e) {
        snprintf(err, errlen, "buildWideBVH: %s: %s", what, cudaGetErrorString(e));
        rc = -3;
    };
    if (!d_bounds || !keys[0] || !keys[1] || !vals[0] || !vals[1] || !child || !count || !clusters[0] ||
        !clusters[1] || !nn || !lead || !keep || !leadOff || !keepOff || !bmin || !bmax || !dp.cost || !dp.split ||
        !dp.wideSplit || !dp.leaf || !items[0] || !items[1] ||
        !counters || !out->nodes || !out->tris || !out->slot_shade) {
        snprintf(err, errlen, "buildWideBVH: device allocation failed for %d triangles", n);
        rc = -4;
    }
    if (rc == 0) {
        const float init[12] = {3e38f, 3e38f, 3e38f, -3e38f, -3e38f, -3e38f,
                                3e38f, 3e38f, 3e38f, -3e38f, -3e38f, -3e38f};
        cudaMemcpyAsync(d_bounds, init, sizeof(init), cudaMemcpyHostToDevice, stream);
        cudaMemsetAsync(counters, 0, sizeof(int) * 4, stream);
        const int T = 256;
        k_prim_bounds<<<std::min((n + T - 1) / T, 1216), T, 0, stream>>>(d_verts, n, d_bounds);
        k_morton<<<(n + T - 1) / T, T, 0, stream>>>(d_verts, n, d_bounds, keys[0], vals[0]);
        cub::DoubleBuffer<uint64_t> kb(keys[0], keys[1]);
        cub::DoubleBuffer<uint32_t> vb(vals[0], vals[1]);
        cub::DeviceRadixSort::SortPairs(nullptr, tmpBytes, kb, vb, n, 0, 64, stream);
        cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, lead, leadOff, n, stream);
        if (cudaMalloc(&tmp, tmpBytes) != cudaSuccess || cudaMalloc(&scanTmp, scanBytes) != cudaSuccess) {
            snprintf(err, errlen, "buildWideBVH: sort scratch allocation failed");
            rc = -4;
        } else {
            cub::DeviceRadixSort::SortPairs(tmp, tmpBytes, kb, vb, n, 0, 64, stream);
            const uint64_t *sk = kb.Current();
            const uint32_t *order = vb.Current();
            (void)sk;
            k_leaf_bounds<<<(n + T - 1) / T, T, 0, stream>>>(d_verts, order, n, bmin, bmax, count, clusters[0],
                                                                 dp);
            // clustering rounds: m clusters, merged nodes numbered downwards from top
            int m = n, top = n - 2, cl = 0, rounds = 0;
            std::vector<int2> roundIds;   // node ids created by each round, in round order
            while (m > 1 && rc == 0) {
                const int B = (m + kPlocBlock - 1) / kPlocBlock;
                k_ploc_nn<<<B, kPlocBlock, 0, stream>>>(clusters[cl], m, bmin, bmax, nn);
                k_ploc_flags<<<B, kPlocBlock, 0, stream>>>(nn, m, lead, keep);
                cub::DeviceScan::ExclusiveSum(scanTmp, scanBytes, lead, leadOff, m, stream);
                cub::DeviceScan::ExclusiveSum(scanTmp, scanBytes, keep, keepOff, m, stream);
                k_ploc_merge<<<B, kPlocBlock, 0, stream>>>(clusters[cl], m, nn, lead, leadOff, keep, keepOff, top,
                                                           child, bmin, bmax, count, clusters[cl ^ 1]);
                int tail[4] = {0, 0, 0, 0};   // leadOff, lead, keepOff, keep of the last cluster
                cudaMemcpyAsync(&tail[0], leadOff + m - 1, sizeof(int), cudaMemcpyDeviceToHost, stream);
                cudaMemcpyAsync(&tail[1], lead + m - 1, sizeof(int), cudaMemcpyDeviceToHost, stream);
                cudaMemcpyAsync(&tail[2], keepOff + m - 1, sizeof(int), cudaMemcpyDeviceToHost, stream);
                cudaMemcpyAsync(&tail[3], keep + m - 1, sizeof(int), cudaMemcpyDeviceToHost, stream);
                const cudaError_t e = cudaStreamSynchronize(stream);
                if (e != cudaSuccess) {
                    fail("clustering", e);
                    break;
                }
                const int merges = tail[0] + tail[1];
                if (merges > 0) roundIds.push_back(make_int2(top - merges + 1, top));
                top -= merges;
                m = tail[2] + tail[3];
                cl ^= 1;
                if (merges == 0 || ++rounds > 100000) {
                    snprintf(err, errlen, "buildWideBVH: clustering made no progress");
                    rc = -5;
                }
            }
            if (rc == 0 && n > 1 && top != -1) {
                snprintf(err, errlen, "buildWideBVH: clustering left %d node ids unused", top + 1);
                rc = -5;
            }
            // the SAH programme, one launch per clustering round (children before parents)
            for (const int2 r : roundIds) {
                const int cnt = r.y - r.x + 1;
                k_dp_round<<<(cnt + T - 1) / T, T, 0, stream>>>(child, count, bmin, bmax, r.x, r.y, dp, kLeafMax);
            }
            CollapseArgs A{d_verts, order, d_tri_mat, d_tri_light, n, child, count, dp, bmin, bmax,
                           out->nodes, out->tris, out->slot_shade, counters};
            // root: wide node 0 from binary root (internal 0, or the single leaf)
            const int one = 1;
            const int2 root = make_int2(n > 1 ? 0 : 0 + (n - 1), 0);
            cudaMemcpyAsync(items[0], &root, sizeof(int2), cudaMemcpyHostToDevice, stream);
            cudaMemcpyAsync(counters, &one, sizeof(int), cudaMemcpyHostToDevice, stream);
            int nitems = rc == 0 ? 1 : 0, depth = 0, cur = 0;
            while (nitems > 0) {
                cudaMemsetAsync(counters + 2, 0, sizeof(int), stream);
                k_collapse<<<(nitems + 127) / 128, 128, 0, stream>>>(A, items[cur], nitems, items[cur ^ 1]);
                cudaMemcpyAsync(&nitems, counters + 2, sizeof(int), cudaMemcpyDeviceToHost, stream);
                cudaError_t e = cudaStreamSynchronize(stream);
                if (e != cudaSuccess) {
                    fail("collapse", e);
                    break;
                }
                cur ^= 1;
                depth++;
                if (depth > 4096) {
                    snprintf(err, errlen, "buildWideBVH: collapse did not terminate");
                    rc = -5;
                    break;
                }
            }
            int hostCounters[4] = {0, 0, 0, 0};
            cudaMemcpyAsync(hostCounters, counters, sizeof(hostCounters), cudaMemcpyDeviceToHost, stream);
            cudaError_t e = cudaStreamSynchronize(stream);
            if (e != cudaSuccess && rc == 0) fail("final sync", e);
            if (rc == 0) {
                float hb[12];
                cudaMemcpy(hb, d_bounds, sizeof(hb), cudaMemcpyDeviceToHost);
                out->lo = mk(hb[0], hb[1], hb[2]);
                out->hi = mk(hb[3], hb[4], hb[5]);
                out->n_nodes = hostCounters[0];
                out->ntri = n;
                out->depth = depth;
                if (hostCounters[1] != n) {
                    snprintf(err, errlen, "buildWideBVH: placed %d of %d triangles", hostCounters[1], n);
                    rc = -6;
                } else if (depth > kStackDepth) {
                    snprintf(err, errlen, "buildWideBVH: tree depth %d exceeds the traversal stack (%d)", depth,
                             kStackDepth);
                    rc = -7;
                }
            }
        }
    }
    cudaFree(tmp);
    cudaFree(scanTmp);
    cudaFree(d_bounds);
    cudaFree(keys[0]);
    cudaFree(keys[1]);
    cudaFree(vals[0]);
    cudaFree(vals[1]);
    cudaFree(child);
    cudaFree(count);
    cudaFree(clusters[0]);
    cudaFree(clusters[1]);
    cudaFree(nn);
    cudaFree(lead);
    cudaFree(keep);
    cudaFree(leadOff);
    cudaFree(keepOff);
    cudaFree(bmin);
    cudaFree(bmax);
    cudaFree(dp.cost);
    cudaFree(dp.split);
    cudaFree(dp.wideSplit);
    cudaFree(dp.leaf);
    cudaFree(items[0]);
    cudaFree(items[1]);
    cudaFree(counters);
    if (rc != 0) freeWideBVH(out);
    return rc;
}

}  // namespace spgpu
