// bvh.cuh -- the device-built compressed 8-wide BVH: its host-side handle and the
// traversal routine shared by the ray-batch kernels and the wavefront renderer.
#pragma once

#include <type_traits>

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace spgpu {

// Largest wide-tree depth the traversal kernels accept.  The per-thread stack holds
// one node group per level of the current path: its first kStackShared entries live
// in shared memory, deeper ones spill to a per-thread local array.
constexpr int kStackDepth = 48;
#ifndef SPGPU_STACK_SHARED
#define SPGPU_STACK_SHARED 8
#endif
constexpr int kStackShared = SPGPU_STACK_SHARED;
constexpr int kTraceBlock = 128;

struct DeviceBVH {
    WideNode *nodes = nullptr;     // [n_nodes]
    TriRecord *tris = nullptr;     // [ntri], leaf order
    int2 *slot_shade = nullptr;    // [ntri]: (material, light index or -1) per leaf slot
    int n_nodes = 0;
    int ntri = 0;
    int depth = 0;                 // levels of wide nodes
    float3 lo{0, 0, 0}, hi{0, 0, 0};
};

struct TraceStats {   // per-ray visit counters, for the roofline's algorithmic bytes
    unsigned long long rays;
    unsigned long long nodes;
    unsigned long long tris;
};

// ---------------------------------------------------------------------------
// Traversal of the compressed wide BVH (after Ylitie, Karras and Laine, "Efficient
// Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs", HPG 2017):
// node groups (child base, pending-child bits in visit order, internal mask) on a
// per-thread stack in shared memory, triangle groups tested as soon as a node is
// opened.  Closest hit keeps the reference's acceptance rule t in (eps, tmax]
// (core/triangle.cc:117), so on an exact tie the later-tested triangle wins.
// Any hit returns on the first triangle with t in (eps, tmax].
// Returns false and sets *overflow if the tree is deeper than the stack.
// ---------------------------------------------------------------------------
// byte k of w as an exact float: PRMT assembles 0x4B0000bb (= 2^23 + b), then one FADD
__device__ __forceinline__ float byteToFloat(uint32_t w, int k) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7650u | static_cast<uint32_t>(k))) - 8388608.0f;
}
__device__ __forceinline__ float fmax3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmin3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
// Per 4 child slots at once (one byte each): the bit index of the slot's hit bits in
// the 32-bit hit mask and the bits themselves.  Internal children (meta 0b001_11sss)
// land on bit 24 + (s ^ octInv), leaves on their triangle offset with 1..3 bits.
__device__ __forceinline__ void metaDecode4(uint32_t meta4, uint32_t octInv4, uint32_t *bitIndex4,
                                           uint32_t *childBits4) {
    const uint32_t isInner4 = (meta4 & (meta4 << 1)) & 0x10101010u;   // bit 4 of each internal byte
    const uint32_t innerMask4 = (isInner4 >> 4) * 0xFFu;               // 0xFF where internal
    *bitIndex4 = (meta4 ^ (octInv4 & innerMask4)) & 0x1F1F1F1Fu;
    *childBits4 = (meta4 >> 5) & 0x07070707u;
}

// Every node and triangle index is checked against the tree's sizes and the loop is
// bounded (kMaxVisits), so a malformed tree ends the ray with *overflow set instead of
// reading out of bounds or spinning.
constexpr uint32_t kMaxVisits = 1u << 22;

// Traversal state of one ray, kept in registers between steps so that a warp can
// retire finished rays and start new ones in the middle of a traversal.
struct TraceLane {
    float3 o, d, idir;
    float tmin, tmax, tEps;
    uint32_t octant, octInv;
    uint2 G;          // node group: child base, pending-child bits (visit order) | internal mask
    int sp;
    uint32_t visits;
    int hitSlot;
    float hu, hv;
    bool found;
};

__device__ __forceinline__ void laneInit(TraceLane &L, float3 o, float3 d, float tmin, float tmax,
                                         uint32_t root = 0) {
    L.o = o;
    L.d = d;
    L.idir = mk(d.x == 0.0f ? kInfT : 1.0f / d.x, d.y == 0.0f ? kInfT : 1.0f / d.y, d.z == 0.0f ? kInfT : 1.0f / d.z);
    L.octant = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    L.octInv = 7u - L.octant;
    L.tmin = tmin;
    L.tmax = tmax;
    L.tEps = fmaxf(tmin, kEpsT);
    L.G = make_uint2(root, (1u << (24 + L.octInv)) | 1u);   // the root as slot 0 of a virtual parent
    L.sp = 0;
    L.visits = 0;
    L.hitSlot = -1;
    L.hu = L.hv = 0.0f;
    L.found = false;
}

// One step of the traversal: open the next pending child of the current node group
// (popping a group from the stack first when the current one is exhausted) and test
// the triangles of the leaves it hits.  Returns true when the ray is finished.
template <bool ANY, bool STATS>
__device__ __forceinline__ bool laneStep(TraceLane &L, const WideNode *__restrict__ nodes,
                                         const TriRecord *__restrict__ tris, uint32_t nNodes, uint32_t nTris,
                                         uint2 *__restrict__ stack, int stride, uint2 *spill, uint32_t *nodeCount,
                                         uint32_t *triCount, bool *overflow) {
    if (++L.visits > kMaxVisits) {
        *overflow = true;
        return true;
    }
    if (!(L.G.y & 0xFF000000u)) {
        if (L.sp == 0) return true;
        L.sp--;
        L.G = L.sp < kStackShared ? stack[L.sp * stride] : spill[L.sp - kStackShared];
    }
    const uint32_t key = __ffs(L.G.y >> 24) - 1;
    L.G.y &= ~(1u << (24 + key));
    const uint32_t slot = key ^ L.octInv;
    const uint32_t child = L.G.x + __popc((L.G.y & 0xFFu) & ((1u << slot) - 1u));
    if (child >= nNodes) {
        *overflow = true;
        return true;
    }
    if (L.G.y & 0xFF000000u) {
        if (L.sp >= kStackDepth) {
            *overflow = true;
            return true;
        }
        if (L.sp < kStackShared) stack[L.sp * stride] = L.G;
        else spill[L.sp - kStackShared] = L.G;
        L.sp++;
    }
    if (STATS) (*nodeCount)++;
    const float4 *nodes4 = reinterpret_cast<const float4 *>(nodes);
    const float4 n0 = __ldg(nodes4 + 5 * child + 0);
    const float4 n1 = __ldg(nodes4 + 5 * child + 1);
    const float4 n2 = __ldg(nodes4 + 5 * child + 2);
    const float4 n3 = __ldg(nodes4 + 5 * child + 3);
    const float4 n4 = __ldg(nodes4 + 5 * child + 4);
    const uint32_t ew = __float_as_uint(n0.w);
    const float sx = __uint_as_float((ew & 0xFFu) << 23);
    const float sy = __uint_as_float(((ew >> 8) & 0xFFu) << 23);
    const float sz = __uint_as_float(((ew >> 16) & 0xFFu) << 23);
    const float ax = sx * L.idir.x, ay = sy * L.idir.y, az = sz * L.idir.z;
    const float bx = (n0.x - L.o.x) * L.idir.x, by = (n0.y - L.o.y) * L.idir.y, bz = (n0.z - L.o.z) * L.idir.z;
    // near / far quantised planes per axis, swapped for negative directions
    const uint2 qlx = make_uint2(__float_as_uint(n2.x), __float_as_uint(n2.y));
    const uint2 qly = make_uint2(__float_as_uint(n2.z), __float_as_uint(n2.w));
    const uint2 qlz = make_uint2(__float_as_uint(n3.x), __float_as_uint(n3.y));
    const uint2 qhx = make_uint2(__float_as_uint(n3.z), __float_as_uint(n3.w));
    const uint2 qhy = make_uint2(__float_as_uint(n4.x), __float_as_uint(n4.y));
    const uint2 qhz = make_uint2(__float_as_uint(n4.z), __float_as_uint(n4.w));
    const uint2 nx = (L.octant & 1u) ? qhx : qlx, fx = (L.octant & 1u) ? qlx : qhx;
    const uint2 ny = (L.octant & 2u) ? qhy : qly, fy = (L.octant & 2u) ? qly : qhy;
    const uint2 nz = (L.octant & 4u) ? qhz : qlz, fz = (L.octant & 4u) ? qlz : qhz;
    const uint32_t octInv4 = L.octInv * 0x01010101u;
    uint32_t bidx[2], cbits[2];
    metaDecode4(__float_as_uint(n1.z), octInv4, &bidx[0], &cbits[0]);
    metaDecode4(__float_as_uint(n1.w), octInv4, &bidx[1], &cbits[1]);
    uint32_t hitmask = 0u;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int h = k >> 2, b = k & 3;
        const float tnx = fmaf(byteToFloat(h ? nx.y : nx.x, b), ax, bx);
        const float tny = fmaf(byteToFloat(h ? ny.y : ny.x, b), ay, by);
        const float tnz = fmaf(byteToFloat(h ? nz.y : nz.x, b), az, bz);
        const float tfx = fmaf(byteToFloat(h ? fx.y : fx.x, b), ax, bx);
        const float tfy = fmaf(byteToFloat(h ? fy.y : fy.x, b), ay, by);
        const float tfz = fmaf(byteToFloat(h ? fz.y : fz.x, b), az, bz);
        const float t0 = fmaxf(fmax3f(tnx, tny, tnz), L.tmin);
        const float t1 = fminf(fmin3f(tfx, tfy, tfz), L.tmax);
        const uint32_t bits = (cbits[h] >> (8 * b)) & 0xFFu;
        const uint32_t shift = (bidx[h] >> (8 * b)) & 0xFFu;
        if (t0 <= t1 * 1.0000010f) hitmask |= bits << shift;
    }
    L.G = make_uint2(__float_as_uint(n1.x), (hitmask & 0xFF000000u) | (ew >> 24));
    uint32_t tbits = hitmask & 0x00FFFFFFu;
    const uint32_t tbase = __float_as_uint(n1.y);
    while (tbits) {
        const int b = __ffs(tbits) - 1;
        tbits &= tbits - 1u;
        const uint32_t ti = tbase + static_cast<uint32_t>(b);
        if (ti >= nTris) {
            *overflow = true;
            return true;
        }
        if (STATS) (*triCount)++;
        const float4 v0 = __ldg(&tris[ti].v0);
        const float4 v1 = __ldg(&tris[ti].v1);
        const float4 v2 = __ldg(&tris[ti].v2);
        const float3 E1 = xyz(v1) - xyz(v0), E2 = xyz(v2) - xyz(v0);
        const float3 pv = cross(L.d, E2);
        const float det = dot(E1, pv);
        if (det > -kEpsT && det < kEpsT) continue;
        const float inv = 1.0f / det;
        const float3 tv = L.o - xyz(v0);
        const float u = dot(tv, pv) * inv;
        if (u < 0.0f || u > 1.0f) continue;
        const float3 qv = cross(tv, E1);
        const float v = dot(L.d, qv) * inv;
        if (v < 0.0f || u + v > 1.0f) continue;
        const float t = dot(E2, qv) * inv;
        if (t <= L.tEps || t > L.tmax) continue;
        L.found = true;
        if (ANY) return true;
        L.tmax = t;
        L.hitSlot = static_cast<int>(ti);
        L.hu = u;
        L.hv = v;
    }
    return !(L.G.y & 0xFF000000u) && L.sp == 0;
}

template <bool ANY, bool STATS>
__device__ __forceinline__ bool traceWide(const WideNode *__restrict__ nodes, const TriRecord *__restrict__ tris,
                                          uint32_t nNodes, uint32_t nTris, float3 o, float3 d, float tmin,
                                          float &tmax, int &hitSlot, float &hu, float &hv, uint2 *__restrict__ stack,
                                          int stride, uint32_t *nodeCount, uint32_t *triCount, bool *overflow,
                                          uint32_t root = 0) {
    uint2 spill[kStackDepth - kStackShared];
    TraceLane L;
    laneInit(L, o, d, tmin, tmax, root);
    while (!laneStep<ANY, STATS>(L, nodes, tris, nNodes, nTris, stack, stride, spill, nodeCount, triCount,
                                 overflow)) {
    }
    tmax = L.tmax;
    hitSlot = L.hitSlot;
    hu = L.hu;
    hv = L.hv;
    return L.found;
}

// Persistent driver: a warp keeps up to 32 rays in flight and refills the lanes whose
// rays have finished, kRefill or more at a time, from a global ray counter (one
// atomicAdd per refill), so lanes do not idle while the slowest ray of a batch finishes
// (after Aila and Laine, "Understanding the Efficiency of Ray Traversal on GPUs", HPG
// 2009).  fetch(i, &o, &d, &tmin, &tmax) loads ray i; done(i, L) consumes its result.
// All 32 lanes of each warp execute every iteration of the loop (warp-uniform control),
// so done() may use warp-collective operations.
#ifndef SPGPU_REFILL
#define SPGPU_REFILL 12
#endif
constexpr int kRefill = SPGPU_REFILL;
// a finished ray's result waits for the warp's next refill, so that the finished lanes
// consume their results together (done() runs on up to 32 lanes instead of one or two)
#ifndef SPGPU_DEFER_DONE
#define SPGPU_DEFER_DONE 1
#endif
constexpr bool kDeferDone = SPGPU_DEFER_DONE != 0;
// traversal steps between two looks at the warp's idle lanes
#ifndef SPGPU_STEPS_PER_CHECK
#define SPGPU_STEPS_PER_CHECK 2
#endif
constexpr int kStepsPerCheck = SPGPU_STEPS_PER_CHECK;

template <bool ANY, bool STATS, class Fetch, class Done>
__device__ __forceinline__ void tracePersistent(const WideNode *__restrict__ nodes,
                                                const TriRecord *__restrict__ tris, uint32_t nNodes,
                                                uint32_t nTris, int n, int *rayCounter, uint2 *__restrict__ stack,
                                                int stride, uint32_t *nodeCount, uint32_t *triCount,
                                                bool *overflow, Fetch fetch, Done done) {
    uint2 spill[kStackDepth - kStackShared];
    TraceLane L;
    int ray = -1;            // >= 0 in flight (or finished), -1 idle, -2 no work left
    bool finished = false;   // the ray has finished, its result not yet consumed
    const int lane = threadIdx.x & 31;
    while (true) {
        if (!kDeferDone) {
            done(finished ? ray : -1, L);
            if (finished) {
                ray = -1;
                finished = false;
            }
        }
        const unsigned idle = __ballot_sync(0xffffffffu, ray == -1 || finished);
        const unsigned busy = __ballot_sync(0xffffffffu, ray >= 0 && !finished);
        if (idle && (__popc(idle) >= kRefill || busy == 0)) {
            if (kDeferDone) {
                // the results of the rays finished since the last refill, consumed together
                done(finished ? ray : -1, L);
                if (finished) {
                    ray = -1;
                    finished = false;
                }
            }
            int base = 0;
            if (lane == __ffs(idle) - 1) base = atomicAdd(rayCounter, __popc(idle));
            base = __shfl_sync(0xffffffffu, base, __ffs(idle) - 1);
            if (ray == -1) {
                const int r = base + __popc(idle & ((1u << lane) - 1u));
                if (r < n) {
                    float3 o, d;
                    float t0, t1;
                    uint32_t root = 0;   // a fetch that takes a sixth argument names the ray's tree root
                    if constexpr (std::is_invocable_v<Fetch &, int, float3 *, float3 *, float *, float *, uint32_t *>)
                        fetch(r, &o, &d, &t0, &t1, &root);
                    else
                        fetch(r, &o, &d, &t0, &t1);
                    laneInit(L, o, d, t0, t1, root);
                    ray = r;
                } else {
                    ray = -2;
                }
            }
        }
        if (__all_sync(0xffffffffu, ray == -2)) break;
#pragma unroll 1
        for (int k = 0; k < kStepsPerCheck; k++) {
            if (ray >= 0 && !finished) {
                finished = laneStep<ANY, STATS>(L, nodes, tris, nNodes, nTris, stack, stride, spill, nodeCount,
                                                triCount, overflow);
            }
        }
    }
}

// host entry points (bvh.cu)
int buildWideBVH(const float *d_verts, int ntri, const int *d_tri_mat, const int *d_tri_light, DeviceBVH *out,
                 cudaStream_t stream, char *err, size_t errlen);
void freeWideBVH(DeviceBVH *b);

}  // namespace spgpu
