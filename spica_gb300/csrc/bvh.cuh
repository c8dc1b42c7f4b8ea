// bvh.cuh -- the device-built compressed 8-wide BVH: its host-side handle and the
// traversal routine shared by the ray-batch kernels and the wavefront renderer.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace spgpu {

// Largest wide-tree depth the traversal kernels accept.  The per-thread stack holds
// one node group per level of the current path: its first kStackShared entries live
// in shared memory, deeper ones spill to a per-thread local array.
constexpr int kStackDepth = 48;
constexpr int kStackShared = 16;
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
__device__ __forceinline__ float byteToFloat(uint32_t w, int k) { return static_cast<float>((w >> (8 * k)) & 0xFFu); }

// Every node and triangle index is checked against the tree's sizes and the loop is
// bounded (kMaxVisits), so a malformed tree ends the ray with *overflow set instead of
// reading out of bounds or spinning.
constexpr uint32_t kMaxVisits = 1u << 22;

template <bool ANY, bool STATS>
__device__ __forceinline__ bool traceWide(const WideNode *__restrict__ nodes, const TriRecord *__restrict__ tris,
                                          uint32_t nNodes, uint32_t nTris, float3 o, float3 d, float tmin,
                                          float &tmax, int &hitSlot, float &hu, float &hv, uint2 *__restrict__ stack,
                                          int stride, uint32_t *nodeCount, uint32_t *triCount, bool *overflow) {
    const float3 idir = mk(d.x == 0.0f ? kInfT : 1.0f / d.x, d.y == 0.0f ? kInfT : 1.0f / d.y,
                           d.z == 0.0f ? kInfT : 1.0f / d.z);
    const uint32_t octant = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    const uint32_t octInv = 7u - octant;
    const float tEps = fmaxf(tmin, kEpsT);
    bool found = false;

    uint2 spill[kStackDepth - kStackShared];
    uint2 G = make_uint2(0u, (1u << (24 + octInv)) | 1u);   // the root as slot 0 of a virtual parent
    uint2 T = make_uint2(0u, 0u);
    int sp = 0;
    uint32_t visits = 0;
    const float4 *nodes4 = reinterpret_cast<const float4 *>(nodes);

    while (true) {
        if (++visits > kMaxVisits) {
            *overflow = true;
            return found;
        }
        if (G.y & 0xFF000000u) {
            const uint32_t key = __ffs(G.y >> 24) - 1;
            G.y &= ~(1u << (24 + key));
            const uint32_t slot = key ^ octInv;
            const uint32_t child = G.x + __popc((G.y & 0xFFu) & ((1u << slot) - 1u));
            if (child >= nNodes) {
                *overflow = true;
                return found;
            }
            if (G.y & 0xFF000000u) {
                if (sp >= kStackDepth) {
                    *overflow = true;
                    return found;
                }
                if (sp < kStackShared) stack[sp * stride] = G;
                else spill[sp - kStackShared] = G;
                sp++;
            }
            if (STATS) (*nodeCount)++;
            const float4 n0 = __ldg(nodes4 + 5 * child + 0);
            const float4 n1 = __ldg(nodes4 + 5 * child + 1);
            const float4 n2 = __ldg(nodes4 + 5 * child + 2);
            const float4 n3 = __ldg(nodes4 + 5 * child + 3);
            const float4 n4 = __ldg(nodes4 + 5 * child + 4);
            const uint32_t ew = __float_as_uint(n0.w);
            const float sx = __uint_as_float((ew & 0xFFu) << 23);
            const float sy = __uint_as_float(((ew >> 8) & 0xFFu) << 23);
            const float sz = __uint_as_float(((ew >> 16) & 0xFFu) << 23);
            const float ax = sx * idir.x, ay = sy * idir.y, az = sz * idir.z;
            const float bx = (n0.x - o.x) * idir.x, by = (n0.y - o.y) * idir.y, bz = (n0.z - o.z) * idir.z;
            // near / far quantised planes per axis, swapped for negative directions
            const uint2 qlx = make_uint2(__float_as_uint(n2.x), __float_as_uint(n2.y));
            const uint2 qly = make_uint2(__float_as_uint(n2.z), __float_as_uint(n2.w));
            const uint2 qlz = make_uint2(__float_as_uint(n3.x), __float_as_uint(n3.y));
            const uint2 qhx = make_uint2(__float_as_uint(n3.z), __float_as_uint(n3.w));
            const uint2 qhy = make_uint2(__float_as_uint(n4.x), __float_as_uint(n4.y));
            const uint2 qhz = make_uint2(__float_as_uint(n4.z), __float_as_uint(n4.w));
            const uint2 nx = (octant & 1u) ? qhx : qlx, fx = (octant & 1u) ? qlx : qhx;
            const uint2 ny = (octant & 2u) ? qhy : qly, fy = (octant & 2u) ? qly : qhy;
            const uint2 nz = (octant & 4u) ? qhz : qlz, fz = (octant & 4u) ? qlz : qhz;
            const uint32_t meta0 = __float_as_uint(n1.z), meta1 = __float_as_uint(n1.w);
            uint32_t hitmask = 0u;
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const int h = k >> 2, b = k & 3;
                const uint32_t m = ((h ? meta1 : meta0) >> (8 * b)) & 0xFFu;
                const float tnx = fmaf(byteToFloat(h ? nx.y : nx.x, b), ax, bx);
                const float tny = fmaf(byteToFloat(h ? ny.y : ny.x, b), ay, by);
                const float tnz = fmaf(byteToFloat(h ? nz.y : nz.x, b), az, bz);
                const float tfx = fmaf(byteToFloat(h ? fx.y : fx.x, b), ax, bx);
                const float tfy = fmaf(byteToFloat(h ? fy.y : fy.x, b), ay, by);
                const float tfz = fmaf(byteToFloat(h ? fz.y : fz.x, b), az, bz);
                const float t0 = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
                const float t1 = fminf(fminf(tfx, tfy), fminf(tfz, tmax));
                if (m != 0u && t0 <= t1 * 1.0000010f) {
                    if ((m & 0x18u) == 0x18u) hitmask |= 1u << (24 + (k ^ octInv));
                    else hitmask |= (m >> 5) << (m & 0x1Fu);
                }
            }
            G = make_uint2(__float_as_uint(n1.x), (hitmask & 0xFF000000u) | (ew >> 24));
            T = make_uint2(__float_as_uint(n1.y), hitmask & 0x00FFFFFFu);
        }

        while (T.y) {
            const int b = __ffs(T.y) - 1;
            T.y &= T.y - 1u;
            const int ti = static_cast<int>(T.x) + b;
            if (static_cast<uint32_t>(ti) >= nTris) {
                *overflow = true;
                return found;
            }
            if (STATS) (*triCount)++;
            const float4 v0 = __ldg(&tris[ti].v0);
            const float4 v1 = __ldg(&tris[ti].v1);
            const float4 v2 = __ldg(&tris[ti].v2);
            const float3 E1 = xyz(v1) - xyz(v0), E2 = xyz(v2) - xyz(v0);
            const float3 pv = cross(d, E2);
            const float det = dot(E1, pv);
            if (det > -kEpsT && det < kEpsT) continue;
            const float inv = 1.0f / det;
            const float3 tv = o - xyz(v0);
            const float u = dot(tv, pv) * inv;
            if (u < 0.0f || u > 1.0f) continue;
            const float3 qv = cross(tv, E1);
            const float v = dot(d, qv) * inv;
            if (v < 0.0f || u + v > 1.0f) continue;
            const float t = dot(E2, qv) * inv;
            if (t <= tEps || t > tmax) continue;
            found = true;
            if (ANY) return true;
            tmax = t;
            hitSlot = ti;
            hu = u;
            hv = v;
        }

        if (!(G.y & 0xFF000000u)) {
            if (sp == 0) break;
            sp--;
            G = sp < kStackShared ? stack[sp * stride] : spill[sp - kStackShared];
        }
    }
    return found;
}

// host entry points (bvh.cu)
int buildWideBVH(const float *d_verts, int ntri, const int *d_tri_mat, const int *d_tri_light, DeviceBVH *out,
                 cudaStream_t stream, char *err, size_t errlen);
void freeWideBVH(DeviceBVH *b);

}  // namespace spgpu
