// wavefront.cu -- the path integrator as a wavefront over SoA queues in HBM.
//
// One pass = one sample for every pixel (the reference's spp loop body,
// core/integrator.cc:64-97), as a fixed kernel sequence captured once into a CUDA
// graph and replayed per sample:
//   raygen                      camera rays (PerspectiveCamera::spawnRay)
//   per bounce b = 0..maxDepth
//     extend                    closest hit of every live path ray; misses add the
//                               environment (b == 0 or after a specular bounce) and
//                               end; hits are appended to one queue per material
//                               class by warp-ballot compaction
//     shade<Lambert|GGX|glass>  material-sorted: emission, next-event estimation with
//                               MIS (both strategies of estimateDirectLight), BSDF
//                               sampling of the continuation, Russian roulette; new
//                               rays and shadow rays appended by warp-ballot compaction
//     shadow                    any-hit for the light-sample and MIS-connection rays;
//                               unoccluded contributions are added to the film
//   finish                      sample index and ray counters
// The estimator is the reference's PathIntegrator::Li (integrators/path/path.cc:42)
// with uniformSampleOneLight / estimateDirectLight (core/mis.cc:21-136).  One change
// of mechanism, not of estimator: the MIS BSDF sample of estimateDirectLight traces a
// closest-hit ray and keeps it only if it lands on the sampled light (mis.cc:117-127).
// Here the light is intersected analytically first (the same intersection that gives
// its pdf, core/shape.cc:39-48), and the ray is queued as an occlusion test up to just
// before the light (area light) or to infinity (environment) -- the same event, with
// one any-hit ray instead of a closest-hit ray, and no ray at all when the sampled
// direction misses the light.
#include <algorithm>
#include <utility>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/spica_gpu.h"
#include "ctx.cuh"
#include "guided_shade.cuh"
#include "shade.cuh"

namespace spgpu {

namespace {

constexpr int kShadeBlock = 128;
constexpr int kCountersPerBounce = 8;

struct PassArgs {
    SceneView sv;
    CameraView cam;
    int W, H, npix;
    int maxDepth;
    uint32_t seed;
    float4 *film;
    int64_t cap;
    float4 *beta;
    float4 *rayO0, *rayO1, *rayD0, *rayD1;
    HitRecord *hits;
    int *classQ;
    float4 *shO, *shD, *shL;
    int *counters;     // per bounce: [0] rays in, [1..3] class counts, [4] shadow rays,
                       // [5] / [6] extend / shadow ray-fetch counters
    int *ctl;          // [0] sample index of the pass
    int ctlStride;     // sample-index step from one pass of this queue set to its next
    int direct;        // direct lighting: no continuation rays after the first hit
    // learned guiding (packFwd == nullptr: plain pass): network weights, scene box of its
    // position input, BSDF share of the proposal, mixture per diffuse-queue entry
    const uint8_t *packFwd;
    const float *biasPad;
    float3 guideLo, guideInvExt;
    float guideAlpha;
    int guidedBounces;   // network sampling at bounces below this one (0: all but the last)
    // training-sample collection (guided passes with collect != 0): radiance gathered by
    // each path, its record count (kRecOpen: the last record waits for the hit of its
    // continuation ray), the records, and the training ring they end in
    int collect;
    float4 *pathL;
    int *recCount;
    float4 *recs;
    float *ring;
    int ringCapacity;
    int *ringCtl;
    unsigned long long *stats;
    unsigned long long *visit;   // [0..1] extend nodes / triangles, [2..3] shadow nodes / triangles
    int *err;
};

__device__ __forceinline__ int filmIndex(const PassArgs &p, int pix) {
    const int y = pix / p.W, x = pix - y * p.W;
    return y * p.W + (p.W - 1 - x);   // film pixel (W-1-x, y), core/integrator.cc:88
}

__device__ __forceinline__ void filmAdd(float4 *film, int idx, float3 c) {
    atomicAdd(&film[idx], make_float4(c.x, c.y, c.z, 0.0f));
}

// ---------------------------------------------------------------- collection
// A record is made at each guided vertex that continues (the megakernel's training
// record): 7 float4 at recs[(k * cap + pid) * 7] for record k of path pid:
//   [0] x0..x3  [1] x4..x7  [2] x8, w  [3] q, f cos  [4] beta, Lafter.x
//   [5] Lafter.yz, E.xy  [6] E.z
// x: network inputs, w: sampled direction, q: proposal pdf, beta: throughput after the
// vertex, Lafter: the path's radiance once the vertex's light samples are resolved, E:
// direct radiance found along w, times the MIS weight of the guided strategy.  At the
// end of the pass each record becomes a ring entry with c = lum(f cos (E + (L_end -
// Lafter) / beta)) / q.
constexpr int kCollectRecs = 12;   // guided vertices per path (max_depth <= 12)
constexpr int kRecOpen = 1 << 30;

// radiance gathered by path pid: the film, and the path's own sum when collecting
template <bool COLLECT>
__device__ __forceinline__ void gather(const PassArgs &p, int pid, int fi, float3 c) {
    filmAdd(p.film, fi, c);
    if (COLLECT) {
        const float4 L = p.pathL[pid];
        p.pathL[pid] = make_float4(L.x + c.x, L.y + c.y, L.z + c.z, 0.0f);
    }
}

// the continuation ray of path pid's open record met its hit (found) or escaped: fill in
// Lafter and E (before anything of the new vertex is gathered)
__device__ __forceinline__ void closeRecord(const PassArgs &p, int pid, bool found, int slot, float t, float3 d) {
    const int rc = p.recCount[pid];
    if (!(rc & kRecOpen)) return;
    const int k = (rc & ~kRecOpen) - 1;
    float *R = reinterpret_cast<float *>(p.recs + (static_cast<int64_t>(k) * p.cap + pid) * 7);
    const float4 L = p.pathL[pid];
    const float q = R[12];
    float3 E = mk(0, 0, 0);
    if (!found) {
        if (p.sv.hasEnv) E = envLe(p.sv.env, d) * powerHeuristic(q, envPdf(p.sv.env, d));
    } else {
        const int lightOf = __ldg(&p.sv.slotShade[slot]).y;
        const float3 n = triNormal(p.sv.tris[slot]);
        if (lightOf >= 0 && dot(n, -d) > 0.0f) {
            const LightRecord &Lr = p.sv.lights[lightOf];
            const float lp = t * t / (dot(n, -d) * Lr.p0.w);
            E = xyz(Lr.L) * powerHeuristic(q, lp);
        }
    }
    R[19] = L.x;
    R[20] = L.y;
    R[21] = L.z;
    R[22] = E.x;
    R[23] = E.y;
    R[24] = E.z;
    p.recCount[pid] = rc & ~kRecOpen;
}

// append to a queue with one atomic per warp: returns this lane's slot (or -1)
__device__ __forceinline__ int warpAppend(bool want, int *counter) {
    const unsigned active = __activemask();
    const unsigned mask = __ballot_sync(active, want);
    if (!mask) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(active, base, leader);
    return want ? base + __popc(mask & ((1u << lane) - 1u)) : -1;
}

// ---------------------------------------------------------------- kernels
__global__ void k_raygen(PassArgs p) {
    const int sample = p.ctl[0];
    for (int pix = blockIdx.x * blockDim.x + threadIdx.x; pix < p.npix; pix += gridDim.x * blockDim.x) {
        const int y = pix / p.W, x = pix - y * p.W;
        const int fi = y * p.W + (p.W - 1 - x);
        const Rand4 r = rand4(p.seed, static_cast<uint32_t>(fi), static_cast<uint32_t>(sample), 0xFFFFu, 0u);
        float3 o, d;
        spawnCameraRay(p.cam, x, y, r.a, r.b, &o, &d);
        p.rayO0[pix] = make_float4(o.x, o.y, o.z, __int_as_float(pix));
        p.rayD0[pix] = make_float4(d.x, d.y, d.z, kInfT);
        p.beta[pix] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        if (p.collect) {
            p.pathL[pix] = make_float4(0, 0, 0, 0);
            p.recCount[pix] = 0;
        }
        atomicAdd(&p.film[fi].w, 1.0f);   // passes of other lanes may add to this pixel concurrently
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) p.counters[0] = p.npix;
}

template <bool STATS, bool COLLECT = false>
__global__ void __launch_bounds__(kTraceBlock, 8) k_extend(PassArgs p, int b) {
    __shared__ uint2 stack[kStackShared * kTraceBlock];
    uint32_t nodeCount = 0, triCount = 0;
    int *cnt = p.counters + b * kCountersPerBounce;
    int *classCnt = cnt + 1;
    const int n = cnt[0];
    const float4 *rO = (b & 1) ? p.rayO1 : p.rayO0;
    const float4 *rD = (b & 1) ? p.rayD1 : p.rayD0;
    bool overflow = false;
    auto fetch = [&](int i, float3 *o, float3 *d, float *t0, float *t1) {
        const float4 d4 = rD[i];
        *o = xyz(rO[i]);
        *d = xyz(d4);
        *t0 = 0.0f;
        *t1 = d4.w;
    };
    auto done = [&](int i, const TraceLane &L) {
        if (!__any_sync(0xffffffffu, i >= 0)) return;
        int cls = -1;
        if (i >= 0) {
            if (COLLECT) closeRecord(p, __float_as_int(rO[i].w), L.found, L.hitSlot, L.tmax, L.d);
            if (L.found) {
                HitRecord h;
                h.t = L.tmax;
                h.prim = L.hitSlot;
                h.u = L.hu;
                h.v = L.hv;
                p.hits[i] = h;
                cls = shadeClass(__ldg(&p.sv.mats[__ldg(&p.sv.slotShade[L.hitSlot]).x].type));
            } else if (p.sv.hasEnv) {
                // escaped: the environment at the first hit or after a specular bounce
                const int pid = __float_as_int(rO[i].w);
                const float4 bt = p.beta[pid];
                if (b == 0 || bt.w != 0.0f) gather<COLLECT>(p, pid, filmIndex(p, pid), xyz(bt) * envLe(p.sv.env, L.d));
            }
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const int k = warpAppend(cls == c, &classCnt[c]);
            if (k >= 0) p.classQ[c * p.cap + k] = i;
        }
    };
    tracePersistent<false, STATS>(p.sv.nodes, p.sv.tris, p.sv.nNodes, p.sv.nTris, n, cnt + 5, stack + threadIdx.x,
                                  kTraceBlock, &nodeCount, &triCount, &overflow, fetch, done);
    if (overflow) atomicOr(p.err, 1);
    if (STATS) {
        atomicAdd(&p.visit[0], static_cast<unsigned long long>(nodeCount));
        atomicAdd(&p.visit[1], static_cast<unsigned long long>(triCount));
    }
}

// append a shaded hit's continuation ray and shadow rays (whole warps call this)
__device__ __forceinline__ void appendShadeResult(const PassArgs &p, const ShadeResult &R, int pid, int *nextCnt,
                                                  int *shCnt, float4 *nO, float4 *nD) {
    const int k = warpAppend(R.cont && !p.direct, nextCnt);
    if (k >= 0) {
        nO[k] = make_float4(R.cO.x, R.cO.y, R.cO.z, __int_as_float(pid));
        nD[k] = R.cD;
        p.beta[pid] = make_float4(R.beta.x, R.beta.y, R.beta.z, R.spec ? 1.0f : 0.0f);
    }
    const int s0 = warpAppend(R.sh0, shCnt);
    if (s0 >= 0) {
        p.shO[s0] = R.s0O;
        p.shD[s0] = R.s0D;
        p.shL[s0] = R.s0L;
    }
    const int s1 = warpAppend(R.sh1, shCnt);
    if (s1 >= 0) {
        p.shO[s1] = R.s1O;
        p.shD[s1] = R.s1D;
        p.shL[s1] = R.s1L;
    }
}

template <int CLS>
__global__ void __launch_bounds__(kShadeBlock) k_shade(PassArgs p, int b) {
    const int *cnt = p.counters + b * kCountersPerBounce;
    const int n = cnt[1 + CLS];
    int *nextCnt = p.counters + (b + 1) * kCountersPerBounce;
    int *shCnt = p.counters + b * kCountersPerBounce + 4;
    const float4 *rO = (b & 1) ? p.rayO1 : p.rayO0;
    const float4 *rD = (b & 1) ? p.rayD1 : p.rayD0;
    float4 *nO = (b & 1) ? p.rayO0 : p.rayO1;
    float4 *nD = (b & 1) ? p.rayD0 : p.rayD1;
    const uint32_t sample = static_cast<uint32_t>(p.ctl[0]);
    const int stride = gridDim.x * blockDim.x;
    const int nIter = (n + stride - 1) / stride;   // uniform trip count keeps warps whole for the ballots
    for (int it = 0; it < nIter; it++) {
        const int j = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
        ShadeResult R;
        R.cont = R.sh0 = R.sh1 = false;
        int pid = 0;
        if (j < n) {
            const int i = p.classQ[CLS * p.cap + j];
            const float4 o4 = rO[i], d4 = rD[i];
            pid = __float_as_int(o4.w);
            const float4 bt = p.beta[pid];
            const int fi = filmIndex(p, pid);
            // shadow rays carry the film pixel, or the path when collecting (k_shadow)
            shadeHit(p.sv, p.hits[i], xyz(o4), xyz(d4), xyz(bt), bt.w != 0.0f, b, p.maxDepth, p.seed,
                     static_cast<uint32_t>(fi), sample, p.collect ? pid : fi, R, p.direct != 0);
            if (!isBlack(R.emit)) {
                if (p.collect) gather<true>(p, pid, fi, R.emit);
                else filmAdd(p.film, fi, R.emit);
            }
        }
        appendShadeResult(p, R, pid, nextCnt, shCnt, nO, nD);
    }
}

// Diffuse hits of a guided pass, bounces before the last.  Each CTA takes 128-entry
// tiles of the diffuse queue: every thread forms its entry's network inputs, the tile
// runs through the four layers on the tensor cores (tcgen05, accumulator in TMEM), and
// each entry is shaded with its mixture (shadeGuidedLambert, the megakernel's shading),
// kept in shared memory in place of the finished input tile (kGsSmem layout).  Several
// CTAs per SM: one's MMA waits overlap another's shading.
#ifndef SPGPU_GUIDED_PASS_MIN_BLOCKS
#define SPGPU_GUIDED_PASS_MIN_BLOCKS 4
#endif
template <bool COLLECT>
__global__ void __launch_bounds__(kGTile, SPGPU_GUIDED_PASS_MIN_BLOCKS) k_shade_guided(PassArgs p, int b) {
    const int *cnt = p.counters + b * kCountersPerBounce;
    const int n = cnt[1 + kMatLambert];
    if (static_cast<int>(blockIdx.x) * kGTile >= n) return;   // no tile for this CTA
    extern __shared__ __align__(128) uint8_t sm[];
    int *nextCnt = p.counters + (b + 1) * kCountersPerBounce;
    int *shCnt = p.counters + b * kCountersPerBounce + 4;
    const float4 *rO = (b & 1) ? p.rayO1 : p.rayO0;
    const float4 *rD = (b & 1) ? p.rayD1 : p.rayD0;
    float4 *nO = (b & 1) ? p.rayO0 : p.rayO1;
    float4 *nD = (b & 1) ? p.rayD0 : p.rayD1;
    const uint32_t sample = static_cast<uint32_t>(p.ctl[0]);
    bool ok = true;
    const uint32_t tmem = tileKernelSetup(sm, p.packFwd, p.biasPad, &ok, kGsOffBar);
    const float *bias = reinterpret_cast<const float *>(sm + kTileSmOffBias);
    uint8_t *xh = sm + kGsOffXH;
    MixRow &mix = reinterpret_cast<MixRow *>(sm + kGsOffXH)[threadIdx.x];
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + kGsOffBar);
    uint32_t phase = 0;
    for (int tile = blockIdx.x; ok && tile * kGTile < n; tile += gridDim.x) {
        const int j = tile * kGTile + static_cast<int>(threadIdx.x);
        const bool live = j < n;
        float4 o4 = make_float4(0, 0, 0, 0), d4 = make_float4(0, 0, 1, 0);
        HitRecord h;
        h.t = 0.0f;
        h.prim = 0;
        float3 ps = mk(0, 0, 0), nn = mk(0, 0, 1);
        float xf[16];
        for (int k = 0; k < 16; k++) xf[k] = 0.0f;
        if (live) {
            const int i = p.classQ[kMatLambert * p.cap + j];
            o4 = rO[i];
            d4 = rD[i];
            h = p.hits[i];
            ps = hitPoint(xyz(o4), xyz(d4), h.t);
            nn = triNormal(p.sv.tris[h.prim]);
            guideFeatures(ps, nn, -xyz(d4), p.guideLo, p.guideInvExt, xf);
        }
        __syncthreads();   // every entry of the last tile is shaded: its mixtures may go
        storeRow8(xh, threadIdx.x, 0, kGK0, xf);
        storeRow8(xh, threadIdx.x, 8, kGK0, xf + 8);
        {
            float raw[kGOut];
            ok = mlpForwardRow(tmem, sm, bias, xh, bar, phase, raw);   // CTA-uniform
            // the last layer's MMA has read the tile, so each row's mixture may take its place
            if (ok) mixtureFromRaw(raw, mix.m);
        }
        if (!ok) break;
        ShadeResult R;
        R.cont = R.sh0 = R.sh1 = false;
        int pid = 0;
        if (live) {
            pid = __float_as_int(o4.w);
            const float4 bt = p.beta[pid];
            const int fi = filmIndex(p, pid);
            const int2 sh = __ldg(&p.sv.slotShade[h.prim]);
            float3 fc;
            float pdf;
            shadeGuidedLambert(p.sv, ps, nn, p.sv.mats[sh.x], sh.y, xyz(d4), xyz(bt), bt.w != 0.0f, b, mix.m,
                               p.guideAlpha, p.seed, static_cast<uint32_t>(fi), sample, R, &fc, &pdf);
            if (!isBlack(R.emit)) gather<COLLECT>(p, pid, fi, R.emit);
            if (COLLECT) {
                R.s0O.w = R.s1O.w = __int_as_float(pid);   // k_shadow gathers per path
                const int nrec = p.recCount[pid];
                if (R.cont && nrec < kCollectRecs) {
                    float4 *Q = p.recs + (static_cast<int64_t>(nrec) * p.cap + pid) * 7;
                    Q[0] = make_float4(xf[0], xf[1], xf[2], xf[3]);
                    Q[1] = make_float4(xf[4], xf[5], xf[6], xf[7]);
                    Q[2] = make_float4(xf[8], R.cD.x, R.cD.y, R.cD.z);
                    Q[3] = make_float4(pdf, fc.x, fc.y, fc.z);
                    Q[4] = make_float4(R.beta.x, R.beta.y, R.beta.z, 0.0f);
                    p.recCount[pid] = (nrec + 1) | kRecOpen;
                }
            }
        }
        appendShadeResult(p, R, pid, nextCnt, shCnt, nO, nD);
    }
    tileKernelTeardown(sm, tmem, ok, phase, kGsOffBar);
    if (!ok && threadIdx.x == 0) atomicOr(p.err, 2);
}

template <bool STATS, bool COLLECT = false>
__global__ void __launch_bounds__(kTraceBlock, 8) k_shadow(PassArgs p, int b) {
    __shared__ uint2 stack[kStackShared * kTraceBlock];
    int *cnt = p.counters + b * kCountersPerBounce;
    const int n = cnt[4];
    bool overflow = false;
    uint32_t nodeCount = 0, triCount = 0;
    auto fetch = [&](int i, float3 *o, float3 *d, float *t0, float *t1) {
        const float4 d4 = p.shD[i];
        *o = xyz(p.shO[i]);
        *d = xyz(d4);
        *t0 = 0.0f;
        *t1 = d4.w;
    };
    auto done = [&](int i, const TraceLane &L) {
        if (i >= 0 && !L.found) {
            const int w = __float_as_int(p.shO[i].w);   // film pixel, or the path when collecting
            const float3 c = xyz(p.shL[i]);
            if (COLLECT) {
                filmAdd(p.film, filmIndex(p, w), c);
                atomicAdd(&p.pathL[w].x, c.x);   // a path's two light samples may finish together
                atomicAdd(&p.pathL[w].y, c.y);
                atomicAdd(&p.pathL[w].z, c.z);
            } else {
                filmAdd(p.film, w, c);
            }
        }
    };
    tracePersistent<true, STATS>(p.sv.nodes, p.sv.tris, p.sv.nNodes, p.sv.nTris, n, cnt + 6, stack + threadIdx.x,
                                 kTraceBlock, &nodeCount, &triCount, &overflow, fetch, done);
    if (overflow) atomicOr(p.err, 1);
    if (STATS) {
        atomicAdd(&p.visit[2], static_cast<unsigned long long>(nodeCount));
        atomicAdd(&p.visit[3], static_cast<unsigned long long>(triCount));
    }
}

// end of a collection pass: every record of every path becomes a training-ring entry
// (16 floats: x[9], w[3], c, q, 0, 0); records whose c is not a positive finite number
// are dropped
__global__ void k_collect(PassArgs p) {
    for (int pid = blockIdx.x * blockDim.x + threadIdx.x; pid < p.npix; pid += gridDim.x * blockDim.x) {
        const int nrec = p.recCount[pid] & ~kRecOpen;
        const float3 Lend = xyz(p.pathL[pid]);
        for (int k = 0; k < nrec; k++) {
            const float4 *Q = p.recs + (static_cast<int64_t>(k) * p.cap + pid) * 7;
            const float4 q3 = Q[3], q4 = Q[4], q5 = Q[5], q6 = Q[6];
            const float3 beta = mk(q4.x, q4.y, q4.z), Lafter = mk(q4.w, q5.x, q5.y);
            float3 Li = mk(q5.z, q5.w, q6.x);   // E
            const float3 rest = Lend - Lafter;
            Li.x += beta.x > 0.0f ? rest.x / beta.x : 0.0f;
            Li.y += beta.y > 0.0f ? rest.y / beta.y : 0.0f;
            Li.z += beta.z > 0.0f ? rest.z / beta.z : 0.0f;
            const float c = gray(mk(q3.y, q3.z, q3.w) * Li) / q3.x;
            if (!(c > 0.0f) || !isfinite(c)) continue;
            const unsigned slot =
                atomicAdd(reinterpret_cast<unsigned *>(p.ringCtl), 1u) % static_cast<unsigned>(p.ringCapacity);
            float4 *D = reinterpret_cast<float4 *>(p.ring + 16 * static_cast<int64_t>(slot));
            D[0] = Q[0];
            D[1] = Q[1];
            D[2] = Q[2];
            D[3] = make_float4(c, q3.x, 0.0f, 0.0f);
        }
    }
}

__global__ void k_finish(PassArgs p) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long rays = 0, shadow = 0;
    for (int b = 0; b <= p.maxDepth; b++) {
        rays += static_cast<unsigned long long>(p.counters[b * kCountersPerBounce]);
        shadow += static_cast<unsigned long long>(p.counters[b * kCountersPerBounce + 4]);
    }
    p.stats[0] += static_cast<unsigned long long>(p.npix);
    p.stats[1] += rays;
    p.stats[2] += shadow;
    p.ctl[0] += p.ctlStride;
}

template <class T>
T *dalloc(size_t n) {
    T *ptr = nullptr;
    if (cudaMalloc(&ptr, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) return nullptr;
    return ptr;
}

int ensureQueues(RenderQueues &q, int64_t npix, int maxDepth) {
    if (q.capacity >= npix && q.maxDepth >= maxDepth && q.pathBeta) return 0;
    freeRenderQueues(&q);
    const int64_t cap = npix;
    q.capacity = cap;
    q.maxDepth = maxDepth;
    q.pathBeta = dalloc<float4>(cap);
    for (int k = 0; k < 2; k++) {
        q.rayO[k] = dalloc<float4>(cap);
        q.rayD[k] = dalloc<float4>(cap);
    }
    q.hits = dalloc<HitRecord>(cap);
    q.classQ = dalloc<int>(3 * cap);
    q.shO = dalloc<float4>(2 * cap);
    q.shD = dalloc<float4>(2 * cap);
    q.shL = dalloc<float4>(2 * cap);
    q.counters = dalloc<int>(static_cast<size_t>(maxDepth + 2) * kCountersPerBounce + 8);
    q.stats = dalloc<unsigned long long>(8);
    q.err = dalloc<int>(1);
    if (!q.pathBeta || !q.rayO[0] || !q.rayO[1] || !q.rayD[0] || !q.rayD[1] || !q.hits || !q.classQ || !q.shO ||
        !q.shD || !q.shL || !q.counters || !q.stats || !q.err) {
        freeRenderQueues(&q);
        setError("spgpu_render: device allocation of the wavefront queues failed");
        return SPGPU_ENOMEM;
    }
    return 0;
}

struct Grids {
    int trace, shade, raygen, guided;
};

Grids passGrids(int device, int64_t npix) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    int occT = 0, occS = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occT, k_extend<false>, kTraceBlock, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occS, k_shade<0>, kShadeBlock, 0);
    Grids g;
    g.trace = sms * std::max(occT, 1);
    g.shade = sms * std::max(occS, 1);
    g.raygen = static_cast<int>(std::min<int64_t>((npix + 255) / 256, static_cast<int64_t>(sms) * 8));
    g.guided = 0;
    return g;
}

// One pass of kernels on stream cs.  With ev (2 events per kernel, in launch order)
// every kernel is bracketed for timing, and STATS variants count BVH visits.
enum KernelClass { kRaygen = 0, kExtend, kShadeL, kShadeC, kShadeD, kShadow, kFinish, kNumClasses };

template <bool STATS>
void launchPass(const PassArgs &a, const Grids &g, cudaStream_t cs, size_t ctrBytes, cudaEvent_t *ev,
                int *evClass, int *nev) {
    auto mark = [&](int cls) {
        if (ev) {
            evClass[*nev / 2] = cls;
            cudaEventRecord(ev[(*nev)++], cs);
        }
    };
    auto done = [&]() {
        if (ev) cudaEventRecord(ev[(*nev)++], cs);
    };
    cudaMemsetAsync(a.counters, 0, ctrBytes, cs);
    mark(kRaygen);
    k_raygen<<<g.raygen, 256, 0, cs>>>(a);
    done();
    for (int b = 0; b <= a.maxDepth; b++) {
        mark(kExtend);
        if (a.collect) k_extend<STATS, true><<<g.trace, kTraceBlock, 0, cs>>>(a, b);
        else k_extend<STATS><<<g.trace, kTraceBlock, 0, cs>>>(a, b);
        done();
        mark(kShadeL);
        if (a.packFwd && b < a.maxDepth && (a.guidedBounces <= 0 || b < a.guidedBounces)) {
            if (a.collect) k_shade_guided<true><<<g.guided, kGTile, kGsSmem, cs>>>(a, b);
            else k_shade_guided<false><<<g.guided, kGTile, kGsSmem, cs>>>(a, b);
        } else {
            k_shade<kMatLambert><<<g.shade, kShadeBlock, 0, cs>>>(a, b);
        }
        done();
        mark(kShadeC);
        k_shade<kMatConductor><<<g.shade, kShadeBlock, 0, cs>>>(a, b);
        done();
        mark(kShadeD);
        k_shade<kMatDielectric><<<g.shade, kShadeBlock, 0, cs>>>(a, b);
        done();
        mark(kShadow);
        if (a.collect) k_shadow<STATS, true><<<g.trace, kTraceBlock, 0, cs>>>(a, b);
        else k_shadow<STATS><<<g.trace, kTraceBlock, 0, cs>>>(a, b);
        done();
    }
    if (a.collect) k_collect<<<g.raygen, 256, 0, cs>>>(a);
    mark(kFinish);
    k_finish<<<1, 32, 0, cs>>>(a);
    done();
}

uint64_t hashBytes(const void *d, size_t n, uint64_t h = 1469598103934665603ull) {
    const unsigned char *c = static_cast<const unsigned char *>(d);
    for (size_t i = 0; i < n; i++) h = (h ^ c[i]) * 1099511628211ull;
    return h;
}

}  // namespace

void freeRenderQueues(RenderQueues *q) {
    if (q->graph) cudaGraphExecDestroy(q->graph);
    if (q->graphAlt) cudaGraphExecDestroy(q->graphAlt);
    cudaFree(q->pathL);
    cudaFree(q->recCount);
    cudaFree(q->recs);
    cudaFree(q->pathBeta);
    for (int k = 0; k < 2; k++) {
        cudaFree(q->rayO[k]);
        cudaFree(q->rayD[k]);
    }
    cudaFree(q->hits);
    cudaFree(q->classQ);
    cudaFree(q->shO);
    cudaFree(q->shD);
    cudaFree(q->shL);
    cudaFree(q->counters);
    cudaFree(q->stats);
    cudaFree(q->err);
    *q = RenderQueues{};
}

namespace {
int setupPass(Ctx &C, RenderQueues &q, const float *camera, int W, int H, int maxDepth, uint32_t seed, float4 *film,
              int ctlStride, int integrator, const GuideView *gv, PassArgs *out) {
    const int64_t npix = static_cast<int64_t>(W) * H;
    int rc = ensureQueues(q, npix, maxDepth);
    if (rc) return rc;
    PassArgs &a = *out;
    std::memset(&a, 0, sizeof(a));
    a.sv = C.view();
    a.cam = makeCamera(camera, W, H);
    a.W = W;
    a.H = H;
    a.npix = static_cast<int>(npix);
    a.maxDepth = maxDepth;
    a.seed = seed;
    a.film = film;
    a.cap = q.capacity;
    a.beta = q.pathBeta;
    a.rayO0 = q.rayO[0];
    a.rayO1 = q.rayO[1];
    a.rayD0 = q.rayD[0];
    a.rayD1 = q.rayD[1];
    a.hits = q.hits;
    a.classQ = q.classQ;
    a.shO = q.shO;
    a.shD = q.shD;
    a.shL = q.shL;
    a.counters = q.counters;
    a.ctl = q.counters + (q.maxDepth + 2) * kCountersPerBounce;
    a.stats = q.stats;
    a.visit = q.stats + 4;
    a.err = q.err;
    a.ctlStride = ctlStride;
    a.direct = integrator == SPGPU_INTEGRATOR_DIRECT ? 1 : 0;
    if (gv) {
        a.packFwd = gv->packFwd;
        a.biasPad = gv->biasPad;
        a.guideAlpha = gv->alpha;
        a.guidedBounces = gv->guidedBounces;
        if (gv->collect) {
            if (!q.recs) {
                cudaMalloc(&q.pathL, sizeof(float4) * q.capacity);
                cudaMalloc(&q.recCount, sizeof(int) * q.capacity);
                if (cudaMalloc(&q.recs, sizeof(float4) * 7 * kCollectRecs * q.capacity) != cudaSuccess || !q.pathL ||
                    !q.recCount) {
                    cudaGetLastError();
                    setError("spgpu_guiding_render: device allocation of the collection records failed");
                    return SPGPU_ENOMEM;
                }
            }
            a.collect = 1;
            a.pathL = q.pathL;
            a.recCount = q.recCount;
            a.recs = q.recs;
            a.ring = gv->ring;
            a.ringCapacity = gv->capacity;
            a.ringCtl = gv->ringCtl;
        }
        const float3 ext = C.bvh.hi - C.bvh.lo;
        a.guideLo = C.bvh.lo;
        a.guideInvExt = mk(ext.x > 0 ? 1.0f / ext.x : 0.0f, ext.y > 0 ? 1.0f / ext.y : 0.0f,
                           ext.z > 0 ? 1.0f / ext.z : 0.0f);
    }
    return 0;
}

// (re)capture the pass graph of queue set q when anything baked into it changes
int ensurePassGraph(Ctx &C, RenderQueues &q, const PassArgs &a, int W, int H, int maxDepth, uint32_t seed,
                    float4 *film) {
    uint64_t key[4];
    key[0] = hashBytes(&a, sizeof(a));
    key[1] = static_cast<uint64_t>(W) << 32 | static_cast<uint32_t>(H);
    key[2] = static_cast<uint64_t>(maxDepth) << 32 | seed;
    key[3] = reinterpret_cast<uint64_t>(film);
    if (q.graph && std::memcmp(key, q.graphKey, sizeof(key)) == 0) return 0;
    if (q.graphAlt && std::memcmp(key, q.graphKeyAlt, sizeof(key)) == 0) {   // swap in the other one
        std::swap(q.graph, q.graphAlt);
        std::swap(q.graphKey, q.graphKeyAlt);
        return 0;
    }
    // keep the current graph as the alternative, capture a new one
    if (q.graphAlt) cudaGraphExecDestroy(q.graphAlt);
    q.graphAlt = q.graph;
    std::memcpy(q.graphKeyAlt, q.graphKey, sizeof(key));
    q.graph = nullptr;
    Grids gr = passGrids(C.device, static_cast<int64_t>(W) * H);
    if (a.packFwd)   // attributes and grid before the capture
        gr.guided = guideTileKernelGrid(a.collect ? reinterpret_cast<const void *>(k_shade_guided<true>)
                                                  : reinterpret_cast<const void *>(k_shade_guided<false>),
                                        C.device, kGsSmem);
    const size_t ctrBytes = sizeof(int) * (q.maxDepth + 2) * kCountersPerBounce;
    cudaStream_t cs = C.stream;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cudaFail("cudaStreamBeginCapture", e);
    launchPass<false>(a, gr, cs, ctrBytes, nullptr, nullptr, nullptr);
    e = cudaStreamEndCapture(cs, &g);
    if (e != cudaSuccess) return cudaFail("cudaStreamEndCapture", e);
    e = cudaGraphInstantiate(&q.graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cudaFail("cudaGraphInstantiate", e);
    std::memcpy(q.graphKey, key, sizeof(key));
    return 0;
}
}  // namespace

int renderFrame(Ctx *ctx, const float *camera, int W, int H, int spp, int sampleOffset, int maxDepth, uint32_t seed,
                int integrator, float4 *film, unsigned long long *statsOut, float *msOut, cudaStream_t stream,
                const GuideView *gv) {
    Ctx &C = *ctx;
    // direct lighting shades the first hit only, with light sampling whatever max_depth says
    if (integrator == SPGPU_INTEGRATOR_DIRECT) maxDepth = 1;
    // pass lanes in use: one per pass up to the context's setting
    const int lanes = std::max(1, std::min(spp, C.passLanes));
    RenderQueues *qs[Ctx::kPassLanes];
    cudaStream_t ss[Ctx::kPassLanes];
    qs[0] = &C.rq;
    ss[0] = stream;
    for (int k = 1; k < lanes; k++) {
        qs[k] = &C.rqLane[k - 1];
        ss[k] = C.laneStream[k - 1];
    }
    for (int k = 0; k < lanes; k++) {
        PassArgs a;
        int rc = setupPass(C, *qs[k], camera, W, H, maxDepth, seed, film, lanes, integrator, gv, &a);
        if (!rc) rc = ensurePassGraph(C, *qs[k], a, W, H, maxDepth, seed, film);
        if (rc) return rc;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaError_t e = cudaEventRecord(e0, stream);
    if (e == cudaSuccess && lanes > 1) e = cudaEventRecord(C.laneFork, stream);
    for (int k = 0; k < lanes && e == cudaSuccess; k++) {
        RenderQueues &q = *qs[k];
        if (k > 0) e = cudaStreamWaitEvent(ss[k], C.laneFork, 0);
        const int first = sampleOffset + k;   // lane k renders samples first, first + lanes, ...
        int *ctl = q.counters + (q.maxDepth + 2) * kCountersPerBounce;
        if (e == cudaSuccess) e = cudaMemsetAsync(q.stats, 0, 8 * sizeof(unsigned long long), ss[k]);
        if (e == cudaSuccess) e = cudaMemsetAsync(q.err, 0, sizeof(int), ss[k]);
        if (e == cudaSuccess) e = cudaMemcpyAsync(ctl, &first, sizeof(int), cudaMemcpyHostToDevice, ss[k]);
    }
    for (int s = 0; s < spp && e == cudaSuccess; s++) e = cudaGraphLaunch(qs[s % lanes]->graph, ss[s % lanes]);
    for (int k = 1; k < lanes && e == cudaSuccess; k++) {
        e = cudaEventRecord(C.laneJoin[k - 1], ss[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, C.laneJoin[k - 1], 0);
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, stream);
    unsigned long long st[Ctx::kPassLanes][4] = {};
    int err[Ctx::kPassLanes] = {};
    for (int k = 0; k < lanes && e == cudaSuccess; k++) {
        e = cudaMemcpyAsync(st[k], qs[k]->stats, sizeof(st[k]), cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&err[k], qs[k]->err, sizeof(int), cudaMemcpyDeviceToHost, stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    float ms = 0.0f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cudaFail("spgpu_render", e);
    int anyErr = 0;
    for (int j = 0; j < 4; j++) statsOut[j] = 0;
    for (int k = 0; k < lanes; k++) {
        for (int j = 0; j < 3; j++) statsOut[j] += st[k][j];
        anyErr |= err[k];
    }
    // raygen, per bounce extend + three shade kernels + shadow, finish (and collect)
    statsOut[3] = static_cast<unsigned long long>(spp) * (2 + 5 * (maxDepth + 1) + (gv && gv->collect ? 1 : 0));
    *msOut = ms;
    if (anyErr) {
        setError((anyErr & 2) ? "spgpu_render: guiding network tensor-core wait timed out"
                              : "spgpu_render: traversal stack overflow");
        return SPGPU_EKERNEL;
    }
    return 0;
}

int renderProfile(Ctx *ctx, const float *camera, int W, int H, int spp, int sampleOffset, int maxDepth, uint32_t seed,
                  int integrator, float4 *film, double *kernelMs, long long *launches, unsigned long long *statsOut,
                  unsigned long long *visitOut, cudaStream_t stream) {
    Ctx &C = *ctx;
    RenderQueues &q = C.rq;
    PassArgs a;
    if (integrator == SPGPU_INTEGRATOR_DIRECT) maxDepth = 1;
    int rc = setupPass(C, q, camera, W, H, maxDepth, seed, film, 1, integrator, nullptr, &a);
    if (rc) return rc;
    const Grids gr = passGrids(C.device, static_cast<int64_t>(W) * H);
    const size_t ctrBytes = sizeof(int) * (q.maxDepth + 2) * kCountersPerBounce;
    const int perPass = 2 * (2 + 5 * (maxDepth + 1));
    std::vector<cudaEvent_t> ev(static_cast<size_t>(perPass) * std::max(spp, 1));
    std::vector<int> cls(ev.size() / 2 + 1);
    for (auto &e : ev) cudaEventCreate(&e);
    for (int k = 0; k < kNumClasses; k++) {
        kernelMs[k] = 0.0;
        launches[k] = 0;
    }
    cudaError_t e = cudaMemsetAsync(q.stats, 0, 8 * sizeof(unsigned long long), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(q.err, 0, sizeof(int), stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(a.ctl, &sampleOffset, sizeof(int), cudaMemcpyHostToDevice, stream);
    // timing: plain kernels, each bracketed by events
    int nev = 0;
    for (int s = 0; s < spp && e == cudaSuccess; s++) {
        launchPass<false>(a, gr, stream, ctrBytes, ev.data(), cls.data(), &nev);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    for (int i = 0; i + 1 < nev && e == cudaSuccess; i += 2) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
        kernelMs[cls[i / 2]] += ms;
        launches[cls[i / 2]] += 1;
    }
    unsigned long long st[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(st, q.stats, sizeof(st), cudaMemcpyDeviceToHost);
    // counting: the same samples again with the visit counters on
    if (e == cudaSuccess) e = cudaMemsetAsync(q.stats, 0, 8 * sizeof(unsigned long long), stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(a.ctl, &sampleOffset, sizeof(int), cudaMemcpyHostToDevice, stream);
    for (int s = 0; s < spp && e == cudaSuccess; s++) {
        launchPass<true>(a, gr, stream, ctrBytes, nullptr, nullptr, nullptr);
        e = cudaGetLastError();
    }
    unsigned long long st2[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int err = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(st2, q.stats, sizeof(st2), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err, q.err, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    for (auto &x : ev) cudaEventDestroy(x);
    if (e != cudaSuccess) return cudaFail("spgpu_render_profile", e);
    for (int k = 0; k < 4; k++) statsOut[k] = st[k];
    for (int k = 0; k < 4; k++) visitOut[k] = st2[4 + k];
    if (err) {
        setError("spgpu_render_profile: traversal stack overflow");
        return SPGPU_EKERNEL;
    }
    return 0;
}

}  // namespace spgpu
