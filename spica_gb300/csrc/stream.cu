// stream.cu -- the path integrator as a streaming wavefront: a fixed pool of path slots
// in HBM that is refilled with new camera paths as paths end, so every launch works on a
// full pool and the latency-bound tail of a sample pass occurs once per render instead of
// once per pass.
//
// One iteration (all slots advance one vertex):
//   regen            new camera rays (PerspectiveCamera::spawnRay) into the free slots,
//                    taken in order from the render's path sequence: path g is sample
//                    sampleOffset + g / npix of pixel g % npix
//   extend           closest hit of every ray in the pool; a miss adds the environment
//                    (first vertex or after a specular bounce) and ends the path; a hit
//                    copies the whole path record (ray, throughput, pixel, sample, depth,
//                    hit) into the queue of its material class, in coalesced 64-byte rows
//   shade<class>     emission, next-event estimation with MIS, BSDF sampling and Russian
//                    roulette (shadeHit, the reference's PathIntegrator::Li,
//                    integrators/path/path.cc:42-125); continuing paths are written back
//                    into the pool, shadow rays into the shadow queue
//   shadow           any-hit for the shadow rays; unoccluded ones add to the film
//   advance          counters for the next iteration, the render's done flag
// A guided render (learned guiding proposal) shades the Lambert queue with the network
// instead (k_sshade_guided: tensor-core tiles of 128 queue rows).
// A path's random numbers are keyed by (seed, film pixel) and counted by (sample, depth,
// stream), exactly as in the pass-by-pass wavefront (wavefront.cu), so a render draws the
// same samples whichever slot or iteration a path runs in; only the order of the film's
// floating-point additions differs.
//
// The iterations are captured into one CUDA graph of kIterPerGraph iterations, replayed
// until the device reports that every path of the render has ended.  The host reads the
// done flag of the replay kReplayLag launches back, so the GPU always has work queued;
// replays past the end find empty queues and return at once.
#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "../../include/spica_gpu.h"
#include "ctx.cuh"
#include "guided_shade.cuh"
#include "shade.cuh"

namespace spgpu {

namespace {

constexpr int kShadeBlockS = 128;
#ifndef SPGPU_TRACE_MIN_BLOCKS
#define SPGPU_TRACE_MIN_BLOCKS 8
#endif
constexpr int kTraceMinBlocks = SPGPU_TRACE_MIN_BLOCKS;   // resident traversal blocks per SM (register budget)
#ifndef SPGPU_SHADE_MIN_BLOCKS
#define SPGPU_SHADE_MIN_BLOCKS 6
#endif
constexpr int kShadeMinBlocks = SPGPU_SHADE_MIN_BLOCKS;   // resident shading blocks per SM (register budget)
#ifndef SPGPU_GUIDED_MIN_BLOCKS
#define SPGPU_GUIDED_MIN_BLOCKS 4
#endif
constexpr int kGuidedMinBlocks = SPGPU_GUIDED_MIN_BLOCKS;   // resident guided shading blocks per SM
#ifndef SPGPU_ITER_PER_GRAPH
#define SPGPU_ITER_PER_GRAPH 8
#endif
#ifndef SPGPU_REPLAY_LAG
#define SPGPU_REPLAY_LAG 1
#endif
constexpr int kIterPerGraph = SPGPU_ITER_PER_GRAPH;   // iterations captured in one graph
constexpr int kReplayLag = SPGPU_REPLAY_LAG;          // replays in flight before the host reads a done flag
constexpr int kDoneRing = StreamQueues::kEvents;
// counters (ints): [0] rays in the pool, [1] continuations written, [2..4] class
// counts, [5] shadow rays, [6] extend ray fetch, [7] shadow ray fetch, [8] done, [9]
// iterations, [10] error flags
enum : int { kCtrRays = 0, kCtrCont, kCtrClass0, kCtrShadow = 5, kCtrFetchE, kCtrFetchS, kCtrDone, kCtrIter, kCtrErr };
constexpr int kNumCtr = 16;
// 64-bit counters: [0] paths started, [1] paths, [2] closest rays, [3] shadow rays,
// [4..7] visits (extend nodes, triangles, shadow nodes, triangles); then the call's own
// parameters, written by the host per render so that one captured graph serves every
// call: [8] paths of the render (spp * npix), [9] sample offset (batches: the lane's
// first path of the batch's sequence), [10] film address; [11] iterations run (batches)
enum : int { kBigStarted = 0, kBigPaths, kBigClosest, kBigShadow, kBigVisit, kBigTotal = 8, kBigOffset, kBigFilm,
             kBigIters };
constexpr int kNumBig = 12;

// a path's depth (bits 0..7), specular flag (bit 8) and, in batches, its render (bits
// 9..), carried in the w of its direction
__device__ __forceinline__ float packMeta(int depth, bool spec, int render = 0) {
    return __int_as_float(depth | (spec ? 256 : 0) | (render << 9));
}
__device__ __forceinline__ int metaRender(int meta) { return static_cast<int>(static_cast<unsigned>(meta) >> 9); }

struct StreamArgs {
    SceneView sv;
    CameraView cam;
    int W, H, npix;
    int maxDepth;
    uint32_t seed;
    int direct;
    int cap;           // path slots
    // the pool: (origin, pixel), (direction, depth | specular << 8), (throughput, sample)
    float4 *rO, *rD, *rB;
    // class queues, cap rows per class: the pool record and the hit (t, slot, u, v)
    float4 *qO, *qD, *qB, *qH;
    float4 *shO, *shD, *shL;   // shadow queue, 2 * cap rows: (origin, film index), (dir, tmax), contribution
    int *ctr;
    unsigned long long *big;
    // guided renders: the network's packed weights and biases (null: plain BSDF
    // sampling), the proposal's BSDF share, the depths that sample it (0: all but the
    // last), and the scene box that normalises the network's position input
    const uint8_t *packFwd;
    const float *biasPad;
    float guideAlpha;
    int guidedBounces;
    float3 guideLo, guideInvExt;
    // batches: the renders, the first path of each in the batch's path sequence
    // (nRenders + 1 entries), paths ended per render, the start and completion times
    // (globaltimer ns: [0] start, [1 + r] render r), the device loop's condition and its
    // iteration limit
    const RenderMeta *renders;
    const long long *pathStart;
    int nRenders;
    unsigned long long *ended;
    unsigned long long *times;
    cudaGraphConditionalHandle cond;
    int devLoop;        // the iterations run in a device loop on cond (else the host drives them)
    long long iterLimit;
};

__device__ __forceinline__ int filmIndexS(const StreamArgs &p, int pix) {
    const int y = pix / p.W, x = pix - y * p.W;
    return y * p.W + (p.W - 1 - x);   // film pixel (W-1-x, y), core/integrator.cc:88
}

// slots refilled this iteration (every kernel of the iteration derives the same number
// from the counters, which only k_sadvance changes)
__device__ __forceinline__ long long totalPaths(const StreamArgs &p) { return static_cast<long long>(p.big[kBigTotal]); }
__device__ __forceinline__ float4 *filmOf(const StreamArgs &p) { return reinterpret_cast<float4 *>(p.big[kBigFilm]); }
__device__ __forceinline__ int newPaths(const StreamArgs &p) {
    const long long left = totalPaths(p) - static_cast<long long>(p.big[kBigStarted]);
    const long long freeSlots = p.cap - p.ctr[kCtrRays];
    return static_cast<int>(max(0LL, min(freeSlots, left)));
}

__device__ __forceinline__ int warpAppendS(bool want, int *counter) {
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

// batches: the render of path g of the batch's sequence (binary search of pathStart)
__device__ __forceinline__ int renderOfPath(const StreamArgs &p, long long g) {
    int lo = 0, hi = p.nRenders;   // pathStart[lo] <= g < pathStart[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&p.pathStart[mid]) <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

// batches: add the warp's ended paths to their renders' counts (whole warps call this)
__device__ __forceinline__ void countEnded(const StreamArgs &p, bool ended, int render) {
    const unsigned mask = __ballot_sync(__activemask(), ended);
    if (!ended) return;
    const unsigned same = __match_any_sync(mask, render);
    if ((threadIdx.x & 31) == __ffs(same) - 1)
        atomicAdd(&p.ended[render], static_cast<unsigned long long>(__popc(same)));
}

// film pixel of raster pixel pix in a film of width W (x mirrored, core/integrator.cc:88)
__device__ __forceinline__ int mirrored(int pix, int W) {
    const int y = pix / W, x = pix - y * W;
    return y * W + (W - 1 - x);
}

template <bool BATCH>
__global__ void k_sregen(StreamArgs p) {
    const int have = p.ctr[kCtrRays];
    const int nNew = newPaths(p);
    const long long started = static_cast<long long>(p.big[kBigStarted]);
    // one render: the first sample of the call; batches: the lane's first path in the
    // batch's sequence
    const long long offset = static_cast<long long>(p.big[kBigOffset]);
    float4 *film = filmOf(p);
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nNew; j += gridDim.x * blockDim.x) {
        const long long g = started + j;
        int render = 0, sample, pix, fi;
        long long filmBase = 0;
        float3 o, d;
        if constexpr (BATCH) {
            const long long gb = offset + g;
            render = renderOfPath(p, gb);
            const RenderMeta &M = p.renders[render];
            const long long local = gb - __ldg(&p.pathStart[render]);
            const int npix = M.W * M.H;
            sample = static_cast<int>(local / npix);
            pix = static_cast<int>(local % npix);
            const int y = pix / M.W, x = pix - y * M.W;
            fi = y * M.W + (M.W - 1 - x);
            const Rand4 r = rand4(M.seed, static_cast<uint32_t>(fi), static_cast<uint32_t>(sample), 0xFFFFu, 0u);
            spawnCameraRay(M.cam, x, y, r.a, r.b, &o, &d);
            filmBase = M.filmOffset;
        } else {
            sample = static_cast<int>(offset) + static_cast<int>(g / p.npix);
            pix = static_cast<int>(g % p.npix);
            const int y = pix / p.W, x = pix - y * p.W;
            fi = y * p.W + (p.W - 1 - x);
            const Rand4 r = rand4(p.seed, static_cast<uint32_t>(fi), static_cast<uint32_t>(sample), 0xFFFFu, 0u);
            spawnCameraRay(p.cam, x, y, r.a, r.b, &o, &d);
        }
        const int k = have + j;
        p.rO[k] = make_float4(o.x, o.y, o.z, __int_as_float(pix));
        p.rD[k] = make_float4(d.x, d.y, d.z, packMeta(0, false, render));
        p.rB[k] = make_float4(1.0f, 1.0f, 1.0f, __int_as_float(sample));
        atomicAdd(&film[filmBase + fi].w, 1.0f);
    }
}

template <bool STATS, bool BATCH>
__global__ void __launch_bounds__(kTraceBlock, kTraceMinBlocks) k_sextend(StreamArgs p) {
    __shared__ uint2 stack[kStackShared * kTraceBlock];
    uint32_t nodeCount = 0, triCount = 0;
    const int n = p.ctr[kCtrRays] + newPaths(p);
    float4 *film = filmOf(p);
    bool overflow = false;
    auto done = [&](int i, const TraceLane &L) {
        if (!__any_sync(0xffffffffu, i >= 0)) return;
        int cls = -1;
        float4 o4 = make_float4(0, 0, 0, 0), d4 = o4, b4 = o4;
        if (i >= 0) {
            o4 = p.rO[i];
            d4 = p.rD[i];
            b4 = p.rB[i];
            if (L.found) {
                cls = shadeClass(__ldg(&p.sv.mats[__ldg(&p.sv.slotShade[L.hitSlot]).x].type));
            } else if (!BATCH && p.sv.hasEnv) {
                // escaped: the environment at the first vertex or after a specular bounce
                const int meta = __float_as_int(d4.w);
                if ((meta & 255) == 0 || (meta & 256)) {
                    const float3 c = xyz(b4) * envLe(p.sv.env, L.d);
                    atomicAdd(&film[filmIndexS(p, __float_as_int(o4.w))], make_float4(c.x, c.y, c.z, 0.0f));
                }
            }
        }
        if constexpr (BATCH) countEnded(p, i >= 0 && !L.found, metaRender(__float_as_int(d4.w)));   // no environment
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const int k = warpAppendS(cls == c, &p.ctr[kCtrClass0 + c]);
            if (k >= 0) {
                const int64_t row = static_cast<int64_t>(c) * p.cap + k;
                p.qO[row] = o4;
                p.qD[row] = d4;
                p.qB[row] = b4;
                p.qH[row] = make_float4(L.tmax, __int_as_float(L.hitSlot), L.hu, L.hv);
            }
        }
    };
    if constexpr (BATCH) {
        // each render's rays start at its own tree's root
        auto fetch = [&](int i, float3 *o, float3 *d, float *t0, float *t1, uint32_t *root) {
            const float4 d4 = p.rD[i];
            *o = xyz(p.rO[i]);
            *d = xyz(d4);
            *t0 = 0.0f;
            *t1 = kInfT;
            *root = p.renders[metaRender(__float_as_int(d4.w))].root;
        };
        tracePersistent<false, STATS>(p.sv.nodes, p.sv.tris, p.sv.nNodes, p.sv.nTris, n, &p.ctr[kCtrFetchE],
                                      stack + threadIdx.x, kTraceBlock, &nodeCount, &triCount, &overflow, fetch,
                                      done);
    } else {
        auto fetch = [&](int i, float3 *o, float3 *d, float *t0, float *t1) {
            *o = xyz(p.rO[i]);
            *d = xyz(p.rD[i]);
            *t0 = 0.0f;
            *t1 = kInfT;
        };
        tracePersistent<false, STATS>(p.sv.nodes, p.sv.tris, p.sv.nNodes, p.sv.nTris, n, &p.ctr[kCtrFetchE],
                                      stack + threadIdx.x, kTraceBlock, &nodeCount, &triCount, &overflow, fetch,
                                      done);
    }
    if (overflow) atomicOr(&p.ctr[kCtrErr], 1);
    if (STATS) {
        atomicAdd(&p.big[kBigVisit + 0], static_cast<unsigned long long>(nodeCount));
        atomicAdd(&p.big[kBigVisit + 1], static_cast<unsigned long long>(triCount));
    }
}

// a shaded hit's emission (at film pixel filmIdx), continuation (back into the pool) and
// shadow rays; whole warps call this.  Batches count the paths that end here.
template <bool BATCH = false>
__device__ __forceinline__ void emitShadeResultS(const StreamArgs &p, const ShadeResult &R, bool live, long long filmIdx,
                                                 int pix, int meta, int sample) {
    if (live && !isBlack(R.emit))
        atomicAdd(&filmOf(p)[filmIdx], make_float4(R.emit.x, R.emit.y, R.emit.z, 0.0f));
    if constexpr (BATCH) countEnded(p, live && !R.cont, metaRender(meta));
    const int k = warpAppendS(R.cont && !p.direct, &p.ctr[kCtrCont]);
    if (k >= 0) {
        p.rO[k] = make_float4(R.cO.x, R.cO.y, R.cO.z, __int_as_float(pix));
        p.rD[k] = make_float4(R.cD.x, R.cD.y, R.cD.z, packMeta((meta & 255) + 1, R.spec, metaRender(meta)));
        p.rB[k] = make_float4(R.beta.x, R.beta.y, R.beta.z, __int_as_float(sample));
    }
    const int s0 = warpAppendS(R.sh0, &p.ctr[kCtrShadow]);
    if (s0 >= 0) {
        p.shO[s0] = R.s0O;
        p.shD[s0] = R.s0D;
        p.shL[s0] = R.s0L;
    }
    const int s1 = warpAppendS(R.sh1, &p.ctr[kCtrShadow]);
    if (s1 >= 0) {
        p.shO[s1] = R.s1O;
        p.shD[s1] = R.s1D;
        p.shL[s1] = R.s1L;
    }
}

__device__ __forceinline__ HitRecord hitOfRow(float4 h4) {
    HitRecord h;
    h.t = h4.x;
    h.prim = __float_as_int(h4.y);
    h.u = h4.z;
    h.v = h4.w;
    return h;
}

template <int CLS, bool BATCH>
__global__ void __launch_bounds__(kShadeBlockS, kShadeMinBlocks) k_sshade(StreamArgs p) {
    const int n = p.ctr[kCtrClass0 + CLS];
    const int stride = gridDim.x * blockDim.x;
    const int nIter = (n + stride - 1) / stride;   // uniform trip count keeps warps whole for the ballots
    const int64_t base = static_cast<int64_t>(CLS) * p.cap;
    for (int it = 0; it < nIter; it++) {
        const int j = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
        ShadeResult R;
        R.cont = R.sh0 = R.sh1 = false;
        int pix = 0, meta = 0, sample = 0;
        long long filmIdx = 0;
        if (j < n) {
            const float4 o4 = p.qO[base + j], d4 = p.qD[base + j], b4 = p.qB[base + j], h4 = p.qH[base + j];
            pix = __float_as_int(o4.w);
            meta = __float_as_int(d4.w);
            sample = __float_as_int(b4.w);
            if constexpr (BATCH) {
                // the render's own lights, film, depth and random streams
                const int render = metaRender(meta);
                const RenderMeta &M = p.renders[render];
                SceneView S = p.sv;
                S.lightBase = M.lightBase;
                S.nArea = M.nArea;
                S.nLights = M.nArea;
                const int fi = mirrored(pix, M.W);
                filmIdx = M.filmOffset + fi;
                shadeHit(S, hitOfRow(h4), xyz(o4), xyz(d4), xyz(b4), (meta & 256) != 0, meta & 255, M.maxDepth, M.seed,
                         static_cast<uint32_t>(fi), static_cast<uint32_t>(sample), static_cast<int>(filmIdx), R, false);
                R.s0L.w = R.s1L.w = __int_as_float(render);   // the shadow rays' tree
            } else {
                const int fi = filmIndexS(p, pix);
                filmIdx = fi;
                shadeHit(p.sv, hitOfRow(h4), xyz(o4), xyz(d4), xyz(b4), (meta & 256) != 0, meta & 255, p.maxDepth,
                         p.seed, static_cast<uint32_t>(fi), static_cast<uint32_t>(sample), fi, R, p.direct != 0);
            }
        }
        emitShadeResultS<BATCH>(p, R, j < n, filmIdx, pix, meta, sample);
    }
}

// Lambert hits of a guided render.  Each CTA takes 128-row tiles of the Lambert queue:
// every thread forms its row's network inputs, the tile runs through the four layers on
// the tensor cores (tcgen05, accumulator in TMEM), and each row is shaded with its
// mixture (shadeGuidedLambert), kept in shared memory.  Rows at the last depth, or past
// the guided depths, are shaded with plain BSDF sampling as in k_sshade.  The queue
// mixes depths, so one launch covers what the pass-by-pass wavefront does in one guided
// launch per bounce.
__global__ void __launch_bounds__(kGTile, kGuidedMinBlocks) k_sshade_guided(StreamArgs p) {
    const int n = p.ctr[kCtrClass0 + kMatLambert];
    if (static_cast<int>(blockIdx.x) * kGTile >= n) return;   // no tile for this CTA
    extern __shared__ __align__(128) uint8_t sm[];
    const int64_t base = static_cast<int64_t>(kMatLambert) * p.cap;
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
        float4 o4 = make_float4(0, 0, 0, 0), d4 = make_float4(0, 0, 1, 0), b4 = o4, h4 = o4;
        float3 ps = mk(0, 0, 0), nn = mk(0, 0, 1);
        float xf[16];
        for (int k = 0; k < 16; k++) xf[k] = 0.0f;
        if (live) {
            o4 = p.qO[base + j];
            d4 = p.qD[base + j];
            b4 = p.qB[base + j];
            h4 = p.qH[base + j];
            ps = hitPoint(xyz(o4), xyz(d4), h4.x);
            nn = triNormal(p.sv.tris[__float_as_int(h4.y)]);
            guideFeatures(ps, nn, -xyz(d4), p.guideLo, p.guideInvExt, xf);
        }
        __syncthreads();   // every row of the last tile is shaded: its mixtures may go
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
        const int pix = __float_as_int(o4.w), meta = __float_as_int(d4.w), sample = __float_as_int(b4.w);
        if (live) {
            const int fi = filmIndexS(p, pix);
            const int depth = meta & 255;
            const bool spec = (meta & 256) != 0;
            if (depth < p.maxDepth && (p.guidedBounces <= 0 || depth < p.guidedBounces)) {
                const int2 sh = __ldg(&p.sv.slotShade[__float_as_int(h4.y)]);
                float3 fc;
                float pdf;
                shadeGuidedLambert(p.sv, ps, nn, p.sv.mats[sh.x], sh.y, xyz(d4), xyz(b4), spec, depth, mix.m,
                                   p.guideAlpha, p.seed, static_cast<uint32_t>(fi), static_cast<uint32_t>(sample), R,
                                   &fc, &pdf);
            } else {
                shadeHit(p.sv, hitOfRow(h4), xyz(o4), xyz(d4), xyz(b4), spec, depth, p.maxDepth, p.seed,
                         static_cast<uint32_t>(fi), static_cast<uint32_t>(sample), fi, R, false);
            }
        }
        emitShadeResultS(p, R, live, live ? filmIndexS(p, pix) : 0, pix, meta, sample);
    }
    tileKernelTeardown(sm, tmem, ok, phase, kGsOffBar);
    if (!ok && threadIdx.x == 0) atomicOr(&p.ctr[kCtrErr], 2);
}

template <bool STATS, bool BATCH>
__global__ void __launch_bounds__(kTraceBlock, kTraceMinBlocks) k_sshadow(StreamArgs p) {
    __shared__ uint2 stack[kStackShared * kTraceBlock];
    const int n = p.ctr[kCtrShadow];
    float4 *film = filmOf(p);
    bool overflow = false;
    uint32_t nodeCount = 0, triCount = 0;
    auto done = [&](int i, const TraceLane &L) {
        if (i >= 0 && !L.found) {
            const float3 c = xyz(p.shL[i]);
            atomicAdd(&film[__float_as_int(p.shO[i].w)], make_float4(c.x, c.y, c.z, 0.0f));
        }
    };
    if constexpr (BATCH) {
        auto fetch = [&](int i, float3 *o, float3 *d, float *t0, float *t1, uint32_t *root) {
            const float4 d4 = p.shD[i];
            *o = xyz(p.shO[i]);
            *d = xyz(d4);
            *t0 = 0.0f;
            *t1 = d4.w;
            *root = p.renders[__float_as_int(p.shL[i].w)].root;
        };
        tracePersistent<true, STATS>(p.sv.nodes, p.sv.tris, p.sv.nNodes, p.sv.nTris, n, &p.ctr[kCtrFetchS],
                                     stack + threadIdx.x, kTraceBlock, &nodeCount, &triCount, &overflow, fetch, done);
    } else {
        auto fetch = [&](int i, float3 *o, float3 *d, float *t0, float *t1) {
            const float4 d4 = p.shD[i];
            *o = xyz(p.shO[i]);
            *d = xyz(d4);
            *t0 = 0.0f;
            *t1 = d4.w;
        };
        tracePersistent<true, STATS>(p.sv.nodes, p.sv.tris, p.sv.nNodes, p.sv.nTris, n, &p.ctr[kCtrFetchS],
                                     stack + threadIdx.x, kTraceBlock, &nodeCount, &triCount, &overflow, fetch, done);
    }
    if (overflow) atomicOr(&p.ctr[kCtrErr], 1);
    if (STATS) {
        atomicAdd(&p.big[kBigVisit + 2], static_cast<unsigned long long>(nodeCount));
        atomicAdd(&p.big[kBigVisit + 3], static_cast<unsigned long long>(triCount));
    }
}

// one thread: account the iteration, hand the continuations to the next one, reset the
// per-iteration counters, raise the done flag once no path is left.  Batches also stamp
// the completion time of every render whose paths have all ended (all the block's
// threads, renders strided over them), and set the device loop's condition: another
// round while paths remain and the iteration limit is not reached.
template <bool BATCH>
__global__ void k_sadvance(StreamArgs p) {
    if (blockIdx.x != 0) return;
    if constexpr (BATCH) {
        // completion stamps, the renders strided over the block's threads
        unsigned long long now;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
        for (int r = threadIdx.x; r < p.nRenders; r += blockDim.x) {
            const unsigned long long paths = static_cast<unsigned long long>(p.pathStart[r + 1] - p.pathStart[r]);
            if (p.times[1 + r] == 0 && atomicAdd(&p.ended[r], 0ull) == paths) atomicCAS(&p.times[1 + r], 0ull, now);
        }
    }
    if (threadIdx.x != 0) return;
    const int nNew = newPaths(p);
    const int n = p.ctr[kCtrRays] + nNew;
    p.big[kBigStarted] += static_cast<unsigned long long>(nNew);
    p.big[kBigPaths] += static_cast<unsigned long long>(nNew);
    p.big[kBigClosest] += static_cast<unsigned long long>(n);
    p.big[kBigShadow] += static_cast<unsigned long long>(p.ctr[kCtrShadow]);
    p.ctr[kCtrRays] = p.ctr[kCtrCont];
    for (int k = kCtrCont; k <= kCtrFetchS; k++) p.ctr[k] = 0;
    if (n > 0) p.ctr[kCtrIter] += 1;
    const bool done = p.ctr[kCtrRays] == 0 && static_cast<long long>(p.big[kBigStarted]) >= totalPaths(p);
    p.ctr[kCtrDone] = done ? 1 : 0;
    if constexpr (BATCH) {
        const long long iters = static_cast<long long>(++p.big[kBigIters]);
        if (!done && iters >= p.iterLimit) p.ctr[kCtrErr] |= 4;   // the pool did not drain in time
        if (p.devLoop) cudaGraphSetConditional(p.cond, !done && iters < p.iterLimit ? 1u : 0u);
    }
}

enum KernelClassS { kSRegen = 0, kSExtend, kSShadeL, kSShadeC, kSShadeD, kSShadow, kSAdvance, kSNumClasses };

struct GridsS {
    int trace, shade, regen, guided;
};

GridsS streamGrids(int device, int cap, bool guided) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    int occT = 0, occS = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occT, k_sextend<false, false>, kTraceBlock, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occS, k_sshade<0, false>, kShadeBlockS, 0);
    GridsS g;
    g.trace = sms * std::max(occT, 1);
    g.shade = sms * std::max(occS, 1);
    g.regen = std::max(1, std::min((cap + 255) / 256, sms * 8));
    g.guided = guided ? guideTileKernelGrid(reinterpret_cast<const void *>(k_sshade_guided), device, kGsSmem) : 0;
    return g;
}

// one iteration on stream s; with ev, every kernel is bracketed by a pair of events
template <bool STATS, bool BATCH = false>
void launchIteration(const StreamArgs &a, const GridsS &g, cudaStream_t s, cudaEvent_t *ev, int *evClass,
                     int *nev) {
    auto mark = [&](int cls) {
        if (ev) {
            evClass[*nev / 2] = cls;
            cudaEventRecord(ev[(*nev)++], s);
        }
    };
    auto done = [&]() {
        if (ev) cudaEventRecord(ev[(*nev)++], s);
    };
    mark(kSRegen);
    k_sregen<BATCH><<<g.regen, 256, 0, s>>>(a);
    done();
    mark(kSExtend);
    k_sextend<STATS, BATCH><<<g.trace, kTraceBlock, 0, s>>>(a);
    done();
    mark(kSShadeL);
    if (a.packFwd) k_sshade_guided<<<g.guided, kGTile, kGsSmem, s>>>(a);
    else k_sshade<kMatLambert, BATCH><<<g.shade, kShadeBlockS, 0, s>>>(a);
    done();
    mark(kSShadeC);
    k_sshade<kMatConductor, BATCH><<<g.shade, kShadeBlockS, 0, s>>>(a);
    done();
    mark(kSShadeD);
    k_sshade<kMatDielectric, BATCH><<<g.shade, kShadeBlockS, 0, s>>>(a);
    done();
    mark(kSShadow);
    k_sshadow<STATS, BATCH><<<g.trace, kTraceBlock, 0, s>>>(a);
    done();
    mark(kSAdvance);
    k_sadvance<BATCH><<<1, BATCH ? 256 : 32, 0, s>>>(a);
    done();
}

uint64_t hashBytesS(const void *d, size_t n, uint64_t h = 1469598103934665603ull) {
    const unsigned char *c = static_cast<const unsigned char *>(d);
    for (size_t i = 0; i < n; i++) h = (h ^ c[i]) * 1099511628211ull;
    return h;
}

int ensureStreamQueues(StreamQueues &q, int cap) {
    if (q.capacity >= cap && q.rO) return 0;
    freeStreamQueues(&q);
    auto alloc = [&](auto **ptr, size_t count) {
        using T = std::remove_pointer_t<std::remove_reference_t<decltype(*ptr)>>;
        return cudaMalloc(reinterpret_cast<void **>(ptr), sizeof(T) * std::max<size_t>(count, 1)) == cudaSuccess;
    };
    const size_t c = static_cast<size_t>(cap);
    bool ok = alloc(&q.rO, c) && alloc(&q.rD, c) && alloc(&q.rB, c) && alloc(&q.qO, 3 * c) && alloc(&q.qD, 3 * c) &&
              alloc(&q.qB, 3 * c) && alloc(&q.qH, 3 * c) && alloc(&q.shO, 2 * c) && alloc(&q.shD, 2 * c) &&
              alloc(&q.shL, 2 * c) && alloc(&q.ctr, kNumCtr) && alloc(&q.big, kNumBig);
    if (ok) ok = cudaMallocHost(reinterpret_cast<void **>(&q.doneHost), sizeof(int) * kDoneRing) == cudaSuccess;
    if (ok) {
        for (int k = 0; k < kDoneRing && ok; k++) ok = cudaEventCreateWithFlags(&q.doneEv[k], cudaEventDisableTiming) == cudaSuccess;
    }
    if (!ok) {
        cudaGetLastError();
        freeStreamQueues(&q);
        setError("spgpu_render: device allocation of the streaming path pool failed");
        return SPGPU_ENOMEM;
    }
    q.capacity = cap;
    return 0;
}

// the render's own parameters for the device (kBigTotal.. kBigFilm), the other counters zero
struct StreamInit {
    unsigned long long big[kNumBig];
};
StreamInit streamInit(long long total, int sampleOffset, float4 *film) {
    StreamInit s;
    std::memset(&s, 0, sizeof(s));
    s.big[kBigTotal] = static_cast<unsigned long long>(total);
    s.big[kBigOffset] = static_cast<unsigned long long>(static_cast<long long>(sampleOffset));
    s.big[kBigFilm] = reinterpret_cast<unsigned long long>(film);
    return s;
}

int setupStream(Ctx &C, StreamQueues &q, const float *camera, int W, int H, int spp, int maxDepth, uint32_t seed,
                int integrator, const GuideView *gv, StreamArgs *out) {
    const long long npix = static_cast<long long>(W) * H;
    const long long total = npix * spp;
    const int cap = static_cast<int>(std::min<long long>(std::max<long long>(total, 1), Ctx::kStreamSlots));
    if (int rc = ensureStreamQueues(q, cap)) return rc;
    StreamArgs &a = *out;
    std::memset(&a, 0, sizeof(a));
    a.sv = C.view();
    a.cam = makeCamera(camera, W, H);
    a.W = W;
    a.H = H;
    a.npix = static_cast<int>(npix);
    a.maxDepth = integrator == SPGPU_INTEGRATOR_DIRECT ? 1 : maxDepth;
    a.seed = seed;
    a.direct = integrator == SPGPU_INTEGRATOR_DIRECT ? 1 : 0;
    a.cap = q.capacity;
    a.rO = q.rO;
    a.rD = q.rD;
    a.rB = q.rB;
    a.qO = q.qO;
    a.qD = q.qD;
    a.qB = q.qB;
    a.qH = q.qH;
    a.shO = q.shO;
    a.shD = q.shD;
    a.shL = q.shL;
    a.ctr = q.ctr;
    a.big = q.big;
    if (gv) {
        a.packFwd = gv->packFwd;
        a.biasPad = gv->biasPad;
        a.guideAlpha = gv->alpha;
        a.guidedBounces = gv->guidedBounces;
        a.guideLo = C.bvh.lo;
        const float3 ext = C.bvh.hi - C.bvh.lo;
        a.guideInvExt = mk(ext.x > 0 ? 1.0f / ext.x : 0.0f, ext.y > 0 ? 1.0f / ext.y : 0.0f,
                           ext.z > 0 ? 1.0f / ext.z : 0.0f);
    }
    return 0;
}

// (re)capture the graph of kIterPerGraph iterations when anything baked into it changes
int ensureStreamGraph(Ctx &C, StreamQueues &q, const StreamArgs &a, cudaStream_t s) {
    const uint64_t key = hashBytesS(&a, sizeof(a));
    if (q.graph && q.graphKey == key) return 0;
    if (q.graph) cudaGraphExecDestroy(q.graph);
    q.graph = nullptr;
    const GridsS g = streamGrids(C.device, a.cap, a.packFwd != nullptr);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cudaFail("cudaStreamBeginCapture", e);
    for (int it = 0; it < kIterPerGraph; it++) launchIteration<false>(a, g, s, nullptr, nullptr, nullptr);
    e = cudaStreamEndCapture(s, &graph);
    if (e != cudaSuccess) return cudaFail("cudaStreamEndCapture", e);
    e = cudaGraphInstantiate(&q.graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cudaFail("cudaGraphInstantiate", e);
    q.graphKey = key;
    return 0;
}

// a generous bound on the iterations of a render: a path ends within maxDepth + 1
// iterations of its start, and a full pool is refilled at least once in that time
long long iterationBound(const StreamArgs &a, long long total) {
    return 2 * (static_cast<long long>(a.maxDepth) + 2) * (total / std::max(a.cap, 1) + 2) + 16;
}

// the start of a batch run: every lane's counters and parameters (its share of the
// batch's path sequence, the film), the per-render counts and times.  One kernel, so
// that the reset is part of the batch's graph.
struct BatchReset {
    int *ctr[Ctx::kPoolLanes];
    unsigned long long *big[Ctx::kPoolLanes];
    long long first[Ctx::kPoolLanes], count[Ctx::kPoolLanes];
    int lanes;
    int nRenders;
    unsigned long long film;
    unsigned long long *ended, *times;
};

__global__ void k_sbatch_reset(BatchReset in) {
    const int t = threadIdx.x;
    for (int k = 0; k < in.lanes; k++) {
        for (int i = t; i < kNumCtr; i += blockDim.x) in.ctr[k][i] = 0;
        for (int i = t; i < kNumBig; i += blockDim.x)
            in.big[k][i] = i == kBigTotal    ? static_cast<unsigned long long>(in.count[k])
                           : i == kBigOffset ? static_cast<unsigned long long>(in.first[k])
                           : i == kBigFilm   ? in.film
                                             : 0ull;
    }
    for (int r = t; r < in.nRenders; r += blockDim.x) {
        in.ended[r] = 0;
        in.times[1 + r] = 0;
    }
    if (t == 0) {
        unsigned long long now;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
        in.times[0] = now;
    }
}

}  // namespace

struct StreamBatch {
    int lanes = 1, iterations = 0;
    StreamQueues q[Ctx::kPoolLanes];   // the batch's own pools (the context's serve spgpu_render)
    SceneView sv{};                    // the merged scenes
    RenderMeta *renders = nullptr;     // device
    long long *pathStart = nullptr;    // device, nRenders + 1
    unsigned long long *ended = nullptr, *times = nullptr;
    int nRenders = 0, maxDepth = 0;
    std::vector<long long> hostStart;
    cudaGraphExec_t exec = nullptr;
    float4 *execFilm = nullptr;
};

void freeStreamBatch(StreamBatch *SB) {
    if (!SB) return;
    if (SB->exec) cudaGraphExecDestroy(SB->exec);
    for (auto &q : SB->q) freeStreamQueues(&q);
    cudaFree(SB->renders);
    cudaFree(SB->pathStart);
    cudaFree(SB->ended);
    cudaFree(SB->times);
    delete SB;
}

int streamBatchCreate(Ctx &C, StreamBatch **slot, const SceneView &merged, const std::vector<RenderMeta> &renders,
                      int poolSlots, int lanes, int iterations) {
    freeStreamBatch(*slot);
    *slot = nullptr;
    // a path carries its render in bits 9..30 of its meta word
    if (renders.empty() || renders.size() >= (1u << 22) || poolSlots <= 0 || lanes < 1 || lanes > Ctx::kPoolLanes ||
        iterations < 1) {
        setError("spgpu_batch_prepare: invalid streaming batch shape (at most 2^22 - 1 renders)");
        return SPGPU_EINVAL;
    }
    auto *SB = new StreamBatch();
    SB->lanes = lanes;
    SB->iterations = iterations;
    SB->sv = merged;
    SB->nRenders = static_cast<int>(renders.size());
    SB->hostStart.assign(renders.size() + 1, 0);
    for (size_t r = 0; r < renders.size(); r++) {
        const RenderMeta &M = renders[r];
        SB->hostStart[r + 1] = SB->hostStart[r] + static_cast<long long>(M.W) * M.H * M.spp;
        SB->maxDepth = std::max(SB->maxDepth, M.maxDepth);
    }
    const long long total = SB->hostStart.back();
    const int cap = static_cast<int>(std::min<long long>(poolSlots, std::max<long long>(1, (total + lanes - 1) / lanes)));
    int rc = 0;
    for (int k = 0; k < lanes && rc == 0; k++) rc = ensureStreamQueues(SB->q[k], cap);
    cudaError_t e = cudaSuccess;
    if (rc == 0) e = cudaMalloc(&SB->renders, sizeof(RenderMeta) * renders.size());
    if (rc == 0 && e == cudaSuccess) e = cudaMalloc(&SB->pathStart, sizeof(long long) * SB->hostStart.size());
    if (rc == 0 && e == cudaSuccess) e = cudaMalloc(&SB->ended, sizeof(unsigned long long) * renders.size());
    if (rc == 0 && e == cudaSuccess) e = cudaMalloc(&SB->times, sizeof(unsigned long long) * (renders.size() + 1));
    if (rc == 0 && e == cudaSuccess)
        e = cudaMemcpy(SB->renders, renders.data(), sizeof(RenderMeta) * renders.size(), cudaMemcpyHostToDevice);
    if (rc == 0 && e == cudaSuccess)
        e = cudaMemcpy(SB->pathStart, SB->hostStart.data(), sizeof(long long) * SB->hostStart.size(),
                       cudaMemcpyHostToDevice);
    if (rc == 0 && e != cudaSuccess) rc = cudaFail("spgpu_batch_prepare", e);
    if (rc) {
        freeStreamBatch(SB);
        return rc;
    }
    *slot = SB;
    return 0;
}

namespace {

// the lane's kernel arguments: the merged scenes, the lane's pool, the batch tables
StreamArgs batchLaneArgs(const StreamBatch &SB, int k, cudaGraphConditionalHandle cond) {
    StreamArgs a;
    std::memset(&a, 0, sizeof(a));
    const StreamQueues &q = SB.q[k];
    a.sv = SB.sv;
    a.maxDepth = SB.maxDepth;
    a.cap = q.capacity;
    a.rO = q.rO;
    a.rD = q.rD;
    a.rB = q.rB;
    a.qO = q.qO;
    a.qD = q.qD;
    a.qB = q.qB;
    a.qH = q.qH;
    a.shO = q.shO;
    a.shD = q.shD;
    a.shL = q.shL;
    a.ctr = q.ctr;
    a.big = q.big;
    a.renders = SB.renders;
    a.pathStart = SB.pathStart;
    a.nRenders = SB.nRenders;
    a.ended = SB.ended;
    a.times = SB.times;
    a.cond = cond;
    return a;
}

// The batch's graph: the reset kernel, then per lane a conditional while node whose
// body is `iterations` wavefront iterations; the body's last k_sadvance decides
// whether the loop goes round again.  Film address baked in (recaptured per film).
int buildBatchGraph(Ctx &C, StreamBatch &SB, float4 *film) {
    if (SB.exec) cudaGraphExecDestroy(SB.exec);
    SB.exec = nullptr;
    const long long total = SB.hostStart.back();
    BatchReset init;
    std::memset(&init, 0, sizeof(init));
    init.lanes = SB.lanes;
    init.nRenders = SB.nRenders;
    init.film = reinterpret_cast<unsigned long long>(film);
    init.ended = SB.ended;
    init.times = SB.times;
    for (int k = 0; k < SB.lanes; k++) {
        init.ctr[k] = SB.q[k].ctr;
        init.big[k] = SB.q[k].big;
        init.first[k] = total * k / SB.lanes;
        init.count[k] = total * (k + 1) / SB.lanes - init.first[k];
    }
    cudaStream_t cs = C.stream;
    cudaGraph_t G = nullptr;
    cudaError_t e = cudaGraphCreate(&G, 0);
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(cs, G, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        k_sbatch_reset<<<1, 256, 0, cs>>>(init);
        e = cudaStreamEndCapture(cs, &G);
    }
    cudaGraphNode_t resetNode = nullptr;
    size_t nNodes = 1;
    if (e == cudaSuccess) e = cudaGraphGetNodes(G, &resetNode, &nNodes);
    const GridsS g = streamGrids(C.device, SB.q[0].capacity, false);
    for (int k = 0; k < SB.lanes && e == cudaSuccess; k++) {
        cudaGraphConditionalHandle h = 0;
        e = cudaGraphConditionalHandleCreate(&h, G, 1, cudaGraphCondAssignDefault);
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node = nullptr;
        if (e == cudaSuccess) e = cudaGraphAddNode(&node, G, &resetNode, nullptr, 1, &cp);
        if (e != cudaSuccess) break;
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        StreamArgs a = batchLaneArgs(SB, k, h);
        a.devLoop = 1;
        a.iterLimit = iterationBound(a, init.count[k]);
        e = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) break;
        for (int it = 0; it < SB.iterations; it++) launchIteration<false, true>(a, g, cs, nullptr, nullptr, nullptr);
        e = cudaStreamEndCapture(cs, &body);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&SB.exec, G, 0);
    if (G) cudaGraphDestroy(G);
    if (e != cudaSuccess) {
        SB.exec = nullptr;
        return cudaFail("spgpu_batch_run (graph)", e);
    }
    SB.execFilm = film;
    return 0;
}

}  // namespace

int streamBatchRun(Ctx &C, StreamBatch &SB, float4 *film, double *renderMs, unsigned long long *statsOut,
                   float *msOut, cudaStream_t stream) {
    if (!SB.exec || SB.execFilm != film) {
        if (int rc = buildBatchGraph(C, SB, film)) return rc;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaError_t e = cudaEventRecord(e0, stream);
    if (e == cudaSuccess) e = cudaGraphLaunch(SB.exec, stream);
    if (e == cudaSuccess) e = cudaEventRecord(e1, stream);
    std::vector<unsigned long long> times(SB.nRenders + 1);
    unsigned long long big[Ctx::kPoolLanes][kNumBig] = {};
    int ctr[Ctx::kPoolLanes][kNumCtr] = {};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(times.data(), SB.times, sizeof(unsigned long long) * times.size(), cudaMemcpyDeviceToHost,
                            stream);
    for (int k = 0; k < SB.lanes && e == cudaSuccess; k++) {
        e = cudaMemcpyAsync(big[k], SB.q[k].big, sizeof(big[k]), cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(ctr[k], SB.q[k].ctr, sizeof(ctr[k]), cudaMemcpyDeviceToHost, stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    float ms = 0.0f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cudaFail("spgpu_batch_run", e);
    int err = 0;
    bool drained = true;
    for (int k = 0; k < 4; k++) statsOut[k] = 0;
    for (int k = 0; k < SB.lanes; k++) {
        statsOut[0] += big[k][kBigPaths];
        statsOut[1] += big[k][kBigClosest];
        statsOut[2] += big[k][kBigShadow];
        statsOut[3] += big[k][kBigIters] * kSNumClasses + 1;
        err |= ctr[k][kCtrErr];
        drained = drained && ctr[k][kCtrDone];
    }
    for (int r = 0; r < SB.nRenders; r++)
        renderMs[r] = times[1 + r] >= times[0] && times[1 + r] ? (times[1 + r] - times[0]) * 1.0e-6 : -1.0;
    *msOut = ms;
    if (err & 1) {
        setError("spgpu_batch_run: traversal stack overflow");
        return SPGPU_EKERNEL;
    }
    if ((err & 4) || !drained) {
        setError("spgpu_batch_run: the path pools did not drain within their iteration bound");
        return SPGPU_EKERNEL;
    }
    return 0;
}

void freeStreamQueues(StreamQueues *q) {
    if (q->graph) cudaGraphExecDestroy(q->graph);
    cudaFree(q->rO);
    cudaFree(q->rD);
    cudaFree(q->rB);
    cudaFree(q->qO);
    cudaFree(q->qD);
    cudaFree(q->qB);
    cudaFree(q->qH);
    cudaFree(q->shO);
    cudaFree(q->shD);
    cudaFree(q->shL);
    cudaFree(q->ctr);
    cudaFree(q->big);
    if (q->doneHost) cudaFreeHost(q->doneHost);
    for (int k = 0; k < StreamQueues::kEvents; k++)
        if (q->doneEv[k]) cudaEventDestroy(q->doneEv[k]);
    *q = StreamQueues{};
}

int renderStream(Ctx *ctx, const float *camera, int W, int H, int spp, int sampleOffset, int maxDepth, uint32_t seed,
                 int integrator, float4 *film, unsigned long long *statsOut, float *msOut, cudaStream_t stream,
                 const GuideView *gv) {
    Ctx &C = *ctx;
    for (int j = 0; j < 4; j++) statsOut[j] = 0;
    *msOut = 0.0f;
    if (spp <= 0 || W <= 0 || H <= 0) return 0;
    // pool lanes: lane k renders a contiguous share of the samples, lane 0 on the caller's
    // stream, lane k > 0 on the context's lane stream k - 1
    const int lanes = std::max(1, std::min(spp, Ctx::kPoolLanes));
    StreamArgs a[Ctx::kPoolLanes];
    StreamInit init[Ctx::kPoolLanes];
    cudaStream_t ls[Ctx::kPoolLanes];
    long long maxReplays[Ctx::kPoolLanes], replays[Ctx::kPoolLanes];
    bool finished[Ctx::kPoolLanes];
    int first = sampleOffset;
    for (int k = 0; k < lanes; k++) {
        const int sppK = spp / lanes + (k < spp % lanes ? 1 : 0);
        if (int rc = setupStream(C, C.sq[k], camera, W, H, sppK, maxDepth, seed, integrator, gv, &a[k])) return rc;
        // captured on the context's own stream (the caller's may be the legacy default
        // stream, which cannot be captured), replayed on the lane's
        if (int rc = ensureStreamGraph(C, C.sq[k], a[k], C.stream)) return rc;
        const long long total = static_cast<long long>(W) * H * sppK;
        init[k] = streamInit(total, first, film);
        first += sppK;
        ls[k] = k == 0 ? stream : C.laneStream[k - 1];
        maxReplays[k] = iterationBound(a[k], total) / kIterPerGraph + kReplayLag + 2;
        replays[k] = 0;
        finished[k] = false;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaError_t e = cudaEventRecord(e0, stream);
    if (e == cudaSuccess && lanes > 1) e = cudaEventRecord(C.laneFork, stream);
    for (int k = 0; k < lanes && e == cudaSuccess; k++) {
        StreamQueues &q = C.sq[k];
        if (k > 0) e = cudaStreamWaitEvent(ls[k], C.laneFork, 0);
        if (e == cudaSuccess) e = cudaMemsetAsync(q.ctr, 0, sizeof(int) * kNumCtr, ls[k]);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(q.big, init[k].big, sizeof(init[k].big), cudaMemcpyHostToDevice, ls[k]);
    }
    // replay each lane's graph until its pool drains, reading each lane's done flag
    // kReplayLag replays back
    int open = lanes;
    while (e == cudaSuccess && open > 0) {
        for (int k = 0; k < lanes && e == cudaSuccess; k++) {
            if (finished[k]) continue;
            StreamQueues &q = C.sq[k];
            if (replays[k] >= maxReplays[k]) {
                finished[k] = true;   // reported below: the done flag stays unset
                open--;
                continue;
            }
            const int slot = static_cast<int>(replays[k] % kDoneRing);
            e = cudaGraphLaunch(q.graph, ls[k]);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(&q.doneHost[slot], q.ctr + kCtrDone, sizeof(int), cudaMemcpyDeviceToHost, ls[k]);
            if (e == cudaSuccess) e = cudaEventRecord(q.doneEv[slot], ls[k]);
            replays[k]++;
            if (e == cudaSuccess && replays[k] > kReplayLag) {
                const int back = static_cast<int>((replays[k] - 1 - kReplayLag) % kDoneRing);
                e = cudaEventSynchronize(q.doneEv[back]);
                if (e == cudaSuccess && q.doneHost[back]) {
                    finished[k] = true;
                    open--;
                }
            }
        }
    }
    for (int k = 1; k < lanes && e == cudaSuccess; k++) {
        e = cudaEventRecord(C.laneJoin[k - 1], ls[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, C.laneJoin[k - 1], 0);
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, stream);
    unsigned long long big[Ctx::kPoolLanes][kNumBig] = {};
    int ctr[Ctx::kPoolLanes][kNumCtr] = {};
    for (int k = 0; k < lanes && e == cudaSuccess; k++) {
        e = cudaMemcpyAsync(big[k], C.sq[k].big, sizeof(big[k]), cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(ctr[k], C.sq[k].ctr, sizeof(ctr[k]), cudaMemcpyDeviceToHost, stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    float ms = 0.0f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cudaFail("spgpu_render", e);
    int err = 0;
    bool drained = true;
    for (int k = 0; k < lanes; k++) {
        statsOut[0] += big[k][kBigPaths];
        statsOut[1] += big[k][kBigClosest];
        statsOut[2] += big[k][kBigShadow];
        statsOut[3] += static_cast<unsigned long long>(replays[k]) * kIterPerGraph * kSNumClasses;
        err |= ctr[k][kCtrErr];
        drained = drained && ctr[k][kCtrDone];
    }
    *msOut = ms;
    if (err) {
        setError(err & 1 ? "spgpu_render: traversal stack overflow"
                         : "spgpu_render: tensor-core wait of the guided shading timed out");
        return SPGPU_EKERNEL;
    }
    if (!drained) {
        setError("spgpu_render: the path pool did not drain within its iteration bound");
        return SPGPU_EKERNEL;
    }
    return 0;
}

int renderStreamProfile(Ctx *ctx, const float *camera, int W, int H, int spp, int sampleOffset, int maxDepth,
                        uint32_t seed, int integrator, float4 *film, double *kernelMs, long long *launches,
                        unsigned long long *statsOut, unsigned long long *visitOut, cudaStream_t stream,
                        const GuideView *gv) {
    Ctx &C = *ctx;
    for (int k = 0; k < kSNumClasses; k++) {
        kernelMs[k] = 0.0;
        launches[k] = 0;
    }
    for (int k = 0; k < 4; k++) statsOut[k] = visitOut[k] = 0;
    if (spp <= 0 || W <= 0 || H <= 0) return 0;
    StreamArgs a;
    StreamQueues &q = C.sq[0];
    if (int rc = setupStream(C, q, camera, W, H, spp, maxDepth, seed, integrator, gv, &a)) return rc;
    const GridsS g = streamGrids(C.device, a.cap, a.packFwd != nullptr);
    const long long total = static_cast<long long>(W) * H * spp;
    const StreamInit init = streamInit(total, sampleOffset, film);
    const long long bound = iterationBound(a, total);
    std::vector<cudaEvent_t> ev(2 * 7);
    std::vector<int> cls(8);
    for (auto &x : ev) cudaEventCreate(&x);
    unsigned long long big[kNumBig] = {};
    int ctr[kNumCtr] = {};
    cudaError_t e = cudaSuccess;
    // pass 0: every kernel timed by events, one iteration at a time; pass 1: the same
    // paths again with the visit counters on
    for (int pass = 0; pass < 2 && e == cudaSuccess; pass++) {
        e = cudaMemsetAsync(q.ctr, 0, sizeof(int) * kNumCtr, stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(q.big, init.big, sizeof(init.big), cudaMemcpyHostToDevice, stream);
        for (long long it = 0; it < bound && e == cudaSuccess; it++) {
            int nev = 0;
            if (pass == 0) launchIteration<false>(a, g, stream, ev.data(), cls.data(), &nev);
            else launchIteration<true>(a, g, stream, nullptr, nullptr, nullptr);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaMemcpyAsync(ctr, q.ctr, sizeof(ctr), cudaMemcpyDeviceToHost, stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
            for (int i = 0; i + 1 < nev && e == cudaSuccess; i += 2) {
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
                kernelMs[cls[i / 2]] += ms;
                launches[cls[i / 2]] += 1;
            }
            if (ctr[kCtrDone]) break;
        }
        if (e == cudaSuccess) e = cudaMemcpy(big, q.big, sizeof(big), cudaMemcpyDeviceToHost);
        if (pass == 0)
            for (int k = 0; k < 3; k++) statsOut[k] = big[kBigPaths + k];
        else
            for (int k = 0; k < 4; k++) visitOut[k] = big[kBigVisit + k];
    }
    for (auto &x : ev) cudaEventDestroy(x);
    if (e != cudaSuccess) return cudaFail("spgpu_render_profile", e);
    if (ctr[kCtrErr]) {
        setError(ctr[kCtrErr] & 1 ? "spgpu_render_profile: traversal stack overflow"
                                  : "spgpu_render_profile: tensor-core wait of the guided shading timed out");
        return SPGPU_EKERNEL;
    }
    return 0;
}

}  // namespace spgpu

namespace spgpu {

// The batch's streaming wavefront launched kernel by kernel from the host (no graph),
// lane 0's pool taking the whole path sequence: pass 0 times every kernel with events,
// pass 1 renders the same paths again with the BVH visit counters on (the film receives
// both passes).  kernelMs/launches per kernel class.
int streamBatchProfile(Ctx &C, StreamBatch &SB, float4 *film, double *kernelMs, long long *launches,
                       unsigned long long *statsOut, unsigned long long *visitOut, cudaStream_t stream) {
    for (int k = 0; k < kSNumClasses; k++) {
        kernelMs[k] = 0.0;
        launches[k] = 0;
    }
    for (int k = 0; k < 4; k++) statsOut[k] = visitOut[k] = 0;
    StreamArgs a = batchLaneArgs(SB, 0, 0);
    const long long total = SB.hostStart.back();
    a.iterLimit = iterationBound(a, total);
    BatchReset init;
    std::memset(&init, 0, sizeof(init));
    init.lanes = 1;
    init.nRenders = SB.nRenders;
    init.film = reinterpret_cast<unsigned long long>(film);
    init.ended = SB.ended;
    init.times = SB.times;
    init.ctr[0] = SB.q[0].ctr;
    init.big[0] = SB.q[0].big;
    init.first[0] = 0;
    init.count[0] = total;
    const GridsS g = streamGrids(C.device, a.cap, false);
    std::vector<cudaEvent_t> ev(2 * kSNumClasses);
    std::vector<int> cls(kSNumClasses + 1);
    for (auto &x : ev) cudaEventCreate(&x);
    unsigned long long big[kNumBig] = {};
    int ctr[kNumCtr] = {};
    cudaError_t e = cudaSuccess;
    for (int pass = 0; pass < 2 && e == cudaSuccess; pass++) {
        k_sbatch_reset<<<1, 256, 0, stream>>>(init);
        e = cudaGetLastError();
        for (long long it = 0; it < a.iterLimit && e == cudaSuccess; it++) {
            int nev = 0;
            if (pass == 0) launchIteration<false, true>(a, g, stream, ev.data(), cls.data(), &nev);
            else launchIteration<true, true>(a, g, stream, nullptr, nullptr, nullptr);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaMemcpyAsync(ctr, SB.q[0].ctr, sizeof(ctr), cudaMemcpyDeviceToHost, stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
            for (int i = 0; i + 1 < nev && e == cudaSuccess; i += 2) {
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
                kernelMs[cls[i / 2]] += ms;
                launches[cls[i / 2]] += 1;
            }
            if (ctr[kCtrDone]) break;
        }
        if (e == cudaSuccess) e = cudaMemcpy(big, SB.q[0].big, sizeof(big), cudaMemcpyDeviceToHost);
        if (pass == 0)
            for (int k = 0; k < 3; k++) statsOut[k] = big[kBigPaths + k];
        else
            for (int k = 0; k < 4; k++) visitOut[k] = big[kBigVisit + k];
    }
    for (auto &x : ev) cudaEventDestroy(x);
    if (e != cudaSuccess) return cudaFail("spgpu_batch_profile", e);
    if (ctr[kCtrErr] & 1) {
        setError("spgpu_batch_profile: traversal stack overflow");
        return SPGPU_EKERNEL;
    }
    if (!ctr[kCtrDone]) {
        setError("spgpu_batch_profile: the path pool did not drain within its iteration bound");
        return SPGPU_EKERNEL;
    }
    return 0;
}

}  // namespace spgpu
