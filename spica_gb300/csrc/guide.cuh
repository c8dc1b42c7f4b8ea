// guide.cuh -- the learned path-guiding proposal: a 9 -> 64 -> 64 -> 64 -> 40 MLP
// (BF16 weights, FP32 accumulation) mapping (position, normal, outgoing direction) at a
// shading point to an 8-lobe von Mises-Fisher mixture over incident directions.
// This part has no counterpart in the reference renderer.
//
// The dense layers run on the 5th-generation tensor cores: a CTA of 128 threads
// evaluates a tile of 128 samples; each layer is tcgen05.mma (M = 128, N = 64 or 48,
// K = 16 per instruction) from bf16 operands in shared memory into an FP32 accumulator
// in tensor memory, whose epilogue (tcgen05.ld, bias, ReLU, bf16) writes the next
// layer's operand back to shared memory.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"
#include "tc.cuh"

namespace spgpu {

constexpr int kGIn = 9;      // inputs
constexpr int kGK0 = 16;     // inputs padded to the MMA's K step
constexpr int kGHid = 64;    // hidden width
constexpr int kGOut = 40;    // outputs: 8 lobes x (direction 3, log-concentration, weight logit)
constexpr int kGN4 = 48;     // outputs padded to a multiple of 16
constexpr int kGLobes = 8;
constexpr int kGTile = 128;  // samples per CTA tile (= MMA M)

// fp32 master parameters, each layer [out][in] row-major followed by its bias
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kGHid * kGIn;
constexpr int kOffW2 = kOffB1 + kGHid;
constexpr int kOffB2 = kOffW2 + kGHid * kGHid;
constexpr int kOffW3 = kOffB2 + kGHid;
constexpr int kOffB3 = kOffW3 + kGHid * kGHid;
constexpr int kOffW4 = kOffB3 + kGHid;
constexpr int kOffB4 = kOffW4 + kGOut * kGHid;
constexpr int kGParams = kOffB4 + kGOut;   // 11,560

// packed bf16 MMA operands (canonical K-major tiles, tc.cuh):
//   forward  B_l = W_l as [N = out][K = in]:  W1f 64x16 | W2f 64x64 | W3f 64x64 | W4f 48x64
//   backward B_l = W_l^T as [N = in][K = out]:            W2b 64x64 | W3b 64x64 | W4b 64x48
constexpr int kW1fBytes = kGHid * kGK0 * 2;
constexpr int kW2fBytes = kGHid * kGHid * 2;
constexpr int kW4fBytes = kGN4 * kGHid * 2;
constexpr int kPackFwdBytes = kW1fBytes + 2 * kW2fBytes + kW4fBytes;   // 24,576
constexpr int kW4bBytes = kGHid * kGN4 * 2;
constexpr int kPackBwdBytes = 2 * kW2fBytes + kW4bBytes;               // 22,528
constexpr int kBiasPad = 3 * kGHid + kGN4;                             // 240

constexpr uint32_t kMmaWaitTries = 1u << 22;

// shared memory of a kernel that evaluates the network for its 128-thread CTA, one tile
// at a time: packed forward weights | biases (padded to 1 KB) | input/hidden tile (bf16
// [128][64]) | MMA mbarrier, TMEM slot, load mbarrier
constexpr int kTileSmOffBias = kPackFwdBytes;
constexpr int kTileSmOffXH = kTileSmOffBias + 1024;
constexpr int kTileSmOffBar = kTileSmOffXH + kGTile * kGHid * 2;
constexpr int kTileSmem = kTileSmOffBar + 24;
static_assert(kBiasPad * 4 % 16 == 0 && kPackFwdBytes % 16 == 0, "bulk copies move multiples of 16 bytes");

// Bounded wait of all threads for a bulk load announced on *bar (phase 0); false if it
// did not complete within kMmaWaitTries polls (CTA-wide result)
__device__ __forceinline__ bool bulkLoadWait(uint64_t *bar) {
    const bool ok = tc::mbarWait(bar, 0, kMmaWaitTries);
    return __syncthreads_and(ok) != 0;
}

// ---------------------------------------------------------------- vMF mixture
struct Mixture {
    float3 mu[kGLobes];
    float kappa[kGLobes];
    float w[kGLobes];
    float wn[kGLobes];   // w times the lobe's normalisation, for the pdf
};

__device__ __forceinline__ float vmfNorm(float kappa) {   // kappa / (2 pi (1 - exp(-2 kappa)))
    return kappa / (2.0f * kPi * -expm1f(-2.0f * kappa));
}
__device__ __forceinline__ float vmfPdf(float3 w, float3 mu, float kappa) {
    return vmfNorm(kappa) * __expf(kappa * (dot(mu, w) - 1.0f));
}
__device__ __forceinline__ float kappaOf(float raw) { return __expf(clampf(raw, -4.0f, 7.0f)); }

// The mixture as the shading kernels sample and evaluate it.  They compute it with the
// hardware's approximate reciprocal, reciprocal square root and exponential: sampling
// and pdf evaluation read the same lobes, so the one-sample MIS estimator stays
// unbiased, and each row's mixture costs a few dozen special-function instructions
// instead of IEEE divisions and expm1 (training keeps the accurate forms, vmfNorm).
__device__ __forceinline__ float3 normalizeFast(float3 v) { return v * rsqrtf(dot(v, v)); }
// kappa / (2 pi (1 - exp(-2 kappa))) for kappa in [e^-4, e^7] (kappaOf's range); the
// cancellation in 1 - exp(-2 kappa) costs at most ~4e-6 relative at the smallest kappa
__device__ __forceinline__ float vmfNormFast(float kappa) {
    return __fdividef(kappa, 2.0f * kPi * (1.0f - __expf(-2.0f * kappa)));
}

// raw network outputs -> mixture (unit lobe axes, concentrations, softmax weights)
__device__ __forceinline__ void mixtureFromRaw(const float *raw, Mixture &M) {
    float mx = -3.0e38f;
#pragma unroll
    for (int k = 0; k < kGLobes; k++) mx = fmaxf(mx, raw[5 * k + 4]);
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < kGLobes; k++) {
        const float3 m = mk(raw[5 * k], raw[5 * k + 1], raw[5 * k + 2]);
        const float len2 = dot(m, m);
        M.mu[k] = len2 > 1.0e-24f ? m * rsqrtf(len2) : mk(0.0f, 0.0f, 1.0f);
        M.kappa[k] = kappaOf(raw[5 * k + 3]);
        M.w[k] = __expf(raw[5 * k + 4] - mx);
        s += M.w[k];
    }
    const float is = __fdividef(1.0f, s);
#pragma unroll
    for (int k = 0; k < kGLobes; k++) {
        M.w[k] *= is;
        M.wn[k] = M.w[k] * vmfNormFast(M.kappa[k]);
    }
}
__device__ __forceinline__ float mixturePdf(const Mixture &M, float3 w) {
    float p = 0.0f;
    for (int k = 0; k < kGLobes; k++) p += M.wn[k] * __expf(M.kappa[k] * (dot(M.mu[k], w) - 1.0f));
    return p;
}
// Sampling a vMF lobe with the numerically stable inversion of W. Jakob, "Numerically
// stable sampling of the von Mises Fisher distribution on S^2 (and other tricks)" (2012).
__device__ __forceinline__ float3 vmfSample(float3 mu, float kappa, float u1, float u2) {
    const float e = __expf(-2.0f * kappa);
    const float c = 1.0f + __fdividef(__logf(u1 + (1.0f - u1) * e), kappa);
    const float cc = clampf(c, -1.0f, 1.0f);
    const float s = sqrtf(fmaxf(0.0f, 1.0f - cc * cc));
    float sp, cp;
    __sincosf(2.0f * kPi * u2, &sp, &cp);
    // the frame of onb() (Duff et al. 2017) with the approximate reciprocal: |s + mu.z| >= 1
    const float sg = copysignf(1.0f, mu.z);
    const float a = -__fdividef(1.0f, sg + mu.z);
    const float cxy = mu.x * mu.y * a;
    const float3 t = mk(1.0f + sg * mu.x * mu.x * a, sg * cxy, -sg * mu.x);
    const float3 b = mk(cxy, sg + mu.y * mu.y * a, -mu.y);
    return normalizeFast(t * (s * cp) + b * (s * sp) + mu * cc);
}
__device__ __forceinline__ float3 mixtureSample(const Mixture &M, float uLobe, float u1, float u2) {
    int k = 0;
    float acc = M.w[0];
    while (k < kGLobes - 1 && uLobe >= acc) {
        k++;
        acc += M.w[k];
    }
    return vmfSample(M.mu[k], M.kappa[k], u1, u2);
}

// network inputs: position normalised to the scene box, shading normal, outgoing dir
__device__ __forceinline__ void guideFeatures(float3 p, float3 n, float3 wo, float3 lo, float3 invExt, float *x) {
    x[0] = (p.x - lo.x) * invExt.x;
    x[1] = (p.y - lo.y) * invExt.y;
    x[2] = (p.z - lo.z) * invExt.z;
    x[3] = n.x;
    x[4] = n.y;
    x[5] = n.z;
    x[6] = wo.x;
    x[7] = wo.y;
    x[8] = wo.z;
}

// ---------------------------------------------------------------- tile MLP
// write row r of a bf16 K-major canonical tile from 8 floats (one core-matrix row)
__device__ __forceinline__ void storeRow8(uint8_t *tile, uint32_t r, uint32_t k0, uint32_t K, const float *v) {
    __nv_bfloat162 p[4];
    for (int i = 0; i < 4; i++) p[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
    *reinterpret_cast<uint4 *>(tile + tc::kmajorOffset(r, k0, K)) = *reinterpret_cast<uint4 *>(p);
}
__device__ __forceinline__ float loadBf16(const uint8_t *tile, uint32_t r, uint32_t k, uint32_t K) {
    return __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(tile + tc::kmajorOffset(r, k, K)));
}

// D = A x B over K (multiple of 16) for a 128-row tile: A [128][K], B [N][K], both
// K-major canonical tiles; called by the issuing thread only
__device__ __forceinline__ void issueTileMma(uint32_t tmem, const uint8_t *a, const uint8_t *b, uint32_t K,
                                             uint32_t N) {
    const uint32_t sbo = (K / 8) * 128;
    const uint32_t idesc = tc::instrDescBf16(128, N);
    const uint32_t aAddr = tc::smemAddr(a), bAddr = tc::smemAddr(b);
    for (uint32_t j = 0; j < K / 16; j++)
        tc::mmaBf16(tmem, tc::smemDesc(aAddr + 256 * j, 128, sbo), tc::smemDesc(bAddr + 256 * j, 128, sbo), idesc,
                    j > 0 ? 1u : 0u);
}

// Runs issue() on thread 0 after making the CTA's shared-memory writes visible to the
// tensor core, commits, and waits (all threads) until every MMA it issued is done.
// Returns false on a timed-out wait (the CTA-wide result is uniform).
// withhold = true (fault injection in tests) issues nothing, so the barrier is never
// signalled and the bounded wait of maxTries polls runs out.
template <class Issue>
__device__ __forceinline__ bool mmaRun(uint64_t *bar, uint32_t &phase, Issue &&issue, bool withhold = false,
                                       uint32_t maxTries = kMmaWaitTries) {
    tc::fenceBeforeSync();
    tc::fenceAsyncShared();
    __syncthreads();
    if (threadIdx.x == 0 && !withhold) {
        tc::fenceAfterSync();
        issue();
        tc::mmaCommit(bar);
    }
    const bool ok = tc::mbarWait(bar, phase, maxTries);
    phase ^= 1u;
    const bool allOk = __syncthreads_and(ok) != 0;
    tc::fenceAfterSync();
    return allOk;
}

// D = A x B (issueTileMma), returning once the tensor core is done
__device__ __forceinline__ bool tileMma(uint32_t tmem, const uint8_t *a, const uint8_t *b, uint32_t K, uint32_t N,
                                        uint64_t *bar, uint32_t &phase, bool withhold = false,
                                        uint32_t maxTries = kMmaWaitTries) {
    return mmaRun(bar, phase, [&] { issueTileMma(tmem, a, b, K, N); }, withhold, maxTries);
}

// this thread's row (its TMEM lane) of the accumulator, columns [c0, c0 + 16)
__device__ __forceinline__ void accRow16(uint32_t tmem, uint32_t c0, float (&v)[16]) {
    const uint32_t warp = threadIdx.x >> 5;
    tc::tmemLoad16(tmem + ((warp * 32u) << 16) + c0, v);
}

// hidden-layer epilogue: relu(acc + bias) -> bf16 tile (K = 64); keeps fp32 copy if asked
__device__ __forceinline__ void hiddenEpilogue(uint32_t tmem, const float *bias, uint8_t *out) {
    const uint32_t r = threadIdx.x;
    for (uint32_t c = 0; c < kGHid; c += 16) {
        float v[16];
        accRow16(tmem, c, v);
        for (int i = 0; i < 16; i++) v[i] = fmaxf(v[i] + bias[c + i], 0.0f);
        storeRow8(out, r, c, kGHid, v);
        storeRow8(out, r, c + 8, kGHid, v + 8);
    }
}

// Full forward of one tile: x (bf16 [128][16]) -> raw outputs (fp32, out[r * stride + j],
// j < 40).  h1..h3 receive the hidden activations (may alias for inference).
__device__ __forceinline__ bool mlpForwardTile(uint32_t tmem, const uint8_t *wf, const float *bias, const uint8_t *x,
                                               uint8_t *h1, uint8_t *h2, uint8_t *h3, float *out, int stride,
                                               uint64_t *bar, uint32_t &phase) {
    const uint8_t *w1 = wf, *w2 = wf + kW1fBytes, *w3 = w2 + kW2fBytes, *w4 = w3 + kW2fBytes;
    if (!tileMma(tmem, x, w1, kGK0, kGHid, bar, phase)) return false;
    hiddenEpilogue(tmem, bias, h1);
    if (!tileMma(tmem, h1, w2, kGHid, kGHid, bar, phase)) return false;
    hiddenEpilogue(tmem, bias + kGHid, h2);
    if (!tileMma(tmem, h2, w3, kGHid, kGHid, bar, phase)) return false;
    hiddenEpilogue(tmem, bias + 2 * kGHid, h3);
    if (!tileMma(tmem, h3, w4, kGHid, kGN4, bar, phase)) return false;
    const uint32_t r = threadIdx.x;
    for (uint32_t c = 0; c < kGN4; c += 16) {
        float v[16];
        accRow16(tmem, c, v);
        for (int i = 0; i < 16; i++)
            if (c + i < kGOut) out[r * stride + c + i] = v[i] + bias[3 * kGHid + c + i];
    }
    tc::fenceBeforeSync();
    __syncthreads();
    return true;
}

// CTA prologue of such a kernel: weights and biases into shared memory by one bulk
// copy each (TMA), the MMA mbarrier, a 64-column TMEM allocation (warp 0); returns the
// TMEM base, and in *ok whether the copies arrived
__device__ __forceinline__ uint32_t tileKernelSetup(uint8_t *sm, const uint8_t *packFwd, const float *biasPad,
                                                    bool *ok, int barOff = kTileSmOffBar) {
    const int t = threadIdx.x;
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + barOff);
    uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 1);
    uint64_t *loadBar = bar + 2;
    if (t == 0) {
        tc::mbarInit(bar, 1);
        tc::mbarInit(loadBar, 1);
        tc::mbarExpectTx(loadBar, kPackFwdBytes + kBiasPad * 4);
        tc::bulkLoad(sm, packFwd, kPackFwdBytes, loadBar);
        tc::bulkLoad(sm + kTileSmOffBias, biasPad, kBiasPad * 4, loadBar);
    }
    if (t < 32) {
        tc::tmemAlloc(slot, 64);
        tc::tmemRelinquish();
    }
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    *ok = bulkLoadWait(loadBar);
    return *slot;
}
// its epilogue: after a failed (timed-out) wait, bounded waits for the copies and MMAs
// still in flight; then the TMEM allocation is released
__device__ __forceinline__ void tileKernelTeardown(uint8_t *sm, uint32_t tmem, bool ok, uint32_t phase,
                                                   int barOff = kTileSmOffBar) {
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + barOff);
    if (!ok) {
        tc::mbarWait(bar + 2, 0, kMmaWaitTries);
        tc::mbarWait(bar, phase ^ 1u, kMmaWaitTries);
    }
    tc::fenceBeforeSync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmemDealloc(tmem, 64);
}

// Shared memory of the guided shading kernels: packed forward weights | biases |
// mbarriers and TMEM slot | the input/hidden tile of the network, which once the network
// is done holds the tile's mixtures instead, one row per thread padded to an odd number
// of words (so the rows of a warp fall into distinct banks).  Keeping the 48-float
// mixture out of registers through the shading lets four CTAs share an SM.
struct MixRow {
    Mixture m;
    float pad;
};
static_assert(sizeof(MixRow) % 8 == 4, "odd word stride");
constexpr int kGsOffBar = kTileSmOffBias + 1024;
constexpr int kGsOffXH = kGsOffBar + 128;
constexpr int kGsSmem = kGsOffXH + (kGTile * kGHid * 2 > kGTile * static_cast<int>(sizeof(MixRow))
                                        ? kGTile * kGHid * 2
                                        : kGTile * static_cast<int>(sizeof(MixRow)));
static_assert(kGsOffXH % 128 == 0 && kGsOffBar % 8 == 0, "alignment");

// Forward of one tile with the outputs left in registers: thread r receives row r's 40
// raw outputs.  xh holds the bf16 input tile [128][16] on entry and is reused for the
// hidden activations (each layer's epilogue runs after the MMA that read it completed).
__device__ __forceinline__ bool mlpForwardRow(uint32_t tmem, const uint8_t *wf, const float *bias, uint8_t *xh,
                                              uint64_t *bar, uint32_t &phase, float (&raw)[kGOut]) {
    const uint8_t *w1 = wf, *w2 = wf + kW1fBytes, *w3 = w2 + kW2fBytes, *w4 = w3 + kW2fBytes;
    if (!tileMma(tmem, xh, w1, kGK0, kGHid, bar, phase)) return false;
    hiddenEpilogue(tmem, bias, xh);
    if (!tileMma(tmem, xh, w2, kGHid, kGHid, bar, phase)) return false;
    hiddenEpilogue(tmem, bias + kGHid, xh);
    if (!tileMma(tmem, xh, w3, kGHid, kGHid, bar, phase)) return false;
    hiddenEpilogue(tmem, bias + 2 * kGHid, xh);
    if (!tileMma(tmem, xh, w4, kGHid, kGN4, bar, phase)) return false;
#pragma unroll
    for (uint32_t c = 0; c < kGN4; c += 16) {
        float v[16];
        accRow16(tmem, c, v);
#pragma unroll
        for (int i = 0; i < 16; i++)
            if (c + i < kGOut) raw[c + i] = v[i] + bias[3 * kGHid + c + i];
    }
    // the next MMA on this accumulator starts with a CTA barrier (tileMma), which
    // orders it after every thread's tcgen05.ld above
    return true;
}

}  // namespace spgpu
