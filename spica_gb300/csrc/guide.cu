// guide.cu -- learned path guiding: parameter storage and packing, the fused training
// kernel (tcgen05 forward + backward, weight gradients), Adam, and the guided path
// tracer.  No counterpart in the reference renderer; the estimator it feeds is the
// reference's PathIntegrator::Li with the BSDF sampling strategy replaced by a
// one-sample MIS mixture of BSDF sampling (probability alpha >= 0.2) and the network's
// vMF mixture, so it stays unbiased whatever the network outputs.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <random>
#include <vector>

#include <cuda_bf16.h>

#include "../../include/spica_gpu.h"
#include "ctx.cuh"
#include "guide.cuh"
#include "guided_shade.cuh"
#include "shade.cuh"

namespace spgpu {

struct GuideState {
    float *master = nullptr, *m = nullptr, *v = nullptr;
    uint8_t *packFwd = nullptr, *packBwd = nullptr;
    float *biasPad = nullptr;
    float *samples = nullptr;   // training ring, 16 floats per sample: x[9], w[3], c, pad
    int capacity = 0;
    int *ctl = nullptr;         // [0] samples written (monotonic), [1] error, [2] work counter
    double *lossAcc = nullptr;  // [0] loss sum, [1] weight sum
    float *wsum = nullptr;      // batch weight sum / max
    float *batch = nullptr;
    int batchCap = 0;
    float *partials = nullptr;  // per training CTA: its partial gradient (kGParams floats)
    int partialRows = 0;
    int step = 0;
    spgpu_guiding_config cfg{};
    double lastLoss = 0.0;
    std::mt19937 rng;   // weight initialisation
};

namespace {

// ------------------------------------------------------------------ packing
// master fp32 -> bf16 canonical K-major tiles (forward and backward B operands)
__global__ void k_guide_pack(const float *__restrict__ P, uint8_t *fwd, uint8_t *bwd, float *biasPad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int stride = gridDim.x * blockDim.x;
    auto put = [](uint8_t *tile, int r, int k, int K, float v) {
        *reinterpret_cast<__nv_bfloat16 *>(tile + tc::kmajorOffset(r, k, K)) = __float2bfloat16_rn(v);
    };
    uint8_t *w1f = fwd, *w2f = w1f + kW1fBytes, *w3f = w2f + kW2fBytes, *w4f = w3f + kW2fBytes;
    uint8_t *w2b = bwd, *w3b = w2b + kW2fBytes, *w4b = w3b + kW2fBytes;
    for (int e = t; e < kGHid * kGK0; e += stride) {   // W1f [64][16]
        const int o = e / kGK0, i = e % kGK0;
        put(w1f, o, i, kGK0, i < kGIn ? P[kOffW1 + o * kGIn + i] : 0.0f);
    }
    for (int e = t; e < kGHid * kGHid; e += stride) {   // W2f, W3f [64][64] and W2b, W3b (transposed)
        const int o = e / kGHid, i = e % kGHid;
        put(w2f, o, i, kGHid, P[kOffW2 + e]);
        put(w3f, o, i, kGHid, P[kOffW3 + e]);
        put(w2b, i, o, kGHid, P[kOffW2 + e]);
        put(w3b, i, o, kGHid, P[kOffW3 + e]);
    }
    for (int e = t; e < kGN4 * kGHid; e += stride) {   // W4f [48][64], W4b [64][48]
        const int o = e / kGHid, i = e % kGHid;
        const float w = o < kGOut ? P[kOffW4 + o * kGHid + i] : 0.0f;
        put(w4f, o, i, kGHid, w);
        put(w4b, i, o, kGN4, w);
    }
    for (int e = t; e < kBiasPad; e += stride) {
        float b = 0.0f;
        if (e < kGHid) b = P[kOffB1 + e];
        else if (e < 2 * kGHid) b = P[kOffB2 + e - kGHid];
        else if (e < 3 * kGHid) b = P[kOffB3 + e - 2 * kGHid];
        else if (e - 3 * kGHid < kGOut) b = P[kOffB4 + e - 3 * kGHid];
        biasPad[e] = b;
    }
}

// ------------------------------------------------------------------ loss
// -c * log p(w) of the mixture for raw outputs r; writes dLoss/draw into g, returns loss.
// Reciprocals, square roots and exponentials are the hardware's approximations (relative
// errors of a few 1e-6 at the smallest concentration, e^-4, far inside the gradient's
// tolerance); the loss the step reports uses the same values.
__device__ __forceinline__ float mixtureLossGrad(const float *r, float3 w, float c, float *g) {
    float mx = -3.0e38f;
#pragma unroll
    for (int k = 0; k < kGLobes; k++) mx = fmaxf(mx, r[5 * k + 4]);
    float wk[kGLobes], vk[kGLobes], s = 0.0f;
    float3 mu[kGLobes];
    float ilen[kGLobes], kap[kGLobes];
#pragma unroll
    for (int k = 0; k < kGLobes; k++) {
        const float3 m = mk(r[5 * k], r[5 * k + 1], r[5 * k + 2]);
        ilen[k] = rsqrtf(fmaxf(dot(m, m), 1.0e-12f));   // 1 / max(|m|, 1e-6)
        mu[k] = m * ilen[k];
        kap[k] = kappaOf(r[5 * k + 3]);
        vk[k] = vmfNormFast(kap[k]) * __expf(kap[k] * (dot(mu[k], w) - 1.0f));
        wk[k] = __expf(r[5 * k + 4] - mx);
        s += wk[k];
    }
    const float is = __fdividef(1.0f, s);
    float p = 0.0f;
#pragma unroll
    for (int k = 0; k < kGLobes; k++) {
        wk[k] *= is;
        p += wk[k] * vk[k];
    }
    p = fmaxf(p, 1.0e-30f);
    const float a = -__fdividef(c, p);
#pragma unroll
    for (int k = 0; k < kGLobes; k++) {
        const float dv = a * wk[k];   // dLoss / dv_k
        const float kr = r[5 * k + 3];
        // d log v / d kappa = 1 / kappa - 2 / (e^(2 kappa) - 1) + (mu.w - 1)
        const float dlogv_dk = __fdividef(1.0f, kap[k]) - __fdividef(2.0f, __expf(2.0f * kap[k]) - 1.0f) +
                               (dot(mu[k], w) - 1.0f);
        g[5 * k + 3] = (kr > -4.0f && kr < 7.0f) ? dv * vk[k] * dlogv_dk * kap[k] : 0.0f;
        const float3 gmu = w * (dv * vk[k] * kap[k]);
        const float3 gm = (gmu - mu[k] * dot(mu[k], gmu)) * ilen[k];
        g[5 * k] = gm.x;
        g[5 * k + 1] = gm.y;
        g[5 * k + 2] = gm.z;
        g[5 * k + 4] = a * wk[k] * (vk[k] - p);
    }
    return -c * __logf(p);
}

// ------------------------------------------------------------------ training
constexpr int kTrainStride = 65;   // fp32 row stride of the dy tile
struct TrainLayout {
    static constexpr int wf = 0;
    static constexpr int wb = wf + kPackFwdBytes;
    static constexpr int bias = wb + kPackBwdBytes;
    static constexpr int x = bias + kBiasPad * 4;
    static constexpr int h1 = x + kGTile * kGK0 * 2;
    static constexpr int h2 = h1 + kGTile * kGHid * 2;
    static constexpr int h3 = h2 + kGTile * kGHid * 2;
    static constexpr int dyb = h3 + kGTile * kGHid * 2;
    static constexpr int dy = dyb + kGTile * kGHid * 2;
    static constexpr int gb = dy + kGTile * kTrainStride * 4;
    static constexpr int bar = gb + kBiasPad * 4;
    static constexpr int tmem = bar + 8;
    static constexpr int loadBar = tmem + 8;
    static constexpr int total = loadBar + 8;
};
static_assert(TrainLayout::x % 16 == 0 && TrainLayout::h1 % 16 == 0 && TrainLayout::dyb % 16 == 0, "alignment");
static_assert(TrainLayout::wb % 16 == 0 && TrainLayout::bias % 16 == 0 && TrainLayout::loadBar % 8 == 0,
              "bulk-copy destinations 16-byte aligned");
static_assert(TrainLayout::bar % 8 == 0, "alignment");
// one training CTA per SM: its 512-column TMEM allocation (all of the SM's tensor
// memory) then never waits for another CTA's
static_assert(2 * TrainLayout::total > 228 * 1024, "training CTA must fill more than half of an SM's shared memory");

// Weight-gradient accumulators in tensor memory (columns after the layer accumulator
// at 0-63), M = 64 (a layer's outputs), N = its inputs, accumulated over all tiles of
// the CTA: dW4 (40 x 64), dW3, dW2 (64 x 64), dW1 (64 x 16, inputs padded)
constexpr uint32_t kTrainTmemCols = 512;
constexpr uint32_t kColDW4 = 64, kColDW3 = 128, kColDW2 = 192, kColDW1 = 256;

// dW (+)= dY^T H over the tile's 128 rows, on the tensor core: dY and H are the tile's
// K-major bf16 tiles ([128][kDy] and [128][kH]) read transposed (MN-major), so the
// tile's rows are the MMA's K; the first 64 columns of dY are the MMA's M rows (rows
// past the layer's outputs are never read back).  Called by the issuing thread.
__device__ __forceinline__ void issueWeightGrad(uint32_t dTmem, const uint8_t *dyTile, uint32_t kDy,
                                                const uint8_t *hTile, uint32_t kH, bool accumulate) {
    const uint32_t aLbo = (kDy / 8) * 128, bLbo = (kH / 8) * 128;
    const uint32_t idesc = tc::instrDescBf16(64, kH) | tc::kTransposeA | tc::kTransposeB;
    const uint32_t aAddr = tc::smemAddr(dyTile), bAddr = tc::smemAddr(hTile);
    for (uint32_t j = 0; j < kGTile / 16; j++)
        tc::mmaBf16(dTmem, tc::smemDesc(aAddr + 2 * aLbo * j, aLbo, 128), tc::smemDesc(bAddr + 2 * bLbo * j, bLbo, 128),
                    idesc, (accumulate || j > 0) ? 1u : 0u);
}

// bias[o] += sum_r dy[r][o] for this tile (fp32 dy)
__device__ __forceinline__ void accumBias(float *gb, int nOut, const float *dy) {
    for (int o = threadIdx.x; o < nOut; o += kGTile) {
        float s = 0.0f;
        for (int r = 0; r < kGTile; r++) s += dy[r * kTrainStride + o];
        gb[o] += s;
    }
}

// one M = 64 weight-gradient accumulator -> row[offW + o * nIn + i], the CTA's own
// partial gradient (plain stores; the partial rows of all CTAs are summed afterwards in a
// fixed order, k_grad_sum); every thread takes part (tcgen05.ld is warp-wide), lanes 0-15
// of each warp hold its rows
__device__ __forceinline__ void flushWeightGrad(uint32_t dTmem, uint32_t nCols, int offW, int nOut, int nIn,
                                                float *row) {
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int o = static_cast<int>(16 * warp + lane);
    for (uint32_t c = 0; c < nCols; c += 16) {
        float v[16];
        tc::tmemLoad16(dTmem + ((warp * 32u) << 16) + c, v);
        if (lane < 16 && o < nOut)
            for (int i = 0; i < 16; i++)
                if (static_cast<int>(c) + i < nIn) row[offW + o * nIn + c + i] = v[i];
    }
}

// backward epilogue: g = acc * relu'(h) -> dy (fp32) and dyb (bf16, K = 64); the row's
// activations come 8 at a time (one core-matrix row, 16 bytes)
__device__ __forceinline__ void backEpilogue(uint32_t tmem, const uint8_t *h, float *dy, uint8_t *dyb) {
    const uint32_t r = threadIdx.x;
    for (uint32_t c = 0; c < kGHid; c += 16) {
        float v[16];
        accRow16(tmem, c, v);
#pragma unroll
        for (int half = 0; half < 2; half++) {
            const uint4 q = *reinterpret_cast<const uint4 *>(h + tc::kmajorOffset(r, c + 8 * half, kGHid));
            const __nv_bfloat162 *hb = reinterpret_cast<const __nv_bfloat162 *>(&q);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const float2 hv = __bfloat1622float2(hb[j]);
                float &a0 = v[8 * half + 2 * j], &a1 = v[8 * half + 2 * j + 1];
                a0 = hv.x > 0.0f ? a0 : 0.0f;
                a1 = hv.y > 0.0f ? a1 : 0.0f;
            }
        }
        for (int i = 0; i < 16; i++) dy[r * kTrainStride + c + i] = v[i];
        storeRow8(dyb, r, c, kGHid, v);
        storeRow8(dyb, r, c + 8, kGHid, v + 8);
    }
}

__global__ void __launch_bounds__(kGTile, 1) k_guide_train(const uint8_t *__restrict__ packFwd,
                                                           const uint8_t *__restrict__ packBwd,
                                                           const float *__restrict__ biasPad,
                                                           const float *__restrict__ samples, int n,
                                                           const float *__restrict__ wsum, float *partials,
                                                           double *lossAcc, int *err) {
    extern __shared__ __align__(128) uint8_t sm[];
    uint8_t *wf = sm + TrainLayout::wf, *wb = sm + TrainLayout::wb;
    float *bias = reinterpret_cast<float *>(sm + TrainLayout::bias);
    uint8_t *x = sm + TrainLayout::x, *h1 = sm + TrainLayout::h1, *h2 = sm + TrainLayout::h2,
            *h3 = sm + TrainLayout::h3, *dyb = sm + TrainLayout::dyb;
    float *dy = reinterpret_cast<float *>(sm + TrainLayout::dy);
    float *gb = reinterpret_cast<float *>(sm + TrainLayout::gb);   // bias gradients B1 | B2 | B3 | B4
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + TrainLayout::bar);
    uint32_t *tmemSlot = reinterpret_cast<uint32_t *>(sm + TrainLayout::tmem);
    const int t = threadIdx.x;
    // c is normalised by the batch's weight sum and clamped at 1000x its mean (rare,
    // bright indirect paths are the signal; only extreme outliers are cut)
    const float cSum = wsum[0];
    const float cScale = cSum > 0.0f ? 1.0f / cSum : 0.0f;
    const float cMax = 1000.0f * cSum / static_cast<float>(n);
    uint64_t *loadBar = reinterpret_cast<uint64_t *>(sm + TrainLayout::loadBar);
    for (int i = t; i < kBiasPad; i += kGTile) gb[i] = 0.0f;
    if (t == 0) {
        // forward and backward weights and biases: one bulk copy (TMA) each
        tc::mbarInit(bar, 1);
        tc::mbarInit(loadBar, 1);
        tc::mbarExpectTx(loadBar, kPackFwdBytes + kPackBwdBytes + kBiasPad * 4);
        tc::bulkLoad(wf, packFwd, kPackFwdBytes, loadBar);
        tc::bulkLoad(wb, packBwd, kPackBwdBytes, loadBar);
        tc::bulkLoad(bias, biasPad, kBiasPad * 4, loadBar);
    }
    if (t < 32) {
        tc::tmemAlloc(tmemSlot, kTrainTmemCols);
        tc::tmemRelinquish();
    }
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t tmem = *tmemSlot;
    uint32_t phase = 0;
    bool ok = bulkLoadWait(loadBar);
    float lossSum = 0.0f, wSum = 0.0f;
    bool acc = false;   // weight-gradient accumulators hold this CTA's earlier tiles
    const uint8_t *w2b = wb, *w3b = wb + kW2fBytes, *w4b = wb + 2 * kW2fBytes;
    for (int tile = blockIdx.x; ok && tile * kGTile < n; tile += gridDim.x) {
        const int s = tile * kGTile + t;
        float xf[16];
        float3 w = mk(0, 0, 1);
        float c = 0.0f;
        for (int i = 0; i < 16; i++) xf[i] = 0.0f;
        if (s < n) {
            const float *S = samples + 16 * static_cast<int64_t>(s);
            for (int i = 0; i < kGIn; i++) xf[i] = S[i];
            w = mk(S[9], S[10], S[11]);
            c = fminf(S[12], cMax) * cScale;
        }
        storeRow8(x, t, 0, kGK0, xf);
        storeRow8(x, t, 8, kGK0, xf + 8);
        ok = mlpForwardTile(tmem, wf, bias, x, h1, h2, h3, dy, kTrainStride, bar, phase);
        if (!ok) break;
        // loss gradient on this thread's row
        {
            float r[kGOut], g[kGN4];
            for (int j = 0; j < kGOut; j++) r[j] = dy[t * kTrainStride + j];
            for (int j = 0; j < kGN4; j++) g[j] = 0.0f;
            if (s < n && c > 0.0f) {
                lossSum += mixtureLossGrad(r, w, c, g);
                wSum += c;
            }
            for (int j = 0; j < kGN4; j++) dy[t * kTrainStride + j] = g[j];
            for (int j = 0; j < kGN4; j += 8) storeRow8(dyb, t, j, kGN4, g + j);
        }
        __syncthreads();
        // each layer: its bias gradient on the CUDA cores, then one commit for the
        // backward MMA (dX = dY W) and the weight-gradient MMA (dW += dY^T H), which
        // read the same dY tile
        accumBias(gb + 3 * kGHid, kGOut, dy);
        ok = mmaRun(bar, phase, [&] {
            issueTileMma(tmem, dyb, w4b, kGN4, kGHid);                    // dX3 = dY4 W4
            issueWeightGrad(tmem + kColDW4, dyb, kGN4, h3, kGHid, acc);   // dW4 += dY4^T H3
        });
        if (!ok) break;
        backEpilogue(tmem, h3, dy, dyb);
        __syncthreads();
        accumBias(gb + 2 * kGHid, kGHid, dy);
        ok = mmaRun(bar, phase, [&] {
            issueTileMma(tmem, dyb, w3b, kGHid, kGHid);                   // dX2 = dY3 W3
            issueWeightGrad(tmem + kColDW3, dyb, kGHid, h2, kGHid, acc);  // dW3 += dY3^T H2
        });
        if (!ok) break;
        backEpilogue(tmem, h2, dy, dyb);
        __syncthreads();
        accumBias(gb + kGHid, kGHid, dy);
        ok = mmaRun(bar, phase, [&] {
            issueTileMma(tmem, dyb, w2b, kGHid, kGHid);                   // dX1 = dY2 W2
            issueWeightGrad(tmem + kColDW2, dyb, kGHid, h1, kGHid, acc);  // dW2 += dY2^T H1
        });
        if (!ok) break;
        backEpilogue(tmem, h1, dy, dyb);
        __syncthreads();
        accumBias(gb, kGHid, dy);
        ok = mmaRun(bar, phase, [&] {
            issueWeightGrad(tmem + kColDW1, dyb, kGHid, x, kGK0, acc);    // dW1 += dY1^T X
        });
        acc = true;
    }
    if (!ok) {
        // a wait gave up: wait (bounded) for the copies and MMAs still in flight before
        // freeing TMEM
        tc::mbarWait(loadBar, 0, kMmaWaitTries);
        tc::mbarWait(bar, phase ^ 1u, kMmaWaitTries);
        tc::fenceBeforeSync();
        __syncthreads();
        if (t < 32) tc::tmemDealloc(tmem, kTrainTmemCols);
        if (t == 0) atomicOr(err, 1);
        return;
    }
    float *row = partials + static_cast<int64_t>(blockIdx.x) * kGParams;
    if (acc) {
        flushWeightGrad(tmem + kColDW4, kGHid, kOffW4, kGOut, kGHid, row);
        flushWeightGrad(tmem + kColDW3, kGHid, kOffW3, kGHid, kGHid, row);
        flushWeightGrad(tmem + kColDW2, kGHid, kOffW2, kGHid, kGHid, row);
        flushWeightGrad(tmem + kColDW1, kGK0, kOffW1, kGHid, kGIn, row);
    } else {
        for (int i = t; i < kGParams; i += kGTile) row[i] = 0.0f;   // no tile: a zero partial
    }
    tc::fenceBeforeSync();
    __syncthreads();
    if (t < 32) tc::tmemDealloc(tmem, kTrainTmemCols);
    for (int o = t; o < kGHid; o += kGTile) {
        row[kOffB1 + o] = gb[o];
        row[kOffB2 + o] = gb[kGHid + o];
        row[kOffB3 + o] = gb[2 * kGHid + o];
        if (o < kGOut) row[kOffB4 + o] = gb[3 * kGHid + o];
    }
    for (int off = 16; off > 0; off >>= 1) {
        lossSum += __shfl_xor_sync(0xffffffffu, lossSum, off);
        wSum += __shfl_xor_sync(0xffffffffu, wSum, off);
    }
    if ((t & 31) == 0) {
        atomicAdd(&lossAcc[0], static_cast<double>(lossSum));
        atomicAdd(&lossAcc[1], static_cast<double>(wSum));
    }
}

// inference only (tests and tools): features [n][9] -> raw outputs [n][40]
__global__ void __launch_bounds__(kGTile, 1) k_guide_forward(const uint8_t *__restrict__ packFwd,
                                                             const float *__restrict__ biasPad,
                                                             const float *__restrict__ feat, int n, float *out,
                                                             int *err, int faultWait) {
    extern __shared__ __align__(128) uint8_t sm[];
    uint8_t *wf = sm;
    float *bias = reinterpret_cast<float *>(sm + kPackFwdBytes);
    uint8_t *x = sm + kPackFwdBytes + kBiasPad * 4;
    uint8_t *h = x + kGTile * kGK0 * 2;
    float *o = reinterpret_cast<float *>(h + kGTile * kGHid * 2);
    uint64_t *bar = reinterpret_cast<uint64_t *>(reinterpret_cast<uint8_t *>(o) + kGTile * 41 * 4);
    uint32_t *tmemSlot = reinterpret_cast<uint32_t *>(bar + 1);
    const int t = threadIdx.x;
    for (int i = t; i < kPackFwdBytes / 16; i += kGTile)
        reinterpret_cast<uint4 *>(wf)[i] = reinterpret_cast<const uint4 *>(packFwd)[i];
    for (int i = t; i < kBiasPad; i += kGTile) bias[i] = biasPad[i];
    if (t == 0) tc::mbarInit(bar, 1);
    if (t < 32) {
        tc::tmemAlloc(tmemSlot, 64);
        tc::tmemRelinquish();
    }
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t tmem = *tmemSlot;
    uint32_t phase = 0;
    bool ok = true;
    for (int tile = blockIdx.x; ok && tile * kGTile < n; tile += gridDim.x) {
        const int s = tile * kGTile + t;
        float xf[16];
        for (int i = 0; i < 16; i++) xf[i] = (s < n && i < kGIn) ? feat[9 * static_cast<int64_t>(s) + i] : 0.0f;
        storeRow8(x, t, 0, kGK0, xf);
        storeRow8(x, t, 8, kGK0, xf + 8);
        if (faultWait)   // fault injection: nothing arrives on the barrier, the short wait runs out
            ok = tileMma(tmem, x, wf, kGK0, kGHid, bar, phase, true, 1024u);
        else
            ok = mlpForwardTile(tmem, wf, bias, x, h, h, h, o, 41, bar, phase);
        if (ok && s < n)
            for (int j = 0; j < kGOut; j++) out[kGOut * static_cast<int64_t>(s) + j] = o[t * 41 + j];
        __syncthreads();
    }
    tc::fenceBeforeSync();
    __syncthreads();
    if (t < 32) tc::tmemDealloc(tmem, 64);
    if (!ok && t == 0) atomicOr(err, 1);
}
constexpr int kForwardSmem = kPackFwdBytes + kBiasPad * 4 + kGTile * kGK0 * 2 + kGTile * kGHid * 2 + kGTile * 41 * 4 + 16;

// ------------------------------------------------------------------ gradient sum, Adam
// The batch gradient is the sum of the training CTAs' partial rows.  Each block takes
// kRedX parameters; its kRedY thread rows add every kRedY-th partial row, and the
// column sums are added in row order, so the sum is the same every time.  ADAM applies
// an Adam step (Kingma and Ba: bias-corrected moments, c1 = 1 - b1^t, c2 = 1 - b2^t) to
// the master parameters out with it; otherwise the sum is written to out.
constexpr int kRedX = 32, kRedY = 8;
template <bool ADAM>
__global__ void __launch_bounds__(kRedX *kRedY) k_grad_sum(const float *__restrict__ partials, int nParts, float *out,
                                                           float *M, float *V, float lr, float b1, float b2, float eps,
                                                           float c1, float c2) {
    __shared__ float part[kRedY][kRedX];
    const int i = blockIdx.x * kRedX + threadIdx.x;
    float s = 0.0f;
    if (i < kGParams)
        for (int p = threadIdx.y; p < nParts; p += kRedY) s += partials[static_cast<int64_t>(p) * kGParams + i];
    part[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y != 0 || i >= kGParams) return;
    float g = 0.0f;
    for (int y = 0; y < kRedY; y++) g += part[y][threadIdx.x];
    if (ADAM) {
        const float m = b1 * M[i] + (1.0f - b1) * g;
        const float v = b2 * V[i] + (1.0f - b2) * g * g;
        M[i] = m;
        V[i] = v;
        out[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
    } else {
        out[i] = g;
    }
}
constexpr int kRedBlocks = (kGParams + kRedX - 1) / kRedX;

// gather a random batch of n samples from the first `avail` ring entries (indices from
// Philox keyed by (seed, step)) and sum their weights
__global__ void k_gather(const float *ring, int avail, uint32_t seed, uint32_t step, int n, float *batch,
                         float *wsum) {
    float part = 0.0f;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const uint4 r = philox4x32_10(make_uint4(static_cast<uint32_t>(s), step, 0x47415448u, 0u), make_uint2(seed, 0u));
        const int idx = static_cast<int>(__umulhi(r.x, static_cast<uint32_t>(avail)));
        const float4 *src = reinterpret_cast<const float4 *>(ring + 16 * static_cast<int64_t>(idx));
        float4 *dst = reinterpret_cast<float4 *>(batch + 16 * static_cast<int64_t>(s));
        const float4 q0 = src[0], q1 = src[1], q2 = src[2], q3 = src[3];
        dst[0] = q0;
        dst[1] = q1;
        dst[2] = q2;
        dst[3] = q3;
        part += q3.x;   // element 12: the weight c
    }
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if ((threadIdx.x & 31) == 0 && part != 0.0f) atomicAdd(&wsum[0], part);
}

// weight sum of a caller-supplied batch
__global__ void k_csum(const float *samples, int n, float *wsum) {
    float part = 0.0f;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x)
        part += samples[16 * static_cast<int64_t>(s) + 12];
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if ((threadIdx.x & 31) == 0 && part != 0.0f) atomicAdd(&wsum[0], part);
}

// ------------------------------------------------------------------ guided tracer
struct TrainRec {
    float x[kGIn];
    float3 w;
    float q;
    float3 fcos, Lafter, beta, E;
};

struct GuidedArgs {
    SceneView sv;
    CameraView cam;
    int W, H, npix;
    long long total;   // paths to trace
    int sampleOffset;
    int maxDepth;
    uint32_t seed;
    float4 *film;
    const uint8_t *packFwd;
    const float *biasPad;
    float3 lo, invExt;
    float alpha;   // BSDF probability in the one-sample MIS mixture
    float *ring;
    int capacity;
    int *ctl;      // [0] samples written, [1] error, [2] path counter
    unsigned long long *stats;
};

// guided kernel shared memory: packed forward weights | biases | input/hidden tile (bf16
// [128][64]; the [128][16] input tile aliases its start) | traversal stacks | mbarrier,
// TMEM slot
constexpr int kGuidedSmOffBias = kPackFwdBytes;
constexpr int kGuidedSmOffXH = kGuidedSmOffBias + 1024;   // biases (960 bytes), padded
constexpr int kGuidedSmOffStack = kGuidedSmOffXH + kGTile * kGHid * 2;
constexpr int kGuidedSmOffBar = kGuidedSmOffStack + kStackShared * kGTile * 8;
constexpr int kGuidedSmem = kGuidedSmOffBar + 16;
static_assert(kBiasPad * 4 <= 1024 && kGuidedSmOffXH % 128 == 0 && kGuidedSmOffStack % 16 == 0 && kGuidedSmOffBar % 8 == 0, "alignment");
constexpr int kPlainSmem = kStackShared * kGTile * 8;
constexpr int kMaxRec = 13;

__device__ __forceinline__ float lum(float3 c) { return gray(c); }

// one-sample MIS mixture of cosine-weighted Lambert sampling and the vMF mixture

template <bool GUIDED, bool COLLECT>
__global__ void __launch_bounds__(kGTile) k_guided(GuidedArgs a) {
    extern __shared__ __align__(128) uint8_t sm[];
    uint8_t *wf = sm;
    float *bias = reinterpret_cast<float *>(sm + kGuidedSmOffBias);
    uint8_t *xh = sm + kGuidedSmOffXH;
    // the plain kernel keeps only the traversal stacks in shared memory
    uint2 *stack = reinterpret_cast<uint2 *>(GUIDED ? sm + kGuidedSmOffStack : sm);
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm + kGuidedSmOffBar);
    uint32_t *tmemSlot = reinterpret_cast<uint32_t *>(bar + 1);
    const int t = threadIdx.x;
    const SceneView &S = a.sv;
    uint32_t tmem = 0, phase = 0;
    if (GUIDED) {
        for (int i = t; i < kPackFwdBytes / 16; i += kGTile)
            reinterpret_cast<uint4 *>(wf)[i] = reinterpret_cast<const uint4 *>(a.packFwd)[i];
        for (int i = t; i < kBiasPad; i += kGTile) bias[i] = a.biasPad[i];
        if (t == 0) tc::mbarInit(bar, 1);
        if (t < 32) {
            tc::tmemAlloc(tmemSlot, 64);
            tc::tmemRelinquish();
        }
        tc::fenceBeforeSync();
        __syncthreads();
        tc::fenceAfterSync();
        tmem = *tmemSlot;
    }
    bool overflow = false, mmaOk = true;
    uint32_t dummy = 0;
    unsigned long long nPaths = 0, nClosest = 0, nShadow = 0;
    // path state
    bool active = false, exhausted = false;
    int fi = 0, b = 0;
    uint32_t sample = 0;
    float3 o = mk(0, 0, 0), d = mk(0, 0, 1), beta = mk(1, 1, 1), L = mk(0, 0, 0);
    bool spec = false;
    TrainRec rec[COLLECT ? kMaxRec : 1];
    int nrec = 0;
    bool recLast = false;   // the current ray is the direction of rec[nrec - 1]
    while (true) {
        // ---- start new paths in idle lanes
        const bool want = !active && !exhausted;
        const unsigned wmask = __ballot_sync(0xffffffffu, want);
        if (wmask) {
            const int lane = t & 31, leader = __ffs(wmask) - 1;
            long long base = 0;
            if (lane == leader) base = atomicAdd(reinterpret_cast<unsigned long long *>(&a.ctl[2]),
                                                 static_cast<unsigned long long>(__popc(wmask)));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (want) {
                const long long id = base + __popc(wmask & ((1u << lane) - 1u));
                if (id < a.total) {
                    const int pix = static_cast<int>(id % a.npix);
                    sample = static_cast<uint32_t>(a.sampleOffset + id / a.npix);
                    const int y = pix / a.W, xx = pix - y * a.W;
                    fi = y * a.W + (a.W - 1 - xx);
                    const Rand4 r = rand4(a.seed, static_cast<uint32_t>(fi), sample, 0xFFFFu, 0u);
                    spawnCameraRay(a.cam, xx, y, r.a, r.b, &o, &d);
                    beta = mk(1, 1, 1);
                    L = mk(0, 0, 0);
                    spec = false;
                    b = 0;
                    nrec = 0;
                    recLast = false;
                    active = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (__syncthreads_and(!active)) break;
        // ---- extend
        HitRecord hr;
        bool hit = false;
        if (active) {
            float tmax = kInfT, u, v;
            int slot = -1;
            nClosest++;
            hit = traceWide<false, false>(S.nodes, S.tris, S.nNodes, S.nTris, o, d, 0.0f, tmax, slot, u, v,
                                          stack + t, kGTile, &dummy, &dummy, &overflow);
            hr.t = tmax;
            hr.prim = slot;
            hr.u = u;
            hr.v = v;
        }
        bool ends = false;
        float3 n = mk(0, 0, 1), ps = mk(0, 0, 0);
        MaterialRecord m;
        m.type = -1;
        int lightOf = -1;
        if (active) {
            if (!hit) {
                const float3 Le = S.hasEnv ? envLe(S.env, d) : mk(0, 0, 0);
                if (b == 0 || spec) L = L + beta * Le;
                // direct radiance along the last guided direction, times the MIS weight of the
                // guided strategy against light sampling: the share of it that guided samples
                // estimate (a sun that light sampling finds is not worth learning)
                if (COLLECT && recLast && S.hasEnv)
                    rec[nrec - 1].E = Le * powerHeuristic(rec[nrec - 1].q, envPdf(S.env, d));
                ends = true;
            } else {
                const TriRecord tr = S.tris[hr.prim];
                n = triNormal(tr);
                const int2 sh = __ldg(&S.slotShade[hr.prim]);
                m = S.mats[sh.x];
                lightOf = sh.y;
                ps = hitPoint(o, d, hr.t);
                if (COLLECT && recLast && lightOf >= 0 && dot(n, -d) > 0.0f) {
                    const LightRecord &Lr = S.lights[lightOf];
                    const float lp = hr.t * hr.t / (dot(n, -d) * Lr.p0.w);
                    rec[nrec - 1].E = xyz(Lr.L) * powerHeuristic(rec[nrec - 1].q, lp);
                }
                if (b >= a.maxDepth) {
                    if ((b == 0 || spec) && lightOf >= 0 && dot(n, -d) > 0.0f) L = L + beta * xyz(S.lights[lightOf].L);
                    ends = true;
                }
            }
        }
        const bool guideMe = GUIDED && active && !ends && m.type == kMatLambert;
        // ---- network inference for the whole CTA (rows of other lanes are zero)
        Mixture mix;
        if (GUIDED) {
            float xf[16];
            for (int i = 0; i < 16; i++) xf[i] = 0.0f;
            if (guideMe) guideFeatures(ps, n, -d, a.lo, a.invExt, xf);
            storeRow8(xh, t, 0, kGK0, xf);
            storeRow8(xh, t, 8, kGK0, xf + 8);
            if (__syncthreads_or(guideMe) && mmaOk) {
                float raw[kGOut];
                mmaOk = mlpForwardRow(tmem, wf, bias, xh, bar, phase, raw);
                if (guideMe && mmaOk) mixtureFromRaw(raw, mix);
            }
        }
        // ---- shade
        if (active && !ends) {
            ShadeResult R;
            if (!guideMe || !mmaOk) {
                shadeHit(S, hr, o, d, beta, spec, b, a.maxDepth, a.seed, static_cast<uint32_t>(fi), sample, fi, R);
                recLast = false;
            } else {
                float3 fc;
                float pdf;
                shadeGuidedLambert(S, ps, n, m, lightOf, d, beta, spec, b, mix, a.alpha, a.seed,
                                   static_cast<uint32_t>(fi), sample, R, &fc, &pdf);
                if (COLLECT) {
                    recLast = false;
                    if (R.cont && nrec < kMaxRec) {
                        TrainRec &T = rec[nrec++];
                        guideFeatures(ps, n, -d, a.lo, a.invExt, T.x);
                        T.w = xyz(R.cD);
                        T.q = pdf;
                        T.fcos = fc;
                        T.beta = R.beta;
                        T.E = mk(0, 0, 0);
                        recLast = true;
                    }
                }
            }
            L = L + R.emit;
            float u, v, tmx;
            int slot;
            if (R.sh0) {
                nShadow++;
                tmx = R.s0D.w;
                if (!traceWide<true, false>(S.nodes, S.tris, S.nNodes, S.nTris, xyz(R.s0O), xyz(R.s0D), 0.0f, tmx,
                                            slot, u, v, stack + t, kGTile, &dummy, &dummy, &overflow))
                    L = L + xyz(R.s0L);
            }
            if (R.sh1) {
                nShadow++;
                tmx = R.s1D.w;
                if (!traceWide<true, false>(S.nodes, S.tris, S.nNodes, S.nTris, xyz(R.s1O), xyz(R.s1D), 0.0f, tmx,
                                            slot, u, v, stack + t, kGTile, &dummy, &dummy, &overflow))
                    L = L + xyz(R.s1L);
            }
            if (COLLECT && guideMe && R.cont && nrec > 0) rec[nrec - 1].Lafter = L;
            if (R.cont) {
                o = xyz(R.cO);
                d = xyz(R.cD);
                beta = R.beta;
                spec = R.spec;
                b++;
            } else {
                ends = true;
            }
        }
        if (active && ends) {
            atomicAdd(&a.film[fi], make_float4(L.x, L.y, L.z, 1.0f));
            nPaths++;
            if (COLLECT) {
                // incident radiance along each guided direction: direct radiance found by the
                // continuation ray plus everything the path gathered afterwards, divided by
                // the throughput at that point
                for (int k = 0; k < nrec; k++) {
                    const TrainRec &T = rec[k];
                    float3 Li = T.E;
                    const float3 rest = L - T.Lafter;
                    Li.x += T.beta.x > 0.0f ? rest.x / T.beta.x : 0.0f;
                    Li.y += T.beta.y > 0.0f ? rest.y / T.beta.y : 0.0f;
                    Li.z += T.beta.z > 0.0f ? rest.z / T.beta.z : 0.0f;
                    const float c = lum(T.fcos * Li) / T.q;
                    if (!(c > 0.0f) || !isfinite(c)) continue;
                    const unsigned slotIdx =
                        atomicAdd(reinterpret_cast<unsigned *>(&a.ctl[0]), 1u) % static_cast<unsigned>(a.capacity);
                    float *D = a.ring + 16 * static_cast<int64_t>(slotIdx);
                    for (int i = 0; i < kGIn; i++) D[i] = T.x[i];
                    D[9] = T.w.x;
                    D[10] = T.w.y;
                    D[11] = T.w.z;
                    D[12] = c;
                    D[13] = T.q;
                }
            }
            active = false;
        }
    }
    if (GUIDED) {
        tc::fenceBeforeSync();
        __syncthreads();
        if (t < 32) tc::tmemDealloc(tmem, 64);
    }
    if (overflow || !mmaOk) atomicOr(&a.ctl[1], 1);
    atomicAdd(&a.stats[0], nPaths);
    atomicAdd(&a.stats[1], nClosest);
    atomicAdd(&a.stats[2], nShadow);
}

// Dynamic shared-memory limits, and the largest shared-memory carveout for the persistent
// megakernels: with the default carveout the occupancy query (and the hardware) would
// fit a single 58 KB guided CTA per SM.
void setGuideKernelAttributes() {
    static std::once_flag once;
    std::call_once(once, [] {
        cudaFuncSetAttribute(k_guide_train, cudaFuncAttributeMaxDynamicSharedMemorySize, TrainLayout::total);
        cudaFuncSetAttribute(k_guide_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, kForwardSmem);
        cudaFuncSetAttribute(k_guided<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGuidedSmem);
        cudaFuncSetAttribute(k_guided<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGuidedSmem);
        cudaFuncSetAttribute(k_guided<true, true>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
        cudaFuncSetAttribute(k_guided<true, false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
        cudaFuncSetAttribute(k_guided<false, false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
        cudaGetLastError();
    });
}

// CTAs of a guided megakernel (kGTile threads, kGuidedSmem bytes of dynamic shared
// memory, one 64-column TMEM allocation) that fit one SM at once, from the kernel's
// register count and the device's limits.  (The occupancy API reports a single CTA
// per SM for kernels that allocate tensor memory; co-resident CTAs are fine as long as
// their allocations fit the SM's 512 TMEM columns, which the last term ensures.)
int tmemKernelResidentCtas(const void *kernel, int device, int dynSmem = kGuidedSmem) {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    int regsSM = 0, smemSM = 0, smemReserved = 0, thrSM = 0, blkSM = 0;
    cudaDeviceGetAttribute(&regsSM, cudaDevAttrMaxRegistersPerMultiprocessor, device);
    cudaDeviceGetAttribute(&smemSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device);
    cudaDeviceGetAttribute(&smemReserved, cudaDevAttrReservedSharedMemoryPerBlock, device);
    cudaDeviceGetAttribute(&thrSM, cudaDevAttrMaxThreadsPerMultiProcessor, device);
    cudaDeviceGetAttribute(&blkSM, cudaDevAttrMaxBlocksPerMultiprocessor, device);
    const int warps = kGTile / 32;
    const int regsPerWarp = ((fa.numRegs * 32 + 255) / 256) * 256;
    const int byRegs = regsPerWarp > 0 ? regsSM / (regsPerWarp * warps) : 1;
    const int bySmem = smemSM / (dynSmem + static_cast<int>(fa.sharedSizeBytes) + smemReserved);
    const int byThreads = thrSM / kGTile;
    constexpr int byTmem = 512 / 64;
    return std::max(1, std::min(std::min(byRegs, bySmem), std::min(std::min(byThreads, blkSM), byTmem)));
}

template <class T>
T *galloc(size_t n) {
    T *p = nullptr;
    return cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)) == cudaSuccess ? p : nullptr;
}

int packWeights(GuideState &G, cudaStream_t s) {
    k_guide_pack<<<32, 256, 0, s>>>(G.master, G.packFwd, G.packBwd, G.biasPad);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : cudaFail("guide pack", e);
}

}  // namespace

int guideTileKernelGrid(const void *kernel, int device, int dynSmem) {
    if (dynSmem <= 0) dynSmem = kTileSmem;
    cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (dynSmem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dynSmem);
    cudaGetLastError();
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    return sms * tmemKernelResidentCtas(kernel, device, dynSmem);
}

void freeGuide(GuideState *G) {
    if (!G) return;
    cudaFree(G->master);
    cudaFree(G->partials);
    cudaFree(G->m);
    cudaFree(G->v);
    cudaFree(G->packFwd);
    cudaFree(G->packBwd);
    cudaFree(G->biasPad);
    cudaFree(G->samples);
    cudaFree(G->ctl);
    cudaFree(G->lossAcc);
    cudaFree(G->wsum);
    cudaFree(G->batch);
    delete G;
}

int guideInit(Ctx &C, GuideState **slot, const spgpu_guiding_config *cfg) {
    freeGuide(*slot);
    *slot = nullptr;
    auto *G = new GuideState();
    G->cfg = *cfg;
    if (G->cfg.learning_rate <= 0.0f) G->cfg.learning_rate = 1.0e-3f;
    if (G->cfg.bsdf_fraction < 0.2f) G->cfg.bsdf_fraction = 0.2f;
    if (G->cfg.batch <= 0) G->cfg.batch = 16384;
    if (G->cfg.capacity <= 0) G->cfg.capacity = 1 << 21;
    G->capacity = G->cfg.capacity;
    G->batchCap = ((G->cfg.batch + kGTile - 1) / kGTile) * kGTile;
    G->rng.seed(G->cfg.seed);
    G->master = galloc<float>(kGParams);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, C.device);
    G->partialRows = std::max(sms, 1);
    G->partials = galloc<float>(static_cast<size_t>(G->partialRows) * kGParams);
    G->m = galloc<float>(kGParams);
    G->v = galloc<float>(kGParams);
    G->packFwd = galloc<uint8_t>(kPackFwdBytes);
    G->packBwd = galloc<uint8_t>(kPackBwdBytes);
    G->biasPad = galloc<float>(kBiasPad);
    G->samples = galloc<float>(static_cast<size_t>(G->capacity) * 16);
    G->ctl = galloc<int>(4);
    G->lossAcc = galloc<double>(2);
    G->wsum = galloc<float>(2);
    G->batch = galloc<float>(static_cast<size_t>(G->batchCap) * 16);
    if (!G->master || !G->partials || !G->m || !G->v || !G->packFwd || !G->packBwd || !G->biasPad || !G->samples ||
        !G->ctl || !G->lossAcc || !G->wsum || !G->batch) {
        freeGuide(G);
        setError("spgpu_guiding_init: device allocation failed");
        return SPGPU_ENOMEM;
    }
    // He-uniform initialisation of the weights, zero biases
    std::vector<float> P(kGParams, 0.0f);
    auto fill = [&](int off, int nOut, int nIn) {
        std::uniform_real_distribution<float> U(-1.0f, 1.0f);
        const float s = std::sqrt(6.0f / nIn);
        for (int i = 0; i < nOut * nIn; i++) P[off + i] = s * U(G->rng);
    };
    fill(kOffW1, kGHid, kGIn);
    fill(kOffW2, kGHid, kGHid);
    fill(kOffW3, kGHid, kGHid);
    fill(kOffW4, kGOut, kGHid);
    for (int i = 0; i < kGOut * kGHid; i++) P[kOffW4 + i] *= 0.1f;   // start near a broad, uniform mixture
    cudaMemcpy(G->master, P.data(), sizeof(float) * kGParams, cudaMemcpyHostToDevice);
    cudaMemset(G->m, 0, sizeof(float) * kGParams);
    cudaMemset(G->v, 0, sizeof(float) * kGParams);
    cudaMemset(G->ctl, 0, sizeof(int) * 4);
    cudaMemset(G->samples, 0, sizeof(float) * 16 * static_cast<size_t>(G->capacity));
    int rc = packWeights(*G, C.stream);
    if (rc == 0 && cudaStreamSynchronize(C.stream) != cudaSuccess) rc = cudaFail("spgpu_guiding_init", cudaGetLastError());
    if (rc) {
        freeGuide(G);
        return rc;
    }
    setGuideKernelAttributes();
    *slot = G;
    return 0;
}

int guideParams(Ctx &C, GuideState &G, float *host, int set) {
    cudaError_t e;
    if (set) {
        e = cudaMemcpy(G.master, host, sizeof(float) * kGParams, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cudaFail("spgpu_guiding_params", e);
        int rc = packWeights(G, C.stream);
        if (rc) return rc;
        e = cudaStreamSynchronize(C.stream);
    } else {
        e = cudaMemcpy(host, G.master, sizeof(float) * kGParams, cudaMemcpyDeviceToHost);
    }
    return e == cudaSuccess ? 0 : cudaFail("spgpu_guiding_params", e);
}

int guideForward(Ctx &C, GuideState &G, const float *feat, int n, float *out, cudaStream_t s) {
    cudaMemsetAsync(G.ctl + 1, 0, sizeof(int), s);
    const int tiles = (n + kGTile - 1) / kGTile;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, C.device);
    k_guide_forward<<<std::min(tiles, sms), kGTile, kForwardSmem, s>>>(G.packFwd, G.biasPad, feat, n, out, G.ctl + 1,
                                                                       G.cfg.fault_injection == SPGPU_GUIDE_FAULT_WAIT);
    int err = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err, G.ctl + 1, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cudaFail("spgpu_guiding_mlp", e);
    if (err) {
        setError("spgpu_guiding_mlp: tensor-core wait timed out");
        return SPGPU_EKERNEL;
    }
    return 0;
}

// Launch the gradient of the batch loss (sum_i c_i * -log p(w_i), c normalised by the
// batch's weight sum in G.wsum[0]): one partial row per training CTA in G.partials,
// *nParts of them; the c-weighted loss is added to G.lossAcc[0].  No host
// synchronisation.
static int launchGrad(Ctx &C, GuideState &G, const float *samples, int n, int *nParts, cudaStream_t s) {
    const int tiles = (n + kGTile - 1) / kGTile;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, C.device);
    *nParts = std::min(std::min(tiles, sms), G.partialRows);
    k_guide_train<<<*nParts, kGTile, TrainLayout::total, s>>>(G.packFwd, G.packBwd, G.biasPad, samples, n, G.wsum,
                                                              G.partials, G.lossAcc, G.ctl + 1);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : cudaFail("guiding gradient", e);
}

static int readLoss(GuideState &G, double *loss, cudaStream_t s, const char *what) {
    double la[2] = {0, 0};
    int err = 0;
    cudaError_t e = cudaMemcpyAsync(la, G.lossAcc, sizeof(la), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err, G.ctl + 1, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cudaFail(what, e);
    if (err) {
        setError(std::string(what) + ": tensor-core wait timed out");
        return SPGPU_EKERNEL;
    }
    if (loss) *loss = la[0];
    return 0;
}

int guideGrad(Ctx &C, GuideState &G, const float *samples, int n, float *gradOut, double *loss, cudaStream_t s) {
    if (n <= 0) {
        if (loss) *loss = 0.0;
        return 0;
    }
    cudaMemsetAsync(G.wsum, 0, 2 * sizeof(float), s);
    cudaMemsetAsync(G.lossAcc, 0, 2 * sizeof(double), s);
    cudaMemsetAsync(G.ctl + 1, 0, sizeof(int), s);
    k_csum<<<64, 256, 0, s>>>(samples, n, G.wsum);
    int nParts = 0;
    int rc = launchGrad(C, G, samples, n, &nParts, s);
    if (rc == 0) {
        k_grad_sum<false><<<kRedBlocks, dim3(kRedX, kRedY), 0, s>>>(G.partials, nParts, gradOut, nullptr, nullptr,
                                                                    0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 1.0f);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cudaFail("guiding gradient sum", e);
    }
    return rc ? rc : readLoss(G, loss, s, "spgpu_guiding_grad");
}

// ring entries holding samples: the write counter wraps as an unsigned 32-bit value
static int ringAvail(const GuideState &G) {
    unsigned written = 0;
    cudaMemcpy(&written, G.ctl, sizeof(unsigned), cudaMemcpyDeviceToHost);
    return static_cast<int>(std::min<unsigned>(written, static_cast<unsigned>(G.capacity)));
}

int guideRing(const GuideState &G, float *dst, int maxSamples, int *count) {
    const int n = std::min(ringAvail(G), maxSamples);
    *count = 0;
    if (n > 0) {
        const cudaError_t e = cudaMemcpy(dst, G.samples, sizeof(float) * 16 * static_cast<size_t>(n),
                                         cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cudaFail("spgpu_guiding_ring", e);
    }
    *count = n;
    return 0;
}

int guideTrain(Ctx &C, GuideState &G, int steps, double *meanLoss) {
    const int avail = ringAvail(G);
    if (avail <= 0) {
        setError("spgpu_guiding_train: no training samples collected yet");
        return SPGPU_ESTATE;
    }
    const int n = std::min(G.batchCap, avail);
    cudaStream_t s = C.stream;
    cudaMemsetAsync(G.lossAcc, 0, 2 * sizeof(double), s);
    cudaMemsetAsync(G.ctl + 1, 0, sizeof(int), s);
    for (int st = 0; st < steps; st++) {
        cudaMemsetAsync(G.wsum, 0, 2 * sizeof(float), s);
        k_gather<<<std::min(64, (n + 255) / 256), 256, 0, s>>>(G.samples, avail, G.cfg.seed,
                                                                static_cast<uint32_t>(G.step), n, G.batch, G.wsum);
        int nParts = 0;
        int rc = launchGrad(C, G, G.batch, n, &nParts, s);
        if (rc) return rc;
        G.step++;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.0f - std::pow(b1, static_cast<float>(G.step));
        const float c2 = 1.0f - std::pow(b2, static_cast<float>(G.step));
        k_grad_sum<true><<<kRedBlocks, dim3(kRedX, kRedY), 0, s>>>(G.partials, nParts, G.master, G.m, G.v,
                                                                   G.cfg.learning_rate, b1, b2, 1.0e-8f, c1, c2);
        rc = packWeights(G, s);
        if (rc) return rc;
    }
    double lossSum = 0.0;
    const int rc = readLoss(G, &lossSum, s, "spgpu_guiding_train");
    if (rc) return rc;
    G.lastLoss = steps ? lossSum / steps : 0.0;
    if (meanLoss) *meanLoss = G.lastLoss;
    return 0;
}

int guideRender(Ctx &C, GuideState *G, const spgpu_render_desc *d, float4 *film, int flags,
                unsigned long long *statsOut, float *msOut, cudaStream_t s) {
    const bool guided = (flags & 1) && G;
    const bool collect = (flags & 2) && G;
    if (!(flags & 4) && (guided || !collect)) {
        // the wavefront, with per-bounce network inference over the diffuse hits (and
        // training records when collecting)
        if (guided && d->integrator != SPGPU_INTEGRATOR_PATH) {
            setError("spgpu_guiding_render: guided rendering needs the path integrator");
            return SPGPU_EINVAL;
        }
        GuideView gv{};
        if (guided) {
            gv.packFwd = G->packFwd;
            gv.biasPad = G->biasPad;
            gv.alpha = G->cfg.bsdf_fraction;
            gv.collect = collect;
            gv.ring = G->samples;
            gv.capacity = G->capacity;
            gv.ringCtl = G->ctl;
            gv.guidedBounces = G->cfg.guided_bounces;
        }
        // plain and guided passes on the streaming wavefront unless the context asks for
        // pass-by-pass passes; collection passes keep per-path records in one slot for
        // the whole path, which the pass-by-pass wavefront provides
        if (!collect && C.wavefront == 0)
            return renderStream(&C, d->camera, d->width, d->height, d->spp, d->sample_offset, d->max_depth, d->seed,
                                d->integrator, film, statsOut, msOut, s, guided ? &gv : nullptr);
        return renderFrame(&C, d->camera, d->width, d->height, d->spp, d->sample_offset, d->max_depth, d->seed,
                           d->integrator, film, statsOut, msOut, s, guided ? &gv : nullptr);
    }
    GuidedArgs a;
    std::memset(&a, 0, sizeof(a));
    a.sv = C.view();
    a.cam = makeCamera(d->camera, d->width, d->height);
    a.W = d->width;
    a.H = d->height;
    a.npix = d->width * d->height;
    a.total = static_cast<long long>(a.npix) * d->spp;
    a.sampleOffset = d->sample_offset;
    a.maxDepth = d->max_depth;
    a.seed = d->seed;
    a.film = film;
    a.lo = C.bvh.lo;
    const float3 ext = C.bvh.hi - C.bvh.lo;
    a.invExt = mk(ext.x > 0 ? 1.0f / ext.x : 0.0f, ext.y > 0 ? 1.0f / ext.y : 0.0f, ext.z > 0 ? 1.0f / ext.z : 0.0f);
    a.alpha = G ? G->cfg.bsdf_fraction : 1.0f;
    unsigned long long *stats = nullptr;
    int *ctl = nullptr;
    if (G) {
        a.packFwd = G->packFwd;
        a.biasPad = G->biasPad;
        a.ring = G->samples;
        a.capacity = G->capacity;
        ctl = G->ctl;
    }
    // plain runs without guiding state use the render queues' counters
    static thread_local int *plainCtl = nullptr;
    static thread_local unsigned long long *plainStats = nullptr;
    if (!plainCtl) {
        cudaMalloc(&plainCtl, 4 * sizeof(int));
        cudaMalloc(&plainStats, 4 * sizeof(unsigned long long));
    }
    if (!ctl) ctl = plainCtl;
    stats = plainStats;
    a.ctl = ctl;
    a.stats = stats;
    cudaMemsetAsync(ctl + 1, 0, 3 * sizeof(int), s);
    cudaMemsetAsync(stats, 0, 4 * sizeof(unsigned long long), s);
    int sms = 0, occ = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, C.device);
    setGuideKernelAttributes();
    if (guided && collect) occ = tmemKernelResidentCtas(reinterpret_cast<const void *>(k_guided<true, true>), C.device);
    else if (guided) occ = tmemKernelResidentCtas(reinterpret_cast<const void *>(k_guided<true, false>), C.device);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_guided<false, false>, kGTile, kPlainSmem);
    const int grid = sms * std::max(1, occ);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    if (guided && collect) k_guided<true, true><<<grid, kGTile, kGuidedSmem, s>>>(a);
    else if (guided) k_guided<true, false><<<grid, kGTile, kGuidedSmem, s>>>(a);
    else k_guided<false, false><<<grid, kGTile, kPlainSmem, s>>>(a);
    cudaError_t e = cudaGetLastError();
    cudaEventRecord(e1, s);
    unsigned long long st[4] = {0, 0, 0, 0};
    int err = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(st, stats, sizeof(st), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err, ctl + 1, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    float ms = 0.0f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cudaFail("spgpu_guiding_render", e);
    for (int k = 0; k < 3; k++) statsOut[k] = st[k];
    statsOut[3] = 1;   // one persistent launch
    *msOut = ms;
    if (err) {
        setError("spgpu_guiding_render: traversal overflow or tensor-core wait timed out");
        return SPGPU_EKERNEL;
    }
    return 0;
}

long long guideSamples(const GuideState &G) {
    unsigned written = 0;
    cudaMemcpy(&written, G.ctl, sizeof(unsigned), cudaMemcpyDeviceToHost);
    return written;
}

}  // namespace spgpu
