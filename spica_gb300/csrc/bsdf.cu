// bsdf.cu -- function-level entry points over the device BSDFs and the sampler: the
// same __device__ functions that shade every hit of a render (common.cuh), evaluated
// on caller-given directions and random numbers, so they can be compared one call at a
// time with the reference's BSDF::f / pdf / sample (core/bsdf.cc:49-136) and with the
// published Philox4x32-10 known answers.
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/spica_gpu.h"
#include "ctx.cuh"

namespace spgpu {
namespace {

constexpr int kBsdfBlock = 256;

__device__ __forceinline__ float3 load3(const float *p, int64_t i) { return mk(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
__device__ __forceinline__ void store3(float *p, int64_t i, float3 v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}

// BSDF::f and BSDF::pdf in the shading frame.  The smooth dielectric's pdf is
// FresnelSpecular::pdf (F or 1 - F inside the 1e-4 cones about the delta directions,
// bxdf.cc:236), which the renderer itself never needs.
__global__ void k_bsdf_eval(MaterialRecord m, int64_t n, const float *wo, const float *wi, float *f, float *pdf) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float3 o = load3(wo, i), w = load3(wi, i);
        store3(f, i, bsdfF(m, o, w));
        pdf[i] = m.type == kMatDielectric ? bsdfPdfDielectricCone(m, o, w) : bsdfPdf(m, o, w);
    }
}

__global__ void k_bsdf_sample(MaterialRecord m, int64_t n, const float *wo, const float *u, float *wi, float *f,
                              float *pdf, int *type) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float3 o = load3(wo, i), r = load3(u, i);
        float3 w = mk(0, 0, 0);
        float p = 0.0f;
        int t = 0;
        const float3 v = bsdfSample(m, o, r.x, r.y, r.z, &w, &p, &t);
        store3(wi, i, w);
        store3(f, i, v);
        pdf[i] = p;
        type[i] = t;
    }
}

__global__ void k_philox(int64_t n, const uint4 *ctr, const uint2 *key, uint4 *raw, float4 *u) {
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const uint4 r = philox4x32_10(ctr[i], key[i]);
        raw[i] = r;
        u[i] = make_float4(u01(r.x), u01(r.y), u01(r.z), u01(r.w));
    }
}

int gridFor(int64_t n) { return static_cast<int>(std::min<int64_t>((n + kBsdfBlock - 1) / kBsdfBlock, 152 * 16)); }

// stream-ordered device staging for one blocking host call: inputs copied in, outputs
// copied back, everything freed, then one synchronise
struct Staging {
    cudaStream_t s;
    std::vector<void *> bufs;
    cudaError_t e = cudaSuccess;
    explicit Staging(cudaStream_t st) : s(st) {}
    template <class T>
    T *in(const T *host, size_t count) {
        T *d = out<T>(count);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d, host, sizeof(T) * count, cudaMemcpyHostToDevice, s);
        return d;
    }
    template <class T>
    T *out(size_t count) {
        void *d = nullptr;
        if (e == cudaSuccess) e = cudaMallocAsync(&d, std::max<size_t>(sizeof(T) * count, 16), s);
        if (e == cudaSuccess) bufs.push_back(d);
        return static_cast<T *>(d);
    }
    template <class T>
    void back(T *host, const T *dev, size_t count) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(host, dev, sizeof(T) * count, cudaMemcpyDeviceToHost, s);
    }
    cudaError_t finish() {
        for (void *d : bufs) cudaFreeAsync(d, s);
        const cudaError_t se = cudaStreamSynchronize(s);
        return e != cudaSuccess ? e : se;
    }
};

int oneMaterial(const char *who, const float *material, MaterialRecord *m) {
    std::vector<MaterialRecord> recs;
    if (int rc = materialRecords(who, material, 1, &recs)) return rc;
    *m = recs[0];
    return 0;
}

}  // namespace
}  // namespace spgpu

using namespace spgpu;

extern "C" {

int spgpu_bsdf_eval(spgpu_ctx *h, const float *material, int64_t n, const float *wo, const float *wi, float *f,
                    float *pdf) {
    return guarded("spgpu_bsdf_eval", [&]() -> int {
        if (!h || !material || n < 0 || (n > 0 && (!wo || !wi || !f || !pdf))) {
            setError("spgpu_bsdf_eval: invalid arguments");
            return SPGPU_EINVAL;
        }
        MaterialRecord m;
        if (int rc = oneMaterial("spgpu_bsdf_eval", material, &m)) return rc;
        if (n == 0) return 0;
        Ctx &C = h->c;
        cudaError_t e = cudaSetDevice(C.device);
        if (e != cudaSuccess) return cudaFail("spgpu_bsdf_eval: cudaSetDevice", e);
        const size_t n3 = static_cast<size_t>(n) * 3;
        Staging S(C.stream);
        const float *dWo = S.in(wo, n3), *dWi = S.in(wi, n3);
        float *dF = S.out<float>(n3), *dPdf = S.out<float>(static_cast<size_t>(n));
        if (S.e == cudaSuccess) {
            k_bsdf_eval<<<gridFor(n), kBsdfBlock, 0, C.stream>>>(m, n, dWo, dWi, dF, dPdf);
            S.e = cudaGetLastError();
        }
        S.back(f, dF, n3);
        S.back(pdf, dPdf, static_cast<size_t>(n));
        e = S.finish();
        return e == cudaSuccess ? 0 : cudaFail("spgpu_bsdf_eval", e);
    });
}

int spgpu_bsdf_sample(spgpu_ctx *h, const float *material, int64_t n, const float *wo, const float *u, float *wi,
                      float *f, float *pdf, int32_t *type) {
    return guarded("spgpu_bsdf_sample", [&]() -> int {
        if (!h || !material || n < 0 || (n > 0 && (!wo || !u || !wi || !f || !pdf || !type))) {
            setError("spgpu_bsdf_sample: invalid arguments");
            return SPGPU_EINVAL;
        }
        MaterialRecord m;
        if (int rc = oneMaterial("spgpu_bsdf_sample", material, &m)) return rc;
        if (n == 0) return 0;
        Ctx &C = h->c;
        cudaError_t e = cudaSetDevice(C.device);
        if (e != cudaSuccess) return cudaFail("spgpu_bsdf_sample: cudaSetDevice", e);
        const size_t n1 = static_cast<size_t>(n), n3 = n1 * 3;
        Staging S(C.stream);
        const float *dWo = S.in(wo, n3), *dU = S.in(u, n3);
        float *dWi = S.out<float>(n3), *dF = S.out<float>(n3), *dPdf = S.out<float>(n1);
        int *dT = S.out<int>(n1);
        if (S.e == cudaSuccess) {
            k_bsdf_sample<<<gridFor(n), kBsdfBlock, 0, C.stream>>>(m, n, dWo, dU, dWi, dF, dPdf, dT);
            S.e = cudaGetLastError();
        }
        S.back(wi, dWi, n3);
        S.back(f, dF, n3);
        S.back(pdf, dPdf, n1);
        S.back(reinterpret_cast<int *>(type), dT, n1);
        e = S.finish();
        return e == cudaSuccess ? 0 : cudaFail("spgpu_bsdf_sample", e);
    });
}

int spgpu_sampler_generate(spgpu_ctx *h, int64_t n, const uint32_t *counter, const uint32_t *key, uint32_t *raw,
                           float *u) {
    return guarded("spgpu_sampler_generate", [&]() -> int {
        if (!h || n < 0 || (n > 0 && (!counter || !key || !raw || !u))) {
            setError("spgpu_sampler_generate: invalid arguments");
            return SPGPU_EINVAL;
        }
        if (n == 0) return 0;
        Ctx &C = h->c;
        cudaError_t e = cudaSetDevice(C.device);
        if (e != cudaSuccess) return cudaFail("spgpu_sampler_generate: cudaSetDevice", e);
        const size_t n1 = static_cast<size_t>(n);
        Staging S(C.stream);
        const uint4 *dC = S.in(reinterpret_cast<const uint4 *>(counter), n1);
        const uint2 *dK = S.in(reinterpret_cast<const uint2 *>(key), n1);
        uint4 *dR = S.out<uint4>(n1);
        float4 *dU = S.out<float4>(n1);
        if (S.e == cudaSuccess) {
            k_philox<<<gridFor(n), kBsdfBlock, 0, C.stream>>>(n, dC, dK, dR, dU);
            S.e = cudaGetLastError();
        }
        S.back(reinterpret_cast<uint4 *>(raw), dR, n1);
        S.back(reinterpret_cast<float4 *>(u), dU, n1);
        e = S.finish();
        return e == cudaSuccess ? 0 : cudaFail("spgpu_sampler_generate", e);
    });
}

}  // extern "C"
