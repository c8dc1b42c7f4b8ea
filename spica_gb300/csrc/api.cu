// api.cu -- the C ABI of include/spica_gpu.h: context, scene upload (materials,
// per-triangle area lights, environment-map sampling tables), BVH build and the
// ray-batch trace kernels.  Rendering lives in wavefront.cu.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/spica_gpu.h"
#include "ctx.cuh"

namespace spgpu {

namespace {
thread_local std::string g_lastError;

template <class T>
int upload(T **dst, const T *src, size_t n, cudaStream_t s) {
    cudaFree(*dst);
    *dst = nullptr;
    if (n == 0) return 0;
    cudaError_t e = cudaMalloc(dst, sizeof(T) * n);
    if (e != cudaSuccess) return cudaFail("cudaMalloc", e);
    e = cudaMemcpyAsync(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cudaFail("cudaMemcpyAsync", e);
    return 0;
}

// --------------------------------------------------------------------------- env map
// Host construction of the sampling tables of Envmap::Envmap (lights/envmap.cc:17-47):
// the weight of texel (u, v) is the luminance of the mip-mapped map looked up at the
// texel centre with filter width 1/max(w, h) (core/mipmap.cc:67, a bilinear lookup on
// mip level 1 for power-of-two maps), times sin(theta); rows become conditional
// distributions and their integrals the marginal (core/sampling.cc:25-150).
struct HostMip {
    std::vector<int> w, h;
    std::vector<std::vector<double>> px;   // rgb interleaved
    void init(const float *img, int W, int H) {
        int n = 1;
        for (int v = std::max(W, H); v != 0; v >>= 1) n++;
        w.resize(n);
        h.resize(n);
        px.resize(n);
        w[0] = W;
        h[0] = H;
        px[0].assign(img, img + static_cast<size_t>(W) * H * 3);
        for (int i = 1; i < n; i++) {
            w[i] = std::max(1, w[i - 1] / 2);
            h[i] = std::max(1, h[i - 1] / 2);
            px[i].assign(static_cast<size_t>(w[i]) * h[i] * 3, 0.0);
            for (int y = 0; y < h[i]; y++)
                for (int x = 0; x < w[i]; x++)
                    for (int c = 0; c < 3; c++) {
                        const double s = texel(i - 1, 2 * x, 2 * y, c) + texel(i - 1, 2 * x + 1, 2 * y, c) +
                                         texel(i - 1, 2 * x, 2 * y + 1, c) + texel(i - 1, 2 * x + 1, 2 * y + 1, c);
                        px[i][(static_cast<size_t>(y) * w[i] + x) * 3 + c] = 0.25 * s;
                    }
        }
    }
    int levels() const { return static_cast<int>(w.size()); }
    double texel(int l, int s, int t, int c) const {
        s = (s % w[l] + w[l]) % w[l];
        t = (t % h[l] + h[l]) % h[l];
        return px[l][(static_cast<size_t>(t) * w[l] + s) * 3 + c];
    }
    void bilinear(int l, double s0, double t0, double *out) const {
        l = std::max(0, std::min(l, levels() - 1));
        const double s = s0 * w[l] - 0.5, t = t0 * h[l] - 0.5;
        const int si = static_cast<int>(s), ti = static_cast<int>(t);
        const double ds = s - si, dt = t - ti;
        for (int c = 0; c < 3; c++)
            out[c] = (1.0 - ds) * (1.0 - dt) * texel(l, si, ti, c) + ds * (1.0 - dt) * texel(l, si + 1, ti, c) +
                     (1.0 - ds) * dt * texel(l, si, ti + 1, c) + ds * dt * texel(l, si + 1, ti + 1, c);
    }
    void lookup(double s, double t, double width, double *out) const {
        const double level = levels() - 1 + std::log2(std::max(width, 1.0e-8));
        if (level < 0) return bilinear(0, s, t, out);
        if (level >= levels() - 1) {
            for (int c = 0; c < 3; c++) out[c] = texel(levels() - 1, 0, 0, c);
            return;
        }
        const double delta = level - static_cast<int>(level);
        double a[3], b[3];
        bilinear(static_cast<int>(level), s, t, a);
        bilinear(static_cast<int>(level + 1), s, t, b);
        for (int c = 0; c < 3; c++) out[c] = (1.0 - delta) * a[c] + delta * b[c];
    }
};

void buildDistribution1D(const double *f, int n, std::vector<float> *cdfOut, double *integral) {
    std::vector<double> cdf(n + 1, 0.0);
    for (int i = 1; i <= n; i++) cdf[i] = cdf[i - 1] + f[i - 1] / n;
    *integral = cdf[n];
    if (*integral == 0.0) {
        for (int i = 1; i <= n; i++) cdf[i] = static_cast<double>(i) / n;
    } else {
        for (int i = 1; i <= n; i++) cdf[i] /= *integral;
    }
    cdfOut->assign(cdf.begin(), cdf.end());
}

// guide table of a cdf over n intervals (sample1DGuided): guide[k] = the largest i with
// cdf[i] <= k / n, k = 0..n
void buildGuide(const float *cdf, int n, int *guide) {
    int i = 0;
    for (int k = 0; k <= n; k++) {
        const double t = static_cast<double>(k) / n;
        while (i < n && static_cast<double>(cdf[i + 1]) <= t) i++;
        guide[k] = i;
    }
}

int uploadEnv(Ctx &C, int W, int H, const float *img, double3 center, double radius) {
    if ((W & (W - 1)) != 0 || (H & (H - 1)) != 0) {
        setError("spgpu_upload_scene: environment map width and height must be powers of two");
        return SPGPU_EINVAL;
    }
    HostMip mip;
    mip.init(img, W, H);
    const double filter = 1.0 / std::max(W, H);
    const double pi = 4.0 * std::atan(1.0);
    std::vector<double> row(W), marg(H);
    std::vector<float> condCdf, condFunc(static_cast<size_t>(W) * H), margCdf, margFunc(H), tmp;
    condCdf.reserve(static_cast<size_t>(W + 1) * H);
    for (int v = 0; v < H; v++) {
        const double vp = (v + 0.5) / H;
        const double sinTheta = std::sin(pi * (v + 0.5) / H);
        for (int u = 0; u < W; u++) {
            double c[3];
            mip.lookup((u + 0.5) / W, vp, filter, c);
            row[u] = (0.2126 * c[0] + 0.7152 * c[1] + 0.0722 * c[2]) * sinTheta;
            condFunc[static_cast<size_t>(v) * W + u] = static_cast<float>(row[u]);
        }
        double integ;
        buildDistribution1D(row.data(), W, &tmp, &integ);
        condCdf.insert(condCdf.end(), tmp.begin(), tmp.end());
        marg[v] = integ;
        margFunc[v] = static_cast<float>(integ);
    }
    double margInt;
    buildDistribution1D(marg.data(), H, &margCdf, &margInt);
    std::vector<int> condGuide(static_cast<size_t>(W + 1) * H), margGuide(H + 1);
    for (int v = 0; v < H; v++)
        buildGuide(condCdf.data() + static_cast<size_t>(v) * (W + 1), W,
                   condGuide.data() + static_cast<size_t>(v) * (W + 1));
    buildGuide(margCdf.data(), H, margGuide.data());
    std::vector<float4> tex(static_cast<size_t>(W) * H);
    for (size_t i = 0; i < tex.size(); i++) tex[i] = make_float4(img[3 * i], img[3 * i + 1], img[3 * i + 2], 0.0f);
    DeviceEnv &E = C.env;
    E.w = W;
    E.h = H;
    int rc = 0;
    if ((rc = upload(&E.tex, tex.data(), tex.size(), C.stream))) return rc;
    if ((rc = upload(&E.condCdf, condCdf.data(), condCdf.size(), C.stream))) return rc;
    if ((rc = upload(&E.condFunc, condFunc.data(), condFunc.size(), C.stream))) return rc;
    if ((rc = upload(&E.margCdf, margCdf.data(), margCdf.size(), C.stream))) return rc;
    if ((rc = upload(&E.margFunc, margFunc.data(), margFunc.size(), C.stream))) return rc;
    if ((rc = upload(&E.condGuide, condGuide.data(), condGuide.size(), C.stream))) return rc;
    if ((rc = upload(&E.margGuide, margGuide.data(), margGuide.size(), C.stream))) return rc;
    E.margIntegral = static_cast<float>(margInt);
    E.center = mk(static_cast<float>(center.x), static_cast<float>(center.y), static_cast<float>(center.z));
    E.radius = static_cast<float>(radius);
    return 0;
}

void freeEnv(DeviceEnv *E) {
    cudaFree(E->tex);
    cudaFree(E->condCdf);
    cudaFree(E->condFunc);
    cudaFree(E->margCdf);
    cudaFree(E->margFunc);
    cudaFree(E->condGuide);
    cudaFree(E->margGuide);
    *E = DeviceEnv{};
}

void freeScene(Ctx &C) {
    cudaFree(C.verts);
    cudaFree(C.triMat);
    cudaFree(C.triLight);
    cudaFree(C.mats);
    cudaFree(C.lights);
    C.verts = nullptr;
    C.triMat = C.triLight = nullptr;
    C.mats = nullptr;
    C.lights = nullptr;
    freeEnv(&C.env);
    freeWideBVH(&C.bvh);
    C.sceneReady = C.bvhReady = false;
    C.hasEnv = false;
    C.ntri = C.nmat = C.nArea = 0;
}

// --------------------------------------------------------------------------- tracing
template <bool ANY, bool STATS>
__global__ void __launch_bounds__(kTraceBlock, 8) k_trace(const float4 *__restrict__ org, const float4 *__restrict__ dir,
                                                       int n, const WideNode *__restrict__ nodes,
                                                       const TriRecord *__restrict__ tris, uint32_t nNodes,
                                                       uint32_t nTris, spgpu_hit *__restrict__ outHit,
                                                       uint32_t *__restrict__ outAny, int *ctl,
                                                       unsigned long long *stats) {
    __shared__ uint2 stack[kStackShared * kTraceBlock];
    uint32_t nodeCount = 0, triCount = 0;
    bool overflow = false;
    auto fetch = [&](int i, float3 *o, float3 *d, float *t0, float *t1) {
        const float4 a = org[i], b = dir[i];
        *o = xyz(a);
        *d = xyz(b);
        *t0 = a.w;
        *t1 = b.w;
    };
    auto done = [&](int i, const TraceLane &L) {
        if (i < 0) return;
        if (ANY) {
            outAny[i] = L.found ? 1u : 0u;
            return;
        }
        float t = L.tmax, u = L.hu, v = L.hv;
        int prim = -1;
        if (L.found) {
            // The FP32 distance has relative error ~ eps * kappa with
            // kappa = (|o - v0| / t + 1) * |e1| |e2| / |det| (grazing incidence or a hit
            // very close to the origin); such hits are re-evaluated in FP64 to keep 1e-5
            // relative accuracy.
            const TriRecord tr = tris[L.hitSlot];
            const float3 e1 = xyz(tr.v1) - xyz(tr.v0), e2 = xyz(tr.v2) - xyz(tr.v0);
            const float det = fabsf(dot(e1, cross(L.d, e2)));
            const float kappa = (length(L.o - xyz(tr.v0)) / t + 1.0f) * length(e1) * length(e2);
            if (!(kappa < 16.0f * det)) refineHitFP64(tr, L.o, L.d, &t, &u, &v);
            prim = __float_as_int(tr.v0.w);
        }
        reinterpret_cast<float4 *>(outHit)[i] = make_float4(L.found ? t : 0.0f, __int_as_float(prim), u, v);
    };
    tracePersistent<ANY, STATS>(nodes, tris, nNodes, nTris, n, ctl + 1, stack + threadIdx.x, kTraceBlock, &nodeCount,
                                &triCount, &overflow, fetch, done);
    if (overflow) atomicOr(ctl, 1);
    if (STATS) {
        atomicAdd(&stats[0], static_cast<unsigned long long>(nodeCount));
        atomicAdd(&stats[1], static_cast<unsigned long long>(triCount));
    }
}

int numSMs(int device) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    return sms > 0 ? sms : 1;
}

// persistent grid: every block resident at once (SMs x blocks per SM)
int residentTraceBlocks(int device) {
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_trace<false, false>, kTraceBlock, 0);
    return numSMs(device) * (occ > 0 ? occ : 1);
}

int launchTrace(Ctx &C, int any, const float *org, const float *dir, int64_t n, void *out, cudaStream_t s,
                bool stats) {
    if (!C.bvhReady) {
        setError("spgpu_trace: no BVH (call spgpu_upload_scene and spgpu_build_bvh first)");
        return SPGPU_ESTATE;
    }
    if (n < 0 || (n > 0 && (!org || !dir || !out))) {
        setError("spgpu_trace: null pointer or negative ray count");
        return SPGPU_EINVAL;
    }
    if ((reinterpret_cast<uintptr_t>(org) | reinterpret_cast<uintptr_t>(dir) | reinterpret_cast<uintptr_t>(out)) & 15) {
        setError("spgpu_trace: ray and hit buffers must be 16-byte aligned");
        return SPGPU_EINVAL;
    }
    if (n == 0) return 0;
    if (n > (int64_t(1) << 30)) {
        setError("spgpu_trace: at most 2^30 rays per call");
        return SPGPU_EINVAL;
    }
    cudaError_t e = cudaMemsetAsync(C.traceErr, 0, 2 * sizeof(int), s);
    if (e != cudaSuccess) return cudaFail("cudaMemsetAsync", e);
    const int64_t blocksNeeded = (n + kTraceBlock - 1) / kTraceBlock;
    const int grid = static_cast<int>(std::min<int64_t>(blocksNeeded, static_cast<int64_t>(residentTraceBlocks(C.device))));
    const uint32_t NN = static_cast<uint32_t>(C.bvh.n_nodes), NT = static_cast<uint32_t>(C.bvh.ntri);
    const float4 *o4 = reinterpret_cast<const float4 *>(org);
    const float4 *d4 = reinterpret_cast<const float4 *>(dir);
    if (any) {
        if (stats) k_trace<true, true><<<grid, kTraceBlock, 0, s>>>(o4, d4, static_cast<int>(n), C.bvh.nodes, C.bvh.tris, NN, NT, nullptr,
                                                                    static_cast<uint32_t *>(out), C.traceErr, C.traceStats);
        else k_trace<true, false><<<grid, kTraceBlock, 0, s>>>(o4, d4, static_cast<int>(n), C.bvh.nodes, C.bvh.tris, NN, NT, nullptr,
                                                               static_cast<uint32_t *>(out), C.traceErr, C.traceStats);
    } else {
        if (stats) k_trace<false, true><<<grid, kTraceBlock, 0, s>>>(o4, d4, static_cast<int>(n), C.bvh.nodes, C.bvh.tris, NN, NT,
                                                                     static_cast<spgpu_hit *>(out), nullptr, C.traceErr,
                                                                     C.traceStats);
        else k_trace<false, false><<<grid, kTraceBlock, 0, s>>>(o4, d4, static_cast<int>(n), C.bvh.nodes, C.bvh.tris, NN, NT,
                                                                static_cast<spgpu_hit *>(out), nullptr, C.traceErr,
                                                                C.traceStats);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return cudaFail("trace launch", e);
    return 0;
}

int checkKernelError(Ctx &C, cudaStream_t s) {
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, C.traceErr, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cudaFail("trace", e);
    if (h) {
        setError("spgpu_trace: traversal stack overflow or malformed tree");
        return SPGPU_EKERNEL;
    }
    return 0;
}

// ---------------------------------------------------------------- static scratch
// Staging scratch of spgpu_trace_host_noalloc, reserved with the module on every device
// it is loaded on: the trace kernel's two control words (error flag, ray counter), then
// kNoAllocMaxRays origins+tmin, directions+tmax and hit records (16 bytes each).
constexpr int64_t kNoAllocMaxRays = int64_t(1) << 16;   // 65,536 rays per call
constexpr size_t kNoAllocCtlBytes = 256;
constexpr size_t kNoAllocRayBytes = static_cast<size_t>(kNoAllocMaxRays) * 16;
constexpr size_t kNoAllocScratchBytes = kNoAllocCtlBytes + 3 * kNoAllocRayBytes;   // 3 MiB + 256 B
static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
struct NoAllocSlot {
    std::once_flag once;
    unsigned char *base = nullptr;
    cudaError_t err = cudaSuccess;
};
NoAllocSlot g_noallocSlots[kNoAllocMaxDevices];

// Device address of the scratch on `device`, looked up once per device with that device
// current (the caller has made it current).
int noallocScratch(int device, unsigned char **base) {
    if (device < 0 || device >= kNoAllocMaxDevices) {
        setError("spgpu_trace_host_noalloc: device ordinal out of range");
        return SPGPU_EINVAL;
    }
    NoAllocSlot &S = g_noallocSlots[device];
    std::call_once(S.once, [&S] {
        void *p = nullptr;
        S.err = cudaGetSymbolAddress(&p, g_noallocScratch);
        S.base = static_cast<unsigned char *>(p);
    });
    if (S.err != cudaSuccess || !S.base) {
        return cudaFail("spgpu_trace_host_noalloc: cudaGetSymbolAddress",
                        S.err != cudaSuccess ? S.err : cudaErrorInvalidSymbol);
    }
    *base = S.base;
    return 0;
}

}  // namespace

void setError(const std::string &msg) { g_lastError = msg; }

// The C ABI's 8-float material records (SPGPU_MAT_*) as device records.  The plugins
// read alpha and IOR through Spectrum::gray() of a constant texture
// (roughconductor.cc:48, dielectric.cc:33); the same value is kept here.
int materialRecords(const char *who, const float *materials, int nmat, std::vector<MaterialRecord> *out) {
    out->assign(nmat, MaterialRecord{});
    auto gray1 = [](double v) { return 0.2126 * v + 0.7152 * v + 0.0722 * v; };
    for (int m = 0; m < nmat; m++) {
        const float *r = materials + 8 * m;
        MaterialRecord &M = (*out)[m];
        std::memset(&M, 0, sizeof(M));
        M.type = static_cast<int>(r[0]);
        const bool beckmannConductor = M.type == SPGPU_MAT_CONDUCTOR_BECKMANN;
        if (beckmannConductor) M.type = kMatConductor;
        if (M.type == kMatLambert) {
            M.a = make_float4(fmaxf(r[1], 0.0f), fmaxf(r[2], 0.0f), fmaxf(r[3], 0.0f), 0.0f);
        } else if (M.type == kMatConductor) {
            M.a = make_float4(r[2], r[3], r[4], static_cast<float>(gray1(r[1])));
            M.b = make_float4(r[5], r[6], r[7], beckmannConductor ? 1.0f : 0.0f);   // b.w: distribution
            if (!(M.a.w > 0.0f)) {
                setError(std::string(who) + ": conductor roughness must be positive (smooth conductors are not "
                         "supported)");
                return SPGPU_EINVAL;
            }
        } else if (M.type == kMatDielectric) {
            M.a = make_float4(0.0f, 0.0f, 0.0f, static_cast<float>(gray1(r[1])));
        } else if (M.type == kMatRoughDielectric) {
            // roughdielectric.cc:41-84: zero roughness is the smooth dielectric's FresnelSpecular
            const float alpha = static_cast<float>(gray1(r[1])), ior = static_cast<float>(gray1(r[2]));
            if (alpha == 0.0f) {
                M.type = kMatDielectric;
                M.a = make_float4(0.0f, 0.0f, 0.0f, ior);
            } else if (!(alpha > 0.0f) || !(ior > 0.0f) || (r[3] != 0.0f && r[3] != 1.0f)) {
                setError(std::string(who) + ": rough dielectric needs alpha >= 0, ior > 0, distribution 0 or 1");
                return SPGPU_EINVAL;
            } else {
                M.a = make_float4(alpha, ior, r[3], 0.0f);
            }
        } else if (M.type == kMatPlastic) {
            // plastic.cc:112-122 and PlasticBRDF's specular sampling weight (plastic.cc:26)
            const double kd = 0.2126 * r[1] + 0.7152 * r[2] + 0.0722 * r[3];
            const double ks = 0.2126 * r[4] + 0.7152 * r[5] + 0.0722 * r[6];
            const float ior = static_cast<float>(gray1(r[7]));
            if (!(ior > 0.0f) || !(kd + ks > 0.0)) {
                setError(std::string(who) + ": plastic needs ior > 0 and a non-black Kd + Ks");
                return SPGPU_EINVAL;
            }
            M.a = make_float4(r[1], r[2], r[3], ior);
            M.b = make_float4(r[4], r[5], r[6], static_cast<float>(ks / (kd + ks)));
        } else {
            setError(std::string(who) + ": unknown material type");
            return SPGPU_EINVAL;
        }
    }
    return 0;
}

int cudaFail(const char *what, cudaError_t e) {
    g_lastError = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? SPGPU_ENOMEM : SPGPU_ECUDA;
}

// The reference camera's transforms in double (core/transform.cc, core/camera.cc:20,
// cameras/perspective.cc:36): raster -> screen -> camera, then camera -> world.
CameraView makeCamera(const float *cam, int W, int H) {
    struct M {
        double m[4][4];
    };
    auto ident = [] {
        M r{};
        for (int i = 0; i < 4; i++) r.m[i][i] = 1.0;
        return r;
    };
    auto mul = [](const M &a, const M &b) {
        M r{};
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
                for (int k = 0; k < 4; k++) r.m[i][j] += a.m[i][k] * b.m[k][j];
        return r;
    };
    auto inv = [](const M &a) {   // Gauss-Jordan with full pivoting
        int ic[4], ir[4], piv[4] = {0, 0, 0, 0};
        M v = a;
        for (int i = 0; i < 4; i++) {
            int irow = 0, icol = 0;
            double big = 0.0;
            for (int j = 0; j < 4; j++) {
                if (piv[j] == 1) continue;
                for (int k = 0; k < 4; k++)
                    if (piv[k] == 0 && std::fabs(v.m[j][k]) >= big) {
                        big = std::fabs(v.m[j][k]);
                        irow = j;
                        icol = k;
                    }
            }
            ++piv[icol];
            if (irow != icol)
                for (int k = 0; k < 4; k++) std::swap(v.m[irow][k], v.m[icol][k]);
            ir[i] = irow;
            ic[i] = icol;
            const double p = 1.0 / v.m[icol][icol];
            v.m[icol][icol] = 1.0;
            for (int j = 0; j < 4; j++) v.m[icol][j] *= p;
            for (int j = 0; j < 4; j++) {
                if (j == icol) continue;
                const double save = v.m[j][icol];
                v.m[j][icol] = 0.0;
                for (int k = 0; k < 4; k++) v.m[j][k] -= v.m[icol][k] * save;
            }
        }
        for (int j = 3; j >= 0; j--)
            if (ir[j] != ic[j])
                for (int k = 0; k < 4; k++) std::swap(v.m[k][ir[j]], v.m[k][ic[j]]);
        return v;
    };
    const double pi = 4.0 * std::atan(1.0);
    double eye[3] = {cam[0], cam[1], cam[2]}, look[3] = {cam[3], cam[4], cam[5]}, up[3] = {cam[6], cam[7], cam[8]};
    auto norm3 = [](double *v) {
        const double n = 1.0 / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        v[0] *= n;
        v[1] *= n;
        v[2] *= n;
    };
    auto cross3 = [](const double *a, const double *b, double *r) {
        r[0] = a[1] * b[2] - a[2] * b[1];
        r[1] = a[2] * b[0] - a[0] * b[2];
        r[2] = a[0] * b[1] - a[1] * b[0];
    };
    double dir[3] = {look[0] - eye[0], look[1] - eye[1], look[2] - eye[2]};
    norm3(dir);
    norm3(up);
    double left[3], newUp[3];
    cross3(up, dir, left);
    norm3(left);
    cross3(dir, left, newUp);
    M c2w{};
    for (int i = 0; i < 3; i++) {
        c2w.m[i][0] = left[i];
        c2w.m[i][1] = newUp[i];
        c2w.m[i][2] = dir[i];
        c2w.m[i][3] = eye[i];
    }
    c2w.m[3][3] = 1.0;
    const double fov = cam[9] * pi / 180.0;
    const double aspect = static_cast<double>(W) / H, n = 1.0e-2, f = 1000.0;
    M pers{};
    pers.m[0][0] = 1.0 / aspect;
    pers.m[1][1] = 1.0;
    pers.m[2][2] = f / (f - n);
    pers.m[2][3] = -f * n / (f - n);
    pers.m[3][2] = 1.0;
    const double it = 1.0 / std::tan(fov / 2.0);
    M sc = ident();
    sc.m[0][0] = it;
    sc.m[1][1] = it;
    const M cameraToScreen = mul(sc, pers);
    M s1 = ident(), s2 = ident(), tr = ident();
    s1.m[0][0] = W;
    s1.m[1][1] = H;
    s2.m[0][0] = 0.5;
    s2.m[1][1] = -0.5;
    tr.m[0][3] = 1.0;
    tr.m[1][3] = -1.0;
    const M screenToRaster = mul(mul(s1, s2), tr);
    const M r2c = mul(inv(cameraToScreen), inv(screenToRaster));
    CameraView cv;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) cv.r2c[4 * i + j] = static_cast<float>(r2c.m[i][j]);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 4; j++) cv.c2w[4 * i + j] = static_cast<float>(c2w.m[i][j]);
    return cv;
}

}  // namespace spgpu

using namespace spgpu;

extern "C" {

const char *spgpu_last_error(void) { return g_lastError.c_str(); }

const char *spgpu_version(void) { return "spica-gb300 0.1 (sm_103a)"; }

int spgpu_create(const spgpu_config *cfg, spgpu_ctx **out) {
    return guarded("spgpu_create", [&]() -> int {
        if (!out) {
            setError("spgpu_create: null output pointer");
            return SPGPU_EINVAL;
        }
        *out = nullptr;
        auto *h = new spgpu_ctx();
        Ctx &C = h->c;
        C.device = cfg ? cfg->device : 0;
        if (cfg && (cfg->pass_lanes < 0 || cfg->pass_lanes > Ctx::kPassLanes)) {
            setError("spgpu_create: pass_lanes must be 0 (default) or 1.." + std::to_string(Ctx::kPassLanes));
            delete h;
            return SPGPU_EINVAL;
        }
        C.passLanes = cfg && cfg->pass_lanes > 0 ? cfg->pass_lanes : Ctx::kPassLanes;
        if (cfg && cfg->wavefront != 0 && cfg->wavefront != 1) {
            setError("spgpu_create: wavefront must be 0 (streaming) or 1 (pass by pass)");
            delete h;
            return SPGPU_EINVAL;
        }
        C.wavefront = cfg ? cfg->wavefront : 0;
        cudaError_t e = cudaSetDevice(C.device);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&C.stream, cudaStreamNonBlocking);
        for (int k = 0; k < Ctx::kPassLanes - 1 && e == cudaSuccess; k++) {
            e = cudaStreamCreateWithFlags(&C.laneStream[k], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&C.laneJoin[k], cudaEventDisableTiming);
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&C.laneFork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMalloc(&C.traceErr, 4 * sizeof(int));
        if (e == cudaSuccess) e = cudaMalloc(&C.traceStats, 4 * sizeof(unsigned long long));
        if (e != cudaSuccess) {
            const int rc = cudaFail("spgpu_create", e);
            delete h;
            return rc;
        }
        *out = h;
        return 0;
    });
}

void spgpu_destroy(spgpu_ctx *h) {
    if (!h) return;
    Ctx &C = h->c;
    cudaSetDevice(C.device);
    if (C.stream) cudaStreamSynchronize(C.stream);
    freeScene(C);
    for (auto &q : C.sq) freeStreamQueues(&q);
    freeRenderQueues(&C.rq);
    for (int k = 0; k < Ctx::kPassLanes - 1; k++) {
        freeRenderQueues(&C.rqLane[k]);
        if (C.laneStream[k]) cudaStreamDestroy(C.laneStream[k]);
        if (C.laneJoin[k]) cudaEventDestroy(C.laneJoin[k]);
    }
    if (C.laneFork) cudaEventDestroy(C.laneFork);
    freeBatch(C.batch);
    C.batch = nullptr;
    freeGuide(C.guide);
    C.guide = nullptr;
    cudaFree(C.traceErr);
    cudaFree(C.traceStats);
    cudaFree(C.hostStage);
    if (C.stream) cudaStreamDestroy(C.stream);
    delete h;
}

int spgpu_upload_scene(spgpu_ctx *h, int32_t ntri, const float *verts, const int32_t *tri_mat, int32_t nmat,
                       const float *materials, const float *tri_emit, int32_t env_w, int32_t env_h, const float *env) {
    return guarded("spgpu_upload_scene", [&]() -> int {
        NvtxRange nvtxRange("spgpu_upload_scene");
        if (!h || ntri <= 0 || !verts || !tri_mat || nmat <= 0 || !materials || (env && (env_w <= 0 || env_h <= 0))) {
            setError("spgpu_upload_scene: invalid arguments");
            return SPGPU_EINVAL;
        }
        Ctx &C = h->c;
        cudaSetDevice(C.device);
        freeScene(C);
        for (int i = 0; i < ntri; i++) {
            if (tri_mat[i] < 0 || tri_mat[i] >= nmat) {
                setError("spgpu_upload_scene: triangle material index out of range");
                return SPGPU_EINVAL;
            }
        }
        std::vector<MaterialRecord> mats;
        if (int rc = materialRecords("spgpu_upload_scene", materials, nmat, &mats)) return rc;
        // area lights: one per emitting triangle, in triangle order (sceneparser.cc:173-179)
        std::vector<LightRecord> lights;
        std::vector<int> triLight(ntri, -1);
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int i = 0; i < ntri; i++) {
            const float *v = verts + 9 * static_cast<int64_t>(i);
            for (int k = 0; k < 3; k++)
                for (int a = 0; a < 3; a++) {
                    lo[a] = std::min(lo[a], static_cast<double>(v[3 * k + a]));
                    hi[a] = std::max(hi[a], static_cast<double>(v[3 * k + a]));
                }
            if (!tri_emit) continue;
            const float *e = tri_emit + 3 * static_cast<int64_t>(i);
            if (e[0] == 0.0f && e[1] == 0.0f && e[2] == 0.0f) continue;
            const double e1[3] = {static_cast<double>(v[3]) - v[0], static_cast<double>(v[4]) - v[1],
                                  static_cast<double>(v[5]) - v[2]};
            const double e2[3] = {static_cast<double>(v[6]) - v[0], static_cast<double>(v[7]) - v[1],
                                  static_cast<double>(v[8]) - v[2]};
            const double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                 e1[0] * e2[1] - e1[1] * e2[0]};
            const double len = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
            if (!(len > 0.0)) {
                setError("spgpu_upload_scene: degenerate emitting triangle");
                return SPGPU_EINVAL;
            }
            LightRecord L;
            L.p0 = make_float4(v[0], v[1], v[2], static_cast<float>(0.5 * len));
            L.e1 = make_float4(v[3] - v[0], v[4] - v[1], v[5] - v[2], 0.0f);
            L.e2 = make_float4(v[6] - v[0], v[7] - v[1], v[8] - v[2], 0.0f);
            L.n = make_float4(static_cast<float>(c[0] / len), static_cast<float>(c[1] / len),
                              static_cast<float>(c[2] / len), 0.0f);
            L.L = make_float4(e[0], e[1], e[2], 0.0f);
            triLight[i] = static_cast<int>(lights.size());
            lights.push_back(L);
        }
        int rc = 0;
        if ((rc = upload(&C.verts, verts, static_cast<size_t>(ntri) * 9, C.stream))) return rc;
        if ((rc = upload(&C.triMat, reinterpret_cast<const int *>(tri_mat), static_cast<size_t>(ntri), C.stream)))
            return rc;
        if ((rc = upload(&C.triLight, triLight.data(), triLight.size(), C.stream))) return rc;
        if ((rc = upload(&C.mats, mats.data(), mats.size(), C.stream))) return rc;
        if (!lights.empty() && (rc = upload(&C.lights, lights.data(), lights.size(), C.stream))) return rc;
        C.ntri = ntri;
        C.nmat = nmat;
        C.nArea = static_cast<int>(lights.size());
        if (env) {
            const double3 center = make_double3(0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]), 0.5 * (lo[2] + hi[2]));
            const double d[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
            const double radius = 0.5 * std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            if ((rc = uploadEnv(C, env_w, env_h, env, center, radius))) return rc;
            C.hasEnv = true;
        }
        cudaError_t e = cudaStreamSynchronize(C.stream);
        if (e != cudaSuccess) return cudaFail("spgpu_upload_scene", e);
        C.sceneReady = true;
        return 0;
    });
}

int spgpu_build_bvh(spgpu_ctx *h) {
    return guarded("spgpu_build_bvh", [&]() -> int {
        NvtxRange nvtxRange("spgpu_build_bvh");
        if (!h) {
            setError("spgpu_build_bvh: null context");
            return SPGPU_EINVAL;
        }
        Ctx &C = h->c;
        if (!C.sceneReady) {
            setError("spgpu_build_bvh: no scene uploaded");
            return SPGPU_ESTATE;
        }
        cudaSetDevice(C.device);
        C.bvhReady = false;
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, C.stream);
        char err[256] = {0};
        const int rc = buildWideBVH(C.verts, C.ntri, C.triMat, C.triLight, &C.bvh, C.stream, err, sizeof(err));
        cudaEventRecord(b, C.stream);
        cudaEventSynchronize(b);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        if (rc != 0) {
            setError(err);
            return SPGPU_EBUILD;
        }
        C.buildMs = ms;
        C.bvhReady = true;
        freeRenderQueues(&C.rq);   // cached graphs refer to the old tree
        for (int k = 0; k < Ctx::kPassLanes - 1; k++) freeRenderQueues(&C.rqLane[k]);
        for (auto &q : C.sq) freeStreamQueues(&q);
        return 0;
    });
}

int spgpu_bvh_stats(spgpu_ctx *h, spgpu_bvh_info *out) {
    if (!h || !out) {
        setError("spgpu_bvh_stats: invalid arguments");
        return SPGPU_EINVAL;
    }
    Ctx &C = h->c;
    std::memset(out, 0, sizeof(*out));
    out->triangles = C.ntri;
    out->wide_nodes = C.bvh.n_nodes;
    out->depth = C.bvh.depth;
    out->lights = C.nArea + (C.hasEnv ? 1 : 0);
    out->build_ms = C.buildMs;
    out->bounds[0] = C.bvh.lo.x;
    out->bounds[1] = C.bvh.lo.y;
    out->bounds[2] = C.bvh.lo.z;
    out->bounds[3] = C.bvh.hi.x;
    out->bounds[4] = C.bvh.hi.y;
    out->bounds[5] = C.bvh.hi.z;
    return 0;
}

int spgpu_trace(spgpu_ctx *h, int any_hit, const float *org_tmin, const float *dir_tmax, int64_t n, void *out,
                void *stream) {
    NvtxRange nvtxRange("spgpu_trace");
    if (!h) {
        setError("spgpu_trace: null context");
        return SPGPU_EINVAL;
    }
    Ctx &C = h->c;
    cudaSetDevice(C.device);
    return launchTrace(C, any_hit, org_tmin, dir_tmax, n, out, static_cast<cudaStream_t>(stream), false);
}

int spgpu_trace_stats(spgpu_ctx *h, int any_hit, const float *org_tmin, const float *dir_tmax, int64_t n, void *out,
                      spgpu_trace_counters *counters) {
    NvtxRange nvtxRange("spgpu_trace_stats");
    if (!h || !counters) {
        setError("spgpu_trace_stats: invalid arguments");
        return SPGPU_EINVAL;
    }
    Ctx &C = h->c;
    cudaSetDevice(C.device);
    cudaError_t e = cudaMemsetAsync(C.traceStats, 0, 4 * sizeof(unsigned long long), C.stream);
    if (e != cudaSuccess) return cudaFail("cudaMemsetAsync", e);
    int rc = launchTrace(C, any_hit, org_tmin, dir_tmax, n, out, C.stream, true);
    if (rc) return rc;
    if ((rc = checkKernelError(C, C.stream))) return rc;
    unsigned long long st[4];
    e = cudaMemcpy(st, C.traceStats, sizeof(st), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cudaFail("cudaMemcpy", e);
    counters->rays = n;
    counters->nodes_per_ray = n ? static_cast<double>(st[0]) / n : 0.0;
    counters->tris_per_ray = n ? static_cast<double>(st[1]) / n : 0.0;
    return 0;
}

int spgpu_trace_host(spgpu_ctx *h, int any_hit, const float *org_tmin, const float *dir_tmax, int64_t n, void *out) {
    return guarded("spgpu_trace_host", [&]() -> int {
        NvtxRange nvtxRange("spgpu_trace_host");
        if (!h) {
            setError("spgpu_trace_host: null context");
            return SPGPU_EINVAL;
        }
        Ctx &C = h->c;
        if (n < 0 || (n > 0 && (!org_tmin || !dir_tmax || !out))) {
            setError("spgpu_trace_host: invalid arguments");
            return SPGPU_EINVAL;
        }
        if (n == 0) return 0;
        if (n > (int64_t(1) << 30)) {
            setError("spgpu_trace_host: at most 2^30 rays per call");
            return SPGPU_EINVAL;
        }
        // one call at a time per context: the calls share the control words and the
        // staging buffer (concurrent callers on one context queue here)
        std::lock_guard<std::mutex> lock(C.hostTraceMu);
        cudaError_t e = cudaSetDevice(C.device);
        if (e != cudaSuccess) return cudaFail("spgpu_trace_host: cudaSetDevice", e);
        const size_t rayBytes = static_cast<size_t>(n) * 16;
        const size_t outBytes = static_cast<size_t>(n) * (any_hit ? 4 : 16);
        const size_t need = 2 * rayBytes + ((outBytes + 255) & ~size_t(255));
        if (need > C.hostStageBytes) {
            // grow geometrically so that a stream of single-ray calls allocates once
            const size_t grow = std::max(need, std::max<size_t>(2 * C.hostStageBytes, size_t(1) << 16));
            if (C.hostStage) {
                e = cudaStreamSynchronize(C.stream);
                if (e != cudaSuccess) return cudaFail("spgpu_trace_host", e);
                cudaFree(C.hostStage);
                C.hostStage = nullptr;
                C.hostStageBytes = 0;
            }
            e = cudaMalloc(&C.hostStage, grow);
            if (e != cudaSuccess) return cudaFail("spgpu_trace_host: staging buffer", e);
            C.hostStageBytes = grow;
        }
        float *dO = reinterpret_cast<float *>(C.hostStage);
        float *dD = reinterpret_cast<float *>(C.hostStage + rayBytes);
        void *dOut = C.hostStage + 2 * rayBytes;
        e = cudaMemcpyAsync(dO, org_tmin, rayBytes, cudaMemcpyHostToDevice, C.stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dD, dir_tmax, rayBytes, cudaMemcpyHostToDevice, C.stream);
        if (e != cudaSuccess) return cudaFail("spgpu_trace_host", e);
        int rc = launchTrace(C, any_hit, dO, dD, n, dOut, C.stream, false);
        if (rc) return rc;
        e = cudaMemcpyAsync(out, dOut, outBytes, cudaMemcpyDeviceToHost, C.stream);
        if (e != cudaSuccess) return cudaFail("spgpu_trace_host", e);
        return checkKernelError(C, C.stream);
    });
}

int spgpu_trace_host_noalloc(spgpu_ctx *h, int any_hit, const float *org_tmin, const float *dir_tmax, int64_t n,
                             void *out) {
    return guarded("spgpu_trace_host_noalloc", [&]() -> int {
        NvtxRange nvtxRange("spgpu_trace_host_noalloc");
        if (!h) {
            setError("spgpu_trace_host_noalloc: null context");
            return SPGPU_EINVAL;
        }
        Ctx &C = h->c;
        if (n < 0 || (n > 0 && (!org_tmin || !dir_tmax || !out))) {
            setError("spgpu_trace_host_noalloc: invalid arguments");
            return SPGPU_EINVAL;
        }
        if (n > kNoAllocMaxRays) {
            setError("spgpu_trace_host_noalloc: " + std::to_string(n) + " rays exceed the static scratch limit of " +
                     std::to_string(kNoAllocMaxRays) + " rays per call (split the batch or use spgpu_trace_host)");
            return SPGPU_EINVAL;
        }
        if (!C.bvhReady) {
            setError("spgpu_trace_host_noalloc: no BVH (call spgpu_upload_scene and spgpu_build_bvh first)");
            return SPGPU_ESTATE;
        }
        if (n == 0) return 0;
        cudaError_t e = cudaSetDevice(C.device);
        if (e != cudaSuccess) return cudaFail("spgpu_trace_host_noalloc: cudaSetDevice", e);
        unsigned char *base = nullptr;
        int rc = noallocScratch(C.device, &base);
        if (rc) return rc;
        int *ctl = reinterpret_cast<int *>(base);
        float4 *dO = reinterpret_cast<float4 *>(base + kNoAllocCtlBytes);
        float4 *dD = reinterpret_cast<float4 *>(base + kNoAllocCtlBytes + kNoAllocRayBytes);
        unsigned char *dOut = base + kNoAllocCtlBytes + 2 * kNoAllocRayBytes;
        const size_t rayBytes = static_cast<size_t>(n) * 16;
        const size_t outBytes = static_cast<size_t>(n) * (any_hit ? 4 : 16);
        cudaStream_t s = C.stream;
        // the error flag and the ray counter start at zero
        e = cudaMemsetAsync(ctl, 0, 2 * sizeof(int), s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dO, org_tmin, rayBytes, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dD, dir_tmax, rayBytes, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return cudaFail("spgpu_trace_host_noalloc", e);
        const int64_t blocksNeeded = (n + kTraceBlock - 1) / kTraceBlock;
        const int grid = static_cast<int>(std::min<int64_t>(blocksNeeded, static_cast<int64_t>(residentTraceBlocks(C.device))));
        const uint32_t NN = static_cast<uint32_t>(C.bvh.n_nodes), NT = static_cast<uint32_t>(C.bvh.ntri);
        if (any_hit)
            k_trace<true, false><<<grid, kTraceBlock, 0, s>>>(dO, dD, static_cast<int>(n), C.bvh.nodes, C.bvh.tris, NN, NT,
                                                              nullptr, reinterpret_cast<uint32_t *>(dOut), ctl, nullptr);
        else
            k_trace<false, false><<<grid, kTraceBlock, 0, s>>>(dO, dD, static_cast<int>(n), C.bvh.nodes, C.bvh.tris, NN,
                                                               NT, reinterpret_cast<spgpu_hit *>(dOut), nullptr, ctl,
                                                               nullptr);
        e = cudaGetLastError();
        if (e != cudaSuccess) return cudaFail("spgpu_trace_host_noalloc: launch", e);
        int flag = 0;
        e = cudaMemcpyAsync(out, dOut, outBytes, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, ctl, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cudaFail("spgpu_trace_host_noalloc", e);
        if (flag) {
            setError("spgpu_trace_host_noalloc: traversal stack overflow or malformed tree");
            return SPGPU_EKERNEL;
        }
        return 0;
    });
}

int spgpu_render(spgpu_ctx *h, const spgpu_render_desc *d, float *film, spgpu_render_stats *stats, void *stream) {
    NvtxRange nvtxRange("spgpu_render");
    if (!h || !d || !film) {
        setError("spgpu_render: invalid arguments");
        return SPGPU_EINVAL;
    }
    Ctx &C = h->c;
    if (!C.bvhReady) {
        setError("spgpu_render: no BVH (call spgpu_upload_scene and spgpu_build_bvh first)");
        return SPGPU_ESTATE;
    }
    if (d->width <= 0 || d->height <= 0 || d->spp < 0 || d->max_depth < 0 || d->max_depth > 64 ||
        (d->integrator != SPGPU_INTEGRATOR_PATH && d->integrator != SPGPU_INTEGRATOR_DIRECT) ||
        static_cast<int64_t>(d->width) * d->height > (int64_t(1) << 28)) {
        setError("spgpu_render: invalid resolution, spp, max_depth or integrator");
        return SPGPU_EINVAL;
    }
    if (reinterpret_cast<uintptr_t>(film) & 15) {
        setError("spgpu_render: film must be 16-byte aligned");
        return SPGPU_EINVAL;
    }
    cudaSetDevice(C.device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned long long st[4] = {0, 0, 0, 0};
    float ms = 0.0f;
    const int rc =
        C.wavefront == 0
            ? renderStream(&C, d->camera, d->width, d->height, d->spp, d->sample_offset, d->max_depth, d->seed,
                           d->integrator, reinterpret_cast<float4 *>(film), st, &ms, s)
            : renderFrame(&C, d->camera, d->width, d->height, d->spp, d->sample_offset, d->max_depth, d->seed,
                          d->integrator, reinterpret_cast<float4 *>(film), st, &ms, s);
    if (stats) {
        stats->paths = static_cast<int64_t>(st[0]);
        stats->rays_closest = static_cast<int64_t>(st[1]);
        stats->rays_shadow = static_cast<int64_t>(st[2]);
        stats->ms = ms;
        stats->kernel_launches = static_cast<int64_t>(st[3]);
    }
    return rc;
}

int spgpu_render_profile(spgpu_ctx *h, const spgpu_render_desc *d, float *film, spgpu_kernel_profile *out,
                         void *stream) {
    NvtxRange nvtxRange("spgpu_render_profile");
    if (!h || !d || !film || !out) {
        setError("spgpu_render_profile: invalid arguments");
        return SPGPU_EINVAL;
    }
    Ctx &C = h->c;
    if (!C.bvhReady) {
        setError("spgpu_render_profile: no BVH");
        return SPGPU_ESTATE;
    }
    if (d->width <= 0 || d->height <= 0 || d->spp < 0 || d->max_depth < 0 || d->max_depth > 64 ||
        (d->integrator != SPGPU_INTEGRATOR_PATH && d->integrator != SPGPU_INTEGRATOR_DIRECT) ||
        (reinterpret_cast<uintptr_t>(film) & 15)) {
        setError("spgpu_render_profile: invalid resolution, spp, max_depth, integrator or film alignment");
        return SPGPU_EINVAL;
    }
    cudaSetDevice(C.device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::memset(out, 0, sizeof(*out));
    long long launches[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    unsigned long long st[4] = {0, 0, 0, 0}, vis[4] = {0, 0, 0, 0};
    const int rc =
        C.wavefront == 0
            ? renderStreamProfile(&C, d->camera, d->width, d->height, d->spp, d->sample_offset, d->max_depth, d->seed,
                                  d->integrator, reinterpret_cast<float4 *>(film), out->kernel_ms, launches, st, vis,
                                  s)
            : renderProfile(&C, d->camera, d->width, d->height, d->spp, d->sample_offset, d->max_depth, d->seed,
                            d->integrator, reinterpret_cast<float4 *>(film), out->kernel_ms, launches, st, vis, s);
    for (int k = 0; k < 8; k++) out->launches[k] = launches[k];
    out->paths = static_cast<int64_t>(st[0]);
    out->rays_closest = static_cast<int64_t>(st[1]);
    out->rays_shadow = static_cast<int64_t>(st[2]);
    out->closest_nodes_per_ray = st[1] ? static_cast<double>(vis[0]) / st[1] : 0.0;
    out->closest_tris_per_ray = st[1] ? static_cast<double>(vis[1]) / st[1] : 0.0;
    out->shadow_nodes_per_ray = st[2] ? static_cast<double>(vis[2]) / st[2] : 0.0;
    out->shadow_tris_per_ray = st[2] ? static_cast<double>(vis[3]) / st[2] : 0.0;
    return rc;
}

int spgpu_batch_prepare(spgpu_ctx *h, int32_t count, const spgpu_batch_item *items, int32_t autotune,
                        spgpu_batch_tuning *tuning) {
    return guarded("spgpu_batch_prepare", [&]() -> int {
        NvtxRange nvtxRange("spgpu_batch_prepare");
        if (!h || count <= 0 || !items || autotune < 0 || autotune > SPGPU_BATCH_PERSISTENT) {
            setError("spgpu_batch_prepare: invalid arguments");
            return SPGPU_EINVAL;
        }
        cudaSetDevice(h->c.device);
        return batchPrepare(h, &h->c.batch, count, items, autotune, tuning);
    });
}

int64_t spgpu_batch_film_pixels(spgpu_ctx *h) { return h && h->c.batch ? batchPixels(*h->c.batch) : -1; }

int spgpu_batch_run(spgpu_ctx *h, float *films, double *render_ms, spgpu_render_stats *stats, void *stream) {
    return guarded("spgpu_batch_run", [&]() -> int {
        NvtxRange nvtxRange("spgpu_batch_run");
        if (!h || !films || !render_ms) {
            setError("spgpu_batch_run: invalid arguments");
            return SPGPU_EINVAL;
        }
        Ctx &C = h->c;
        if (!C.batch) {
            setError("spgpu_batch_run: no batch prepared");
            return SPGPU_ESTATE;
        }
        if (reinterpret_cast<uintptr_t>(films) & 15) {
            setError("spgpu_batch_run: films must be 16-byte aligned");
            return SPGPU_EINVAL;
        }
        cudaSetDevice(C.device);
        unsigned long long st[4] = {0, 0, 0, 0};
        float ms = 0.0f;
        const int rc = batchRun(C, *C.batch, reinterpret_cast<float4 *>(films), render_ms, st, &ms,
                                static_cast<cudaStream_t>(stream));
        if (stats) {
            stats->paths = static_cast<int64_t>(st[0]);
            stats->rays_closest = static_cast<int64_t>(st[1]);
            stats->rays_shadow = static_cast<int64_t>(st[2]);
            stats->ms = ms;
            stats->kernel_launches = static_cast<int64_t>(st[3]);
        }
        return rc;
    });
}

int spgpu_batch_profile(spgpu_ctx *h, float *films, spgpu_kernel_profile *out, void *stream) {
    return guarded("spgpu_batch_profile", [&]() -> int {
        NvtxRange nvtxRange("spgpu_batch_profile");
        if (!h || !films || !out || (reinterpret_cast<uintptr_t>(films) & 15)) {
            setError("spgpu_batch_profile: invalid arguments (films 16-byte aligned)");
            return SPGPU_EINVAL;
        }
        Ctx &C = h->c;
        if (!C.batch) {
            setError("spgpu_batch_profile: no batch prepared");
            return SPGPU_ESTATE;
        }
        cudaSetDevice(C.device);
        std::memset(out, 0, sizeof(*out));
        long long launches[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        unsigned long long st[4] = {0, 0, 0, 0}, vis[4] = {0, 0, 0, 0};
        const int rc = batchProfile(C, *C.batch, reinterpret_cast<float4 *>(films), out->kernel_ms, launches, st, vis,
                                    static_cast<cudaStream_t>(stream));
        for (int k = 0; k < 8; k++) out->launches[k] = launches[k];
        out->paths = static_cast<int64_t>(st[0]);
        out->rays_closest = static_cast<int64_t>(st[1]);
        out->rays_shadow = static_cast<int64_t>(st[2]);
        out->closest_nodes_per_ray = st[1] ? static_cast<double>(vis[0]) / st[1] : 0.0;
        out->closest_tris_per_ray = st[1] ? static_cast<double>(vis[1]) / st[1] : 0.0;
        out->shadow_nodes_per_ray = st[2] ? static_cast<double>(vis[2]) / st[2] : 0.0;
        out->shadow_tris_per_ray = st[2] ? static_cast<double>(vis[3]) / st[2] : 0.0;
        return rc;
    });
}

int spgpu_guiding_init(spgpu_ctx *h, const spgpu_guiding_config *cfg) {
    return guarded("spgpu_guiding_init", [&]() -> int {
        NvtxRange nvtxRange("spgpu_guiding_init");
        if (!h || !cfg) {
            setError("spgpu_guiding_init: invalid arguments");
            return SPGPU_EINVAL;
        }
        cudaSetDevice(h->c.device);
        return guideInit(h->c, &h->c.guide, cfg);
    });
}

int spgpu_guiding_render(spgpu_ctx *h, const spgpu_render_desc *d, float *film, int32_t flags,
                         spgpu_render_stats *stats, void *stream) {
    NvtxRange nvtxRange("spgpu_guiding_render");
    if (!h || !d || !film || d->width <= 0 || d->height <= 0 || d->spp < 0 || d->max_depth < 0 ||
        d->max_depth > 12 || d->integrator != SPGPU_INTEGRATOR_PATH || (reinterpret_cast<uintptr_t>(film) & 15) ||
        (flags & ~(SPGPU_GUIDE_GUIDED | SPGPU_GUIDE_COLLECT | SPGPU_GUIDE_MEGAKERNEL))) {
        setError("spgpu_guiding_render: invalid arguments (path integrator, max_depth <= 12, aligned film, flags)");
        return SPGPU_EINVAL;
    }
    Ctx &C = h->c;
    if (!C.bvhReady) {
        setError("spgpu_guiding_render: no BVH");
        return SPGPU_ESTATE;
    }
    if ((flags & (SPGPU_GUIDE_GUIDED | SPGPU_GUIDE_COLLECT)) && !C.guide) {
        setError("spgpu_guiding_render: call spgpu_guiding_init first");
        return SPGPU_ESTATE;
    }
    cudaSetDevice(C.device);
    unsigned long long st[4] = {0, 0, 0, 0};
    float ms = 0.0f;
    const int rc = guideRender(C, flags ? C.guide : nullptr, d, reinterpret_cast<float4 *>(film), flags, st, &ms,
                               static_cast<cudaStream_t>(stream));
    if (stats) {
        stats->paths = static_cast<int64_t>(st[0]);
        stats->rays_closest = static_cast<int64_t>(st[1]);
        stats->rays_shadow = static_cast<int64_t>(st[2]);
        stats->ms = ms;
        stats->kernel_launches = static_cast<int64_t>(st[3]);
    }
    return rc;
}

int spgpu_guiding_train(spgpu_ctx *h, int32_t steps, double *mean_loss) {
    NvtxRange nvtxRange("spgpu_guiding_train");
    if (!h || steps < 0) {
        setError("spgpu_guiding_train: invalid arguments");
        return SPGPU_EINVAL;
    }
    if (!h->c.guide) {
        setError("spgpu_guiding_train: call spgpu_guiding_init first");
        return SPGPU_ESTATE;
    }
    cudaSetDevice(h->c.device);
    return guideTrain(h->c, *h->c.guide, steps, mean_loss);
}

int64_t spgpu_guiding_samples(spgpu_ctx *h) { return h && h->c.guide ? guideSamples(*h->c.guide) : -1; }

int spgpu_guiding_ring(spgpu_ctx *h, float *dst, int32_t max_samples, int32_t *count) {
    if (!h || !h->c.guide || max_samples < 0 || (max_samples > 0 && !dst) || !count) {
        setError("spgpu_guiding_ring: invalid arguments or no guiding state");
        return SPGPU_EINVAL;
    }
    cudaSetDevice(h->c.device);
    return guideRing(*h->c.guide, dst, max_samples, count);
}

int spgpu_guiding_params(spgpu_ctx *h, float *params, int32_t set) {
    if (!h || !params || !h->c.guide) {
        setError("spgpu_guiding_params: invalid arguments or no guiding state");
        return SPGPU_EINVAL;
    }
    cudaSetDevice(h->c.device);
    return guideParams(h->c, *h->c.guide, params, set);
}

int spgpu_guiding_mlp(spgpu_ctx *h, const float *features, int32_t n, float *raw, void *stream) {
    NvtxRange nvtxRange("spgpu_guiding_mlp");
    if (!h || !h->c.guide || n < 0 || (n > 0 && (!features || !raw))) {
        setError("spgpu_guiding_mlp: invalid arguments or no guiding state");
        return SPGPU_EINVAL;
    }
    if (n == 0) return 0;
    cudaSetDevice(h->c.device);
    return guideForward(h->c, *h->c.guide, features, n, raw, static_cast<cudaStream_t>(stream));
}

int spgpu_guiding_grad(spgpu_ctx *h, const float *samples, int32_t n, float *grad, double *loss, void *stream) {
    NvtxRange nvtxRange("spgpu_guiding_grad");
    if (!h || !h->c.guide || n <= 0 || !samples || !grad) {
        setError("spgpu_guiding_grad: invalid arguments or no guiding state");
        return SPGPU_EINVAL;
    }
    cudaSetDevice(h->c.device);
    return guideGrad(h->c, *h->c.guide, samples, n, grad, loss, static_cast<cudaStream_t>(stream));
}

int spgpu_film_resolve(spgpu_ctx *h, const float *film, int32_t width, int32_t height, int32_t format,
                       double param, void *out, void *stream) {
    NvtxRange nvtxRange("spgpu_film_resolve");
    if (!h || !film || !out || width <= 0 || height <= 0 || static_cast<int64_t>(width) * height > (int64_t(1) << 28) ||
        format < SPGPU_FILM_RGBE || format > SPGPU_FILM_DURAND ||
        (format != SPGPU_FILM_RGBE && !(param > 0.0)) || (reinterpret_cast<uintptr_t>(film) & 15) ||
        (format != SPGPU_FILM_GAMMA_BYTES && (reinterpret_cast<uintptr_t>(out) & 3))) {
        setError("spgpu_film_resolve: invalid arguments (16-byte aligned film, 4-byte aligned RGBE or float "
                 "output, known format, param > 0)");
        return SPGPU_EINVAL;
    }
    cudaSetDevice(h->c.device);
    return filmResolve(h->c, film, width, height, format, param, out, static_cast<cudaStream_t>(stream));
}

int spgpu_write_hdr(const char *path, const uint8_t *rgbe, int32_t width, int32_t height) {
    return guarded("spgpu_write_hdr", [&]() -> int {
        if (!path || !rgbe || width <= 0 || height <= 0 || width > 0x7FFF) {
            setError("spgpu_write_hdr: invalid arguments (scanline width < 32768)");
            return SPGPU_EINVAL;
        }
        return writeHdr(path, rgbe, width, height);
    });
}

int spgpu_write_png(const char *path, const uint8_t *rgb, int32_t width, int32_t height) {
    return guarded("spgpu_write_png", [&]() -> int {
        if (!path || !rgb || width <= 0 || height <= 0) {
            setError("spgpu_write_png: invalid arguments");
            return SPGPU_EINVAL;
        }
        return writePng(path, rgb, width, height);
    });
}

int spgpu_render_host(spgpu_ctx *h, const spgpu_render_desc *d, float *film, spgpu_render_stats *stats) {
    return guarded("spgpu_render_host", [&]() -> int {
        NvtxRange nvtxRange("spgpu_render_host");
        if (!h || !d || !film) {
            setError("spgpu_render_host: invalid arguments");
            return SPGPU_EINVAL;
        }
        Ctx &C = h->c;
        if (d->width <= 0 || d->height <= 0) {
            setError("spgpu_render_host: invalid resolution");
            return SPGPU_EINVAL;
        }
        cudaSetDevice(C.device);
        const size_t bytes = static_cast<size_t>(d->width) * d->height * 16;
        float *dFilm = nullptr;
        cudaError_t e = cudaMallocAsync(&dFilm, bytes, C.stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dFilm, film, bytes, cudaMemcpyHostToDevice, C.stream);
        if (e != cudaSuccess) {
            cudaFreeAsync(dFilm, C.stream);
            return cudaFail("spgpu_render_host", e);
        }
        int rc = spgpu_render(h, d, dFilm, stats, C.stream);
        if (rc == 0) {
            e = cudaMemcpyAsync(film, dFilm, bytes, cudaMemcpyDeviceToHost, C.stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(C.stream);
            if (e != cudaSuccess) rc = cudaFail("spgpu_render_host", e);
        }
        cudaFreeAsync(dFilm, C.stream);
        cudaStreamSynchronize(C.stream);
        return rc;
    });
}

}  // extern "C"
