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
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/spica_gpu.h"
#include "ctx.cuh"

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

// ---------------------------------------------------------------- environment map
// MipMap::bilinear on level 0 with repeat wrap (core/mipmap.cc:81-93)
__device__ __forceinline__ float3 envTexel(const DeviceEnv &E, int s, int t) {
    s = (s % E.w + E.w) % E.w;
    t = (t % E.h + E.h) % E.h;
    return xyz(__ldg(&E.tex[t * E.w + s]));
}
__device__ __forceinline__ float3 envLookup(const DeviceEnv &E, float u, float v) {
    const float s = u * E.w - 0.5f, t = v * E.h - 0.5f;
    const int si = static_cast<int>(s), ti = static_cast<int>(t);
    const float ds = s - si, dt = t - ti;
    return (1.0f - ds) * (1.0f - dt) * envTexel(E, si, ti) + ds * (1.0f - dt) * envTexel(E, si + 1, ti) +
           (1.0f - ds) * dt * envTexel(E, si, ti + 1) + ds * dt * envTexel(E, si + 1, ti + 1);
}
__device__ __forceinline__ void dirToUV(float3 d, float *u, float *v) {
    float phi = atan2f(d.y, d.x);
    if (phi < 0.0f) phi += 2.0f * kPi;
    *u = phi * (0.5f * kInvPi);
    *v = acosf(clampf(d.z, -1.0f, 1.0f)) * kInvPi;
}
__device__ __forceinline__ float3 envLe(const DeviceEnv &E, float3 d) {   // Envmap::Le, envmap.cc:130
    float u, v;
    dirToUV(normalize(d), &u, &v);
    return envLookup(E, u, v);
}
// Distribution1D::sample over cdf[0..n] / func[0..n-1] (core/sampling.cc:75)
__device__ __forceinline__ float sample1D(const float *cdf, const float *func, int n, float integral, float u,
                                          float *pdf, int *off) {
    int lo = 0, hi = n;   // largest i in [0, n] with cdf[i] <= u
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&cdf[mid]) <= u) lo = mid;
        else hi = mid - 1;
    }
    const int o = min(lo, n - 1);
    *off = o;
    const float c0 = __ldg(&cdf[o]), c1 = __ldg(&cdf[o + 1]);
    float du = u - c0;
    if (c1 - c0 > 0.0f) du /= (c1 - c0);
    *pdf = integral > 0.0f ? __ldg(&func[o]) / integral : 0.0f;
    return (o + du) / n;
}
__device__ __forceinline__ float envPdf(const DeviceEnv &E, float3 d) {   // Envmap::pdfLi, envmap.cc:81
    float u, v;
    dirToUV(d, &u, &v);
    const float sinTheta = sinf(v * kPi);
    if (sinTheta == 0.0f || E.margIntegral <= 0.0f) return 0.0f;
    const int iu = min(max(static_cast<int>(u * E.w), 0), E.w - 1);
    const int iv = min(max(static_cast<int>(v * E.h), 0), E.h - 1);
    return (__ldg(&E.condFunc[iv * E.w + iu]) / E.margIntegral) / (2.0f * kPi * kPi * sinTheta);
}

// Shape::pdf(Interaction, wi) for an area-light triangle (core/shape.cc:39): intersect
// the light from the offset origin; solid-angle pdf from the hit distance.
__device__ __forceinline__ float lightTriPdf(const LightRecord &L, float3 p, float3 n, float3 wi, float *tHit) {
    const float3 o = offsetOrigin(p, n, wi);
    const float3 e1 = xyz(L.e1), e2 = xyz(L.e2);
    const float3 pv = cross(wi, e2);
    const float det = dot(e1, pv);
    if (det > -kEpsT && det < kEpsT) return 0.0f;
    const float inv = 1.0f / det;
    const float3 tv = o - xyz(L.p0);
    const float u = dot(tv, pv) * inv;
    if (u < 0.0f || u > 1.0f) return 0.0f;
    const float3 qv = cross(tv, e1);
    const float v = dot(wi, qv) * inv;
    if (v < 0.0f || u + v > 1.0f) return 0.0f;
    const float t = dot(e2, qv) * inv;
    if (t <= kEpsT) return 0.0f;
    *tHit = t;
    const float3 hp = o + wi * t;
    const float3 dd = p - hp;
    const float pdf = dot(dd, dd) / (fabsf(dot(xyz(L.n), wi)) * L.p0.w);
    return isinf(pdf) ? 0.0f : pdf;
}

// ---------------------------------------------------------------- kernels
__global__ void k_raygen(PassArgs p) {
    const int sample = p.ctl[0];
    for (int pix = blockIdx.x * blockDim.x + threadIdx.x; pix < p.npix; pix += gridDim.x * blockDim.x) {
        const int y = pix / p.W, x = pix - y * p.W;
        const int fi = y * p.W + (p.W - 1 - x);
        const Rand4 r = rand4(p.seed, static_cast<uint32_t>(fi), static_cast<uint32_t>(sample), 0xFFFFu, 0u);
        const float fx = x + r.a, fy = y + r.b;
        const float *M = p.cam.r2c;
        float c[4];
        for (int i = 0; i < 4; i++) c[i] = M[4 * i + 0] * fx + M[4 * i + 1] * fy + M[4 * i + 3];
        if (c[3] != 1.0f) {
            c[0] /= (c[3] + 1.0e-12f);
            c[1] /= (c[3] + 1.0e-12f);
            c[2] /= (c[3] + 1.0e-12f);
        }
        const float inv = 1.0f / sqrtf(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        const float3 dc = mk(c[0] * inv, c[1] * inv, c[2] * inv);
        const float *W = p.cam.c2w;
        const float3 d = normalize(mk(W[0] * dc.x + W[1] * dc.y + W[2] * dc.z, W[4] * dc.x + W[5] * dc.y + W[6] * dc.z,
                                      W[8] * dc.x + W[9] * dc.y + W[10] * dc.z));
        p.rayO0[pix] = make_float4(W[3], W[7], W[11], __int_as_float(pix));
        p.rayD0[pix] = make_float4(d.x, d.y, d.z, kInfT);
        p.beta[pix] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        float4 f = p.film[fi];
        f.w += 1.0f;
        p.film[fi] = f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) p.counters[0] = p.npix;
}

template <bool STATS>
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
            if (L.found) {
                HitRecord h;
                h.t = L.tmax;
                h.prim = L.hitSlot;
                h.u = L.hu;
                h.v = L.hv;
                p.hits[i] = h;
                cls = __ldg(&p.sv.mats[__ldg(&p.sv.slotShade[L.hitSlot]).x].type);
            } else if (p.sv.hasEnv) {
                // escaped: the environment at the first hit or after a specular bounce
                const int pid = __float_as_int(rO[i].w);
                const float4 bt = p.beta[pid];
                if (b == 0 || bt.w != 0.0f) filmAdd(p.film, filmIndex(p, pid), xyz(bt) * envLe(p.sv.env, L.d));
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
    const int sample = p.ctl[0];
    const SceneView &S = p.sv;
    const int stride = gridDim.x * blockDim.x;
    const int nIter = (n + stride - 1) / stride;
    for (int it = 0; it < nIter; it++) {
        const int j = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
        const bool live = j < n;
        bool cont = false, sh0 = false, sh1 = false;
        float4 c0O, c0D, c0L, c1O, c1D, c1L, cO, cD;
        int pid = 0;
        float3 beta = mk(0, 0, 0);
        bool spec = false;
        if (live) {
            const int i = p.classQ[CLS * p.cap + j];
            const float4 o4 = rO[i], d4 = rD[i];
            const HitRecord h = p.hits[i];
            pid = __float_as_int(o4.w);
            const float4 bt = p.beta[pid];
            beta = xyz(bt);
            spec = bt.w != 0.0f;
            const int fi = filmIndex(p, pid);
            const TriRecord tr = S.tris[h.prim];
            const float3 n = normalize(cross(xyz(tr.v1) - xyz(tr.v0), xyz(tr.v2) - xyz(tr.v0)));
            const int2 sh = __ldg(&S.slotShade[h.prim]);
            const MaterialRecord m = S.mats[sh.x];
            const float3 d = xyz(d4);
            const float3 ps = xyz(o4) + d * h.t;
            // emitted radiance at the first hit or after a specular bounce (path.cc:58-66)
            if ((b == 0 || spec) && sh.y >= 0) {
                const LightRecord &L = S.lights[sh.y];
                if (dot(n, -d) > 0.0f) filmAdd(p.film, fi, beta * xyz(L.L));
            }
            if (b < p.maxDepth) {
                float3 tg, bg;
                onb(n, &tg, &bg);
                const float3 wo = -d;
                const float3 woL = mk(dot(wo, tg), dot(wo, bg), dot(wo, n));
                const Rand4 r0 = rand4(p.seed, static_cast<uint32_t>(fi), static_cast<uint32_t>(sample),
                                       static_cast<uint32_t>(b), 0u);
                const Rand4 r1 = rand4(p.seed, static_cast<uint32_t>(fi), static_cast<uint32_t>(sample),
                                       static_cast<uint32_t>(b), 1u);
                if (CLS != kMatDielectric && S.nLights > 0) {
                    // ---- uniformSampleOneLight + estimateDirectLight (mis.cc:21-136)
                    const int nL = S.nLights;
                    const int li = min(static_cast<int>(r0.a * nL), nL - 1);
                    const bool isEnv = li >= S.nArea;
                    const float3 scale = beta * static_cast<float>(nL);
                    // light sampling
                    float3 wi = mk(0, 0, 0), Li = mk(0, 0, 0), target = mk(0, 0, 0), tn = mk(0, 0, 0);
                    float lightPdf = 0.0f;
                    if (!isEnv) {
                        const LightRecord L = S.lights[li];
                        float u0 = r0.b, u1 = r0.c;
                        if (u0 + u1 >= 1.0f) {
                            u0 = 1.0f - u0;
                            u1 = 1.0f - u1;
                        }
                        target = xyz(L.p0) + xyz(L.e1) * u0 + xyz(L.e2) * u1;
                        tn = xyz(L.n);
                        wi = normalize(target - ps);
                        float tl;
                        lightPdf = lightTriPdf(L, ps, n, wi, &tl);
                        if (dot(tn, -wi) > 0.0f) Li = xyz(L.L);
                    } else {
                        const DeviceEnv &E = S.env;
                        float pv, pu;
                        int vOff, uOff;
                        const float vv = sample1D(E.margCdf, E.margFunc, E.h, E.margIntegral, r0.c, &pv, &vOff);
                        const float uu = sample1D(E.condCdf + static_cast<int64_t>(vOff) * (E.w + 1),
                                                  E.condFunc + static_cast<int64_t>(vOff) * E.w, E.w,
                                                  __ldg(&E.margFunc[vOff]), r0.b, &pu, &uOff);
                        const float mapPdf = pu * pv;
                        if (mapPdf > 0.0f) {
                            float st, ct, sp, cp;
                            sincosf(vv * kPi, &st, &ct);
                            sincosf(uu * 2.0f * kPi, &sp, &cp);
                            wi = mk(st * cp, st * sp, ct);
                            lightPdf = st == 0.0f ? 0.0f : mapPdf / (2.0f * kPi * kPi * st);
                            Li = envLookup(E, uu, vv);
                            target = ps + wi * (2.0f * E.radius);
                        }
                    }
                    if (lightPdf > 0.0f && !isBlack(Li)) {
                        const float3 wiL = mk(dot(wi, tg), dot(wi, bg), dot(wi, n));
                        const float3 f = bsdfF(m, woL, wiL) * fabsf(dot(wi, n));
                        if (!isBlack(f)) {
                            const float bp = bsdfPdf(m, woL, wiL);
                            const float w = powerHeuristic(lightPdf, bp);
                            const float3 c = scale * f * Li * (w / lightPdf);
                            // VisibilityTester::unoccluded via spawnRayTo (interaction.cc:88)
                            const float3 o = offsetOrigin(ps, n, target - ps);
                            const float3 t2 = isEnv ? mk(nextafterf(target.x, -INFINITY), nextafterf(target.y, -INFINITY),
                                                         nextafterf(target.z, -INFINITY))
                                                    : offsetOrigin(target, tn, o - target);
                            const float3 dd = t2 - o;
                            const float len = length(dd);
                            if (len > 0.0f) {
                                sh0 = true;
                                c0O = make_float4(o.x, o.y, o.z, __int_as_float(fi));
                                c0D = make_float4(dd.x / len, dd.y / len, dd.z / len, len);
                                c0L = make_float4(c.x, c.y, c.z, 0.0f);
                            }
                        }
                    }
                    // BSDF sampling with MIS
                    float3 wiL2;
                    float pdf2;
                    int type2;
                    float3 f2 = bsdfSample(m, woL, r0.d, r1.a, &wiL2, &pdf2, &type2);
                    if (!isBlack(f2) && pdf2 > 0.0f) {
                        const float3 wi2 = normalize(tg * wiL2.x + bg * wiL2.y + n * wiL2.z);
                        f2 = f2 * fabsf(dot(wi2, n));
                        float lp = 0.0f, tl = 0.0f;
                        float3 L2 = mk(0, 0, 0);
                        if (!isEnv) {
                            const LightRecord L = S.lights[li];
                            lp = lightTriPdf(L, ps, n, wi2, &tl);
                            if (lp > 0.0f && dot(xyz(L.n), -wi2) > 0.0f) L2 = xyz(L.L);
                        } else {
                            lp = envPdf(S.env, wi2);
                            if (lp > 0.0f) L2 = envLe(S.env, wi2);
                        }
                        if (lp > 0.0f && !isBlack(L2) && !isBlack(f2)) {
                            const float w = powerHeuristic(pdf2, lp);
                            const float3 c = scale * f2 * L2 * (w / pdf2);
                            const float3 o = offsetOrigin(ps, n, wi2);
                            sh1 = true;
                            c1O = make_float4(o.x, o.y, o.z, __int_as_float(fi));
                            c1D = make_float4(wi2.x, wi2.y, wi2.z, isEnv ? kInfT : tl * (1.0f - 1.0e-5f));
                            c1L = make_float4(c.x, c.y, c.z, 0.0f);
                        }
                    }
                }
                // ---- continuation (path.cc:82-95) and Russian roulette (path.cc:117-121)
                float3 wiL;
                float pdf;
                int type;
                const float3 f = bsdfSample(m, woL, r1.b, r1.c, &wiL, &pdf, &type);
                if (!isBlack(f) && pdf > 0.0f) {
                    const float3 wi = normalize(tg * wiL.x + bg * wiL.y + n * wiL.z);
                    beta = beta * f * (fabsf(dot(wi, n)) / pdf);
                    spec = (type & kSpecular) != 0;
                    cont = true;
                    if (b > 3) {
                        const float q = fminf(0.95f, gray(beta));
                        if (r1.d > q) cont = false;
                        else beta = beta / q;
                    }
                    if (cont) {
                        const float3 o = offsetOrigin(ps, n, wi);
                        cO = make_float4(o.x, o.y, o.z, __int_as_float(pid));
                        cD = make_float4(wi.x, wi.y, wi.z, kInfT);
                    }
                }
            }
        }
        const int k = warpAppend(cont, nextCnt);
        if (k >= 0) {
            nO[k] = cO;
            nD[k] = cD;
            p.beta[pid] = make_float4(beta.x, beta.y, beta.z, spec ? 1.0f : 0.0f);
        }
        const int s0 = warpAppend(sh0, shCnt);
        if (s0 >= 0) {
            p.shO[s0] = c0O;
            p.shD[s0] = c0D;
            p.shL[s0] = c0L;
        }
        const int s1 = warpAppend(sh1, shCnt);
        if (s1 >= 0) {
            p.shO[s1] = c1O;
            p.shD[s1] = c1D;
            p.shL[s1] = c1L;
        }
    }
}

template <bool STATS>
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
        if (i >= 0 && !L.found) filmAdd(p.film, __float_as_int(p.shO[i].w), xyz(p.shL[i]));
    };
    tracePersistent<true, STATS>(p.sv.nodes, p.sv.tris, p.sv.nNodes, p.sv.nTris, n, cnt + 6, stack + threadIdx.x,
                                 kTraceBlock, &nodeCount, &triCount, &overflow, fetch, done);
    if (overflow) atomicOr(p.err, 1);
    if (STATS) {
        atomicAdd(&p.visit[2], static_cast<unsigned long long>(nodeCount));
        atomicAdd(&p.visit[3], static_cast<unsigned long long>(triCount));
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
    p.ctl[0] += 1;
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
    int trace, shade, raygen;
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
        k_extend<STATS><<<g.trace, kTraceBlock, 0, cs>>>(a, b);
        done();
        mark(kShadeL);
        k_shade<kMatLambert><<<g.shade, kShadeBlock, 0, cs>>>(a, b);
        done();
        mark(kShadeC);
        k_shade<kMatConductor><<<g.shade, kShadeBlock, 0, cs>>>(a, b);
        done();
        mark(kShadeD);
        k_shade<kMatDielectric><<<g.shade, kShadeBlock, 0, cs>>>(a, b);
        done();
        mark(kShadow);
        k_shadow<STATS><<<g.trace, kTraceBlock, 0, cs>>>(a, b);
        done();
    }
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
int setupPass(Ctx &C, const float *camera, int W, int H, int maxDepth, uint32_t seed, float4 *film, PassArgs *out) {
    RenderQueues &q = C.rq;
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
    return 0;
}
}  // namespace

int renderFrame(Ctx *ctx, const float *camera, int W, int H, int spp, int sampleOffset, int maxDepth, uint32_t seed,
                float4 *film, unsigned long long *statsOut, float *msOut, cudaStream_t stream) {
    Ctx &C = *ctx;
    RenderQueues &q = C.rq;
    const int64_t npix = static_cast<int64_t>(W) * H;
    PassArgs a;
    int rc = setupPass(C, camera, W, H, maxDepth, seed, film, &a);
    if (rc) return rc;

    // (re)capture the pass graph when anything baked into it changes
    uint64_t key[4];
    key[0] = hashBytes(&a, sizeof(a));
    key[1] = static_cast<uint64_t>(W) << 32 | static_cast<uint32_t>(H);
    key[2] = static_cast<uint64_t>(maxDepth) << 32 | seed;
    key[3] = reinterpret_cast<uint64_t>(film);
    if (!q.graph || std::memcmp(key, q.graphKey, sizeof(key)) != 0) {
        if (q.graph) {
            cudaGraphExecDestroy(q.graph);
            q.graph = nullptr;
        }
        const Grids gr = passGrids(C.device, npix);
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
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaError_t e = cudaMemsetAsync(q.stats, 0, 8 * sizeof(unsigned long long), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(q.err, 0, sizeof(int), stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(a.ctl, &sampleOffset, sizeof(int), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaEventRecord(e0, stream);
    for (int s = 0; s < spp && e == cudaSuccess; s++) e = cudaGraphLaunch(q.graph, stream);
    if (e == cudaSuccess) e = cudaEventRecord(e1, stream);
    unsigned long long st[4] = {0, 0, 0, 0};
    int err = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(st, q.stats, sizeof(st), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err, q.err, sizeof(int), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    float ms = 0.0f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cudaFail("spgpu_render", e);
    for (int k = 0; k < 4; k++) statsOut[k] = st[k];
    *msOut = ms;
    if (err) {
        setError("spgpu_render: traversal stack overflow");
        return SPGPU_EKERNEL;
    }
    return 0;
}

int renderProfile(Ctx *ctx, const float *camera, int W, int H, int spp, int sampleOffset, int maxDepth, uint32_t seed,
                  float4 *film, double *kernelMs, long long *launches, unsigned long long *statsOut,
                  unsigned long long *visitOut, cudaStream_t stream) {
    Ctx &C = *ctx;
    RenderQueues &q = C.rq;
    PassArgs a;
    int rc = setupPass(C, camera, W, H, maxDepth, seed, film, &a);
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
