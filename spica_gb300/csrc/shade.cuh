// shade.cuh -- the per-hit part of the path integrator, shared by the wavefront
// shade kernels and the batched persistent renderer: emission (path.cc:58-66),
// uniformSampleOneLight + estimateDirectLight with both MIS strategies
// (core/mis.cc:21-136), BSDF sampling of the continuation (path.cc:82-95) and Russian
// roulette (path.cc:117-121); plus the environment-map and area-light helpers.
#pragma once

#include "ctx.cuh"

namespace spgpu {

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
// Distribution1D::sample over cdf[0..n] / func[0..n-1] (core/sampling.cc:75): the
// interval i of the largest cdf[i] <= u, the offset within it, and the pdf
// func[i] / integral.  The search is
// narrowed by a guide table (the cutpoint method of Chen and Asau, 1974): guide[k] is
// the largest i with cdf[i] <= k / n, and for k = floor(u n)
// computed in float, (k - 1) / n < u < (k + 2) / n, so [guide[k - 1], guide[k + 2]] holds
// the answer.  The same comparisons on that range give the full search's result in two
// or three steps instead of log2(n).
__device__ __forceinline__ float sample1DGuided(const float *cdf, const int *guide, const float *func, int n,
                                                float integral, float u, float *pdf, int *off) {
    const int k = min(max(static_cast<int>(u * n), 0), n);
    int lo = __ldg(&guide[max(k - 1, 0)]), hi = __ldg(&guide[min(k + 2, n)]);
    while (lo < hi) {   // largest i in [lo, hi] with cdf[i] <= u
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

// PerspectiveCamera::spawnRay (cameras/perspective.cc:53) for raster pixel (x, y) and
// film sample (u0, u1), with the raster->camera and camera->world matrices of the
// reference camera (pinhole: the lens sample is unused).
__device__ __forceinline__ void spawnCameraRay(const CameraView &cam, int x, int y, float u0, float u1, float3 *o,
                                               float3 *d) {
    const float fx = x + u0, fy = y + u1;
    const float *M = cam.r2c;
    float c[4];
    for (int i = 0; i < 4; i++) c[i] = M[4 * i + 0] * fx + M[4 * i + 1] * fy + M[4 * i + 3];
    if (c[3] != 1.0f) {
        c[0] /= (c[3] + 1.0e-12f);
        c[1] /= (c[3] + 1.0e-12f);
        c[2] /= (c[3] + 1.0e-12f);
    }
    const float inv = 1.0f / sqrtf(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    const float3 dc = mk(c[0] * inv, c[1] * inv, c[2] * inv);
    const float *W = cam.c2w;
    *d = normalize(mk(W[0] * dc.x + W[1] * dc.y + W[2] * dc.z, W[4] * dc.x + W[5] * dc.y + W[6] * dc.z,
                      W[8] * dc.x + W[9] * dc.y + W[10] * dc.z));
    *o = mk(W[3], W[7], W[11]);
}

// What one bounce produces.  Shadow entries: origin (w = film index bits), direction
// (w = tmax), contribution.  The continuation ray's origin has w = 0.
struct ShadeResult {
    float3 emit;
    bool cont, spec;
    float3 beta;
    float4 cO, cD;
    bool sh0, sh1;
    float4 s0O, s0D, s0L, s1O, s1D, s1L;
};

// Shade the hit h of ray (o, d) for a path with throughput beta at bounce b.
// pixelKey / sample select the counter-based random streams; filmIdx is stored in the
// shadow entries.  S.lights[S.lightBase + k] are the area lights of this scene.
// direct = true is DirectLightingIntegrator's estimator (no continuation is used):
// light sampling at every material, since its BSDF::f matches any BxDF sharing a type
// bit with the non-specular set (bsdf.cc:49-60); the path integrator light-samples only
// materials with a non-specular BxDF (path.cc:77).
__device__ __forceinline__ void shadeHit(const SceneView &S, const HitRecord &h, float3 o, float3 d, float3 beta,
                                         bool spec, int b, int maxDepth, uint32_t seed, uint32_t pixelKey,
                                         uint32_t sample, int filmIdx, ShadeResult &R, bool direct = false) {
    R.emit = mk(0, 0, 0);
    R.cont = false;
    R.sh0 = R.sh1 = false;
    const TriRecord tr = S.tris[h.prim];
    const float3 n = normalize(cross(xyz(tr.v1) - xyz(tr.v0), xyz(tr.v2) - xyz(tr.v0)));
    const int2 sh = __ldg(&S.slotShade[h.prim]);
    const MaterialRecord m = S.mats[sh.x];
    const float3 ps = o + d * h.t;
    // emitted radiance at the first hit or after a specular bounce (path.cc:58-66)
    if ((b == 0 || spec) && sh.y >= 0) {
        const LightRecord &L = S.lights[sh.y];
        if (dot(n, -d) > 0.0f) R.emit = beta * xyz(L.L);
    }
    if (b < maxDepth) {
        float3 tg, bg;
        onb(n, &tg, &bg);
        const float3 wo = -d;
        const float3 woL = mk(dot(wo, tg), dot(wo, bg), dot(wo, n));
        const Rand4 r0 = rand4(seed, pixelKey, sample,
                               static_cast<uint32_t>(b), 0u);
        const Rand4 r1 = rand4(seed, pixelKey, sample,
                               static_cast<uint32_t>(b), 1u);
        // the draws the reference takes from its BxDFs' hidden generator
        const bool hidden = m.type == kMatRoughDielectric || m.type == kMatPlastic;
        const Rand4 r3 = hidden ? rand4(seed, pixelKey, sample, static_cast<uint32_t>(b), 3u) : Rand4{0, 0, 0, 0};
        // materials with a non-specular BxDF (numComponents(All & ~Specular) > 0)
        const bool nonSpecular = m.type == kMatLambert || m.type == kMatConductor || m.type == kMatRoughDielectric;
        if ((nonSpecular || direct) && S.nLights > 0) {
            // ---- uniformSampleOneLight + estimateDirectLight (mis.cc:21-136)
            const int nL = S.nLights;
            const int li = min(static_cast<int>(r0.a * nL), nL - 1);
            const bool isEnv = li >= S.nArea;
            const float3 scale = beta * static_cast<float>(nL);
            // light sampling
            float3 wi = mk(0, 0, 0), Li = mk(0, 0, 0), target = mk(0, 0, 0), tn = mk(0, 0, 0);
            float lightPdf = 0.0f;
            if (!isEnv) {
                const LightRecord L = S.lights[S.lightBase + li];
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
                const float vv = sample1DGuided(E.margCdf, E.margGuide, E.margFunc, E.h, E.margIntegral, r0.c, &pv, &vOff);
                const float uu = sample1DGuided(E.condCdf + static_cast<int64_t>(vOff) * (E.w + 1),
                                          E.condGuide + static_cast<int64_t>(vOff) * (E.w + 1),
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
                    const float bp = m.type == kMatDielectric ? bsdfPdfDielectricCone(m, woL, wiL)
                                                              : bsdfPdf(m, woL, wiL);
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
                        R.sh0 = true;
                        R.s0O = make_float4(o.x, o.y, o.z, __int_as_float(filmIdx));
                        R.s0D = make_float4(dd.x / len, dd.y / len, dd.z / len, len);
                        R.s0L = make_float4(c.x, c.y, c.z, 0.0f);
                    }
                }
            }
            // BSDF sampling with MIS (only BxDFs of the non-specular set can be sampled)
            float3 wiL2;
            float pdf2 = 0.0f;
            int type2;
            float3 f2 = mk(0, 0, 0);
            if (nonSpecular) f2 = bsdfSample(m, woL, r0.d, r1.a, r3.a, &wiL2, &pdf2, &type2);
            if (!isBlack(f2) && pdf2 > 0.0f) {
                const float3 wi2 = normalize(tg * wiL2.x + bg * wiL2.y + n * wiL2.z);
                f2 = f2 * fabsf(dot(wi2, n));
                float lp = 0.0f, tl = 0.0f;
                float3 L2 = mk(0, 0, 0);
                if (!isEnv) {
                    const LightRecord L = S.lights[S.lightBase + li];
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
                    R.sh1 = true;
                    R.s1O = make_float4(o.x, o.y, o.z, __int_as_float(filmIdx));
                    R.s1D = make_float4(wi2.x, wi2.y, wi2.z, isEnv ? kInfT : tl * (1.0f - 1.0e-5f));
                    R.s1L = make_float4(c.x, c.y, c.z, 0.0f);
                }
            }
        }
        // ---- continuation (path.cc:82-95) and Russian roulette (path.cc:117-121)
        float3 wiL;
        float pdf;
        int type;
        const float3 f = bsdfSample(m, woL, r1.b, r1.c, r3.b, &wiL, &pdf, &type);
        if (!isBlack(f) && pdf > 0.0f) {
            const float3 wi = normalize(tg * wiL.x + bg * wiL.y + n * wiL.z);
            beta = beta * f * (fabsf(dot(wi, n)) / pdf);
            spec = (type & kSpecular) != 0;
            R.cont = true;
            if (b > 3) {
                const float q = fminf(0.95f, gray(beta));
                if (r1.d > q) R.cont = false;
                else beta = beta / q;
            }
            if (R.cont) {
                const float3 o = offsetOrigin(ps, n, wi);
                R.cO = make_float4(o.x, o.y, o.z, 0.0f);
                R.cD = make_float4(wi.x, wi.y, wi.z, kInfT);
            }
        }
    }
    R.beta = beta;
    R.spec = spec;
}

}  // namespace spgpu
