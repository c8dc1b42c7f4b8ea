// guided_shade.cuh -- shading of a Lambert hit with the learned guiding proposal,
// shared by the guided megakernel (collection passes) and the guided wavefront.
// This part has no counterpart in the reference renderer.
#pragma once

#include "guide.cuh"
#include "shade.cuh"

namespace spgpu {

// one-sample MIS proposal: the BSDF with probability alpha, else the vMF mixture
struct MixProposal {
    const Mixture *M;
    float alpha;
    __device__ float pdf(const MaterialRecord &m, float3 woL, float3 wiL, float3 wiW) const {
        const float pb = bsdfPdf(m, woL, wiL);
        return M ? alpha * pb + (1.0f - alpha) * mixturePdf(*M, wiW) : pb;
    }
    // returns f (times nothing), world direction, pdf; false if the sample is invalid
    __device__ bool sample(const MaterialRecord &m, float3 woL, float3 tg, float3 bg, float3 n, float uSel,
                           float uLobe, float u1, float u2, float3 *wiW, float3 *f, float *pdf) const {
        float3 wiL;
        if (!M || uSel < alpha) {
            float pb;
            int type;
            const float3 fb = bsdfSample(m, woL, u1, u2, 0.0f, &wiL, &pb, &type);   // Lambert only
            if (isBlack(fb) || pb <= 0.0f) return false;
            *wiW = normalize(tg * wiL.x + bg * wiL.y + n * wiL.z);
        } else {
            *wiW = mixtureSample(*M, uLobe, u1, u2);
            wiL = mk(dot(*wiW, tg), dot(*wiW, bg), dot(*wiW, n));
        }
        *f = bsdfF(m, woL, wiL);
        *pdf = this->pdf(m, woL, wiL, *wiW);
        return *pdf > 0.0f;
    }
};

// hit point of a ray, written once for every kernel that needs it (the network's
// inputs must be the same wherever they are computed)
__device__ __forceinline__ float3 hitPoint(float3 o, float3 d, float t) {
    return mk(__fmaf_rn(d.x, t, o.x), __fmaf_rn(d.y, t, o.y), __fmaf_rn(d.z, t, o.z));
}

// geometric normal of a triangle as the network sees it (unflipped)
__device__ __forceinline__ float3 triNormal(const TriRecord &tr) {
    return normalize(cross(xyz(tr.v1) - xyz(tr.v0), xyz(tr.v2) - xyz(tr.v0)));
}

// A Lambert hit at ps (geometric normal n, material m, light lightOf or -1) reached by
// direction d with throughput beta: the wavefront's shadeHit for a Lambert hit (one-light
// next-event estimation with both MIS strategies, BSDF continuation, Russian roulette
// after bounce 3), with the BSDF strategy replaced by the proposal alpha * BSDF +
// (1 - alpha) * mix everywhere, MIS weights included.  Sampler streams 0-2 of
// (seed, fi, sample, b); shadow-ray origins carry the film pixel fi in w, as shadeHit's
// do.  On a continuation, *fcOut and *pdfOut receive f cos and the proposal's pdf of
// the sampled direction.
__device__ __forceinline__ void shadeGuidedLambert(const SceneView &S, float3 ps, float3 n, const MaterialRecord &m,
                                                   int lightOf, float3 d, float3 beta, bool spec, int b,
                                                   const Mixture &mix, float alpha, uint32_t seed, uint32_t fi,
                                                   uint32_t sample, ShadeResult &R, float3 *fcOut, float *pdfOut) {
    R.emit = mk(0, 0, 0);
    R.cont = R.sh0 = R.sh1 = false;
    if ((b == 0 || spec) && lightOf >= 0 && dot(n, -d) > 0.0f) R.emit = beta * xyz(S.lights[lightOf].L);
    MixProposal P{&mix, alpha};
    float3 tg, bg;
    onb(n, &tg, &bg);
    const float3 wo = -d;
    const float3 woL = mk(dot(wo, tg), dot(wo, bg), dot(wo, n));
    const Rand4 r0 = rand4(seed, fi, sample, static_cast<uint32_t>(b), 0u);
    const Rand4 r1 = rand4(seed, fi, sample, static_cast<uint32_t>(b), 1u);
    const Rand4 r2 = rand4(seed, fi, sample, static_cast<uint32_t>(b), 2u);
    if (S.nLights > 0) {
        const int nL = S.nLights;
        const int li = min(static_cast<int>(r0.a * nL), nL - 1);
        const bool isEnv = li >= S.nArea;
        const float3 scale = beta * static_cast<float>(nL);
        float3 wi = mk(0, 0, 0), Li = mk(0, 0, 0), target = mk(0, 0, 0), tn = mk(0, 0, 0);
        float lightPdf = 0.0f;
        if (!isEnv) {
            const LightRecord Lr = S.lights[S.lightBase + li];
            float u0 = r0.b, u1 = r0.c;
            if (u0 + u1 >= 1.0f) {
                u0 = 1.0f - u0;
                u1 = 1.0f - u1;
            }
            target = xyz(Lr.p0) + xyz(Lr.e1) * u0 + xyz(Lr.e2) * u1;
            tn = xyz(Lr.n);
            wi = normalize(target - ps);
            float tl;
            lightPdf = lightTriPdf(Lr, ps, n, wi, &tl);
            if (dot(tn, -wi) > 0.0f) Li = xyz(Lr.L);
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
                // the hardware's sine and cosine: direction and pdf take the same values
                float st, ct, sp, cp;
                __sincosf(vv * kPi, &st, &ct);
                __sincosf(uu * 2.0f * kPi, &sp, &cp);
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
                const float w = powerHeuristic(lightPdf, P.pdf(m, woL, wiL, wi));
                const float3 c = scale * f * Li * (w / lightPdf);
                const float3 oo = offsetOrigin(ps, n, target - ps);
                const float3 t2 = isEnv ? mk(nextafterf(target.x, -INFINITY),
                                             nextafterf(target.y, -INFINITY),
                                             nextafterf(target.z, -INFINITY))
                                        : offsetOrigin(target, tn, oo - target);
                const float3 dd = t2 - oo;
                const float len = length(dd);
                if (len > 0.0f) {
                    R.sh0 = true;
                    R.s0O = make_float4(oo.x, oo.y, oo.z, __int_as_float(static_cast<int>(fi)));
                    R.s0D = make_float4(dd.x / len, dd.y / len, dd.z / len, len);
                    R.s0L = make_float4(c.x, c.y, c.z, 0.0f);
                }
            }
        }
        // the mixture strategy of MIS
        float3 wi2, f2;
        float pdf2;
        if (P.sample(m, woL, tg, bg, n, r2.a, r2.b, r0.d, r1.a, &wi2, &f2, &pdf2) && !isBlack(f2)) {
            f2 = f2 * fabsf(dot(wi2, n));
            float lp = 0.0f, tl = 0.0f;
            float3 L2 = mk(0, 0, 0);
            if (!isEnv) {
                const LightRecord Lr = S.lights[S.lightBase + li];
                lp = lightTriPdf(Lr, ps, n, wi2, &tl);
                if (lp > 0.0f && dot(xyz(Lr.n), -wi2) > 0.0f) L2 = xyz(Lr.L);
            } else {
                lp = envPdf(S.env, wi2);
                if (lp > 0.0f) L2 = envLe(S.env, wi2);
            }
            if (lp > 0.0f && !isBlack(L2)) {
                const float w = powerHeuristic(pdf2, lp);
                const float3 c = scale * f2 * L2 * (w / pdf2);
                const float3 oo = offsetOrigin(ps, n, wi2);
                R.sh1 = true;
                R.s1O = make_float4(oo.x, oo.y, oo.z, __int_as_float(static_cast<int>(fi)));
                R.s1D = make_float4(wi2.x, wi2.y, wi2.z, isEnv ? kInfT : tl * (1.0f - 1.0e-5f));
                R.s1L = make_float4(c.x, c.y, c.z, 0.0f);
            }
        }
    }
    // continuation from the mixture, Russian roulette
    float3 wi, f;
    float pdf;
    R.beta = beta;
    R.spec = false;
    if (P.sample(m, woL, tg, bg, n, r2.c, r2.d, r1.b, r1.c, &wi, &f, &pdf) && !isBlack(f)) {
        const float3 fc = f * fabsf(dot(wi, n));
        *fcOut = fc;
        *pdfOut = pdf;
        R.beta = beta * fc * (1.0f / pdf);
        R.cont = true;
        if (b > 3) {
            const float q = fminf(0.95f, gray(R.beta));
            if (r1.d > q) R.cont = false;
            else R.beta = R.beta / q;
        }
        if (R.cont) {
            const float3 oo = offsetOrigin(ps, n, wi);
            R.cO = make_float4(oo.x, oo.y, oo.z, 0.0f);
            R.cD = make_float4(wi.x, wi.y, wi.z, kInfT);
        }
    }
}

}  // namespace spgpu
