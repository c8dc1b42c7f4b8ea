// common.cuh -- device-side math shared by the BVH, trace and wavefront kernels:
// float3 helpers, the counter-based sampler, the three BSDFs, and the layouts of
// the compressed wide BVH node and the triangle records.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace spgpu {

// ---------------------------------------------------------------------------
// constants shared with the reference (core/common.h:52-55)
// ---------------------------------------------------------------------------
constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.318309886183790671538f;
constexpr float kEpsT = 1.0e-12f;        // triangle t and determinant threshold
constexpr float kInfT = 1.0e32f;         // the reference's INFTY
constexpr float kOffset = 1.0e-3f;       // spawn-ray origin offset (interaction.cc:17)

// ---------------------------------------------------------------------------
// float3
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ float3 mk(float x, float y, float z) { return make_float3(x, y, z); }
__host__ __device__ __forceinline__ float3 operator+(float3 a, float3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ float3 operator-(float3 a, float3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ float3 operator-(float3 a) { return mk(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ float3 operator*(float3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float3 operator*(float s, float3 a) { return mk(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float3 operator*(float3 a, float3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ __forceinline__ float3 operator/(float3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
__host__ __device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ float length(float3 a) { return sqrtf(dot(a, a)); }
__host__ __device__ __forceinline__ float3 normalize(float3 a) { return a * (1.0f / sqrtf(dot(a, a))); }
__host__ __device__ __forceinline__ float3 fminf3(float3 a, float3 b) { return mk(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
__host__ __device__ __forceinline__ float3 fmaxf3(float3 a, float3 b) { return mk(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
__host__ __device__ __forceinline__ float3 xyz(float4 v) { return mk(v.x, v.y, v.z); }
__host__ __device__ __forceinline__ float gray(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
__host__ __device__ __forceinline__ bool isBlack(float3 c) { return c.x == 0.0f && c.y == 0.0f && c.z == 0.0f; }
__host__ __device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }

// ---------------------------------------------------------------------------
// Compressed 8-wide BVH node: 80 bytes = 5 x 16 B, loaded with five 128-bit loads.
// Child boxes are quantised to 8 bits per plane on a per-node grid:
//   lo = p + qlo * 2^(e-127), hi = p + qhi * 2^(e-127)   (per axis)
// meta[k] (one byte per child slot):
//   0                      empty slot
//   0b001_11sss (24 + s)   internal child in slot s; its node index is
//                          child_base + popc(imask & ((1 << s) - 1))
//   0bnnn_ooooo            leaf: triangles tri_base + o ... (n = 1, 3, 7 -> 1..3 triangles)
// Slots are assigned so that a ray with direction-sign octant d visits slot s in
// the order of s ^ (7 - d), i.e. roughly front to back.
// ---------------------------------------------------------------------------
struct alignas(16) WideNode {
    float px, py, pz;
    uint8_t ex, ey, ez, imask;
    uint32_t child_base;
    uint32_t tri_base;
    uint8_t meta[8];
    uint8_t qlo_x[8], qlo_y[8], qlo_z[8];
    uint8_t qhi_x[8], qhi_y[8], qhi_z[8];
};
static_assert(sizeof(WideNode) == 80, "wide node must be 80 bytes");

// Triangle record in leaf order: 3 x float4 = 48 bytes, the input vertices unchanged
// (edges are formed in registers, so an exact FP64 re-evaluation stays possible):
//   v0.xyz + primitive id (int bits in .w), v1.xyz, v2.xyz
struct alignas(16) TriRecord {
    float4 v0;
    float4 v1;
    float4 v2;
};

// Moller-Trumbore of the reference (core/triangle.cc:98) re-evaluated in double for
// one ray / triangle pair, with the direction renormalised in double as the
// reference's Ray constructor does (core/ray.cc:15).  Used for near-grazing hits,
// where the FP32 distance loses relative accuracy in proportion to 1/cos(theta).
__device__ __forceinline__ void refineHitFP64(const TriRecord &tr, float3 o, float3 d, float *t, float *u,
                                              float *v) {
    const double ox = o.x, oy = o.y, oz = o.z;
    const double dn = sqrt(static_cast<double>(d.x) * d.x + static_cast<double>(d.y) * d.y +
                           static_cast<double>(d.z) * d.z);
    const double dx = d.x / dn, dy = d.y / dn, dz = d.z / dn;
    const double ax = tr.v0.x, ay = tr.v0.y, az = tr.v0.z;
    const double e1x = static_cast<double>(tr.v1.x) - ax, e1y = static_cast<double>(tr.v1.y) - ay,
                 e1z = static_cast<double>(tr.v1.z) - az;
    const double e2x = static_cast<double>(tr.v2.x) - ax, e2y = static_cast<double>(tr.v2.y) - ay,
                 e2z = static_cast<double>(tr.v2.z) - az;
    const double px = dy * e2z - dz * e2y, py = dz * e2x - dx * e2z, pz = dx * e2y - dy * e2x;
    const double det = e1x * px + e1y * py + e1z * pz;
    if (det == 0.0) return;
    const double inv = 1.0 / det;
    const double tx = ox - ax, ty = oy - ay, tz = oz - az;
    const double qx = ty * e1z - tz * e1y, qy = tz * e1x - tx * e1z, qz = tx * e1y - ty * e1x;
    *u = static_cast<float>((tx * px + ty * py + tz * pz) * inv);
    *v = static_cast<float>((dx * qx + dy * qy + dz * qz) * inv);
    *t = static_cast<float>((e2x * qx + e2y * qy + e2z * qz) * inv);
}

// Closest-hit record (16 B): t, primitive id (-1 = miss), barycentric u, v.
struct alignas(16) HitRecord {
    float t;
    int prim;
    float u;
    float v;
};

// ---------------------------------------------------------------------------
// Sampler: Philox4x32-10, the counter-based generator of Salmon, Moraes, Dror and
// Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC 2011).  Every sample
// dimension of every (pixel, sample index) has its own counter, so paths are
// reproducible regardless of scheduling.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ void mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
#ifdef __CUDA_ARCH__
    *hi = __umulhi(a, b);
    *lo = a * b;
#else
    const uint64_t p = static_cast<uint64_t>(a) * b;
    *hi = static_cast<uint32_t>(p >> 32);
    *lo = static_cast<uint32_t>(p);
#endif
}

__host__ __device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
    constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    constexpr uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(M0, c.x, &hi0, &lo0);
        mulhilo32(M1, c.z, &hi1, &lo1);
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += W0;
        k.y += W1;
    }
    return c;
}

// uniform in [0, 1) from the top 24 bits
__host__ __device__ __forceinline__ float u01(uint32_t x) { return static_cast<float>(x >> 8) * (1.0f / 16777216.0f); }

struct Rand4 {
    float a, b, c, d;
};
// key = (seed, pixel), counter = (sample index, bounce, stream, 0)
__host__ __device__ __forceinline__ Rand4 rand4(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t bounce,
                                                uint32_t stream) {
    const uint4 r = philox4x32_10(make_uint4(sample, bounce, stream, 0x5350u), make_uint2(seed, pixel));
    return {u01(r.x), u01(r.y), u01(r.z), u01(r.w)};
}

// ---------------------------------------------------------------------------
// orthonormal basis around n: Duff, Burgess, Christensen, Hery, Kensler, Liani and
// Villemin, "Building an Orthonormal Basis, Revisited" (JCGT 2017)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void onb(float3 n, float3 *t, float3 *b) {
    const float s = copysignf(1.0f, n.z);
    const float a = -1.0f / (s + n.z);
    const float c = n.x * n.y * a;
    *t = mk(1.0f + s * n.x * n.x * a, s * c, -s * n.x);
    *b = mk(c, s + n.y * n.y * a, -n.y);
}

// spawn-ray origin offset (core/interaction.cc:16): p + sign * 1e-3 * n, then one
// float ulp further in the direction of the offset on every axis.
__device__ __forceinline__ float3 offsetOrigin(float3 p, float3 n, float3 w) {
    float3 off = n * kOffset;
    if (dot(w, n) < 0.0f) off = -off;
    const float3 po = p + off;
    return mk(off.x > 0.0f ? nextafterf(po.x, INFINITY) : nextafterf(po.x, -INFINITY),
              off.y > 0.0f ? nextafterf(po.y, INFINITY) : nextafterf(po.y, -INFINITY),
              off.z > 0.0f ? nextafterf(po.z, INFINITY) : nextafterf(po.z, -INFINITY));
}

// ---------------------------------------------------------------------------
// BSDFs in the local frame (z = shading normal), following the reference's
// core/bxdf.cc, core/microfacet.cc and core/fresnel.cc in single precision.
// ---------------------------------------------------------------------------
enum : int { kReflection = 1, kTransmission = 2, kDiffuse = 4, kGlossy = 8, kSpecular = 16, kAll = 31 };
enum : int { kMatLambert = 0, kMatConductor = 1, kMatDielectric = 2 };

// material record on the device: 2 x float4
//   Lambert:    a = (R.rgb, 0),          b = 0
//   conductor:  a = (eta.rgb, alpha),    b = (k.rgb, 0)
//   dielectric: a = (0, 0, 0, ior)
struct alignas(16) MaterialRecord {
    float4 a;
    float4 b;
    int type;
    int pad[3];
};

__device__ __forceinline__ float cos2T(float3 w) { return w.z * w.z; }
__device__ __forceinline__ float sin2T(float3 w) { return fmaxf(0.0f, 1.0f - w.z * w.z); }
__device__ __forceinline__ float tan2T(float3 w) { return sin2T(w) / (cos2T(w) + kEpsT); }

// concentric disk, cosine hemisphere (core/sampling.cc:151-179)
__device__ __forceinline__ float3 cosineHemisphere(float u0, float u1) {
    const float ox = 2.0f * u0 - 1.0f, oy = 2.0f * u1 - 1.0f;
    float x = 0.0f, y = 0.0f;
    if (ox != 0.0f || oy != 0.0f) {
        float r, th;
        if (fabsf(ox) > fabsf(oy)) {
            r = ox;
            th = (kPi / 4.0f) * (oy / ox);
        } else {
            r = oy;
            th = kPi / 2.0f - (kPi / 4.0f) * (ox / oy);
        }
        float s, c;
        __sincosf(th, &s, &c);
        x = r * c;
        y = r * s;
    }
    return mk(x, y, sqrtf(fmaxf(0.0f, 1.0f - x * x - y * y)));
}

// FrDielectric (fresnel.cc:65)
__device__ __forceinline__ float frDielectric(float cI, float etaI, float etaT) {
    cI = clampf(cI, -1.0f, 1.0f);
    if (!(cI > 0.0f)) {
        const float t = etaI;
        etaI = etaT;
        etaT = t;
        cI = fabsf(cI);
    }
    const float sI = sqrtf(fmaxf(0.0f, 1.0f - cI * cI));
    const float sT = etaI / etaT * sI;
    if (sT >= 1.0f) return 1.0f;
    const float cT = sqrtf(fmaxf(0.0f, 1.0f - sT * sT));
    const float rpar = (etaT * cI - etaI * cT) / (etaT * cI + etaI * cT);
    const float rperp = (etaI * cI - etaT * cT) / (etaI * cI + etaT * cT);
    return 0.5f * (rpar * rpar + rperp * rperp);
}

// FrConductor with etaI = 1 (fresnel.cc:40), per channel
__device__ __forceinline__ float frConductor1(float cI, float eta, float k) {
    cI = clampf(cI, -1.0f, 1.0f);
    const float c2 = cI * cI, s2 = 1.0f - c2;
    const float eta2 = eta * eta, k2 = k * k;
    const float t0 = eta2 - k2 - s2;
    const float a2b2 = sqrtf(fmaxf(0.0f, t0 * t0 + 4.0f * eta2 * k2));
    const float t1 = a2b2 + c2;
    const float a = sqrtf(fmaxf(0.0f, 0.5f * (a2b2 + t0)));
    const float t2 = 2.0f * cI * a;
    const float rs = (t1 - t2) / (t1 + t2);
    const float t3 = c2 * a2b2 + s2 * s2;
    const float t4 = t2 * s2;
    const float rp = rs * (t3 - t4) / (t3 + t4 + kEpsT);
    return 0.5f * (rp + rs);
}
__device__ __forceinline__ float3 frConductor(float cI, float3 eta, float3 k) {
    return mk(frConductor1(cI, eta.x, k.x), frConductor1(cI, eta.y, k.y), frConductor1(cI, eta.z, k.z));
}

// Trowbridge-Reitz (GGX), isotropic alpha (microfacet.cc:205-270)
__device__ __forceinline__ float ggxD(float3 wh, float a) {
    const float t2 = tan2T(wh);
    if (isinf(t2)) return 0.0f;
    const float c4 = cos2T(wh) * cos2T(wh);
    const float e = t2 / (a * a);
    return 1.0f / (kPi * a * a * c4 * (1.0f + e) * (1.0f + e));
}
__device__ __forceinline__ float ggxLambda(float3 w, float a) {
    const float at = fabsf(sqrtf(sin2T(w)) / (w.z + kEpsT));
    if (isinf(at)) return 0.0f;
    const float ai = a * at;
    return (-1.0f + sqrtf(1.0f + ai * ai)) * 0.5f;
}
__device__ __forceinline__ float ggxG1(float3 w, float3 wh, float a) {
    if (w.z * dot(w, wh) <= 0.0f) return 0.0f;
    return 1.0f / (1.0f + ggxLambda(w, a));
}
__device__ __forceinline__ float ggxG(float3 wo, float3 wi, float3 wh, float a) {
    if (wi.z * dot(wi, wh) <= 0.0f) return 0.0f;
    if (wo.z * dot(wo, wh) <= 0.0f) return 0.0f;
    return 1.0f / (1.0f + ggxLambda(wo, a) + ggxLambda(wi, a));
}
__device__ __forceinline__ float ggxPdf(float3 wo, float3 wh, float a) {   // visible normals
    return ggxD(wh, a) * ggxG1(wo, wh, a) * fabsf(dot(wo, wh)) / fabsf(wo.z);
}
// visible-normal sampling, Heitz and d'Eon, "Importance Sampling Microfacet-Based
// BSDFs using the Distribution of Visible Normals" (EGSR 2014): stretch, sample the
// slopes of the unit-roughness distribution, rotate, unstretch.
__device__ __forceinline__ void ggxSample11(float cosTheta, float u0, float u1, float *sx, float *sy) {
    if (cosTheta > 0.9999f) {
        const float r = sqrtf(u0 / (1.0f - u0));
        float s, c;
        __sincosf(2.0f * kPi * u1, &s, &c);
        *sx = r * c;
        *sy = r * s;
        return;
    }
    const float sinTheta = sqrtf(fmaxf(0.0f, 1.0f - cosTheta * cosTheta));
    const float tanTheta = sinTheta / cosTheta;
    const float a = 1.0f / tanTheta;
    const float G1 = 2.0f / (1.0f + sqrtf(1.0f + 1.0f / (a * a)));
    const float A = 2.0f * u0 / G1 - 1.0f;
    float tmp = 1.0f / (A * A - 1.0f);
    if (tmp > 1.0e10f) tmp = 1.0e10f;
    const float B = tanTheta;
    const float D = sqrtf(fmaxf(0.0f, B * B * tmp * tmp - (A * A - B * B) * tmp));
    const float x1 = B * tmp - D, x2 = B * tmp + D;
    *sx = (A < 0.0f || x2 > 1.0f / tanTheta) ? x1 : x2;
    float S, U;
    if (u1 > 0.5f) {
        S = 1.0f;
        U = 2.0f * (u1 - 0.5f);
    } else {
        S = -1.0f;
        U = 2.0f * (0.5f - u1);
    }
    const float z = (U * (U * (U * 0.27385f - 0.73369f) + 0.46341f)) /
                    (U * (U * (U * 0.093073f + 0.309420f) - 1.0f) + 0.597999f);
    *sy = S * z * sqrtf(1.0f + (*sx) * (*sx));
}
__device__ __forceinline__ float3 ggxSampleWh(float3 wo, float a, float u0, float u1) {
    const bool flip = wo.z < 0.0f;
    const float3 w = flip ? -wo : wo;
    const float3 ws = normalize(mk(a * w.x, a * w.y, w.z));
    float sx, sy;
    ggxSample11(ws.z, u0, u1, &sx, &sy);
    const float st = sqrtf(fmaxf(0.0f, 1.0f - ws.z * ws.z));
    const float cp = st == 0.0f ? 1.0f : clampf(ws.x / st, -1.0f, 1.0f);
    const float sp = st == 0.0f ? 0.0f : clampf(ws.y / st, -1.0f, 1.0f);
    const float tmp = cp * sx - sp * sy;
    sy = sp * sx + cp * sy;
    sx = tmp * a;
    sy = sy * a;
    float3 wh = normalize(mk(-sx, -sy, 1.0f));
    return flip ? -wh : wh;
}

__device__ __forceinline__ bool refract(float3 wi, float3 n, float eta, float3 *wt) {
    const float cI = dot(n, wi);
    const float s2I = fmaxf(0.0f, 1.0f - cI * cI);
    const float s2T = eta * eta * s2I;
    if (s2T >= 1.0f) return false;
    const float cT = sqrtf(1.0f - s2T);
    *wt = eta * (-wi) + (eta * cI - cT) * n;
    return true;
}

// f(wo, wi) for the non-specular materials (BSDF::f restricted to one lobe)
__device__ __forceinline__ float3 bsdfF(const MaterialRecord &m, float3 wo, float3 wi) {
    if (m.type == kMatLambert) {
        if (wo.z * wi.z <= 0.0f) return mk(0, 0, 0);
        return xyz(m.a) * kInvPi;
    }
    if (m.type == kMatConductor) {
        if (wo.z * wi.z <= 0.0f) return mk(0, 0, 0);
        const float cO = fabsf(wo.z), cI = fabsf(wi.z);
        if (cI == 0.0f || cO == 0.0f) return mk(0, 0, 0);
        float3 wh = wi + wo;
        if (wh.x == 0.0f && wh.y == 0.0f && wh.z == 0.0f) return mk(0, 0, 0);
        wh = normalize(wh);
        const float a = m.a.w;
        const float3 F = frConductor(fabsf(dot(wi, wh)), xyz(m.a), xyz(m.b));
        return F * (ggxD(wh, a) * ggxG(wo, wi, wh, a) / (4.0f * cI * cO));
    }
    return mk(0, 0, 0);   // specular: zero for any finite pair
}
__device__ __forceinline__ float bsdfPdf(const MaterialRecord &m, float3 wo, float3 wi) {
    if (wo.z * wi.z <= 0.0f) return 0.0f;
    if (m.type == kMatLambert) return fabsf(wi.z) * kInvPi;
    if (m.type == kMatConductor) {
        const float3 wh = normalize(wo + wi);
        return ggxPdf(wo, wh, m.a.w) / (4.0f * dot(wo, wh));
    }
    return 0.0f;
}
// BSDF::sample for one lobe; returns f, sets wi, pdf and the sampled type bits
__device__ __forceinline__ float3 bsdfSample(const MaterialRecord &m, float3 wo, float u0, float u1, float3 *wi,
                                             float *pdf, int *type) {
    *pdf = 0.0f;
    *type = 0;
    if (wo.z == 0.0f) return mk(0, 0, 0);
    const float ur0 = fminf(u0, 1.0f - 6.0e-8f);
    if (m.type == kMatLambert) {
        float3 w = cosineHemisphere(ur0, u1);
        if (wo.z < 0.0f) w.z = -w.z;
        *wi = w;
        *pdf = bsdfPdf(m, wo, w);
        *type = kReflection | kDiffuse;
        return bsdfF(m, wo, w);
    }
    if (m.type == kMatConductor) {
        const float3 wh = ggxSampleWh(wo, m.a.w, ur0, u1);
        const float3 w = -wo + wh * (2.0f * dot(wh, wo));
        if (wo.z * w.z <= 0.0f) return mk(0, 0, 0);
        *wi = w;
        *pdf = ggxPdf(wo, wh, m.a.w) / (4.0f * dot(wo, wh));
        *type = kReflection | kGlossy;
        return bsdfF(m, wo, w);
    }
    // smooth dielectric (FresnelSpecular::sample, bxdf.cc:198)
    const float ior = m.a.w;
    const float F = frDielectric(wo.z, 1.0f, ior);
    if (ur0 < F) {
        *wi = mk(-wo.x, -wo.y, wo.z);
        *pdf = F;
        *type = kSpecular | kReflection;
        return mk(1, 1, 1) * (F / fabsf(wo.z));
    }
    const bool entering = wo.z > 0.0f;
    const float eI = entering ? 1.0f : ior, eT = entering ? ior : 1.0f;
    float3 w;
    if (!refract(wo, mk(0.0f, 0.0f, entering ? 1.0f : -1.0f), eI / eT, &w)) return mk(0, 0, 0);
    *wi = w;
    *pdf = 1.0f - F;
    *type = kSpecular | kTransmission;
    const float ft = (1.0f - F) * ((eI * eI) / (eT * eT));
    return mk(ft, ft, ft) / fabsf(w.z);
}

__device__ __forceinline__ float powerHeuristic(float f, float g) { return (f * f) / (f * f + g * g); }

}  // namespace spgpu
