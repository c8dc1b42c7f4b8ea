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
enum : int { kMatLambert = 0, kMatConductor = 1, kMatDielectric = 2, kMatRoughDielectric = 3, kMatPlastic = 4 };

// material record on the device: 2 x float4
//   Lambert:          a = (R.rgb, 0),                       b = 0
//   conductor:        a = (eta.rgb, alpha),                 b = (k.rgb, 0)
//   dielectric:       a = (0, 0, 0, ior)
//   rough dielectric: a = (alpha, ior, 0 Beckmann / 1 GGX, 0)
//   plastic:          a = (Kd.rgb, ior),                    b = (Ks.rgb, specular sampling weight)
struct alignas(16) MaterialRecord {
    float4 a;
    float4 b;
    int type;
    int pad[3];
};

__device__ __forceinline__ float cos2T(float3 w) { return w.z * w.z; }
// sin^2 of a unit vector from its x and y (the reference's 1 - cos^2 in double): in
// float32, 1 - z^2 keeps few digits near the normal, where sharp lobes are evaluated
__device__ __forceinline__ float sin2T(float3 w) { return fminf(1.0f, w.x * w.x + w.y * w.y); }
__device__ __forceinline__ float tan2T(float3 w) { return sin2T(w) / (cos2T(w) + kEpsT); }

// concentric disk, cosine hemisphere (core/sampling.cc:151-179)
__device__ __forceinline__ float3 cosineHemisphere(float u0, float u1) {
    const float ox = 2.0f * u0 - 1.0f, oy = 2.0f * u1 - 1.0f;
    float x = 0.0f, y = 0.0f, r = 0.0f;
    if (ox != 0.0f || oy != 0.0f) {
        float th;
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
    // z = sqrt(1 - x^2 - y^2) with x^2 + y^2 = r^2, as (1 - |r|)(1 + |r|): grazing
    // samples keep their digits
    const float ar = fabsf(r);
    return mk(x, y, sqrtf(fmaxf(0.0f, (1.0f - ar) * (1.0f + ar))));
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
// visible-normal sampling, Heitz and d'Eon, "Importance Sampling Microfacet-Based
// BSDFs using the Distribution of Visible Normals" (EGSR 2014): stretch, sample the
// slopes of the unit-roughness distribution, rotate, unstretch.
// sinTheta is passed in, computed from the direction's x and y: 1 - cos^2 would lose
// most of its float32 digits near normal incidence.
__device__ __forceinline__ void ggxSample11(float cosTheta, float sinTheta, float u0, float u1, float *sx,
                                           float *sy) {
    if (cosTheta > 0.9999f) {
        const float r = sqrtf(u0 / (1.0f - u0));
        float s, c;
        __sincosf(2.0f * kPi * u1, &s, &c);
        *sx = r * c;
        *sy = r * s;
        return;
    }
    const float tanTheta = sinTheta / cosTheta;
    const float a = 1.0f / tanTheta;
    const float G1 = 2.0f / (1.0f + sqrtf(1.0f + 1.0f / (a * a)));
    const float Ap1 = 2.0f * u0 / G1;   // A + 1, so that A^2 - 1 = (A + 1)(A - 1) keeps its digits
    const float A = Ap1 - 1.0f;
    float tmp = 1.0f / (Ap1 * (Ap1 - 2.0f));
    if (tmp > 1.0e10f) tmp = 1.0e10f;
    const float B = tanTheta;
    const float D = sqrtf(fmaxf(0.0f, B * B * tmp * tmp - (A * A - B * B) * tmp));
    // the roots B tmp -+ D: the one of larger magnitude directly, the other from their
    // product (A^2 - B^2) tmp, so that neither is a difference of near-equal terms
    float x1, x2;
    if (B * tmp < 0.0f) {
        x1 = B * tmp - D;
        x2 = x1 != 0.0f ? (A * A - B * B) * tmp / x1 : B * tmp + D;
    } else {
        x2 = B * tmp + D;
        x1 = x2 != 0.0f ? (A * A - B * B) * tmp / x2 : B * tmp - D;
    }
    *sx = (A < 0.0f || x2 > 1.0f / tanTheta) ? x1 : x2;
    float S, U;
    if (u1 > 0.5f) {
        S = 1.0f;
        U = 2.0f * (u1 - 0.5f);
    } else {
        S = -1.0f;
        U = 2.0f * (0.5f - u1);
    }
    // the rational fit's numerator and denominator both nearly vanish as U -> 1, so they
    // are evaluated in double (a few FP64 operations per sample)
    const double Ud = U;
    const float z = static_cast<float>((Ud * (Ud * (Ud * 0.27385 - 0.73369) + 0.46341)) /
                                       (Ud * (Ud * (Ud * 0.093073 + 0.309420) - 1.0) + 0.597999));
    *sy = S * z * sqrtf(1.0f + (*sx) * (*sx));
}

// The reference's own erfinv and erf (core/math.h:14-67): Giles' single-precision
// polynomial and Abramowitz & Stegun 7.1.26, used by its Beckmann sampler; the same
// approximations here, so that the sampled distribution is the reference's.
// Giles' polynomial given w = -log((1 - x)(1 + x)) and x
__device__ __forceinline__ float gilesErfinv(float w, float x) {
    float p;
    if (w < 5.0f) {
        w = w - 2.5f;
        p = 2.81022636e-08f;
        p = 3.43273939e-07f + p * w;
        p = -3.5233877e-06f + p * w;
        p = -4.39150654e-06f + p * w;
        p = 0.00021858087f + p * w;
        p = -0.00125372503f + p * w;
        p = -0.00417768164f + p * w;
        p = 0.246640727f + p * w;
        p = 1.50140941f + p * w;
    } else {
        w = sqrtf(w) - 3.0f;
        p = -0.000200214257f;
        p = 0.000100950558f + p * w;
        p = 0.00134934322f + p * w;
        p = -0.00367342844f + p * w;
        p = 0.00573950773f + p * w;
        p = -0.0076224613f + p * w;
        p = 0.00943887047f + p * w;
        p = 1.00167406f + p * w;
        p = 2.83297682f + p * w;
    }
    return p * x;
}
// the reference's erfinv(x) (x clamped to +-0.99999) evaluated as erfinv(q - 1) for q in
// [0, 2] from q itself: (1 - x)(1 + x) = (2 - q) q keeps its digits for x near -1, where
// 1 + x would have lost them
__device__ __forceinline__ float refErfinvq(float q) {
    q = clampf(q, 1.0f - 0.99999f, 1.0f + 0.99999f);
    return gilesErfinv(-logf((2.0f - q) * q), q - 1.0f);
}
__device__ __forceinline__ float refErff(float x) {
    const float a1 = 0.254829592f, a2 = -0.284496736f, a3 = 1.421413741f, a4 = -1.453152027f, a5 = 1.061405429f,
                p = 0.3275911f;
    const float sgn = x < 0.0f ? -1.0f : 1.0f;
    x = fabsf(x);
    const float t = 1.0f / (1.0f + p * x);
    const float y = 1.0f - (((((a5 * t + a4) * t) + a3) * t + a2) * t + a1) * t * expf(-x * x);
    return sgn * y;
}

// Beckmann, isotropic alpha, visible-normal sampling (microfacet.cc:79-150, 273-356)
__device__ __forceinline__ float beckD(float3 wh, float a) {
    const float t2 = tan2T(wh);
    if (isinf(t2)) return 0.0f;
    const float c4 = cos2T(wh) * cos2T(wh);
    return expf(-t2 / (a * a)) / (kPi * a * a * c4);
}
__device__ __forceinline__ float beckLambda(float3 w, float a) {
    const float at = fabsf(sqrtf(sin2T(w)) / (w.z + kEpsT));
    if (isinf(at)) return 0.0f;
    const float x = 1.0f / (a * at);
    if (x >= 1.6f) return 0.0f;
    return (1.0f - 1.259f * x + 0.396f * x * x) / (3.535f * x + 2.181f * x * x);
}
// slopes of the unit-roughness distribution seen from cosThetaI: Jakob's inversion of
// the slope CDF by bisection / Newton steps (at most 16)
__device__ __forceinline__ void beckSample11(float cosThetaI, float sinThetaI, float U1, float U2, float *sx,
                                            float *sy) {
    if (cosThetaI > 0.9999f) {
        const float r = sqrtf(-logf(1.0f - U1));
        float s, c;
        sincosf(2.0f * kPi * U2, &s, &c);
        *sx = r * c;
        *sy = r * s;
        return;
    }
    const float tanThetaI = sinThetaI / cosThetaI;
    const float cotThetaI = 1.0f / tanThetaI;
    float a = -1.0f, c = refErff(cotThetaI);
    const float samplex = fmaxf(U1, 1.0e-6f);
    const float thetaI = atan2f(sinThetaI, cosThetaI);   // acos loses digits near normal incidence
    const float fit = 1.0f + thetaI * (-0.876f + thetaI * (0.4265f - 0.0594f * thetaI));
    // The reference iterates on b in [-1, erf(cot)]; here on q = 1 + b in [0, 1 + erf(cot)],
    // the same iteration, because b sits near -1 for small samples, where float32 would
    // keep few digits of 1 + b (and erfinv is steep).  Start: b = c - (1 + c)
    // (1 - samplex)^fit, i.e. q = (1 + c)(1 - (1 - samplex)^fit).
    float q = (1.0f + c) * -expm1f(fit * log1pf(-samplex));
    float qa = a + 1.0f, qc = c + 1.0f;
    const float sqrtPiInv = 0.5641895835f;   // 1 / sqrt(pi)
    const float norm = 1.0f / (1.0f + c + sqrtPiInv * tanThetaI * expf(-cotThetaI * cotThetaI));
    for (int it = 0; it < 16; it++) {
        if (q < qa || qc < q) q = 0.5f * (qa + qc);
        const float xm = refErfinvq(q);
        const float value = norm * (q + sqrtPiInv * tanThetaI * expf(-xm * xm)) - samplex;
        const float deriv = norm * (1.0f - xm * tanThetaI);
        if (fabsf(value) < 1.0e-6f) break;
        if (value > 0.0f) qc = q;
        else qa = q;
        q -= value / deriv;
    }
    *sx = refErfinvq(q);
    *sy = refErfinvq(2.0f * fmaxf(U2, 1.0e-6f));   // erfinv(2 U2 - 1)
}
// stretch, sample the slopes, rotate, unstretch (shared by both distributions)
template <bool BECKMANN>
__device__ __forceinline__ float3 visibleNormal(float3 wo, float a, float u0, float u1) {
    const bool flip = wo.z < 0.0f;
    const float3 w = flip ? -wo : wo;
    const float3 ws = normalize(mk(a * w.x, a * w.y, w.z));
    const float st = sqrtf(ws.x * ws.x + ws.y * ws.y);
    float sx, sy;
    if (BECKMANN) beckSample11(ws.z, st, u0, u1, &sx, &sy);
    else ggxSample11(ws.z, st, u0, u1, &sx, &sy);
    const float cp = st == 0.0f ? 1.0f : clampf(ws.x / st, -1.0f, 1.0f);
    const float sp = st == 0.0f ? 0.0f : clampf(ws.y / st, -1.0f, 1.0f);
    const float tmp = cp * sx - sp * sy;
    sy = sp * sx + cp * sy;
    sx = tmp * a;
    sy = sy * a;
    const float3 wh = normalize(mk(-sx, -sy, 1.0f));
    return flip ? -wh : wh;
}

// microfacet distribution of a rough conductor (a.w alpha, b.w 0 GGX / 1 Beckmann):
// MicrofacetDistribution's D, G and visible-normal pdf (microfacet.cc:15-60)
__device__ __forceinline__ float condD(const MaterialRecord &m, float3 wh) {
    return m.b.w != 0.0f ? beckD(wh, m.a.w) : ggxD(wh, m.a.w);
}
__device__ __forceinline__ float condLambda(const MaterialRecord &m, float3 w) {
    return m.b.w != 0.0f ? beckLambda(w, m.a.w) : ggxLambda(w, m.a.w);
}
__device__ __forceinline__ float condG(const MaterialRecord &m, float3 wo, float3 wi, float3 wh) {
    if (wi.z * dot(wi, wh) <= 0.0f) return 0.0f;
    if (wo.z * dot(wo, wh) <= 0.0f) return 0.0f;
    return 1.0f / (1.0f + condLambda(m, wo) + condLambda(m, wi));
}
__device__ __forceinline__ float condPdf(const MaterialRecord &m, float3 wo, float3 wh) {
    const float g1 = wo.z * dot(wo, wh) <= 0.0f ? 0.0f : 1.0f / (1.0f + condLambda(m, wo));
    return condD(m, wh) * g1 * fabsf(dot(wo, wh)) / fabsf(wo.z);
}

// microfacet distribution of a rough dielectric (a.x alpha, a.z 0 Beckmann / 1 GGX)
__device__ __forceinline__ float mfD(const MaterialRecord &m, float3 wh) {
    return m.a.z == 0.0f ? beckD(wh, m.a.x) : ggxD(wh, m.a.x);
}
__device__ __forceinline__ float mfLambda(const MaterialRecord &m, float3 w) {
    return m.a.z == 0.0f ? beckLambda(w, m.a.x) : ggxLambda(w, m.a.x);
}
__device__ __forceinline__ float mfG(const MaterialRecord &m, float3 wo, float3 wi, float3 wh) {
    if (wi.z * dot(wi, wh) <= 0.0f) return 0.0f;
    if (wo.z * dot(wo, wh) <= 0.0f) return 0.0f;
    return 1.0f / (1.0f + mfLambda(m, wo) + mfLambda(m, wi));
}
__device__ __forceinline__ float mfPdf(const MaterialRecord &m, float3 wo, float3 wh) {
    if (wo.z * dot(wo, wh) <= 0.0f) return 0.0f;
    const float g1 = 1.0f / (1.0f + mfLambda(m, wo));
    return mfD(m, wh) * g1 * fabsf(dot(wo, wh)) / fabsf(wo.z);
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

// MicrofacetTransmission (bxdf.cc:304-427) with etaA = 1, etaB = ior, white Kr / Kt
__device__ __forceinline__ float3 mtHalf(const MaterialRecord &m, float3 wo, float3 wi) {
    float3 wh;
    if (wo.z * wi.z > 0.0f) {
        wh = normalize(wo + wi);
    } else {
        const float eta = wo.z > 0.0f ? m.a.y : 1.0f / m.a.y;
        wh = normalize(wo + wi * eta);
    }
    return wh.z >= 0.0f ? wh : -wh;
}
__device__ __forceinline__ float mtF(const MaterialRecord &m, float3 wo, float3 wi, float3 wh) {
    const float cO = wo.z, cI = wi.z;
    if (cO == 0.0f || cI == 0.0f) return 0.0f;
    if (wo.z * dot(wo, wh) <= 0.0f) return 0.0f;
    if (wi.z * dot(wi, wh) <= 0.0f) return 0.0f;
    const float F = frDielectric(dot(wo, wh), 1.0f, m.a.y);
    if (wo.z * wi.z > 0.0f) return F * mfD(m, wh) * mfG(m, wo, wi, wh) / (4.0f * cO * cI);
    const float eta = dot(wo, wh) > 0.0f ? m.a.y : 1.0f / m.a.y;
    const float factor = 1.0f / eta;
    const float sd = dot(wo, wh) + eta * dot(wi, wh);
    return (1.0f - F) * fabsf(mfD(m, wh) * mfG(m, wo, wi, wh) * eta * eta * fabsf(dot(wi, wh)) *
                              fabsf(dot(wo, wh)) * factor * factor / (cI * cO * sd * sd));
}
__device__ __forceinline__ float mtPdf(const MaterialRecord &m, float3 wo, float3 wi, float3 wh) {
    if (wo.z * dot(wo, wh) <= 0.0f) return 0.0f;
    if (wi.z * dot(wi, wh) <= 0.0f) return 0.0f;
    const float F = frDielectric(dot(wo, wh), 1.0f, m.a.y);
    if (wo.z * wi.z > 0.0f) return F * mfPdf(m, wo, wh) / (4.0f * fabsf(dot(wo, wh)));
    const float eta = dot(wo, wh) > 0.0f ? m.a.y : 1.0f / m.a.y;
    const float sd = dot(wo, wh) + eta * dot(wi, wh);
    return (1.0f - F) * mfPdf(m, wo, wh) * fabsf((eta * eta * dot(wi, wh)) / (sd * sd));
}

// PlasticBRDF (bsdfs/plastic.cc:18-95) with etaA = 1, etaB = ior
__device__ __forceinline__ float frDiffuseReflectance(float eta) {   // fresnel.cc:87
    if (eta >= 1.0f) return -1.4399f / (eta * eta) + 0.7099f / eta + 0.6681f + 0.0636f * eta;
    return -0.4399f + 0.7099f / eta - 0.3319f / (eta * eta) + 0.0636f / (eta * eta * eta);
}
__device__ __forceinline__ float plasticProbSpecular(const MaterialRecord &m, float3 wo) {
    const float Fo = frDielectric(wo.z, 1.0f, m.a.w), s = m.b.w;
    return (Fo * s) / (Fo * s + (1.0f - Fo) * (1.0f - s));
}
// PlasticBRDF::f and pdf test wi against its own mirror image (plastic.cc:33,76):
// true only for wi along the normal
__device__ __forceinline__ bool plasticMirror(float3 wi) { return wi.z * wi.z - wi.x * wi.x - wi.y * wi.y > 1.0f - 1.0e-12f; }
__device__ __forceinline__ float3 plasticDiffuse(const MaterialRecord &m, float3 wo, float3 wi) {
    const float Fo = frDielectric(wo.z, 1.0f, m.a.w), Fi = frDielectric(wi.z, 1.0f, m.a.w);
    const float invEta = 1.0f / m.a.w;
    return xyz(m.a) * ((1.0f - Fo) * (1.0f - Fi) * invEta * invEta * kInvPi / (1.0f - frDiffuseReflectance(m.a.w)));
}

// FresnelSpecular's f and pdf treat wi within 1e-4 (in cosine) of the mirror or the
// refracted direction as the delta direction: F (reflection) or 1 - F (transmission)
// there, 0 elsewhere (bxdf.cc:171-196, 236-247)
__device__ __forceinline__ float dielectricCone(const MaterialRecord &m, float3 wo, float3 wi) {
    const float F = frDielectric(wo.z, 1.0f, m.a.w);
    if (wo.z * wi.z > 0.0f) return dot(mk(-wo.x, -wo.y, wo.z), wi) > 1.0f - 1.0e-4f ? F : 0.0f;
    const bool entering = wo.z > 0.0f;
    const float eI = entering ? 1.0f : m.a.w, eT = entering ? m.a.w : 1.0f;
    float3 wt;
    if (!refract(wo, mk(0.0f, 0.0f, entering ? 1.0f : -1.0f), eI / eT, &wt)) return 0.0f;
    return dot(wi, wt) > 1.0f - 1.0e-4f ? 1.0f - F : 0.0f;
}

// f(wo, wi) of the material's BxDF (BSDF::f)
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
        const float3 F = frConductor(fabsf(dot(wi, wh)), xyz(m.a), xyz(m.b));
        return F * (condD(m, wh) * condG(m, wo, wi, wh) / (4.0f * cI * cO));
    }
    if (m.type == kMatRoughDielectric) {
        if (wo.z == 0.0f || wi.z == 0.0f) return mk(0, 0, 0);
        const float v = mtF(m, wo, wi, mtHalf(m, wo, wi));
        return mk(v, v, v);
    }
    if (m.type == kMatPlastic) {
        if (wo.z * wi.z <= 0.0f) return mk(0, 0, 0);   // reflection only (BSDF::f, bsdf.cc:57)
        if (plasticMirror(wi)) return xyz(m.b) * (frDielectric(wo.z, 1.0f, m.a.w) / fabsf(wi.z));
        return plasticDiffuse(m, wo, wi);
    }
    if (m.type == kMatDielectric) {   // FresnelSpecular::f (bxdf.cc:171): a 1e-4 cone about the deltas
        const float v = dielectricCone(m, wo, wi);
        return mk(v, v, v) / fabsf(wi.z);
    }
    return mk(0, 0, 0);
}
__device__ __forceinline__ float bsdfPdf(const MaterialRecord &m, float3 wo, float3 wi) {
    if (m.type == kMatRoughDielectric) return mtPdf(m, wo, wi, mtHalf(m, wo, wi));
    if (m.type == kMatPlastic) {   // PlasticBRDF::pdf (plastic.cc:69) tests no hemisphere
        const float ps = plasticProbSpecular(m, wo);
        return plasticMirror(wi) ? ps : (1.0f - ps) * fabsf(wi.z) * kInvPi;
    }
    if (wo.z * wi.z <= 0.0f) return 0.0f;
    if (m.type == kMatLambert) return fabsf(wi.z) * kInvPi;
    if (m.type == kMatConductor) {
        const float3 wh = normalize(wo + wi);
        return condPdf(m, wo, wh) / (4.0f * dot(wo, wh));
    }
    return 0.0f;
}
__device__ __forceinline__ float bsdfPdfDielectricCone(const MaterialRecord &m, float3 wo, float3 wi) {
    return dielectricCone(m, wo, wi);   // FresnelSpecular::pdf (bxdf.cc:236): F or 1 - F inside the cones
}
// The material's BxDF::sample; returns f, sets wi, pdf and the sampled type bits.  uc is
// the draw the reference takes from its BxDFs' hidden generator (core/bxdf.cc:18,
// bsdfs/plastic.cc:18): the rough dielectric's reflect / refract and the plastic's
// specular / diffuse choice.
__device__ __forceinline__ float3 bxdfSample(const MaterialRecord &m, float3 wo, float u0, float u1, float uc,
                                             float3 *wi, float *pdf, int *type) {
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
    if (m.type == kMatConductor) {   // MicrofacetReflection::sample, bxdf.cc:282
        const float3 wh = m.b.w != 0.0f ? visibleNormal<true>(wo, m.a.w, ur0, u1)
                                        : visibleNormal<false>(wo, m.a.w, ur0, u1);
        const float3 w = -wo + wh * (2.0f * dot(wh, wo));
        if (wo.z * w.z <= 0.0f) return mk(0, 0, 0);
        *wi = w;
        *pdf = condPdf(m, wo, wh) / (4.0f * dot(wo, wh));
        *type = kReflection | kGlossy;
        return bsdfF(m, wo, w);
    }
    if (m.type == kMatRoughDielectric) {   // MicrofacetTransmission::sample, bxdf.cc:356
        const float3 wh = m.a.z == 0.0f ? visibleNormal<true>(wo, m.a.x, ur0, u1)
                                        : visibleNormal<false>(wo, m.a.x, ur0, u1);
        const float cO = dot(wo, wh.z > 0.0f ? wh : -wh);
        const float F = frDielectric(cO, 1.0f, m.a.y);
        float3 w;
        int t;
        if (uc < F) {
            w = -wo + wh * (2.0f * dot(wh, wo));
            if (wo.z * w.z <= 0.0f) return mk(0, 0, 0);
            t = kReflection | kGlossy;
        } else {
            const float eta = cO > 0.0f ? 1.0f / m.a.y : m.a.y;
            if (!refract(wo, wh, eta, &w) || wo.z * w.z > 0.0f) return mk(0, 0, 0);
            t = kTransmission | kGlossy;
        }
        const float3 whp = wh.z >= 0.0f ? wh : -wh;
        *wi = w;
        *pdf = mtPdf(m, wo, w, whp);
        *type = t;
        const float v = mtF(m, wo, w, whp);
        return mk(v, v, v);
    }
    if (m.type == kMatPlastic) {   // PlasticBRDF::sample, plastic.cc:44; the BxDF's own type is reported
        const float ps = plasticProbSpecular(m, wo);
        *type = kReflection | kSpecular | kDiffuse;
        if (uc < ps) {
            *wi = mk(-wo.x, -wo.y, wo.z);
            *pdf = ps;
            return xyz(m.b) * (frDielectric(wo.z, 1.0f, m.a.w) / fabsf(wo.z));
        }
        const float3 w = cosineHemisphere(ur0, u1);
        *wi = w;
        *pdf = (1.0f - ps) * fabsf(w.z) * kInvPi;
        return plasticDiffuse(m, wo, w);
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

// BSDF::sample (core/bsdf.cc:65-110) over the material's one BxDF: a sample of pdf 0 is
// no sample (type 0, f 0)
__device__ __forceinline__ float3 bsdfSample(const MaterialRecord &m, float3 wo, float u0, float u1, float uc,
                                             float3 *wi, float *pdf, int *type) {
    const float3 f = bxdfSample(m, wo, u0, u1, uc, wi, pdf, type);
    if (*pdf == 0.0f) {
        *type = 0;
        return mk(0, 0, 0);
    }
    return f;
}

// wavefront shading class (sort key of the material-sorted queues): 0 diffuse, 1 glossy,
// 2 specular-typed
__device__ __forceinline__ int shadeClass(int type) {
    return type == kMatLambert ? 0 : (type == kMatConductor || type == kMatRoughDielectric) ? 1 : 2;
}

__device__ __forceinline__ float powerHeuristic(float f, float g) { return (f * f) / (f * f + g * g); }

}  // namespace spgpu
