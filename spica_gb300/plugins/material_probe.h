// material_probe.h -- translation of a reference BSDF into a spgpu material record
// (include/spica_gpu.h, SPGPU_MAT_*), through the BSDF's public interface only:
// hasType, numComponents, f, pdf and eta (core/bsdf.h:20-54), with the reference's
// exported Fresnel and microfacet functions (core/fresnel.h:64-66,
// core/microfacet.h:16-72) to check the result.
//
// The BSDF must be built in a unit frame (shading normal z, dpdu x, dpdv y), so that
// world and local directions coincide.  BxDF types (core/bxdf.cc) decide the material:
//   Reflection|Diffuse                     Lambert          R = pi f(z, z)
//   Reflection|Glossy                      rough conductor  alpha from pdf(z, z) = 1 / (4 pi alpha^2),
//                                                           F0 = 4 pi alpha^2 f(z, z), stored as
//                                                           eta = 1, k = 2 sqrt(F0 / (1 - F0)) (exact
//                                                           for F0-authored conductors; others are
//                                                           matched at normal incidence); GGX or
//                                                           Beckmann from f along a retro direction
//   Reflection|Transmission|Specular       dielectric       IOR = BSDF::eta() (bsdfs/dielectric.cc:38)
//   Reflection|Transmission|Glossy         rough dielectric IOR = BSDF::eta(); alpha from
//                                                           pdf(z, z) = F0 / (4 pi alpha^2); Beckmann
//                                                           or GGX: the one whose MicrofacetTransmission
//                                                           reproduces f on reflected and refracted pairs
//                                                           (bsdfs/roughdielectric.cc:41-84)
//   Reflection|Specular|Diffuse            plastic          IOR from the angular shape of the Fresnel
//                                                           term, Ks = f(z, z) / F0, Kd from the diffuse
//                                                           lobe (bsdfs/plastic.cc:29-46)
// Anything else (smooth conductors, rough plastic, subsurface, anisotropic or tinted
// rough dielectrics, IOR < 1 plastics) is refused with a reason: the GPU path has no
// such material, and a silent approximation would render a different image.
#pragma once

#include <cmath>
#include <string>
#include <vector>

#include "core/bsdf.h"
#include "core/bxdf.h"
#include "core/common.h"
#include "core/fresnel.h"
#include "core/microfacet.h"
#include "core/spectrum.h"

#include "spica_gpu.h"

namespace spgpu_probe {

using spica::BSDF;
using spica::BxDFType;
using spica::Spectrum;
using spica::Vector3d;

inline Vector3d direction(double theta, double phi) {
    return Vector3d(std::sin(theta) * std::cos(phi), std::sin(theta) * std::sin(phi), std::cos(theta));
}

inline double relDiff(double a, double b) {
    const double s = std::max(std::abs(a), std::abs(b));
    return s == 0.0 ? 0.0 : std::abs(a - b) / s;
}

inline double maxRelDiff(const Spectrum &a, const Spectrum &b) {
    return std::max(relDiff(a.red(), b.red()), std::max(relDiff(a.green(), b.green()), relDiff(a.blue(), b.blue())));
}

// the indices in (1, 6] with ratio(eta) == target: a scan for sign changes, then
// bisection in each bracket (Fresnel ratios need not be monotone in eta: Brewster's
// angle moves with it)
template <class Ratio>
std::vector<double> solveEta(const Ratio &ratio, double target) {
    std::vector<double> roots;
    const int n = 1024;
    double a = 1.0 + 1e-9, ga = ratio(a) - target;
    for (int k = 1; k <= n; k++) {
        const double b = 1.0 + 5.0 * k / n, gb = ratio(b) - target;
        if (ga == 0.0) roots.push_back(a);
        if ((ga < 0.0) != (gb < 0.0) && gb != 0.0) {
            double lo = a, hi = b, glo = ga;
            for (int it = 0; it < 200 && hi - lo > 1e-15 * hi; it++) {
                const double mid = 0.5 * (lo + hi), gm = ratio(mid) - target;
                if ((gm < 0.0) == (glo < 0.0)) { lo = mid; glo = gm; } else { hi = mid; }
            }
            roots.push_back(0.5 * (lo + hi));
        }
        a = b;
        ga = gb;
    }
    return roots;
}

inline int refuse(std::string *why, const char *msg) {
    if (why) *why = msg;
    return -1;
}

inline int probeRoughDielectric(const BSDF &b, float rec[8], std::string *why) {
    const Vector3d z(0.0, 0.0, 1.0);
    const double eta = b.eta();
    const double F0 = spica::FrDielectric(1.0, 1.0, eta);
    const double p0 = b.pdf(z, z);
    if (!(eta > 0.0) || !(F0 > 0.0) || !(p0 > 0.0)) return refuse(why, "rough dielectric with index 1 or no reflection lobe");
    const double alpha = std::sqrt(F0 / (4.0 * ::PI * p0));
    // reflected and refracted pairs, from above and from inside, at several azimuths
    const Vector3d wo[4] = {direction(0.4, 0.3), direction(0.9, 2.1), direction(0.5, 1.0), direction(2.5, 4.0)};
    const Vector3d wi[4] = {direction(0.7, 2.5), direction(0.3, 5.0), direction(2.6, 3.9), direction(0.8, 0.7)};
    spica::BeckmannDistribution beckmann(alpha, alpha);
    spica::TrowbridgeReitzDistribution ggx(alpha, alpha);
    spica::MicrofacetDistribution *cand[2] = {&beckmann, &ggx};
    for (int d = 0; d < 2; d++) {
        spica::MicrofacetTransmission model(Spectrum(1.0), Spectrum(1.0), cand[d], 1.0, eta);
        double err = 0.0;
        for (int k = 0; k < 4; k++) err = std::max(err, maxRelDiff(b.f(wo[k], wi[k]), model.f(wo[k], wi[k])));
        if (err < 1e-6) {
            rec[0] = SPGPU_MAT_ROUGH_DIELECTRIC;
            rec[1] = static_cast<float>(alpha);
            rec[2] = static_cast<float>(eta);
            rec[3] = static_cast<float>(d);
            return 0;
        }
    }
    return refuse(why, "rough dielectric that is anisotropic, tinted (Kr, Kt not white) or neither Beckmann nor GGX");
}

inline int probePlastic(const BSDF &b, float rec[8], std::string *why) {
    const Vector3d z(0.0, 0.0, 1.0);
    const double thetaO = 1.0, thetaD = 0.8;
    const Vector3d wd = direction(thetaD, 0.6);   // a diffuse-lobe direction (not along the normal)
    const Spectrum fs = b.f(z, z);                 // specular branch: F0 Ks
    const Spectrum fd = b.f(z, wd);                 // diffuse branch
    // the index from the angular shape of a Fresnel term: of the specular branch
    // f(wo, z) = Fo(wo) Ks where Ks is not black, else of the diffuse branch
    // f(z, wi) ~ 1 - Fi(wi); a second angle picks between several roots
    const bool spec = fs.gray() > 0.0;
    if (!spec && !(fd.gray() > 0.0)) return refuse(why, "plastic with no positive reflection lobe");
    const double th[3] = {spec ? 0.0 : thetaD, 1.0, 1.35};
    double meas[3];
    for (int k = 0; k < 3; k++) {
        meas[k] = spec ? b.f(direction(th[k], 1.7), z).gray() : b.f(z, direction(th[k], 0.6)).gray();
    }
    auto shape = [&](int k, double e) {
        return spec ? spica::FrDielectric(std::cos(th[k]), 1.0, e) / spica::FrDielectric(1.0, 1.0, e)
                    : (1.0 - spica::FrDielectric(std::cos(th[k]), 1.0, e)) / (1.0 - spica::FrDielectric(std::cos(th[0]), 1.0, e));
    };
    double eta = NAN, best = 1e-6;
    for (double e : solveEta([&](double x) { return shape(1, x); }, meas[1] / meas[0])) {
        const double r = relDiff(shape(2, e), meas[2] / meas[0]);
        if (r < best) { best = r; eta = e; }
    }
    if (!(eta > 1.0)) return refuse(why, "plastic whose index is not in (1, 6]");
    const double F0 = spica::FrDielectric(1.0, 1.0, eta);
    const double Fi = spica::FrDielectric(std::cos(thetaD), 1.0, eta);
    const double Fdr = spica::FrDiffuseReflectance(eta);
    const double kdScale = ::PI * (1.0 - Fdr) * eta * eta / ((1.0 - F0) * (1.0 - Fi));
    const double kd[3] = {fd.red() * kdScale, fd.green() * kdScale, fd.blue() * kdScale};
    const double ks[3] = {fs.red() / F0, fs.green() / F0, fs.blue() / F0};
    // check against the plastic's pdf: the diffuse lobe's share follows from the Fresnel
    // term and the specular sampling weight Ks.gray / (Kd.gray + Ks.gray) (plastic.cc:26)
    const double kdg = Spectrum(kd[0], kd[1], kd[2]).gray(), ksg = Spectrum(ks[0], ks[1], ks[2]).gray();
    const double w = ksg / (kdg + ksg);
    const double Fo = spica::FrDielectric(std::cos(thetaO), 1.0, eta);
    const double probSpec = Fo * w / (Fo * w + (1.0 - Fo) * (1.0 - w));
    const double pdfModel = (1.0 - probSpec) * std::cos(thetaD) * ::INV_PI;
    if (relDiff(b.pdf(direction(thetaO, 1.7), wd), pdfModel) > 1e-6) {
        return refuse(why, "plastic-typed BSDF that does not follow the plastic model");
    }
    rec[0] = SPGPU_MAT_PLASTIC;
    for (int c = 0; c < 3; c++) {
        rec[1 + c] = static_cast<float>(kd[c]);
        rec[4 + c] = static_cast<float>(ks[c]);
    }
    rec[7] = static_cast<float>(eta);
    return 0;
}

// 0 and a record in rec[0..7], or -1 and the reason in *why
inline int probeMaterial(const BSDF *b, float rec[8], std::string *why) {
    for (int i = 0; i < 8; i++) rec[i] = 0.0f;
    rec[0] = SPGPU_MAT_LAMBERT;
    if (!b || b->numComponents() == 0) return 0;   // black
    const bool T = b->hasType(BxDFType::Transmission), S = b->hasType(BxDFType::Specular);
    const bool G = b->hasType(BxDFType::Glossy), D = b->hasType(BxDFType::Diffuse);
    const Vector3d z(0.0, 0.0, 1.0);
    if (T && S && !G && !D) {
        rec[0] = SPGPU_MAT_DIELECTRIC;
        rec[1] = static_cast<float>(b->eta());
        return 0;
    }
    if (T && G && !S && !D) return probeRoughDielectric(*b, rec, why);
    if (S && D && !T && !G) return probePlastic(*b, rec, why);
    if (G && !T && !S && !D) {
        const double pdf = b->pdf(z, z);
        const double alpha = std::sqrt(1.0 / (4.0 * ::PI * pdf));
        const Spectrum f = b->f(z, z);
        const double f0[3] = {f.red(), f.green(), f.blue()};
        // the distribution: along the retro-reflection direction w (half vector w, so the
        // Fresnel factor is the normal-incidence one) f(w, w) / f(z, z) is
        // D(w) G(w, w, w) / (cos^2 D(z)), which tells Beckmann from GGX
        const Vector3d w = direction(0.9, 0.4);
        const double ratio = b->f(w, w).gray() / f.gray();
        spica::BeckmannDistribution beckmann(alpha, alpha);
        spica::TrowbridgeReitzDistribution ggx(alpha, alpha);
        auto shape = [&](const spica::MicrofacetDistribution &d) {
            return d.D(w) * d.G(w, w, w) / (w.z() * w.z() * d.D(z));
        };
        int type;
        if (relDiff(ratio, shape(ggx)) < 1e-6) type = SPGPU_MAT_CONDUCTOR;
        else if (relDiff(ratio, shape(beckmann)) < 1e-6) type = SPGPU_MAT_CONDUCTOR_BECKMANN;
        else return refuse(why, "rough conductor that is anisotropic or neither Beckmann nor GGX");
        rec[0] = static_cast<float>(type);
        rec[1] = static_cast<float>(alpha);
        for (int c = 0; c < 3; c++) {
            const double F0 = std::min(0.999, 4.0 * ::PI * alpha * alpha * f0[c]);
            rec[2 + c] = 1.0f;
            rec[5 + c] = static_cast<float>(2.0 * std::sqrt(F0 / (1.0 - F0)));
        }
        return 0;
    }
    if (D && !T && !S && !G) {
        const Spectrum f = b->f(z, z);
        rec[1] = static_cast<float>(::PI * f.red());
        rec[2] = static_cast<float>(::PI * f.green());
        rec[3] = static_cast<float>(::PI * f.blue());
        return 0;
    }
    return refuse(why, "material type with no GPU counterpart (smooth conductor, rough plastic, subsurface, ...)");
}

}  // namespace spgpu_probe
