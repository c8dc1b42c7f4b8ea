// ref_driver.cc -- drives the reference renderer's own, unmodified hot-path code
// through the spo_* C API (spo_api.h).  TEST INFRASTRUCTURE ONLY: it is compiled
// by oracle/Makefile (target "ref") together with the reference sources into
// oracle/_ref/libspica_ref.so, which tests use to pin the C++ restatement
// (spica_oracle.cc) and to generate the golden fixtures under tests/golden/.
//
// What it calls, all reference code:
//   scene:       Triangle (core/triangle.cc:17), GeometricPrimitive (core/primitive.cc:49),
//                AreaLight (lights/area.cc:6), Envmap (lights/envmap.cc:17),
//                BVHAccel (accelerators/bvh.cc:112), Scene (core/scene.cc)
//   materials:   Diffuse, RoughConductor(distribution "ggx", no remap), Dielectric
//   tracing:     BVHAccel::intersect(Ray&, SurfaceInteraction*) / intersect(Ray&)
//   rendering:   PerspectiveCamera::spawnRay (cameras/perspective.cc:53) and
//                PathIntegrator::Li (integrators/path/path.cc:42), with the x-mirrored
//                film write of SamplerIntegrator::render (core/integrator.cc:88)
//   BSDFs:       BSDF::f / pdf / sample (core/bsdf.cc:49-136)
#include "core/cobject.h"
// Each plugin header expands its export macro; the driver links every plugin into
// one library, so the macros are emptied here (the objects were compiled with the
// entry points renamed, see oracle/Makefile).
#undef SPICA_EXPORT_PLUGIN
#undef SPICA_EXPORT_ACCEL_PLUGIN
#define SPICA_EXPORT_PLUGIN(name, descr)
#define SPICA_EXPORT_ACCEL_PLUGIN(name, descr)

#include "core/common.h"
#include "core/constant.h"
#include "core/bsphere.h"
#include "core/image.h"
#include "core/tmo.h"
#include "core/interaction.h"
#include "core/bsdf.h"
#include "core/bxdf.h"
#include "core/memory.h"
#include "core/material.h"
#include "core/primitive.h"
#include "core/ray.h"
#include "core/renderparams.h"
#include "core/scene.h"
#include "core/transform.h"
#include "core/triangle.h"
#include "core/bounds2d.h"
#include "core/spectrum.h"

#include "accelerators/bvh.h"
#include "bsdfs/dielectric.h"
#include "bsdfs/plastic.h"
#include "bsdfs/roughdielectric.h"
#include "bsdfs/diffuse.h"
#include "bsdfs/roughconductor.h"
#include "cameras/perspective.h"
#include "films/hdrfilm.h"
#include "filters/box.h"
#include "integrators/directlighting/directlighting.h"
#include "integrators/path/path.h"
#include "lights/area.h"
#include "lights/envmap.h"
#include "samplers/independent.h"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "core/meshio.h"
#include "material_probe.h"   // the drop-in plugin's material translation, under test
#include "spo_api.h"

using namespace spica;

namespace {

using SpecTex = Texture<Spectrum>;

std::shared_ptr<SpecTex> constTex(const Spectrum &s) {
    return std::make_shared<ConstantTexture<Spectrum>>(s);
}

std::shared_ptr<SurfaceMaterial> makeSurface(const double *m) {
    const int type = static_cast<int>(m[0]);
    if (type == SPO_MAT_LAMBERT) {
        return std::make_shared<Diffuse>(constTex(Spectrum(m[1], m[2], m[3])));
    }
    if (type == SPO_MAT_CONDUCTOR || type == SPO_MAT_CONDUCTOR_BECKMANN) {
        auto alpha = constTex(Spectrum(m[1]));
        return std::make_shared<RoughConductor>(constTex(Spectrum(m[2], m[3], m[4])),
                                                constTex(Spectrum(m[5], m[6], m[7])), alpha, alpha,
                                                type == SPO_MAT_CONDUCTOR ? "ggx" : "beckmann", nullptr, false);
    }
    if (type == SPO_MAT_ROUGH_DIELECTRIC) {
        auto alpha = constTex(Spectrum(m[1]));
        return std::make_shared<RoughDielectric>(constTex(Spectrum(1.0)), constTex(Spectrum(1.0)), alpha, alpha,
                                                 constTex(Spectrum(m[2])), m[3] != 0.0 ? "ggx" : "beckmann",
                                                 nullptr, false);
    }
    if (type == SPO_MAT_PLASTIC) {
        return std::make_shared<Plastic>(constTex(Spectrum(m[1], m[2], m[3])), constTex(Spectrum(m[4], m[5], m[6])),
                                         constTex(Spectrum(m[7])), nullptr);
    }
    return std::make_shared<Dielectric>(constTex(Spectrum(1.0)), constTex(Spectrum(1.0)),
                                        constTex(Spectrum(m[1])), nullptr);
}

// PathIntegrator::Li is protected; the driver only re-exposes it.
class OpenPath : public PathIntegrator {
public:
    explicit OpenPath(const std::shared_ptr<Sampler> &s) : PathIntegrator{s} {}
    Spectrum radiance(const Scene &scene, RenderParams &params, const Ray &ray,
                      Sampler &sampler, MemoryArena &arena) const {
        return Li(scene, params, ray, sampler, arena, 0);
    }
};

// DirectLightingIntegrator::Li (integrators/directlighting/directlighting.cc:21)
class OpenDirect : public DirectLightingIntegrator {
public:
    explicit OpenDirect(const std::shared_ptr<Sampler> &s) : DirectLightingIntegrator{s} {}
    Spectrum radiance(const Scene &scene, RenderParams &params, const Ray &ray,
                      Sampler &sampler, MemoryArena &arena) const {
        return Li(scene, params, ray, sampler, arena, 0);
    }
};

template <class F>
void parallelRange(int64_t n, int nthreads, int64_t chunk, F &&body) {
    if (nthreads <= 1) {
        // one fresh thread: the BxDFs' hidden thread_local generators (core/bxdf.cc:18,
        // bsdfs/plastic.cc:18) start from their seed, so single-threaded results are
        // reproducible
        std::thread th([&]() {
            for (int64_t i = 0; i < n; i += chunk) body(i, std::min(n, i + chunk));
        });
        th.join();
        return;
    }
    std::atomic<int64_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; t++) {
        pool.emplace_back([&]() {
            for (;;) {
                const int64_t b = next.fetch_add(chunk);
                if (b >= n) break;
                body(b, std::min(n, b + chunk));
            }
        });
    }
    for (auto &th : pool) th.join();
}

}  // namespace

struct spo_scene {
    std::vector<std::shared_ptr<Primitive>> prims;
    std::vector<std::shared_ptr<Light>> lights;
    std::shared_ptr<BVHAccel> accel;
    std::unique_ptr<Scene> scene;
};

extern "C" {

const char *spo_name(void) { return "reference"; }

spo_scene *spo_scene_create(int ntri, const double *verts, const int32_t *tri_mat, int nmat,
                            const double *mats, const double *tri_emit, int env_w, int env_h,
                            const float *env, int use_simd) {
    auto *s = new spo_scene();
    std::vector<std::shared_ptr<Material>> materials;
    for (int m = 0; m < nmat; m++) {
        materials.push_back(std::make_shared<Material>(makeSurface(mats + SPO_MAT_STRIDE * m)));
    }
    Bounds3d bounds;
    for (int i = 0; i < ntri; i++) {
        const double *v = verts + 9 * i;
        const Point3d p0(v[0], v[1], v[2]), p1(v[3], v[4], v[5]), p2(v[6], v[7], v[8]);
        bounds.merge(p0);
        bounds.merge(p1);
        bounds.merge(p2);
        auto tri = std::make_shared<Triangle>(p0, p1, p2, Transform());
        std::shared_ptr<Light> area;
        if (tri_emit) {
            const double *e = tri_emit + 3 * i;
            if (e[0] != 0.0 || e[1] != 0.0 || e[2] != 0.0) {
                area = std::make_shared<AreaLight>(tri, Transform(), Spectrum(e[0], e[1], e[2]));
                s->lights.push_back(area);
            }
        }
        s->prims.push_back(std::make_shared<GeometricPrimitive>(tri, materials[tri_mat[i]], area));
    }
    if (env) {
        Image img(env_w, env_h);
        for (int y = 0; y < env_h; y++) {
            for (int x = 0; x < env_w; x++) {
                const float *p = env + 3 * (static_cast<int64_t>(y) * env_w + x);
                img.pixel(x, y) = RGBSpectrum(p[0], p[1], p[2]);
            }
        }
        const Point3d c = 0.5 * (bounds.posMin() + bounds.posMax());
        const double r = 0.5 * (bounds.posMax() - bounds.posMin()).norm();
        s->lights.push_back(std::make_shared<Envmap>(BSphere(c, r), img, Transform(), 1.0));
    }
    s->accel = std::make_shared<BVHAccel>(s->prims, use_simd != 0);
    s->scene = std::make_unique<Scene>(s->accel, s->lights);
    return s;
}

void spo_scene_destroy(spo_scene *s) { delete s; }

double spo_triangle_area(const double *v) {
    const Triangle tri(Point3d(v[0], v[1], v[2]), Point3d(v[3], v[4], v[5]), Point3d(v[6], v[7], v[8]),
                       Transform());
    return tri.area();
}

int spo_box_intersect(const double *lo, const double *hi, const double *org, const double *dir, double tmax,
                      double *tnear, double *tfar) {
    const Bounds3d b(Point3d(lo[0], lo[1], lo[2]), Point3d(hi[0], hi[1], hi[2]));
    return b.intersect(Ray(Point3d(org[0], org[1], org[2]), Vector3d(dir[0], dir[1], dir[2]), tmax), tnear, tfar)
               ? 1
               : 0;
}

void spo_ray_invdir(const double *org, const double *dir, double *inv) {
    const Ray r(Point3d(org[0], org[1], org[2]), Vector3d(dir[0], dir[1], dir[2]));
    inv[0] = r.invdir().x();
    inv[1] = r.invdir().y();
    inv[2] = r.invdir().z();
}

int spo_scene_num_lights(const spo_scene *s) { return static_cast<int>(s->lights.size()); }

int spo_trace(spo_scene *s, int any, int64_t n, const double *org, const double *dir,
              const double *tmax, int32_t *prim, double *t, uint8_t *hit, int nthreads) {
    // map primitive pointers back to triangle indices
    std::unordered_map<const Primitive *, int32_t> index;
    if (!any) {
        for (size_t i = 0; i < s->prims.size(); i++) index[s->prims[i].get()] = (int32_t)i;
    }
    parallelRange(n, nthreads, 256, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) {
            Ray ray(Point3d(org[3 * i], org[3 * i + 1], org[3 * i + 2]),
                    Vector3d(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]),
                    tmax ? tmax[i] : INFTY);
            if (any) {
                const bool h = s->scene->intersect(ray);
                if (hit) hit[i] = h ? 1 : 0;
            } else {
                SurfaceInteraction isect;
                const bool h = s->scene->intersect(ray, &isect);
                if (prim) prim[i] = h ? index.at(isect.primitive()) : -1;
                if (t) t[i] = h ? ray.maxDist() : 0.0;
                if (hit) hit[i] = h ? 1 : 0;
            }
        }
    });
    return 0;
}

}  // extern "C"

namespace {
// Film window render shared by the integrators: radiance(ray, sampler, arena) gives Li.
template <class Integ>
int renderWindow(spo_scene *s, const double *cam, int W, int H, int fx0, int fy0, int w, int h, int spp,
                 int max_depth, uint32_t seed, double *sum, double *sumsq, int nthreads) {
    RenderParams &params = RenderParams::getInstance();
    params.add("maxDepth", max_depth);
    auto film = std::make_shared<HDRFilm>(Point2i(W, H),
                                          std::make_shared<BoxFilter>(Vector2d(0.5, 0.5)),
                                          std::string("unused"));
    const Transform c2w = Transform::lookAt(Point3d(cam[0], cam[1], cam[2]),
                                            Point3d(cam[3], cam[4], cam[5]),
                                            Vector3d(cam[6], cam[7], cam[8]));
    auto camera = std::make_shared<PerspectiveCamera>(c2w, Bounds2d(-1.0, -1.0, 1.0, 1.0), 0.0,
                                                      50.0, cam[9] * PI / 180.0, film);
    auto proto = std::make_shared<Independent>(0u);
    Integ integrator(proto);
    const int64_t npix = static_cast<int64_t>(w) * h;
    parallelRange(npix, nthreads, 1, [&](int64_t b, int64_t e) {
        MemoryArena arena;
        for (int64_t q = b; q < e; q++) {
            const int fy = fy0 + static_cast<int>(q / w);
            const int fx = fx0 + static_cast<int>(q % w);
            const int x = W - 1 - fx;  // film pixel (W-1-x, y) holds raster pixel (x, y)
            const int y = fy;
            Independent sampler(spo_pixel_seed(seed, static_cast<uint32_t>(fy * W + fx)));
            double acc[3] = {0, 0, 0}, acc2[3] = {0, 0, 0};
            for (int k = 0; k < spp; k++) {
                const Point2d randFilm = sampler.get2D();
                const Point2d randLens = sampler.get2D();
                const Ray ray = camera->spawnRay(Point2i(x, y), randFilm, randLens);
                const Spectrum L = integrator.radiance(*s->scene, params, ray, sampler, arena);
                const double c[3] = {L.red(), L.green(), L.blue()};
                for (int j = 0; j < 3; j++) {
                    acc[j] += c[j];
                    acc2[j] += c[j] * c[j];
                }
                arena.reset();
            }
            for (int j = 0; j < 3; j++) {
                sum[3 * q + j] = acc[j];
                sumsq[3 * q + j] = acc2[j];
            }
        }
    });
    return 0;
}
}  // namespace

extern "C" {
int spo_render(spo_scene *s, const double *cam, int W, int H, int fx0, int fy0, int w, int h,
               int spp, int max_depth, uint32_t seed, double *sum, double *sumsq, int nthreads) {
    return renderWindow<OpenPath>(s, cam, W, H, fx0, fy0, w, h, spp, max_depth, seed, sum, sumsq, nthreads);
}

int spo_render_direct(spo_scene *s, const double *cam, int W, int H, int fx0, int fy0, int w, int h,
                      int spp, int max_depth, uint32_t seed, double *sum, double *sumsq, int nthreads) {
    return renderWindow<OpenDirect>(s, cam, W, H, fx0, fy0, w, h, spp, max_depth, seed, sum, sumsq, nthreads);
}

namespace {

struct LocalBSDF {
    MemoryArena arena;
    SurfaceInteraction isect;
    std::shared_ptr<SurfaceMaterial> surf;
    explicit LocalBSDF(const double *mat)
        : isect(Point3d(0, 0, 0), Point2d(0, 0), Vector3d(0, 0, 1), Vector3d(1, 0, 0),
                Vector3d(0, 1, 0), Normal3d(), Normal3d(), nullptr),
          surf(makeSurface(mat)) {
        surf->setScatterFuncs(&isect, arena);
    }
};

}  // namespace

int spo_bsdf_eval(const double *mat, int64_t n, const double *wo, const double *wi, double *f,
                  double *pdf) {
    LocalBSDF b(mat);
    for (int64_t i = 0; i < n; i++) {
        const Vector3d o(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
        const Vector3d d(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
        const Spectrum v = b.isect.bsdf()->f(o, d);
        f[3 * i] = v.red();
        f[3 * i + 1] = v.green();
        f[3 * i + 2] = v.blue();
        pdf[i] = b.isect.bsdf()->pdf(o, d);
    }
    return 0;
}

int spo_load_ply(const char *path, const double *m16, int64_t max_tris, double *verts, int64_t *ntri) {
    double m[4][4];
    for (int i = 0; i < 16; i++) m[i / 4][i % 4] = m16[i];
    const std::vector<ShapeGroup> groups = meshio::loadPLY(path, Transform(m));
    int64_t n = 0;
    for (const auto &g : groups) {
        for (const auto &s : g.shapes()) {
            for (const Triangle &t : s->triangulate()) {
                if (n < max_tris) {
                    for (int k = 0; k < 3; k++) {
                        verts[9 * n + 3 * k] = t[k].x();
                        verts[9 * n + 3 * k + 1] = t[k].y();
                        verts[9 * n + 3 * k + 2] = t[k].z();
                    }
                }
                n++;
            }
        }
    }
    *ntri = n;
    return 0;
}

int spo_load_hdr(const char *path, int64_t max_pixels, double *rgb, int *width, int *height) {
    Image img;
    img.load(path);
    *width = img.width();
    *height = img.height();
    if (static_cast<int64_t>(img.width()) * img.height() > max_pixels) return 1;
    for (int y = 0; y < img.height(); y++) {
        for (int x = 0; x < img.width(); x++) {
            const RGBSpectrum &p = img(x, y);
            double *o = rgb + 3 * (static_cast<int64_t>(y) * img.width() + x);
            o[0] = p.red();
            o[1] = p.green();
            o[2] = p.blue();
        }
    }
    return 0;
}

int spo_transform_chain(int n, const int *kinds, const double *params, double *out16) {
    Transform trans;
    for (int i = 0; i < n; i++) {
        const double *q = params + 16 * i;
        Transform sub;
        if (kinds[i] == 0) {
            sub = Transform::translate(Vector3d(q[0], q[1], q[2]));
        } else if (kinds[i] == 1) {
            sub = Transform::scale(q[0], q[1], q[2]);
        } else if (kinds[i] == 2) {
            sub = Transform::rotate(q[0], Vector3d(q[1], q[2], q[3]));
        } else if (kinds[i] == 3) {
            sub = Transform::lookAt(Point3d(q[0], q[1], q[2]), Point3d(q[3], q[4], q[5]), Vector3d(q[6], q[7], q[8]));
        } else {
            double m[4][4];
            for (int k = 0; k < 16; k++) m[k / 4][k % 4] = q[k];
            sub = Transform(m);
        }
        trans = sub * trans;   // spica/sceneparser.cc:168
    }
    for (int k = 0; k < 16; k++) out16[k] = trans.getMat()(k / 4, k % 4);
    return 0;
}

int spo_probe_material(const double *mat, float *rec, char *why, int why_len) {
    LocalBSDF b(mat);
    std::string reason;
    const int rc = spgpu_probe::probeMaterial(b.isect.bsdf(), rec, &reason);
    if (why && why_len > 0) std::snprintf(why, why_len, "%s", reason.c_str());
    return rc;
}

int spo_bsdf_sample(const double *mat, int64_t n, const double *wo, const double *u, double *wi,
                    double *f, double *pdf, int32_t *type) {
    LocalBSDF b(mat);
    // in a fresh thread, so that the hidden generators of the BxDFs start from their seed
    std::thread th([&]() {
        for (int64_t i = 0; i < n; i++) {
            const Vector3d o(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
            Vector3d d(0, 0, 0);
            double p = 0.0;
            BxDFType st = BxDFType::None;
            const Spectrum v = b.isect.bsdf()->sample(o, &d, Point2d(u[2 * i], u[2 * i + 1]), &p,
                                                      BxDFType::All, &st);
            wi[3 * i] = d.x();
            wi[3 * i + 1] = d.y();
            wi[3 * i + 2] = d.z();
            f[3 * i] = v.red();
            f[3 * i + 1] = v.green();
            f[3 * i + 2] = v.blue();
            pdf[i] = p;
            type[i] = static_cast<int32_t>(st);
        }
    });
    th.join();
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------- film output
namespace {
// Film::save's resolve (core/film.cc:25-28) of a W x H film of float4 (sum, weight)
Image resolveFilm(const float *film, int W, int H) {
    Image img(W, H);
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const float *f = film + 4 * (static_cast<size_t>(y) * W + x);
            img.pixel(x, y) = RGBSpectrum(f[0], f[1], f[2]);
            img.pixel(x, y) /= (static_cast<double>(f[3]) + EPS);
        }
    return img;
}
}  // namespace

extern "C" {
int spo_film_save_hdr(const float *film, int W, int H, const char *path) {
    resolveFilm(film, W, H).save(path);   // Image::save -> saveHdr (core/image.cc:199,390)
    return 0;
}

int spo_film_gamma(const float *film, int W, int H, double gamma, uint8_t *out) {
    const Image g = GammaTmo(gamma).apply(resolveFilm(film, W, H));
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const RGBSpectrum &c = g(x, y);
            const double v[3] = {c.red(), c.green(), c.blue()};
            for (int k = 0; k < 3; k++) {   // Image::toByte (core/image.cc:476)
                const double d = std::max(0.0, std::min(v[k], 1.0));
                out[3 * (static_cast<size_t>(y) * W + x) + k] = static_cast<uint8_t>(255.0 * d);
            }
        }
    return 0;
}

namespace {
void copyImage(const Image &r, int W, int H, double *out) {
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const RGBSpectrum &c = r(x, y);
            double *o = out + 3 * (static_cast<size_t>(y) * W + x);
            o[0] = c.red();
            o[1] = c.green();
            o[2] = c.blue();
        }
}
}  // namespace

int spo_film_reinhard(const float *film, int W, int H, double alpha, double *out) {
    copyImage(ReinhardTmo(alpha).apply(resolveFilm(film, W, H)), W, H, out);
    return 0;
}

int spo_film_drago(const float *film, int W, int H, double p, double *out) {
    copyImage(DragoTmo(100.0, p).apply(resolveFilm(film, W, H)), W, H, out);
    return 0;
}

int spo_film_durand(const float *film, int W, int H, double contrast, double *out) {
    copyImage(DurandTMO(0.02, 0.4, contrast).apply(resolveFilm(film, W, H)), W, H, out);
    return 0;
}
}  // extern "C"
