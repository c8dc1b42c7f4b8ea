// gpupath.cc -- reference-side integrator plugin: spica's Integrator interface
// (core/integrator.h:29-37) backed by the GB300 wavefront path integrator.
//
// A drop-in for integrators/path (integrator type="gpupath" in a scene file); built a
// second time with -DSPGPU_PLUGIN_DIRECT it is the drop-in for
// integrators/directlighting (type="gpudirect", SPGPU_INTEGRATOR_DIRECT).  It
// overrides render(camera, scene, params) -- the same call SceneParser makes
// (spica/sceneparser.cc:105) -- translates the scene through the reference's public
// interfaces, renders "sampleCount" samples of "maxDepth" bounces on the GPU and
// writes the reference film's pixels (Film::setImage, core/film.cc:60).
//
// Translation uses only public API:
//   geometry   Primitive::triangulate (core/primitive.h:26)
//   materials  Primitive::setScatterFuncs on a unit-frame SurfaceInteraction, then the
//              BSDF's public f / pdf / hasType / eta (core/bsdf.h:20-54), read as one of
//              the GPU's materials by material_probe.h (Lambert, GGX conductor,
//              dielectric, rough dielectric, plastic); any other material is a FatalError
//   lights     Primitive::light() + Light::L for area lights; Light::Le sampled at texel
//              centres (envmapWidth x envmapWidth/2, default 1024) for the environment
//   camera     Camera::cameraToWorld / cameraToScreen (core/camera.h:43-44): eye, view
//              direction, up and vertical field of view
#include "core/cobject.h"
#undef SPICA_EXPORT_PLUGIN
#define SPICA_EXPORT_PLUGIN(name, descr)

#include <cmath>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "core/bsdf.h"
#include "core/bxdf.h"
#include "core/camera.h"
#include "core/common.h"
#include "core/film.h"
#include "core/image.h"
#include "core/integrator.h"
#include "core/interaction.h"
#include "core/light.h"
#include "core/memory.h"
#include "core/primitive.h"
#include "core/ray.h"
#include "core/renderparams.h"
#include "core/sampler.h"
#include "core/scene.h"
#include "core/transform.h"
#include "core/triangle.h"

#include "material_probe.h"
#include "spica_gpu.h"

namespace spica {

class GpuPathIntegrator : public Integrator {
public:
    explicit GpuPathIntegrator(RenderParams &params)
        : device_{params.getInt("gpuDevice", 0, true)},
          passLanes_{params.getInt("gpuPassLanes", 0, true)},
          wavefront_{params.getInt("gpuWavefront", 0, true)},
          seed_{static_cast<uint32_t>(params.getInt("seed", 0, true))} {}

    void render(const std::shared_ptr<const Camera> &camera, const Scene &scene, RenderParams &params) override {
        std::vector<float> verts, mats, emit;
        std::vector<int32_t> triMat;
        std::map<const Material *, int> matIndex;
        for (const auto &prim : scene.primitives()) {
            const int m = materialOf(*prim, &mats, &matIndex);
            Spectrum Le(0.0);
            const auto tris = prim->triangulate();
            for (const Triangle &t : tris) {
                if (const Light *l = prim->light()) {
                    const Vector3d n = Vector3d::cross(t[1] - t[0], t[2] - t[0]).normalized();
                    Le = l->L(Interaction(t[0], Normal3d(n)), n);   // one-sided emission, lights/area.cc:29
                }
                for (int k = 0; k < 3; k++) {
                    verts.push_back((float)t[k].x());
                    verts.push_back((float)t[k].y());
                    verts.push_back((float)t[k].z());
                }
                triMat.push_back(m);
                emit.push_back((float)Le.red());
                emit.push_back((float)Le.green());
                emit.push_back((float)Le.blue());
            }
        }
        std::vector<float> env;
        int ew = 0, eh = 0;
        for (const auto &l : scene.lights()) {
            if (l->type() != LightType::Envmap) continue;
            ew = params.getInt("envmapWidth", 1024, false);
            eh = ew / 2;
            env.resize(static_cast<size_t>(ew) * eh * 3);
            for (int y = 0; y < eh; y++)
                for (int x = 0; x < ew; x++) {   // texel centre -> direction (lights/envmap.cc:130)
                    const double th = PI * (y + 0.5) / eh, ph = 2.0 * PI * (x + 0.5) / ew;
                    const Spectrum L = l->Le(Ray(Point3d(), Vector3d(std::sin(th) * std::cos(ph),
                                                                     std::sin(th) * std::sin(ph), std::cos(th))));
                    float *p = &env[3 * (static_cast<size_t>(y) * ew + x)];
                    p[0] = (float)L.red();
                    p[1] = (float)L.green();
                    p[2] = (float)L.blue();
                }
        }
        spgpu_ctx *ctx = nullptr;
        spgpu_config cfg = {device_, passLanes_, wavefront_, {0}};
        check(spgpu_create(&cfg, &ctx));
        check(spgpu_upload_scene(ctx, static_cast<int32_t>(triMat.size()), verts.data(), triMat.data(),
                                 static_cast<int32_t>(mats.size() / 8), mats.data(), emit.data(), ew, eh,
                                 env.empty() ? nullptr : env.data()));
        check(spgpu_build_bvh(ctx));

        const auto film = camera->film();
        const int W = film->resolution().x(), H = film->resolution().y();
        spgpu_render_desc d = {};
        const Transform &c2w = camera->cameraToWorld();
        const Point3d eye = c2w.apply(Point3d(0.0, 0.0, 0.0));
        const Vector3d dir = c2w.apply(Vector3d(0.0, 0.0, 1.0));
        const Vector3d up = c2w.apply(Vector3d(0.0, 1.0, 0.0));
        const float cam[10] = {(float)eye.x(), (float)eye.y(), (float)eye.z(),
                               (float)(eye.x() + dir.x()), (float)(eye.y() + dir.y()), (float)(eye.z() + dir.z()),
                               (float)up.x(), (float)up.y(), (float)up.z(),
                               (float)(2.0 * std::atan(1.0 / camera->cameraToScreen().getMat()(1, 1)) * 180.0 / PI)};
        for (int i = 0; i < 10; i++) d.camera[i] = cam[i];
        d.width = W;
        d.height = H;
        d.spp = params.getInt("sampleCount");
        d.max_depth = params.getInt("maxDepth");
        d.seed = seed_;
#ifdef SPGPU_PLUGIN_DIRECT
        d.integrator = SPGPU_INTEGRATOR_DIRECT;
#else
        d.integrator = SPGPU_INTEGRATOR_PATH;
#endif
        std::vector<float> pix(static_cast<size_t>(W) * H * 4, 0.0f);
        spgpu_render_stats st;
        check(spgpu_render_host(ctx, &d, pix.data(), &st));
        spgpu_destroy(ctx);
        Image img(W, H);
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                const float *p = &pix[4 * (static_cast<size_t>(y) * W + x)];
                const double w = p[3] > 0.0f ? 1.0 / p[3] : 0.0;
                img.pixel(x, y) = Spectrum(p[0] * w, p[1] * w, p[2] * w);
            }
        film->setImage(img);
        film->save(d.spp);
    }

private:
    static void check(int rc) {
        if (rc != 0) FatalError("gpupath: %s", spgpu_last_error());
    }

    // material record of a primitive, probed through its BSDF in a unit frame
    static int materialOf(const Primitive &prim, std::vector<float> *mats, std::map<const Material *, int> *index) {
        const Material *key = prim.material();
        auto it = index->find(key);
        if (it != index->end()) return it->second;
        MemoryArena arena;
        SurfaceInteraction si(Point3d(0, 0, 0), Point2d(0, 0), Vector3d(0, 0, 1), Vector3d(1, 0, 0),
                              Vector3d(0, 1, 0), Normal3d(), Normal3d(), nullptr);
        prim.setScatterFuncs(&si, arena);
        float rec[8];
        std::string why;
        if (spgpu_probe::probeMaterial(si.bsdf(), rec, &why) != 0) FatalError("gpupath: %s", why.c_str());
        const int m = static_cast<int>(mats->size() / 8);
        mats->insert(mats->end(), rec, rec + 8);
        (*index)[key] = m;
        return m;
    }

    int device_;
    int passLanes_;   // pass-by-pass wavefront: sample passes in flight (spgpu_config::pass_lanes; 0 = default)
    int wavefront_;   // spgpu_config::wavefront: 0 streaming (default), 1 pass by pass
    uint32_t seed_;
};

}  // namespace spica

extern "C" {
spica::CObject *createInstance(spica::RenderParams &params) {
    return (spica::CObject *)(new spica::GpuPathIntegrator(params));
}
#ifdef SPGPU_PLUGIN_DIRECT
const char *getDescription() { return "GB300 wavefront direct-lighting integrator"; }
#else
const char *getDescription() { return "GB300 wavefront path integrator"; }
#endif
}
