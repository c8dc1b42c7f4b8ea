// gpubvh.cc -- reference-side accelerator plugin: spica's Accelerator interface
// (core/accelerator.h:23) backed by the GB300 library's C ABI (include/spica_gpu.h).
//
// Built against the reference's own headers and libspica_core, it is a drop-in for
// accelerators/bvh (selected with accelerator="gpubvh" in a scene file): the scene
// parser hands it the primitive vector (spica/sceneparser.cc:91-94) exactly as it
// hands it to BVHAccel.  Single-ray intersect() calls go through the host entry point
// one ray at a time and then let the owning primitive rebuild the SurfaceInteraction
// in double, so callers see the same interaction object as with BVHAccel; batched
// callers should use spgpu_trace on device buffers instead.  The reference calls
// intersect() from every parallel_for thread (core/integrator.cc:77); spgpu_trace_host
// serialises those calls on the context (they share its control words and staging
// buffer), so the plugin is safe under that caller.
#include "core/cobject.h"
#undef SPICA_EXPORT_PLUGIN
#define SPICA_EXPORT_PLUGIN(name, descr)

#include <memory>
#include <stdexcept>
#include <vector>

#include "core/accelerator.h"
#include "core/bounds3d.h"
#include "core/common.h"
#include "core/interaction.h"
#include "core/primitive.h"
#include "core/ray.h"
#include "core/renderparams.h"
#include "core/triangle.h"

#include "spica_gpu.h"

namespace spica {

class GpuBVHAccel : public Accelerator {
public:
    GpuBVHAccel(const std::vector<std::shared_ptr<Primitive>> &prims, RenderParams &params)
        : Accelerator{prims}, device_{params.getInt("gpuDevice", 0, true)} {
        construct();
    }
    ~GpuBVHAccel() override { spgpu_destroy(ctx_); }

    // Accelerator::construct: triangulate every primitive, upload, build on the GPU
    void construct() override {
        std::vector<float> verts;
        owner_.clear();
        for (size_t i = 0; i < primitives_.size(); i++) {
            for (const Triangle &t : primitives_[i]->triangulate()) {
                for (int k = 0; k < 3; k++) {
                    verts.push_back(static_cast<float>(t[k].x()));
                    verts.push_back(static_cast<float>(t[k].y()));
                    verts.push_back(static_cast<float>(t[k].z()));
                    worldBound_.merge(t[k]);
                }
                owner_.push_back(static_cast<int>(i));
            }
        }
        const int n = static_cast<int>(owner_.size());
        std::vector<int32_t> mat(n, 0);
        const float grey[8] = {SPGPU_MAT_LAMBERT, 0.5f, 0.5f, 0.5f, 0, 0, 0, 0};
        spgpu_config cfg = {device_, 0, 0, {0}};
        check(spgpu_create(&cfg, &ctx_));
        check(spgpu_upload_scene(ctx_, n, verts.data(), mat.data(), 1, grey, nullptr, 0, 0, nullptr));
        check(spgpu_build_bvh(ctx_));
    }

    Bounds3d worldBound() const override { return worldBound_; }

    bool intersect(Ray &ray, SurfaceInteraction *isect) const override {
        alignas(16) float o[4] = {(float)ray.org().x(), (float)ray.org().y(), (float)ray.org().z(), 0.0f};
        alignas(16) float d[4] = {(float)ray.dir().x(), (float)ray.dir().y(), (float)ray.dir().z(),
                                  (float)ray.maxDist()};
        alignas(16) spgpu_hit h;
        check(spgpu_trace_host(ctx_, 0, o, d, 1, &h));
        if (h.prim < 0) return false;
        // the owning primitive fills the interaction and shortens ray.maxDist
        // (GeometricPrimitive::intersect, core/primitive.cc:49)
        return primitives_[owner_[h.prim]]->intersect(ray, isect);
    }

    bool intersect(Ray &ray) const override {
        alignas(16) float o[4] = {(float)ray.org().x(), (float)ray.org().y(), (float)ray.org().z(), 0.0f};
        alignas(16) float d[4] = {(float)ray.dir().x(), (float)ray.dir().y(), (float)ray.dir().z(),
                                  (float)ray.maxDist()};
        alignas(16) uint32_t occluded = 0;
        check(spgpu_trace_host(ctx_, 1, o, d, 1, &occluded));
        return occluded != 0;
    }

    std::vector<Triangle> triangulate() const override {
        std::vector<Triangle> out;
        for (const auto &p : primitives_) {
            auto t = p->triangulate();
            out.insert(out.end(), t.begin(), t.end());
        }
        return out;
    }

    spgpu_ctx *context() const { return ctx_; }

private:
    static void check(int rc) {
        if (rc != 0) FatalError("gpubvh: %s", spgpu_last_error());
    }
    int device_;
    spgpu_ctx *ctx_ = nullptr;
    std::vector<int> owner_;
};

}  // namespace spica

extern "C" {
spica::CObject *createInstance(const std::vector<std::shared_ptr<spica::Primitive>> &primitives,
                               spica::RenderParams &params) {
    return (spica::CObject *)(new spica::GpuBVHAccel(primitives, params));
}
const char *getDescription() { return "GB300 compressed 8-wide BVH (device build and traversal)"; }
}
