// ctx.cuh -- the library context behind spgpu_ctx: scene, lights, environment map,
// BVH and the renderer's queues, all resident in device memory.
#pragma once

#include <cstdint>
#include <exception>
#include <mutex>
#include <new>
#include <string>

#include <nvtx3/nvToolsExt.h>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/spica_gpu.h"
#include "bvh.cuh"
#include "common.cuh"

namespace spgpu {

// Area light record (one per emitting triangle, in triangle order, like the
// reference's per-triangle AreaLight list): 5 x float4.
struct alignas(16) LightRecord {
    float4 p0;     // xyz vertex 0, w = area
    float4 e1;     // xyz p1 - p0
    float4 e2;     // xyz p2 - p0
    float4 n;      // xyz unit face normal (one-sided emission side)
    float4 L;      // xyz emitted radiance
};

// Environment map: level-0 texels for lookups plus the sampling distribution of
// Envmap::Envmap (lights/envmap.cc:17-47) -- conditional rows and the marginal.
struct DeviceEnv {
    int w = 0, h = 0;
    float4 *tex = nullptr;        // [h*w] radiance
    float *condCdf = nullptr;     // [h*(w+1)]
    float *condFunc = nullptr;    // [h*w]
    float *margCdf = nullptr;     // [h+1]
    float *margFunc = nullptr;    // [h]  (= row integrals)
    int *condGuide = nullptr;     // [h*(w+1)] guide tables of the rows (sample1DGuided)
    int *margGuide = nullptr;     // [h+1]
    float margIntegral = 0.0f;
    float3 center{0, 0, 0};
    float radius = 0.0f;
};

// Everything the wavefront kernels read about the scene, passed by value.
struct SceneView {
    const WideNode *nodes;
    const TriRecord *tris;
    const int2 *slotShade;        // (material, light) per leaf slot
    uint32_t nNodes, nTris;
    const MaterialRecord *mats;
    const LightRecord *lights;
    int lightBase;                // first area light of this scene in `lights`
    int nArea;                    // area lights
    int nLights;                  // nArea + (env ? 1 : 0)
    int hasEnv;
    DeviceEnv env;
};

// Per-pass queues of the wavefront renderer (sized for one path per pixel).
struct RenderQueues {
    int64_t capacity = 0;         // paths per pass
    int maxDepth = 0;
    float4 *pathBeta = nullptr;   // [cap] beta.rgb, w = specular flag
    float4 *rayO[2] = {nullptr, nullptr};   // [cap] origin, w = path id bits
    float4 *rayD[2] = {nullptr, nullptr};   // [cap] direction, w = tmax
    HitRecord *hits = nullptr;    // [cap]
    // training-sample collection (lazy): radiance gathered per path, record count and
    // records per path (kCollectRecs x 7 float4 per path, wavefront.cu)
    float4 *pathL = nullptr;
    int *recCount = nullptr;
    float4 *recs = nullptr;
    int *classQ = nullptr;        // [3*cap] ray indices per material class
    float4 *shO = nullptr;        // [2*cap] origin, w = film pixel bits
    float4 *shD = nullptr;        // [2*cap] direction, w = tmax
    float4 *shL = nullptr;        // [2*cap] contribution
    int *counters = nullptr;      // [(maxDepth+2) * 8]
    unsigned long long *stats = nullptr;   // [4] paths, closest rays, shadow rays, spare
    int *err = nullptr;           // [1] kernel error flags
    cudaGraphExec_t graph = nullptr;   // the pass graph last used
    uint64_t graphKey[4] = {0, 0, 0, 0};
    cudaGraphExec_t graphAlt = nullptr;   // the one used before it (guided passes alternate
    uint64_t graphKeyAlt[4] = {0, 0, 0, 0};   // with collection passes)
};

// The streaming wavefront's path pool (stream.cu): a fixed number of path slots,
// refilled with new camera paths as paths end.
struct StreamQueues {
    static constexpr int kEvents = 4;
    int capacity = 0;                                      // path slots
    float4 *rO = nullptr, *rD = nullptr, *rB = nullptr;   // [cap] the pool
    float4 *qO = nullptr, *qD = nullptr, *qB = nullptr, *qH = nullptr;   // [3 * cap] class queues
    float4 *shO = nullptr, *shD = nullptr, *shL = nullptr;               // [2 * cap] shadow queue
    int *ctr = nullptr;                                    // per-iteration counters
    unsigned long long *big = nullptr;                     // paths started, statistics
    int *doneHost = nullptr;                               // pinned: done flags read back per replay
    cudaEvent_t doneEv[kEvents] = {};
    cudaGraphExec_t graph = nullptr;                       // kIterPerGraph iterations
    uint64_t graphKey = 0;
};
void freeStreamQueues(StreamQueues *q);

struct BatchState;
void freeBatch(BatchState *B);
struct GuideState;
void freeGuide(GuideState *G);

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    // scene
    int ntri = 0;
    float *verts = nullptr;
    int *triMat = nullptr;
    int *triLight = nullptr;
    int nmat = 0;
    MaterialRecord *mats = nullptr;
    int nArea = 0;
    LightRecord *lights = nullptr;
    bool hasEnv = false;
    DeviceEnv env;
    bool sceneReady = false;
    // accelerator
    DeviceBVH bvh;
    bool bvhReady = false;
    double buildMs = 0.0;
    // ray-batch scratch
    int *traceErr = nullptr;
    unsigned long long *traceStats = nullptr;
    // spgpu_trace_host: calls on one context from several host threads (the reference
    // calls Accelerator::intersect from every render thread) take this lock, because they
    // share traceErr, the ray counter behind it and the staging buffer below
    std::mutex hostTraceMu;
    unsigned char *hostStage = nullptr;   // rays in, hits out; grown on demand, kept
    size_t hostStageBytes = 0;
    // renderer
    // Render pass lanes: consecutive sample passes alternate between kPassLanes queue
    // sets (each with its own pass graph), lane k > 0 on laneStream[k - 1], so one
    // pass's latency-bound last bounces overlap the next pass's first ones.
    static constexpr int kPassLanes = 8;   // most lanes a context can use
    int passLanes = kPassLanes;            // lanes in use (spgpu_config::pass_lanes)
    // spgpu_render's streaming wavefront (the default); the pass-by-pass wavefront with
    // pass lanes below serves guided passes and spgpu_config.wavefront = 1
#ifndef SPGPU_STREAM_SLOTS_LOG2
#define SPGPU_STREAM_SLOTS_LOG2 23
#endif
#ifndef SPGPU_POOL_LANES
#define SPGPU_POOL_LANES 2
#endif
    // path slots of one streaming pool; pools in flight at once, each on its own stream
    // rendering its share of the samples, so that one pool's latency-bound kernel tails
    // overlap the other's work
    static constexpr int kStreamSlots = 1 << SPGPU_STREAM_SLOTS_LOG2;
    static constexpr int kPoolLanes = SPGPU_POOL_LANES;
    StreamQueues sq[kPoolLanes];
    int wavefront = 0;                             // spgpu_config.wavefront
    RenderQueues rq;                          // lane 0 (also the profiling pass)
    RenderQueues rqLane[kPassLanes - 1];      // lanes 1..
    cudaStream_t laneStream[kPassLanes - 1] = {};
    cudaEvent_t laneFork = nullptr, laneJoin[kPassLanes - 1] = {};
    // batched renders (spgpu_batch_prepare / spgpu_batch_run)
    BatchState *batch = nullptr;
    // learned guiding (spgpu_guiding_*)
    GuideState *guide = nullptr;

    SceneView view() const {
        SceneView v;
        v.nodes = bvh.nodes;
        v.tris = bvh.tris;
        v.slotShade = bvh.slot_shade;
        v.nNodes = static_cast<uint32_t>(bvh.n_nodes);
        v.nTris = static_cast<uint32_t>(bvh.ntri);
        v.mats = mats;
        v.lights = lights;
        v.lightBase = 0;
        v.nArea = nArea;
        v.nLights = nArea + (hasEnv ? 1 : 0);
        v.hasEnv = hasEnv ? 1 : 0;
        v.env = env;
        return v;
    }
};

// NVTX range over a host API call (visible in Nsight Systems timelines; a no-op
// without a profiler attached)
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

void setError(const std::string &msg);
int cudaFail(const char *what, cudaError_t e);

// Runs the body of a C entry point so that no C++ exception crosses the C ABI: a failed
// host allocation becomes SPGPU_ENOMEM, any other exception SPGPU_EINVAL, each with a
// message.
template <class F>
int guarded(const char *name, F &&body) noexcept {
    try {
        return body();
    } catch (const std::bad_alloc &) {
        setError(std::string(name) + ": out of host memory");
        return SPGPU_ENOMEM;
    } catch (const std::exception &e) {
        setError(std::string(name) + ": " + e.what());
        return SPGPU_EINVAL;
    }
}

// C-ABI material records (SPGPU_MAT_*, 8 floats each) as device records; `who` names
// the entry point in error messages
int materialRecords(const char *who, const float *materials, int nmat, std::vector<MaterialRecord> *out);
void freeRenderQueues(RenderQueues *q);

// camera matrices of the reference's PerspectiveCamera, computed in double on the
// host and rounded once: raster -> camera (4x4, projective) and camera -> world.
struct CameraView {
    float r2c[16];
    float c2w[12];
};
CameraView makeCamera(const float *camera, int width, int height);

// One render of a batch: its camera, film, samples, and where its scene sits in the
// batch's merged tree, light and film arrays
struct RenderMeta {
    CameraView cam;
    int W, H, spp, maxDepth;
    uint32_t seed;
    uint32_t root;        // its tree's root node in the merged node array
    int lightBase, nArea;
    int64_t filmOffset;   // in pixels
};

// stream.cu: a batch on the streaming wavefront -- one path sequence over all renders
// (render after render, sample after sample), traced by pools of path slots whose
// iteration loop runs on the device (a CUDA graph with a conditional while node), so a
// run is one graph launch
struct StreamBatch;
int streamBatchCreate(Ctx &C, StreamBatch **slot, const SceneView &merged, const std::vector<RenderMeta> &renders,
                      int poolSlots, int lanes, int iterations);
int streamBatchRun(Ctx &C, StreamBatch &SB, float4 *film, double *renderMs, unsigned long long *statsOut,
                   float *msOut, cudaStream_t stream);
int streamBatchProfile(Ctx &C, StreamBatch &SB, float4 *film, double *kernelMs, long long *launches,
                       unsigned long long *statsOut, unsigned long long *visitOut, cudaStream_t stream);
void freeStreamBatch(StreamBatch *SB);

// learned-guiding state that a guided wavefront pass reads (guide.cu fills it)
struct GuideView {
    const uint8_t *packFwd;   // packed bf16 forward weights
    const float *biasPad;     // biases
    float alpha;              // BSDF share of the one-sample proposal
    bool collect;             // record training samples into the ring
    float *ring;              // training-sample ring, 16 floats per entry
    int capacity;
    int *ringCtl;             // [0] entries written (monotonic)
    int guidedBounces;        // bounces 0 .. guidedBounces-1 sample the network (0: all but the last)
};

// guide.cu: grid of a persistent kernel that runs the network per 128-thread CTA
// (kTileSmem bytes of dynamic shared memory, 64 TMEM columns): SMs x CTAs that fit one
// SM; sets the kernel's shared-memory carveout (call before stream capture)
int guideTileKernelGrid(const void *kernel, int device, int dynSmem = 0);

// wavefront.cu: trace desc->spp samples per pixel into film (device, float4 per pixel);
// with gv, diffuse hits sample the learned guiding proposal (path integrator only)
int renderFrame(Ctx *ctx, const float *camera, int width, int height, int spp, int sampleOffset, int maxDepth,
                uint32_t seed, int integrator, float4 *film, unsigned long long *statsOut, float *msOut,
                cudaStream_t stream, const GuideView *gv = nullptr);
// stream.cu: the same render on the streaming wavefront (path pool refilled as paths end);
// with gv, guided (never collecting) passes
int renderStream(Ctx *ctx, const float *camera, int W, int H, int spp, int sampleOffset, int maxDepth, uint32_t seed,
                 int integrator, float4 *film, unsigned long long *statsOut, float *msOut, cudaStream_t stream,
                 const GuideView *gv = nullptr);
int renderStreamProfile(Ctx *ctx, const float *camera, int W, int H, int spp, int sampleOffset, int maxDepth,
                        uint32_t seed, int integrator, float4 *film, double *kernelMs, long long *launches,
                        unsigned long long *statsOut, unsigned long long *visitOut, cudaStream_t stream,
                        const GuideView *gv = nullptr);
// the same samples launched kernel by kernel (no graph), each timed by events, then
// again with BVH visit counters; kernelMs/launches per kernel class
int renderProfile(Ctx *ctx, const float *camera, int W, int H, int spp, int sampleOffset, int maxDepth, uint32_t seed,
                  int integrator, float4 *film, double *kernelMs, long long *launches, unsigned long long *statsOut,
                  unsigned long long *visitOut, cudaStream_t stream);

}  // namespace spgpu

// the opaque handle of include/spica_gpu.h
struct spgpu_ctx {
    spgpu::Ctx c;
};

namespace spgpu {
struct BatchState;
int batchPrepare(spgpu_ctx *self, BatchState **slot, int count, const spgpu_batch_item *items, int autotune,
                 spgpu_batch_tuning *tuning);
int batchRun(Ctx &C, BatchState &B, float4 *film, double *renderMs, unsigned long long *statsOut, float *msOut,
             cudaStream_t stream);
int batchProfile(Ctx &C, BatchState &B, float4 *film, double *kernelMs, long long *launches,
                 unsigned long long *statsOut, unsigned long long *visitOut, cudaStream_t stream);
int64_t batchPixels(const BatchState &B);
int guideInit(Ctx &C, GuideState **slot, const spgpu_guiding_config *cfg);
int guideParams(Ctx &C, GuideState &G, float *host, int set);
int guideForward(Ctx &C, GuideState &G, const float *feat, int n, float *out, cudaStream_t s);
int guideGrad(Ctx &C, GuideState &G, const float *samples, int n, float *gradOut, double *loss, cudaStream_t s);
int guideTrain(Ctx &C, GuideState &G, int steps, double *meanLoss);
int guideRing(const GuideState &G, float *dst, int maxSamples, int *count);
int guideRender(Ctx &C, GuideState *G, const spgpu_render_desc *d, float4 *film, int flags,
                unsigned long long *statsOut, float *msOut, cudaStream_t s);
long long guideSamples(const GuideState &G);

// film output (film.cu)
int filmResolve(Ctx &C, const float *film, int W, int H, int format, double param, void *out, cudaStream_t s);
int writeHdr(const char *path, const uint8_t *rgbe, int W, int H);
int writePng(const char *path, const uint8_t *rgb, int W, int H);
}  // namespace spgpu
