// batch.cu -- many uneven renders (resolution, spp, scene) in one persistent launch.
//
// The reference renders one scene per Integrator::render call (core/integrator.cc:46).
// Here a batch of small scenes is prepared once -- one wide BVH per scene, merged into
// one node / triangle array with a root per render, materials and lights with per-
// render offsets -- and traced by a persistent kernel that pulls work items
// (render, tile of pixels, chunk of samples) from a global counter.  Each thread traces
// whole paths (extend, shade with the wavefront's shadeHit, shadow rays inline): the
// scenes are small enough that the per-bounce queues of the wavefront would cost more
// than they save.  Random streams, camera rays and the estimator are the wavefront's,
// so a render in a batch gives the same film as spgpu_render up to summation order.
// The launch (counter reset + kernel) is captured in a CUDA graph and replayed.
// Block size, tile size and samples per item are picked by a small autotuner that
// times each candidate on a reduced-spp copy of the batch.
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/spica_gpu.h"
#include "ctx.cuh"
#include "shade.cuh"

namespace spgpu {

struct BatchItem {
    int render;
    int pix0, npix;   // raster pixels [pix0, pix0 + npix)
    int s0, ns;       // samples [s0, s0 + ns)
};

struct BatchState {
    int count = 0;
    WideNode *nodes = nullptr;
    TriRecord *tris = nullptr;
    int2 *slotShade = nullptr;
    MaterialRecord *mats = nullptr;
    LightRecord *lights = nullptr;
    int nNodes = 0, nTris = 0;
    RenderMeta *meta = nullptr;
    std::vector<RenderMeta> hostMeta;
    BatchItem *items = nullptr;
    int nItems = 0;
    int *ctl = nullptr;                  // [0] item counter, [1] error, [2..] remaining items per render
    int *perRender = nullptr;            // items per render of the current item list
    unsigned long long *times = nullptr; // [0] start, [1 + r] done of render r (globaltimer ns)
    unsigned long long *stats = nullptr; // [0] paths, [1] closest rays, [2] shadow rays
    int64_t totalPixels = 0;
    int64_t totalSamples = 0;
    int block = 128, tile = 128, chunk = 4;
    cudaGraphExec_t graph = nullptr;
    float *graphFilm = nullptr;
    // engine: SPGPU_BATCH_STREAM (the streaming wavefront over all renders, stream.cu) or
    // SPGPU_BATCH_PERSISTENT (the megakernel below)
    int engine = SPGPU_BATCH_STREAM;
    StreamBatch *sb = nullptr;
    int poolSlots = 0, poolLanes = 0, iterations = 0;
};

namespace {

constexpr int kMaxBatchBlock = 256;
// resident threads per SM the megakernel is compiled for (0: no bound; the register
// budget is then the compiler's)
#ifndef SPGPU_BATCH_THREADS_PER_SM
#define SPGPU_BATCH_THREADS_PER_SM 1024
#endif
template <int BLOCK>
constexpr int batchMinBlocks() {
    return SPGPU_BATCH_THREADS_PER_SM > 0 ? (SPGPU_BATCH_THREADS_PER_SM + BLOCK - 1) / BLOCK : 1;
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, batchMinBlocks<BLOCK>()) k_batch(SceneView base, const RenderMeta *__restrict__ meta,
                                                 const BatchItem *__restrict__ items, int nItems, float4 *film,
                                                 int *ctl, unsigned long long *times, unsigned long long *stats) {
    __shared__ uint2 stack[kStackShared * BLOCK];
    __shared__ int sItem;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        atomicMin(&times[0], t);
    }
    bool overflow = false;
    uint32_t dummy = 0;
    unsigned long long nClosest = 0, nShadow = 0, nPaths = 0;
    while (true) {
        if (threadIdx.x == 0) sItem = atomicAdd(&ctl[0], 1);
        __syncthreads();
        const int it = sItem;
        __syncthreads();
        if (it >= nItems) break;
        const BatchItem w = items[it];
        const RenderMeta &M = meta[w.render];
        SceneView S = base;
        S.lightBase = M.lightBase;
        S.nArea = M.nArea;
        S.nLights = M.nArea;
        S.hasEnv = 0;
        const int work = w.npix * w.ns;
        for (int k = threadIdx.x; k < work; k += BLOCK) {
            const int pix = w.pix0 + k % w.npix;
            const uint32_t sample = static_cast<uint32_t>(w.s0 + k / w.npix);
            const int y = pix / M.W, x = pix - y * M.W;
            const int fi = y * M.W + (M.W - 1 - x);
            const Rand4 r = rand4(M.seed, static_cast<uint32_t>(fi), sample, 0xFFFFu, 0u);
            float3 o, d;
            spawnCameraRay(M.cam, x, y, r.a, r.b, &o, &d);
            float3 beta = mk(1, 1, 1), L = mk(0, 0, 0);
            bool spec = false;
            for (int b = 0; b <= M.maxDepth; b++) {
                float tmax = kInfT, u, v;
                int slot;
                nClosest++;
                const bool hit = traceWide<false, false>(S.nodes, S.tris, S.nNodes, S.nTris, o, d, 0.0f, tmax, slot,
                                                         u, v, stack + threadIdx.x, BLOCK, &dummy, &dummy,
                                                         &overflow, M.root);
                if (!hit) break;   // no environment light in batched scenes
                HitRecord h;
                h.t = tmax;
                h.prim = slot;
                h.u = u;
                h.v = v;
                ShadeResult R;
                shadeHit(S, h, o, d, beta, spec, b, M.maxDepth, M.seed, static_cast<uint32_t>(fi), sample, fi, R);
                L = L + R.emit;
                if (R.sh0) {
                    nShadow++;
                    float tm = R.s0D.w;
                    if (!traceWide<true, false>(S.nodes, S.tris, S.nNodes, S.nTris, xyz(R.s0O), xyz(R.s0D), 0.0f, tm,
                                                slot, u, v, stack + threadIdx.x, BLOCK, &dummy, &dummy, &overflow,
                                                M.root))
                        L = L + xyz(R.s0L);
                }
                if (R.sh1) {
                    nShadow++;
                    float tm = R.s1D.w;
                    if (!traceWide<true, false>(S.nodes, S.tris, S.nNodes, S.nTris, xyz(R.s1O), xyz(R.s1D), 0.0f, tm,
                                                slot, u, v, stack + threadIdx.x, BLOCK, &dummy, &dummy, &overflow,
                                                M.root))
                        L = L + xyz(R.s1L);
                }
                if (!R.cont) break;
                o = xyz(R.cO);
                d = xyz(R.cD);
                beta = R.beta;
                spec = R.spec;
            }
            nPaths++;
            atomicAdd(&film[M.filmOffset + fi], make_float4(L.x, L.y, L.z, 1.0f));
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicSub(&ctl[2 + w.render], 1) == 1) {
                unsigned long long t;
                asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
                times[1 + w.render] = t;
            }
        }
    }
    if (overflow) atomicOr(&ctl[1], 1);
    atomicAdd(&stats[0], nPaths);
    atomicAdd(&stats[1], nClosest);
    atomicAdd(&stats[2], nShadow);
}

__global__ void k_batch_reset(int count, const int *perRender, int *ctl, unsigned long long *times,
                              unsigned long long *stats) {
    for (int i = threadIdx.x; i < count + 2; i += blockDim.x) ctl[i] = i < 2 ? 0 : perRender[i - 2];
    for (int i = threadIdx.x; i < count + 1; i += blockDim.x) times[i] = i == 0 ? ~0ull : 0ull;
    if (threadIdx.x < 4) stats[threadIdx.x] = 0;
}

template <class T>
int devUpload(T **dst, const std::vector<T> &src) {
    cudaFree(*dst);
    *dst = nullptr;
    if (src.empty()) return 0;
    cudaError_t e = cudaMalloc(dst, sizeof(T) * src.size());
    if (e == cudaSuccess) e = cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? 0 : cudaFail("spgpu_batch_prepare", e);
}

void buildItems(BatchState &B, int tile, int chunk, int sppDiv, std::vector<BatchItem> *out,
                std::vector<int> *perRender) {
    out->clear();
    perRender->assign(B.count, 0);
    for (int r = 0; r < B.count; r++) {
        const RenderMeta &M = B.hostMeta[r];
        const int npix = M.W * M.H;
        const int spp = std::max(1, M.spp / sppDiv);
        for (int s0 = 0; s0 < spp; s0 += chunk)
            for (int p0 = 0; p0 < npix; p0 += tile) {
                out->push_back({r, p0, std::min(tile, npix - p0), s0, std::min(chunk, spp - s0)});
                (*perRender)[r]++;
            }
    }
}

int launchBatch(Ctx &C, BatchState &B, const BatchItem *items, int nItems, float4 *film, cudaStream_t s, int block) {
    SceneView v{};
    v.nodes = B.nodes;
    v.tris = B.tris;
    v.slotShade = B.slotShade;
    v.nNodes = static_cast<uint32_t>(B.nNodes);
    v.nTris = static_cast<uint32_t>(B.nTris);
    v.mats = B.mats;
    v.lights = B.lights;
    int sms = 0, occ = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, C.device);
    if (block == 64) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch<64>, 64, 0);
    else if (block == 256) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch<256>, 256, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch<128>, 128, 0);
    const int grid = sms * std::max(occ, 1);
    if (block == 64) k_batch<64><<<grid, 64, 0, s>>>(v, B.meta, items, nItems, film, B.ctl, B.times, B.stats);
    else if (block == 256) k_batch<256><<<grid, 256, 0, s>>>(v, B.meta, items, nItems, film, B.ctl, B.times, B.stats);
    else k_batch<128><<<grid, 128, 0, s>>>(v, B.meta, items, nItems, film, B.ctl, B.times, B.stats);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : cudaFail("k_batch launch", e);
}

// reset counters for a run over items with perRender item counts (a kernel, so that
// the reset can live in the captured graph)
int resetBatch(BatchState &B, const std::vector<int> &perRender, cudaStream_t s, bool upload) {
    if (upload) {
        int rc = devUpload(&B.perRender, perRender);
        if (rc) return rc;
    }
    k_batch_reset<<<1, 256, 0, s>>>(B.count, B.perRender, B.ctl, B.times, B.stats);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : cudaFail("batch reset", e);
}

}  // namespace

void freeBatch(BatchState *B) {
    if (!B) return;
    freeStreamBatch(B->sb);
    if (B->graph) cudaGraphExecDestroy(B->graph);
    cudaFree(B->nodes);
    cudaFree(B->tris);
    cudaFree(B->slotShade);
    cudaFree(B->mats);
    cudaFree(B->lights);
    cudaFree(B->meta);
    cudaFree(B->items);
    cudaFree(B->ctl);
    cudaFree(B->perRender);
    cudaFree(B->times);
    cudaFree(B->stats);
    delete B;
}

int batchPrepare(spgpu_ctx *self, BatchState **slot, int count, const spgpu_batch_item *items, int autotune,
                 spgpu_batch_tuning *tuning) {
    Ctx &C = self->c;
    freeBatch(*slot);
    *slot = nullptr;
    auto *B = new BatchState();
    B->count = count;
    std::vector<WideNode> nodes;
    std::vector<TriRecord> tris;
    std::vector<int2> shade;
    std::vector<MaterialRecord> mats;
    std::vector<LightRecord> lights;
    int rc = 0;
    for (int r = 0; r < count && rc == 0; r++) {
        const spgpu_batch_item &it = items[r];
        const spgpu_render_desc &d = it.desc;
        if (it.ntri <= 0 || !it.verts || !it.tri_mat || it.nmat <= 0 || !it.materials || d.width <= 0 ||
            d.height <= 0 || d.spp <= 0 || d.max_depth < 0 || d.max_depth > 64 ||
            d.integrator != SPGPU_INTEGRATOR_PATH) {
            setError("spgpu_batch_prepare: invalid item (batches take the path integrator)");
            rc = SPGPU_EINVAL;
            break;
        }
        // one scene at a time through the context's ordinary upload and build
        rc = spgpu_upload_scene(self, it.ntri, it.verts, it.tri_mat, it.nmat, it.materials, it.tri_emit, 0, 0, nullptr);
        if (rc == 0) rc = spgpu_build_bvh(self);
        if (rc) break;
        const int nb = C.bvh.n_nodes, nt = C.bvh.ntri;
        std::vector<WideNode> hn(nb);
        std::vector<TriRecord> ht(nt);
        std::vector<int2> hs(nt);
        std::vector<MaterialRecord> hm(C.nmat);
        std::vector<LightRecord> hl(C.nArea);
        cudaMemcpy(hn.data(), C.bvh.nodes, sizeof(WideNode) * nb, cudaMemcpyDeviceToHost);
        cudaMemcpy(ht.data(), C.bvh.tris, sizeof(TriRecord) * nt, cudaMemcpyDeviceToHost);
        cudaMemcpy(hs.data(), C.bvh.slot_shade, sizeof(int2) * nt, cudaMemcpyDeviceToHost);
        cudaMemcpy(hm.data(), C.mats, sizeof(MaterialRecord) * C.nmat, cudaMemcpyDeviceToHost);
        if (C.nArea) cudaMemcpy(hl.data(), C.lights, sizeof(LightRecord) * C.nArea, cudaMemcpyDeviceToHost);
        const int nodeOff = static_cast<int>(nodes.size()), triOff = static_cast<int>(tris.size());
        const int matOff = static_cast<int>(mats.size()), lightOff = static_cast<int>(lights.size());
        for (auto &n : hn) {
            if (n.imask) n.child_base += nodeOff;
            n.tri_base += triOff;
        }
        for (auto &x : hs) {
            x.x += matOff;
            if (x.y >= 0) x.y += lightOff;
        }
        nodes.insert(nodes.end(), hn.begin(), hn.end());
        tris.insert(tris.end(), ht.begin(), ht.end());
        shade.insert(shade.end(), hs.begin(), hs.end());
        mats.insert(mats.end(), hm.begin(), hm.end());
        lights.insert(lights.end(), hl.begin(), hl.end());
        RenderMeta M;
        M.cam = makeCamera(d.camera, d.width, d.height);
        M.W = d.width;
        M.H = d.height;
        M.spp = d.spp;
        M.maxDepth = d.max_depth;
        M.seed = d.seed;
        M.root = static_cast<uint32_t>(nodeOff);
        M.lightBase = lightOff;
        M.nArea = C.nArea;
        M.filmOffset = B->totalPixels;
        B->totalPixels += static_cast<int64_t>(d.width) * d.height;
        B->totalSamples += static_cast<int64_t>(d.width) * d.height * d.spp;
        B->hostMeta.push_back(M);
    }
    if (rc == 0 && B->totalPixels > INT32_MAX) {
        setError("spgpu_batch_prepare: the batch's films exceed 2^31 pixels");
        rc = SPGPU_EINVAL;
    }
    if (rc == 0) {
        B->nNodes = static_cast<int>(nodes.size());
        B->nTris = static_cast<int>(tris.size());
        if ((rc = devUpload(&B->nodes, nodes)) == 0 && (rc = devUpload(&B->tris, tris)) == 0 &&
            (rc = devUpload(&B->slotShade, shade)) == 0 && (rc = devUpload(&B->mats, mats)) == 0 &&
            (rc = devUpload(&B->lights, lights)) == 0 && (rc = devUpload(&B->meta, B->hostMeta)) == 0) {
            cudaError_t e = cudaMalloc(&B->ctl, sizeof(int) * (2 + count));
            if (e == cudaSuccess) e = cudaMalloc(&B->times, sizeof(unsigned long long) * (1 + count));
            if (e == cudaSuccess) e = cudaMalloc(&B->stats, sizeof(unsigned long long) * 4);
            if (e != cudaSuccess) rc = cudaFail("spgpu_batch_prepare", e);
        }
    }
    // The launch: by default the streaming wavefront with its default pool; with
    // autotune, every candidate of both engines -- pool slots and lanes of the streaming
    // wavefront, (block, tile, chunk) of the persistent megakernel -- is timed on a copy of
    // the batch with 1/16 of the samples, and the fastest is kept
    if (rc == 0) {
        struct Cand {
            int engine, block, tile, chunk, slots, lanes;
        };
        constexpr int kIters = 8;   // wavefront iterations per round of the device loop
        std::vector<Cand> cands;
        if (autotune == SPGPU_BATCH_PERSISTENT) {
            cands.push_back({SPGPU_BATCH_PERSISTENT, 128, 128, 4, 0, 0});
        } else if (autotune) {
            for (int sl : {1 << 20, 1 << 21, 1 << 22})
                for (int ln : {1, 2}) cands.push_back({SPGPU_BATCH_STREAM, 0, 0, 0, sl, ln});
            for (int bl : {64, 128, 256})
                for (int ti : {64, 256})
                    for (int ch : {1, 4, 16}) cands.push_back({SPGPU_BATCH_PERSISTENT, bl, ti, ch, 0, 0});
        } else if (tuning && tuning->pool_slots > 0) {
            cands.push_back({SPGPU_BATCH_STREAM, 0, 0, 0, tuning->pool_slots, tuning->pool_lanes});   // the caller's pool
        } else {
            cands.push_back({SPGPU_BATCH_STREAM, 0, 0, 0, 1 << 22, 2});
        }
        SceneView merged{};
        merged.nodes = B->nodes;
        merged.tris = B->tris;
        merged.slotShade = B->slotShade;
        merged.nNodes = static_cast<uint32_t>(B->nNodes);
        merged.nTris = static_cast<uint32_t>(B->nTris);
        merged.mats = B->mats;
        merged.lights = B->lights;
        std::vector<RenderMeta> reduced = B->hostMeta;
        for (auto &M : reduced) M.spp = std::max(1, M.spp / 16);
        float4 *scratchFilm = nullptr;
        if (cands.size() > 1) {
            cudaError_t e = cudaMalloc(&scratchFilm, sizeof(float4) * std::max<int64_t>(B->totalPixels, 1));
            if (e != cudaSuccess) rc = cudaFail("spgpu_batch_prepare", e);
        }
        BatchItem *dItems = nullptr;
        float best = 3.0e38f;
        Cand bestC = cands[0];
        double calibMs = 0.0;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        for (size_t ci = 0; ci < cands.size() && rc == 0 && cands.size() > 1; ci++) {
            const Cand &c = cands[ci];
            float msBest = 3.0e38f;
            if (c.engine == SPGPU_BATCH_STREAM) {
                StreamBatch *tb = nullptr;
                rc = streamBatchCreate(C, &tb, merged, reduced, c.slots, c.lanes, kIters);
                std::vector<double> rms(reduced.size());
                unsigned long long st[4];
                for (int rep = 0; rep < 2 && rc == 0; rep++) {
                    float ms = 0.0f;
                    rc = streamBatchRun(C, *tb, scratchFilm, rms.data(), st, &ms, C.stream);
                    msBest = std::min(msBest, ms);
                    calibMs += ms;
                }
                freeStreamBatch(tb);
            } else {
                std::vector<BatchItem> its;
                std::vector<int> per;
                buildItems(*B, c.tile, c.chunk, 16, &its, &per);
                cudaFree(dItems);
                dItems = nullptr;
                if ((rc = devUpload(&dItems, its))) break;
                for (int rep = 0; rep < 2 && rc == 0; rep++) {
                    if ((rc = resetBatch(*B, per, C.stream, rep == 0))) break;
                    cudaEventRecord(e0, C.stream);
                    rc = launchBatch(C, *B, dItems, static_cast<int>(its.size()), scratchFilm, C.stream, c.block);
                    cudaEventRecord(e1, C.stream);
                    cudaEventSynchronize(e1);
                    float ms = 0.0f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    msBest = std::min(msBest, ms);
                    calibMs += ms;
                }
            }
            if (msBest < best) {
                best = msBest;
                bestC = c;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(dItems);
        cudaFree(scratchFilm);
        B->engine = bestC.engine;
        if (bestC.engine == SPGPU_BATCH_PERSISTENT) {
            B->block = bestC.block;
            B->tile = bestC.tile;
            B->chunk = bestC.chunk;
        } else {
            B->poolSlots = bestC.slots;
            B->poolLanes = bestC.lanes;
            B->iterations = kIters;
        }
        if (tuning) {
            tuning->engine = bestC.engine;
            tuning->block = bestC.engine == SPGPU_BATCH_PERSISTENT ? bestC.block : 0;
            tuning->tile_pixels = bestC.engine == SPGPU_BATCH_PERSISTENT ? bestC.tile : 0;
            tuning->chunk_spp = bestC.engine == SPGPU_BATCH_PERSISTENT ? bestC.chunk : 0;
            tuning->pool_slots = bestC.slots;
            tuning->pool_lanes = bestC.lanes;
            tuning->iterations = bestC.engine == SPGPU_BATCH_STREAM ? kIters : 0;
            tuning->candidates = static_cast<int32_t>(cands.size());
            tuning->calib_ms = calibMs;
        }
        if (rc == 0 && B->engine == SPGPU_BATCH_STREAM) {
            rc = streamBatchCreate(C, &B->sb, merged, B->hostMeta, B->poolSlots, B->poolLanes, B->iterations);
        } else if (rc == 0) {
            std::vector<BatchItem> its;
            std::vector<int> per;
            buildItems(*B, B->tile, B->chunk, 1, &its, &per);
            B->nItems = static_cast<int>(its.size());
            rc = devUpload(&B->items, its);
        }
    }
    if (rc) {
        freeBatch(B);
        return rc;
    }
    *slot = B;
    return 0;
}

int64_t batchPixels(const BatchState &B) { return B.totalPixels; }

int batchRun(Ctx &C, BatchState &B, float4 *film, double *renderMs, unsigned long long *statsOut, float *msOut,
             cudaStream_t stream) {
    if (B.engine == SPGPU_BATCH_STREAM) return streamBatchRun(C, *B.sb, film, renderMs, statsOut, msOut, stream);
    std::vector<BatchItem> its;
    std::vector<int> per;
    buildItems(B, B.tile, B.chunk, 1, &its, &per);
    // the graph holds the counter reset and the launch; captured once per film pointer
    if (!B.graph || B.graphFilm != reinterpret_cast<float *>(film)) {
        int urc = devUpload(&B.perRender, per);
        if (urc) return urc;
        if (B.graph) cudaGraphExecDestroy(B.graph);
        B.graph = nullptr;
        cudaStream_t cs = C.stream;
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cudaFail("cudaStreamBeginCapture", e);
        int rc = resetBatch(B, per, cs, false);
        if (rc == 0) rc = launchBatch(C, B, B.items, B.nItems, film, cs, B.block);
        e = cudaStreamEndCapture(cs, &g);
        if (rc) return rc;
        if (e != cudaSuccess) return cudaFail("cudaStreamEndCapture", e);
        e = cudaGraphInstantiate(&B.graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cudaFail("cudaGraphInstantiate", e);
        B.graphFilm = reinterpret_cast<float *>(film);
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaError_t e = cudaEventRecord(e0, stream);
    if (e == cudaSuccess) e = cudaGraphLaunch(B.graph, stream);
    if (e == cudaSuccess) e = cudaEventRecord(e1, stream);
    std::vector<unsigned long long> times(1 + B.count);
    unsigned long long st[4] = {0, 0, 0, 0};
    int ctl[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(times.data(), B.times, sizeof(unsigned long long) * times.size(),
                                              cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(st, B.stats, sizeof(st), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctl, B.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    float ms = 0.0f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cudaFail("spgpu_batch_run", e);
    for (int r = 0; r < B.count; r++)
        renderMs[r] = times[1 + r] >= times[0] ? (times[1 + r] - times[0]) * 1.0e-6 : -1.0;
    for (int k = 0; k < 3; k++) statsOut[k] = st[k];
    statsOut[3] = 2;   // counter reset and the persistent kernel
    *msOut = ms;
    if (ctl[1]) {
        setError("spgpu_batch_run: traversal stack overflow");
        return SPGPU_EKERNEL;
    }
    return 0;
}

int batchProfile(Ctx &C, BatchState &B, float4 *film, double *kernelMs, long long *launches,
                 unsigned long long *statsOut, unsigned long long *visitOut, cudaStream_t stream) {
    if (B.engine != SPGPU_BATCH_STREAM || !B.sb) {
        setError("spgpu_batch_profile: the batch runs on the persistent megakernel; profiles cover the streaming "
                 "wavefront");
        return SPGPU_ESTATE;
    }
    return streamBatchProfile(C, *B.sb, film, kernelMs, launches, statsOut, visitOut, stream);
}

}  // namespace spgpu
