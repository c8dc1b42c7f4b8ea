/* spica_gpu.h -- C ABI of the GB300 path-tracing library (libspica_gpu.so).
 *
 * This is the drop-in boundary for the reference renderer's hot path.  Plain C:
 * pointers, sizes and status codes only.  Every call returns 0 on success or a
 * negative status; spgpu_last_error() gives the message of the last failure on the
 * calling thread (the reference aborts through Assertion/FatalError instead,
 * core/common.h:69-115; a C++ plugin wrapper turns a negative status into FatalError).
 *
 * One context = one device + one scene + its BVH.  A context is used by one host
 * thread at a time, except spgpu_trace_host, which any number of host threads may call
 * on one context at once (the calls are serialised inside).  "device pointer" arguments are CUDA device memory (for example
 * a torch tensor's data_ptr); "host" entry points take host memory and copy both
 * ways themselves.  `stream` is a cudaStream_t passed as void*; NULL is CUDA's
 * legacy default stream (the one torch uses unless told otherwise).
 */
#ifndef SPICA_GPU_H
#define SPICA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct spgpu_ctx spgpu_ctx;

/* status codes */
#define SPGPU_OK 0
#define SPGPU_EINVAL (-1)     /* bad argument */
#define SPGPU_EBUILD (-2)     /* BVH build failed (see message) */
#define SPGPU_ECUDA (-3)      /* CUDA runtime error */
#define SPGPU_ENOMEM (-4)     /* device allocation failed */
#define SPGPU_ESTATE (-5)     /* call order: no scene / no BVH yet */
#define SPGPU_EKERNEL (-6)    /* a kernel reported an error (stack overflow, bounded wait expired) */

/* material records: 8 floats, [0] = type; the same records the reference's
 * Diffuse, RoughConductor ("ggx", no roughness remap) and Dielectric plugins take
 * (bsdfs/diffuse.cc:23, bsdfs/roughconductor.cc:38, bsdfs/dielectric.cc:30) */
#define SPGPU_MAT_LAMBERT 0    /* [1..3] reflectance */
#define SPGPU_MAT_CONDUCTOR 1  /* [1] alpha, [2..4] eta, [5..7] k */
#define SPGPU_MAT_DIELECTRIC 2 /* [1] interior IOR */
#define SPGPU_MAT_ROUGH_DIELECTRIC 3 /* [1] alpha, [2] interior IOR, [3] 0 Beckmann / 1 GGX
                                        (bsdfs/roughdielectric.cc, white Kr / Kt) */
#define SPGPU_MAT_PLASTIC 4    /* [1..3] Kd, [4..6] Ks, [7] IOR (bsdfs/plastic.cc) */
#define SPGPU_MAT_CONDUCTOR_BECKMANN 5 /* as SPGPU_MAT_CONDUCTOR with the Beckmann distribution
                                          (bsdfs/roughconductor.cc, distribution "beckmann") */

typedef struct {
    int device;          /* CUDA device ordinal */
    int pass_lanes;      /* pass-by-pass wavefront (wavefront = 1) and guided passes: sample
                            passes in flight at once, each with its own wavefront queues
                            (~200 bytes per pixel) and stream; 0 = 8, at most 8 */
    int wavefront;       /* spgpu_render: 0 = streaming (default): two pools of 2^23 path
                            slots (~2.8 GB each) refilled with new camera paths as paths
                            end, each rendering half of the samples on its own stream;
                            1 = pass by pass: one sample per pixel at a time, in pass lanes.
                            Both draw the same samples; films agree up to the order of
                            floating-point additions */
    int reserved[5];
} spgpu_config;

typedef struct {
    int64_t triangles;
    int64_t wide_nodes;
    int32_t depth;       /* wide-node levels */
    int32_t lights;      /* area-light triangles + environment map */
    double build_ms;     /* last spgpu_build_bvh, device time */
    float bounds[6];     /* scene box lo.xyz, hi.xyz */
} spgpu_bvh_info;

/* Closest-hit result, 16 bytes: t along the unit direction, primitive index
 * (-1 = miss), barycentrics u, v of the reference's Moller-Trumbore test
 * (core/triangle.cc:98). */
typedef struct {
    float t;
    int32_t prim;
    float u, v;
} spgpu_hit;

/* Traversal counters of the last spgpu_trace_stats call: mean nodes and triangles
 * visited per ray (used for the roofline's algorithmic bytes). */
typedef struct {
    int64_t rays;
    double nodes_per_ray;
    double tris_per_ray;
} spgpu_trace_counters;

/* Render request.  camera = eye[3], look[3], up[3], vertical fov in degrees: the
 * reference's PerspectiveCamera with Transform::lookAt (cameras/perspective.cc:36,
 * core/transform.cc:167).  Samples sample_offset .. sample_offset+spp-1 of every
 * pixel are traced; the film is accumulated, not cleared. */
typedef struct {
    float camera[10];
    int32_t width, height;
    int32_t spp;
    int32_t sample_offset;
    int32_t max_depth;   /* the reference's "maxDepth" render parameter */
    uint32_t seed;
    int32_t integrator;  /* SPGPU_INTEGRATOR_PATH (0) or SPGPU_INTEGRATOR_DIRECT (1) */
    int32_t reserved[3];
} spgpu_render_desc;

/* PathIntegrator::Li (integrators/path/path.cc:42) */
#define SPGPU_INTEGRATOR_PATH 0
/* DirectLightingIntegrator::Li (integrators/directlighting/directlighting.cc:21): the
 * camera ray's emission or environment radiance plus one-light NEE with both MIS
 * strategies at its first hit.  Its specular recursion (specularReflect /
 * specularTransmit, core/integrator.cc:112-152) samples only BxDFs whose type is
 * Reflection|Specular or Transmission|Specular alone; none of the three materials has
 * one, so it never recurses and max_depth has no effect.  spgpu_render and
 * spgpu_render_host only; batches and guided renders take the path integrator. */
#define SPGPU_INTEGRATOR_DIRECT 1

typedef struct {
    int64_t paths;             /* camera paths traced */
    int64_t rays_closest;      /* camera + continuation rays */
    int64_t rays_shadow;       /* light-sample and MIS-connection rays (any hit) */
    double ms;                 /* device time of the call */
    int64_t kernel_launches;   /* kernels this library launched for the call (spgpu_render;
                                  0 where not counted) */
} spgpu_render_stats;

/* ---- context ----------------------------------------------------------------- */
/* replaces: PluginManager::createObject / createAccelerator (core/cobject.cc:60,68) */
int spgpu_create(const spgpu_config *cfg, spgpu_ctx **out);
void spgpu_destroy(spgpu_ctx *ctx);
const char *spgpu_last_error(void);
const char *spgpu_version(void);

/* ---- scene (host pointers) ------------------------------------------------------
 * replaces: the primitive vector handed to the accelerator plugin's createInstance
 * (core/cobject.h:66-75) and Scene(accel, lights) (core/scene.h:25-30).
 * verts: ntri*9 floats (p0, p1, p2); tri_mat: material index per triangle;
 * materials: nmat*8 floats; tri_emit: ntri*3 floats (zero = not an emitter, else a
 * one-sided AreaLight, lights/area.cc:29), may be NULL; env: env_w*env_h*3 floats, a
 * lat-long map whose row 0 is the +z pole (lights/envmap.cc:17), may be NULL. */
int spgpu_upload_scene(spgpu_ctx *ctx, int32_t ntri, const float *verts, const int32_t *tri_mat, int32_t nmat,
                       const float *materials, const float *tri_emit, int32_t env_w, int32_t env_h,
                       const float *env);

/* replaces: Accelerator::construct() (core/accelerator.h:35; BVHAccel::construct,
 * accelerators/bvh.cc:139) -- builds the compressed 8-wide BVH on the device. */
int spgpu_build_bvh(spgpu_ctx *ctx);
int spgpu_bvh_stats(spgpu_ctx *ctx, spgpu_bvh_info *out);

/* ---- ray batches ----------------------------------------------------------------
 * replaces: Primitive::intersect(Ray&, SurfaceInteraction*) and intersect(Ray&)
 * of the accelerator (core/primitive.h:22-23; BVHAccel::intersect,
 * accelerators/bvh.cc:315-329) for n rays at once.
 * org_tmin, dir_tmax: n float4 (16-byte aligned) -- origin + tmin, unit direction +
 * tmax (the reference's ray.maxDist).  Closest: out = n spgpu_hit.  Any: out = n
 * uint32 (1 = occluded). */
int spgpu_trace(spgpu_ctx *ctx, int any_hit, const float *org_tmin, const float *dir_tmax, int64_t n, void *out,
                void *stream);                                                       /* device pointers */
/* host pointers; blocking.  Safe to call from several host threads on one context, as
 * the reference calls Accelerator::intersect from every render thread
 * (core/integrator.cc:77): the calls queue on a per-context lock.  Rays and hits are
 * staged in a per-context device buffer, allocated on the first call and regrown only
 * when a larger batch arrives. */
int spgpu_trace_host(spgpu_ctx *ctx, int any_hit, const float *org_tmin, const float *dir_tmax, int64_t n,
                     void *out);
/* spgpu_trace_host without any device allocation (no counterpart in the reference).
 * spgpu_trace_host allocates its device staging buffer on a context's first call and
 * again whenever a larger batch arrives; this variant stages rays and hits instead in a static device array
 * reserved with the library on each device (3 MiB + 256 bytes), so it suits callers whose
 * device memory is fully held by their own allocator or arena, or that must not grow
 * or trim a memory pool in a latency-critical loop.
 * Limit: at most 65,536 rays per call; larger n returns SPGPU_EINVAL (split the batch).
 * The first call on a device looks up the scratch address (set-up); make that first
 * call before any stream capture.  The scratch is shared by every context on the
 * device: calls that overlap in time (other threads, other contexts) race on it.
 * Blocking, like spgpu_trace_host; same arguments and results. */
int spgpu_trace_host_noalloc(spgpu_ctx *ctx, int any_hit, const float *org_tmin, const float *dir_tmax, int64_t n,
                             void *out);
/* same as spgpu_trace on device pointers, counting node and triangle visits */
int spgpu_trace_stats(spgpu_ctx *ctx, int any_hit, const float *org_tmin, const float *dir_tmax, int64_t n,
                      void *out, spgpu_trace_counters *counters);

/* ---- BSDFs and the sampler, one function at a time ------------------------------
 * The device functions that shade every hit of spgpu_render, evaluated on caller-given
 * directions and random numbers.  Host pointers; blocking; the context supplies the
 * device and stream only (no scene needed).
 *
 * replaces: BSDF::f, BSDF::pdf and BSDF::sample (core/bsdf.cc:49-136) of one material
 * (an 8-float SPGPU_MAT_* record, as in spgpu_upload_scene), with directions in the
 * shading frame: z = shading normal (the reference's BSDF with normal z, tangent x,
 * binormal y, where world and local directions coincide).
 * eval:   wo, wi: n x 3  ->  f: n x 3, pdf: n.  For the smooth dielectric, pdf is
 *         FresnelSpecular::pdf (core/bxdf.cc:236: F or 1 - F within the 1e-4 cones about
 *         the mirror and refracted directions).
 * sample: wo: n x 3, u: n x 3 -- u[0], u[1] the 2D sample of BSDF::sample and u[2] the
 *         draw the reference takes from its BxDFs' own generator (core/bxdf.cc:18 for the
 *         rough dielectric's reflect-or-refract choice, bsdfs/plastic.cc:18 for the
 *         plastic's specular-or-diffuse choice; unused by the other materials)
 *         ->  wi: n x 3, f: n x 3, pdf: n, type: n (BxDFType bits of the sample:
 *         1 reflection, 2 transmission, 4 diffuse, 8 glossy, 16 specular; 0 and pdf 0
 *         when BSDF::sample finds none, wi then undefined). */
int spgpu_bsdf_eval(spgpu_ctx *ctx, const float *material, int64_t n, const float *wo, const float *wi, float *f,
                    float *pdf);
int spgpu_bsdf_sample(spgpu_ctx *ctx, const float *material, int64_t n, const float *wo, const float *u, float *wi,
                      float *f, float *pdf, int32_t *type);
/* replaces: the random-number stream behind Sampler::get1D / get2D (core/sampler.h:28-36;
 * samplers/independent.cc:6-23 over core/random.cc's MT19937).  The renderer draws its
 * numbers from Philox4x32-10 (Salmon, Moraes, Dror and Shaw, SC 2011) instead, keyed by
 * (seed, film pixel index) and counted by (sample index, bounce -- 0xFFFF for the camera
 * ray --, stream, 0x5350); each block gives four uniforms in [0, 1) from the top 24 bits
 * of each word.  This entry point runs that generator on the device for n arbitrary
 * counters (n x 4 words) and keys (n x 2 words): raw: n x 4 words, u: n x 4 uniforms. */
int spgpu_sampler_generate(spgpu_ctx *ctx, int64_t n, const uint32_t *counter, const uint32_t *key, uint32_t *raw,
                           float *u);

/* ---- rendering -------------------------------------------------------------------
 * replaces: Integrator::render(camera, scene, params) of the path integrator plugin
 * (core/integrator.h:34; SamplerIntegrator::render, core/integrator.cc:46, with
 * PathIntegrator::Li, integrators/path/path.cc:42).
 * film: width*height float4 (sum r, g, b, sample count) in the reference film's
 * pixel order (x mirrored, core/integrator.cc:88); accumulated in place. */
int spgpu_render(spgpu_ctx *ctx, const spgpu_render_desc *desc, float *film, spgpu_render_stats *stats,
                 void *stream);                                                      /* device film */
int spgpu_render_host(spgpu_ctx *ctx, const spgpu_render_desc *desc, float *film,
                      spgpu_render_stats *stats);                                    /* host film   */

/* ---- batched renders ---------------------------------------------------------------
 * replaces: a sequence of Integrator::render calls on many small scenes
 * (core/integrator.cc:46), one per scene.  A batch is prepared once (scenes uploaded,
 * one BVH each, merged) and then traced by spgpu_batch_run as ONE launch of a CUDA
 * graph, by one of two engines:
 *   SPGPU_BATCH_STREAM      the streaming wavefront over all renders of the batch: pools
 *                           of path slots refilled from one path sequence (render after
 *                           render), whose iteration loop runs on the device inside the
 *                           graph (a conditional while node); at most 2^22 - 1 renders;
 *   SPGPU_BATCH_PERSISTENT  one persistent megakernel pulling (render, pixel tile,
 *                           sample chunk) work items, each thread tracing whole paths.
 * autotune: 0 takes the streaming wavefront with its default pool (or, when `tuning` is
 * given with pool_slots > 0 on input, with pool_slots slots in each of pool_lanes
 * pools); 1 times every
 * candidate of both engines (pool slots and lanes; block, tile and chunk) on a copy of
 * the batch with 1/16 of the samples and keeps the fastest; SPGPU_BATCH_PERSISTENT takes
 * the megakernel with its default shape.  Preparing a batch replaces the context's
 * scene (the last item's scene remains uploaded).  Scenes of a batch have no
 * environment map.  films: device memory of spgpu_batch_film_pixels() float4 pixels
 * (fewer than 2^31), the items' films back to back in item order, each in the
 * reference film's pixel order; accumulated in place.  render_ms[i]: time from the
 * launch's start until the last path of item i ended (streaming) or its last sample
 * was added (persistent). */
#define SPGPU_BATCH_STREAM 1
#define SPGPU_BATCH_PERSISTENT 2
typedef struct {
    int32_t ntri;
    const float *verts;
    const int32_t *tri_mat;
    int32_t nmat;
    const float *materials;
    const float *tri_emit;
    spgpu_render_desc desc;
} spgpu_batch_item;

typedef struct {
    int32_t block;          /* persistent: threads per block */
    int32_t tile_pixels;    /* persistent: pixels per work item */
    int32_t chunk_spp;      /* persistent: samples per pixel per work item */
    int32_t candidates;     /* configurations the autotuner timed */
    double calib_ms;        /* device time spent timing them */
    int32_t engine;         /* SPGPU_BATCH_STREAM or SPGPU_BATCH_PERSISTENT */
    int32_t pool_slots;     /* streaming: path slots per pool */
    int32_t pool_lanes;     /* streaming: pools in flight, each on its own share of the paths */
    int32_t iterations;     /* streaming: wavefront iterations per round of the device loop */
} spgpu_batch_tuning;

int spgpu_batch_prepare(spgpu_ctx *ctx, int32_t count, const spgpu_batch_item *items, int32_t autotune,
                        spgpu_batch_tuning *tuning);
int64_t spgpu_batch_film_pixels(spgpu_ctx *ctx);
int spgpu_batch_run(spgpu_ctx *ctx, float *films, double *render_ms, spgpu_render_stats *stats, void *stream);

/* ---- learned path guiding ---------------------------------------------------------
 * No counterpart in the reference renderer.  A 9 -> 64 -> 64 -> 64 -> 40 MLP (BF16
 * weights, FP32 accumulation, tensor cores) maps (position, normal, outgoing direction)
 * at a Lambertian shading point to an 8-lobe von Mises-Fisher mixture; the path tracer
 * samples directions from the one-sample MIS mixture bsdf_fraction * BSDF +
 * (1 - bsdf_fraction) * network for both the continuation and the BSDF strategy of
 * next-event estimation, which keeps the estimator of PathIntegrator::Li unbiased.
 * Training is online: spgpu_guiding_render with SPGPU_GUIDE_COLLECT records incident-
 * radiance samples gathered by the paths it traces, spgpu_guiding_train runs Adam
 * steps on random batches of them. */
typedef struct {
    float learning_rate;   /* Adam step size (0: 1e-3) */
    float bsdf_fraction;   /* BSDF probability in the sampling mixture (clamped to >= 0.2) */
    int32_t batch;         /* training samples per Adam step (0: 16384) */
    uint32_t seed;         /* weight initialisation */
    int32_t capacity;      /* training-sample ring size (0: 2^21) */
    int32_t fault_injection; /* tests only: SPGPU_GUIDE_FAULT_WAIT makes spgpu_guiding_mlp's
                              * tensor-core completion wait run out (no MMA is issued, so
                              * the barrier is never signalled; the wait is cut to 1024
                              * polls); the call then returns SPGPU_EKERNEL and the context
                              * stays usable.  0 otherwise. */
    int32_t guided_bounces;   /* wavefront guided passes: the network samples at bounces
                                 0 .. guided_bounces - 1 and plain BSDF sampling at the
                                 others; 0 (or negative): at every bounce but the last */
    int32_t reserved[1];
} spgpu_guiding_config;

#define SPGPU_GUIDE_FAULT_WAIT 1

#define SPGPU_GUIDE_GUIDED 1   /* sample with the network mixture */
#define SPGPU_GUIDE_COLLECT 2  /* record training samples */
#define SPGPU_GUIDE_MEGAKERNEL 4 /* trace with the persistent megakernel, which runs the
                                  * network for a whole CTA at every bounce; collection
                                  * passes always do.  Otherwise the wavefront of
                                  * spgpu_render traces, and at each bounce a tensor-core
                                  * kernel runs the network over the compacted queue of
                                  * diffuse hits before they are shaded. */
#define SPGPU_GUIDE_PARAMS 11560

int spgpu_guiding_init(spgpu_ctx *ctx, const spgpu_guiding_config *cfg);
/* desc->spp samples per pixel (flags 0: plain BSDF sampling, the same estimator as
 * spgpu_render; guided rendering needs desc->integrator SPGPU_INTEGRATOR_PATH); film as
 * for spgpu_render (device) */
int spgpu_guiding_render(spgpu_ctx *ctx, const spgpu_render_desc *desc, float *film, int32_t flags,
                         spgpu_render_stats *stats, void *stream);
int spgpu_guiding_train(spgpu_ctx *ctx, int32_t steps, double *mean_loss);
int64_t spgpu_guiding_samples(spgpu_ctx *ctx);   /* training samples recorded so far (mod 2^32) */
/* copy up to max_samples entries of the training ring (host, 16 floats each: features 9,
 * direction 3, weight c, proposal pdf q, 2 unused) into dst; *count = entries copied */
int spgpu_guiding_ring(spgpu_ctx *ctx, float *dst, int32_t max_samples, int32_t *count);
/* parameters, fp32: each layer's weights [out][in] row-major then its bias */
int spgpu_guiding_params(spgpu_ctx *ctx, float *params, int32_t set);
/* network outputs for n feature rows (device: features n*9, raw n*40) */
int spgpu_guiding_mlp(spgpu_ctx *ctx, const float *features, int32_t n, float *raw, void *stream);
/* gradient of the training loss sum_i c_i (-log q(w_i)) / sum_i c_i for n samples of 16
 * floats laid out as the ring's (only features, direction and c are read) (device;
 * grad: 11560 floats) */
int spgpu_guiding_grad(spgpu_ctx *ctx, const float *samples, int32_t n, float *grad, double *loss, void *stream);

/* ---- film output -------------------------------------------------------------
 * Resolve of an accumulated film (device, W*H float4 of sum of L and sample weight,
 * film pixel order) into an output encoding, on the device:
 *   SPGPU_FILM_RGBE         out = W*H*4 bytes: the reference's HDRPixel (R, G, B, E)
 *                           of sum / (weight + 1e-12) -- Film::save (core/film.cc:23-30)
 *                           then Image::saveHdr's per-pixel encoding (core/image.cc:72-88)
 *   SPGPU_FILM_GAMMA_BYTES  out = W*H*3 bytes: GammaTmo(param = gamma) then
 *                           Image::toByte -- LDRFilm::saveImage (films/ldrfilm.cc:25-31,
 *                           core/tmo.cc:53, core/image.cc:476)
 *   SPGPU_FILM_REINHARD     out = W*H*3 floats: ReinhardTmo(param = alpha)::apply of the
 *                           resolved image (core/tmo.cc:81-124)
 *   SPGPU_FILM_DRAGO        out = W*H*3 floats: DragoTmo(Ldmax = 100, param = p)::apply
 *                           (core/tmo.cc:125-159)
 *   SPGPU_FILM_DURAND       out = W*H*3 floats: DurandTMO(sigmaSpace = 0.02, sigmaColor =
 *                           0.4, param = targetContrast)::apply (core/tmo.cc:161-243) with
 *                           the reference's domain-transform bilateral filter
 *                           (core/birateral.cc, 20 iterations)
 * Blocking on `stream`. */
#define SPGPU_FILM_RGBE 0
#define SPGPU_FILM_GAMMA_BYTES 1
#define SPGPU_FILM_REINHARD 2
#define SPGPU_FILM_DRAGO 3
#define SPGPU_FILM_DURAND 4
int spgpu_film_resolve(spgpu_ctx *ctx, const float *film, int32_t width, int32_t height, int32_t format,
                       double param, void *out, void *stream);
/* Host-side writers.  spgpu_write_hdr writes W*H RGBE pixels in the byte layout of the
 * reference's Image::saveHdr (core/image.cc:390-434: Radiance header, per scanline the
 * (2, 2, width) marker and each channel as literal runs of <= 127 bytes);
 * spgpu_write_png writes W*H 8-bit RGB pixels as a PNG (stored deflate blocks; the
 * reference's savePng goes through an image library, core/image.cc:459). */
int spgpu_write_hdr(const char *path, const uint8_t *rgbe, int32_t width, int32_t height);
int spgpu_write_png(const char *path, const uint8_t *rgb, int32_t width, int32_t height);

/* ---- scene files ---------------------------------------------------------------
 * replaces: SceneParser (spica/sceneparser.cc:72-335) with meshio::loadPLY / loadOBJ
 * (core/meshio.cc:76-250), up to the point where it hands the camera, primitives and
 * lights to Integrator::render.  spgpu_scene_load reads a scene file of the reference's
 * XML format into the arrays spgpu_upload_scene takes and the request spgpu_render
 * takes (camera, film size, sampleCount, maxDepth, integrator; seed and sample_offset
 * 0).  Accepted: perspective sensors, hdr / ldr films, the independent sampler, the
 * path and direct-lighting integrators (or the gpupath / gpudirect drop-ins), BSDFs
 * diffuse, roughconductor, dielectric, roughdielectric and plastic with constant
 * parameters, PLY (binary little endian) and OBJ meshes, area emitters and one
 * untransformed .hdr environment map; anything else is SPGPU_EINVAL with the element
 * and the reason in spgpu_last_error().  Free the result with spgpu_scene_free. */
typedef struct {
    int32_t ntri;
    const float *verts;        /* ntri*9 */
    const int32_t *tri_mat;    /* ntri */
    int32_t nmat;
    const float *materials;    /* nmat*8 */
    const float *tri_emit;     /* ntri*3 */
    int32_t env_width, env_height;
    const float *env;          /* env_width*env_height*3, or NULL */
    spgpu_render_desc desc;
    void *internal;            /* owned by the library */
} spgpu_scene_file;
int spgpu_scene_load(const char *path, spgpu_scene_file **out);
void spgpu_scene_free(spgpu_scene_file *scene);
/* Image::loadHdr (core/image.cc:252-385): a Radiance .hdr file (run-length-encoded
 * scanlines) as RGB floats; with rgb NULL only the size is returned */
int spgpu_load_hdr(const char *path, float *rgb, int32_t max_pixels, int32_t *width, int32_t *height);

/* Profiling (no counterpart in the reference, which has only a progress printf,
 * core/integrator.cc:92-96): the same samples as spgpu_render, launched kernel by
 * kernel without the graph and timed with CUDA events on `stream`, then repeated
 * with BVH visit counters.  Kernel classes: 0 raygen, 1 extend (closest hit),
 * 2 shade Lambert, 3 shade GGX conductor, 4 shade dielectric, 5 shadow (any hit),
 * 6 finish.  The film receives both runs' samples. */
typedef struct {
    double kernel_ms[8];
    int64_t launches[8];
    int64_t paths, rays_closest, rays_shadow;
    double closest_nodes_per_ray, closest_tris_per_ray;
    double shadow_nodes_per_ray, shadow_tris_per_ray;
} spgpu_kernel_profile;
int spgpu_render_profile(spgpu_ctx *ctx, const spgpu_render_desc *desc, float *film, spgpu_kernel_profile *out,
                         void *stream);
/* the same for a prepared streaming batch (engine SPGPU_BATCH_STREAM): the batch's
 * wavefront launched kernel by kernel from the host with one pool, timed per kernel
 * class, then again with BVH visit counters; films receive both runs */
int spgpu_batch_profile(spgpu_ctx *ctx, float *films, spgpu_kernel_profile *out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SPICA_GPU_H */
