/* spo_api.h -- C API shared by the two CPU oracles of this project.
 *
 * TEST INFRASTRUCTURE ONLY.  Two shared libraries implement this header:
 *   oracle/_ref/libspica_ref.so    the reference renderer's own sources, compiled
 *                                  unmodified (oracle/Makefile, target "ref"), driven
 *                                  by oracle/ref_driver.cc;
 *   oracle/_port/libspica_oracle.so this project's C++ restatement of the same path
 *                                  (oracle/spica_oracle.cc), which builds on any host.
 * Only tests, the smoke check and the benchmark's CPU-baseline arm load them; the
 * GPU product path never does.
 *
 * Everything is double precision, like the reference (core/common.h:52-55).
 * Scenes are flat triangle soups: one GeometricPrimitive per triangle, an optional
 * one-sided AreaLight per emitting triangle (sceneparser.cc:168-188 does the same
 * for meshes) and an optional lat-long environment map.
 */
#ifndef SPICA_ORACLE_SPO_API_H
#define SPICA_ORACLE_SPO_API_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* material records: 8 doubles each, [0] = type */
#define SPO_MAT_LAMBERT    0 /* [1..3] reflectance RGB                       (bsdfs/diffuse.cc)        */
#define SPO_MAT_CONDUCTOR  1 /* [1] GGX alpha, [2..4] eta RGB, [5..7] k RGB  (bsdfs/roughconductor.cc) */
#define SPO_MAT_DIELECTRIC 2 /* [1] interior IOR (exterior 1.0), white Kr/Kt (bsdfs/dielectric.cc)    */
#define SPO_MAT_ROUGH_DIELECTRIC 3 /* [1] alpha, [2] interior IOR, [3] 0 Beckmann / 1 GGX, white Kr/Kt
                                     (bsdfs/roughdielectric.cc)                                  */
#define SPO_MAT_PLASTIC    4 /* [1..3] Kd RGB, [4..6] Ks RGB, [7] IOR     (bsdfs/plastic.cc)          */
#define SPO_MAT_CONDUCTOR_BECKMANN 5 /* as SPO_MAT_CONDUCTOR, distribution "beckmann"                  */
#define SPO_MAT_STRIDE     8

typedef struct spo_scene spo_scene;

/* verts: ntri*9 (p0,p1,p2); tri_mat: material index per triangle;
 * tri_emit: ntri*3 emitted radiance (all zero = not a light), may be NULL;
 * env: env_w*env_h*3 floats, row 0 = +z pole (lights/envmap.cc:60-79), may be NULL;
 * use_simd: reference only -- selects its 4-wide QBVH traversal (bvh.cc:389). */
spo_scene *spo_scene_create(int ntri, const double *verts, const int32_t *tri_mat,
                            int nmat, const double *mats, const double *tri_emit,
                            int env_w, int env_h, const float *env, int use_simd);
void spo_scene_destroy(spo_scene *s);
int spo_scene_num_lights(const spo_scene *s);

/* Closest hit (any == 0) or any hit (any != 0) for n rays (org/dir: n*3, tmax: n).
 * Closest: prim[i] = hit triangle or -1, t[i] = hit distance along the normalised
 * direction.  Any: hit[i] = 0/1.  Unused outputs may be NULL. */
int spo_trace(spo_scene *s, int any, int64_t n, const double *org, const double *dir,
              const double *tmax, int32_t *prim, double *t, uint8_t *hit, int nthreads);

/* Render a film-space window [fx0, fx0+w) x [fy0, fy0+h) of a W x H image with the
 * path integrator (integrators/path/path.cc:42).  cam = eye[3], look[3], up[3],
 * vertical fov in degrees.  Each film pixel p = fy*W + fx owns one Independent
 * (MT19937) sampler seeded spo_pixel_seed(seed, p) and draws its spp samples in
 * sequence.  sum/sumsq: h*w*3, per-pixel sum of L and of L^2 over the samples. */
int spo_render(spo_scene *s, const double *cam, int W, int H, int fx0, int fy0, int w,
               int h, int spp, int max_depth, uint32_t seed, double *sum, double *sumsq,
               int nthreads);
/* Same with the direct-lighting integrator
 * (integrators/directlighting/directlighting.cc:21). */
int spo_render_direct(spo_scene *s, const double *cam, int W, int H, int fx0, int fy0, int w,
                      int h, int spp, int max_depth, uint32_t seed, double *sum, double *sumsq,
                      int nthreads);

/* BSDF of one material in its local frame (z = shading normal).
 * eval: f (n*3) and pdf (n) for (wo, wi) pairs (core/bsdf.cc:49,119).
 * sample: wi (n*3), f (n*3), pdf (n), sampled type bits (n) from (wo, u) (core/bsdf.cc:65). */
int spo_bsdf_eval(const double *mat, int64_t n, const double *wo, const double *wi,
                  double *f, double *pdf);
int spo_bsdf_sample(const double *mat, int64_t n, const double *wo, const double *u,
                    double *wi, double *f, double *pdf, int32_t *type);
/* The restatement only: spo_bsdf_sample with the draws of the BxDFs' hidden generators
 * (core/bxdf.cc:18, bsdfs/plastic.cc:18) made visible.  uc_in == NULL: drawn as in
 * spo_bsdf_sample, row i's draw reported in uc_out[i] (NaN if none); else row i uses
 * uc_in[i]. */
int spo_bsdf_sample_uc(const double *mat, int64_t n, const double *wo, const double *u,
                       const double *uc_in, double *wi, double *f, double *pdf, int32_t *type,
                       double *uc_out);

/* Known-answer probes of the geometry primitives, the objects of the reference's own
 * unit tests: Triangle::area (core/triangle.cc; tests/test_geometry.cc:79-84) of the
 * triangle v[0..8]; Bounds3d::intersect (core/bounds3d_detail.h:64-79;
 * tests/test_geometry.cc:119-125) of the box [lo, hi] and the ray (org, dir, tmax),
 * returning 1 on a hit with the entry and exit distances; Ray's inverse direction with
 * INFTY for zero components (core/ray.cc:43-47; tests/test_ray.cc:14-21). */
double spo_triangle_area(const double *v);
int spo_box_intersect(const double *lo, const double *hi, const double *org, const double *dir, double tmax,
                      double *tnear, double *tfar);
void spo_ray_invdir(const double *org, const double *dir, double *inv);

const char *spo_name(void);

/* Film output through the reference (compiled reference only): a W x H film of float4
 * (sum of L, weight) resolved as Film::save does (core/film.cc:25-28), then
 *   spo_film_save_hdr  Image::save to a .hdr path (core/image.cc:390)
 *   spo_film_gamma     GammaTmo(gamma) and Image::toByte: W*H*3 bytes (core/tmo.cc:53)
 *   spo_film_reinhard  ReinhardTmo(alpha)::apply: W*H*3 doubles (core/tmo.cc:81) */
int spo_film_save_hdr(const float *film, int W, int H, const char *path);
int spo_film_gamma(const float *film, int W, int H, double gamma, uint8_t *out);
int spo_film_reinhard(const float *film, int W, int H, double alpha, double *out);
/* DragoTmo(Ldmax 100, bias p)::apply and DurandTMO(sigmaSpace 0.02, sigmaColor 0.4,
 * targetContrast)::apply of the resolved film (core/tmo.cc:135, 171): W*H*3 doubles */
int spo_film_drago(const float *film, int W, int H, double p, double *out);
int spo_film_durand(const float *film, int W, int H, double contrast, double *out);

/* The drop-in integrator plugin's material translation (spica_gb300/plugins/
 * material_probe.h) run on the reference's own BSDF for a material record (compiled
 * reference only): 0 and the spgpu record in rec[0..7], or -1 and the refusal in why. */
int spo_probe_material(const double *mat, float *rec, char *why, int why_len);

/* Scene front-end pieces of the reference (compiled reference only):
 *   spo_load_ply         meshio::loadPLY (core/meshio.cc:76) with the row-major 4x4
 *                        objectToWorld m16: world-space triangles (9 doubles each) of up
 *                        to max_tris into verts, the count into *ntri
 *   spo_transform_chain  the scene parser's composition of <transform> children
 *                        (spica/sceneparser.cc:128-171): for each element, kind 0
 *                        translate(x,y,z), 1 scale(x,y,z), 2 rotate(angle, axis x,y,z),
 *                        3 lookAt(origin, target, up), 4 matrix (16 values), parameters
 *                        16 doubles per element; trans = sub * trans; row-major result */
int spo_load_ply(const char *path, const double *m16, int64_t max_tris, double *verts, int64_t *ntri);
/* Image::load of a .hdr file (core/image.cc:252): RGB doubles, row-major */
int spo_load_hdr(const char *path, int64_t max_pixels, double *rgb, int *width, int *height);
int spo_transform_chain(int n, const int *kinds, const double *params, double *out16);

/* per-pixel sampler seed: splitmix-style mix of (seed, pixel) folded to 32 bits */
static inline uint32_t spo_pixel_seed(uint32_t seed, uint32_t pixel) {
    uint64_t z = ((uint64_t)seed << 32) ^ (uint64_t)pixel;
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (uint32_t)(z ^ (z >> 32));
}

#ifdef __cplusplus
}
#endif
#endif
