/*
 * wr_oracle.h — CPU restatement of WalkRay's unidirectional path-tracing hot
 * path, in plain C.  TEST INFRASTRUCTURE ONLY: tests/, the smoke check and the
 * CPU-baseline legs of bench.py load it as the checker and the timed CPU
 * reference.  The library (walkray_gb300/csrc) never links, calls or falls
 * back to it.
 *
 * Pinning: the tree build and closest-hit traversal are checked bit for bit
 * against WalkRay's own kdtree.cpp/scene.cpp/noself.cpp (compiled unmodified
 * into oracle/_ref by oracle/Makefile) and against committed golden fixtures
 * made from it; the path tracer is checked statistically against the
 * reference's PathTracer::renderPixels.
 *
 * Floating point: every operation is IEEE single precision in the reference's
 * order, built with -ffp-contract=off (no FMA), so that traversal results are
 * identical on x86-64 and aarch64 hosts.
 */
#ifndef WR_ORACLE_H
#define WR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- tree (kdtree.cpp) --------------------------------------------------- */
typedef struct wro_tree wro_tree;

/* Median-split build (KDTree::build(BEST) -> splitBest, kdtree.cpp:141-258)
 * over triangles given by GLOBAL vertex indices. */
wro_tree* wro_build(const float* verts, uint32_t nv, const uint32_t* tris, uint32_t nt);
void wro_tree_free(wro_tree* t);
uint32_t wro_tree_num_nodes(const wro_tree* t);
/* Pre-order dump in the layout of ref_harness `dumptree`; returns bytes
 * written (or needed when buf is NULL). */
uint64_t wro_tree_dump(const wro_tree* t, void* buf, uint64_t cap);

/* Closest hit of n rays (n x 6 floats).  Without a filter (inside == NULL)
 * this is KDTree::intersect (kdtree.cpp:279-353); with per-ray inside /
 * contact object ids (-1 = none) each candidate goes through
 * NoSelfCondition::legal (noself.cpp:13-20), which needs tri_obj (object id
 * per triangle).  out_tri gets the triangle id or 0xffffffff, out_t the
 * distance (-1 on a miss).  Counters (may be NULL) receive the numbers of
 * AABB and ray-triangle tests.  nthreads <= 0: all OpenMP threads. */
void wro_trace(const wro_tree* t, const float* rays, uint64_t n, const int32_t* inside, const int32_t* contact,
               const int32_t* tri_obj, uint32_t* out_tri, float* out_t, int nthreads, uint64_t* box_tests,
               uint64_t* tri_tests);

/* ---- counter-based RNG --------------------------------------------------- */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). */
void wro_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* The uniform float in [0,1) for draw `dim` of sample `sample` of pixel
 * `pixel` under `seed` (the same stream the GPU kernels use). */
float wro_draw(uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t dim);

/* ---- path tracer --------------------------------------------------------- */
typedef struct wro_scene wro_scene;
/* Builds a scene from the wr_scene_desc arrays (objects, vertices,
 * object-local triangles, grids, camera): the global tree and one tree per
 * object (Scene::buildKDTree / buildObjKDTrees, scene.cpp:20-65). */
wro_scene* wro_scene_create(const void* scene_desc /* const wr_scene_desc* */);
void wro_scene_free(wro_scene* s);

#define WRO_RNG_PHILOX 0   /* counter-based stream shared with the GPU */
#define WRO_NEE 1u         /* PathTracer NEE branch (pathTracer.cpp:39-66) */
#define WRO_DELTA 4u       /* heterogeneous media by delta / ratio tracking (the GPU's scheme) */

/* PathTracer::renderPixels inner loop for pixels [p0, p1) and samples
 * [s0, s1): accumulates per-pixel sums of the path contribution (after
 * fixVignetting and isLegalColor) into sum (3 floats per pixel, doubles for
 * accuracy) and of its square into sumsq (may be NULL).  OpenMP over pixels. */
void wro_render(const wro_scene* s, uint32_t max_path_len, uint64_t seed, uint32_t flags, uint32_t p0, uint32_t p1,
                uint32_t s0, uint32_t s1, double* sum, double* sumsq, int nthreads, uint64_t* rays_traced);

/* ---- bidirectional path tracer ----------------------------------------- */
/* BidirectionalPathTracer::renderPixels (bidirPathTracer.cpp:10-56) for
 * samples [s0, s1) of every pixel: eye and light sub-paths, all their
 * connections with balance-heuristic MIS weights and light-tracing splats;
 * each sample's image after isLegalColor and fixVignetting is added to sum
 * (and its square to sumsq).  Surfaces and both kinds of media; returns 0. */
int wro_render_bpt(const wro_scene* s, uint32_t max_path_len, uint64_t seed, uint32_t s0, uint32_t s1, double* sum,
                   double* sumsq, int nthreads, uint64_t* rays_traced);
int wro_scene_has_media(const wro_scene* s);
int wro_scene_has_hetero(const wro_scene* s);

/* ---- vertex connection and merging -------------------------------------- */
/* VCMTracer::renderPixels (vcmTracer.cpp:6-92) for samples [s0, s1) with base
 * merge radius r0 (VCMTracer::setRadius): connections with VCM weights and
 * merges through the reference's hash grid; sums as wro_render_bpt; returns 0. */
int wro_render_vcm(const wro_scene* s, uint32_t max_path_len, uint64_t seed, float r0, uint32_t s0, uint32_t s1,
                   double* sum, double* sumsq, int nthreads, uint64_t* rays_traced);
/* the merge radius of iteration s (vcmTracer.cpp:27) */
float wro_vcm_radius(float base, uint32_t s);

/* ---- progressive photon mapping ----------------------------------------- */
/* PhotonMap::renderPixels (photonMap.cpp:20-148, PPM) for samples [s0, s1)
 * with base radius r0 (PhotonMap::setRadius); sums as wro_render_bpt.
 * Surfaces and both kinds of media (volume photons, marched eye segments); returns 0. */
int wro_render_ppm(const wro_scene* s, uint32_t max_path_len, uint64_t seed, float r0, uint32_t s0, uint32_t s1,
                   double* sum, double* sumsq, int nthreads, uint64_t* rays_traced);
/* the elliptic query's set-up (photonMap.cpp:384-613) at a diffuse point of
 * normal hn reached along sp from an anisotropic surface of normal n and
 * exponents Nu, Nv entered along in_d: 0 with the axis ratio and the ellipse
 * frame's ex (long axis) and ey; 1 or 2 for the reference's two fallbacks to
 * the round kernel (sharp ellipse; degenerate projection or Xi_s/Xi_f <= 1) */
int wro_ppm_ellipse(const float in_d[3], const float n[3], const float sp[3], const float hn[3], float nu, float nv,
                    float* ratio, float ex[3], float ey[3]);

#ifdef __cplusplus
}
#endif
#endif
