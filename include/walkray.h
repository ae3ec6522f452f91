/*
 * walkray.h — C ABI of the GB300 path-tracing library (libwalkray_gpu.so).
 *
 * This is the only boundary between host code and the sm_103a kernels.  It
 * replaces, for WalkRay's unidirectional path tracer, the in-process calls
 * that the reference makes between its renderer plugin and its scene:
 *
 *   reference interface (WalkRay)                    entry point here
 *   ----------------------------------------------   ------------------------
 *   Config::load builds objects + Scene::buildKDTree  wr_scene_upload
 *     (config.cpp:432-519, scene.cpp:20-44)
 *   KDTree::intersect / Scene::intersect             wr_trace_closest
 *     (kdtree.cpp:349-353, scene.cpp:102-113,
 *      NoSelfCondition::legal noself.cpp:13-20)
 *   MCRenderer::renderPixels (mcRenderer.h:27),      wr_render
 *     PathTracer::renderPixels (pathTracer.cpp:7-76)
 *   RenderEngine::renderFilm (renderEngine.cpp:27-30) wr_submit/wr_poll/wr_fetch
 *     called once per request                          (serving loop)
 *
 * Conventions: every function returns an int status (WR_OK or WR_ERR_*); no
 * C++ exception crosses this boundary; wr_last_error() gives a message for
 * the last failure on a context.  Host buffers belong to the caller; device
 * memory belongs to the library.  A context is not thread-safe: use one per
 * host thread, or serialise calls.
 */
#ifndef WALKRAY_H
#define WALKRAY_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WR_ABI_VERSION 2u

/* status codes */
#define WR_OK 0
#define WR_ERR_INVALID_ARGUMENT 1
#define WR_ERR_OUT_OF_MEMORY 2
#define WR_ERR_CUDA 3
#define WR_ERR_NOT_FOUND 4
#define WR_ERR_TIMEOUT 5
#define WR_ERR_BUSY 6
#define WR_ERR_CANCELLED 7
#define WR_ERR_UNSUPPORTED 8
#define WR_ERR_INTERNAL 9

#define WR_NO_HIT 0xffffffffu
#define WR_NO_OBJECT (-1)

/* material / object kinds (one per reference scene-object class) */
#define WR_MAT_DIFFUSE 0       /* DiffuseObject            diffuseObj.h */
#define WR_MAT_GLOSSY 1        /* GlossyObject (iso Phong)  glossyObj.h */
#define WR_MAT_ANISO 2         /* AnisotropicGlossyObject   anisotropicGlossyObj.h */
#define WR_MAT_REFRACTIVE 3    /* RefractiveObject          refractiveObj.h */
#define WR_MAT_EMISSIVE 4      /* EmissiveObject            emissiveObj.h */
#define WR_MAT_HOMOGENEOUS 5   /* HomogeneousVolume         homogeneousVolume.h */
#define WR_MAT_HETEROGENEOUS 6 /* HeterogeneousVolume       HeterogeneousVolume.h */
#define WR_MAT_REFLECTIVE 7    /* ReflectiveObject (mirror)  reflectiveObj.h; colour in albedo */

/* One scene object: a triangle mesh with world-space vertices (the
 * reference's Mesh with an identity transform) and its material.  Fields a
 * material does not use are ignored.  136 bytes, all 4-byte fields. */
typedef struct wr_object_desc {
    uint32_t type;           /* WR_MAT_* */
    uint32_t vert_begin;     /* first vertex of this object in wr_scene_desc.vertices */
    uint32_t vert_count;
    uint32_t tri_begin;      /* first triangle of this object in wr_scene_desc.triangles */
    uint32_t tri_count;
    uint32_t grid_index;     /* heterogeneous media: index into wr_scene_desc.grids */
    float albedo[3];         /* diffuse / glossy reflectanceAlbedo, reflective color */
    float emission[3];       /* emissive color */
    float power;             /* isotropic Phong exponent */
    float ior;               /* refractive object / medium index of refraction */
    float decay[3];          /* refractive decayColor (per unit distance) */
    float rs[3];             /* anisotropic Phong Rs */
    float rd[3];             /* anisotropic Phong Rd */
    float nu, nv;            /* anisotropic Phong exponents */
    float sigma_s[3];        /* media scattering coefficient */
    float sigma_a[3];        /* media absorption coefficient */
    float g;                 /* Henyey-Greenstein asymmetry */
    float density_scale;     /* heterogeneous: density multiplier (reference default 100) */
    float step_size;         /* media: ray-marching step (HeterogeneousVolume default 0.002; photon mapping
                                marches homogeneous media with it too) */
} wr_object_desc;

/* Pinhole camera (Camera::setup, camera.h:28-48); image_plane_dist is the
 * reference's mImagePlaneDist in pixels.  lens_radius > 0 enables the
 * thin-lens path (camera.cpp:30-47). */
typedef struct wr_camera_desc {
    float position[3];
    float focus[3];
    float up[3];
    uint32_t width;
    uint32_t height;
    float image_plane_dist;
    float lens_radius;
    float focal_dist;
} wr_camera_desc;

/* Density grid of a heterogeneous medium, z-major (index z*nx*ny + y*nx + x,
 * HeterogeneousVolume.h:31-36), spanning the box [p0, p1]. */
typedef struct wr_grid_desc {
    uint32_t nx, ny, nz;
    uint32_t pad;
    const float* density;
    float p0[3];
    float p1[3];
} wr_grid_desc;

typedef struct wr_scene_desc {
    uint32_t num_objects;
    uint32_t num_vertices;
    uint32_t num_triangles;
    uint32_t num_grids;
    const wr_object_desc* objects;
    const float* vertices;     /* num_vertices x 3, world space, object by object */
    const uint32_t* triangles; /* num_triangles x 3, vertex indices LOCAL to the object */
    const wr_grid_desc* grids;
    wr_camera_desc camera;
} wr_scene_desc;

/* Closest hit: tri is the global triangle index (scene order, object by
 * object) or WR_NO_HIT; t the reference's hit distance; b1, b2 the
 * barycentric coordinates of the hit point (mesh.h:67-73 formula). */
typedef struct wr_hit {
    uint32_t tri;
    float t;
    float b1;
    float b2;
} wr_hit;

typedef struct wr_ctx wr_ctx;
typedef uint32_t wr_scene_id;

typedef struct wr_ctx_desc {
    int device;                      /* CUDA device ordinal */
    uint64_t device_memory_budget;   /* bytes the serving loop may use; 0 = 90% of free */
    uint32_t flags;                  /* WR_CTX_* */
    uint32_t pad;
} wr_ctx_desc;

/* wr_trace_closest visits every box the reference visits (KDTree::intersect,
 * kdtree.cpp:308-347, which never prunes by distance).  Without this flag it
 * skips a box entered beyond 1.001 x the closest hit found so far (plus the
 * box margin), except for a ray whose closest hit so far grazes its
 * triangle's plane (|n.d| < |d| / 32), which keeps every box: a triangle's
 * hit lies in its box up to the triangle test's rounding, which only a
 * near-grazing ray can make large.  Same hits on every test set (all 2^24
 * rays of the 1.31M-triangle icosphere workload included). */
#define WR_CTX_EXACT_TRAVERSAL 1u

/* ---- context ------------------------------------------------------------ */
int wr_get_abi_version(uint32_t* version);
int wr_ctx_create(const wr_ctx_desc* desc, wr_ctx** out);
int wr_ctx_destroy(wr_ctx* ctx);
const char* wr_last_error(const wr_ctx* ctx);
/* Number of kernels the library has launched on this context so far (graph
 * replays count every kernel node).  No reference counterpart. */
int wr_kernel_launches(const wr_ctx* ctx, uint64_t* out);

/* ---- scenes ------------------------------------------------------------- */
/* Flattens the scene (Scene::buildKDTree, scene.cpp:20-44), builds the
 * reference's median-split tree over all triangles (KDTree::build with
 * splitBest, kdtree.cpp:141-258) and makes it resident on the device. */
int wr_scene_upload(wr_ctx* ctx, const wr_scene_desc* desc, wr_scene_id* out);
int wr_scene_release(wr_ctx* ctx, wr_scene_id scene);

typedef struct wr_scene_info {
    uint32_t num_triangles;
    uint32_t num_nodes;        /* reference tree nodes (root + children) */
    uint32_t num_leaves;
    uint32_t max_depth;
    uint64_t device_bytes;     /* resident bytes of this scene */
    double build_seconds;      /* host tree build time */
} wr_scene_info;
int wr_scene_get_info(wr_ctx* ctx, wr_scene_id scene, wr_scene_info* out);

/* ---- traversal ---------------------------------------------------------- */
/* Per-ray self-intersection filter (NoSelfCondition, noself.cpp:13-20):
 * inside_obj / contact_obj are object indices or WR_NO_OBJECT.  Pass NULL
 * for the unfiltered query (KDTree::intersect with condition == NULL). */
typedef struct wr_trace_filter {
    const int32_t* inside_obj;
    const int32_t* contact_obj;
} wr_trace_filter;

/* Closest hit of n rays (origin xyz, direction xyz; n x 6 floats).  Host
 * buffers: the call copies rays to the device and hits back, from 2^20 rays
 * on in 2 or 4 chunks whose copies overlap the other chunks' traversal
 * (page-locked buffers let the copies run asynchronously).
 * Replaces KDTree::intersect (kdtree.cpp:349-353) and Scene::intersect
 * (scene.cpp:102-113). */
int wr_trace_closest(wr_ctx* ctx, wr_scene_id scene, const float* rays, uint64_t n,
                     const wr_trace_filter* filter, wr_hit* hits);

/* Same on device buffers already resident in HBM, enqueued on `stream`
 * (a cudaStream_t; NULL = the legacy default stream). */
int wr_trace_closest_device(wr_ctx* ctx, wr_scene_id scene, const float* d_rays, uint64_t n,
                            const int32_t* d_inside_obj, const int32_t* d_contact_obj,
                            wr_hit* d_hits, void* stream);

/* ---- rendering ---------------------------------------------------------- */
#define WR_MODE_MEGAKERNEL 0u /* one thread per pixel runs whole paths */
#define WR_MODE_WAVEFRONT 1u  /* generate / extend / shade queues, persistent kernels, graph bounce loop */
#define WR_MODE_BIDIRECTIONAL 2u /* BidirectionalPathTracer (bidirPathTracer.cpp:10-313): eye and light
                                    sub-paths, all connections, balance-heuristic MIS, light tracing;
                                    surfaces and both kinds of media (a heterogeneous medium with the
                                    reference's own distance sampler and marched integrals),
                                    max_path_len <= 30 */
#define WR_MODE_VCM 3u           /* VCMTracer (vcmTracer.cpp:6-446): the bidirectional connections with
                                    VCM weights plus vertex merging of every eye vertex with the light
                                    points within the iteration's radius (the reference's hash grid);
                                    wr_render_desc.radius is the base radius (VCMTracer::setRadius;
                                    0 = the reference's default 0.01); surfaces and both kinds of
                                    media, max_path_len <= 30 */
#define WR_MODE_PHOTON_MAP 4u    /* PhotonMap (photonMap.cpp:20-625) as the reference builds it (progressive:
                                    radius r_s of VCM's schedule, no ray marching): light sub-paths as
                                    photons in the reference's hash grid, each eye path's first diffuse
                                    record estimates the photon density (kernel 3(1-d^2/r^2)^2/pi; the
                                    Gaussian-weighted elliptic estimate behind an anisotropic glossy
                                    reflection, photonMap.cpp:383-652); wr_render_desc.radius is the base
                                    radius (PhotonMap::setRadius; 0 = 0.01); media: volume photons and
                                    ray-marched eye segments in steps of each medium's step_size
                                    (photonMap.cpp:306-367); max_path_len <= 30 */

#define WR_RENDER_NEE 1u      /* PathTracer's next-event-estimation branch (pathTracer.cpp:39-66) */
/* Rendering traverses front to back and skips a box whose entry distance is
 * beyond the closest hit found so far (with a 0.1 % relative margin).  That
 * gives the reference's closest hit except for a ray that grazes a triangle
 * so nearly in its plane that the triangle test's rounding moves the hit
 * outside the triangle's box.  This flag visits every box the reference
 * visits (KDTree::intersect, kdtree.cpp:308-347), as wr_trace_closest does. */
#define WR_RENDER_EXACT_TRAVERSAL 2u
/* Low-variance estimators (no reference counterpart; the reference's
 * expectation is kept, only the variance changes).  Path tracing modes
 * (WR_MODE_MEGAKERNEL, WR_MODE_WAVEFRONT, serving) only.
 * WR_RENDER_NEE_MIS: unbiased next-event estimation at every diffuse,
 * isotropic-Phong and anisotropic-Phong surface vertex outside media (one
 * light sample per vertex, SurfaceSampler's area-proportional pick), combined
 * with the BSDF-sampled hits of emitters by multiple importance sampling
 * (power heuristic).  The reference's NEE branch (WR_RENDER_NEE, biased)
 * cannot be combined with it.
 * WR_RENDER_PHONG_MIRROR: isotropic Phong directions sampled about the mirror
 * direction with the density (n+1)/(2 pi) (R.w)^n (the reference samples
 * about the normal, isotropicPhong.h:20-38, whose weights are unbounded for
 * large exponents); samples below the surface end the path with zero
 * radiance. */
#define WR_RENDER_NEE_MIS 4u
#define WR_RENDER_PHONG_MIRROR 8u

typedef struct wr_render_desc {
    uint32_t spp;          /* samples per pixel (PathTracer spp) */
    uint32_t max_path_len; /* MCRenderer maxPathLen */
    uint64_t seed;         /* key of the per-path counter-based random stream */
    uint32_t mode;         /* WR_MODE_* */
    uint32_t flags;        /* WR_RENDER_* */
    uint32_t spp_offset;   /* index of the first sample (progressive rendering / resume) */
    float radius;          /* WR_MODE_VCM / WR_MODE_PHOTON_MAP: base radius (0 = 0.01); ignored otherwise */
} wr_render_desc;

/* PathTracer::renderPixels (pathTracer.cpp:7-76) on the GPU: rgb_out gets
 * the W*H*3 mean image (p = y*W + x, row 0 at the top), host buffer. */
int wr_render(wr_ctx* ctx, wr_scene_id scene, const wr_render_desc* desc, float* rgb_out);

/* PathTracer::renderPixels (pathTracer.cpp:15-73) refines its image one
 * sample per pixel at a time and shows / saves the running mean after each
 * (Film::setBuffer, savePFM); without an <iter> in the configuration its
 * spp is INT_MAX (config.cpp:534) and it runs until stopped.  This entry
 * point renders the same way in chunks of at most chunk_spp samples per
 * pixel (0 = about 16M paths per chunk): after each chunk rgb_out (host,
 * W*H*3) holds the mean of the samples so far and progress(user, rgb_out,
 * spp_done) is called (progress may be NULL); a nonzero return stops the
 * render there.  *spp_done (may be NULL) gets the samples rendered.  The
 * samples are those of one wr_render of desc->spp samples. */
typedef int (*wr_progress_fn)(void* user, const float* rgb, uint32_t spp_done);
int wr_render_progressive(wr_ctx* ctx, wr_scene_id scene, const wr_render_desc* desc, uint32_t chunk_spp,
                          float* rgb_out, wr_progress_fn progress, void* user, uint32_t* spp_done);

/* Adds the desc->spp samples starting at desc->spp_offset to a device film:
 * d_sum[3p+c] += colour, d_sumsq (may be NULL) += colour^2.  Enqueued on
 * `stream` (cudaStream_t; NULL = the context's stream), asynchronous. */
int wr_render_device(wr_ctx* ctx, wr_scene_id scene, const wr_render_desc* desc, float* d_sum, float* d_sumsq,
                     void* stream);

/* Rendering without any device allocation.  No counterpart in the reference
 * (the reference renders on the CPU).  wr_render allocates an accumulation
 * film on every call, which some callers cannot allow: real-time loops that
 * avoid cudaMalloc / cudaFree because they can synchronise the device and
 * stall a frame, and applications whose device memory belongs to their own
 * pool or allocator.  This entry point renders like wr_render in
 * WR_MODE_MEGAKERNEL but keeps the film in a fixed array inside the library
 * (WR_NOALLOC_MAX_PIXELS pixels, 12 MiB per GPU that loads the library, held
 * until exit) and writes the W*H*3 mean image to the caller's device buffer
 * d_rgb_out, asynchronously on `stream` (NULL = the context's stream).  Larger
 * images are rejected with WR_ERR_INVALID_ARGUMENT, scenes wr_render refuses
 * with the same WR_ERR_UNSUPPORTED.  It calls no allocation routine: the scene
 * must have been rendered once before (wr_render / wr_render_device build its
 * rendering tables), and the first call on a device looks up the array's
 * device address in the device's primary context (the CUDA runtime's), with
 * which every call must be made.  All calls share the array: calls whose work
 * overlaps on the GPU race and must be serialised. */
#define WR_NOALLOC_MAX_PIXELS 1048576u
int wr_render_noalloc(wr_ctx* ctx, wr_scene_id scene, const wr_render_desc* desc, float* d_rgb_out, void* stream);
/* Traversal status of the most recent wr_render_noalloc on this context's
 * device, read without allocating: waits for `stream` (NULL = the context's
 * stream) and stores the error word in *out_err: 0 when every traversal
 * finished, nonzero when a traversal stack would have overflowed (the image
 * of that call is then incomplete; wr_render reports the same case as
 * WR_ERR_INTERNAL).  Companion of wr_render_noalloc; no reference counterpart. */
int wr_render_noalloc_status(wr_ctx* ctx, void* stream, unsigned int* out_err);

/* Per-stage profile of one wavefront render (no reference counterpart: the
 * reference has no timers).  The stages are launched one by one instead of
 * as a graph, each between CUDA events on the context's stream; the
 * traversal stage also counts its work. */
typedef struct wr_render_profile {
    double ms_extend, ms_shade, ms_shadow, ms_generate, ms_total;
    uint64_t iterations;       /* bounce iterations run */
    uint64_t rays;             /* rays traced by the extend stage */
    uint64_t box_tests;        /* AABB predicate evaluations (reference count) */
    uint64_t tri_tests;        /* ray-triangle tests */
    uint64_t paths;
    double ms_drain;           /* the per-path finish of the last paths (k_wf_drain) */
    uint64_t drained_paths;    /* paths it finished */
    uint32_t iter_rays[32];    /* rays in the queue of bounce iteration i (first 32 iterations) */
    float iter_extend_ms[32];  /* extend stage time of iteration i */
    float iter_shade_ms[32];   /* shade stage time of iteration i */
} wr_render_profile;
int wr_profile_render(wr_ctx* ctx, wr_scene_id scene, const wr_render_desc* desc, float* d_sum,
                      wr_render_profile* out);

/* ---- random stream ----------------------------------------------------- */
/* The renderers' device random stream, read back for known-answer checks.
 * The reference draws from one std::mt19937_64 shared by its threads
 * (rng.h:6-59, Rng::genFloat); this library gives every path its own
 * counter-based stream instead: draw `dim` of (pixel, sample) under the
 * render seed is word dim % 4 of Philox4x32-10 on the counter
 * {dim / 4, sample, pixel, 0} with key {seed low, seed high}, top 24 bits
 * times 2^-24.  For each i < n the device draws sequentially from 0 to
 * dim[i] with the renderers' own generator and stores the last draw in
 * draws[i] and the four Philox words of its block in words[4i..4i+3].  Host
 * buffers; n <= 2^24, dim[i] < 65536. */
int wr_rng_draws(wr_ctx* ctx, uint64_t seed, const uint32_t* pixel, const uint32_t* sample, const uint32_t* dim,
                 uint64_t n, uint32_t* words, float* draws);

/* ---- serving ------------------------------------------------------------- */
/* A request loop over resident scenes: RenderEngine::renderFilm
 * (renderEngine.cpp:27-30) once per request, with requests admitted while
 * others run (continuous batching) and their paths sharing the wavefront
 * queues.  A request is admitted when a job slot is free and its film fits
 * in the serving film memory; until then it waits in FIFO order.  While the
 * loop runs, only wr_submit / wr_poll / wr_fetch / wr_cancel / wr_serve_stop
 * may be called on the context; scenes are uploaded before wr_serve_start. */
#define WR_REQ_QUEUED 0u
#define WR_REQ_RUNNING 1u
#define WR_REQ_DONE 2u
#define WR_REQ_CANCELLED 3u
#define WR_REQ_FAILED 4u

typedef uint64_t wr_req_id;

typedef struct wr_serve_desc {
    uint64_t film_bytes;      /* device memory for request films; 0 = a quarter of the context budget */
    uint32_t max_active;      /* requests in flight at once; 0 = 64 */
    uint32_t flags;           /* WR_SERVE_* */
    uint32_t paths_in_flight; /* queue length while no request waits for admission (1024 .. 2^25,
                                 at most the wavefront configuration's capacity, which the queue
                                 holds while requests wait); 0 = WR_SERVE_DEFAULT_PATHS */
    uint32_t reserved;        /* 0 */
} wr_serve_desc;
/* Every bounce of a request's paths waits for one pass of the bounce loop over
 * the whole queue, so a shorter queue than the renderer's 2^24 cuts the
 * latency of small requests; on GB300 2^22 paths keep 97 % of the
 * throughput, and a saturated loop (requests waiting) uses the full queue. */
#define WR_SERVE_DEFAULT_PATHS 4194304u
/* Queue slots freed by finished paths go to the running requests in
 * admission order (first come, first served) instead of in equal shares to
 * every request with paths left (the default: a small request admitted
 * behind a large one starts at once). */
#define WR_SERVE_FIFO 1u

typedef struct wr_request_desc {
    wr_scene_id scene;
    uint32_t width, height;  /* resolution; the scene camera's field of view is kept */
    uint32_t spp;
    uint32_t max_path_len;
    uint32_t flags;          /* WR_RENDER_* */
    uint64_t seed;
} wr_request_desc;

typedef struct wr_req_status {
    uint32_t state;          /* WR_REQ_* */
    uint32_t pad;
    uint64_t paths_total;
    uint64_t paths_done;
    double submit_s, admit_s, finish_s; /* seconds since wr_serve_start */
} wr_req_status;

int wr_serve_start(wr_ctx* ctx, const wr_serve_desc* desc);
int wr_serve_stop(wr_ctx* ctx);  /* cancels what has not finished */
int wr_submit(wr_ctx* ctx, const wr_request_desc* req, wr_req_id* out);
int wr_poll(wr_ctx* ctx, wr_req_id id, wr_req_status* out);
/* mean image (height x width x 3, row 0 at the top) of a finished request;
 * releases it */
int wr_fetch(wr_ctx* ctx, wr_req_id id, float* rgb_out);
int wr_cancel(wr_ctx* ctx, wr_req_id id);

/* ---- wavefront configuration and autotuner ------------------------------- */
/* No reference counterpart (the reference renders with one OpenMP loop,
 * pathTracer.cpp:20): these size the wavefront renderer's queues. */
typedef struct wr_wavefront_config {
    uint32_t capacity;       /* paths in flight (queue length) */
    int32_t extend_block;    /* threads per CTA of the traversal stage (32..128) */
    int32_t shade_block;     /* threads per CTA of the shade / generate stages (32..128) */
    int32_t ctas_per_sm;     /* traversal kernels compiled for at least 1-5, 6, 7 or 8+ resident CTAs
                                per SM (fewer registers per thread as it grows), launched with at most
                                that many; 0 = tuned defaults (6 for rendering, 7 for
                                wr_trace_closest); also applies to wr_trace_closest */
    int32_t iters_per_graph; /* bounce-loop iterations (pairs) per CUDA-graph launch */
    int32_t refill_min;      /* traversal: idle lanes of a warp that trigger a ray refill (1..32, 0 = default) */
    int32_t leaf_min;        /* traversal: lanes holding leaves that start a warp's leaf tests (1..32,
                                0 = default); both also apply to wr_trace_closest */
    int32_t drain_paths;     /* wr_render: once every path is generated and at most this many remain,
                                finish them in one per-path kernel (0 = never) */
    int32_t pixel_tile;      /* camera paths generated tile by tile, square tiles of this many pixels a
                                side (0 = row by row); the image does not depend on it */
    int32_t steps_per_turn;  /* traversal: steps a searching lane takes per turn of a warp's loop (1..8,
                                0 = default 6); also applies to wr_trace_closest */
    double mpaths_per_s;     /* filled by wr_autotune */
} wr_wavefront_config;

int wr_set_wavefront_config(wr_ctx* ctx, const wr_wavefront_config* cfg);

/* Picks the wavefront configuration for `scene` by timing short renders
 * (spp_per_trial samples per pixel, max_path_len) on the device: starting
 * from the defaults, one dimension at a time -- paths in flight, traversal
 * CTAs per SM, the warp loop's refill and leaf thresholds and steps per
 * turn, the camera-path pixel tile, bounce iterations per graph launch --
 * keeping each value that renders faster (coordinate descent).  The best
 * configuration stays in the context; `best` gets it with its Mpaths/s.  No
 * reference counterpart. */
int wr_autotune(wr_ctx* ctx, wr_scene_id scene, uint32_t spp_per_trial, uint32_t max_path_len,
                wr_wavefront_config* best);

/* ---- scene files (no GPU needed) ----------------------------------------- */
/* WalkRay's scene configuration read into a wr_scene_desc: Config::load
 * (config.cpp:432-575) with its <Scene>, <Object>, <GroupObject>, <Camera>
 * and <Material> nodes, and Mesh::loadShape (mesh.cpp:5-130) for .obj and
 * .shp meshes, including the reference's unitizing of every mesh.  The
 * description's arrays belong to the wr_scene_file and live until
 * wr_scene_file_free.  On failure `err` (may be NULL) gets a message. */
typedef struct wr_scene_file wr_scene_file;
typedef struct wr_scene_file_settings {
    char renderer[32];     /* the <renderer> name, e.g. "PathTracer" / "PT" */
    uint32_t spp;          /* <iter> (0 when absent) */
    uint32_t max_path_len; /* 20, as Config::load sets for every renderer */
    float radius;          /* <radius> of the VCM / photon-map renderers (0 when absent) */
    uint32_t mode;         /* the WR_MODE_* of the renderer name (config.cpp:530-572):
                              PathTracer/PT -> WR_MODE_WAVEFRONT, BidirPathTracer/BPT ->
                              WR_MODE_BIDIRECTIONAL, VCMTracer/VCM -> WR_MODE_VCM,
                              PhotonMap/PM -> WR_MODE_PHOTON_MAP; 0xffffffff for any other */
} wr_scene_file_settings;
int wr_scene_file_load(const char* config_path, wr_scene_file** out, char* err, size_t err_len);
int wr_scene_file_get(const wr_scene_file* f, wr_scene_desc* desc, wr_scene_file_settings* settings);
int wr_scene_file_free(wr_scene_file* f);

/* ---- host-side tree (no GPU needed) ------------------------------------- */
/* Builds the reference tree on the host only and returns its flattened
 * form, so that host logic can be checked without a device.
 * nodes: per node {first, count_or_child} as described in kdtree_host.h;
 * boxes: per node min xyz, max xyz; leaf_tris: global triangle ids in
 * leaf order. */
typedef struct wr_kdtree_host wr_kdtree_host;
int wr_kdtree_build_host(const float* vertices, uint32_t num_vertices, const uint32_t* triangles,
                         uint32_t num_triangles, int num_threads, wr_kdtree_host** out);
int wr_kdtree_host_sizes(const wr_kdtree_host* t, uint32_t* num_nodes, uint32_t* num_leaf_tris,
                         uint32_t* max_depth);
int wr_kdtree_host_export(const wr_kdtree_host* t, int32_t* left, int32_t* right, float* boxes,
                          uint32_t* leaf_first, uint32_t* leaf_count, uint32_t* leaf_tris);
int wr_kdtree_host_free(wr_kdtree_host* t);

#ifdef __cplusplus
}
#endif
#endif /* WALKRAY_H */
