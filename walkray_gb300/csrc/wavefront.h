// wavefront.h — the batched form of the renderer: path state in HBM, one
// kernel per stage, several renders (jobs) sharing the same queues.
//
//   extend    persistent warps trace every queued ray (closest hit, the same
//             bit-exact traversal as k_trace_closest)
//   sort      buckets the queue by the material each ray hit
//   shade     one bounce of the reference loop per path (scatter, throughput,
//             termination) in bucket order; survivors are compacted into the
//             other state buffer with warp-aggregated appends, finished
//             paths go to their job's film, NEE and light connections to
//             the shadow queue
//   shadow    the connections' closest hits through the same persistent
//             warp loop (k_wf_shadow_trace), then their visible
//             contributions to the film or the path (k_wf_shadow)
//   plan      shares the free queue slots among the jobs
//   generate  refills free queue slots with camera paths of the jobs as
//             planned (continuous batching)
//
// The [reset, extend, sort, shade, shadow trace, shadow, plan, generate] x 2
// sequence (one per ping-pong side; the two shadow kernels only while a job
// in the table connects to lights) is captured once into a CUDA graph and
// replayed until every job is done; kernel sizes never depend on host-side
// counts.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "render_launch.h"
#include "wr_context.h"

namespace wr {

struct RenderData;
struct RenderDataView {  // what the engine needs from RenderData (render_api.cu)
    static const RenderScene& scene(const RenderData* rd);
    static const std::string& unsupported(const RenderData* rd);  // non-empty: why the scene cannot render
};

struct WfJob {
    int scene;  // index into the engine's scene table
    int active;
    CamParams cam;
    uint64_t seed;
    uint32_t s0, spp, max_path_len, flags;
    uint32_t npix;
    uint32_t tile;             // camera paths in pixel tiles of this side (0: by rows)
    unsigned long long total;  // npix * spp paths
    float* film;
    float* film2;
};

struct WfJobCounters {
    unsigned long long claimed;   // paths handed to the queues
    unsigned long long finished;  // paths whose colour reached the film
};

// path state, one ping-pong side: one 128-byte record (a cache line) per
// path, so that the shade stage, which reads the queue in material-bucket
// order, fetches each path's state as whole lines; the extend stage reads
// its first 48 bytes (origin, direction, ids)
enum : int {
    WF_O = 0,     // o.xyz, oP
    WF_D = 1,     // d.xyz, dP
    WF_IDS = 2,   // inside, contact, job, pixel (int bits)
    WF_MISC = 3,  // sample, rng dim, depth | stack_n << 16, cnorm.z bits
    WF_RAD = 4,   // rad.xyz, cnorm.x
    WF_COL = 5,   // color.xyz, cnorm.y
    WF_STK = 6,   // inside stack (int bits)
    WF_PREV = 7,  // direction of the ray before the current one (next-event estimation), MIS density
    WF_REC = 8    // float4 per record
};
struct WfSide {
    float4* rec;  // WF_REC float4 per path
    float4* a5;   // light connections counted so far (WR_RENDER_NEE_MIS jobs only)
    unsigned int* counts;  // [0] survivors written by shade, [1] paths appended by generate
};

// the extend stage's queue bucketed by the material that shades each path
// (0 = no hit, 1 + WR_MAT_* of the inside or hit object), so that the shade
// stage runs one material's code per warp
constexpr int WF_SORT_KEYS = 9;
struct WfSort {
    unsigned int* counts;  // [WF_SORT_KEYS]
    uint32_t* idx;         // bucket k at idx + k * capacity
};

// shadow rays of next-event estimation, written by shade, traced by
// k_wf_shadow_trace and resolved by k_wf_shadow
struct WfShadow {
    float4* o;    // origin, distance to the light sample
    float4* d;    // direction, light object (int bits; WR_RENDER_NEE_MIS)
    float4* c;    // contribution if visible, kind (int bits: WF_SHADOW_*)
    float4* r;    // WF_SHADOW_MIS_DONE: the path's own result; target path slot (int bits)
    int4* ids;    // inside, contact, job, pixel
    unsigned int* count;
};
// what a visible shadow ray does: the reference's NEE adds its colour to the
// film; a light connection of a path that goes on adds it to the path's
// accumulator (slot `target` of the side shade wrote); one of a path that
// ended adds it to the path's result, which goes to the film
enum : int { WF_SHADOW_NEE = 0, WF_SHADOW_MIS_KEEP = 1, WF_SHADOW_MIS_DONE = 2 };

struct WfConfig {
    uint32_t capacity = 1u << 24;  // paths in flight (16M x 128 B of state per side): a 1024^2 x 16-spp call at once
    int extend_block = 128;
    int shade_block = 128;
    int ctas_per_sm = 0;           // 0 = occupancy calculator
    int iters_per_graph = 4;       // ping-pong pairs per graph launch
    TraceTune trace = default_trace_tune();  // warp traversal loop of the extend stage
    int drain_paths = 0;           // per-path finish of a render's last paths at most this many (0 = never)
    int pixel_tile = 0;            // generate camera paths tile by tile, tiles of this side (0: by rows)

    uint32_t drain_threshold() const {
        return drain_paths > 0 ? (uint32_t)drain_paths : 0u;
    }
};

// the share-out of free queue slots among jobs for one generate stage
// (k_wf_plan): entry k is job slot slot[k] with path indices
// [first[k], first[k] + off[k+1] - off[k]) at queue positions off[k]..
struct WfPlan {
    int* slot;
    unsigned long long* first;
    uint32_t* off;  // n + 1 offsets
    int* n;
};

struct WfEngine;

// Device tables of the jobs in flight (up to max_jobs) and of the scenes
// they reference.
int wf_engine_get(wr_ctx* ctx, const WfConfig& cfg, WfEngine** out);
uint32_t wf_max_jobs();

// Renders spp samples of one scene through the wavefront (wr_render_device).
int render_wavefront(wr_ctx* ctx, RenderData& rd, const RenderParams& P, uint32_t spp_offset, uint32_t spp,
                     float* film, float* film2, cudaStream_t stream);

// Lower-level interface used by the serving loop.  Jobs live in fixed slots
// (in-flight paths carry their slot), generated in the order of `order`.
struct WfJobHost {
    WfJob job;
    const RenderData* rd = nullptr;  // scene of the job (nullptr: keep the slot's scene)
};
struct WfSlotUpdate {
    int slot = 0;
    WfJobHost jh;
    bool reset_counters = false;
};
int wf_update_jobs(wr_ctx* ctx, WfEngine* E, const std::vector<WfSlotUpdate>& updates, const std::vector<int>& order,
                   cudaStream_t s);
int wf_launch(wr_ctx* ctx, WfEngine* E, cudaStream_t s);  // one graph replay
// per-job counters; `waiting` (optional) gets the number of paths waiting in
// queue side `side` (side 0 after a graph replay)
int wf_read_counters(wr_ctx* ctx, WfEngine* E, std::vector<WfJobCounters>& out, cudaStream_t s,
                     uint32_t* waiting = nullptr, int side = 0);
// finishes the n paths waiting in side `side`, one thread per path (k_wf_drain)
int wf_drain(wr_ctx* ctx, WfEngine* E, int side, uint32_t n, cudaStream_t s);
int wf_error_word(wr_ctx* ctx, WfEngine* E, unsigned int* herr, cudaStream_t s);
int wf_reset_queues(wr_ctx* ctx, WfEngine* E, cudaStream_t s);
// free queue slots shared equally among the jobs with paths left (default)
// or handed out in admission order
int wf_set_equal_share(wr_ctx* ctx, WfEngine* E, bool on);
// the queue is filled up to `paths` (clamped to 1 .. capacity; capacity when
// the engine is made); takes effect from the next bounce loop on stream s
int wf_set_live_cap(wr_ctx* ctx, WfEngine* E, uint32_t paths, cudaStream_t s);
uint32_t wf_live_cap(const WfEngine* E);
const WfConfig& wf_config(const WfEngine* E);
int wf_set_config(wr_ctx* ctx, const WfConfig& cfg);
WfConfig wf_tuned_config(wr_ctx* ctx);
WfJob make_job(const RenderScene& S, const CamParams& cam, uint64_t seed, uint32_t s0, uint32_t spp,
               uint32_t max_path_len, uint32_t flags, float* film, float* film2);
CamParams camera_params_for(const RenderData* rd, uint32_t width, uint32_t height);

}  // namespace wr
