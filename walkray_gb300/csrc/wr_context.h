// wr_context.h — the library's internal state behind the opaque wr_ctx.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/walkray.h"
#include "kdtree_build.h"
#include "wr_device.cuh"

namespace wr {

struct DeviceBuffer {
    void* p = nullptr;
    size_t bytes = 0;
    DeviceBuffer() = default;
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    ~DeviceBuffer() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    // grows (never shrinks) to at least n bytes; contents are not kept
    cudaError_t reserve(size_t n) {
        if (n <= bytes) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        else p = nullptr;
        return e;
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

// one resident scene
struct SceneGPU {
    uint32_t id = 0;
    DevTree tree{};
    DeviceBuffer pairs, tris;
    wr_scene_info info{};
    // scene description kept on the host for rendering set-up
    std::vector<wr_object_desc> objects;
    std::vector<float> vertices;
    std::vector<uint32_t> triangles;  // object-local
    std::vector<int32_t> tri_obj;
    std::vector<uint32_t> tri_local;
    wr_camera_desc camera{};
    std::vector<wr_grid_desc> grids;
    std::vector<std::vector<float>> grid_data;
    // rendering tables (materials, lights, grids) on the device, filled lazily
    std::shared_ptr<void> render_data;
};

}  // namespace wr

struct wr_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    uint64_t memory_budget = 0;
    std::map<uint32_t, std::unique_ptr<wr::SceneGPU>> scenes;
    uint32_t next_scene = 1;
    wr::DeviceBuffer rays, hits, inside, contact;
    wr::DeviceBuffer scratch_words;  // counters / error flags
    wr::DeviceBuffer film;           // wr_render's image, kept between calls (no allocation per call)
    // wr_trace_closest's copy pipeline: host-to-device and device-to-host
    // streams beside `stream` (which runs the kernels), and its events
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaEvent_t pipe_ev[9] = {};
    bool trace_prune = true;  // wr_trace_closest skips boxes beyond the closest hit (WR_CTX_EXACT_TRAVERSAL: never)
    int last_trace_blocks = 0;
    uint64_t kernel_launches = 0;  // kernels this library has launched on the context
    std::shared_ptr<void> serving;    // serving loop state (serve.cpp)
    std::shared_ptr<void> wavefront;  // wavefront engine (wavefront.cu)
    std::shared_ptr<void> bidir;      // bidirectional renderer's sub-path buffers (bpt.cu)
    // wavefront configuration chosen by wr_autotune (0 = defaults)
    uint32_t wf_capacity = 0;
    int wf_extend_block = 0, wf_shade_block = 0, wf_ctas_per_sm = 0, wf_iters = 0;
    int trace_refill_min = 0, trace_leaf_min = 0;  // warp traversal loop (0 = defaults)
    int trace_steps = 0;                            // traversal steps per turn of the warp loop (0 = default)
    int wf_drain_paths = 0;                          // drain threshold of wr_render (0 = never)
    int wf_pixel_tile = 0;                           // camera paths generated tile by tile (0 = by rows)
};

namespace wr {
struct RenderData;
// drops a scene from the wavefront engine's scene table (wavefront.cu)
void wf_forget_scene(wr_ctx* ctx, const RenderData* rd);
int set_error(wr_ctx* ctx, int code, const std::string& msg);
int cuda_error(wr_ctx* ctx, cudaError_t e, const char* what);
SceneGPU* find_scene(wr_ctx* ctx, wr_scene_id id);
// the traversal loop's knobs: set by wr_set_wavefront_config / wr_autotune, else defaults
inline TraceTune trace_tune_of(const wr_ctx* ctx) {
    TraceTune t = default_trace_tune();
    if (ctx->trace_refill_min) t.refill_min = ctx->trace_refill_min;
    if (ctx->trace_leaf_min) t.leaf_min = ctx->trace_leaf_min;
    if (ctx->trace_steps) t.steps = ctx->trace_steps;
    return t;
}
}  // namespace wr

#define WR_CUDA(ctx, call)                                        \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return wr::cuda_error(ctx, e_, #call); \
    } while (0)
