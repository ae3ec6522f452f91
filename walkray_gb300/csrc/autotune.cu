// autotune.cpp — wr_autotune: picks the wavefront configuration (paths in
// flight, block shapes, persistent CTAs per SM, bounce iterations per graph
// launch) for a scene by timing short renders of each candidate on the
// device, and keeps the fastest in the context for later wavefront renders.
#include <cuda_runtime.h>

#include <vector>

#include "wavefront.h"
#include "wr_context.h"

using namespace wr;

extern "C" {

int wr_set_wavefront_config(wr_ctx* ctx, const wr_wavefront_config* cfg) {
    if (!ctx || !cfg) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null argument");
    if (cfg->capacity < 1024 || cfg->capacity > (1u << 25) || (cfg->extend_block % 32) || (cfg->shade_block % 32) ||
        cfg->extend_block <= 0 || cfg->extend_block > 128 || cfg->shade_block <= 0 || cfg->shade_block > 128 ||
        cfg->iters_per_graph <= 0 || cfg->iters_per_graph > 64 || cfg->ctas_per_sm < 0 || cfg->refill_min < 0 ||
        cfg->refill_min > 32 || cfg->leaf_min < 0 || cfg->leaf_min > 32 || cfg->drain_paths < 0)
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "wavefront configuration out of range");
    ctx->wf_capacity = cfg->capacity;
    ctx->wf_extend_block = cfg->extend_block;
    ctx->wf_shade_block = cfg->shade_block;
    ctx->wf_ctas_per_sm = cfg->ctas_per_sm;
    ctx->wf_iters = cfg->iters_per_graph;
    ctx->trace_refill_min = cfg->refill_min;
    ctx->trace_leaf_min = cfg->leaf_min;
    ctx->wf_drain_paths = cfg->drain_paths;
    return WR_OK;
}

int wr_autotune(wr_ctx* ctx, wr_scene_id scene, uint32_t spp_per_trial, uint32_t max_path_len,
                wr_wavefront_config* best) {
    if (!ctx || !best) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null argument");
    SceneGPU* sc = find_scene(ctx, scene);
    if (!sc) return set_error(ctx, WR_ERR_NOT_FOUND, "no such scene");
    if (spp_per_trial == 0) spp_per_trial = 1;
    WR_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t n = 3ull * sc->camera.width * sc->camera.height;
    DeviceBuffer film;
    WR_CUDA(ctx, film.reserve(sizeof(float) * (n ? n : 1)));
    std::vector<wr_wavefront_config> cands;
    for (uint32_t cap : {1u << 19, 1u << 20, 1u << 21, 1u << 22})
        for (int eb : {64, 128})
            for (int sb : {64, 128})  // the shade / generate kernels are built for at most 128 threads
                for (int it : {2, 8}) cands.push_back(wr_wavefront_config{cap, eb, sb, 0, it, 0, 0, 0, 0.0});
    cudaEvent_t a, b;
    WR_CUDA(ctx, cudaEventCreate(&a));
    WR_CUDA(ctx, cudaEventCreate(&b));
    wr_wavefront_config top{};
    double top_rate = -1.0;
    wr_render_desc d{};
    d.spp = spp_per_trial;
    d.max_path_len = max_path_len;
    d.seed = 0x5eed;
    d.mode = WR_MODE_WAVEFRONT;
    for (auto& c : cands) {
        int rc = wr_set_wavefront_config(ctx, &c);
        if (rc != WR_OK) continue;
        // warm (also builds the engine and captures the graph), then time
        rc = wr_render_device(ctx, scene, &d, film.as<float>(), nullptr, ctx->stream);
        if (rc != WR_OK) continue;
        cudaEventRecord(a, ctx->stream);
        rc = wr_render_device(ctx, scene, &d, film.as<float>(), nullptr, ctx->stream);
        cudaEventRecord(b, ctx->stream);
        if (rc != WR_OK || cudaEventSynchronize(b) != cudaSuccess) continue;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        const double rate = (double)n / 3 * spp_per_trial / (ms * 1e-3) / 1e6;
        c.mpaths_per_s = rate;
        if (rate > top_rate) {
            top_rate = rate;
            top = c;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (top_rate < 0) return set_error(ctx, WR_ERR_INTERNAL, "no wavefront configuration ran");
    int rc = wr_set_wavefront_config(ctx, &top);
    if (rc != WR_OK) return rc;
    *best = top;
    return WR_OK;
}

}  // extern "C"
