// autotune.cu — wr_autotune: picks the wavefront configuration of a scene by
// timing short renders on the device, and keeps the fastest in the context
// for later wavefront renders.  The search is coordinate descent from the
// shipped defaults (2^24 paths in flight, the 6-CTA extend variant, refill
// and leaf thresholds 8, six traversal steps per turn, rows, 4 iteration
// pairs per graph launch): each dimension in turn tries its candidate values
// with the others held at the best so far, and keeps a value only if it
// renders faster.
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
        cfg->refill_min > 32 || cfg->leaf_min < 0 || cfg->leaf_min > 32 || cfg->drain_paths < 0 ||
        cfg->pixel_tile < 0 || cfg->pixel_tile > 1024 || cfg->steps_per_turn < 0 || cfg->steps_per_turn > 8)
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "wavefront configuration out of range");
    ctx->wf_capacity = cfg->capacity;
    ctx->wf_extend_block = cfg->extend_block;
    ctx->wf_shade_block = cfg->shade_block;
    ctx->wf_ctas_per_sm = cfg->ctas_per_sm;
    ctx->wf_iters = cfg->iters_per_graph;
    ctx->trace_refill_min = cfg->refill_min;
    ctx->trace_leaf_min = cfg->leaf_min;
    ctx->wf_drain_paths = cfg->drain_paths;
    ctx->wf_pixel_tile = cfg->pixel_tile;
    ctx->trace_steps = cfg->steps_per_turn;
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
    cudaEvent_t a, b;
    WR_CUDA(ctx, cudaEventCreate(&a));
    WR_CUDA(ctx, cudaEventCreate(&b));
    wr_render_desc d{};
    d.spp = spp_per_trial;
    d.max_path_len = max_path_len;
    d.seed = 0x5eed;
    d.mode = WR_MODE_WAVEFRONT;
    // Mpaths/s of one configuration (a warm-up render builds the engine and
    // captures the graph, the second is timed); < 0 if it cannot run
    auto trial = [&](wr_wavefront_config c) -> double {
        if (wr_set_wavefront_config(ctx, &c) != WR_OK) return -1.0;
        if (wr_render_device(ctx, scene, &d, film.as<float>(), nullptr, ctx->stream) != WR_OK) return -1.0;
        cudaEventRecord(a, ctx->stream);
        const int rc = wr_render_device(ctx, scene, &d, film.as<float>(), nullptr, ctx->stream);
        cudaEventRecord(b, ctx->stream);
        if (rc != WR_OK || cudaEventSynchronize(b) != cudaSuccess) return -1.0;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        return (double)n / 3 * spp_per_trial / (ms * 1e-3) / 1e6;
    };
    // the shipped defaults, then one dimension at a time
    wr_wavefront_config top{1u << 24, 128, 128, 6, 4, 8, 8, 0, 0, 6, 0.0};
    double top_rate = trial(top);
    enum { CAP, CTAS, REFILL, LEAF, STEPS, TILE, ITERS, NDIM };
    const std::vector<int> values[NDIM] = {
        {1 << 22, 1 << 23, 1 << 24}, {6, 7, 8}, {4, 8, 16}, {4, 8, 16}, {1, 2, 4, 6, 8}, {0, 8, 16, 32}, {2, 4, 8}};
    for (int dim = 0; dim < NDIM; dim++) {
        for (int v : values[dim]) {
            wr_wavefront_config c = top;
            int* field = dim == CTAS ? &c.ctas_per_sm
                         : dim == REFILL ? &c.refill_min
                         : dim == LEAF ? &c.leaf_min
                         : dim == STEPS ? &c.steps_per_turn
                         : dim == TILE ? &c.pixel_tile
                         : dim == ITERS ? &c.iters_per_graph
                                        : nullptr;
            if (dim == CAP) {
                if ((uint32_t)v == c.capacity) continue;
                c.capacity = (uint32_t)v;
            } else {
                if (*field == v) continue;
                *field = v;
            }
            const double rate = trial(c);
            if (rate > top_rate) {
                top_rate = rate;
                top = c;
            }
        }
    }
    top.mpaths_per_s = top_rate;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (top_rate < 0) return set_error(ctx, WR_ERR_INTERNAL, "no wavefront configuration ran");
    int rc = wr_set_wavefront_config(ctx, &top);
    if (rc != WR_OK) return rc;
    *best = top;
    return WR_OK;
}

}  // extern "C"
