// render_noalloc.cu — wr_render_noalloc: a render entry point that allocates
// no device memory at all.
//
// Who needs it: callers that may not call cudaMalloc / cudaFree while they
// render.  Examples are real-time loops that forbid allocation because
// cudaMalloc and cudaFree can synchronise the device and stall a frame, and
// applications whose device memory is owned by their own pool or allocator
// (an engine that reserves its device memory up front and lets no library
// allocate behind its back).  wr_render allocates an accumulation film on
// every call; this variant keeps that film in one fixed array in the library
// instead.
//
// The scratch: `g_film` below, a file-scope device array of
// WR_NOALLOC_MAX_PIXELS * 3 floats (12 MiB) plus an error word.  Every GPU
// that loads the library holds it until the process exits.  All calls on a
// device share it, and it keeps the previous call's contents; each call clears
// the part it uses first.  Two calls whose work overlaps on the GPU (for
// example on two streams) therefore race on it: serialise them.
//
// Host code cannot pass `g_film` to a kernel by name (in host code that name
// is a host-side stand-in, not a device address); the device address is
// obtained once per device with cudaGetSymbolAddress, on the first call made
// with that device current.  The address belongs to the device's primary
// context (the one the CUDA runtime uses); calls must be made with that
// context current.
//
// The traversal error word (a per-thread stack that would overflow) is
// cleared by each call and set by its kernels; wr_render_noalloc_status reads
// it back, also without allocating.
#include <cuda_runtime.h>

#include <algorithm>
#include <exception>
#include <mutex>

#include "render_launch.h"
#include "wavefront.h"
#include "wr_context.h"

namespace wr {

static __device__ __align__(256) float g_film[3 * WR_NOALLOC_MAX_PIXELS];
static __device__ __align__(256) unsigned int g_err_word[64];

namespace {

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
float* g_film_addr[MAX_DEVICES] = {};
unsigned int* g_err_addr[MAX_DEVICES] = {};

// device addresses of the scratch arrays on `dev` (set-up on first use)
int scratch_for(wr_ctx* ctx, float** film, unsigned int** err) {
    const int dev = ctx->device;
    if (dev < 0 || dev >= MAX_DEVICES) return set_error(ctx, WR_ERR_UNSUPPORTED, "device ordinal too large");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_film_addr[dev]) {
        void* f = nullptr;
        void* e = nullptr;
        cudaError_t rc = cudaGetSymbolAddress(&f, g_film);
        if (rc != cudaSuccess) return cuda_error(ctx, rc, "cudaGetSymbolAddress(film)");
        rc = cudaGetSymbolAddress(&e, g_err_word);
        if (rc != cudaSuccess) return cuda_error(ctx, rc, "cudaGetSymbolAddress(error word)");
        g_film_addr[dev] = static_cast<float*>(f);
        g_err_addr[dev] = static_cast<unsigned int*>(e);
    }
    *film = g_film_addr[dev];
    *err = g_err_addr[dev];
    return WR_OK;
}

__global__ void k_film_mean(const float* __restrict__ sum, float* __restrict__ out, size_t n, float inv) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = sum[i] * inv;
}

}  // namespace
}  // namespace wr

using namespace wr;

static int render_noalloc_body(wr_ctx* ctx, wr_scene_id id, const wr_render_desc* desc, float* d_rgb_out,
                               void* stream) {
    SceneGPU* sc = find_scene(ctx, id);
    if (!sc) return set_error(ctx, WR_ERR_NOT_FOUND, "no such scene");
    if (desc->mode != WR_MODE_MEGAKERNEL)
        return set_error(ctx, WR_ERR_UNSUPPORTED, "wr_render_noalloc renders with the megakernel (WR_MODE_MEGAKERNEL)");
    if (const char* why = render_flags_problem(desc->flags, desc->mode))
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, why);
    const uint64_t npix = (uint64_t)sc->camera.width * sc->camera.height;
    if (npix > WR_NOALLOC_MAX_PIXELS)
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT,
                         "image larger than the no-allocation film (WR_NOALLOC_MAX_PIXELS = 1048576 pixels)");
    if ((uint64_t)desc->spp_offset + desc->spp > 0xffffffffull)
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "sample index range overflows 32 bits");
    if (!sc->render_data)
        return set_error(ctx, WR_ERR_UNSUPPORTED,
                         "the scene's rendering tables are not resident yet: render it once with wr_render or "
                         "wr_render_device (which build them) before calling wr_render_noalloc");
    const RenderData* rd = static_cast<const RenderData*>(sc->render_data.get());
    // the same refusals as wr_render (for example a heterogeneous medium whose
    // sigma_t is not grey, which delta tracking cannot render)
    if (!RenderDataView::unsupported(rd).empty())
        return set_error(ctx, WR_ERR_UNSUPPORTED, RenderDataView::unsupported(rd));
    const RenderScene& S = RenderDataView::scene(rd);
    WR_CUDA(ctx, cudaSetDevice(ctx->device));
    float* film = nullptr;
    unsigned int* err = nullptr;
    int rc = scratch_for(ctx, &film, &err);
    if (rc != WR_OK) return rc;
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    const size_t n = 3 * (size_t)npix;
    WR_CUDA(ctx, cudaMemsetAsync(film, 0, sizeof(float) * n, s));
    WR_CUDA(ctx, cudaMemsetAsync(err, 0, sizeof(unsigned int), s));
    RenderParams P{};
    P.seed = desc->seed;
    P.max_path_len = desc->max_path_len;
    P.flags = desc->flags;
    P.stack_cap = (int)sc->tree.max_depth + 3;
    const uint64_t per_launch = std::max<uint64_t>(1, (16ull << 20) / std::max<uint64_t>(1, npix));
    for (uint64_t s0 = 0; s0 < desc->spp; s0 += per_launch) {
        P.s0 = (uint32_t)(desc->spp_offset + s0);
        P.s1 = (uint32_t)(desc->spp_offset + std::min<uint64_t>(desc->spp, s0 + per_launch));
        WR_CUDA(ctx, launch_megakernel(S, P, film, nullptr, err, s));
    }
    const float inv = desc->spp ? 1.0f / (float)desc->spp : 0.f;
    k_film_mean<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, s>>>(film, d_rgb_out, n, inv);
    WR_CUDA(ctx, cudaGetLastError());
    return WR_OK;
}

extern "C" int wr_render_noalloc(wr_ctx* ctx, wr_scene_id id, const wr_render_desc* desc, float* d_rgb_out,
                                 void* stream) {
    if (!ctx || !desc || !d_rgb_out) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null argument");
    try {
        return render_noalloc_body(ctx, id, desc, d_rgb_out, stream);
    } catch (const std::exception& ex) {
        return set_error(ctx, WR_ERR_INTERNAL, ex.what());
    }
}

extern "C" int wr_render_noalloc_status(wr_ctx* ctx, void* stream, unsigned int* out_err) {
    if (!ctx || !out_err) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null argument");
    try {
        WR_CUDA(ctx, cudaSetDevice(ctx->device));
        float* film = nullptr;
        unsigned int* err = nullptr;
        int rc = scratch_for(ctx, &film, &err);
        if (rc != WR_OK) return rc;
        cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
        unsigned int word = 0;
        WR_CUDA(ctx, cudaMemcpyAsync(&word, err, sizeof word, cudaMemcpyDeviceToHost, s));
        WR_CUDA(ctx, cudaStreamSynchronize(s));
        *out_err = word;
        return WR_OK;
    } catch (const std::exception& ex) {
        return set_error(ctx, WR_ERR_INTERNAL, ex.what());
    }
}
