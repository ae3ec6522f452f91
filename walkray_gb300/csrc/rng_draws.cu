// rng_draws.cu — wr_rng_draws: the renderers' device random stream, read
// back for known-answer checks against a host restatement.
//
// Every path of the path tracer owns the counter-based stream of
// wr_device.cuh: draw `dim` of (pixel, sample) under the render seed is word
// dim % 4 of Philox4x32-10 on the counter {dim / 4, sample, pixel, 0}, top
// 24 bits times 2^-24.  The kernel here runs the same PathRng the shading
// code runs, drawing sequentially from 0 up to the requested index (so the
// block caching between consecutive draws is exercised too), and returns the
// raw Philox words of the block the last draw came from.
#include <cuda_runtime.h>

#include <algorithm>
#include <exception>

#include "wr_context.h"
#include "wr_device.cuh"

namespace wr {
namespace {

__global__ void k_rng_draws(uint64_t seed, const uint32_t* __restrict__ pixel, const uint32_t* __restrict__ sample,
                            const uint32_t* __restrict__ dim, uint64_t n, uint4* __restrict__ words,
                            float* __restrict__ draws) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    PathRng g;
    g.init(seed, pixel[i], sample[i]);
    float v = 0.f;
    for (uint32_t d = 0; d <= dim[i]; d++) v = g.next();
    draws[i] = v;
    words[i] = philox_block(dim[i] >> 2, sample[i], pixel[i], (uint32_t)seed, (uint32_t)(seed >> 32));
}

}  // namespace
}  // namespace wr

using namespace wr;

extern "C" int wr_rng_draws(wr_ctx* ctx, uint64_t seed, const uint32_t* pixel, const uint32_t* sample,
                            const uint32_t* dim, uint64_t n, uint32_t* words, float* draws) {
    if (!ctx) return WR_ERR_INVALID_ARGUMENT;
    if (n == 0) return WR_OK;
    if (!pixel || !sample || !dim || !words || !draws) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null argument");
    if (n > (1ull << 24)) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "at most 2^24 draws per call");
    for (uint64_t i = 0; i < n; i++)
        if (dim[i] >= (1u << 16)) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "draw index above 65535");
    try {
        WR_CUDA(ctx, cudaSetDevice(ctx->device));
        DeviceBuffer buf;
        const size_t in_bytes = 3 * sizeof(uint32_t) * n, out_bytes = (sizeof(uint4) + sizeof(float)) * n;
        WR_CUDA(ctx, buf.reserve(in_bytes + out_bytes + 64));
        uint32_t* d_px = buf.as<uint32_t>();
        uint32_t* d_sm = d_px + n;
        uint32_t* d_dm = d_sm + n;
        uint4* d_words = reinterpret_cast<uint4*>(buf.as<char>() + ((in_bytes + 15) & ~size_t(15)));
        float* d_draws = reinterpret_cast<float*>(d_words + n);
        cudaStream_t s = ctx->stream;
        WR_CUDA(ctx, cudaMemcpyAsync(d_px, pixel, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s));
        WR_CUDA(ctx, cudaMemcpyAsync(d_sm, sample, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s));
        WR_CUDA(ctx, cudaMemcpyAsync(d_dm, dim, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s));
        const int block = 128;
        k_rng_draws<<<(unsigned)((n + block - 1) / block), block, 0, s>>>(seed, d_px, d_sm, d_dm, n, d_words,
                                                                          d_draws);
        WR_CUDA(ctx, cudaGetLastError());
        ctx->kernel_launches++;
        WR_CUDA(ctx, cudaMemcpyAsync(words, d_words, sizeof(uint4) * n, cudaMemcpyDeviceToHost, s));
        WR_CUDA(ctx, cudaMemcpyAsync(draws, d_draws, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
        WR_CUDA(ctx, cudaStreamSynchronize(s));
        return WR_OK;
    } catch (const std::exception& ex) {
        return set_error(ctx, WR_ERR_INTERNAL, ex.what());
    }
}
