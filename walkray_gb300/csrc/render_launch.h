// render_launch.h — host-side launchers of the rendering kernels.
#pragma once

#include <cuda_runtime.h>

#include "wr_shade.cuh"

struct wr_ctx;

namespace wr {

constexpr uint32_t RENDER_KNOWN_FLAGS =
    WR_RENDER_NEE | WR_RENDER_EXACT_TRAVERSAL | WR_RENDER_NEE_MIS | WR_RENDER_PHONG_MIRROR;
// flags of the unidirectional path tracer only
constexpr uint32_t RENDER_PT_ONLY_FLAGS = WR_RENDER_NEE_MIS | WR_RENDER_PHONG_MIRROR;

// why a set of render flags cannot be used with a mode (nullptr: it can)
inline const char* render_flags_problem(uint32_t flags, uint32_t mode) {
    if (flags & ~RENDER_KNOWN_FLAGS) return "unknown render flags";
    if ((flags & WR_RENDER_NEE) && (flags & WR_RENDER_NEE_MIS))
        return "WR_RENDER_NEE (the reference's branch) and WR_RENDER_NEE_MIS exclude each other";
    if ((flags & RENDER_PT_ONLY_FLAGS) && mode != WR_MODE_MEGAKERNEL && mode != WR_MODE_WAVEFRONT)
        return "WR_RENDER_NEE_MIS and WR_RENDER_PHONG_MIRROR apply to the path tracing modes only";
    return nullptr;
}

// factor on the closest hit's distance beyond which a box is skipped
__host__ __device__ __forceinline__ float prune_factor(uint32_t flags) {
    return (flags & WR_RENDER_EXACT_TRAVERSAL) ? INFINITY : 1.001f;
}

struct RenderParams {
    uint64_t seed;
    uint32_t s0, s1;          // sample range [s0, s1)
    uint32_t max_path_len;    // MCRenderer maxPathLen
    uint32_t flags;
    int stack_cap;            // traversal stack entries per thread (tree depth + 3)
};

// plain megakernel: film[3*p+c] += sum over samples of the pixel colour
// (film2 != NULL: also the sum of squares)
cudaError_t launch_megakernel(const RenderScene& S, const RenderParams& P, float* film, float* film2,
                              unsigned int* err, cudaStream_t stream);

// WR_MODE_BIDIRECTIONAL, WR_MODE_VCM and WR_MODE_PHOTON_MAP (bpt.cu): adds
// samples [spp_offset, spp_offset + spp) of every pixel to d_sum (and their
// squares to d_sumsq, may be NULL); `base_radius` is the merge / photon
// radius of the first iteration; `hetero`: the scene has a heterogeneous
// medium (its integrals are marched inside the weights); `media`: it has a
// participating medium (photon mapping's volume photons and marched segments)
enum : int { BIDIR_BPT = 0, BIDIR_VCM = 1, BIDIR_PHOTON_MAP = 2 };
int render_bidirectional(wr_ctx* ctx, const RenderScene& S, const RenderParams& P, uint32_t spp_offset, uint32_t spp,
                         float* d_sum, float* d_sumsq, unsigned int* err, cudaStream_t stream, int kind = BIDIR_BPT,
                         float base_radius = 0.01f, bool hetero = false, bool media = false);

}  // namespace wr
