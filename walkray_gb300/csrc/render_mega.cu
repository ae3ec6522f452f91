// render_mega.cu — k_megakernel: the plain form of the renderer.  One thread
// per pixel runs whole paths (PathTracer::renderPixels inner loop,
// pathTracer.cpp:21-70: camera ray, samplePath bounce loop, throughput,
// isLegalColor, fixVignetting) for a range of samples and adds the results
// to an FP32 film (sum and optional sum of squares per channel).
#include "render_launch.h"
#include "wr_shade.cuh"

namespace wr {

template <bool STATS, bool MIS>
__global__ void __launch_bounds__(128) k_megakernel(RenderScene S, RenderParams P, float* __restrict__ film,
                                                      float* __restrict__ film2, unsigned int* __restrict__ err) {
    extern __shared__ uint32_t s_stack[];
    uint32_t* stack = s_stack + threadIdx.x;
    const int stride = blockDim.x;
    const uint32_t npix = S.cam.width * S.cam.height;
    const uint32_t pixel = blockIdx.x * blockDim.x + threadIdx.x;
    if (pixel >= npix) return;
    f3 acc = mk(0, 0, 0), acc2 = mk(0, 0, 0);
    const float pf = prune_factor(P.flags);
    const bool nee = (P.flags & WR_RENDER_NEE) != 0;
    for (uint32_t s = P.s0; s < P.s1; s++) {
        PathRng g;
        g.init(P.seed, pixel, s);
        PRay cur = camera_ray(S.cam, pixel, g);
        InsideStack st;
        st.reset(cur.inside);
        f3 color = mk(1, 1, 1), result = mk(0, 0, 0), prev_d = mk(0, 0, 0), lit = mk(0, 0, 0);
        uint32_t depth = 0;
        bool filtered = false;  // the eye ray is traced without a condition (camera.cpp:52)
        bool nee_here = false, has_lr = false;
        float mis_pdf = 0.f;
        LightReq lr;
        for (;;) {
            RayQ q = make_rayq(cur.o, cur.d, S.tree.scene_mag);
            q.pf = pf;
            const Hit h = filtered ? trace_closest<true, true>(S.tree, q, cur.inside, cur.contact, stack, stride,
                                                               P.stack_cap, err)
                                   : trace_closest<false, true>(S.tree, q, -1, -1, stack, stride, P.stack_cap, err);
            if (h.slot < 0 && filtered) {  // a scattered ray that escapes ends with zero radiance
                nee_here = nee;
                break;
            }
            set_hit(S, cur, h);
            filtered = true;
            const bool done = path_advance<MIS>(S, cur, color, prev_d, depth, st, g, P.max_path_len, P.flags,
                                                result, nee_here, mis_pdf, lr, has_lr);
            if (MIS && has_lr) {  // the light connection of WR_RENDER_NEE_MIS, traced inline
                RayQ lq = make_rayq(lr.o, lr.d, S.tree.scene_mag);
                lq.pf = pf;
                const Hit lh =
                    trace_closest<true, true>(S.tree, lq, lr.inside, lr.contact, stack, stride, P.stack_cap, err);
                if (light_req_visible(S, lh, lr)) lit = lit + lr.contrib;
            }
            if (done) break;
        }
        if (nee_here) {  // the connection of the NEE branch, traced inline
            ShadowReq sr;
            if (nee_prepare(S, cur, prev_d, color, g, sr)) {
                RayQ q = make_rayq(sr.o, sr.d, S.tree.scene_mag);
                q.pf = pf;
                const Hit h =
                    trace_closest<true, true>(S.tree, q, sr.inside, sr.contact, stack, stride, P.stack_cap, err);
                if (nee_visible(h, sr.dist)) result = sr.contrib;
            }
        }
        if (!legal(result)) result = mk(0, 0, 0);
        result = result + lit;
        const f3 c = fix_vignetting(S.cam, result, pixel);
        acc = acc + c;
        if (STATS) acc2 = acc2 + vmul(c, c);
    }
    float* f = film + 3 * (size_t)pixel;
    f[0] += acc.x;
    f[1] += acc.y;
    f[2] += acc.z;
    if (STATS) {
        float* f2 = film2 + 3 * (size_t)pixel;
        f2[0] += acc2.x;
        f2[1] += acc2.y;
        f2[2] += acc2.z;
    }
}

cudaError_t launch_megakernel(const RenderScene& S, const RenderParams& P, float* film, float* film2,
                              unsigned int* err, cudaStream_t stream) {
    const int block = 128;
    const size_t smem = (size_t)P.stack_cap * block * sizeof(uint32_t);
    const uint32_t npix = S.cam.width * S.cam.height;
    const int grid = (int)((npix + block - 1) / block);
    const bool mis = (P.flags & WR_RENDER_NEE_MIS) != 0;
    auto kern = film2 ? (mis ? k_megakernel<true, true> : k_megakernel<true, false>)
                      : (mis ? k_megakernel<false, true> : k_megakernel<false, false>);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    kern<<<grid, block, smem, stream>>>(S, P, film, film2, err);
    return cudaGetLastError();
}

}  // namespace wr
