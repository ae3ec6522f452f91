// render_api.cpp — wr_render / wr_render_device: per-scene rendering tables
// on the device and the launch loop over sample chunks.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>

#include "render_launch.h"
#include "wavefront.h"
#include "wr_context.h"

namespace wr {

struct RenderData {
    RenderScene S{};
    DeviceBuffer objs, tri_slot, light_obj, light_thresh, obj_area, pick_prob, tri_thresh, grids, light_inside;
    std::vector<std::unique_ptr<DeviceBuffer>> grid_data;
    std::string unsupported;  // non-empty: this scene cannot be rendered (why)
    bool has_media = false;
    bool has_hetero = false;
};

namespace {

// KDTree::intersect(ray, tri) restated for host set-up queries (kdtree.cpp:279-301)
float host_tri(f3 v0, f3 v1, f3 v2, f3 o, f3 d) {
    const f3 l0 = v1 - v0, l1 = v2 - v1, l2 = v0 - v2;
    const float s0 = dot(d, cross(l0, v0 - o)), s1 = dot(d, cross(l1, v1 - o)), s2 = dot(d, cross(l2, v2 - o));
    const bool pos = s0 >= 0 && s1 >= 0 && s2 >= 0, neg = s0 <= 0 && s1 <= 0 && s2 <= 0;
    if (!pos && !neg) return -1.f;
    const f3 n = normalize(cross(l0, l1));
    const float dd = dot(n, d);
    if (dd == 0.f) return -1.f;
    const float t = dot(n, v2 - o) / dd;
    return t >= 0.f ? t : -1.f;
}

// Scene::findInsideObject (scene.cpp:115-144) for one ray, skipping object
// `skip`, each object's closest hit found by brute force over its triangles
int host_find_inside(const SceneGPU& sc, f3 o, f3 d, int skip = -1) {
    auto closest = [&](int obj, f3 dir, f3* nrm) -> bool {
        const wr_object_desc& m = sc.objects[obj];
        float best = -1.f;
        for (uint32_t t = 0; t < m.tri_count; t++) {
            const uint32_t* lt = &sc.triangles[3 * ((size_t)m.tri_begin + t)];
            const float* V = &sc.vertices[3 * (size_t)m.vert_begin];
            f3 v0 = mk(V[3 * lt[0]], V[3 * lt[0] + 1], V[3 * lt[0] + 2]);
            f3 v1 = mk(V[3 * lt[1]], V[3 * lt[1] + 1], V[3 * lt[1] + 2]);
            f3 v2 = mk(V[3 * lt[2]], V[3 * lt[2] + 1], V[3 * lt[2] + 2]);
            float dist = host_tri(v0, v1, v2, o, dir);
            if (dist >= 0 && (dist < best || best < 0)) {
                best = dist;
                *nrm = normalize(cross(v1 - v0, v2 - v0));
            }
        }
        return best >= 0;
    };
    for (int i = (int)sc.objects.size() - 1; i >= 0; i--) {
        if (i == skip) continue;
        f3 n;
        if (!closest(i, -d, &n) || dot(n, -d) < 0) continue;
        if (!closest(i, d, &n) || dot(n, d) < 0) continue;
        return i;
    }
    return -1;
}

template <class T>
cudaError_t upload(DeviceBuffer& b, const std::vector<T>& v) {
    cudaError_t e = b.reserve(sizeof(T) * std::max<size_t>(1, v.size()));
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpy(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice);
}

}  // namespace

// camera frame (camera.cpp:7-11) in FP32 with the same operations, at a given
// resolution; the inside object of camera rays (camera.cpp:56) is taken on
// the image-centre ray: for closed meshes it does not depend on the pixel
CamParams camera_params(const SceneGPU& sc, uint32_t width, uint32_t height, float ipd) {
    CamParams C{};
    const wr_camera_desc& c = sc.camera;
    C.pos = mk(c.position[0], c.position[1], c.position[2]);
    C.focus = mk(c.focus[0], c.focus[1], c.focus[2]);
    const f3 up = mk(c.up[0], c.up[1], c.up[2]);
    C.front = normalize(C.focus - C.pos);
    C.right = normalize(cross(C.front, up));
    C.top = cross(C.right, C.front);
    C.width = width;
    C.height = height;
    C.ipd = ipd;
    C.lens_radius = c.lens_radius;
    C.focal_dist = c.focal_dist;
    C.inside = host_find_inside(sc, C.pos, normalize(C.front * C.ipd));
    return C;
}

// builds the scene's rendering tables once (lazily, on first render)
int prepare_render(wr_ctx* ctx, SceneGPU* sc, RenderData** out) {
    if (sc->render_data) {
        *out = static_cast<RenderData*>(sc->render_data.get());
        return WR_OK;
    }
    auto rd = std::make_shared<RenderData>();
    RenderScene& S = rd->S;
    S.tree = sc->tree;
    S.num_objs = (uint32_t)sc->objects.size();
    WR_CUDA(ctx, upload(rd->objs, sc->objects));
    S.objs = rd->objs.as<wr_object_desc>();
    // triangle slots: rebuild the mapping from the resident records
    {
        std::vector<TriRec> recs(sc->tree.num_slots);
        if (!recs.empty())
            WR_CUDA(ctx, cudaMemcpy(recs.data(), sc->tree.tris, sizeof(TriRec) * recs.size(), cudaMemcpyDeviceToHost));
        std::vector<uint32_t> slot_of(sc->info.num_triangles, 0u);
        for (uint32_t s = 0; s < recs.size(); s++) {
            uint32_t gid;
            std::memcpy(&gid, &recs[s].v0.w, 4);
            if (gid < slot_of.size()) slot_of[gid] = s;
        }
        WR_CUDA(ctx, upload(rd->tri_slot, slot_of));
        S.tri_slot = rd->tri_slot.as<uint32_t>();
    }
    // camera frame (camera.cpp:7-11), computed once in FP32 with the same operations
    S.cam = camera_params(*sc, sc->camera.width, sc->camera.height, sc->camera.image_plane_dist);
    if (S.cam.width == 0 || S.cam.height == 0) rd->unsupported = "camera has no pixels";
    // lights (Scene::prepareForLightSampling, SurfaceSampler::prepareForSampling, Mesh::getTriangleArea)
    std::vector<int> light_obj;
    std::vector<float> light_thresh, obj_area(sc->objects.size(), 0.f), pick(sc->objects.size(), 0.f),
        tri_thresh(sc->info.num_triangles, 0.f);
    float bound = 0.f;
    for (uint32_t o = 0; o < sc->objects.size(); o++) {
        const wr_object_desc& m = sc->objects[o];
        if (m.type != WR_MAT_EMISSIVE) continue;
        float area = 0.f;
        const float* V = &sc->vertices[3 * (size_t)m.vert_begin];
        for (uint32_t t = 0; t < m.tri_count; t++) {
            const uint32_t* lt = &sc->triangles[3 * ((size_t)m.tri_begin + t)];
            f3 v0 = mk(V[3 * lt[0]], V[3 * lt[0] + 1], V[3 * lt[0] + 2]);
            f3 v1 = mk(V[3 * lt[1]], V[3 * lt[1] + 1], V[3 * lt[1] + 2]);
            f3 v2 = mk(V[3 * lt[2]], V[3 * lt[2] + 1], V[3 * lt[2] + 2]);
            area += length(cross(v1 - v0, v2 - v1)) / 2.f;
            tri_thresh[m.tri_begin + t] = area;
        }
        obj_area[o] = area;
        bound += area;
        light_obj.push_back((int)o);
        light_thresh.push_back(bound);
    }
    for (int o : light_obj) pick[o] = obj_area[o] / bound;
    // the object enclosing each emitter (the inside object of its emitted rays,
    // abstractObj.cpp:39), taken on its first triangle's centroid along the
    // face normal: for closed, properly nested meshes it does not depend on the point
    std::vector<int> light_inside(sc->objects.size() + 1, -1);
    for (int o : light_obj) {
        const wr_object_desc& m = sc->objects[o];
        if (!m.tri_count) continue;
        const uint32_t* lt = &sc->triangles[3 * (size_t)m.tri_begin];
        const float* V = &sc->vertices[3 * (size_t)m.vert_begin];
        f3 v0 = mk(V[3 * lt[0]], V[3 * lt[0] + 1], V[3 * lt[0] + 2]);
        f3 v1 = mk(V[3 * lt[1]], V[3 * lt[1] + 1], V[3 * lt[1] + 2]);
        f3 v2 = mk(V[3 * lt[2]], V[3 * lt[2] + 1], V[3 * lt[2] + 2]);
        light_inside[o] = host_find_inside(*sc, (v0 + v1 + v2) * (1.f / 3.f), normalize(cross(v1 - v0, v2 - v0)), o);
    }
    WR_CUDA(ctx, upload(rd->light_inside, light_inside));
    S.light_inside = rd->light_inside.as<int>();
    S.nlights = (uint32_t)light_obj.size();
    S.light_area = bound;
    WR_CUDA(ctx, upload(rd->light_obj, light_obj));
    WR_CUDA(ctx, upload(rd->light_thresh, light_thresh));
    WR_CUDA(ctx, upload(rd->obj_area, obj_area));
    WR_CUDA(ctx, upload(rd->pick_prob, pick));
    WR_CUDA(ctx, upload(rd->tri_thresh, tri_thresh));
    S.light_obj = rd->light_obj.as<int>();
    S.light_thresh = rd->light_thresh.as<float>();
    S.obj_area = rd->obj_area.as<float>();
    S.pick_prob = rd->pick_prob.as<float>();
    S.tri_thresh = rd->tri_thresh.as<float>();
    // density grids
    std::vector<GridDev> gd(sc->grids.size());
    for (size_t g = 0; g < sc->grids.size(); g++) {
        const wr_grid_desc& G = sc->grids[g];
        auto buf = std::make_unique<DeviceBuffer>();
        WR_CUDA(ctx, upload(*buf, sc->grid_data[g]));
        gd[g].nx = G.nx;
        gd[g].ny = G.ny;
        gd[g].nz = G.nz;
        for (int k = 0; k < 3; k++) {
            gd[g].p0[k] = G.p0[k];
            gd[g].p1[k] = G.p1[k];
        }
        float mx = 0.f;
        for (float v : sc->grid_data[g]) mx = std::max(mx, v);
        gd[g].majorant = mx;
        gd[g].data = buf->as<float>();
        rd->grid_data.push_back(std::move(buf));
    }
    WR_CUDA(ctx, upload(rd->grids, gd));
    S.grids = rd->grids.as<GridDev>();
    for (const wr_object_desc& m : sc->objects) {
        if (m.type == WR_MAT_HOMOGENEOUS || m.type == WR_MAT_HETEROGENEOUS) rd->has_media = true;
        if (m.type == WR_MAT_HETEROGENEOUS) rd->has_hetero = true;
    }
    for (const wr_object_desc& m : sc->objects)
        if (m.type == WR_MAT_HETEROGENEOUS &&
            !(m.sigma_s[0] + m.sigma_a[0] == m.sigma_s[1] + m.sigma_a[1] &&
              m.sigma_s[0] + m.sigma_a[0] == m.sigma_s[2] + m.sigma_a[2]))
            rd->unsupported = "heterogeneous media need a grey sigma_t (equal channels) for delta tracking";
    sc->render_data = rd;
    *out = rd.get();
    return WR_OK;
}

}  // namespace wr

using namespace wr;

extern "C" {

int wr_render_device(wr_ctx* ctx, wr_scene_id id, const wr_render_desc* desc, float* d_sum, float* d_sumsq,
                     void* stream) {
    if (!ctx || !desc || !d_sum) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null argument");
    SceneGPU* sc = find_scene(ctx, id);
    if (!sc) return set_error(ctx, WR_ERR_NOT_FOUND, "no such scene");
    if (desc->mode != WR_MODE_MEGAKERNEL && desc->mode != WR_MODE_WAVEFRONT && desc->mode != WR_MODE_BIDIRECTIONAL &&
        desc->mode != WR_MODE_VCM && desc->mode != WR_MODE_PHOTON_MAP)
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "unknown render mode");
    if ((desc->mode == WR_MODE_VCM || desc->mode == WR_MODE_PHOTON_MAP) && !(desc->radius >= 0.f && desc->radius < 1e30f))
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "merge / photon radius must be finite and >= 0");
    if (const char* why = render_flags_problem(desc->flags, desc->mode))
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, why);
    if ((uint64_t)desc->spp_offset + desc->spp > 0xffffffffull)
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "sample index range overflows 32 bits");
    try {
        WR_CUDA(ctx, cudaSetDevice(ctx->device));
        RenderData* rd = nullptr;
        int rc = prepare_render(ctx, sc, &rd);
        if (rc != WR_OK) return rc;
        if (!rd->unsupported.empty()) return set_error(ctx, WR_ERR_UNSUPPORTED, rd->unsupported);
        if (desc->spp == 0) return WR_OK;
        cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
        unsigned int* err = reinterpret_cast<unsigned int*>(ctx->scratch_words.as<unsigned long long>() + 1);
        RenderParams P{};
        P.seed = desc->seed;
        P.max_path_len = desc->max_path_len;
        P.flags = desc->flags;
        P.stack_cap = (int)sc->tree.max_depth + 3;
        const uint64_t npix = (uint64_t)rd->S.cam.width * rd->S.cam.height;
        if (desc->mode == WR_MODE_BIDIRECTIONAL || desc->mode == WR_MODE_VCM || desc->mode == WR_MODE_PHOTON_MAP) {
            if (desc->mode == WR_MODE_PHOTON_MAP && rd->has_media)  // the march step of each medium's segments
                for (const wr_object_desc& m : sc->objects)
                    if ((m.type == WR_MAT_HOMOGENEOUS || m.type == WR_MAT_HETEROGENEOUS) &&
                        !(m.step_size > 0.f && m.step_size < 3.0e38f))
                        return set_error(ctx, WR_ERR_INVALID_ARGUMENT,
                                         "photon-mapping mode: a medium's step_size must be positive and finite");
            if (desc->flags & WR_RENDER_NEE)
                return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "bidirectional / VCM / photon-mapping mode has no NEE switch");
            const int kind = desc->mode == WR_MODE_VCM ? BIDIR_VCM
                           : desc->mode == WR_MODE_PHOTON_MAP ? BIDIR_PHOTON_MAP : BIDIR_BPT;
            return render_bidirectional(ctx, rd->S, P, desc->spp_offset, desc->spp, d_sum, d_sumsq, err, s, kind,
                                        desc->radius > 0.f ? desc->radius : 0.01f, rd->has_hetero, rd->has_media);
        }
        if (desc->mode == WR_MODE_WAVEFRONT) {
            rc = render_wavefront(ctx, *rd, P, desc->spp_offset, desc->spp, d_sum, d_sumsq, s);
            if (rc != WR_OK) return rc;
            return WR_OK;
        }
        const uint64_t per_launch = std::max<uint64_t>(1, (16ull << 20) / std::max<uint64_t>(1, npix));
        for (uint64_t s0 = 0; s0 < desc->spp; s0 += per_launch) {
            P.s0 = (uint32_t)(desc->spp_offset + s0);
            P.s1 = (uint32_t)(desc->spp_offset + std::min<uint64_t>(desc->spp, s0 + per_launch));
            WR_CUDA(ctx, launch_megakernel(rd->S, P, d_sum, d_sumsq, err, s));
            ctx->kernel_launches++;
        }
        return WR_OK;
    } catch (const std::exception& ex) {
        return set_error(ctx, WR_ERR_INTERNAL, ex.what());
    }
}

// the film's sum over samples times 1/spp, in place (grid-stride)
__global__ void k_scale(float* __restrict__ a, size_t n, float s) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        a[i] *= s;
}

int wr_render(wr_ctx* ctx, wr_scene_id id, const wr_render_desc* desc, float* rgb_out) {
    if (!ctx || !desc || !rgb_out) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null argument");
    SceneGPU* sc = find_scene(ctx, id);
    if (!sc) return set_error(ctx, WR_ERR_NOT_FOUND, "no such scene");
    try {
        WR_CUDA(ctx, cudaSetDevice(ctx->device));
        const size_t n = 3ull * sc->camera.width * sc->camera.height;
        // the context's film (grown when a larger image comes; a context is
        // used by one thread at a time), the mean taken on the device
        DeviceBuffer& film = ctx->film;
        WR_CUDA(ctx, film.reserve(sizeof(float) * std::max<size_t>(n, 1)));
        cudaStream_t s = ctx->stream;
        unsigned int* err = reinterpret_cast<unsigned int*>(ctx->scratch_words.as<unsigned long long>() + 1);
        WR_CUDA(ctx, cudaMemsetAsync(err, 0, sizeof(unsigned int), s));
        WR_CUDA(ctx, cudaMemsetAsync(film.p, 0, sizeof(float) * n, s));
        int rc = wr_render_device(ctx, id, desc, film.as<float>(), nullptr, s);
        if (rc != WR_OK) return rc;
        const float inv = desc->spp ? 1.0f / (float)desc->spp : 0.f;
        k_scale<<<(unsigned)std::min<size_t>((n + 255) / 256, 65535), 256, 0, s>>>(film.as<float>(), n, inv);
        WR_CUDA(ctx, cudaGetLastError());
        ctx->kernel_launches++;
        WR_CUDA(ctx, cudaMemcpyAsync(rgb_out, film.p, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
        unsigned int herr = 0;
        WR_CUDA(ctx, cudaMemcpyAsync(&herr, err, sizeof herr, cudaMemcpyDeviceToHost, s));
        WR_CUDA(ctx, cudaStreamSynchronize(s));
        if (herr) return set_error(ctx, WR_ERR_INTERNAL, "traversal stack overflow");
        return WR_OK;
    } catch (const std::exception& ex) {
        return set_error(ctx, WR_ERR_INTERNAL, ex.what());
    }
}

// out = sum * s (grid-stride)
__global__ void k_scale_to(const float* __restrict__ a, float* __restrict__ out, size_t n, float s) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = a[i] * s;
}

int wr_render_progressive(wr_ctx* ctx, wr_scene_id id, const wr_render_desc* desc, uint32_t chunk_spp,
                          float* rgb_out, wr_progress_fn progress, void* user, uint32_t* spp_done) {
    if (!ctx || !desc || !rgb_out) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null argument");
    if (spp_done) *spp_done = 0;
    SceneGPU* sc = find_scene(ctx, id);
    if (!sc) return set_error(ctx, WR_ERR_NOT_FOUND, "no such scene");
    try {
        WR_CUDA(ctx, cudaSetDevice(ctx->device));
        const size_t npix = (size_t)sc->camera.width * sc->camera.height, n = 3 * npix;
        if (chunk_spp == 0) chunk_spp = (uint32_t)std::max<size_t>(1, (16ull << 20) / std::max<size_t>(1, npix));
        // the running sum stays on the device between chunks; the mean of the
        // samples so far is taken into a second buffer and copied out
        DeviceBuffer& film = ctx->film;
        WR_CUDA(ctx, film.reserve(sizeof(float) * std::max<size_t>(2 * n, 1)));
        float* sum = film.as<float>();
        float* mean = sum + n;
        cudaStream_t s = ctx->stream;
        unsigned int* err = reinterpret_cast<unsigned int*>(ctx->scratch_words.as<unsigned long long>() + 1);
        WR_CUDA(ctx, cudaMemsetAsync(err, 0, sizeof(unsigned int), s));
        WR_CUDA(ctx, cudaMemsetAsync(sum, 0, sizeof(float) * n, s));
        uint32_t done = 0;
        while (done < desc->spp) {
            wr_render_desc d = *desc;
            d.spp_offset = desc->spp_offset + done;
            d.spp = std::min<uint32_t>(chunk_spp, desc->spp - done);
            int rc = wr_render_device(ctx, id, &d, sum, nullptr, s);
            if (rc != WR_OK) return rc;
            done += d.spp;
            k_scale_to<<<(unsigned)std::min<size_t>((n + 255) / 256, 65535), 256, 0, s>>>(sum, mean, n,
                                                                                       1.0f / (float)done);
            WR_CUDA(ctx, cudaGetLastError());
            ctx->kernel_launches++;
            WR_CUDA(ctx, cudaMemcpyAsync(rgb_out, mean, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
            unsigned int herr = 0;
            WR_CUDA(ctx, cudaMemcpyAsync(&herr, err, sizeof herr, cudaMemcpyDeviceToHost, s));
            WR_CUDA(ctx, cudaStreamSynchronize(s));
            if (herr) return set_error(ctx, WR_ERR_INTERNAL, "traversal stack overflow");
            if (spp_done) *spp_done = done;
            if (progress && progress(user, rgb_out, done) != 0) break;
        }
        return WR_OK;
    } catch (const std::exception& ex) {
        return set_error(ctx, WR_ERR_INTERNAL, ex.what());
    }
}

}  // extern "C"

namespace wr {

const RenderScene& RenderDataView::scene(const RenderData* rd) { return rd->S; }
const std::string& RenderDataView::unsupported(const RenderData* rd) { return rd->unsupported; }

// the wavefront configuration: what wr_autotune picked for this context, else defaults
WfConfig wf_tuned_config(wr_ctx* ctx) {
    WfConfig c;
    if (ctx->wf_capacity) c.capacity = ctx->wf_capacity;
    if (ctx->wf_extend_block) c.extend_block = ctx->wf_extend_block;
    if (ctx->wf_shade_block) c.shade_block = ctx->wf_shade_block;
    if (ctx->wf_ctas_per_sm) c.ctas_per_sm = ctx->wf_ctas_per_sm;
    if (ctx->wf_iters) c.iters_per_graph = ctx->wf_iters;
    c.trace = trace_tune_of(ctx);
    c.drain_paths = ctx->wf_drain_paths;
    c.pixel_tile = ctx->wf_pixel_tile;
    return c;
}

}  // namespace wr

namespace wr {
int profile_wavefront(wr_ctx* ctx, RenderData& rd, const RenderParams& P, uint32_t spp_offset, uint32_t spp,
                      float* film, wr_render_profile* out);
}

extern "C" int wr_profile_render(wr_ctx* ctx, wr_scene_id id, const wr_render_desc* desc, float* d_sum,
                                 wr_render_profile* out) {
    if (!ctx || !desc || !d_sum || !out) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null argument");
    SceneGPU* sc = find_scene(ctx, id);
    if (!sc) return set_error(ctx, WR_ERR_NOT_FOUND, "no such scene");
    if (const char* why = render_flags_problem(desc->flags, WR_MODE_WAVEFRONT))
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, why);
    WR_CUDA(ctx, cudaSetDevice(ctx->device));
    RenderData* rd = nullptr;
    int rc = prepare_render(ctx, sc, &rd);
    if (rc != WR_OK) return rc;
    if (!rd->unsupported.empty()) return set_error(ctx, WR_ERR_UNSUPPORTED, rd->unsupported);
    RenderParams P{};
    P.seed = desc->seed;
    P.max_path_len = desc->max_path_len;
    P.flags = desc->flags;
    P.stack_cap = (int)sc->tree.max_depth + 3;
    return profile_wavefront(ctx, *rd, P, desc->spp_offset, desc->spp, d_sum, out);
}
