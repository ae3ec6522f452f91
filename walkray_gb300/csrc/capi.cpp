// capi.cpp — the extern "C" boundary (include/walkray.h): contexts, scene
// residency and the traversal entry points.  No exception crosses it; every
// failure becomes a status code plus wr_last_error().
#include <algorithm>
#include <chrono>
#include <cstring>
#include <new>
#include <stdexcept>

#include "kdtree_build.h"
#include "trace_launch.h"
#include "wr_context.h"

namespace wr {

int set_error(wr_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int cuda_error(wr_ctx* ctx, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();  // clear a sticky-free error so the context stays usable
    return set_error(ctx, e == cudaErrorMemoryAllocation ? WR_ERR_OUT_OF_MEMORY : WR_ERR_CUDA, m);
}

SceneGPU* find_scene(wr_ctx* ctx, wr_scene_id id) {
    auto it = ctx->scenes.find(id);
    return it == ctx->scenes.end() ? nullptr : it->second.get();
}

}  // namespace wr

using namespace wr;

#define WR_GUARD_BEGIN try {
#define WR_GUARD_END                                                            \
    }                                                                           \
    catch (const std::bad_alloc&) {                                             \
        return set_error(ctx, WR_ERR_OUT_OF_MEMORY, "host allocation failed");  \
    }                                                                           \
    catch (const std::exception& ex) {                                          \
        return set_error(ctx, WR_ERR_INTERNAL, ex.what());                      \
    }                                                                           \
    catch (...) {                                                               \
        return set_error(ctx, WR_ERR_INTERNAL, "unknown exception");            \
    }

extern "C" {

int wr_get_abi_version(uint32_t* version) {
    if (!version) return WR_ERR_INVALID_ARGUMENT;
    *version = WR_ABI_VERSION;
    return WR_OK;
}

int wr_ctx_create(const wr_ctx_desc* desc, wr_ctx** out) {
    if (!out) return WR_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    wr_ctx* ctx = nullptr;
    try {
        ctx = new wr_ctx();
    } catch (...) {
        return WR_ERR_OUT_OF_MEMORY;
    }
    ctx->device = desc ? desc->device : 0;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0 || ctx->device < 0 || ctx->device >= ndev) {
        cudaGetLastError();
        delete ctx;
        return e == cudaSuccess ? WR_ERR_INVALID_ARGUMENT : WR_ERR_CUDA;
    }
    if ((e = cudaSetDevice(ctx->device)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = ctx->scratch_words.reserve(256)) != cudaSuccess) {
        cudaGetLastError();
        delete ctx;
        return WR_ERR_CUDA;
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    ctx->memory_budget = (desc && desc->device_memory_budget) ? desc->device_memory_budget : (uint64_t)(free_b * 0.9);
    ctx->trace_prune = !(desc && (desc->flags & WR_CTX_EXACT_TRAVERSAL));
    *out = ctx;
    return WR_OK;
}

int wr_ctx_destroy(wr_ctx* ctx) {
    if (!ctx) return WR_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->serving.reset();
    ctx->wavefront.reset();
    ctx->scenes.clear();
    ctx->rays.release();
    ctx->hits.release();
    ctx->inside.release();
    ctx->contact.release();
    ctx->scratch_words.release();
    ctx->film.release();
    if (ctx->copy_in) cudaStreamSynchronize(ctx->copy_in);
    if (ctx->copy_out) cudaStreamSynchronize(ctx->copy_out);
    for (cudaEvent_t& e : ctx->pipe_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->copy_in) cudaStreamDestroy(ctx->copy_in);
    if (ctx->copy_out) cudaStreamDestroy(ctx->copy_out);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return WR_OK;
}

const char* wr_last_error(const wr_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int wr_kernel_launches(const wr_ctx* ctx, uint64_t* out) {
    if (!ctx || !out) return WR_ERR_INVALID_ARGUMENT;
    *out = ctx->kernel_launches;
    return WR_OK;
}

int wr_scene_upload(wr_ctx* ctx, const wr_scene_desc* d, wr_scene_id* out) {
    if (!ctx || !d || !out) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null argument");
    if ((d->num_objects && !d->objects) || (d->num_vertices && !d->vertices) || (d->num_triangles && !d->triangles) ||
        (d->num_grids && !d->grids))
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null scene array");
    // the bidirectional renderers' vertex records hold an object id in 28 bits
    if (d->num_objects > (1u << 27)) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "more than 2^27 objects");
    WR_GUARD_BEGIN
    // validate object ranges (Scene::buildKDTree trusts its objects; this boundary does not)
    uint64_t tri_sum = 0;
    for (uint32_t o = 0; o < d->num_objects; o++) {
        const wr_object_desc& m = d->objects[o];
        if (m.type > WR_MAT_REFLECTIVE) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "unknown object type");
        if ((uint64_t)m.vert_begin + m.vert_count > d->num_vertices ||
            (uint64_t)m.tri_begin + m.tri_count > d->num_triangles)
            return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "object range outside the scene arrays");
        if (m.tri_begin != tri_sum)
            return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "objects must list triangles contiguously in order");
        tri_sum += m.tri_count;
        for (uint32_t t = 0; t < m.tri_count; t++)
            for (int k = 0; k < 3; k++)
                if (d->triangles[3 * ((size_t)m.tri_begin + t) + k] >= m.vert_count)
                    return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "triangle vertex index outside its object");
        if (m.type == WR_MAT_HETEROGENEOUS && m.grid_index >= d->num_grids)
            return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "heterogeneous medium without a grid");
    }
    if (tri_sum != d->num_triangles) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "triangles not covered by objects");

    auto sc = std::make_unique<SceneGPU>();
    sc->objects.assign(d->objects, d->objects + d->num_objects);
    sc->vertices.assign(d->vertices, d->vertices + 3 * (size_t)d->num_vertices);
    sc->triangles.assign(d->triangles, d->triangles + 3 * (size_t)d->num_triangles);
    sc->camera = d->camera;
    for (uint32_t g = 0; g < d->num_grids; g++) {
        const wr_grid_desc& gd = d->grids[g];
        size_t cnt = (size_t)gd.nx * gd.ny * gd.nz;
        if (!gd.density || cnt == 0) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "empty density grid");
        sc->grid_data.emplace_back(gd.density, gd.density + cnt);
        sc->grids.push_back(gd);
        sc->grids.back().density = sc->grid_data.back().data();
    }
    // global vertex indices (the vi_offset renumbering of Scene::buildKDTree, scene.cpp:20-44)
    const uint32_t nt = d->num_triangles;
    std::vector<uint32_t> gtris(3 * (size_t)nt);
    sc->tri_obj.resize(nt);
    sc->tri_local.resize(nt);
    for (uint32_t o = 0; o < d->num_objects; o++) {
        const wr_object_desc& m = d->objects[o];
        for (uint32_t t = 0; t < m.tri_count; t++) {
            size_t gi = (size_t)m.tri_begin + t;
            for (int k = 0; k < 3; k++) gtris[3 * gi + k] = d->triangles[3 * gi + k] + m.vert_begin;
            sc->tri_obj[gi] = (int32_t)o;
            sc->tri_local[gi] = t;
        }
    }
    auto t0 = std::chrono::steady_clock::now();
    HostTree ht = build_reference_tree(d->vertices, d->num_vertices, gtris.data(), nt, 0);
    DeviceLayout L = layout_for_device(ht, d->vertices, d->num_vertices, gtris.data(), sc->tri_obj.data(),
                                       sc->tri_local.data());
    auto t1 = std::chrono::steady_clock::now();
    WR_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t pb = sizeof(NodePair) * (L.pairs.size() ? L.pairs.size() : 1);
    const size_t tb = sizeof(TriRec) * (L.slots.size() ? L.slots.size() : 1);
    WR_CUDA(ctx, sc->pairs.reserve(pb));
    WR_CUDA(ctx, sc->tris.reserve(tb));
    if (!L.pairs.empty())
        WR_CUDA(ctx, cudaMemcpy(sc->pairs.p, L.pairs.data(), sizeof(NodePair) * L.pairs.size(), cudaMemcpyHostToDevice));
    if (!L.slots.empty())
        WR_CUDA(ctx, cudaMemcpy(sc->tris.p, L.slots.data(), sizeof(TriRec) * L.slots.size(), cudaMemcpyHostToDevice));
    DevTree& T = sc->tree;
    T.pairs = sc->pairs.as<NodePair>();
    T.tris = sc->tris.as<TriRec>();
    for (int k = 0; k < 3; k++) {
        T.root_lo[k] = L.root_lo[k];
        T.root_hi[k] = L.root_hi[k];
    }
    T.root_w0 = L.root_w0;
    T.root_w1 = L.root_w1;
    T.scene_mag = L.scene_mag;
    T.max_depth = ht.max_depth;
    T.num_pairs = (uint32_t)L.pairs.size();
    T.num_slots = (uint32_t)L.slots.size();
    sc->info.num_triangles = nt;
    sc->info.num_nodes = ht.num_nodes();
    sc->info.num_leaves = ht.num_leaves;
    sc->info.max_depth = ht.max_depth;
    sc->info.device_bytes = pb + tb;
    sc->info.build_seconds = std::chrono::duration<double>(t1 - t0).count();
    sc->id = ctx->next_scene++;
    *out = sc->id;
    ctx->scenes[sc->id] = std::move(sc);
    return WR_OK;
    WR_GUARD_END
}

int wr_scene_release(wr_ctx* ctx, wr_scene_id id) {
    if (!ctx) return WR_ERR_INVALID_ARGUMENT;
    auto it = ctx->scenes.find(id);
    if (it == ctx->scenes.end()) return set_error(ctx, WR_ERR_NOT_FOUND, "no such scene");
    if (ctx->serving) return set_error(ctx, WR_ERR_BUSY, "scenes stay resident while the serving loop runs");
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    wf_forget_scene(ctx, static_cast<const RenderData*>(it->second->render_data.get()));
    ctx->scenes.erase(it);
    return WR_OK;
}

int wr_scene_get_info(wr_ctx* ctx, wr_scene_id id, wr_scene_info* out) {
    if (!ctx || !out) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null argument");
    SceneGPU* sc = find_scene(ctx, id);
    if (!sc) return set_error(ctx, WR_ERR_NOT_FOUND, "no such scene");
    *out = sc->info;
    return WR_OK;
}

int wr_trace_closest_device(wr_ctx* ctx, wr_scene_id id, const float* d_rays, uint64_t n, const int32_t* d_inside,
                            const int32_t* d_contact, wr_hit* d_hits, void* stream) {
    if (!ctx) return WR_ERR_INVALID_ARGUMENT;
    SceneGPU* sc = find_scene(ctx, id);
    if (!sc) return set_error(ctx, WR_ERR_NOT_FOUND, "no such scene");
    if (n == 0) return WR_OK;
    if (!d_rays || !d_hits) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null ray or hit buffer");
    if ((d_inside == nullptr) != (d_contact == nullptr))
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "inside and contact ids go together");
    if ((reinterpret_cast<uintptr_t>(d_hits) & 15u) || (reinterpret_cast<uintptr_t>(d_rays) & 3u))
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "hit buffer must be 16-byte aligned, rays 4-byte aligned");
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    WR_CUDA(ctx, cudaSetDevice(ctx->device));
    unsigned long long* counter = ctx->scratch_words.as<unsigned long long>();
    unsigned int* err = reinterpret_cast<unsigned int*>(counter + 1);
    WR_CUDA(ctx, cudaMemsetAsync(err, 0, sizeof(unsigned int), s));
    const TraceTune tt = trace_tune_of(ctx);
    WR_CUDA(ctx, launch_trace_closest(sc->tree, d_rays, n, d_inside, d_contact, d_hits, counter, err, ctx->num_sms,
                                      ctx->trace_prune, s, &ctx->last_trace_blocks, &tt, ctx->wf_ctas_per_sm));
    ctx->kernel_launches++;
    return WR_OK;
}

// wr_trace_closest's copies and launches: rays in on `sin`, chunks traced on
// the context's stream, hits (and, last, the error word into *herr) out on
// `sout`; the caller synchronises all three
static cudaError_t enqueue_trace(wr_ctx* ctx, SceneGPU* sc, const float* rays, uint64_t n,
                                 const wr_trace_filter* filter, wr_hit* hits, int K, cudaStream_t sin,
                                 cudaStream_t sout, unsigned int* herr) {
    cudaStream_t s = ctx->stream;
    unsigned long long* counter = ctx->scratch_words.as<unsigned long long>();
    unsigned int* err = reinterpret_cast<unsigned int*>(counter + 1);
    const TraceTune tt = trace_tune_of(ctx);
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(unsigned int), s);
#define WR_TRY(call)                     \
    do {                                 \
        if (e == cudaSuccess) e = (call); \
    } while (0)
    if (K > 1) {  // the copies wait for earlier work on the context's stream (it may still use the buffers)
        WR_TRY(cudaEventRecord(ctx->pipe_ev[8], s));
        WR_TRY(cudaStreamWaitEvent(sin, ctx->pipe_ev[8], 0));
        WR_TRY(cudaStreamWaitEvent(sout, ctx->pipe_ev[8], 0));
    }
    const uint64_t chunk = (n + K - 1) / K;
    for (int k = 0; k < K && e == cudaSuccess; k++) {
        const uint64_t a = k * chunk, m = std::min<uint64_t>(n, a + chunk) - a;
        if (m == 0) break;
        WR_TRY(cudaMemcpyAsync(ctx->rays.as<float>() + 6 * a, rays + 6 * a, m * 6 * sizeof(float),
                               cudaMemcpyHostToDevice, sin));
        if (filter) {
            WR_TRY(cudaMemcpyAsync(ctx->inside.as<int32_t>() + a, filter->inside_obj + a, m * 4,
                                   cudaMemcpyHostToDevice, sin));
            WR_TRY(cudaMemcpyAsync(ctx->contact.as<int32_t>() + a, filter->contact_obj + a, m * 4,
                                   cudaMemcpyHostToDevice, sin));
        }
        if (K > 1) {
            WR_TRY(cudaEventRecord(ctx->pipe_ev[2 * k], sin));
            WR_TRY(cudaStreamWaitEvent(s, ctx->pipe_ev[2 * k], 0));
        }
        WR_TRY(launch_trace_closest(sc->tree, ctx->rays.as<float>() + 6 * a, m,
                                    filter ? ctx->inside.as<int32_t>() + a : nullptr,
                                    filter ? ctx->contact.as<int32_t>() + a : nullptr, ctx->hits.as<wr_hit>() + a,
                                    counter, err, ctx->num_sms, ctx->trace_prune, s, &ctx->last_trace_blocks, &tt,
                                    ctx->wf_ctas_per_sm));
        if (e == cudaSuccess) ctx->kernel_launches++;
        if (K > 1) {
            WR_TRY(cudaEventRecord(ctx->pipe_ev[2 * k + 1], s));
            WR_TRY(cudaStreamWaitEvent(sout, ctx->pipe_ev[2 * k + 1], 0));
        }
        WR_TRY(cudaMemcpyAsync(hits + a, ctx->hits.as<wr_hit>() + a, m * sizeof(wr_hit), cudaMemcpyDeviceToHost,
                               sout));
    }
    // the error word after the last kernel (sout waited for it)
    WR_TRY(cudaMemcpyAsync(herr, err, sizeof *herr, cudaMemcpyDeviceToHost, sout));
#undef WR_TRY
    return e;
}

int wr_trace_closest(wr_ctx* ctx, wr_scene_id id, const float* rays, uint64_t n, const wr_trace_filter* filter,
                     wr_hit* hits) {
    if (!ctx) return WR_ERR_INVALID_ARGUMENT;
    SceneGPU* sc = find_scene(ctx, id);
    if (!sc) return set_error(ctx, WR_ERR_NOT_FOUND, "no such scene");
    if (n == 0) return WR_OK;
    if (!rays || !hits) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null ray or hit buffer");
    const bool filtered = filter && filter->inside_obj && filter->contact_obj;
    if (filter && !filtered && (filter->inside_obj || filter->contact_obj))
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "inside and contact ids go together");
    WR_GUARD_BEGIN
    WR_CUDA(ctx, cudaSetDevice(ctx->device));
    WR_CUDA(ctx, ctx->rays.reserve(n * 6 * sizeof(float)));
    WR_CUDA(ctx, ctx->hits.reserve(n * sizeof(wr_hit)));
    if (filtered) {
        WR_CUDA(ctx, ctx->inside.reserve(n * sizeof(int32_t)));
        WR_CUDA(ctx, ctx->contact.reserve(n * sizeof(int32_t)));
    }
    // K chunks in a pipeline: chunk k's rays go in on copy_in while chunk k-1
    // is traced on `stream` and chunk k-2's hits come out on copy_out (2^24
    // rays: 6.7 -> 5.3 ms with 4 chunks on GB300; with 8 the chunks' launch
    // tails cost more than the overlap saves)
    const int K = n >= (1ull << 22) ? 4 : (n >= (1ull << 20) ? 2 : 1);
    if (K > 1 && !ctx->copy_out) {  // made once per context; copy_out last, so that it marks them all made
        if (!ctx->copy_in) WR_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_in, cudaStreamNonBlocking));
        for (cudaEvent_t& e : ctx->pipe_ev)
            if (!e) WR_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        WR_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_out, cudaStreamNonBlocking));
    }
    cudaStream_t s = ctx->stream;
    cudaStream_t sin = K > 1 ? ctx->copy_in : s, sout = K > 1 ? ctx->copy_out : s;
    unsigned int herr = 0;
    const cudaError_t e = enqueue_trace(ctx, sc, rays, n, filtered ? filter : nullptr, hits, K, sin, sout, &herr);
    // even after a failed call, nothing may still read the caller's rays or
    // write its hits once this returns
    const cudaError_t e_in = cudaStreamSynchronize(sin), e_k = cudaStreamSynchronize(s);
    const cudaError_t e_out = cudaStreamSynchronize(sout);
    if (e != cudaSuccess) return cuda_error(ctx, e, "wr_trace_closest");
    for (cudaError_t f : {e_in, e_k, e_out})
        if (f != cudaSuccess) return cuda_error(ctx, f, "wr_trace_closest");
    if (herr) return set_error(ctx, WR_ERR_INTERNAL, "traversal stack overflow");
    return WR_OK;
    WR_GUARD_END
}

// ---- host-only tree export ----------------------------------------------
struct wr_kdtree_host {
    HostTree t;
};

int wr_kdtree_build_host(const float* vertices, uint32_t nv, const uint32_t* triangles, uint32_t nt, int threads,
                         wr_kdtree_host** out) {
    wr_ctx* ctx = nullptr;
    if (!out || (nv && !vertices) || (nt && !triangles)) return WR_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < 3 * (size_t)nt; i++)
        if (triangles[i] >= nv) return WR_ERR_INVALID_ARGUMENT;
    WR_GUARD_BEGIN
    auto* h = new wr_kdtree_host();
    h->t = build_reference_tree(vertices, nv, triangles, nt, threads);
    *out = h;
    return WR_OK;
    WR_GUARD_END
}

int wr_kdtree_host_sizes(const wr_kdtree_host* h, uint32_t* num_nodes, uint32_t* num_leaf_tris, uint32_t* max_depth) {
    if (!h) return WR_ERR_INVALID_ARGUMENT;
    if (num_nodes) *num_nodes = h->t.num_nodes();
    if (num_leaf_tris) *num_leaf_tris = (uint32_t)h->t.leaf_tris.size();
    if (max_depth) *max_depth = h->t.max_depth;
    return WR_OK;
}

int wr_kdtree_host_export(const wr_kdtree_host* h, int32_t* left, int32_t* right, float* boxes, uint32_t* leaf_first,
                          uint32_t* leaf_count, uint32_t* leaf_tris) {
    if (!h) return WR_ERR_INVALID_ARGUMENT;
    const HostTree& t = h->t;
    const size_t N = t.num_nodes();
    if (left) std::memcpy(left, t.left.data(), 4 * N);
    if (right) std::memcpy(right, t.right.data(), 4 * N);
    if (boxes) std::memcpy(boxes, t.box.data(), 24 * N);
    if (leaf_first) std::memcpy(leaf_first, t.leaf_first.data(), 4 * N);
    if (leaf_count) std::memcpy(leaf_count, t.leaf_count.data(), 4 * N);
    if (leaf_tris) std::memcpy(leaf_tris, t.leaf_tris.data(), 4 * t.leaf_tris.size());
    return WR_OK;
}

int wr_kdtree_host_free(wr_kdtree_host* h) {
    delete h;
    return WR_OK;
}

}  // extern "C"
