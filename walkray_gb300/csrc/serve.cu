// serve.cu — the serving loop: continuous batching of render requests over
// the wavefront queues (wr_serve_start / wr_submit / wr_poll / wr_fetch /
// wr_cancel / wr_serve_stop).
//
// One host thread owns the wavefront engine while serving.  Each turn it
// (1) admits queued requests in FIFO order while a job slot is free and the
// request's FP32 film fits in the serving film arena, (2) replays the
// captured bounce loop once -- its generate stage shares the queue slots that
// finished paths free among the running requests (k_wf_plan: equal shares,
// or admission order with WR_SERVE_FIFO) -- (3) reads the per-job path
// counters and retires
// every request whose paths have all reached its film (copy to the host,
// free the arena block and the slot).  The queue length adapts to the load:
// while no request waits for admission it holds wr_serve_desc.paths_in_flight
// paths (2^22 by default), because every bounce of a request waits for one
// pass of the loop over the whole queue and a short queue keeps small
// requests fast; while requests wait (the loop is saturated) it holds the
// renderer's full capacity, which gives the most paths per second.  New requests therefore join while
// older ones run, and their paths share the same queues; a request's image
// depends only on its own seed, not on what else is in flight.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>

#include "wavefront.h"
#include "wr_context.h"

namespace wr {

int prepare_render(wr_ctx* ctx, SceneGPU* sc, RenderData** out);

namespace {

// first-fit allocator over one device block (the film memory)
struct Arena {
    char* base = nullptr;
    size_t size = 0;
    std::map<size_t, size_t> free_;  // offset -> bytes
    void init(char* b, size_t n) {
        base = b;
        size = n;
        free_.clear();
        free_[0] = n;
    }
    bool alloc(size_t bytes, size_t* off) {
        bytes = (bytes + 255) & ~size_t(255);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes;
                const size_t roff = it->first + bytes;
                free_.erase(it);
                if (rest) free_[roff] = rest;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = (bytes + 255) & ~size_t(255);
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

struct Req {
    wr_request_desc d{};
    uint32_t state = WR_REQ_QUEUED;
    int slot = -1;
    size_t off = 0, bytes = 0;
    unsigned long long total = 0, done = 0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    bool cancel = false;
    RenderData* rd = nullptr;
    std::vector<float> image;
};

struct Server {
    wr_ctx* ctx = nullptr;
    WfEngine* E = nullptr;
    cudaStream_t stream = nullptr;
    std::thread th;
    std::mutex mu;
    std::condition_variable cv;
    bool stop = false;
    std::deque<wr_req_id> pending;
    std::map<wr_req_id, Req> reqs;
    wr_req_id next_id = 1;
    std::vector<wr_req_id> slot_owner;
    std::vector<int> order;  // active slots in admission order
    uint32_t max_active = 64;
    uint32_t short_queue = WR_SERVE_DEFAULT_PATHS;  // queue length while nobody waits for admission
    DeviceBuffer arena_mem;
    Arena arena;
    std::chrono::steady_clock::time_point t0;
    std::string fail;

    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }

    ~Server() {
        if (stream) cudaStreamDestroy(stream);
    }

    void fail_all(const std::string& why) {
        std::lock_guard<std::mutex> lk(mu);
        fail = why;
        for (auto& kv : reqs)
            if (kv.second.state == WR_REQ_QUEUED || kv.second.state == WR_REQ_RUNNING) kv.second.state = WR_REQ_FAILED;
        pending.clear();
        order.clear();
    }

    void loop() {
        cudaSetDevice(ctx->device);
        std::vector<WfJobCounters> cnt;
        std::vector<int> last_order;
        for (;;) {
            std::vector<WfSlotUpdate> ups;
            std::vector<int> ord;
            bool have_work;
            uint32_t want_queue = short_queue;
            {
                std::unique_lock<std::mutex> lk(mu);
                if (stop) break;
                // admit in FIFO order while a slot and film memory are free
                while (!pending.empty() && order.size() < max_active) {
                    Req& r = reqs[pending.front()];
                    int slot = -1;
                    for (int k = 0; k < (int)slot_owner.size(); k++)
                        if (!slot_owner[k]) {
                            slot = k;
                            break;
                        }
                    if (slot < 0) break;
                    size_t off;
                    r.bytes = sizeof(float) * 3ull * r.d.width * r.d.height;
                    if (!arena.alloc(r.bytes, &off)) break;  // wait for memory (FIFO: no overtaking)
                    r.off = off;
                    r.slot = slot;
                    r.state = WR_REQ_RUNNING;
                    r.t_admit = now();
                    slot_owner[slot] = pending.front();
                    pending.pop_front();
                    float* film = reinterpret_cast<float*>(arena.base + off);
                    cudaMemsetAsync(film, 0, r.bytes, stream);
                    WfSlotUpdate u;
                    u.slot = slot;
                    u.jh.rd = r.rd;
                    const CamParams cam = camera_params_for(r.rd, r.d.width, r.d.height);
                    u.jh.job = make_job(RenderDataView::scene(r.rd), cam, r.d.seed, 0, r.d.spp, r.d.max_path_len,
                                        r.d.flags, film, nullptr);
                    r.total = u.jh.job.total;
                    u.reset_counters = true;
                    ups.push_back(u);
                    order.push_back(slot);
                }
                // cancelled requests stop receiving new paths
                for (int s : order) {
                    Req& r = reqs[slot_owner[s]];
                    if (r.cancel && E && r.state == WR_REQ_RUNNING) {
                        WfSlotUpdate u;
                        u.slot = s;
                        u.jh.job = make_job(RenderDataView::scene(r.rd), camera_params_for(r.rd, r.d.width, r.d.height),
                                            r.d.seed, 0, r.d.spp, r.d.max_path_len, r.d.flags,
                                            reinterpret_cast<float*>(arena.base + r.off), nullptr);
                        u.jh.job.active = 0;
                        ups.push_back(u);
                    }
                }
                for (int s : order)
                    if (!reqs[slot_owner[s]].cancel) ord.push_back(s);
                have_work = !order.empty();
                want_queue = pending.empty() ? short_queue : wf_config(E).capacity;
                if (!have_work && ups.empty()) {
                    cv.wait_for(lk, std::chrono::milliseconds(2));
                    continue;
                }
            }
            int rc = wf_set_live_cap(ctx, E, want_queue, stream);
            if (rc == WR_OK && (!ups.empty() || ord != last_order)) rc = wf_update_jobs(ctx, E, ups, ord, stream);
            last_order = ord;
            if (rc == WR_OK && have_work) rc = wf_launch(ctx, E, stream);
            if (rc == WR_OK) rc = wf_read_counters(ctx, E, cnt, stream);
            if (rc != WR_OK) {
                fail_all(ctx->err);
                return;
            }
            // retire finished (or drained cancelled) requests
            std::vector<int> finished;
            {
                std::lock_guard<std::mutex> lk(mu);
                for (int s : order) {
                    Req& r = reqs[slot_owner[s]];
                    r.done = cnt[s].finished;
                    const unsigned long long issued = std::min<unsigned long long>(cnt[s].claimed, r.total);
                    if ((!r.cancel && cnt[s].finished >= r.total) || (r.cancel && cnt[s].finished >= issued))
                        finished.push_back(s);
                }
            }
            for (int s : finished) {
                Req* r;
                {
                    std::lock_guard<std::mutex> lk(mu);
                    r = &reqs[slot_owner[s]];
                }
                std::vector<float> img;
                if (!r->cancel) {
                    img.resize(3ull * r->d.width * r->d.height);
                    cudaError_t e = cudaMemcpyAsync(img.data(), arena.base + r->off, r->bytes, cudaMemcpyDeviceToHost,
                                                    stream);
                    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
                    if (e != cudaSuccess) {
                        fail_all(cudaGetErrorString(e));
                        return;
                    }
                    const float inv = r->d.spp ? 1.f / (float)r->d.spp : 0.f;
                    for (float& v : img) v *= inv;
                }
                std::lock_guard<std::mutex> lk(mu);
                r->image.swap(img);
                r->state = r->cancel ? WR_REQ_CANCELLED : WR_REQ_DONE;
                r->t_done = now();
                arena.release(r->off, r->bytes);
                slot_owner[s] = 0;
                order.erase(std::find(order.begin(), order.end(), s));
            }
        }
    }
};

}  // namespace

CamParams camera_params_for(const RenderData* rd, uint32_t width, uint32_t height) {
    CamParams c = RenderDataView::scene(rd).cam;
    // the image plane distance is in pixels: keep the field of view
    c.ipd = c.height ? c.ipd * ((float)height / (float)c.height) : c.ipd;
    c.width = width;
    c.height = height;
    return c;
}

}  // namespace wr

using namespace wr;

static Server* server_of(wr_ctx* ctx) { return static_cast<Server*>(ctx->serving.get()); }

extern "C" {

int wr_serve_start(wr_ctx* ctx, const wr_serve_desc* desc) {
    if (!ctx) return WR_ERR_INVALID_ARGUMENT;
    if (ctx->serving) return set_error(ctx, WR_ERR_BUSY, "the serving loop is already running");
    try {
        WR_CUDA(ctx, cudaSetDevice(ctx->device));
        auto S = std::make_shared<Server>();
        S->ctx = ctx;
        S->max_active = (desc && desc->max_active) ? std::min<uint32_t>(desc->max_active, wf_max_jobs()) : 64;
        uint64_t film = desc && desc->film_bytes ? desc->film_bytes : ctx->memory_budget / 4;
        WR_CUDA(ctx, S->arena_mem.reserve(film));
        S->arena.init(S->arena_mem.as<char>(), film);
        WR_CUDA(ctx, cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
        const uint32_t pif = desc && desc->paths_in_flight ? desc->paths_in_flight : WR_SERVE_DEFAULT_PATHS;
        if (pif < 1024 || pif > (1u << 25) || (desc && desc->reserved))
            return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "paths_in_flight must be 1024 .. 2^25, reserved 0");
        int rc = wf_engine_get(ctx, wf_tuned_config(ctx), &S->E);
        if (rc != WR_OK) return rc;
        S->short_queue = std::min(pif, wf_config(S->E).capacity);
        if ((rc = wf_set_live_cap(ctx, S->E, S->short_queue, S->stream)) != WR_OK) return rc;
        if ((rc = wf_set_equal_share(ctx, S->E, !(desc && (desc->flags & WR_SERVE_FIFO)))) != WR_OK) return rc;
        // start from an empty job table and empty queues
        std::vector<WfSlotUpdate> clear;
        for (uint32_t k = 0; k < wf_max_jobs(); k++) {
            WfSlotUpdate u;
            u.slot = (int)k;
            std::memset(&u.jh.job, 0, sizeof(u.jh.job));
            u.reset_counters = true;
            clear.push_back(u);
        }
        if ((rc = wf_update_jobs(ctx, S->E, clear, {}, S->stream)) != WR_OK) return rc;
        if ((rc = wf_reset_queues(ctx, S->E, S->stream)) != WR_OK) return rc;
        S->slot_owner.assign(wf_max_jobs(), 0);
        S->t0 = std::chrono::steady_clock::now();
        ctx->serving = S;
        S->th = std::thread([S]() { S->loop(); });
        return WR_OK;
    } catch (const std::exception& ex) {
        return set_error(ctx, WR_ERR_INTERNAL, ex.what());
    }
}

int wr_serve_stop(wr_ctx* ctx) {
    if (!ctx) return WR_ERR_INVALID_ARGUMENT;
    Server* S = server_of(ctx);
    if (!S) return set_error(ctx, WR_ERR_NOT_FOUND, "the serving loop is not running");
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv.notify_all();
    if (S->th.joinable()) S->th.join();
    cudaStreamSynchronize(S->stream);
    ctx->serving.reset();
    return WR_OK;
}

int wr_submit(wr_ctx* ctx, const wr_request_desc* req, wr_req_id* out) {
    if (!ctx || !req || !out) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null argument");
    Server* S = server_of(ctx);
    if (!S) return set_error(ctx, WR_ERR_NOT_FOUND, "the serving loop is not running");
    if (req->width == 0 || req->height == 0 || req->width > 16384 || req->height > 16384)
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "bad resolution");
    if (const char* why = render_flags_problem(req->flags, WR_MODE_WAVEFRONT))
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, why);
    if ((uint64_t)req->width * req->height * req->spp == 0)
        return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "a request needs at least one path");
    const uint64_t film = sizeof(float) * 3ull * req->width * req->height;
    if (film > S->arena.size) return set_error(ctx, WR_ERR_OUT_OF_MEMORY, "the request's film exceeds the film memory");
    SceneGPU* sc = find_scene(ctx, req->scene);
    if (!sc) return set_error(ctx, WR_ERR_NOT_FOUND, "no such scene");
    std::lock_guard<std::mutex> lk(S->mu);
    if (!S->fail.empty()) return set_error(ctx, WR_ERR_INTERNAL, "serving loop failed: " + S->fail);
    RenderData* rd = nullptr;
    int rc = prepare_render(ctx, sc, &rd);
    if (rc != WR_OK) return rc;
    wr_req_id id = S->next_id++;
    Req& r = S->reqs[id];
    r.d = *req;
    r.rd = rd;
    r.t_submit = S->now();
    r.total = (unsigned long long)req->width * req->height * req->spp;
    S->pending.push_back(id);
    *out = id;
    S->cv.notify_all();
    return WR_OK;
}

int wr_poll(wr_ctx* ctx, wr_req_id id, wr_req_status* out) {
    if (!ctx || !out) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null argument");
    Server* S = server_of(ctx);
    if (!S) return set_error(ctx, WR_ERR_NOT_FOUND, "the serving loop is not running");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return set_error(ctx, WR_ERR_NOT_FOUND, "no such request");
    const Req& r = it->second;
    std::memset(out, 0, sizeof *out);
    out->state = r.state;
    out->paths_total = r.total;
    out->paths_done = r.state == WR_REQ_DONE ? r.total : r.done;
    out->submit_s = r.t_submit;
    out->admit_s = r.t_admit;
    out->finish_s = r.t_done;
    return WR_OK;
}

int wr_fetch(wr_ctx* ctx, wr_req_id id, float* rgb_out) {
    if (!ctx || !rgb_out) return set_error(ctx, WR_ERR_INVALID_ARGUMENT, "null argument");
    Server* S = server_of(ctx);
    if (!S) return set_error(ctx, WR_ERR_NOT_FOUND, "the serving loop is not running");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return set_error(ctx, WR_ERR_NOT_FOUND, "no such request");
    if (it->second.state != WR_REQ_DONE) return set_error(ctx, WR_ERR_BUSY, "request not finished");
    std::memcpy(rgb_out, it->second.image.data(), sizeof(float) * it->second.image.size());
    S->reqs.erase(it);
    return WR_OK;
}

int wr_cancel(wr_ctx* ctx, wr_req_id id) {
    if (!ctx) return WR_ERR_INVALID_ARGUMENT;
    Server* S = server_of(ctx);
    if (!S) return set_error(ctx, WR_ERR_NOT_FOUND, "the serving loop is not running");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(id);
    if (it == S->reqs.end()) return set_error(ctx, WR_ERR_NOT_FOUND, "no such request");
    Req& r = it->second;
    if (r.state == WR_REQ_QUEUED) {
        S->pending.erase(std::find(S->pending.begin(), S->pending.end(), id));
        r.state = WR_REQ_CANCELLED;
    } else if (r.state == WR_REQ_RUNNING) {
        r.cancel = true;
    }
    S->cv.notify_all();
    return WR_OK;
}

}  // extern "C"
