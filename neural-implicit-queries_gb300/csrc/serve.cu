// serve.cu -- continuous batching of mixed query requests over resident models.
//
// The reference has no serving path (its queries are called one at a time from a GUI);
// this runtime turns the query entry points of this library into a service.  A server
// owns a fixed set of lanes.  A lane is a host worker thread with its own CUDA stream and
// its own scratch, allocated once when the server is created, so no request allocates.
// niq_batch_submit cuts a request into slices and queues them; the lanes take slices as
// they free up -- ray tiles before closest-point and intersection work, so a short ray
// tile never waits behind a long closest-point batch -- and run them on their streams,
// so slices of different requests overlap on the device.  A request completes when its
// last slice does; niq_batch_poll and niq_batch_wait report it.
//
// Slices: a ray request of n rays becomes tiles of at most slice_rays rays
// (niq_cast_rays on each tile, outputs written in place); a closest-point request of n
// queries becomes slices of at most slice_queries queries (niq_closest_point_persistent
// with the request's node budget; a slice that spends the budget marks the request
// NIQ_ERR_TIMEOUT, with every result written, an upper bound); an intersection request
// is one slice (niq_find_any_intersection).
#include <atomic>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>
#include "niq_host.cuh"

namespace niq {

struct ServeRequest {
    niq_request r;
    std::atomic<int> pending{0};
    std::atomic<int> status{NIQ_OK};
    bool done = false;
};

struct ServeSlice {
    std::shared_ptr<ServeRequest> req;
    long long i0 = 0, n = 0;
};

struct ServeLane {
    cudaStream_t stream = nullptr;
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    int64_t* small = nullptr;     // device: n_evals, intersection counts
    std::thread thread;
};

}  // namespace niq

struct niq_server {
    niq_server_opts opts;
    int device = 0;
    std::vector<niq::ServeLane> lanes;
    std::mutex mu;
    std::condition_variable cv_work;   // slices queued / shutdown
    std::condition_variable cv_done;   // a request completed
    std::deque<niq::ServeSlice> q_rays, q_other;
    std::unordered_map<long long, std::shared_ptr<niq::ServeRequest>> live;
    long long next_ticket = 1;
    long long completed = 0, in_flight = 0;
    bool stop = false;
};

namespace niq {

static void serve_finish(niq_server* S, const std::shared_ptr<ServeRequest>& req, int rc) {
    if (rc != NIQ_OK) {
        int expected = NIQ_OK;
        // the first error wins; a spent node budget never hides a harder error
        if (!req->status.compare_exchange_strong(expected, rc) && expected == NIQ_ERR_TIMEOUT && rc != NIQ_ERR_TIMEOUT)
            req->status.store(rc);
    }
    if (req->pending.fetch_sub(1) == 1) {
        std::lock_guard<std::mutex> lk(S->mu);
        req->done = true;
        S->completed += 1;
        S->in_flight -= 1;
        S->cv_done.notify_all();
    }
}

static int serve_run_slice(ServeLane& L, const ServeSlice& sl) {
    const niq_request& r = sl.req->r;
    void* st = reinterpret_cast<void*>(L.stream);
    if (r.kind == NIQ_REQ_RAYS) {
        const niq_model* m[1] = {r.model};
        const size_t need = niq_cast_rays_workspace_size(m, 1, &r.opts, sl.n);
        NIQ_REQUIRE(need <= L.scratch_bytes, NIQ_ERR_CAPACITY, "ray tile needs %zu bytes of lane scratch", need);
        int rc = niq_cast_rays(m, 1, &r.opts, sl.n, r.in0 + 3 * sl.i0, r.in1 + 3 * sl.i0, &r.cast, r.out_f + sl.i0,
                               r.out_i + sl.i0, r.out_i2 + sl.i0, L.small, L.scratch, L.scratch_bytes, st);
        if (rc) return rc;
        NIQ_CUDA(cudaStreamSynchronize(L.stream));
        return NIQ_OK;
    }
    if (r.kind == NIQ_REQ_CLOSEST) {
        const size_t need = niq_closest_point_persistent_workspace_size(sl.n);
        NIQ_REQUIRE(need <= L.scratch_bytes, NIQ_ERR_CAPACITY, "closest-point slice needs %zu bytes of lane scratch",
                    need);
        return niq_closest_point_persistent(r.model, &r.opts, r.lower, r.upper, sl.n, r.in0 + 3 * sl.i0, r.eps,
                                            r.node_budget, r.out_f + sl.i0, r.out_f2 + 3 * sl.i0, L.scratch,
                                            L.scratch_bytes, st);
    }
    // intersection: one slice
    const long long cap = r.node_capacity > 0 ? r.node_capacity : (1ll << 20);
    const size_t need = niq_intersect_workspace_size(r.model, r.model_b, &r.opts, cap);
    NIQ_REQUIRE(need <= L.scratch_bytes, NIQ_ERR_CAPACITY, "intersection needs %zu bytes of lane scratch", need);
    int rc = niq_find_any_intersection(r.model, r.model_b, &r.opts, r.lower, r.upper, r.eps, cap, r.out_i, r.out_f2,
                                       L.small + 1, L.scratch, L.scratch_bytes, st);
    if (rc) return rc;
    NIQ_CUDA(cudaStreamSynchronize(L.stream));
    return NIQ_OK;
}

static void serve_lane_main(niq_server* S, int li) {
    cudaSetDevice(S->device);
    ServeLane& L = S->lanes[li];
    while (true) {
        ServeSlice sl;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] { return S->stop || !S->q_rays.empty() || !S->q_other.empty(); });
            if (S->stop && S->q_rays.empty() && S->q_other.empty()) return;
            std::deque<ServeSlice>& q = !S->q_rays.empty() ? S->q_rays : S->q_other;
            sl = q.front();
            q.pop_front();
        }
        serve_finish(S, sl.req, serve_run_slice(L, sl));
    }
}

}  // namespace niq

using namespace niq;

extern "C" {

int niq_server_create(const niq_server_opts* opts, niq_server** out) {
    NIQ_REQUIRE(opts && out, NIQ_ERR_INVALID_ARG, "null argument");
    NIQ_REQUIRE(opts->n_lanes >= 1 && opts->n_lanes <= 64, NIQ_ERR_INVALID_ARG, "n_lanes must be in [1, 64]");
    NIQ_REQUIRE(opts->slice_rays >= 1 && opts->slice_queries >= 1 && opts->lane_scratch_bytes >= 4096,
                NIQ_ERR_INVALID_ARG, "slice sizes >= 1 and lane scratch >= 4096 bytes");
    std::unique_ptr<niq_server> S(new niq_server());
    S->opts = *opts;
    NIQ_CUDA(cudaGetDevice(&S->device));
    S->lanes.resize(opts->n_lanes);
    auto release = [&]() {   // undo a partial set-up
        for (auto& L : S->lanes) {
            if (L.scratch) cudaFree(L.scratch);
            if (L.small) cudaFree(L.small);
            if (L.stream) cudaStreamDestroy(L.stream);
        }
    };
    for (auto& L : S->lanes) {
        cudaError_t e = cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaMalloc(&L.scratch, (size_t)opts->lane_scratch_bytes);
        if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&L.small), 8 * sizeof(int64_t));
        if (e != cudaSuccess) {
            release();
            return cuda_fail(e, "server lane set-up");
        }
        L.scratch_bytes = (size_t)opts->lane_scratch_bytes;
    }
    niq_server* raw = S.release();
    for (int i = 0; i < opts->n_lanes; ++i) raw->lanes[i].thread = std::thread(serve_lane_main, raw, i);
    *out = raw;
    return NIQ_OK;
}

int niq_server_destroy(niq_server* S) {
    NIQ_REQUIRE(S, NIQ_ERR_INVALID_ARG, "null server");
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;   // lanes finish the queued slices, then exit
    }
    S->cv_work.notify_all();
    for (auto& L : S->lanes)
        if (L.thread.joinable()) L.thread.join();
    for (auto& L : S->lanes) {
        cudaFree(L.scratch);
        cudaFree(L.small);
        cudaStreamDestroy(L.stream);
    }
    delete S;
    return NIQ_OK;
}

int niq_batch_submit(niq_server* S, const niq_request* req, int64_t* ticket_out) {
    NIQ_REQUIRE(S && req && ticket_out, NIQ_ERR_INVALID_ARG, "null argument");
    NIQ_REQUIRE(req->model && req->n >= 0, NIQ_ERR_INVALID_ARG, "request needs a model and n >= 0");
    NIQ_REQUIRE(req->kind == NIQ_REQ_RAYS || req->kind == NIQ_REQ_CLOSEST || req->kind == NIQ_REQ_INTERSECT,
                NIQ_ERR_INVALID_ARG, "unknown request kind %d", req->kind);
    if (req->kind == NIQ_REQ_RAYS)
        NIQ_REQUIRE(req->n == 0 || (req->in0 && req->in1 && req->out_f && req->out_i && req->out_i2),
                    NIQ_ERR_INVALID_ARG, "ray request needs roots, dirs, t, hit_id and count");
    if (req->kind == NIQ_REQ_CLOSEST)
        NIQ_REQUIRE(req->n == 0 || (req->in0 && req->out_f && req->out_f2), NIQ_ERR_INVALID_ARG,
                    "closest-point request needs points, distances and locations");
    if (req->kind == NIQ_REQ_INTERSECT)
        NIQ_REQUIRE(req->model_b && req->out_i && req->out_f2, NIQ_ERR_INVALID_ARG,
                    "intersection request needs model_b, found and location");
    auto R = std::make_shared<ServeRequest>();
    R->r = *req;
    std::vector<ServeSlice> slices;
    if (req->kind == NIQ_REQ_INTERSECT) {
        slices.push_back(ServeSlice{R, 0, 1});
    } else {
        const long long step = req->kind == NIQ_REQ_RAYS ? S->opts.slice_rays : S->opts.slice_queries;
        for (long long i0 = 0; i0 < req->n; i0 += step)
            slices.push_back(ServeSlice{R, i0, req->n - i0 < step ? req->n - i0 : step});
    }
    {
        std::lock_guard<std::mutex> lk(S->mu);
        const long long t = S->next_ticket++;
        *ticket_out = t;
        S->live[t] = R;
        S->in_flight += 1;
        if (slices.empty()) {   // nothing to do: done at once
            R->done = true;
            S->completed += 1;
            S->in_flight -= 1;
            return NIQ_OK;
        }
        R->pending.store((int)slices.size());
        auto& q = req->kind == NIQ_REQ_RAYS ? S->q_rays : S->q_other;
        for (auto& s : slices) q.push_back(s);
    }
    S->cv_work.notify_all();
    return NIQ_OK;
}

int niq_batch_poll(niq_server* S, int64_t ticket, int32_t* done_out, int32_t* status_out) {
    NIQ_REQUIRE(S && done_out, NIQ_ERR_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->live.find(ticket);
    NIQ_REQUIRE(it != S->live.end(), NIQ_ERR_INVALID_ARG, "unknown ticket %lld", (long long)ticket);
    *done_out = it->second->done ? 1 : 0;
    if (status_out) *status_out = it->second->status.load();
    if (it->second->done) S->live.erase(it);   // a finished ticket is reported once
    return NIQ_OK;
}

int niq_batch_wait(niq_server* S, int64_t ticket, double timeout_s, int32_t* status_out) {
    NIQ_REQUIRE(S, NIQ_ERR_INVALID_ARG, "null argument");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->live.find(ticket);
    NIQ_REQUIRE(it != S->live.end(), NIQ_ERR_INVALID_ARG, "unknown ticket %lld", (long long)ticket);
    std::shared_ptr<ServeRequest> R = it->second;
    const bool ok = S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return R->done; });
    NIQ_REQUIRE(ok, NIQ_ERR_TIMEOUT, "request %lld not done after %.3f s", (long long)ticket, timeout_s);
    if (status_out) *status_out = R->status.load();
    S->live.erase(ticket);
    return NIQ_OK;
}

int niq_server_stats(niq_server* S, int64_t* completed, int64_t* in_flight) {
    NIQ_REQUIRE(S, NIQ_ERR_INVALID_ARG, "null server");
    std::lock_guard<std::mutex> lk(S->mu);
    if (completed) *completed = S->completed;
    if (in_flight) *in_flight = S->in_flight;
    return NIQ_OK;
}

}  // extern "C"
