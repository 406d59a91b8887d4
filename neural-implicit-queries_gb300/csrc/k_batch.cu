// k_batch.cu -- closest-point queries (src/kd_tree.py:659-802) for many models in one
// persistent launch.
//
// The host splits every job (model, query range) into chunks of at most kChunk queries
// and orders chunks by decreasing cost.  CTAs claim chunks from a global counter; a chunk
// runs on the tile-engine instantiation of its model's width class (all classes live in
// one kernel, so models of any width share the launch), each CTA slot traversing one
// query's depth-first stack (nearer child first) until the chunk is drained.  Weights are
// restaged only when a CTA moves to a different model.
#include "niq_host.cuh"

namespace niq {

constexpr int kChunk = 128;     // default queries per chunk (tunable: NIQ_TUNE_BATCHED_CHUNK)
constexpr int kMinChunk = 32;   // smallest tunable chunk: sizes the workspace
constexpr int kBStack = 96;
constexpr int kBNT = 256;

struct BChunk {
    int model;
    int q_begin;   // absolute row in query_points
    int q_count;
    int pad;
};

struct BArgs {
    const NiqModelRef* models;   // device table
    const BChunk* chunks;
    int n_chunks;
    const float* q;
    float* min_dist;
    float* min_loc;
    float lu[6];
    float eps_w;
    int interval;
    float* stacks;               // (grid * 64 slots) x kBStack x 6
    unsigned long long* next_chunk;
    unsigned long long* n_spent;  // queries stopped at their node budget
    unsigned long long* n_nodes;  // nodes bounded (one box bound and its samples each)
    int* err;
    int smem_floats;             // dynamic shared memory in floats
    long long node_budget;       // nodes one query may visit
    float prune_tol;             // prune when box distance >= best - prune_tol (eps)
};

// per-slot state shared by every width class (at most 64 slots per CTA)
struct BSlots {
    float lo[64][3], hi[64][3], qp[64][3], best[64], loc[64][3], lohi[64][2];
    int top[64], act[64], qid[64], next;
    long long nodes[64];
};

template <int TPI, bool C, bool SLOPE>
__device__ void run_chunk(const BArgs& a, const BChunk ch, NiqSpecHeader& H, BSlots& S, float* smem, int& staged_model) {
    using CB = typename std::conditional<SLOPE, TileCfg<8, 4, TPI, kBNT>, TileCfg<5, 1, TPI, kBNT>>::type;
    using CP = TileCfg<8, 0, TPI, kBNT>;
    constexpr int ITEMS = CP::ITEMS;
    const int fixed = (CP::STATE_FLOATS + ((ITEMS * 8 + 3) & ~3) + 3) & ~3;
    float* st = smem;
    float* ob = st + CP::STATE_FLOATS;
    float* sW = smem + fixed;
    const int sw_cap = a.smem_floats - fixed;
    auto& s_lo = S.lo; auto& s_hi = S.hi; auto& s_qp = S.qp; auto& s_best = S.best; auto& s_loc = S.loc;
    auto& s_lohi = S.lohi; auto& s_top = S.top; auto& s_act = S.act; auto& s_qid = S.qid; int& s_next = S.next;
    const NiqModelRef M = a.models[ch.model];
    __syncthreads();
    if (staged_model != ch.model) {
        load_header(H, M.hdr);
        __syncthreads();
    }
    const bool resident = H.n_weight_floats <= sw_cap;
    if (resident && staged_model != ch.model) {
        stage_floats(sW, M.w, H.n_weight_floats);
    }
    staged_model = ch.model;
    const int item = threadIdx.x / TPI, g = threadIdx.x % TPI;
    const float gam0 = C ? H.layers[0].gamma : 0.f;
    const RowPlan pb{SLOPE ? ROWS_SLOPE : ROWS_AFFINE, a.interval ? 0 : 3, 0};
    const RowPlan pp{ROWS_POINTS, 0, 8};
    float* my_stack = a.stacks + ((long long)blockIdx.x * 64 + item) * kBStack * 6;
    if (threadIdx.x == 0) s_next = 0;
    __syncthreads();
    auto claim = [&]() {
        const int k = atomicAdd(&s_next, 1);
        if (k < ch.q_count) {
            const int qi = ch.q_begin + k;
            s_qid[item] = qi;
            for (int j = 0; j < 3; ++j) {
                s_qp[item][j] = a.q[3 * (long long)qi + j];
                my_stack[j] = a.lu[j];
                my_stack[3 + j] = a.lu[3 + j];
                s_loc[item][j] = -777.f;
            }
            s_top[item] = 1;
            s_best[item] = INFINITY;
            S.nodes[item] = 0;
        } else {
            s_qid[item] = -1;
            s_top[item] = 0;
        }
    };
    if (g == 0) claim();
    __syncthreads();
    while (true) {
        if (g == 0) {
            while (s_qid[item] >= 0 && s_top[item] == 0) {
                const long long id = s_qid[item];
                a.min_dist[id] = s_best[item];
                for (int j = 0; j < 3; ++j) a.min_loc[3 * id + j] = s_loc[item][j];
                claim();
            }
            // node budget per query: past it the query keeps its best so far (an upper
            // bound) and the call reports NIQ_ERR_TIMEOUT
            if (s_qid[item] >= 0 && s_top[item] > 0 && ++S.nodes[item] > a.node_budget) {
                niq_flag_error(a.err, NIQ_ERR_TIMEOUT);
                atomicAdd(a.n_spent, 1ull);
                s_top[item] = 0;
                const long long id = s_qid[item];
                a.min_dist[id] = s_best[item];
                for (int j = 0; j < 3; ++j) a.min_loc[3 * id + j] = s_loc[item][j];
                claim();
                if (s_qid[item] >= 0) S.nodes[item] = 1;
            }
            s_act[item] = s_qid[item] >= 0;
            if (s_act[item]) {
                const int t = --s_top[item];
                for (int j = 0; j < 3; ++j) { s_lo[item][j] = my_stack[6 * t + j]; s_hi[item][j] = my_stack[6 * t + 3 + j]; }
            }
        }
        const int n_act = __syncthreads_count(g == 0 && s_act[item]);   // nodes bounded this round
        if (n_act == 0) break;
        if (threadIdx.x == 0) atomicAdd(a.n_nodes, (unsigned long long)n_act);
        const bool valid = s_act[item];
        // bound rows of the node
        {
            float* xs = st + item * CB::R * CB::LD;
            if (g < 4) {
                const int k = g;
                for (int r = 0; r < CB::R; ++r) xs[r * CB::LD + k] = 0.f;
                if (valid && k < 3) {
                    const float lo = s_lo[item][k], hi = s_hi[item][k];
                    const float c = __fmul_rn(0.5f, __fadd_rn(lo, hi));
                    float h = __fsub_rn(hi, c);
                    if (C) h = fmaxf(__fsub_ru(hi, c), __fsub_ru(c, lo));
                    xs[k] = c;
                    if (SLOPE) {
                        xs[(1 + k) * CB::LD + k] = h;
                        xs[(5 + k) * CB::LD + k] = C ? __fmul_ru(gam0, h) : 0.f;
                        xs[4 * CB::LD + k] = C ? __fmul_ru(gam0, fabsf(c)) : 0.f;
                    } else if (a.interval) {
                        xs[(CB::R - 1) * CB::LD + k] = C ? __fmaf_ru(gam0, fabsf(c), h) : h;
                    } else {
                        xs[(1 + k) * CB::LD + k] = h;
                        xs[(CB::R - 1) * CB::LD + k] = C ? __fmul_ru(gam0, __fadd_ru(fabsf(c), h)) : 0.f;
                    }
                }
            }
        }
        __syncthreads();
        tile_forward<CB, C>(H, M.w, sW, sw_cap, resident, pb, st, ob);
        if (g == 0 && valid) {
            float lo, hi;
            if (SLOPE) slope_out_bounds<C>(ob + item * CB::R, pb.v, lo, hi);
            else affine_out_bounds<CB::R, C>(ob + item * CB::R, pb.v, lo, hi);
            s_lohi[item][0] = lo;
            s_lohi[item][1] = hi;
        }
        __syncthreads();
        // the 7 samples at center + extents * {0, +e_i, -e_i}
        {
            float* xs = st + item * CP::R * CP::LD;
            for (int r = g; r < 8; r += TPI) {
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (valid && r < 7) {
                    float p[3];
                    for (int k = 0; k < 3; ++k) p[k] = __fmul_rn(0.5f, __fadd_rn(s_lo[item][k], s_hi[item][k]));
                    if (r >= 1) {
                        const int ax = (r - 1) % 3;
                        const float w = __fsub_rn(s_hi[item][ax], s_lo[item][ax]);
                        p[ax] = __fadd_rn(p[ax], r <= 3 ? w : -w);
                    }
                    v.x = p[0]; v.y = p[1]; v.z = p[2];
                }
                *reinterpret_cast<float4*>(xs + r * CP::LD) = v;
            }
        }
        __syncthreads();
        tile_forward<CP, false>(H, M.w, sW, sw_cap, resident, pp, st, ob);
        if (g == 0 && valid) {
            const float* lo = s_lo[item];
            const float* hi = s_hi[item];
            const int type = sign_of_bounds(s_lohi[item][0], s_lohi[item][1], 0.f);
            float c[3], w[3];
            for (int k = 0; k < 3; ++k) { c[k] = __fmul_rn(0.5f, __fadd_rn(lo[k], hi[k])); w[k] = __fsub_rn(hi[k], lo[k]); }
            const float width = fmaxf(fmaxf(w[0], w[1]), w[2]);
            const float diag = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(w[0], w[0]), __fmul_rn(w[1], w[1])), __fmul_rn(w[2], w[2])));
            const float* q = s_qp[item];
            const float dx = __fsub_rn(q[0], c[0]), dy = __fsub_rn(q[1], c[1]), dz = __fsub_rn(q[2], c[2]);
            const float cd = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
            const float* v = ob + item * 8;
            bool neg = true, pos = true;
            for (int i = 0; i < 7; ++i) { neg &= v[i] < 0.f; pos &= v[i] > 0.f; }
            if (!(neg || pos)) {
                const float d = __fadd_rn(cd, diag);
                if (d < s_best[item]) {
                    s_best[item] = d;
                    for (int k = 0; k < 3; ++k) s_loc[item][k] = c[k];
                }
            }
            // prune with the query-to-box distance, a true lower bound (see k_search.cu)
            float bd2 = 0.f;
            for (int k = 0; k < 3; ++k) {
                const float dd = fmaxf(fmaxf(__fsub_rd(lo[k], q[k]), __fsub_rd(q[k], hi[k])), 0.f);
                bd2 = __fmaf_rd(dd, dd, bd2);
            }
            if (type == NIQ_SIGN_UNKNOWN && !(width < a.eps_w) && __fsqrt_rd(bd2) < s_best[item] - a.prune_tol) {
                const int t = s_top[item];
                if (t + 2 <= kBStack) {
                    int d = 0;
                    if (w[1] > w[d]) d = 1;
                    if (w[2] > w[d]) d = 2;
                    const float mid = __fmul_rn(0.5f, __fadd_rn(lo[d], hi[d]));
                    float alo[3] = {lo[0], lo[1], lo[2]}, ahi[3] = {hi[0], hi[1], hi[2]};
                    float blo[3] = {lo[0], lo[1], lo[2]}, bhi[3] = {hi[0], hi[1], hi[2]};
                    ahi[d] = mid;
                    blo[d] = mid;
                    const bool a_near = fabsf(q[d] - 0.5f * (lo[d] + mid)) <= fabsf(q[d] - 0.5f * (mid + hi[d]));
                    const float* f_lo = a_near ? blo : alo;
                    const float* f_hi = a_near ? bhi : ahi;
                    const float* s_lo2 = a_near ? alo : blo;
                    const float* s_hi2 = a_near ? ahi : bhi;
                    for (int k = 0; k < 3; ++k) {
                        my_stack[6 * t + k] = f_lo[k];
                        my_stack[6 * t + 3 + k] = f_hi[k];
                        my_stack[6 * (t + 1) + k] = s_lo2[k];
                        my_stack[6 * (t + 1) + 3 + k] = s_hi2[k];
                    }
                    s_top[item] = t + 2;
                } else {
                    niq_flag_error(a.err, NIQ_ERR_CAPACITY);
                }
            }
        }
        __syncthreads();
    }
}

template <bool C, bool SLOPE>
__global__ void __launch_bounds__(kBNT) k_batched_cp(BArgs a, const int* chunk_tpi) {
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    __shared__ NiqSpecHeader H;
    __shared__ BSlots S;
    __shared__ int s_chunk;
    int staged_model = -1;
    while (true) {
        __syncthreads();
        if (threadIdx.x == 0) s_chunk = (int)atomicAdd(a.next_chunk, 1ull);
        __syncthreads();
        const int c = s_chunk;
        if (c >= a.n_chunks) break;
        const BChunk ch = a.chunks[c];
        switch (chunk_tpi[c]) {
            case 4: run_chunk<4, C, SLOPE>(a, ch, H, S, smem, staged_model); break;
            case 8: run_chunk<8, C, SLOPE>(a, ch, H, S, smem, staged_model); break;
            case 16: run_chunk<16, C, SLOPE>(a, ch, H, S, smem, staged_model); break;
            default: run_chunk<32, C, SLOPE>(a, ch, H, S, smem, staged_model); break;
        }
    }
}

}  // namespace niq

#include <algorithm>
#include <vector>

using namespace niq;

namespace {
size_t al(size_t x) { return (x + 255) & ~size_t(255); }
size_t slots_max() { return (size_t)device_info().sm_count * 8 * 64; }
}  // namespace

extern "C" {

int niq_batched_closest_point_stats(const void* workspace, int64_t* budget_spent_out, int64_t* nodes_out,
                                    void* stream) {
    NIQ_REQUIRE(workspace, NIQ_ERR_INVALID_ARG, "null workspace");
    const char* b = reinterpret_cast<const char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
    unsigned long long v[2] = {0ull, 0ull};
    cudaStream_t s = as_stream(stream);
    NIQ_CUDA(cudaMemcpyAsync(v, b + 16, sizeof(v), cudaMemcpyDeviceToHost, s));
    NIQ_CUDA(cudaStreamSynchronize(s));
    if (budget_spent_out) *budget_spent_out = (int64_t)v[0];
    if (nodes_out) *nodes_out = (int64_t)v[1];
    return NIQ_OK;
}

size_t niq_batched_closest_point_workspace_size(int64_t total_queries, int32_t n_jobs) {
    const size_t n_chunks = (size_t)(total_queries / kMinChunk) + (size_t)n_jobs + 1;
    return al(64) + al(n_chunks * sizeof(BChunk)) + al(n_chunks * 4) + al((size_t)(n_jobs + 1) * sizeof(NiqModelRef)) +
           al(slots_max() * kBStack * 24) + 1024;
}

int niq_batched_closest_point(const niq_model* const* models, int32_t n_models, const niq_bound_opts* opts,
                              int32_t n_jobs, const int32_t* job_model, const int64_t* query_offset,
                              const int64_t* query_count, const float* query_points, const float* lower,
                              const float* upper, float eps, float* min_dist_out, float* min_loc_out,
                              int64_t node_budget, int32_t* status_out, void* workspace, size_t workspace_bytes,
                              void* stream) {
    NIQ_REQUIRE(models && opts && lower && upper && n_models >= 1 && n_jobs >= 0, NIQ_ERR_INVALID_ARG, "bad argument");
    NIQ_REQUIRE(opts->mode == NIQ_MODE_AFFINE_FIXED || opts->mode == NIQ_MODE_INTERVAL ||
                    opts->mode == NIQ_MODE_SLOPE_INTERVAL,
                NIQ_ERR_UNSUPPORTED, "batched closest point supports interval, affine_fixed and slope_interval");
    if (n_jobs == 0) return NIQ_OK;
    NIQ_REQUIRE(job_model && query_offset && query_count && query_points && min_dist_out && min_loc_out,
                NIQ_ERR_INVALID_ARG, "null array");
    long long total = 0;
    for (int j = 0; j < n_jobs; ++j) {
        NIQ_REQUIRE(job_model[j] >= 0 && job_model[j] < n_models && models[job_model[j]], NIQ_ERR_INVALID_ARG,
                    "job %d: bad model index", j);
        NIQ_REQUIRE(query_count[j] >= 0 && query_offset[j] >= 0 && query_offset[j] + query_count[j] < (1ll << 31),
                    NIQ_ERR_INVALID_ARG, "job %d: bad query range", j);
        total += query_count[j];
    }
    const size_t need = niq_batched_closest_point_workspace_size(total, n_jobs);
    NIQ_REQUIRE(workspace && workspace_bytes >= need, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed", need);
    cudaStream_t s = as_stream(stream);
    // the models the jobs use, in a compact table (at most n_jobs entries, which the
    // workspace size allows for, however large the caller's table is)
    std::vector<int> compact(n_models, -1);
    std::vector<NiqModelRef> refs;
    std::vector<int> used;
    for (int j = 0; j < n_jobs; ++j) {
        const int m = job_model[j];
        if (compact[m] < 0) {
            compact[m] = (int)refs.size();
            refs.push_back(models[m]->ref());
            used.push_back(m);
        }
    }
    // chunks, largest model cost first (longest-processing-time order)
    std::vector<BChunk> chunks;
    std::vector<double> cost;
    const int chunk_q = tune_value(kTuneBatchedChunk) > 0 ? tune_value(kTuneBatchedChunk) : kChunk;
    for (int j = 0; j < n_jobs; ++j) {
        const NiqSpecHeader& H = models[job_model[j]]->hdr;
        double per_q = 0;
        for (int l = 0; l < H.n_layers; ++l) per_q += (double)H.layers[l].in * H.layers[l].out;
        for (long long b = 0; b < query_count[j]; b += chunk_q) {
            BChunk c;
            c.model = compact[job_model[j]];
            c.q_begin = (int)(query_offset[j] + b);
            c.q_count = (int)std::min<long long>(chunk_q, query_count[j] - b);
            c.pad = 0;
            chunks.push_back(c);
            cost.push_back(per_q * c.q_count);
        }
    }
    std::vector<int> order(chunks.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
    std::vector<BChunk> sorted(chunks.size());
    std::vector<int> tpis(chunks.size());
    for (size_t i = 0; i < order.size(); ++i) {
        sorted[i] = chunks[order[i]];
        tpis[i] = tpi_for_width(models[used[sorted[i].model]]->hdr.max_width);
    }
    const int n_refs = (int)refs.size();
    const size_t n_chunks = sorted.size();
    char* b = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
    size_t off = 0;
    unsigned long long* next = reinterpret_cast<unsigned long long*>(b + off);
    int* err = reinterpret_cast<int*>(b + off + 8);
    off += al(64);
    BChunk* d_chunks = reinterpret_cast<BChunk*>(b + off);
    off += al(std::max<size_t>(n_chunks, 1) * sizeof(BChunk));
    int* d_tpi = reinterpret_cast<int*>(b + off);
    off += al(std::max<size_t>(n_chunks, 1) * 4);
    NiqModelRef* d_models = reinterpret_cast<NiqModelRef*>(b + off);
    off += al((size_t)n_refs * sizeof(NiqModelRef));
    float* stacks = reinterpret_cast<float*>(b + off);
    NIQ_REQUIRE(off + slots_max() * kBStack * 24 <= workspace_bytes - 256, NIQ_ERR_CAPACITY, "workspace too small");
    NIQ_CUDA(cudaMemsetAsync(b, 0, 64, s));
    if (status_out) NIQ_CUDA(cudaMemsetAsync(status_out, 0, 4, s));
    if (n_chunks == 0) return NIQ_OK;
    // host staging: these copies are synchronous w.r.t. the host buffers (pageable memory)
    NIQ_CUDA(cudaMemcpyAsync(d_chunks, sorted.data(), n_chunks * sizeof(BChunk), cudaMemcpyHostToDevice, s));
    NIQ_CUDA(cudaMemcpyAsync(d_tpi, tpis.data(), n_chunks * 4, cudaMemcpyHostToDevice, s));
    NIQ_CUDA(cudaMemcpyAsync(d_models, refs.data(), n_refs * sizeof(NiqModelRef), cudaMemcpyHostToDevice, s));
    BArgs a;
    a.models = d_models;
    a.chunks = d_chunks;
    a.n_chunks = (int)n_chunks;
    a.q = query_points;
    a.min_dist = min_dist_out;
    a.min_loc = min_loc_out;
    for (int k = 0; k < 3; ++k) { a.lu[k] = lower[k]; a.lu[3 + k] = upper[k]; }
    a.eps_w = eps / sqrtf(3.f);
    a.interval = opts->mode == NIQ_MODE_INTERVAL;
    a.stacks = stacks;
    a.next_chunk = next;
    a.n_spent = reinterpret_cast<unsigned long long*>(b + 16);   // in the header cleared above
    a.n_nodes = reinterpret_cast<unsigned long long*>(b + 24);
    a.err = status_out ? reinterpret_cast<int*>(status_out) : err;
    a.node_budget = node_budget > 0 ? node_budget : (1ll << 62);
    a.prune_tol = eps;
    const size_t smem = kSmemBudget;
    a.smem_floats = (int)(smem / 4);
    const bool cons = opts->conservative != 0, slope = opts->mode == NIQ_MODE_SLOPE_INTERVAL;
    auto run = [&](auto kern) -> int {
        int rc = prepare_kernel(kern, smem);
        if (rc) return rc;
        int grid = 0;
        rc = persistent_grid(kern, kBNT, smem, (long long)n_chunks, &grid, tune_value(kTuneBatchedCtasPerSm));
        if (rc) return rc;
        NIQ_REQUIRE((size_t)grid * 64 <= slots_max(), NIQ_ERR_UNSUPPORTED, "slot count");
        kern<<<grid, kBNT, smem, s>>>(a, d_tpi);
        NIQ_CUDA(cudaGetLastError());
        return NIQ_OK;
    };
    int rc;
    if (slope) rc = cons ? run(k_batched_cp<true, true>) : run(k_batched_cp<false, true>);
    else rc = cons ? run(k_batched_cp<true, false>) : run(k_batched_cp<false, false>);
    if (rc) return rc;
    if (status_out) return NIQ_OK;
    int e = 0;
    NIQ_CUDA(cudaMemcpyAsync(&e, err, 4, cudaMemcpyDeviceToHost, s));
    NIQ_CUDA(cudaStreamSynchronize(s));
    NIQ_REQUIRE(e != NIQ_ERR_CAPACITY, NIQ_ERR_CAPACITY, "closest-point stack depth %d exceeded", kBStack);
    NIQ_REQUIRE(e == 0, e, "closest-point node budget of %lld nodes per query exhausted; results are upper bounds",
                (long long)a.node_budget);
    return NIQ_OK;
}

}  // extern "C"
