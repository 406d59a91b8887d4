// k_tree.cu -- construct_uniform_unknown_levelset_tree (src/kd_tree.py:19-218).
//
// Breadth-first: level L classifies every node of the level (classify_box, v = 3,
// src/implicit_function.py:28-37); NEGATIVE nodes go to the interior list and POSITIVE
// ones to the exterior list when requested; UNKNOWN nodes split at the midpoint of
// their first longest axis into children A = [lo, hi with hi[d] = mid] and
// B = [lo with lo[d] = mid, hi] (src/kd_tree.py:38,70-77) -- or, on the last round, are
// the result.  A round is the last when it starts with >= node_terminate_thresh nodes
// or is round split_depth (src/kd_tree.py:136-152).
//
// k_tree<COOP=true>: one cooperative launch runs every level; CTAs claim chunks of the
// level's node array with an atomic counter, and a bounded grid barrier separates
// levels.  k_tree<COOP=false>: one level per launch, the host reads the next level's
// size after each (the plain form, as the reference's per-level host loop).
// Node order inside a level is whatever the atomics produce; results are node sets.
#include <mutex>
#include "tree_common.cuh"

namespace niq {

template <int TPI, bool C, bool SLOPE, bool COOP>
__global__ void __launch_bounds__(kNT) k_tree(NiqModelRef M, TreeParams P, TreeWs* ws, TreeBufs B, int level0,
                                              int fixed_floats, int sw_cap, int resident) {
    using Cfg = typename std::conditional<SLOPE, TileCfg<8, 4, TPI, kNT>, TileCfg<5, 1, TPI, kNT>>::type;
    constexpr int ITEMS = Cfg::ITEMS, R = Cfg::R, LD = Cfg::LD;
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    float* st = smem;
    float* ob = st + Cfg::STATE_FLOATS;
    float* sW = smem + fixed_floats;
    __shared__ NiqSpecHeader H;
    __shared__ float s_lo[ITEMS][3], s_hi[ITEMS][3];
    __shared__ long long s_base;
    __shared__ unsigned long long s_boxes;
    load_header(H, M.hdr);
    __syncthreads();
    if (resident) stage_floats(sW, M.w, H.n_weight_floats);
    const RowPlan plan{SLOPE ? ROWS_SLOPE : ROWS_AFFINE, P.mode_interval ? 0 : 3, 0};
    const int item = threadIdx.x / TPI, g = threadIdx.x % TPI;
    const float gam0 = C ? H.layers[0].gamma : 0.f;
    unsigned int epoch = 0;
    if (threadIdx.x == 0) s_boxes = 0;
    __syncthreads();  // staged weights and the counter visible before warps start on their own

    for (int L = level0; L < kTreeMaxLevels; ++L) {
        const long long n_in_raw = (long long)*((volatile unsigned long long*)&ws->level_count[L]);
        if (n_in_raw > B.cap) {  // the previous level overflowed: its nodes were not stored
            niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
            break;
        }
        const long long n_in = n_in_raw;
        const bool quit = (n_in >= P.thresh) || (L + 1 >= P.n_rounds) || (n_in == 0) || (L + 1 == kTreeMaxLevels);
        const long long n_lim = n_in < P.batch_end ? n_in : P.batch_end;   // end of this launch's nodes
        const float* in_lo = B.lvl_lo[L & 1];
        const float* in_hi = B.lvl_hi[L & 1];
        float* out_lo = B.lvl_lo[(L + 1) & 1];
        float* out_hi = B.lvl_hi[(L + 1) & 1];
        // One tile of nodes starting at nid0: the items of the whole CTA (block mode) or of
        // this warp only (warp mode: weights resident, warps claim and run independently).
        auto tile = [&](long long nid0, auto warp_mode) {
            constexpr bool WM = decltype(warp_mode)::value;
            const long long nid = nid0 + (WM ? (item % (32 / TPI)) : item);
            const bool valid = nid < n_lim;
            // ---- input rows: center and diagonal half extents (src/implicit_function.py:33-37)
            float* xs = st + item * R * LD;
            if (g < 4) {
                const int k = g;
                for (int r = 0; r < R; ++r) xs[r * LD + k] = 0.f;
                if (valid && k < 3) {
                    const float lo = in_lo[3 * nid + k], hi = in_hi[3 * nid + k];
                    s_lo[item][k] = lo;
                    s_hi[item][k] = hi;
                    const float c = __fmul_rn(0.5f, __fadd_rn(lo, hi));
                    float h = __fsub_rn(hi, c);
                    if (C) h = fmaxf(__fsub_ru(hi, c), __fsub_ru(c, lo));
                    xs[k] = c;
                    if (SLOPE) {
                        xs[(1 + k) * LD + k] = h;
                        xs[(5 + k) * LD + k] = C ? __fmul_ru(gam0, h) : 0.f;
                        xs[4 * LD + k] = C ? __fmul_ru(gam0, fabsf(c)) : 0.f;
                    } else if (P.mode_interval) {
                        xs[(R - 1) * LD + k] = C ? __fmaf_ru(gam0, fabsf(c), h) : h;
                    } else {
                        xs[(1 + k) * LD + k] = h;
                        xs[(R - 1) * LD + k] = C ? __fmul_ru(gam0, __fadd_ru(fabsf(c), h)) : 0.f;
                    }
                }
            }
            if (WM) __syncwarp();
            else __syncthreads();
            tile_forward<Cfg, C, WM>(H, M.w, sW, sw_cap, resident, plan, st, ob);
            // ---- consume: one owner lane per item; every lane joins the warp votes
            int type = -1;
            if (g == 0 && valid) {
                float lo, hi;
                if (SLOPE) slope_out_bounds<C>(ob + item * R, plan.v, lo, hi);
                else affine_out_bounds<Cfg::R, C>(ob + item * R, plan.v, lo, hi);
                type = sign_of_bounds(lo, hi, P.offset);
            }
            const bool is_unknown = type == NIQ_SIGN_UNKNOWN;
            const bool is_int = P.with_interior && type == NIQ_SIGN_NEGATIVE;
            const bool is_ext = P.with_exterior && type == NIQ_SIGN_POSITIVE;
            const long long pi = niq_warp_reserve(&ws->n_interior, is_int, 1);
            const long long pe = niq_warp_reserve(&ws->n_exterior, is_ext, 1);
            const long long pu = quit ? niq_warp_reserve(&ws->n_unknown, is_unknown, 1) : -1;
            const long long pc = quit ? -1 : niq_warp_reserve(&ws->level_count[L + 1], is_unknown, 2);
            if (g == 0 && valid) {
                const float* lo = s_lo[item];
                const float* hi = s_hi[item];
                if (is_int) { if (pi < B.cap) put_node(B.res_lo[1], B.res_hi[1], pi, lo, hi); else niq_flag_error(&ws->err, NIQ_ERR_CAPACITY); }
                if (is_ext) { if (pe < B.cap) put_node(B.res_lo[2], B.res_hi[2], pe, lo, hi); else niq_flag_error(&ws->err, NIQ_ERR_CAPACITY); }
                if (is_unknown) {
                    if (quit) {
                        if (pu < B.cap) put_node(B.res_lo[0], B.res_hi[0], pu, lo, hi);
                        else niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
                    } else if (pc + 1 < B.cap) {
                        // split along the first longest axis (jnp.argmax: first maximum);
                        // selects rather than a runtime index keep the boxes in registers
                        const float l0 = lo[0], l1 = lo[1], l2 = lo[2], h0 = hi[0], h1 = hi[1], h2 = hi[2];
                        const float e0 = __fsub_rn(h0, l0), e1 = __fsub_rn(h1, l1), e2 = __fsub_rn(h2, l2);
                        int d = 0;
                        float em = e0;
                        if (e1 > em) { d = 1; em = e1; }
                        if (e2 > em) { d = 2; }
                        const float mid = d == 0 ? __fmul_rn(0.5f, __fadd_rn(l0, h0))
                                        : d == 1 ? __fmul_rn(0.5f, __fadd_rn(l1, h1))
                                                 : __fmul_rn(0.5f, __fadd_rn(l2, h2));
                        // child A = [lo, hi with hi[d] = mid], child B = [lo with lo[d] = mid, hi]
                        float* ol = out_lo + 3 * pc;
                        float* oh = out_hi + 3 * pc;
                        ol[0] = l0; ol[1] = l1; ol[2] = l2;
                        oh[0] = d == 0 ? mid : h0; oh[1] = d == 1 ? mid : h1; oh[2] = d == 2 ? mid : h2;
                        ol[3] = d == 0 ? mid : l0; ol[4] = d == 1 ? mid : l1; ol[5] = d == 2 ? mid : l2;
                        oh[3] = h0; oh[4] = h1; oh[5] = h2;
                    } else {
                        niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
                    }
                }
                atomicAdd(&s_boxes, 1ull);
            }
        };
        if (resident) {
            // warp mode: a warp claims 32 / TPI consecutive nodes at a time
            while (true) {
                unsigned long long b0 = 0;
                if ((threadIdx.x & 31) == 0)
                    b0 = (unsigned long long)P.batch_start + atomicAdd(&ws->grab[L], (unsigned long long)(32 / TPI));
                b0 = __shfl_sync(0xffffffffu, b0, 0);
                if ((long long)b0 >= n_lim) break;
                tile((long long)b0, std::integral_constant<bool, true>());
            }
        } else {
            while (true) {
                __syncthreads();
                if (threadIdx.x == 0)
                    s_base = P.batch_start + (long long)atomicAdd(&ws->grab[L], (unsigned long long)ITEMS);
                __syncthreads();
                const long long base = s_base;
                if (base >= n_lim) break;
                tile(base, std::integral_constant<bool, false>());
            }
        }
        if (!COOP) {
            if (threadIdx.x == 0) {
                if (quit) atomicMax(&ws->last_level, L);
            }
            break;
        }
        if (quit) {
            if (blockIdx.x == 0 && threadIdx.x == 0) ws->last_level = L;
            break;
        }
        if (!niq_grid_barrier(&ws->barrier, gridDim.x, epoch, &ws->err, P.barrier_polls)) break;
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_boxes) atomicAdd(&ws->n_boxes, s_boxes);
}

struct TreeLayout {
    size_t hdr, lvl[2], res[3], total;
};

static TreeLayout tree_layout(long long cap, int flags) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    TreeLayout L;
    const size_t nb = al((size_t)cap * 24);  // lower (cap,3) then upper (cap,3)
    L.hdr = 0;
    size_t off = al(sizeof(TreeWs));
    L.lvl[0] = off; off += nb;
    L.lvl[1] = off; off += nb;
    L.res[0] = off; off += nb;
    L.res[1] = off; if (flags & NIQ_TREE_WITH_INTERIOR) off += nb;
    L.res[2] = off; if (flags & NIQ_TREE_WITH_EXTERIOR) off += nb;
    L.total = off + 256;
    return L;
}

static char* ws_base(void* ws) {
    return reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
}

static void tree_bufs(void* workspace, long long cap, int flags, TreeBufs& B) {
    const TreeLayout TL = tree_layout(cap, flags);
    char* base = ws_base(workspace);
    auto lo = [&](size_t off) { return reinterpret_cast<float*>(base + off); };
    auto hi = [&](size_t off) { return reinterpret_cast<float*>(base + off + (size_t)cap * 12); };
    for (int i = 0; i < 2; ++i) { B.lvl_lo[i] = lo(TL.lvl[i]); B.lvl_hi[i] = hi(TL.lvl[i]); }
    for (int i = 0; i < 3; ++i) { B.res_lo[i] = lo(TL.res[i]); B.res_hi[i] = hi(TL.res[i]); }
    B.cap = cap;
}

__global__ void k_tree_finish(TreeWs* ws, long long* counts) {
    counts[0] = (long long)ws->n_unknown;
    counts[1] = (long long)ws->n_interior;
    counts[2] = (long long)ws->n_exterior;
    counts[3] = (long long)ws->n_boxes;
}

// The tensor-core tree serves affine_fixed with outward rounding when 3xTF32 products
// are asked for, on the models it supports.  It is not the default: measured on the
// 12-sphere model it is slower than the FP32 tile engine (one 8-warp CTA per SM leaves
// its CUDA-core work -- the err row, the linearisations -- latency-bound), and the
// larger rounding bound of split products keeps about 1/4 more leaves unknown at 24
// bisections.
static bool use_tree_tc(const NiqSpecHeader& H, const niq_bound_opts* opts) {
    return opts->mode == NIQ_MODE_AFFINE_FIXED && opts->conservative != 0 && opts->products == NIQ_PRODUCTS_3XTF32 &&
           tree_tc_eligible(H);
}

// Counts to the caller's array, then the kernels' error status (syncs the stream).
static int finish_tree(TreeWs* ws, long long* counts, long long cap, cudaStream_t s) {
    k_tree_finish<<<1, 1, 0, s>>>(ws, counts);
    NIQ_CUDA(cudaGetLastError());
    int err = 0;
    NIQ_CUDA(cudaMemcpyAsync(&err, &ws->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    NIQ_CUDA(cudaStreamSynchronize(s));
    NIQ_REQUIRE(err == 0, err, err == NIQ_ERR_CAPACITY ? "node capacity %lld exceeded" : "tree kernel error (%lld)",
                err == NIQ_ERR_CAPACITY ? cap : (long long)err);
    return NIQ_OK;
}

template <bool COOP>
static int run_tree(const niq_model* m, const niq_bound_opts* opts, const float* lower, const float* upper,
                    int split_depth, long long thresh, float offset, int flags, long long cap, long long* counts,
                    void* workspace, size_t ws_bytes, cudaStream_t s, long long batch = 0) {
    NIQ_REQUIRE(m && opts && lower && upper && counts, NIQ_ERR_INVALID_ARG, "null argument");
    const int mode = opts->mode;
    NIQ_REQUIRE(mode == NIQ_MODE_AFFINE_FIXED || mode == NIQ_MODE_INTERVAL || mode == NIQ_MODE_SLOPE_INTERVAL,
                NIQ_ERR_UNSUPPORTED, "the tree kernels support the interval, affine_fixed and slope_interval modes");
    NIQ_REQUIRE(split_depth >= 0 || thresh > 0, NIQ_ERR_INVALID_ARG,
                "must specify at least one of node_terminate_thresh or split_depth as a terminating condition");
    NIQ_REQUIRE(split_depth < kTreeMaxLevels, NIQ_ERR_INVALID_ARG, "split_depth %d exceeds %d", split_depth, kTreeMaxLevels - 1);
    NIQ_REQUIRE(cap >= 2, NIQ_ERR_INVALID_ARG, "node capacity too small");
    const TreeLayout TL = tree_layout(cap, flags);
    NIQ_REQUIRE(workspace && ws_bytes >= TL.total, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed", TL.total);
    TreeBufs B;
    tree_bufs(workspace, cap, flags, B);
    TreeWs* ws = reinterpret_cast<TreeWs*>(ws_base(workspace));
    NIQ_CUDA(cudaMemsetAsync(ws, 0, sizeof(TreeWs), s));
    // root node and level 0 count
    NIQ_CUDA(cudaMemcpyAsync(B.lvl_lo[0], lower, 12, cudaMemcpyHostToDevice, s));
    NIQ_CUDA(cudaMemcpyAsync(B.lvl_hi[0], upper, 12, cudaMemcpyHostToDevice, s));
    const unsigned long long one = 1;
    NIQ_CUDA(cudaMemcpyAsync(&ws->level_count[0], &one, 8, cudaMemcpyHostToDevice, s));
    TreeParams P;
    P.n_rounds = split_depth >= 0 ? split_depth + 1 : kTreeMaxLevels;
    P.thresh = thresh > 0 ? thresh : (1ll << 62);
    P.offset = offset;
    P.with_interior = (flags & NIQ_TREE_WITH_INTERIOR) != 0;
    P.with_exterior = (flags & NIQ_TREE_WITH_EXTERIOR) != 0;
    P.mode_interval = mode == NIQ_MODE_INTERVAL;
    P.batch_start = 0;
    P.batch_end = 1ll << 62;
    P.barrier_polls = barrier_polls();
    P.mbar_polls = mbar_polls();
    const bool cons = opts->conservative != 0, slope = mode == NIQ_MODE_SLOPE_INTERVAL;
    const int tpi = tpi_for_width(m->hdr.max_width);
    int rc = NIQ_OK;
    if (use_tree_tc(m->hdr, opts)) {
        TreeLaunch T{m->ref(), &m->hdr, P, ws, B, s, COOP, batch};
        rc = run_tree_tc(T);
        if (rc) return rc;
        return finish_tree(ws, counts, cap, s);
    }
    auto run = [&](auto kern, int R, int TPIv) -> int {
        const int items = kNT / TPIv;
        const int state = items * R * (TPIv * 8 + 4) + ((items * R + 3) & ~3);
        SmemPlan p = plan_smem(state, m->hdr.n_weight_floats, max_layer_floats(m->hdr));
        NIQ_REQUIRE(p.resident || p.sw_cap >= 5 * m->hdr.max_width, NIQ_ERR_UNSUPPORTED, "shared memory too small");
        int r2 = prepare_kernel(kern, p.bytes);
        if (r2) return r2;
        int per_sm = 0;
        NIQ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kNT, p.bytes));
        NIQ_REQUIRE(per_sm >= 1, NIQ_ERR_UNSUPPORTED, "tree kernel does not fit on an SM");
        if (tune_value(kTuneTreeCtasPerSm) > 0 && per_sm > tune_value(kTuneTreeCtasPerSm))
            per_sm = tune_value(kTuneTreeCtasPerSm);
        const int grid = per_sm * device_info().sm_count;
        NiqModelRef M = m->ref();
        int level0 = 0;
        int fixed = p.fixed_floats, cap_ = p.sw_cap, res = p.resident;
        if (COOP) {
            void* args[] = {&M, &P, &ws, &B, &level0, &fixed, &cap_, &res};
            NIQ_CUDA(cudaLaunchCooperativeKernel((const void*)kern, grid, kNT, args, p.bytes, s));
            return NIQ_OK;
        }
        // plain: one launch per level, host reads the next level size (src/kd_tree.py:137-198)
        for (int L = 0; L < kTreeMaxLevels; ++L) {
            unsigned long long cnt[2] = {0, 0};
            NIQ_CUDA(cudaMemcpyAsync(cnt, &ws->level_count[L], 8, cudaMemcpyDeviceToHost, s));
            NIQ_CUDA(cudaStreamSynchronize(s));
            const long long n_in = (long long)cnt[0];
            const bool quit = (n_in >= P.thresh) || (L + 1 >= P.n_rounds) || (n_in == 0) || (L + 1 == kTreeMaxLevels);
            // whole level per launch, or the reference's schedule: one launch per batch of
            // `batch` nodes (src/kd_tree.py:161-172)
            const long long step = batch > 0 ? batch : (n_in > 0 ? n_in : 1);
            for (long long b0 = 0; b0 < (n_in > 0 ? n_in : 1); b0 += step) {
                TreeParams Pb = P;
                Pb.batch_start = b0;
                Pb.batch_end = b0 + step;
                if (b0 > 0) NIQ_CUDA(cudaMemsetAsync(&ws->grab[L], 0, sizeof(unsigned long long), s));
                const long long nb = (n_in - b0 < step ? n_in - b0 : step);
                long long tiles = (nb + items - 1) / items;
                int g = (int)(tiles < grid ? (tiles < 1 ? 1 : tiles) : grid);
                kern<<<g, kNT, p.bytes, s>>>(M, Pb, ws, B, L, fixed, cap_, res);
                NIQ_CUDA(cudaGetLastError());
            }
            if (quit) break;
        }
        return NIQ_OK;
    };
#define NIQ_TREE(CC, SL) NIQ_DISPATCH_TPI(tpi, { rc = run(k_tree<TPI, CC, SL, COOP>, SL ? 8 : 5, TPI); })
    if (slope) { if (cons) { NIQ_TREE(true, true); } else { NIQ_TREE(false, true); } }
    else { if (cons) { NIQ_TREE(true, false); } else { NIQ_TREE(false, false); } }
#undef NIQ_TREE
    if (rc) return rc;
    return finish_tree(ws, counts, cap, s);
}

}  // namespace niq

using namespace niq;

extern "C" {

size_t niq_tree_workspace_size(int64_t node_capacity, int32_t flags) { return tree_layout(node_capacity, flags).total; }

int niq_levelset_tree(const niq_model* model, const niq_bound_opts* opts, const float* lower, const float* upper,
                      int32_t split_depth, int64_t node_terminate_thresh, float offset, int32_t flags,
                      int64_t node_capacity, int64_t* counts_out, void* workspace, size_t workspace_bytes,
                      void* stream) {
    return run_tree<true>(model, opts, lower, upper, split_depth, node_terminate_thresh, offset, flags, node_capacity,
                          reinterpret_cast<long long*>(counts_out), workspace, workspace_bytes, as_stream(stream));
}

int niq_levelset_tree_plain(const niq_model* model, const niq_bound_opts* opts, const float* lower,
                            const float* upper, int32_t split_depth, int64_t node_terminate_thresh, float offset,
                            int32_t flags, int64_t node_capacity, int64_t* counts_out, void* workspace,
                            size_t workspace_bytes, void* stream) {
    return run_tree<false>(model, opts, lower, upper, split_depth, node_terminate_thresh, offset, flags, node_capacity,
                           reinterpret_cast<long long*>(counts_out), workspace, workspace_bytes, as_stream(stream));
}

int niq_levelset_tree_batches(const niq_model* model, const niq_bound_opts* opts, const float* lower,
                              const float* upper, int32_t split_depth, int64_t node_terminate_thresh, float offset,
                              int32_t flags, int64_t batch_process_size, int64_t node_capacity, int64_t* counts_out,
                              void* workspace, size_t workspace_bytes, void* stream) {
    NIQ_REQUIRE(batch_process_size >= 1, NIQ_ERR_INVALID_ARG, "batch_process_size must be >= 1");
    return run_tree<false>(model, opts, lower, upper, split_depth, node_terminate_thresh, offset, flags, node_capacity,
                           reinterpret_cast<long long*>(counts_out), workspace, workspace_bytes, as_stream(stream),
                           batch_process_size);
}

int niq_tree_engine(const niq_model* model, const niq_bound_opts* opts, int32_t* engine_out) {
    NIQ_REQUIRE(model && opts && engine_out, NIQ_ERR_INVALID_ARG, "null argument");
    const int mode = opts->mode;
    if (mode == NIQ_MODE_AFFINE_TRUNCATE || mode == NIQ_MODE_AFFINE_APPEND || mode == NIQ_MODE_AFFINE_ALL)
        *engine_out = NIQ_TREE_ENGINE_GROWING;
    else
        *engine_out = use_tree_tc(model->hdr, opts) ? NIQ_TREE_ENGINE_TENSOR : NIQ_TREE_ENGINE_FP32;
    return NIQ_OK;
}

int niq_tree_result(void* workspace, int64_t node_capacity, int32_t flags, int32_t kind, float** lower, float** upper) {
    NIQ_REQUIRE(workspace && lower && upper && kind >= 0 && kind <= 2, NIQ_ERR_INVALID_ARG, "bad argument");
    NIQ_REQUIRE(kind != 1 || (flags & NIQ_TREE_WITH_INTERIOR), NIQ_ERR_INVALID_ARG, "tree built without interior nodes");
    NIQ_REQUIRE(kind != 2 || (flags & NIQ_TREE_WITH_EXTERIOR), NIQ_ERR_INVALID_ARG, "tree built without exterior nodes");
    TreeBufs B;
    tree_bufs(workspace, node_capacity, flags, B);
    *lower = B.res_lo[kind];
    *upper = B.res_hi[kind];
    return NIQ_OK;
}

}  // extern "C"

// ==========================================================================================
// Growing-term modes (affine_truncate, affine_append, affine_all): the reference's level
// loop (src/kd_tree.py:137-198) over the growing-term engine of niq_classify_boxes.  Each
// level is cut into chunks of kTreeGrowChunk nodes: a kernel writes their boxes as
// center + diagonal vectors (src/implicit_function.py:33-37), the engine classifies them,
// and a second kernel appends results and children exactly as k_tree does; the host reads
// the next level's size.  Any mode is accepted (the fixed ones give k_tree's node sets).
// ==========================================================================================
namespace niq {

constexpr long long kTreeGrowChunk = 1 << 16;

__global__ void k_tree_boxes(const float* lo, const float* hi, long long s, long long n, int cons, float* center,
                             float* vecs) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float l = lo[3 * (s + i) + k], h = hi[3 * (s + i) + k];
        const float c = __fmul_rn(0.5f, __fadd_rn(l, h));
        const float half = cons ? fmaxf(__fsub_ru(h, c), __fsub_ru(c, l)) : __fsub_rn(h, c);
        center[3 * i + k] = c;
#pragma unroll
        for (int j = 0; j < 3; ++j) vecs[9 * i + 3 * k + j] = j == k ? half : 0.f;
    }
}

// Results and children of nodes s .. s + n - 1 of level L from their signs (k_tree's
// consume step, one thread per node; every lane of a warp joins the votes).
__global__ void k_tree_consume(const int* sign, long long s, long long n, int quit, TreeParams P, TreeWs* ws, TreeBufs B,
                               int L) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    const long long nid = s + i;
    const int type = valid ? sign[i] : -1;
    const bool is_unknown = type == NIQ_SIGN_UNKNOWN;
    const bool is_int = P.with_interior && type == NIQ_SIGN_NEGATIVE;
    const bool is_ext = P.with_exterior && type == NIQ_SIGN_POSITIVE;
    const long long pi = niq_warp_reserve(&ws->n_interior, is_int, 1);
    const long long pe = niq_warp_reserve(&ws->n_exterior, is_ext, 1);
    const long long pu = quit ? niq_warp_reserve(&ws->n_unknown, is_unknown, 1) : -1;
    const long long pc = quit ? -1 : niq_warp_reserve(&ws->level_count[L + 1], is_unknown, 2);
    niq_warp_reserve(&ws->n_boxes, valid, 1);
    if (!valid) return;
    const float* in_lo = B.lvl_lo[L & 1];
    const float* in_hi = B.lvl_hi[L & 1];
    const float lo[3] = {in_lo[3 * nid], in_lo[3 * nid + 1], in_lo[3 * nid + 2]};
    const float hi[3] = {in_hi[3 * nid], in_hi[3 * nid + 1], in_hi[3 * nid + 2]};
    if (is_int) { if (pi < B.cap) put_node(B.res_lo[1], B.res_hi[1], pi, lo, hi); else niq_flag_error(&ws->err, NIQ_ERR_CAPACITY); }
    if (is_ext) { if (pe < B.cap) put_node(B.res_lo[2], B.res_hi[2], pe, lo, hi); else niq_flag_error(&ws->err, NIQ_ERR_CAPACITY); }
    if (!is_unknown) return;
    if (quit) {
        if (pu < B.cap) put_node(B.res_lo[0], B.res_hi[0], pu, lo, hi);
        else niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
        return;
    }
    if (pc + 1 >= B.cap) {
        niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
        return;
    }
    // split along the first longest axis (src/kd_tree.py:38,70-77)
    const float e0 = __fsub_rn(hi[0], lo[0]), e1 = __fsub_rn(hi[1], lo[1]), e2 = __fsub_rn(hi[2], lo[2]);
    int d = 0;
    float em = e0;
    if (e1 > em) { d = 1; em = e1; }
    if (e2 > em) { d = 2; }
    const float mid = d == 0 ? __fmul_rn(0.5f, __fadd_rn(lo[0], hi[0]))
                    : d == 1 ? __fmul_rn(0.5f, __fadd_rn(lo[1], hi[1]))
                             : __fmul_rn(0.5f, __fadd_rn(lo[2], hi[2]));
    const float ahi[3] = {d == 0 ? mid : hi[0], d == 1 ? mid : hi[1], d == 2 ? mid : hi[2]};
    const float blo[3] = {d == 0 ? mid : lo[0], d == 1 ? mid : lo[1], d == 2 ? mid : lo[2]};
    float* out_lo = B.lvl_lo[(L + 1) & 1];
    float* out_hi = B.lvl_hi[(L + 1) & 1];
    put_node(out_lo, out_hi, pc, lo, ahi);
    put_node(out_lo, out_hi, pc + 1, blo, hi);
}

// Scratch after the tree layout: chunk boxes (center, vecs), signs, the engine's workspace.
struct GrowLayout {
    size_t center, vecs, sign, cws, cws_bytes, total;
};

static GrowLayout grow_layout(const niq_model* m, const niq_bound_opts* opts, long long cap, int flags) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    GrowLayout G;
    size_t off = al(tree_layout(cap, flags).total);
    G.center = off; off += al((size_t)kTreeGrowChunk * 12);
    G.vecs = off; off += al((size_t)kTreeGrowChunk * 36);
    G.sign = off; off += al((size_t)kTreeGrowChunk * 4);
    G.cws = off;
    G.cws_bytes = niq_classify_workspace_size(m, opts, kTreeGrowChunk, 3);
    off += al(G.cws_bytes);
    G.total = off + 256;
    return G;
}

}  // namespace niq

extern "C" size_t niq_tree_growing_workspace_size(const niq_model* model, const niq_bound_opts* opts,
                                                  int64_t node_capacity, int32_t flags) {
    if (!model || !opts || node_capacity < 2) return 0;
    return niq::grow_layout(model, opts, node_capacity, flags).total;
}

extern "C" int niq_levelset_tree_growing(const niq_model* model, const niq_bound_opts* opts, const float* lower,
                                         const float* upper, int32_t split_depth, int64_t node_terminate_thresh,
                                         float offset, int32_t flags, int64_t node_capacity, int64_t* counts_out,
                                         void* workspace, size_t workspace_bytes, void* stream) {
    using namespace niq;
    NIQ_REQUIRE(model && opts && lower && upper && counts_out, NIQ_ERR_INVALID_ARG, "null argument");
    NIQ_REQUIRE(split_depth >= 0 || node_terminate_thresh > 0, NIQ_ERR_INVALID_ARG,
                "must specify at least one of node_terminate_thresh or split_depth as a terminating condition");
    NIQ_REQUIRE(split_depth < kTreeMaxLevels, NIQ_ERR_INVALID_ARG, "split_depth %d exceeds %d", split_depth,
                kTreeMaxLevels - 1);
    NIQ_REQUIRE(node_capacity >= 2, NIQ_ERR_INVALID_ARG, "node capacity too small");
    const GrowLayout G = grow_layout(model, opts, node_capacity, flags);
    NIQ_REQUIRE(workspace && workspace_bytes >= G.total, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed", G.total);
    cudaStream_t s = as_stream(stream);
    TreeBufs B;
    tree_bufs(workspace, node_capacity, flags, B);
    char* base = ws_base(workspace);
    TreeWs* ws = reinterpret_cast<TreeWs*>(base);
    float* center = reinterpret_cast<float*>(base + G.center);
    float* vecs = reinterpret_cast<float*>(base + G.vecs);
    int* sign = reinterpret_cast<int*>(base + G.sign);
    void* cws = base + G.cws;
    NIQ_CUDA(cudaMemsetAsync(ws, 0, sizeof(TreeWs), s));
    NIQ_CUDA(cudaMemcpyAsync(B.lvl_lo[0], lower, 12, cudaMemcpyHostToDevice, s));
    NIQ_CUDA(cudaMemcpyAsync(B.lvl_hi[0], upper, 12, cudaMemcpyHostToDevice, s));
    const unsigned long long one = 1;
    NIQ_CUDA(cudaMemcpyAsync(&ws->level_count[0], &one, 8, cudaMemcpyHostToDevice, s));
    TreeParams P{};
    P.n_rounds = split_depth >= 0 ? split_depth + 1 : kTreeMaxLevels;
    P.thresh = node_terminate_thresh > 0 ? node_terminate_thresh : (1ll << 62);
    P.offset = offset;
    P.with_interior = (flags & NIQ_TREE_WITH_INTERIOR) != 0;
    P.with_exterior = (flags & NIQ_TREE_WITH_EXTERIOR) != 0;
    const int cons = opts->conservative != 0;
    for (int L = 0; L < kTreeMaxLevels; ++L) {
        unsigned long long cnt = 0;
        NIQ_CUDA(cudaMemcpyAsync(&cnt, &ws->level_count[L], 8, cudaMemcpyDeviceToHost, s));
        NIQ_CUDA(cudaStreamSynchronize(s));
        const long long n_in = (long long)cnt;
        if (n_in > node_capacity) break;   // reported by the capacity flag of the level before
        const bool quit = (n_in >= P.thresh) || (L + 1 >= P.n_rounds) || (n_in == 0) || (L + 1 == kTreeMaxLevels);
        for (long long c0 = 0; c0 < n_in; c0 += kTreeGrowChunk) {
            const long long n = n_in - c0 < kTreeGrowChunk ? n_in - c0 : kTreeGrowChunk;
            const int blocks = (int)((n + 255) / 256);
            k_tree_boxes<<<blocks, 256, 0, s>>>(B.lvl_lo[L & 1], B.lvl_hi[L & 1], c0, n, cons, center, vecs);
            NIQ_CUDA(cudaGetLastError());
            const int rc = niq_classify_boxes(model, opts, n, center, vecs, 3, offset, sign, nullptr, cws, G.cws_bytes,
                                              stream);
            if (rc) return rc;
            k_tree_consume<<<blocks, 256, 0, s>>>(sign, c0, n, quit ? 1 : 0, P, ws, B, L);
            NIQ_CUDA(cudaGetLastError());
        }
        if (quit) break;
    }
    return finish_tree(ws, reinterpret_cast<long long*>(counts_out), node_capacity, s);
}

// ==========================================================================================
// Level-set tree without device allocation.
//
// For callers that cannot allocate device memory at the time of the call: hosts whose
// device memory is owned by a pool or arena they cannot grow, plug-ins handed only
// pre-allocated buffers, and latency-critical loops that must not enter the allocator
// (a device allocation can synchronise the device).  The tree's scratch (level counters and two
// ping-pong node buffers) lives in the file-scope array below, which every GPU that
// loads the library holds until the process exits; the model blob, the root box and the
// result arrays come from the caller.
// ==========================================================================================
namespace niq {

// Largest number of nodes one level may hold (each node is 24 bytes).
constexpr long long kStaticTreeNodes = NIQ_STATIC_TREE_NODES;
constexpr size_t kStaticTreeHdr = (sizeof(TreeWs) + 255) & ~size_t(255);
constexpr size_t kStaticTreeBytes = kStaticTreeHdr + 2 * (size_t)kStaticTreeNodes * 24;

static __device__ __align__(256) unsigned char g_static_tree_scratch[kStaticTreeBytes];

static void* g_static_tree_ptr[64] = {nullptr};
static std::mutex g_static_tree_mu;

// Device address of the scratch array on the current device, looked up once per device
// (the first call on it) and kept for the process: after cudaDeviceReset the address is
// stale, so no call may follow a device reset.
static int static_tree_scratch(void** out) {
    int dev = 0;
    NIQ_CUDA(cudaGetDevice(&dev));
    NIQ_REQUIRE(dev >= 0 && dev < 64, NIQ_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_static_tree_mu);
    if (!g_static_tree_ptr[dev]) {
        void* p = nullptr;
        NIQ_CUDA(cudaGetSymbolAddress(&p, g_static_tree_scratch));
        g_static_tree_ptr[dev] = p;
    }
    *out = g_static_tree_ptr[dev];
    return NIQ_OK;
}

// Clears the counters of the scratch header and writes the root node (no host copies).
__global__ void k_tree_static_init(TreeWs* ws, float* lo0, float* hi0, float l0, float l1, float l2, float u0,
                                   float u1, float u2) {
    unsigned int* w = reinterpret_cast<unsigned int*>(ws);
    for (size_t i = threadIdx.x; i < sizeof(TreeWs) / 4; i += blockDim.x) w[i] = 0u;
    __syncthreads();
    if (threadIdx.x == 0) {
        lo0[0] = l0; lo0[1] = l1; lo0[2] = l2;
        hi0[0] = u0; hi0[1] = u1; hi0[2] = u2;
        ws->level_count[0] = 1ull;
    }
}

}  // namespace niq

extern "C" int niq_levelset_tree_static(const void* packed_spec_host, const void* packed_spec_device,
                                        size_t spec_bytes, const niq_bound_opts* opts, const float* lower,
                                        const float* upper, int32_t split_depth, int64_t node_terminate_thresh,
                                        float offset, int32_t flags, float* unknown_lower, float* unknown_upper,
                                        float* interior_lower, float* interior_upper, float* exterior_lower,
                                        float* exterior_upper, int64_t* counts_out, void* stream) {
    using namespace niq;
    NIQ_REQUIRE(packed_spec_host && packed_spec_device && opts && lower && upper && counts_out && unknown_lower &&
                    unknown_upper,
                NIQ_ERR_INVALID_ARG, "null argument");
    NIQ_REQUIRE(spec_bytes >= sizeof(NiqSpecHeader), NIQ_ERR_BAD_SPEC, "spec too short (%zu bytes)", spec_bytes);
    NIQ_REQUIRE(reinterpret_cast<uintptr_t>(packed_spec_device) % 16 == 0, NIQ_ERR_INVALID_ARG,
                "the device copy of the spec must be 16-byte aligned");
    NiqSpecHeader H;
    memcpy(&H, packed_spec_host, sizeof(H));
    int rc = validate_spec(H, spec_bytes);
    if (rc) return rc;
    const int mode = opts->mode;
    NIQ_REQUIRE(mode == NIQ_MODE_AFFINE_FIXED || mode == NIQ_MODE_INTERVAL || mode == NIQ_MODE_SLOPE_INTERVAL,
                NIQ_ERR_UNSUPPORTED, "the tree kernels support the interval, affine_fixed and slope_interval modes");
    NIQ_REQUIRE(split_depth >= 0 || node_terminate_thresh > 0, NIQ_ERR_INVALID_ARG,
                "must specify at least one of node_terminate_thresh or split_depth as a terminating condition");
    NIQ_REQUIRE(split_depth < kTreeMaxLevels, NIQ_ERR_INVALID_ARG, "split_depth %d exceeds %d", split_depth,
                kTreeMaxLevels - 1);
    NIQ_REQUIRE(!(flags & NIQ_TREE_WITH_INTERIOR) || (interior_lower && interior_upper), NIQ_ERR_INVALID_ARG,
                "interior output arrays required by the flags");
    NIQ_REQUIRE(!(flags & NIQ_TREE_WITH_EXTERIOR) || (exterior_lower && exterior_upper), NIQ_ERR_INVALID_ARG,
                "exterior output arrays required by the flags");
    void* scratch = nullptr;
    rc = static_tree_scratch(&scratch);
    if (rc) return rc;
    cudaStream_t s = as_stream(stream);
    // Launch planning (threads per item, shared-memory size, resident weights) uses the
    // host copy while the kernel stages weights by the device copy's header: the two
    // headers must be the same bytes, or the kernel would write past the shared memory
    // it was planned for.  A stack copy of the device header, no allocation.
    {
        NiqSpecHeader Hd;
        NIQ_CUDA(cudaMemcpyAsync(&Hd, packed_spec_device, sizeof(Hd), cudaMemcpyDeviceToHost, s));
        NIQ_CUDA(cudaStreamSynchronize(s));
        NIQ_REQUIRE(memcmp(&Hd, &H, sizeof(H)) == 0, NIQ_ERR_BAD_SPEC,
                    "the device copy of the spec has another header than the host copy");
    }
    char* base = reinterpret_cast<char*>(scratch);
    TreeWs* ws = reinterpret_cast<TreeWs*>(base);
    TreeBufs B;
    const long long cap = kStaticTreeNodes;
    for (int i = 0; i < 2; ++i) {
        B.lvl_lo[i] = reinterpret_cast<float*>(base + kStaticTreeHdr + (size_t)i * cap * 24);
        B.lvl_hi[i] = B.lvl_lo[i] + 3 * cap;
    }
    B.res_lo[0] = unknown_lower;  B.res_hi[0] = unknown_upper;
    B.res_lo[1] = interior_lower; B.res_hi[1] = interior_upper;
    B.res_lo[2] = exterior_lower; B.res_hi[2] = exterior_upper;
    B.cap = cap;
    k_tree_static_init<<<1, 256, 0, s>>>(ws, B.lvl_lo[0], B.lvl_hi[0], lower[0], lower[1], lower[2], upper[0],
                                          upper[1], upper[2]);
    NIQ_CUDA(cudaGetLastError());
    TreeParams P;
    P.n_rounds = split_depth >= 0 ? split_depth + 1 : kTreeMaxLevels;
    P.thresh = node_terminate_thresh > 0 ? node_terminate_thresh : (1ll << 62);
    P.offset = offset;
    P.with_interior = (flags & NIQ_TREE_WITH_INTERIOR) != 0;
    P.with_exterior = (flags & NIQ_TREE_WITH_EXTERIOR) != 0;
    P.mode_interval = mode == NIQ_MODE_INTERVAL;
    P.batch_start = 0;
    P.batch_end = 1ll << 62;
    P.barrier_polls = barrier_polls();
    P.mbar_polls = mbar_polls();
    NiqModelRef M;
    M.hdr = reinterpret_cast<const NiqSpecHeader*>(packed_spec_device);
    M.w = reinterpret_cast<const float*>(reinterpret_cast<const char*>(packed_spec_device) + sizeof(NiqSpecHeader));
    const bool cons = opts->conservative != 0, slope = mode == NIQ_MODE_SLOPE_INTERVAL;
    const int tpi = tpi_for_width(H.max_width);
    auto run = [&](auto kern, int R, int TPIv) -> int {
        const int items = kNT / TPIv;
        const int state = items * R * (TPIv * 8 + 4) + ((items * R + 3) & ~3);
        SmemPlan p = plan_smem(state, H.n_weight_floats, max_layer_floats(H));
        NIQ_REQUIRE(p.resident || p.sw_cap >= 5 * H.max_width, NIQ_ERR_UNSUPPORTED, "shared memory too small");
        int r2 = prepare_kernel(kern, p.bytes);
        if (r2) return r2;
        int per_sm = 0;
        NIQ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kNT, p.bytes));
        NIQ_REQUIRE(per_sm >= 1, NIQ_ERR_UNSUPPORTED, "tree kernel does not fit on an SM");
        if (tune_value(kTuneTreeCtasPerSm) > 0 && per_sm > tune_value(kTuneTreeCtasPerSm))
            per_sm = tune_value(kTuneTreeCtasPerSm);
        const int grid = per_sm * device_info().sm_count;
        int level0 = 0;
        int fixed = p.fixed_floats, swc = p.sw_cap, res = p.resident;
        void* args[] = {&M, &P, &ws, &B, &level0, &fixed, &swc, &res};
        NIQ_CUDA(cudaLaunchCooperativeKernel((const void*)kern, grid, kNT, args, p.bytes, s));
        return NIQ_OK;
    };
#define NIQ_TREE_S(CC, SL) NIQ_DISPATCH_TPI(tpi, { rc = run(k_tree<TPI, CC, SL, true>, SL ? 8 : 5, TPI); })
    if (use_tree_tc(H, opts)) {
        // the same kernel as niq_levelset_tree picks for this model (no allocation either)
        TreeLaunch T{M, &H, P, ws, B, s, true, 0};
        rc = run_tree_tc(T);
    } else if (slope) { if (cons) { NIQ_TREE_S(true, true); } else { NIQ_TREE_S(false, true); } }
    else { if (cons) { NIQ_TREE_S(true, false); } else { NIQ_TREE_S(false, false); } }
#undef NIQ_TREE_S
    if (rc) return rc;
    k_tree_finish<<<1, 1, 0, s>>>(ws, reinterpret_cast<long long*>(counts_out));
    NIQ_CUDA(cudaGetLastError());
    int err = 0;
    NIQ_CUDA(cudaMemcpyAsync(&err, &ws->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    NIQ_CUDA(cudaStreamSynchronize(s));
    NIQ_REQUIRE(err == 0, err,
                err == NIQ_ERR_CAPACITY
                    ? "a level or a result list outgrew the static scratch of %lld nodes (NIQ_STATIC_TREE_NODES)"
                    : "tree kernel error (%lld)",
                err == NIQ_ERR_CAPACITY ? cap : (long long)err);
    return NIQ_OK;
}
