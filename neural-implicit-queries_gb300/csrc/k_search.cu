// k_search.cu -- closest_point (src/kd_tree.py:659-802) and find_any_intersection
// (src/kd_tree.py:402-655).
//
// Node geometry shared by both (src/kd_tree.py:459-464, 695-704): width = max extent,
// split along the first longest axis at the midpoint, 7 samples at
// center + s * {0, +e_i, -e_i} with s = eps/sqrt(3) (intersection) or s = the node's
// extents (closest point).  A node is small when width < eps/sqrt(3).
#include "niq_host.cuh"

namespace niq {

// Builds the bound rows (affine R=5 or slope R=8) of the box [lo, hi] for the owner
// threads g < 4 of an item; shared by the search kernels.
template <int R, int LD, bool C, bool SLOPE>
__device__ __forceinline__ void box_rows(float* xs, int g, bool valid, const float* lo, const float* hi, int interval,
                                         float gam0) {
    if (g >= 4) return;
    const int k = g;
    for (int r = 0; r < R; ++r) xs[r * LD + k] = 0.f;
    if (!valid || k == 3) return;
    const float c = __fmul_rn(0.5f, __fadd_rn(lo[k], hi[k]));
    float h = __fsub_rn(hi[k], c);
    if (C) h = fmaxf(__fsub_ru(hi[k], c), __fsub_ru(c, lo[k]));
    xs[k] = c;
    if (SLOPE) {
        xs[(1 + k) * LD + k] = h;
        xs[(5 + k) * LD + k] = C ? __fmul_ru(gam0, h) : 0.f;
        xs[4 * LD + k] = C ? __fmul_ru(gam0, fabsf(c)) : 0.f;
    } else if (interval) {
        xs[(R - 1) * LD + k] = C ? __fmaf_ru(gam0, fabsf(c), h) : h;
    } else {
        xs[(1 + k) * LD + k] = h;
        xs[(R - 1) * LD + k] = C ? __fmul_ru(gam0, __fadd_ru(fabsf(c), h)) : 0.f;
    }
}

// The 7 sample points of a node into the point rows 0..6 (row 7 zero).
template <int LD>
__device__ __forceinline__ void sample_rows(float* xs, int g, int TPI, bool valid, const float* c, const float* s) {
    for (int r = g; r < 8; r += TPI) {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (valid && r < 7) {
            float p[3] = {c[0], c[1], c[2]};
            if (r >= 1) {
                const int ax = (r - 1) % 3;
                const float sg = r <= 3 ? 1.f : -1.f;
                p[ax] = __fadd_rn(c[ax], __fmul_rn(s[ax], sg));
            }
            v.x = p[0]; v.y = p[1]; v.z = p[2];
        }
        *reinterpret_cast<float4*>(xs + r * LD) = v;
    }
}

__device__ __forceinline__ int first_longest(const float* lo, const float* hi) {
    const float e0 = __fsub_rn(hi[0], lo[0]), e1 = __fsub_rn(hi[1], lo[1]), e2 = __fsub_rn(hi[2], lo[2]);
    int d = 0;
    float em = e0;
    if (e1 > em) { d = 1; em = e1; }
    if (e2 > em) d = 2;
    return d;
}

__device__ __forceinline__ bool all_same_sign7(const float* v) {
    bool neg = true, pos = true;
    for (int i = 0; i < 7; ++i) { neg &= v[i] < 0.f; pos &= v[i] > 0.f; }
    return neg || pos;  // src/utils.py:146-150
}

// float distance as an order-preserving integer (distances are >= 0 or +inf)
__device__ __forceinline__ void atomic_min_dist(float* addr, float v) {
    atomicMin(reinterpret_cast<int*>(addr), __float_as_int(v));
}

__device__ __forceinline__ float norm3(float a, float b, float c) {
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b)), __fmul_rn(c, c)));
}

// Distance from q to the box [lo, hi], rounded down (a lower bound).
__device__ __forceinline__ float box_dist(const float* q, const float* lo, const float* hi) {
    float s = 0.f;
    for (int k = 0; k < 3; ++k) {
        const float d = fmaxf(fmaxf(__fsub_rd(lo[k], q[k]), __fsub_rd(q[k], hi[k])), 0.f);
        s = __fmaf_rd(d, d, s);
    }
    return __fsqrt_rd(s);
}

// ======================================================================== closest point
struct CpArgs {
    const float* q;          // (Q,3)
    float* min_dist;         // (Q)
    float* min_loc;          // (Q,3)
    float eps_w;             // eps / sqrt(3)
    int interval;
    long long node_budget;   // persistent form: nodes one query may visit
    float prune_tol;         // persistent form: prune when box distance >= best - prune_tol
};

// ---- reference schedule: process one popped batch [pop, top) of the global stack.
// EXT: the batch's box signs come from ext_type (the growing-term engine classified them
// beforehand); otherwise the tile engine bounds each box here.
template <int TPI, bool C, bool SLOPE, bool EXT>
__global__ void __launch_bounds__(kNT) k_cp_batch(NiqModelRef M, CpArgs a, const float* __restrict__ st_lo,
                                                  const float* __restrict__ st_hi, const int* __restrict__ st_id,
                                                  long long pop, long long n, float* tmp_lo, float* tmp_hi, int* tmp_id,
                                                  float* tmp_d, int* tmp_need, int fixed_floats, int sw_cap,
                                                  int resident, const int* __restrict__ ext_type) {
    using CB = typename std::conditional<SLOPE, TileCfg<8, 4, TPI, kNT>, TileCfg<5, 1, TPI, kNT>>::type;
    using CP = TileCfg<8, 0, TPI, kNT>;
    constexpr int ITEMS = CP::ITEMS;
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    float* st = smem;                       // sized for R = 8
    float* ob = st + CP::STATE_FLOATS;
    float* sW = smem + fixed_floats;
    __shared__ NiqSpecHeader H;
    __shared__ float s_lo[ITEMS][3], s_hi[ITEMS][3];
    __shared__ float s_lohi[ITEMS][2];
    load_header(H, M.hdr);
    __syncthreads();
    if (resident) stage_floats(sW, M.w, H.n_weight_floats);
    const int item = threadIdx.x / TPI, g = threadIdx.x % TPI;
    const float gam0 = C ? H.layers[0].gamma : 0.f;
    const RowPlan pb{SLOPE ? ROWS_SLOPE : ROWS_AFFINE, a.interval ? 0 : 3, 0};
    const RowPlan pp{ROWS_POINTS, 0, 8};
    for (long long t0 = (long long)blockIdx.x * ITEMS; t0 < n; t0 += (long long)gridDim.x * ITEMS) {
        const long long e = t0 + item;
        const bool valid = e < n;
        if (g < 3 && valid) {
            s_lo[item][g] = st_lo[3 * (pop + e) + g];
            s_hi[item][g] = st_hi[3 * (pop + e) + g];
        }
        __syncthreads();
        if (!EXT) {
            box_rows<CB::R, CB::LD, C, SLOPE>(st + item * CB::R * CB::LD, g, valid, s_lo[item], s_hi[item], a.interval,
                                              gam0);
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
        }
        {
            float c[3], s[3];
            for (int k = 0; k < 3; ++k) {
                c[k] = __fmul_rn(0.5f, __fadd_rn(s_lo[item][k], s_hi[item][k]));
                s[k] = __fsub_rn(s_hi[item][k], s_lo[item][k]);
            }
            sample_rows<CP::LD>(st + item * CP::R * CP::LD, g, TPI, valid, c, s);
        }
        __syncthreads();
        tile_forward<CP, false>(H, M.w, sW, sw_cap, resident, pp, st, ob);
        if (g == 0 && valid) {
            const float* lo = s_lo[item];
            const float* hi = s_hi[item];
            const int id = st_id[pop + e];
            const int type = EXT ? ext_type[e] : sign_of_bounds(s_lohi[item][0], s_lohi[item][1], 0.f);
            const bool outside = type != NIQ_SIGN_UNKNOWN;
            float c[3], w[3];
            for (int k = 0; k < 3; ++k) { c[k] = __fmul_rn(0.5f, __fadd_rn(lo[k], hi[k])); w[k] = __fsub_rn(hi[k], lo[k]); }
            const float width = fmaxf(fmaxf(w[0], w[1]), w[2]);
            const float diag = norm3(w[0], w[1], w[2]);
            const float* q = a.q + 3 * id;
            const float cd = norm3(__fsub_rn(q[0], c[0]), __fsub_rn(q[1], c[1]), __fsub_rn(q[2], c[2]));
            const bool spans = !all_same_sign7(ob + item * 8);
            const float this_d = spans ? __fadd_rn(cd, diag) : INFINITY;
            const float qmd = a.min_dist[id];   // read before this batch's updates
            const bool need = !outside && !(width < a.eps_w) && (cd < qmd);
            for (int k = 0; k < 3; ++k) { tmp_lo[3 * e + k] = lo[k]; tmp_hi[3 * e + k] = hi[k]; }
            tmp_id[e] = id;
            tmp_d[e] = this_d;
            tmp_need[e] = need;
        }
        __syncthreads();
    }
}

// ---- reference schedule: scatter-min, location update, stable push of the children
__global__ void __launch_bounds__(1024) k_cp_finish(CpArgs a, long long pop, long long n, const float* tmp_lo,
                                                    const float* tmp_hi, const int* tmp_id, const float* tmp_d,
                                                    const int* tmp_need, float* st_lo, float* st_hi, int* st_id,
                                                    long long cap, long long* top_out, int* err) {
    __shared__ int s_scan[1024];
    __shared__ long long s_carry;
    for (long long e = threadIdx.x; e < n; e += blockDim.x) atomic_min_dist(&a.min_dist[tmp_id[e]], tmp_d[e]);
    __syncthreads();
    __threadfence_block();
    // src/kd_tree.py:726-729: every entry whose distance equals the new minimum writes its center
    for (long long e = threadIdx.x; e < n; e += blockDim.x) {
        const int id = tmp_id[e];
        if (tmp_d[e] == a.min_dist[id])
            for (int k = 0; k < 3; ++k) a.min_loc[3 * id + k] = __fmul_rn(0.5f, __fadd_rn(tmp_lo[3 * e + k], tmp_hi[3 * e + k]));
    }
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    // stable compaction: children A_i, B_i of the i-th subdivided entry land at pop + 2i, +1
    for (long long base = 0; base < n; base += blockDim.x) {
        const long long e = base + threadIdx.x;
        const int f = (e < n) ? tmp_need[e] : 0;
        s_scan[threadIdx.x] = f;
        __syncthreads();
        for (int off = 1; off < (int)blockDim.x; off <<= 1) {
            const int y = threadIdx.x >= (unsigned)off ? s_scan[threadIdx.x - off] : 0;
            __syncthreads();
            s_scan[threadIdx.x] += y;
            __syncthreads();
        }
        const long long rank = s_carry + s_scan[threadIdx.x] - f;
        if (f) {
            const long long dst = pop + 2 * rank;
            if (dst + 1 < cap) {
                float lo[3], hi[3];
                for (int k = 0; k < 3; ++k) { lo[k] = tmp_lo[3 * e + k]; hi[k] = tmp_hi[3 * e + k]; }
                const int d = first_longest(lo, hi);
                const float mid = __fmul_rn(0.5f, __fadd_rn(lo[d], hi[d]));
                for (int k = 0; k < 3; ++k) {
                    st_lo[3 * dst + k] = lo[k];
                    st_hi[3 * dst + k] = k == d ? mid : hi[k];
                    st_lo[3 * (dst + 1) + k] = k == d ? mid : lo[k];
                    st_hi[3 * (dst + 1) + k] = hi[k];
                }
                st_id[dst] = tmp_id[e];
                st_id[dst + 1] = tmp_id[e];
            } else {
                niq_flag_error(err, NIQ_ERR_CAPACITY);
            }
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_carry += s_scan[threadIdx.x];
        __syncthreads();
    }
    if (threadIdx.x == 0) *top_out = pop + 2 * s_carry;
}

__global__ void k_cp_init(const float* lower_upper, float* st_lo, float* st_hi, int* st_id, float* min_dist,
                          float* min_loc, long long Q) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < Q; i += (long long)gridDim.x * blockDim.x) {
        for (int k = 0; k < 3; ++k) {
            st_lo[3 * i + k] = lower_upper[k];
            st_hi[3 * i + k] = lower_upper[3 + k];
            min_loc[3 * i + k] = -777.f;
        }
        st_id[i] = (int)i;
        min_dist[i] = INFINITY;
    }
}

// ---- persistent form: one depth-first stack per query slot
constexpr int kCpStack = 96;

template <int TPI, bool C, bool SLOPE>
__global__ void __launch_bounds__(kNT) k_cp_persistent(NiqModelRef M, CpArgs a, long long Q, const float* root,
                                                       float* stacks, unsigned long long* next_query, int* err,
                                                       int fixed_floats, int sw_cap, int resident) {
    using CB = typename std::conditional<SLOPE, TileCfg<8, 4, TPI, kNT>, TileCfg<5, 1, TPI, kNT>>::type;
    using CP = TileCfg<8, 0, TPI, kNT>;
    constexpr int ITEMS = CP::ITEMS;
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    float* st = smem;
    float* ob = st + CP::STATE_FLOATS;
    float* sW = smem + fixed_floats;
    __shared__ NiqSpecHeader H;
    __shared__ float s_lo[ITEMS][3], s_hi[ITEMS][3], s_q[ITEMS][3], s_best[ITEMS], s_loc[ITEMS][3];
    __shared__ float s_lohi[ITEMS][2];
    __shared__ int s_top[ITEMS], s_act[ITEMS];
    __shared__ long long s_nodes[ITEMS];
    __shared__ long long s_qid[ITEMS];
    load_header(H, M.hdr);
    __syncthreads();
    if (resident) stage_floats(sW, M.w, H.n_weight_floats);
    const int item = threadIdx.x / TPI, g = threadIdx.x % TPI;
    const float gam0 = C ? H.layers[0].gamma : 0.f;
    const RowPlan pb{SLOPE ? ROWS_SLOPE : ROWS_AFFINE, a.interval ? 0 : 3, 0};
    const RowPlan pp{ROWS_POINTS, 0, 8};
    float* my_stack = stacks + ((long long)blockIdx.x * ITEMS + item) * kCpStack * 6;

    auto claim = [&]() {
        const unsigned long long k = atomicAdd(next_query, 1ull);
        if ((long long)k < Q) {
            s_qid[item] = (long long)k;
            for (int j = 0; j < 3; ++j) { s_q[item][j] = a.q[3 * k + j]; my_stack[j] = root[j]; my_stack[3 + j] = root[3 + j]; s_loc[item][j] = -777.f; }
            s_top[item] = 1;
            s_best[item] = INFINITY;
            s_nodes[item] = 0;
        } else {
            s_qid[item] = -1;
            s_top[item] = 0;
        }
    };
    if (g == 0) claim();
    __syncthreads();
    while (true) {
        // pop one node per live slot; finished slots publish and refill
        if (g == 0) {
            while (s_qid[item] >= 0 && s_top[item] == 0) {
                const long long id = s_qid[item];
                a.min_dist[id] = s_best[item];
                for (int j = 0; j < 3; ++j) a.min_loc[3 * id + j] = s_loc[item][j];
                claim();
            }
            // node budget per query: past it the traversal stops with its best so far (a
            // valid upper bound) and the call reports NIQ_ERR_TIMEOUT
            if (s_qid[item] >= 0 && s_top[item] > 0 && ++s_nodes[item] > a.node_budget) {
                niq_flag_error(err, NIQ_ERR_TIMEOUT);
                s_top[item] = 0;
                const long long id = s_qid[item];
                a.min_dist[id] = s_best[item];
                for (int j = 0; j < 3; ++j) a.min_loc[3 * id + j] = s_loc[item][j];
                claim();
                if (s_qid[item] >= 0) s_nodes[item] = 1;
            }
            s_act[item] = s_qid[item] >= 0;
            if (s_act[item]) {
                const int t = --s_top[item];
                for (int j = 0; j < 3; ++j) { s_lo[item][j] = my_stack[6 * t + j]; s_hi[item][j] = my_stack[6 * t + 3 + j]; }
            }
        }
        if (!__syncthreads_or(g == 0 && s_act[item])) break;
        const bool valid = s_act[item];
        box_rows<CB::R, CB::LD, C, SLOPE>(st + item * CB::R * CB::LD, g, valid, s_lo[item], s_hi[item], a.interval, gam0);
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
        {
            float c[3], s[3];
            for (int k = 0; k < 3; ++k) {
                c[k] = __fmul_rn(0.5f, __fadd_rn(s_lo[item][k], s_hi[item][k]));
                s[k] = __fsub_rn(s_hi[item][k], s_lo[item][k]);
            }
            sample_rows<CP::LD>(st + item * CP::R * CP::LD, g, TPI, valid, c, s);
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
            const float diag = norm3(w[0], w[1], w[2]);
            const float* q = s_q[item];
            const float cd = norm3(__fsub_rn(q[0], c[0]), __fsub_rn(q[1], c[1]), __fsub_rn(q[2], c[2]));
            if (!all_same_sign7(ob + item * 8)) {
                const float d = __fadd_rn(cd, diag);
                if (d < s_best[item]) {
                    s_best[item] = d;
                    for (int k = 0; k < 3; ++k) s_loc[item][k] = c[k];
                }
            }
            // prune with the distance from the query to the box, a true lower bound on every
            // candidate inside it (the reference computes it, src/kd_tree.py:699, but prunes
            // with the center distance, which under depth-first order would drop subtrees
            // that hold the closest candidate), less a tolerance of eps: candidates carry a
            // leaf-diagonal (<= eps) slack anyway, and proving that no node of the
            // surface cap within eps of the best is better would visit the whole cap
            if (type == NIQ_SIGN_UNKNOWN && !(width < a.eps_w) && box_dist(q, lo, hi) < s_best[item] - a.prune_tol) {
                const int t = s_top[item];
                if (t + 2 <= kCpStack) {
                    const int d = first_longest(lo, hi);
                    const float mid = __fmul_rn(0.5f, __fadd_rn(lo[d], hi[d]));
                    float alo[3] = {lo[0], lo[1], lo[2]}, ahi[3] = {hi[0], hi[1], hi[2]};
                    float blo[3] = {lo[0], lo[1], lo[2]}, bhi[3] = {hi[0], hi[1], hi[2]};
                    ahi[d] = mid;
                    blo[d] = mid;
                    // the child nearer to the query is popped first
                    const bool a_near = fabsf(q[d] - 0.5f * (lo[d] + mid)) <= fabsf(q[d] - 0.5f * (mid + hi[d]));
                    const float* first_lo = a_near ? blo : alo;
                    const float* first_hi = a_near ? bhi : ahi;
                    const float* second_lo = a_near ? alo : blo;
                    const float* second_hi = a_near ? ahi : bhi;
                    for (int k = 0; k < 3; ++k) {
                        my_stack[6 * t + k] = first_lo[k];
                        my_stack[6 * t + 3 + k] = first_hi[k];
                        my_stack[6 * (t + 1) + k] = second_lo[k];
                        my_stack[6 * (t + 1) + 3 + k] = second_hi[k];
                    }
                    s_top[item] = t + 2;
                } else {
                    niq_flag_error(err, NIQ_ERR_CAPACITY);
                }
            }
        }
        __syncthreads();
    }
}

// ======================================================================== intersection
struct IsWs {
    unsigned long long level_count[129];
    unsigned long long grab[129];
    int found_at[129];      // set during level L when a node of L holds an intersection
    unsigned long long processed;
    unsigned int barrier;
    int found;
    int err;
    int depth;
    float loc[3];
};

constexpr int kIsMaxLevels = 128;

template <int TPI, bool C, bool SLOPE>
__global__ void __launch_bounds__(kNT) k_intersect(NiqModelRef MA, NiqModelRef MB, int interval, float eps_w,
                                                   IsWs* ws, float* lv_lo0, float* lv_hi0, float* lv_lo1, float* lv_hi1,
                                                   long long cap, int woffB, int fixed_floats, int sw_cap,
                                                   int resident, unsigned int polls) {
    using CB = typename std::conditional<SLOPE, TileCfg<8, 4, TPI, kNT>, TileCfg<5, 1, TPI, kNT>>::type;
    using CP = TileCfg<8, 0, TPI, kNT>;
    constexpr int ITEMS = CP::ITEMS;
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    float* st = smem;
    float* ob = st + CP::STATE_FLOATS;
    float* sW = smem + fixed_floats;
    __shared__ NiqSpecHeader H;
    __shared__ float s_lo[ITEMS][3], s_hi[ITEMS][3];
    __shared__ int s_type[2][ITEMS];
    __shared__ float s_val[2][ITEMS][8];
    __shared__ long long s_base;
    __shared__ unsigned long long s_proc;
    const int item = threadIdx.x / TPI, g = threadIdx.x % TPI;
    if (resident) {
        load_header(H, MA.hdr);
        __syncthreads();
        stage_floats(sW, MA.w, H.n_weight_floats);
        __syncthreads();
        load_header(H, MB.hdr);
        __syncthreads();
        stage_floats(sW + woffB, MB.w, H.n_weight_floats);
        __syncthreads();
    }
    if (threadIdx.x == 0) s_proc = 0;
    const RowPlan pb{SLOPE ? ROWS_SLOPE : ROWS_AFFINE, interval ? 0 : 3, 0};
    const RowPlan pp{ROWS_POINTS, 0, 8};
    unsigned int epoch = 0;
    for (int L = 0; L < kIsMaxLevels; ++L) {
        const long long n_in = (long long)*((volatile unsigned long long*)&ws->level_count[L]);
        // stable after the barrier: written only while the previous level ran
        if (n_in == 0 || n_in > cap || (L > 0 && *((volatile int*)&ws->found_at[L - 1]))) break;
        const float* in_lo = (L & 1) ? lv_lo1 : lv_lo0;
        const float* in_hi = (L & 1) ? lv_hi1 : lv_hi0;
        float* out_lo = (L & 1) ? lv_lo0 : lv_lo1;
        float* out_hi = (L & 1) ? lv_hi0 : lv_hi1;
        while (true) {
            __syncthreads();
            if (threadIdx.x == 0) s_base = (long long)atomicAdd(&ws->grab[L], (unsigned long long)ITEMS);
            __syncthreads();
            const long long base = s_base;
            if (base >= n_in) break;
            const long long nid = base + item;
            const bool valid = nid < n_in;
            if (g < 3 && valid) { s_lo[item][g] = in_lo[3 * nid + g]; s_hi[item][g] = in_hi[3 * nid + g]; }
            __syncthreads();
            for (int f = 0; f < 2; ++f) {
                const NiqModelRef& M = f ? MB : MA;
                load_header(H, M.hdr);
                __syncthreads();
                const float gam0 = C ? H.layers[0].gamma : 0.f;
                float* sWf = resident ? sW + (f ? woffB : 0) : sW;
                box_rows<CB::R, CB::LD, C, SLOPE>(st + item * CB::R * CB::LD, g, valid, s_lo[item], s_hi[item], interval, gam0);
                __syncthreads();
                tile_forward<CB, C>(H, M.w, sWf, sw_cap, resident, pb, st, ob);
                if (g == 0 && valid) {
                    float lo, hi;
                    if (SLOPE) slope_out_bounds<C>(ob + item * CB::R, pb.v, lo, hi);
                    else affine_out_bounds<CB::R, C>(ob + item * CB::R, pb.v, lo, hi);
                    s_type[f][item] = sign_of_bounds(lo, hi, 0.f);
                }
                __syncthreads();
                {
                    float c[3], s[3];
                    for (int k = 0; k < 3; ++k) { c[k] = __fmul_rn(0.5f, __fadd_rn(s_lo[item][k], s_hi[item][k])); s[k] = eps_w; }
                    sample_rows<CP::LD>(st + item * CP::R * CP::LD, g, TPI, valid, c, s);
                }
                __syncthreads();
                tile_forward<CP, false>(H, M.w, sWf, sw_cap, resident, pp, st, ob);
                if (g == 0 && valid)
                    for (int i = 0; i < 8; ++i) s_val[f][item][i] = ob[item * 8 + i];
                __syncthreads();
            }
            // ---- decisions (src/kd_tree.py:449-518)
            bool need = false;
            if (g == 0 && valid) {
                const float* lo = s_lo[item];
                const float* hi = s_hi[item];
                float c[3], w[3];
                for (int k = 0; k < 3; ++k) { c[k] = __fmul_rn(0.5f, __fadd_rn(lo[k], hi[k])); w[k] = __fsub_rn(hi[k], lo[k]); }
                const bool small = fmaxf(fmaxf(w[0], w[1]), w[2]) < eps_w;
                const float* vA = s_val[0][item];
                const float* vB = s_val[1][item];
                const bool nearA = small && !all_same_sign7(vA);
                const bool nearB = small && !all_same_sign7(vB);
                int iA = -1, iB = -1, iAB = -1;
                for (int i = 0; i < 7; ++i) {
                    if (iA < 0 && vA[i] < 0.f) iA = i;
                    if (iB < 0 && vB[i] < 0.f) iB = i;
                    if (iAB < 0 && vA[i] < 0.f && vB[i] < 0.f) iAB = i;
                }
                auto sample = [&](int i, float* p) {
                    for (int k = 0; k < 3; ++k) p[k] = c[k];
                    if (i >= 1) { const int ax = (i - 1) % 3; p[ax] = __fadd_rn(c[ax], i <= 3 ? eps_w : -eps_w); }
                };
                bool found = false;
                float loc[3] = {-777.f, -777.f, -777.f};
                if (small && iA >= 0 && iB >= 0) {
                    float pa[3], pb_[3];
                    sample(iA, pa);
                    sample(iB, pb_);
                    for (int k = 0; k < 3; ++k) loc[k] = __fmul_rn(0.5f, __fadd_rn(pa[k], pb_[k]));
                    found = true;
                }
                if (iAB >= 0) { sample(iAB, loc); found = true; }
                if (found) {
                    atomicExch(&ws->found_at[L], 1);
                    if (atomicCAS(&ws->found, 0, 1) == 0) {
                        ws->loc[0] = loc[0]; ws->loc[1] = loc[1]; ws->loc[2] = loc[2];
                        ws->depth = L;
                    }
                }
                const int tA = s_type[0][item], tB = s_type[1][item];
                const bool inA = tA == NIQ_SIGN_NEGATIVE || (tA == NIQ_SIGN_UNKNOWN && !nearA);
                const bool inB = tB == NIQ_SIGN_NEGATIVE || (tB == NIQ_SIGN_UNKNOWN && !nearB);
                need = inA && inB && !found;
                atomicAdd(&s_proc, 1ull);
            }
            const long long pc = niq_warp_reserve(&ws->level_count[L + 1], need, 2);
            if (need) {
                if (pc + 1 < cap) {
                    const float* lo = s_lo[item];
                    const float* hi = s_hi[item];
                    const int d = first_longest(lo, hi);
                    const float mid = __fmul_rn(0.5f, __fadd_rn(lo[d], hi[d]));
                    for (int k = 0; k < 3; ++k) {
                        out_lo[3 * pc + k] = lo[k];
                        out_hi[3 * pc + k] = k == d ? mid : hi[k];
                        out_lo[3 * (pc + 1) + k] = k == d ? mid : lo[k];
                        out_hi[3 * (pc + 1) + k] = hi[k];
                    }
                } else {
                    niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
                }
            }
        }
        if (!niq_grid_barrier(&ws->barrier, gridDim.x, epoch, &ws->err, polls)) break;
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_proc) atomicAdd(&ws->processed, s_proc);
}

__global__ void k_is_finish(IsWs* ws, int* found_out, float* loc_out, long long* counts_out) {
    found_out[0] = ws->found;
    for (int k = 0; k < 3; ++k) loc_out[k] = ws->found ? ws->loc[k] : -777.f;
    counts_out[0] = (long long)ws->processed;
    int depth = 0;
    for (int L = 0; L < kIsMaxLevels; ++L)
        if (ws->level_count[L]) depth = L;
    counts_out[1] = ws->found ? ws->depth : depth;
}

// ---- plain intersection for every mode: one level per host iteration, bounds from
// niq_classify_boxes (the growing-term engine for affine_all/truncate/append)
__global__ void k_is_prepare(long long n, const float* lo, const float* hi, float eps_w, float* center, float* vecs,
                             float* samples) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float c[3];
        for (int k = 0; k < 3; ++k) {
            c[k] = __fmul_rn(0.5f, __fadd_rn(lo[3 * i + k], hi[3 * i + k]));
            center[3 * i + k] = c[k];
            for (int j = 0; j < 3; ++j) vecs[9 * i + 3 * j + k] = j == k ? __fsub_rn(hi[3 * i + k], c[k]) : 0.f;
        }
        for (int r = 0; r < 7; ++r)
            for (int k = 0; k < 3; ++k) {
                float p = c[k];
                if (r >= 1 && (r - 1) % 3 == k) p = __fadd_rn(c[k], r <= 3 ? eps_w : -eps_w);
                samples[21 * i + 3 * r + k] = p;
            }
    }
}

__global__ void k_is_decide(long long n, int level, const float* lo, const float* hi, float eps_w, const int* tA,
                            const int* tB, const float* vA7, const float* vB7, const float* samples, IsWs* ws,
                            float* out_lo, float* out_hi, long long cap) {
    for (long long i0 = blockIdx.x * (long long)blockDim.x; i0 < n; i0 += (long long)gridDim.x * blockDim.x) {
        const long long i = i0 + threadIdx.x;
        bool need = false;
        if (i < n) {
            float w[3];
            for (int k = 0; k < 3; ++k) w[k] = __fsub_rn(hi[3 * i + k], lo[3 * i + k]);
            const bool small = fmaxf(fmaxf(w[0], w[1]), w[2]) < eps_w;
            const float* vA = vA7 + 7 * i;
            const float* vB = vB7 + 7 * i;
            const bool nearA = small && !all_same_sign7(vA), nearB = small && !all_same_sign7(vB);
            int iA = -1, iB = -1, iAB = -1;
            for (int s = 0; s < 7; ++s) {
                if (iA < 0 && vA[s] < 0.f) iA = s;
                if (iB < 0 && vB[s] < 0.f) iB = s;
                if (iAB < 0 && vA[s] < 0.f && vB[s] < 0.f) iAB = s;
            }
            bool found = false;
            float loc[3];
            if (small && iA >= 0 && iB >= 0) {
                for (int k = 0; k < 3; ++k)
                    loc[k] = __fmul_rn(0.5f, __fadd_rn(samples[21 * i + 3 * iA + k], samples[21 * i + 3 * iB + k]));
                found = true;
            }
            if (iAB >= 0) { for (int k = 0; k < 3; ++k) loc[k] = samples[21 * i + 3 * iAB + k]; found = true; }
            if (found && atomicCAS(&ws->found, 0, 1) == 0) {
                ws->loc[0] = loc[0]; ws->loc[1] = loc[1]; ws->loc[2] = loc[2];
                ws->depth = level;
            }
            const bool inA = tA[i] == NIQ_SIGN_NEGATIVE || (tA[i] == NIQ_SIGN_UNKNOWN && !nearA);
            const bool inB = tB[i] == NIQ_SIGN_NEGATIVE || (tB[i] == NIQ_SIGN_UNKNOWN && !nearB);
            need = inA && inB && !found;
        }
        const long long pc = niq_warp_reserve(&ws->level_count[level + 1], need, 2);
        if (need) {
            if (pc + 1 < cap) {
                const float* l = lo + 3 * i;
                const float* h = hi + 3 * i;
                const int d = first_longest(l, h);
                const float mid = __fmul_rn(0.5f, __fadd_rn(l[d], h[d]));
                for (int k = 0; k < 3; ++k) {
                    out_lo[3 * pc + k] = l[k];
                    out_hi[3 * pc + k] = k == d ? mid : h[k];
                    out_lo[3 * (pc + 1) + k] = k == d ? mid : l[k];
                    out_hi[3 * (pc + 1) + k] = h[k];
                }
            } else {
                niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
            }
        }
    }
    if (threadIdx.x == 0 && blockIdx.x == 0) atomicAdd(&ws->processed, (unsigned long long)n);
}

}  // namespace niq

#include "wide_engine.cuh"

using namespace niq;

namespace {

size_t al256(size_t x) { return (x + 255) & ~size_t(255); }
char* base256(void* p) { return reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255)); }

bool fixed_mode(int mode) {
    return mode == NIQ_MODE_AFFINE_FIXED || mode == NIQ_MODE_INTERVAL || mode == NIQ_MODE_SLOPE_INTERVAL;
}

struct CpLayout { size_t hdr, st_lo, st_hi, st_id, t_lo, t_hi, t_id, t_d, t_need, root, total; };

CpLayout cp_layout(long long Q, int B, long long cap) {
    CpLayout L;
    L.hdr = 0;
    L.st_lo = al256(64);
    L.st_hi = L.st_lo + al256(12 * cap);
    L.st_id = L.st_hi + al256(12 * cap);
    L.t_lo = L.st_id + al256(4 * cap);
    L.t_hi = L.t_lo + al256(12 * (size_t)B);
    L.t_id = L.t_hi + al256(12 * (size_t)B);
    L.t_d = L.t_id + al256(4 * (size_t)B);
    L.t_need = L.t_d + al256(4 * (size_t)B);
    L.root = L.t_need + al256(4 * (size_t)B);
    L.total = L.root + 256 + 256;
    (void)Q;
    return L;
}

size_t cp_persistent_bytes(long long Q) {
    (void)Q;
    const size_t slots = (size_t)device_info().sm_count * 8 * 64;
    return al256(64) + al256(24) + al256(slots * kCpStack * 24) + 256;
}

template <class K>
int cp_plan(K kern, const niq_model* m, int R, int TPIv, SmemPlan& p) {
    const int items = kNT / TPIv;
    const int state = items * R * (TPIv * 8 + 4) + ((items * R + 3) & ~3);
    p = plan_smem(state, m->hdr.n_weight_floats, max_layer_floats(m->hdr), smem_budget(kern, kNT));
    NIQ_REQUIRE(p.resident || p.sw_cap >= 5 * m->hdr.max_width, NIQ_ERR_UNSUPPORTED, "shared memory too small");
    return prepare_kernel(kern, p.bytes);
}

// Boxes [pop, pop + n) of the stack as center + diagonal vectors (src/implicit_function.py:33-37)
// for the growing-term engine.
__global__ void k_cp_boxes(const float* st_lo, const float* st_hi, long long pop, long long n, int cons, float* center,
                           float* vecs) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = 0; k < 3; ++k) {
        const float l = st_lo[3 * (pop + i) + k], h = st_hi[3 * (pop + i) + k];
        const float c = __fmul_rn(0.5f, __fadd_rn(l, h));
        const float half = cons ? fmaxf(__fsub_ru(h, c), __fsub_ru(c, l)) : __fsub_rn(h, c);
        center[3 * i + k] = c;
        for (int j = 0; j < 3; ++j) vecs[9 * i + 3 * k + j] = j == k ? half : 0.f;
    }
}

// Scratch of the growing-term modes after the reference schedule's layout.
struct CpGrowLayout {
    size_t center, vecs, type, cws, cws_bytes, total;
};

CpGrowLayout cp_grow_layout(const niq_model* m, const niq_bound_opts* opts, size_t base, long long B) {
    CpGrowLayout G;
    size_t off = al256(base);
    G.center = off; off += al256((size_t)B * 12);
    G.vecs = off; off += al256((size_t)B * 36);
    G.type = off; off += al256((size_t)B * 4);
    G.cws = off;
    G.cws_bytes = niq_classify_workspace_size(m, opts, B, 3);
    off += al256(G.cws_bytes);
    G.total = off + 256;
    return G;
}

}  // namespace

extern "C" {

size_t niq_closest_point_workspace_size(int64_t n_queries, int32_t batch_process_size, int64_t stack_capacity) {
    return cp_layout(n_queries, batch_process_size, stack_capacity).total;
}

size_t niq_closest_point_growing_workspace_size(const niq_model* model, const niq_bound_opts* opts, int64_t n_queries,
                                                int32_t batch_process_size, int64_t stack_capacity) {
    if (!model || !opts || batch_process_size < 1) return 0;
    return cp_grow_layout(model, opts, cp_layout(n_queries, batch_process_size, stack_capacity).total,
                          batch_process_size).total;
}

int niq_closest_point(const niq_model* model, const niq_bound_opts* opts, const float* lower, const float* upper,
                      int64_t n_queries, const float* query_points, float eps, int32_t batch_process_size,
                      int64_t stack_capacity, float* min_dist_out, float* min_loc_out, void* workspace,
                      size_t workspace_bytes, void* stream) {
    NIQ_REQUIRE(model && opts && lower && upper, NIQ_ERR_INVALID_ARG, "null argument");
    NIQ_REQUIRE(n_queries >= 0 && n_queries < (1ll << 31) && batch_process_size >= 1, NIQ_ERR_INVALID_ARG, "bad sizes");
    NIQ_REQUIRE(stack_capacity >= n_queries + 2 * (long long)batch_process_size, NIQ_ERR_INVALID_ARG,
                "stack_capacity must be >= n_queries + 2 * batch_process_size");
    const CpLayout CL = cp_layout(n_queries, batch_process_size, stack_capacity);
    const bool growing = !fixed_mode(opts->mode);
    const CpGrowLayout GL = cp_grow_layout(model, opts, CL.total, batch_process_size);
    const size_t need = growing ? GL.total : CL.total;
    NIQ_REQUIRE(workspace && workspace_bytes >= need, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed", need);
    if (n_queries == 0) return NIQ_OK;
    NIQ_REQUIRE(query_points && min_dist_out && min_loc_out, NIQ_ERR_INVALID_ARG, "null array");
    cudaStream_t s = as_stream(stream);
    char* b = base256(workspace);
    long long* top_d = reinterpret_cast<long long*>(b + CL.hdr);
    int* err = reinterpret_cast<int*>(b + CL.hdr + 8);
    float* st_lo = reinterpret_cast<float*>(b + CL.st_lo);
    float* st_hi = reinterpret_cast<float*>(b + CL.st_hi);
    int* st_id = reinterpret_cast<int*>(b + CL.st_id);
    float* t_lo = reinterpret_cast<float*>(b + CL.t_lo);
    float* t_hi = reinterpret_cast<float*>(b + CL.t_hi);
    int* t_id = reinterpret_cast<int*>(b + CL.t_id);
    float* t_d = reinterpret_cast<float*>(b + CL.t_d);
    int* t_need = reinterpret_cast<int*>(b + CL.t_need);
    float* root = reinterpret_cast<float*>(b + CL.root);
    float lu[6] = {lower[0], lower[1], lower[2], upper[0], upper[1], upper[2]};
    NIQ_CUDA(cudaMemsetAsync(b, 0, 64, s));
    NIQ_CUDA(cudaMemcpyAsync(root, lu, 24, cudaMemcpyHostToDevice, s));
    {
        long long blocks = (n_queries + 255) / 256;
        k_cp_init<<<(int)(blocks > 4096 ? 4096 : blocks), 256, 0, s>>>(root, st_lo, st_hi, st_id, min_dist_out,
                                                                       min_loc_out, n_queries);
        NIQ_CUDA(cudaGetLastError());
    }
    CpArgs a;
    a.q = query_points;
    a.min_dist = min_dist_out;
    a.min_loc = min_loc_out;
    a.eps_w = eps / sqrtf(3.f);
    a.interval = opts->mode == NIQ_MODE_INTERVAL;
    a.node_budget = 1ll << 62;   // the reference schedule is bounded by its stack capacity
    a.prune_tol = 0.f;
    const bool cons = opts->conservative != 0, slope = opts->mode == NIQ_MODE_SLOPE_INTERVAL;
    const int tpi = tpi_for_width(model->hdr.max_width);
    int rc = NIQ_OK;
    float* g_center = reinterpret_cast<float*>(b + GL.center);
    float* g_vecs = reinterpret_cast<float*>(b + GL.vecs);
    int* g_type = reinterpret_cast<int*>(b + GL.type);
    void* g_cws = b + GL.cws;
    auto run = [&](auto kern, int TPIv) -> int {
        SmemPlan p;
        int r2 = cp_plan(kern, model, 8, TPIv, p);
        if (r2) return r2;
        const int items = kNT / TPIv;
        int grid_max = 0;
        r2 = persistent_grid(kern, kNT, p.bytes, (batch_process_size + items - 1) / items, &grid_max);
        if (r2) return r2;
        long long top = n_queries;
        const long long B = batch_process_size;
        while (top > 0) {  // src/kd_tree.py:780-800
            const long long pop = top - B > 0 ? top - B : 0;
            const long long n = top - pop;
            const long long tiles = (n + items - 1) / items;
            if (growing) {
                // the batch's boxes through the growing-term engine first
                k_cp_boxes<<<(int)((n + 255) / 256), 256, 0, s>>>(st_lo, st_hi, pop, n, opts->conservative != 0,
                                                                  g_center, g_vecs);
                NIQ_CUDA(cudaGetLastError());
                const int rc2 = niq_classify_boxes(model, opts, n, g_center, g_vecs, 3, 0.f, g_type, nullptr, g_cws,
                                                   GL.cws_bytes, stream);
                if (rc2) return rc2;
            }
            kern<<<(int)(tiles < grid_max ? tiles : grid_max), kNT, p.bytes, s>>>(
                model->ref(), a, st_lo, st_hi, st_id, pop, n, t_lo, t_hi, t_id, t_d, t_need, p.fixed_floats, p.sw_cap,
                p.resident, g_type);
            NIQ_CUDA(cudaGetLastError());
            k_cp_finish<<<1, 1024, 0, s>>>(a, pop, n, t_lo, t_hi, t_id, t_d, t_need, st_lo, st_hi, st_id,
                                           stack_capacity, top_d, err);
            NIQ_CUDA(cudaGetLastError());
            long long hv[2] = {0, 0};
            NIQ_CUDA(cudaMemcpyAsync(hv, top_d, 16, cudaMemcpyDeviceToHost, s));
            NIQ_CUDA(cudaStreamSynchronize(s));
            top = hv[0];
            const int e = (int)(hv[1] & 0xffffffff);
            NIQ_REQUIRE(e == 0, NIQ_ERR_CAPACITY, "closest_point stack capacity %lld exceeded", (long long)stack_capacity);
        }
        return NIQ_OK;
    };
#define NIQ_CP(CC, SL) NIQ_DISPATCH_TPI(tpi, { rc = run(k_cp_batch<TPI, CC, SL, false>, TPI); })
    if (growing) { NIQ_DISPATCH_TPI(tpi, { rc = run(k_cp_batch<TPI, false, false, true>, TPI); }); }
    else if (slope) { if (cons) { NIQ_CP(true, true); } else { NIQ_CP(false, true); } }
    else { if (cons) { NIQ_CP(true, false); } else { NIQ_CP(false, false); } }
#undef NIQ_CP
    return rc;
}

size_t niq_closest_point_persistent_workspace_size(int64_t n_queries) { return cp_persistent_bytes(n_queries); }

int niq_closest_point_persistent(const niq_model* model, const niq_bound_opts* opts, const float* lower,
                                 const float* upper, int64_t n_queries, const float* query_points, float eps,
                                 int64_t node_budget, float* min_dist_out, float* min_loc_out, void* workspace,
                                 size_t workspace_bytes, void* stream) {
    NIQ_REQUIRE(model && opts && lower && upper, NIQ_ERR_INVALID_ARG, "null argument");
    NIQ_REQUIRE(fixed_mode(opts->mode), NIQ_ERR_UNSUPPORTED, "closest_point supports interval, affine_fixed, slope_interval");
    NIQ_REQUIRE(n_queries >= 0, NIQ_ERR_INVALID_ARG, "bad sizes");
    const size_t need = cp_persistent_bytes(n_queries);
    NIQ_REQUIRE(workspace && workspace_bytes >= need, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed", need);
    if (n_queries == 0) return NIQ_OK;
    NIQ_REQUIRE(query_points && min_dist_out && min_loc_out, NIQ_ERR_INVALID_ARG, "null array");
    cudaStream_t s = as_stream(stream);
    char* b = base256(workspace);
    unsigned long long* next = reinterpret_cast<unsigned long long*>(b);
    int* err = reinterpret_cast<int*>(b + 8);
    float* root = reinterpret_cast<float*>(b + al256(64));
    float* stacks = reinterpret_cast<float*>(b + al256(64) + al256(24));
    float lu[6] = {lower[0], lower[1], lower[2], upper[0], upper[1], upper[2]};
    NIQ_CUDA(cudaMemsetAsync(b, 0, 64, s));
    NIQ_CUDA(cudaMemcpyAsync(root, lu, 24, cudaMemcpyHostToDevice, s));
    CpArgs a;
    a.q = query_points;
    a.min_dist = min_dist_out;
    a.min_loc = min_loc_out;
    a.eps_w = eps / sqrtf(3.f);
    a.interval = opts->mode == NIQ_MODE_INTERVAL;
    a.node_budget = node_budget > 0 ? node_budget : (1ll << 62);
    a.prune_tol = eps;
    const bool cons = opts->conservative != 0, slope = opts->mode == NIQ_MODE_SLOPE_INTERVAL;
    const int tpi = tpi_for_width(model->hdr.max_width);
    int rc = NIQ_OK;
    auto run = [&](auto kern, int TPIv) -> int {
        SmemPlan p;
        int r2 = cp_plan(kern, model, 8, TPIv, p);
        if (r2) return r2;
        const int items = kNT / TPIv;
        int grid = 0;
        r2 = persistent_grid(kern, kNT, p.bytes, (n_queries + items - 1) / items, &grid);
        if (r2) return r2;
        NIQ_REQUIRE((size_t)grid * items <= (size_t)device_info().sm_count * 8 * 64, NIQ_ERR_UNSUPPORTED, "slot count");
        kern<<<grid, kNT, p.bytes, s>>>(model->ref(), a, n_queries, root, stacks, next, err, p.fixed_floats, p.sw_cap,
                                        p.resident);
        NIQ_CUDA(cudaGetLastError());
        return NIQ_OK;
    };
#define NIQ_CPP(CC, SL) NIQ_DISPATCH_TPI(tpi, { rc = run(k_cp_persistent<TPI, CC, SL>, TPI); })
    if (slope) { if (cons) { NIQ_CPP(true, true); } else { NIQ_CPP(false, true); } }
    else { if (cons) { NIQ_CPP(true, false); } else { NIQ_CPP(false, false); } }
#undef NIQ_CPP
    if (rc) return rc;
    int e = 0;
    NIQ_CUDA(cudaMemcpyAsync(&e, err, 4, cudaMemcpyDeviceToHost, s));
    NIQ_CUDA(cudaStreamSynchronize(s));
    NIQ_REQUIRE(e != NIQ_ERR_CAPACITY, NIQ_ERR_CAPACITY, "closest-point stack depth %d exceeded", kCpStack);
    NIQ_REQUIRE(e == 0, e, "closest-point node budget of %lld nodes per query exhausted; results are upper bounds",
                (long long)a.node_budget);
    return NIQ_OK;
}

size_t niq_intersect_workspace_size(const niq_model* model_a, const niq_model* model_b, const niq_bound_opts* opts,
                                    int64_t node_capacity) {
    size_t t = al256(sizeof(IsWs)) + 4 * al256(12 * (size_t)node_capacity);
    // plain path scratch: centers, vecs, samples, types, sample values
    t += al256(12 * (size_t)node_capacity) + al256(36 * (size_t)node_capacity) + al256(84 * (size_t)node_capacity) +
         2 * al256(4 * (size_t)node_capacity) + 2 * al256(28 * (size_t)node_capacity);
    if (model_a && model_b && opts && !fixed_mode(opts->mode)) {
        const size_t wa = wide_workspace_bytes(model_a->hdr, *opts, 3), wb = wide_workspace_bytes(model_b->hdr, *opts, 3);
        t += al256(wa > wb ? wa : wb);
    }
    return t + 512;
}

int niq_find_any_intersection(const niq_model* model_a, const niq_model* model_b, const niq_bound_opts* opts,
                              const float* lower, const float* upper, float eps, int64_t node_capacity,
                              int32_t* found_out, float* loc_out, int64_t* counts_out, void* workspace,
                              size_t workspace_bytes, void* stream) {
    NIQ_REQUIRE(model_a && model_b && opts && lower && upper && found_out && loc_out && counts_out,
                NIQ_ERR_INVALID_ARG, "null argument");
    NIQ_REQUIRE(node_capacity >= 2, NIQ_ERR_INVALID_ARG, "node capacity too small");
    const size_t need = niq_intersect_workspace_size(model_a, model_b, opts, node_capacity);
    NIQ_REQUIRE(workspace && workspace_bytes >= need, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed", need);
    cudaStream_t s = as_stream(stream);
    char* b = base256(workspace);
    IsWs* ws = reinterpret_cast<IsWs*>(b);
    size_t off = al256(sizeof(IsWs));
    float* lv[4];
    for (int i = 0; i < 4; ++i) { lv[i] = reinterpret_cast<float*>(b + off); off += al256(12 * (size_t)node_capacity); }
    NIQ_CUDA(cudaMemsetAsync(ws, 0, sizeof(IsWs), s));
    NIQ_CUDA(cudaMemcpyAsync(lv[0], lower, 12, cudaMemcpyHostToDevice, s));
    NIQ_CUDA(cudaMemcpyAsync(lv[1], upper, 12, cudaMemcpyHostToDevice, s));
    const unsigned long long one = 1;
    NIQ_CUDA(cudaMemcpyAsync(&ws->level_count[0], &one, 8, cudaMemcpyHostToDevice, s));
    const float eps_w = eps / sqrtf(3.f);
    const int mode = opts->mode;
    int rc = NIQ_OK;
    if (fixed_mode(mode)) {
        const bool cons = opts->conservative != 0, slope = mode == NIQ_MODE_SLOPE_INTERVAL;
        const int maxw = model_a->hdr.max_width > model_b->hdr.max_width ? model_a->hdr.max_width : model_b->hdr.max_width;
        const int tpi = tpi_for_width(maxw);
        const int wfl = model_a->hdr.n_weight_floats + model_b->hdr.n_weight_floats;
        const int ml = max_layer_floats(model_a->hdr) > max_layer_floats(model_b->hdr) ? max_layer_floats(model_a->hdr)
                                                                                        : max_layer_floats(model_b->hdr);
        auto run = [&](auto kern, int TPIv) -> int {
            const int items = kNT / TPIv;
            const int state = items * 8 * (TPIv * 8 + 4) + ((items * 8 + 3) & ~3);
            SmemPlan p = plan_smem(state, wfl, ml, smem_budget(kern, kNT));
            NIQ_REQUIRE(p.resident || p.sw_cap >= 5 * maxw, NIQ_ERR_UNSUPPORTED, "shared memory too small");
            int r2 = prepare_kernel(kern, p.bytes);
            if (r2) return r2;
            int per_sm = 0;
            NIQ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kNT, p.bytes));
            NIQ_REQUIRE(per_sm >= 1, NIQ_ERR_UNSUPPORTED, "intersection kernel does not fit");
            const int grid = per_sm * device_info().sm_count;
            NiqModelRef A = model_a->ref(), Bm = model_b->ref();
            int interval = mode == NIQ_MODE_INTERVAL;
            float ew = eps_w;
            long long cap = node_capacity;
            int woffB = model_a->hdr.n_weight_floats;
            int fixed = p.fixed_floats, swc = p.sw_cap, res = p.resident;
            unsigned int polls = barrier_polls();
            void* args[] = {&A, &Bm, &interval, &ew, &ws, &lv[0], &lv[1], &lv[2], &lv[3], &cap, &woffB, &fixed, &swc, &res,
                            &polls};
            NIQ_CUDA(cudaLaunchCooperativeKernel((const void*)kern, grid, kNT, args, p.bytes, s));
            return NIQ_OK;
        };
#define NIQ_IS(CC, SL) NIQ_DISPATCH_TPI(tpi, { rc = run(k_intersect<TPI, CC, SL>, TPI); })
        if (slope) { if (cons) { NIQ_IS(true, true); } else { NIQ_IS(false, true); } }
        else { if (cons) { NIQ_IS(true, false); } else { NIQ_IS(false, false); } }
#undef NIQ_IS
        if (rc) return rc;
    } else {
        // plain host loop (src/kd_tree.py:592-655)
        float* center = reinterpret_cast<float*>(b + off); off += al256(12 * (size_t)node_capacity);
        float* vecs = reinterpret_cast<float*>(b + off); off += al256(36 * (size_t)node_capacity);
        float* samples = reinterpret_cast<float*>(b + off); off += al256(84 * (size_t)node_capacity);
        int* tA = reinterpret_cast<int*>(b + off); off += al256(4 * (size_t)node_capacity);
        int* tB = reinterpret_cast<int*>(b + off); off += al256(4 * (size_t)node_capacity);
        float* vA = reinterpret_cast<float*>(b + off); off += al256(28 * (size_t)node_capacity);
        float* vB = reinterpret_cast<float*>(b + off); off += al256(28 * (size_t)node_capacity);
        void* wws = b + off;
        const size_t wws_bytes = workspace_bytes - (size_t)(b - reinterpret_cast<char*>(workspace)) - off;
        long long n = 1;
        for (int L = 0; L < kIsMaxLevels && n > 0; ++L) {
            const float* lo = lv[(L & 1) ? 2 : 0];
            const float* hi = lv[(L & 1) ? 3 : 1];
            float* olo = lv[(L & 1) ? 0 : 2];
            float* ohi = lv[(L & 1) ? 1 : 3];
            const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
            k_is_prepare<<<blocks, 256, 0, s>>>(n, lo, hi, eps_w, center, vecs, samples);
            NIQ_CUDA(cudaGetLastError());
            rc = niq_classify_boxes(model_a, opts, n, center, vecs, 3, 0.f, tA, nullptr, wws, wws_bytes, s);
            if (rc) return rc;
            rc = niq_classify_boxes(model_b, opts, n, center, vecs, 3, 0.f, tB, nullptr, wws, wws_bytes, s);
            if (rc) return rc;
            rc = niq_eval_points(model_a, 7 * n, samples, vA, s);
            if (rc) return rc;
            rc = niq_eval_points(model_b, 7 * n, samples, vB, s);
            if (rc) return rc;
            k_is_decide<<<blocks, 256, 0, s>>>(n, L, lo, hi, eps_w, tA, tB, vA, vB, samples, ws, olo, ohi,
                                               node_capacity);
            NIQ_CUDA(cudaGetLastError());
            int hv[2];
            unsigned long long nn = 0;
            NIQ_CUDA(cudaMemcpyAsync(&nn, &ws->level_count[L + 1], 8, cudaMemcpyDeviceToHost, s));
            NIQ_CUDA(cudaMemcpyAsync(hv, &ws->found, 8, cudaMemcpyDeviceToHost, s));
            NIQ_CUDA(cudaStreamSynchronize(s));
            if (hv[0] || hv[1]) break;
            n = (long long)nn;
            NIQ_REQUIRE(n <= node_capacity, NIQ_ERR_CAPACITY, "node capacity %lld exceeded", (long long)node_capacity);
        }
    }
    k_is_finish<<<1, 1, 0, s>>>(ws, found_out, loc_out, reinterpret_cast<long long*>(counts_out));
    NIQ_CUDA(cudaGetLastError());
    int e = 0;
    NIQ_CUDA(cudaMemcpyAsync(&e, &ws->err, 4, cudaMemcpyDeviceToHost, s));
    NIQ_CUDA(cudaStreamSynchronize(s));
    NIQ_REQUIRE(e == 0, e, "intersection search failed (%d)", e);
    return NIQ_OK;
}

}  // extern "C"
