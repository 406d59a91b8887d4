// wide_engine.cuh -- range propagation for the modes whose noise-term count grows:
// 'affine_all', 'affine_truncate' and 'affine_append' (src/affine.py:127-193).
//
// One CTA propagates one box at a time.  Its affine form lives in a per-CTA slot of the
// caller's workspace: row 0 base, row 1 err, rows 2.. the noise terms, each row wmax
// floats.  A dense layer is a thread-per-column product over row chunks staged in shared
// memory; the activation appends diag(delta) rows ('all'/'truncate'), then 'truncate'
// ranks every row by its L1 magnitude (stable, descending: src/affine.py:144-162) and
// keeps the first truncate_count, folding the rest into err; 'append' keeps the
// n_append largest deltas as new rows (ties to the lower index, as lax.top_k) and adds
// the remainder, as one scalar, to every err entry (src/affine.py:183-191).
//
// Conservative mode.  The rounding error of a layer's dot products (at most gamma times
// |base| + sum_r |aff_r| pushed through |A|, plus the bias addition) is a per-neuron
// quantity rho_j.  These modes give it its own noise symbol: it widens the bounds that
// choose the linearisation, and alpha_j rho_j joins neuron j's new noise row delta_j
// (together with the rounding of alpha*base + beta and alpha*aff).  A symbol travels
// through the next layers with A, not |A| as err does, so the outward terms stay
// proportional to the values instead of growing like |A|^depth.
#pragma once
#include "niq_host.cuh"

namespace niq {

constexpr int kWideNT = 256;
constexpr int kWideRB = 16;

// Rows a box's affine form can reach at any point of the pass (before truncation).
NIQ_HOST_DEVICE int wide_rows_cap(const NiqSpecHeader& H, const niq_bound_opts& o, int v) {
    int rows = v, cap = v;
    for (int i = 0; i < H.n_layers; ++i) {
        const NiqLayer& L = H.layers[i];
        if (L.act == NIQ_ACT_NONE) continue;
        if (o.mode == NIQ_MODE_AFFINE_APPEND) rows += o.n_append;
        else rows += L.out;
        cap = cap > rows ? cap : rows;
        if (o.mode == NIQ_MODE_AFFINE_TRUNCATE && rows > o.truncate_count) rows = o.truncate_count;
    }
    return cap;
}

inline long long wide_slot_floats(const NiqSpecHeader& H, const niq_bound_opts& o, int v) {
    const long long rows = wide_rows_cap(H, o, v) + 2;
    const long long w = H.max_width;
    return 2 * rows * w + 2 * rows + 4;
}

inline int wide_slots() { return device_info().sm_count * 2; }

// The tensor-core (3xTF32) form of this engine (k_wide_tc.cu).
bool wide_tc_eligible(const NiqSpecHeader& H, const niq_bound_opts& o, int v);
bool wide_use_tc(const NiqSpecHeader& H, const niq_bound_opts& o, int v);
size_t wide_tc_workspace_bytes();
int wide_tc_classify(const niq_model* m, const niq_bound_opts& o, long long n, const float* center, const float* vecs,
                     int v, float offset, int* sign_out, float* lohi_out, void* ws, size_t ws_bytes, cudaStream_t s);

inline size_t wide_workspace_bytes(const NiqSpecHeader& H, const niq_bound_opts& o, int v) {
    if (wide_use_tc(H, o, v)) return wide_tc_workspace_bytes();
    return (size_t)wide_slot_floats(H, o, v) * wide_slots() * 4 + 256;
}

template <bool C>
__device__ float wide_block_sum(float x, float* red) {
    for (int off = 16; off > 0; off >>= 1) {
        const float y = __shfl_down_sync(0xffffffffu, x, off);
        x = C ? __fadd_ru(x, y) : x + y;
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    float s = 0.f;
    if (threadIdx.x == 0) {
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s = C ? __fadd_ru(s, red[i]) : s + red[i];
        red[32] = s;
    }
    __syncthreads();
    return red[32];
}

template <bool C>
__global__ void __launch_bounds__(kWideNT) k_wide_classify(NiqModelRef M, niq_bound_opts opts, long long n,
                                                           const float* __restrict__ center, const float* __restrict__ vecs,
                                                           int v, float offset, int* __restrict__ sign_out,
                                                           float* __restrict__ lohi_out, float* __restrict__ ws,
                                                           long long slot_floats, int rows_cap) {
    __shared__ NiqSpecHeader H;
    __shared__ float xin[kWideRB][NIQ_MAX_WIDTH + 4];
    __shared__ float red[40];
    __shared__ float sdelta[NIQ_MAX_WIDTH];
    __shared__ float sfold[NIQ_MAX_WIDTH];   // gamma (|base_k| + sum_r |aff_rk|) before the layer (conservative)
    load_header(H, M.hdr);
    __syncthreads();
    const int W = H.max_width;
    float* slot = ws + (long long)blockIdx.x * slot_floats;
    float* bufA = slot;
    float* bufB = slot + (long long)(rows_cap + 2) * W;
    float* mags = bufB + (long long)(rows_cap + 2) * W;
    int* rank = reinterpret_cast<int*>(mags + rows_cap + 2);
    const int j = threadIdx.x;
    const int mode = opts.mode;

    for (long long b = blockIdx.x; b < n; b += gridDim.x) {
        float* cur = bufA;
        float* nxt = bufB;
        int nrows = v;
        // input: base = center, aff = vecs, err = 0 (src/affine.py:109-117)
        if (j < 4) {
            const int k = j;
            const bool real = k < 3;
            const float c = real ? center[3 * b + k] : 0.f;
            float S = fabsf(c);
            cur[k] = c;
            for (int r = 0; r < v; ++r) {
                const float a = real ? vecs[3 * v * b + 3 * r + k] : 0.f;
                cur[(2 + r) * W + k] = a;
                S = __fadd_ru(S, fabsf(a));
            }
            cur[W + k] = 0.f;
            sfold[k] = C ? __fmul_ru(H.layers[0].gamma, S) : 0.f;
        }
        __syncthreads();
        for (int li = 0; li < H.n_layers; ++li) {
            const NiqLayer L = H.layers[li];
            const float* A = M.w + L.a_off;
            const float bj = (j < L.out) ? __ldg(M.w + L.b_off + j) : 0.f;
            const float gam = C ? L.gamma : 0.f;
            const int total = nrows + 2;
            // ---- dense: rows 0 (base, +b), 1 (err, |A|), 2.. (noise)
            for (int r0 = 0; r0 < total; r0 += kWideRB) {
                const int rn = min(kWideRB, total - r0);
                for (int i = threadIdx.x; i < rn * L.in_pad; i += blockDim.x) {
                    const int rr = i / L.in_pad, k = i % L.in_pad;
                    xin[rr][k] = cur[(long long)(r0 + rr) * W + k];
                }
                __syncthreads();
                if (j < L.out_pad) {
                    float acc[kWideRB];
#pragma unroll
                    for (int rr = 0; rr < kWideRB; ++rr) acc[rr] = 0.f;
                    for (int k = 0; k < L.in_pad; ++k) {
                        const float a = __ldg(A + k * L.out_pad + j);
                        const float aa = fabsf(a);
#pragma unroll
                        for (int rr = 0; rr < kWideRB; ++rr) {
                            const int row = r0 + rr;
                            acc[rr] = fmaf(xin[rr][k], row == 1 ? aa : a, acc[rr]);
                        }
                    }
                    for (int rr = 0; rr < rn; ++rr) {
                        const int row = r0 + rr;
                        float val = acc[rr];
                        if (j >= L.out) val = 0.f;
                        else if (row == 0) val = __fadd_rn(val, bj);
                        else if (row == 1 && C) val = __fmul_ru(val, 1.f + 2.f * gam);
                        nxt[(long long)row * W + j] = val;
                    }
                }
                __syncthreads();
            }
            // rounding bound of this layer's dot products and bias addition, per neuron
            float rho = 0.f;
            if (C && j < L.out) {
                for (int k = 0; k < L.in; ++k) rho = __fmaf_ru(sfold[k], fabsf(__ldg(A + k * L.out_pad + j)), rho);
                rho = __fadd_ru(__fmaf_ru(rho, 1.f + 2.f * gam, __fmul_ru(gam, fabsf(bj))), (float)(L.in + 2) * NIQ_TINY);
            }
            float* t = cur; cur = nxt; nxt = t;   // cur: this layer's output
            __syncthreads();  // every thread has read sfold
            if (L.act == NIQ_ACT_NONE) {
                // no new symbol without an activation: the rounding goes to err
                if (C && j < L.out) {
                    cur[W + j] = __fadd_ru(cur[W + j], rho);
                    if (li + 1 < H.n_layers) {
                        float S = 0.f;
                        for (int r = 0; r < nrows; ++r) S = __fadd_ru(S, fabsf(cur[(long long)(2 + r) * W + j]));
                        sfold[j] = __fmul_ru(H.layers[li + 1].gamma, __fadd_ru(fabsf(cur[j]), S));
                    }
                }
                __syncthreads();
                continue;
            }
            // ---- activation (src/affine.py:164-193)
            const float gam_next = (C && li + 1 < H.n_layers) ? H.layers[li + 1].gamma : 0.f;
            float delta_j = 0.f, aS = 0.f, alpha = 0.f;
            if (j < L.out) {
                float S = 0.f;
                for (int r = 0; r < nrows; ++r) S = add_up<C>(S, fabsf(cur[(long long)(2 + r) * W + j]));
                const float base = cur[j], err = cur[W + j];
                const float rad = add_up<C>(add_up<C>(S, err), rho);
                const float lo = sub_dn<C>(base, rad), hi = add_up<C>(base, rad);
                const Lin z = linearize<C>(L.act, lo, hi);
                alpha = z.a;
                const float nb = C ? fmaf(z.a, base, z.b) : __fadd_rn(__fmul_rn(z.a, base), z.b);
                for (int r = 0; r < nrows; ++r) {
                    float* p = cur + (long long)(2 + r) * W + j;
                    *p = __fmul_rn(z.a, *p);
                }
                delta_j = fabsf(z.d);
                aS = C ? __fmul_ru(__fmul_ru(z.a, S), 1.f + NIQ_ULP_REL) : 0.f;
                if (C) {
                    // neuron j's symbol: linearisation, this layer's rounding, alpha*base + beta and alpha*aff
                    delta_j = __fmaf_ru(z.a, rho, delta_j);
                    delta_j = __fmaf_ru(__fadd_ru(fabsf(nb), aS), NIQ_ULP_REL, delta_j);
                }
                cur[j] = nb;
                cur[W + j] = C ? __fmul_ru(z.a, err) : __fmul_rn(z.a, err);
            }
            if (mode == NIQ_MODE_AFFINE_APPEND) {
                if (j < NIQ_MAX_WIDTH) sdelta[j] = (j < L.out) ? delta_j : -INFINITY;
                __syncthreads();
                const int k = opts.n_append;
                // rank of delta_j: larger first, ties to the lower index (lax.top_k)
                int rk = 0;
                if (j < L.out)
                    for (int i = 0; i < L.out; ++i) rk += (sdelta[i] > delta_j) || (sdelta[i] == delta_j && i < j);
                const float kept = (j < L.out && rk < k) ? delta_j : 0.f;
                const float dsum = wide_block_sum<C>(j < L.out ? delta_j : 0.f, red);
                const float ksum = wide_block_sum<false>(kept, red);
                for (int r = 0; r < k; ++r)
                    if (j < L.out_pad) cur[(long long)(2 + nrows + r) * W + j] = (j < L.out && rk == r) ? delta_j : 0.f;
                if (j < L.out) {
                    const float rest = C ? __fsub_ru(dsum, ksum) : dsum - ksum;
                    cur[W + j] = add_up<C>(cur[W + j], rest);
                    if (C) sfold[j] = __fmul_ru(gam_next, __fadd_ru(__fadd_ru(fabsf(cur[j]), aS), delta_j));
                }
                nrows += k;
                __syncthreads();
                continue;
            }
            // 'affine_all' / 'affine_truncate': append diag(delta)
            for (int r = 0; r < L.out; ++r)
                if (j < L.out_pad) cur[(long long)(2 + nrows + r) * W + j] = (j == r) ? delta_j : 0.f;
            if (C && j < L.out) sfold[j] = __fmul_ru(gam_next, __fadd_ru(__fadd_ru(fabsf(cur[j]), aS), delta_j));
            nrows += L.out;
            __syncthreads();
            if (mode == NIQ_MODE_AFFINE_TRUNCATE && nrows > opts.truncate_count) {
                const int K = opts.truncate_count;
                for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
                    float m = 0.f;
                    const float* row = cur + (long long)(2 + r) * W;
                    for (int c = 0; c < L.out; ++c) m += fabsf(row[c]);
                    mags[r] = m;
                }
                __syncthreads();
                for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
                    const float m = mags[r];
                    int rk = 0;
                    for (int i = 0; i < nrows; ++i) rk += (mags[i] > m) || (mags[i] == m && i < r);
                    rank[r] = rk;
                }
                __syncthreads();
                if (j < L.out_pad) {
                    float drop = 0.f;
                    for (int r = 0; r < nrows; ++r) {
                        const float x = cur[(long long)(2 + r) * W + j];
                        const int rk = rank[r];
                        if (rk < K) nxt[(long long)(2 + rk) * W + j] = x;
                        else drop = add_up<C>(drop, fabsf(x));
                    }
                    nxt[j] = cur[j];
                    nxt[W + j] = add_up<C>(cur[W + j], drop);
                }
                nrows = K;
                float* t2 = cur; cur = nxt; nxt = t2;
                __syncthreads();
            }
        }
        // ---- output bounds of column 0 (src/affine.py:119-125)
        float part = 0.f;
        for (int r = threadIdx.x; r < nrows; r += blockDim.x) part = add_up<C>(part, fabsf(cur[(long long)(2 + r) * W]));
        const float S = wide_block_sum<C>(part, red);
        if (threadIdx.x == 0) {
            const float rad = add_up<C>(S, cur[W]);
            const float lo = sub_dn<C>(cur[0], rad), hi = add_up<C>(cur[0], rad);
            sign_out[b] = sign_of_bounds(lo, hi, offset);
            if (lohi_out) { lohi_out[2 * b] = lo; lohi_out[2 * b + 1] = hi; }
        }
        __syncthreads();
    }
}

inline int wide_classify(const niq_model* m, const niq_bound_opts& o, long long n, const float* center, const float* vecs,
                         int v, float offset, int* sign_out, float* lohi_out, void* ws, size_t ws_bytes, cudaStream_t s) {
    NIQ_REQUIRE(o.mode == NIQ_MODE_AFFINE_ALL || o.mode == NIQ_MODE_AFFINE_TRUNCATE || o.mode == NIQ_MODE_AFFINE_APPEND,
                NIQ_ERR_INVALID_ARG, "unknown mode %d", o.mode);
    NIQ_REQUIRE(o.mode != NIQ_MODE_AFFINE_TRUNCATE || o.truncate_count >= 1, NIQ_ERR_INVALID_ARG, "truncate_count must be >= 1");
    if (o.mode == NIQ_MODE_AFFINE_APPEND) {
        NIQ_REQUIRE(o.n_append >= 1, NIQ_ERR_INVALID_ARG, "n_append must be >= 1");
        for (int i = 0; i < m->hdr.n_layers; ++i)
            NIQ_REQUIRE(m->hdr.layers[i].act == NIQ_ACT_NONE || m->hdr.layers[i].out >= o.n_append, NIQ_ERR_INVALID_ARG,
                        "n_append %d exceeds layer %d width %d", o.n_append, i, m->hdr.layers[i].out);
    }
    NIQ_REQUIRE(o.products >= NIQ_PRODUCTS_AUTO && o.products <= NIQ_PRODUCTS_3XTF32, NIQ_ERR_INVALID_ARG,
                "unknown products %d", o.products);
    NIQ_REQUIRE(o.products != NIQ_PRODUCTS_3XTF32 || wide_tc_eligible(m->hdr, o, v), NIQ_ERR_UNSUPPORTED,
                "3xTF32 products need truncate_count <= 256 (or <= 256 rows in affine_all), activated hidden "
                "layers and widths <= 256");
    if (wide_use_tc(m->hdr, o, v))
        return wide_tc_classify(m, o, n, center, vecs, v, offset, sign_out, lohi_out, ws, ws_bytes, s);
    const size_t need = wide_workspace_bytes(m->hdr, o, v);
    NIQ_REQUIRE(ws && ws_bytes >= need, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed, %zu given", need, ws_bytes);
    const long long slot = wide_slot_floats(m->hdr, o, v);
    const int rows_cap = wide_rows_cap(m->hdr, o, v);
    long long grid = wide_slots();
    if (grid > n) grid = n;
    float* w = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    if (o.conservative)
        k_wide_classify<true><<<(int)grid, kWideNT, 0, s>>>(m->ref(), o, n, center, vecs, v, offset, sign_out, lohi_out, w, slot, rows_cap);
    else
        k_wide_classify<false><<<(int)grid, kWideNT, 0, s>>>(m->ref(), o, n, center, vecs, v, offset, sign_out, lohi_out, w, slot, rows_cap);
    NIQ_CUDA(cudaGetLastError());
    return NIQ_OK;
}

}  // namespace niq
