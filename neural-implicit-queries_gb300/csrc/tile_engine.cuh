// tile_engine.cuh -- fused multi-layer range propagation over a CTA tile of items.
//
// One CTA holds ITEMS items; each item is R rows of width <= W (the widest layer) kept
// in shared memory for the whole forward pass, so every layer reads its input from
// on-chip memory.  A thread owns one item and COLS output columns of every row (8; 4 in
// the narrow tile, which gives an item twice the lanes and each lane half the work), so
// the per-column range rules (radius, linearisation, rounding terms) run in registers.
//
// Row layouts (template R rows, the last NABS rows multiply |A| instead of A):
//   ROWS_AFFINE (NABS=1): 0 base | 1..v noise rows | v+1..v+np points | R-1 err
//       the affine form of src/affine.py:59-60 (base, aff, err) plus plain points
//   ROWS_SLOPE  (R=8, NABS=4): 0 primal | 1..v slope centers | v+1..v+np points |
//       4 primal rounding error | 5..4+v slope widths      (src/slope_interval.py:164-210)
//   ROWS_POINTS (NABS=0): every row is a point evaluation (src/mlp.py:253-347)
//   ROWS_JVP    (NABS=0, R=8): two points, each a value row and three tangent rows
//       (d/dx, d/dy, d/dz): forward-mode derivatives, jax.jacfwd of src/render.py:61-63
//
// Dense rule (src/affine_layers.py:11-31, src/slope_interval_layers.py:11-33):
//   base <- base@A + b, aff <- aff@A, err <- err@|A|.
// Activation rules: ReLU Chebyshev (src/affine_layers.py:34-56), ELU
// (src/affine_layers.py:59-97), TanH (new), applied as src/affine.py:164-193
// ('interval'/'affine_fixed': err <- alpha*err + delta).
//
// Outward rounding (conservative mode).  For a dense layer with n = in inputs, every
// computed dot product is within gamma = (n+1)u/(1-(n+1)u) of its exact value relative
// to sum |x_k||A_kj| + |b_j| (u = 2^-24, any summation order, FMA or not).  Those
// errors are charged to the err row by storing err'_k = err_k + gamma(|base_k| +
// sum_r |aff_rk|) before the layer ("fold") and scaling the computed err@|A| by
// (1 + 2 gamma) after it.  Each linearisation computes its offset interval [rlo, rhi]
// with directed rounding plus the documented error of tanhf/expf, and charges the
// rounding of alpha*base + beta and alpha*aff to err.  The resulting [lower, upper]
// contains the exact real-arithmetic range of the network over the box.
#pragma once
#include "niq_common.cuh"

namespace niq {

enum RowMode : int { ROWS_AFFINE = 0, ROWS_SLOPE = 1, ROWS_POINTS = 2, ROWS_JVP = 3 };

struct RowPlan {
    int mode;  // RowMode
    int v;     // noise rows (affine) / slope rows
    int np;    // point rows
};

// Relative allowance for tanhf/expf/expm1f results (their documented maximum errors
// are 2 ulp or less; 2^-21 is four times that).
#define NIQ_FN_REL 4.76837158203125e-07f
#define NIQ_FN_ABS 1.0e-37f

template <int R_, int NABS_, int TPI_, int NT_, int COLS_ = 8>
struct TileCfg {
    static constexpr int R = R_;
    static constexpr int NABS = NABS_;
    static constexpr int TPI = TPI_;          // threads per item
    static constexpr int NT = NT_;            // threads per CTA
    static constexpr int COLS = COLS_;        // columns per thread
    static constexpr int NQ = COLS / 4;       // float4 groups per thread
    static constexpr int W = TPI * COLS;      // widest layer this tile supports
    static constexpr int LD = W + 4;          // row stride in floats (bank spread)
    static constexpr int ITEMS = NT / TPI;
    static constexpr int STATE_FLOATS = ITEMS * R * LD;
    // k-slices of a single-group layer (the width-1 output layer): the narrow tile splits
    // k as the 8-column tile with half its lanes does, so both give the same sums
    static constexpr int KSPLIT = COLS == 4 ? (TPI > 1 ? TPI / 2 : 1) : TPI;
    static_assert(NT % TPI == 0, "tile");
    static_assert(COLS == 4 || COLS == 8, "columns per thread");
};

// Column of float4 group q, lane j for thread g of an item: groups interleave across
// the item's threads so a warp's weight loads are contiguous.
template <int TPI>
__device__ __forceinline__ int col_of(int g, int q) { return (q * TPI + g) * 4; }

// ----------------------------------------------------------------------------------
// Linearisations.  Return alpha, beta, delta such that act(x) lies in
// [alpha x + beta - delta, alpha x + beta + delta] for all x in [l, u].
// ----------------------------------------------------------------------------------
struct Lin { float a, b, d; };

template <bool C>
__device__ __forceinline__ Lin lin_relu(float l, float u) {
    Lin r;
    if (!C) {
        float a;
        if (l >= 0.f) a = 1.f;
        else if (u < 0.f) a = 0.f;
        else a = __fdiv_rn(__fsub_rn(fmaxf(u, 0.f), fmaxf(l, 0.f)), __fsub_rn(u, l));
        a = fminf(fmaxf(a, 0.f), 1.f);  // NaN -> 0 (fmaxf drops NaN), clip to [0, 1]
        r.a = a;
        // src/affine_layers.py:55-56: beta = (relu(l) - alpha l) / 2, delta = beta
        r.b = __fmul_rn(__fsub_rn(fmaxf(l, 0.f), __fmul_rn(a, l)), 0.5f);
        r.d = fabsf(r.b);
        return r;
    }
    // Conservative: any alpha in [0, 1] gives a valid enclosure, because the offset
    // interval below is computed for the alpha actually used.  So the secant slope
    // u / (u - l) (l < 0 <= u) takes the fast divide (within 2 ulp, no slow path).
    // Otherwise g(x) = relu(x) - a x is exactly 0 (identity, a = 1) or relu(x) = 0
    // (a = 0); a NaN bound (overflowed input) leaves nothing known: unbounded offset.
    r.a = (l >= 0.f) ? 1.f : 0.f;
    r.b = 0.f;
    r.d = (l == l && u == u) ? 0.f : INFINITY;
    if ((l < 0.f) && (u >= 0.f)) {
        const float a = fminf(fmaxf(__fdividef(u, __fsub_rn(u, l)), 0.f), 1.f);  // NaN -> 0
        r.a = a;
        // g is piecewise linear here: extrema at l, u and 0
        const float gl_lo = __fmul_rd(-a, l), gl_hi = __fmul_ru(-a, l);
        const float gu_lo = __fmaf_rd(-a, u, u), gu_hi = __fmaf_ru(-a, u, u);
        const float rlo = fminf(fminf(gl_lo, gu_lo), 0.f);
        const float rhi = fmaxf(fmaxf(gl_hi, gu_hi), 0.f);
        r.b = 0.5f * (rlo + rhi);
        r.d = fmaxf(__fsub_ru(rhi, r.b), __fsub_ru(r.b, rlo));
    }
    return r;
}

__device__ __forceinline__ float elu_f(float x) { return x > 0.f ? x : expm1f(x); }

template <bool C>
__device__ __forceinline__ Lin lin_elu(float l, float u) {
    Lin r;
    const float lF = elu_f(l), uF = elu_f(u);
    const float lS = fminf(expf(l), 1.f), uS = fminf(expf(u), 1.f);
    float a = __fdiv_rn(__fsub_rn(uF, lF), __fsub_rn(u, l));
    if (l >= 0.f) a = 1.f;
    if (a != a) a = 0.f;
    a = fminf(fmaxf(a, lS), uS);       // src/affine_layers.py:81
    if (l >= 0.f) { r.a = 1.f; r.b = 0.f; r.d = 0.f; return r; }
    r.a = a;
    if (!C) {
        const float r_upper = __fsub_rn(lF, __fmul_rn(a, l));
        const float xl = fminf(fmaxf(logf(a), l), u);
        const float r_lower = __fsub_rn(__fsub_rn(a, 1.f), __fmul_rn(a, xl));
        r.b = __fmul_rn(0.5f, __fadd_rn(r_upper, r_lower));
        r.d = __fmul_rn(0.5f, fabsf(__fsub_rn(r_upper, r_lower)));
        return r;
    }
    // g(x) = elu(x) - a x is convex: the max is at an endpoint; the min is bounded by the
    // supporting line at x~ = clip(log a, l, u): g >= g(x~) - |g'(x~)| (u - l).
    auto e_hi = [](float x) { float e = elu_f(x); return x > 0.f ? e : __fadd_ru(e, __fmaf_ru(fabsf(e), NIQ_FN_REL, NIQ_FN_ABS)); };
    auto e_lo = [](float x) { float e = elu_f(x); return x > 0.f ? e : __fsub_rd(e, __fmaf_ru(fabsf(e), NIQ_FN_REL, NIQ_FN_ABS)); };
    const float rhi = fmaxf(__fmaf_ru(-a, l, e_hi(l)), __fmaf_ru(-a, u, e_hi(u)));
    const float xt = fminf(fmaxf(logf(a), l), u);
    const float dxt = xt > 0.f ? 1.f : expf(xt);
    const float gp = __fadd_ru(fabsf(__fsub_rn(dxt, a)), __fmaf_ru(dxt, NIQ_FN_REL, 1e-7f));
    float rlo = __fsub_rd(__fmaf_rd(-a, xt, e_lo(xt)), __fmul_ru(gp, __fsub_ru(u, l)));
    rlo = fminf(rlo, fminf(__fmaf_rd(-a, l, e_lo(l)), __fmaf_rd(-a, u, e_lo(u))));
    r.b = 0.5f * (rlo + rhi);
    r.d = fmaxf(__fsub_ru(rhi, r.b), __fsub_ru(r.b, rlo));
    return r;
}

__device__ __forceinline__ float tanh_hi(float x) { float t = tanhf(x); return __fadd_ru(t, __fmaf_ru(fabsf(t), NIQ_FN_REL, NIQ_FN_ABS)); }
__device__ __forceinline__ float tanh_lo(float x) { float t = tanhf(x); return __fsub_rd(t, __fmaf_ru(fabsf(t), NIQ_FN_REL, NIQ_FN_ABS)); }

template <bool C>
__device__ __forceinline__ Lin lin_tanh(float l, float u) {
    // No TanH rule exists in the reference.  alpha is the secant slope on [l, u]; the
    // offset g(x) = tanh(x) - alpha x is convex for x <= 0 and concave for x >= 0 with
    // stationary points +-xs, xs = atanh(sqrt(1 - alpha)).
    Lin r;
    const float tl = tanhf(l), tu = tanhf(u);
    const float w = __fsub_rn(u, l);
    float a;
    if (w > 0.f) a = __fdiv_rn(__fsub_rn(tu, tl), w);
    else { const float tm = tanhf(0.5f * (l + u)); a = 1.f - tm * tm; }
    a = fminf(fmaxf(a, 0.f), 1.f);
    r.a = a;
    const float xs = atanhf(sqrtf(fmaxf(1.f - a, 0.f)));  // +inf when a == 0
    if (!C) {
        const float c2 = fminf(fmaxf(xs, l), u), c3 = fminf(fmaxf(-xs, l), u);
        const float g0 = __fsub_rn(tl, __fmul_rn(a, l)), g1 = __fsub_rn(tu, __fmul_rn(a, u));
        const float g2 = __fsub_rn(tanhf(c2), __fmul_rn(a, c2)), g3 = __fsub_rn(tanhf(c3), __fmul_rn(a, c3));
        const float rlo = fminf(fminf(g0, g1), fminf(g2, g3));
        const float rhi = fmaxf(fmaxf(g0, g1), fmaxf(g2, g3));
        r.b = __fmul_rn(0.5f, __fadd_rn(rhi, rlo));
        r.d = __fmul_rn(0.5f, __fsub_rn(rhi, rlo));
        return r;
    }
    // g'(x) = sech^2(x) - a: increasing on x <= 0, decreasing on x >= 0.
    auto gp = [a](float x) { const float t = tanhf(x); return 1.f - t * t - a; };
    const float GPS = 2e-6f;  // slack on the sign of a computed g'
    auto ghi = [a](float x) { return __fmaf_ru(-a, x, tanh_hi(x)); };
    auto glo = [a](float x) { return __fmaf_rd(-a, x, tanh_lo(x)); };
    float rlo = INFINITY, rhi = -INFINITY;
    if (l < 0.f) {                       // convex piece [pa, pb]
        const float pa = l, pb = fminf(u, 0.f);
        rhi = fmaxf(rhi, fmaxf(ghi(pa), ghi(pb)));
        const float da = gp(pa), db = gp(pb);
        float mn;
        if (da >= GPS) mn = glo(pa);              // increasing
        else if (db <= -GPS) mn = glo(pb);        // decreasing
        else {
            const float xt = fminf(fmaxf(-xs, pa), pb);
            const float s = __fadd_ru(fabsf(gp(xt)), GPS);
            mn = __fsub_rd(glo(xt), __fmul_ru(s, __fsub_ru(pb, pa)));
            mn = fminf(mn, fminf(glo(pa), glo(pb)));
        }
        rlo = fminf(rlo, mn);
    }
    if (u > 0.f) {                       // concave piece [pa, pb]
        const float pa = fmaxf(l, 0.f), pb = u;
        rlo = fminf(rlo, fminf(glo(pa), glo(pb)));
        const float da = gp(pa), db = gp(pb);
        float mx;
        if (db >= GPS) mx = ghi(pb);              // increasing
        else if (da <= -GPS) mx = ghi(pa);        // decreasing
        else {
            const float xt = fminf(fmaxf(xs, pa), pb);
            const float s = __fadd_ru(fabsf(gp(xt)), GPS);
            mx = __fadd_ru(ghi(xt), __fmul_ru(s, __fsub_ru(pb, pa)));
            mx = fmaxf(mx, fmaxf(ghi(pa), ghi(pb)));
        }
        rhi = fmaxf(rhi, mx);
    }
    if (!(l < 0.f) && !(u > 0.f)) { rlo = fminf(glo(l), 0.f); rhi = fmaxf(ghi(l), 0.f); }  // l = u = 0
    r.b = 0.5f * (rlo + rhi);
    r.d = fmaxf(__fsub_ru(rhi, r.b), __fsub_ru(r.b, rlo));
    return r;
}

template <bool C>
__device__ __forceinline__ Lin linearize(int act, float l, float u) {
    if (act == NIQ_ACT_RELU) return lin_relu<C>(l, u);
    if (act == NIQ_ACT_ELU) return lin_elu<C>(l, u);
    return lin_tanh<C>(l, u);
}

__device__ __forceinline__ float act_point(int act, float x) {
    if (act == NIQ_ACT_RELU) return fmaxf(x, 0.f);
    if (act == NIQ_ACT_ELU) return elu_f(x);
    if (act == NIQ_ACT_TANH) return tanhf(x);
    return x;
}

// Derivative of the activation at x, given y = act(x), as JAX differentiates it:
// relu' = 1 where x > 0 else 0 (jax.nn.relu), elu' = 1 where x > 0 else exp(x)
// (jax.nn.elu), tanh' = 1 - tanh(x)^2.
__device__ __forceinline__ float act_deriv(int act, float x, float y) {
    if (act == NIQ_ACT_RELU) return x > 0.f ? 1.f : 0.f;
    if (act == NIQ_ACT_ELU) return x > 0.f ? 1.f : expf(x);
    if (act == NIQ_ACT_TANH) return __fsub_rn(1.f, __fmul_rn(y, y));
    return 1.f;
}

// Derivative bounds of the activation over [pl, pu] for slope intervals
// (src/slope_interval_layers.py:36-82); both are >= 0 for all three activations.
template <bool C>
__device__ __forceinline__ void slope_df(int act, float pl, float pu, float& dfl, float& dfu) {
    if (act == NIQ_ACT_RELU) {
        dfl = pl > 0.f ? 1.f : 0.f;
        dfu = pu < 0.f ? 0.f : 1.f;
    } else if (act == NIQ_ACT_ELU) {
        dfl = fminf(expf(pl), 1.f);
        dfu = fminf(expf(pu), 1.f);
        if (C) { dfl = fmaxf(__fmul_rd(dfl, 1.f - NIQ_FN_REL), 0.f); dfu = fminf(__fmul_ru(dfu, 1.f + NIQ_FN_REL), 1.f); }
    } else {
        const float tl = tanhf(pl), tu = tanhf(pu);
        float dl = 1.f - tl * tl, du = 1.f - tu * tu;
        if (C) {
            const float al = __fadd_ru(fabsf(tl), __fmaf_ru(fabsf(tl), NIQ_FN_REL, NIQ_FN_ABS));
            const float au = __fadd_ru(fabsf(tu), __fmaf_ru(fabsf(tu), NIQ_FN_REL, NIQ_FN_ABS));
            const float bl = fmaxf(__fsub_rd(fabsf(tl), __fmaf_ru(fabsf(tl), NIQ_FN_REL, NIQ_FN_ABS)), 0.f);
            const float bu = fmaxf(__fsub_rd(fabsf(tu), __fmaf_ru(fabsf(tu), NIQ_FN_REL, NIQ_FN_ABS)), 0.f);
            const float dl_lo = fmaxf(__fmaf_rd(-al, al, 1.f), 0.f), du_lo = fmaxf(__fmaf_rd(-au, au, 1.f), 0.f);
            const float dl_hi = fminf(__fmaf_ru(-bl, bl, 1.f), 1.f), du_hi = fminf(__fmaf_ru(-bu, bu, 1.f), 1.f);
            dfl = fminf(dl_lo, du_lo);
            dfu = (pl <= 0.f && pu >= 0.f) ? 1.f : fmaxf(dl_hi, du_hi);
            return;
        }
        dfl = fminf(dl, du);
        dfu = (pl <= 0.f && pu >= 0.f) ? 1.f : fmaxf(dl, du);
    }
}

// ----------------------------------------------------------------------------------
// Weight staging.  `sW` receives layer `l` (A then b) or, when the whole model is
// resident, already holds every layer at its global offset.
// ----------------------------------------------------------------------------------
__device__ __forceinline__ void stage_floats(float* __restrict__ dst, const float* __restrict__ src, int n) {
    // n is a multiple of 4 and both pointers are 16-byte aligned
    const float4* s4 = reinterpret_cast<const float4*>(src);
    float4* d4 = reinterpret_cast<float4*>(dst);
    for (int i = threadIdx.x; i < (n >> 2); i += blockDim.x) d4[i] = __ldg(s4 + i);
}

// Floats needed to hold one layer's weights (A then b).
NIQ_HOST_DEVICE int layer_floats(const NiqLayer& L) { return L.in_pad * L.out_pad + L.out_pad; }

// Per-thread accumulator tile: R rows x COLS columns, stored in column pairs when the
// dense loop uses packed FMAs (PK) and as plain floats otherwise.
template <int R, int COLS, bool PK>
struct AccTile {
    float v[R][COLS];
    __device__ __forceinline__ float& at(int r, int c) { return v[r][c]; }
};
template <int R, int COLS>
struct AccTile<R, COLS, true> {
    float2 v[R][COLS / 2];
    __device__ __forceinline__ float& at(int r, int c) { return (c & 1) ? v[r][c >> 1].y : v[r][c >> 1].x; }
    __device__ __forceinline__ float2& pair(int r, int c2) { return v[r][c2]; }
};

// ----------------------------------------------------------------------------------
// The fused forward pass.
//
// st   : shared state [ITEMS][R][LD]; the caller writes each item's input rows into
//        columns 0..3 (the input is 3-D; column 3 must be 0) and the err-type rows with
//        the first layer's fold already applied (see fold_input below).
// out  : shared [ITEMS][R]: column 0 of every row after the last layer (with bias and
//        error scaling applied); the caller interprets it (affine_out_bounds etc.).
// sW   : shared weight buffer.  If `resident`, it holds the model's whole weight area;
//        otherwise it must hold at least max_layer_floats floats and each layer is
//        staged in turn (chunked over k if it does not fit `sw_cap`).
// ----------------------------------------------------------------------------------
// WARP: the caller's warps work independently (their own items, weights resident): the
// pass then ends with a warp barrier, and `out` is visible to the item's own warp only.
template <class Cfg, bool C, bool WARP = false>
__device__ void tile_forward(const NiqSpecHeader& H, const float* __restrict__ gW, float* __restrict__ sW,
                             int sw_cap, bool resident, const RowPlan plan,
                             float* __restrict__ st, float* __restrict__ out) {
    constexpr int R = Cfg::R, NABS = Cfg::NABS, TPI = Cfg::TPI, COLS = Cfg::COLS, NQ = Cfg::NQ, LD = Cfg::LD;
    const int tid = threadIdx.x;
    const int item = tid / TPI;
    const int g = tid % TPI;
    float* xs = st + item * R * LD;
    const int nl = H.n_layers;

    for (int li = 0; li < nl; ++li) {
        const NiqLayer L = H.layers[li];
        const bool last = (li + 1 == nl);
        // accumulators; for bound rows in column pairs, which the dense loop updates with
        // one packed FMA (two correctly rounded fp32 FMAs in one instruction)
        AccTile<R, COLS, (NABS > 0)> acc;
#define ACC(r, c) acc.at(r, c)
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int c = 0; c < COLS; ++c) ACC(r, c) = 0.f;

        bool qv[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) qv[q] = col_of<TPI>(g, q) < L.out_pad;

        // A layer with a single 4-column group (the width-1 output layer): thread g of the
        // item sums a k-slice of all R rows x 4 columns, then the item's TPI lanes reduce
        // with shuffles, instead of one thread looping over all k while the others idle.
        const bool narrow = (L.out_pad == 4) && (TPI > 1) && (resident || L.in_pad * 4 + 4 <= sw_cap);
        if (narrow) {
            const float* A = sW + L.a_off;
            if (!resident) {
                __syncthreads();
                stage_floats(sW, gW + L.a_off, L.in_pad * 4);
                stage_floats(sW + (sw_cap - 4), gW + L.b_off, 4);
                __syncthreads();
                A = sW;
            }
            const int kg = L.in_pad >> 2;                       // k groups of 4
            constexpr int KS = Cfg::KSPLIT;                     // lanes g >= KS get no slice
            const int per = (kg + KS - 1) / KS;
            const int kb = min(kg, g * per), ke = min(kg, kb + per);
            for (int k4 = kb; k4 < ke; ++k4) {
                const int k = 4 * k4;
                float4 x[R];
#pragma unroll
                for (int r = 0; r < R; ++r) x[r] = *reinterpret_cast<const float4*>(xs + r * LD + k);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    const float4 av = *reinterpret_cast<const float4*>(A + (k + kk) * 4);
                    const float a[4] = {av.x, av.y, av.z, av.w};
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const float xv = kk == 0 ? x[r].x : kk == 1 ? x[r].y : kk == 2 ? x[r].z : x[r].w;
#pragma unroll
                        for (int c = 0; c < 4; ++c)
                            ACC(r, c) = fmaf(xv, r < R - NABS ? a[c] : fabsf(a[c]), ACC(r, c));
                    }
                }
            }
            // reduce over the item's lanes (TPI consecutive lanes of one warp); in the narrow
            // tile the first step adds the empty slices' zeros, exactly
#pragma unroll
            for (int off = TPI / 2; off > 0; off >>= 1)
#pragma unroll
                for (int r = 0; r < R; ++r)
#pragma unroll
                    for (int c = 0; c < 4; ++c) ACC(r, c) += __shfl_xor_sync(0xffffffffu, ACC(r, c), off);
            // lanes g > 0 now hold copies; only g == 0 owns column group 0 below
            if (g != 0) {
#pragma unroll
                for (int r = 0; r < R; ++r)
#pragma unroll
                    for (int c = 0; c < 4; ++c) ACC(r, c) = 0.f;
            }
        }

        // k-chunking when the layer is staged and does not fit the buffer
        const int row_floats = L.out_pad;
        int kc = L.in_pad;
        if (!resident) {
            const int cap_rows = (sw_cap - L.out_pad) / row_floats;
            kc = min(L.in_pad, (cap_rows / 4) * 4);
        }
        for (int k0 = 0; k0 < (narrow ? 0 : L.in_pad); k0 += kc) {
            const int k1 = min(L.in_pad, k0 + kc);
            const float* A;
            if (resident) {
                A = sW + L.a_off;
            } else {
                __syncthreads();  // previous chunk / layer fully consumed
                stage_floats(sW, gW + L.a_off + k0 * row_floats, (k1 - k0) * row_floats);
                if (k0 == 0) stage_floats(sW + (sw_cap - L.out_pad), gW + L.b_off, L.out_pad);
                __syncthreads();
                A = sW - k0 * row_floats;
            }
            for (int k = k0; k < k1; k += 4) {
                float4 x[R];
#pragma unroll
                for (int r = 0; r < R; ++r) x[r] = *reinterpret_cast<const float4*>(xs + r * LD + k);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    float a[COLS];
#pragma unroll
                    for (int q = 0; q < NQ; ++q) {
                        float4 av = qv[q] ? *reinterpret_cast<const float4*>(A + (k + kk) * row_floats + col_of<TPI>(g, q))
                                          : make_float4(0.f, 0.f, 0.f, 0.f);
                        a[4 * q + 0] = av.x; a[4 * q + 1] = av.y; a[4 * q + 2] = av.z; a[4 * q + 3] = av.w;
                    }
                    if constexpr (NABS == 1) {
                        // affine tiles: the signed rows with packed FMAs (issue-bound, so
                        // they pay for the pair rebuilt from each input value); the one
                        // |A| row with scalar FMAs, whose |.| is an operand modifier, where
                        // a packed form would need the absolute weights built first.  Each
                        // lane of a packed FMA is a correctly rounded fp32 FMA, so the
                        // results are those of scalar FMAs either way.
                        float2 w[COLS / 2];
#pragma unroll
                        for (int c = 0; c < COLS / 2; ++c) w[c] = make_float2(a[2 * c], a[2 * c + 1]);
#pragma unroll
                        for (int r = 0; r < R - 1; ++r) {
                            const float xv = kk == 0 ? x[r].x : kk == 1 ? x[r].y : kk == 2 ? x[r].z : x[r].w;
                            const float2 x2 = make_float2(xv, xv);
#pragma unroll
                            for (int c = 0; c < COLS / 2; ++c) acc.pair(r, c) = __ffma2_rn(x2, w[c], acc.pair(r, c));
                        }
                        {
                            const float xv = kk == 0 ? x[R - 1].x : kk == 1 ? x[R - 1].y : kk == 2 ? x[R - 1].z
                                                                                              : x[R - 1].w;
#pragma unroll
                            for (int c = 0; c < COLS; ++c) ACC(R - 1, c) = fmaf(xv, fabsf(a[c]), ACC(R - 1, c));
                        }
                    } else if constexpr (NABS > 0) {
                        // slope tiles (four |A| rows): packed FMAs, the absolute weights
                        // built once per input and shared by those rows
                        float2 w[COLS / 2], wa[COLS / 2];
#pragma unroll
                        for (int c = 0; c < COLS / 2; ++c) {
                            w[c] = make_float2(a[2 * c], a[2 * c + 1]);
                            wa[c] = make_float2(fabsf(a[2 * c]), fabsf(a[2 * c + 1]));
                        }
#pragma unroll
                        for (int r = 0; r < R; ++r) {
                            const float xv = kk == 0 ? x[r].x : kk == 1 ? x[r].y : kk == 2 ? x[r].z : x[r].w;
                            const float2 x2 = make_float2(xv, xv);
#pragma unroll
                            for (int c = 0; c < COLS / 2; ++c)
                                acc.pair(r, c) = __ffma2_rn(x2, r < R - NABS ? w[c] : wa[c], acc.pair(r, c));
                        }
                    } else {
                        // point rows only: plain FMAs (no pair to rebuild per input value)
#pragma unroll
                        for (int r = 0; r < R; ++r) {
                            const float xv = kk == 0 ? x[r].x : kk == 1 ? x[r].y : kk == 2 ? x[r].z : x[r].w;
#pragma unroll
                            for (int c = 0; c < COLS; ++c) ACC(r, c) = fmaf(xv, a[c], ACC(r, c));
                        }
                    }
                }
            }
        }
        const float* bsrc = resident ? (sW + L.b_off) : (sW + (sw_cap - L.out_pad));
        // All reads of the layer input are done before it is overwritten.  An item's state
        // is read and written only by its own TPI lanes, which share one warp; the shared
        // weight buffer has its own block barrier before every restage.
        __syncwarp();

        const float gam = C ? L.gamma : 0.f;
        const float gam_next = (C && !last) ? H.layers[li + 1].gamma : 0.f;
        const float scale = 1.f + 2.f * gam;
        const float tiny = (float)(L.in + 2) * NIQ_TINY;
        const int act = L.act;

        // Affine rows (and point rows) of an activated hidden layer: the same rules as
        // the general loop below, done in three passes over each group of 4 columns
        // (bounds, then the linearisations, then the updates), so that the branch-free
        // passes of different columns overlap instead of each column's chain running alone.
        constexpr bool AFFINE_TILE = (NABS == 1);
        const bool phased = AFFINE_TILE && plan.mode == ROWS_AFFINE && !last && act != NIQ_ACT_NONE;
        if (phased) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            if (!qv[q]) continue;
            float base4[4], err4[4], S4[4], lo4[4], hi4[4], b4[4];
            bool live4[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = 4 * q + j;
                const int col = col_of<TPI>(g, q) + j;
                live4[j] = col < L.out;
                const float b = live4[j] ? bsrc[col] : 0.f;
                b4[j] = b;
                base4[j] = __fadd_rn(ACC(0, c), b);
                float err = ACC(R - 1, c);
                if (C) err = __fadd_ru(__fmaf_ru(err, scale, __fmul_ru(gam, fabsf(b))), tiny);
                err4[j] = err;
                float S = 0.f;
#pragma unroll
                for (int r = 1; r < R - 1; ++r)
                    if (r <= plan.v) S = add_up<C>(S, fabsf(ACC(r, c)));
                S4[j] = S;
                const float rad = add_up<C>(S, err);
                lo4[j] = sub_dn<C>(base4[j], rad);
                hi4[j] = add_up<C>(base4[j], rad);
            }
            Lin z4[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) z4[j] = linearize<C>(act, lo4[j], hi4[j]);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = 4 * q + j;
                const Lin z = z4[j];
                float base = base4[j], err = err4[j];
                const float nb = C ? fmaf(z.a, base, z.b) : __fadd_rn(__fmul_rn(z.a, base), z.b);
#pragma unroll
                for (int r = 1; r < R - 1; ++r) {
                    if (r <= plan.v) ACC(r, c) = __fmul_rn(z.a, ACC(r, c));
                    else if (r <= plan.v + plan.np) ACC(r, c) = act_point(act, __fadd_rn(ACC(r, c), b4[j]));
                }
                if (C) {
                    const float aS = __fmul_ru(z.a, S4[j]);
                    err = __fmaf_ru(z.a, err, z.d);
                    err = __fmaf_ru(__fadd_ru(fabsf(nb), aS), NIQ_ULP_REL, err);
                    base = nb;
                    err = __fmaf_ru(gam_next, __fadd_ru(fabsf(base), __fmul_ru(aS, 1.f + NIQ_ULP_REL)), err);
                } else {
                    err = __fadd_rn(__fmul_rn(z.a, err), z.d);
                    base = nb;
                }
                ACC(0, c) = base;
                ACC(R - 1, c) = err;
                if (!live4[j]) {
#pragma unroll
                    for (int r = 0; r < R; ++r) ACC(r, c) = 0.f;
                }
            }
            const int col0 = col_of<TPI>(g, q);
#pragma unroll
            for (int r = 0; r < R; ++r)
                *reinterpret_cast<float4*>(xs + r * LD + col0) =
                    make_float4(ACC(r, 4 * q), ACC(r, 4 * q + 1), ACC(r, 4 * q + 2), ACC(r, 4 * q + 3));
        }
        } else {
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = 4 * q + j;
                const int col = col_of<TPI>(g, q) + j;
                if (!qv[q]) continue;
                const bool live = col < L.out;
                const float b = live ? bsrc[col] : 0.f;
                float v[R];
#pragma unroll
                for (int r = 0; r < R; ++r) v[r] = ACC(r, c);

                if (plan.mode == ROWS_POINTS) {
#pragma unroll
                    for (int r = 0; r < R; ++r) v[r] = act_point(act, __fadd_rn(v[r], b));
                } else if (NABS == 0 && plan.mode == ROWS_JVP) {
                    // value rows 0 and 4 get the bias and the activation; their tangent rows
                    // the activation's derivative at the pre-activation
#pragma unroll
                    for (int p0 = 0; p0 + 3 < R; p0 += 4) {
                        const float pre = __fadd_rn(v[p0], b);
                        const float y = act_point(act, pre);
                        const float d = act_deriv(act, pre, y);
                        v[p0] = y;
#pragma unroll
                        for (int r = p0 + 1; r < p0 + 4; ++r) v[r] = __fmul_rn(d, v[r]);
                    }
                } else if (plan.mode == ROWS_AFFINE) {
                    float base = __fadd_rn(v[0], b);
                    float err = v[R - 1];
                    if (C) err = __fadd_ru(__fmaf_ru(err, scale, __fmul_ru(gam, fabsf(b))), tiny);
                    // point rows
#pragma unroll
                    for (int r = 1; r < R - 1; ++r)
                        if (r > plan.v && r <= plan.v + plan.np) v[r] = act_point(act, __fadd_rn(v[r], b));
                    if (act != NIQ_ACT_NONE) {
                        float S = 0.f;
#pragma unroll
                        for (int r = 1; r < R - 1; ++r)
                            if (r <= plan.v) S = add_up<C>(S, fabsf(v[r]));
                        const float rad = add_up<C>(S, err);
                        const float lo = sub_dn<C>(base, rad), hi = add_up<C>(base, rad);
                        const Lin z = linearize<C>(act, lo, hi);
                        const float nb = C ? fmaf(z.a, base, z.b) : __fadd_rn(__fmul_rn(z.a, base), z.b);
#pragma unroll
                        for (int r = 1; r < R - 1; ++r)
                            if (r <= plan.v) v[r] = __fmul_rn(z.a, v[r]);
                        if (C) {
                            const float aS = __fmul_ru(z.a, S);
                            err = __fmaf_ru(z.a, err, z.d);
                            err = __fmaf_ru(__fadd_ru(fabsf(nb), aS), NIQ_ULP_REL, err);
                            base = nb;
                            // fold the next layer's dot-product rounding into err
                            err = __fmaf_ru(gam_next, __fadd_ru(fabsf(base), __fmul_ru(aS, 1.f + NIQ_ULP_REL)), err);
                        } else {
                            err = __fadd_rn(__fmul_rn(z.a, err), z.d);
                            base = nb;
                        }
                    } else if (C && !last) {
                        float S = 0.f;
#pragma unroll
                        for (int r = 1; r < R - 1; ++r)
                            if (r <= plan.v) S = __fadd_ru(S, fabsf(v[r]));
                        err = __fmaf_ru(gam_next, __fadd_ru(fabsf(base), S), err);
                    }
                    v[0] = base;
                    v[R - 1] = err;
                } else {  // ROWS_SLOPE: 0 primal | 1..v centers | points | 4 perr | 5..4+v widths
                    float primal = __fadd_rn(v[0], b);
                    float perr = v[4];
                    if (C) {
                        perr = __fadd_ru(__fmaf_ru(perr, scale, __fmul_ru(gam, fabsf(b))), tiny);
#pragma unroll
                        for (int r = 5; r < R; ++r)
                            if (r - 4 <= plan.v) v[r] = __fadd_ru(__fmul_ru(v[r], scale), tiny);
                    }
#pragma unroll
                    for (int r = 1; r < 4; ++r)
                        if (r > plan.v && r <= plan.v + plan.np) v[r] = act_point(act, __fadd_rn(v[r], b));
                    if (act != NIQ_ACT_NONE) {
                        // primal bounds from the slope bounds (src/slope_interval.py:205-210)
                        float rad = 0.f;
#pragma unroll
                        for (int r = 1; r < 4; ++r)
                            if (r <= plan.v) {
                                const float sl = sub_dn<C>(v[r], v[r + 4]), su = add_up<C>(v[r], v[r + 4]);
                                rad = add_up<C>(rad, fmaxf(su, -sl));
                            }
                        if (C) rad = __fadd_ru(rad, perr);
                        const float pl = sub_dn<C>(primal, rad), pu = add_up<C>(primal, rad);
                        float dfl, dfu;
                        slope_df<C>(act, pl, pu, dfl, dfu);
#pragma unroll
                        for (int r = 1; r < 4; ++r)
                            if (r <= plan.v) {
                                const float sl = sub_dn<C>(v[r], v[r + 4]), su = add_up<C>(v[r], v[r + 4]);
                                float nl, nu;
                                if (C) {
                                    nl = fminf(__fmul_rd(sl, dfl), __fmul_rd(sl, dfu));
                                    nu = fmaxf(__fmul_ru(su, dfl), __fmul_ru(su, dfu));
                                } else {
                                    nl = fminf(__fmul_rn(sl, dfl), __fmul_rn(sl, dfu));
                                    nu = fmaxf(__fmul_rn(su, dfl), __fmul_rn(su, dfu));
                                }
                                const float cc = __fmul_rn(0.5f, __fadd_rn(nl, nu));
                                v[r] = cc;
                                v[r + 4] = C ? fmaxf(__fsub_ru(nu, cc), __fsub_ru(cc, nl)) : __fsub_rn(nu, cc);
                            }
                        const float np_ = act_point(act, primal);
                        if (C) perr = __fadd_ru(perr, __fmaf_ru(fabsf(np_), NIQ_FN_REL, NIQ_FN_ABS));
                        primal = np_;
                    }
                    if (C && !last) {
                        perr = __fmaf_ru(gam_next, fabsf(primal), perr);
#pragma unroll
                        for (int r = 5; r < R; ++r)
                            if (r - 4 <= plan.v) v[r] = __fmaf_ru(gam_next, fabsf(v[r - 4]), v[r]);
                    }
                    v[0] = primal;
                    v[4] = perr;
                }
                if (!live) {
#pragma unroll
                    for (int r = 0; r < R; ++r) v[r] = 0.f;
                }
                if (last) {
                    if (col == 0) {
#pragma unroll
                        for (int r = 0; r < R; ++r) out[item * R + r] = v[r];
                    }
                } else {
#pragma unroll
                    for (int r = 0; r < R; ++r) ACC(r, c) = v[r];
                }
            }
            // one 16-byte store per row for the thread's 4 columns (scalar stores of
            // 4 strided columns conflicted on the shared-memory banks)
            if (!last && qv[q]) {
                const int col0 = col_of<TPI>(g, q);
#pragma unroll
                for (int r = 0; r < R; ++r)
                    *reinterpret_cast<float4*>(xs + r * LD + col0) =
                        make_float4(ACC(r, 4 * q), ACC(r, 4 * q + 1), ACC(r, 4 * q + 2), ACC(r, 4 * q + 3));
            }
        }
        }  // general epilogue
        // layer output visible before the next layer reads it (the item's own warp), and
        // after the last layer, every item's `out` row visible to the whole block
        if (last && !WARP) __syncthreads();
        else __syncwarp();
#undef ACC
    }
}

// First-layer fold of dot-product rounding into the |A| rows of an affine item whose
// rows 0..R-1 (columns 0..2) are already written.  Called by the thread owning the
// item's column k (k < 3).
template <int R>
__device__ __forceinline__ void fold_input_affine(float* xs, int LD, int v, float gamma0, int k) {
    float S = fabsf(xs[k]);
    for (int r = 1; r <= v; ++r) S = __fadd_ru(S, fabsf(xs[r * LD + k]));
    xs[(R - 1) * LD + k] = __fmaf_ru(gamma0, S, xs[(R - 1) * LD + k]);
}

// Bounds of the scalar output of an affine item (src/affine.py:85-91,119-125).
template <int R, bool C>
__device__ __forceinline__ void affine_out_bounds(const float* o, int v, float& lo, float& hi) {
    float S = 0.f;
    for (int r = 1; r <= v; ++r) S = add_up<C>(S, fabsf(o[r]));
    const float rad = add_up<C>(S, o[R - 1]);
    lo = sub_dn<C>(o[0], rad);
    hi = add_up<C>(o[0], rad);
}

// Bounds of the scalar output of a slope item (src/slope_interval.py:200-210).
template <bool C>
__device__ __forceinline__ void slope_out_bounds(const float* o, int v, float& lo, float& hi) {
    float rad = 0.f;
    for (int r = 1; r <= v; ++r) {
        const float sl = sub_dn<C>(o[r], o[r + 4]), su = add_up<C>(o[r], o[r + 4]);
        rad = add_up<C>(rad, fmaxf(su, -sl));
    }
    if (C) rad = __fadd_ru(rad, o[4]);
    lo = sub_dn<C>(o[0], rad);
    hi = add_up<C>(o[0], rad);
}

__device__ __forceinline__ int sign_of_bounds(float lo, float hi, float offset) {
    int s = NIQ_SIGN_UNKNOWN;
    if (lo > offset) s = NIQ_SIGN_POSITIVE;
    if (hi < -offset) s = NIQ_SIGN_NEGATIVE;
    return s;
}

}  // namespace niq
