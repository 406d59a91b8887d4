// k_eval.cu -- point evaluation and box classification over caller-given batches.
//
// niq_eval_points      : ImplicitFunction.__call__ (src/affine.py:26-28) for N points.
// niq_eval_gradients   : value and gradient at N points (jax.jacfwd, src/render.py:61-63).
// niq_classify_boxes   : classify_general_box (src/affine.py:34-55,
//                        src/slope_interval.py:29-51) for N general boxes.
// Both are persistent grid-stride kernels over CTA tiles of the fused tile engine.
#include "niq_host.cuh"
#include "wide_engine.cuh"

namespace niq {

// ---------------------------------------------------------------- point evaluation
template <int TPI>
__global__ void __launch_bounds__(kNT) k_eval_points(NiqModelRef M, long long n, const float* __restrict__ xyz,
                                                     float* __restrict__ out, int fixed_floats, int sw_cap,
                                                     int resident) {
    using Cfg = TileCfg<8, 0, TPI, kNT>;
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    float* st = smem;
    float* o = st + Cfg::STATE_FLOATS;
    float* sW = smem + fixed_floats;
    __shared__ NiqSpecHeader H;
    load_header(H, M.hdr);
    __syncthreads();
    if (resident) stage_floats(sW, M.w, H.n_weight_floats);
    const RowPlan plan{ROWS_POINTS, 0, 8};
    const int item = threadIdx.x / TPI, g = threadIdx.x % TPI;
    const long long per_tile = (long long)Cfg::ITEMS * 8;
    for (long long tile = blockIdx.x; tile * per_tile < n; tile += gridDim.x) {
        float* xs = st + item * Cfg::R * Cfg::LD;
        for (int r = g; r < 8; r += TPI) {
            const long long p = tile * per_tile + item * 8 + r;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (p < n) { v.x = xyz[3 * p]; v.y = xyz[3 * p + 1]; v.z = xyz[3 * p + 2]; }
            *reinterpret_cast<float4*>(xs + r * Cfg::LD) = v;
        }
        __syncthreads();
        tile_forward<Cfg, false>(H, M.w, sW, sw_cap, resident, plan, st, o);
        for (int r = g; r < 8; r += TPI) {
            const long long p = tile * per_tile + item * 8 + r;
            if (p < n) out[p] = o[item * 8 + r];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- gradients
// Forward-mode derivatives: an item holds two points, each a value row and the three
// tangent rows d/dx, d/dy, d/dz (input: the point and the unit vectors), which the dense
// rule multiplies by A and the activation by its derivative at the pre-activation.
template <int TPI>
__global__ void __launch_bounds__(kNT) k_eval_grad(NiqModelRef M, long long n, const float* __restrict__ xyz,
                                                   float* __restrict__ val, float* __restrict__ grad,
                                                   int fixed_floats, int sw_cap, int resident) {
    using Cfg = TileCfg<8, 0, TPI, kNT>;
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    float* st = smem;
    float* o = st + Cfg::STATE_FLOATS;
    float* sW = smem + fixed_floats;
    __shared__ NiqSpecHeader H;
    load_header(H, M.hdr);
    __syncthreads();
    if (resident) stage_floats(sW, M.w, H.n_weight_floats);
    const RowPlan plan{ROWS_JVP, 0, 0};
    const int item = threadIdx.x / TPI, g = threadIdx.x % TPI;
    const long long per_tile = (long long)Cfg::ITEMS * 2;
    for (long long tile = blockIdx.x; tile * per_tile < n; tile += gridDim.x) {
        float* xs = st + item * Cfg::R * Cfg::LD;
        for (int r = g; r < 8; r += TPI) {
            const long long p = tile * per_tile + item * 2 + r / 4;
            const int kind = r % 4;   // 0: the point, 1..3: the tangent of input kind - 1
            float4 v = make_float4(kind == 1 ? 1.f : 0.f, kind == 2 ? 1.f : 0.f, kind == 3 ? 1.f : 0.f, 0.f);
            if (kind == 0 && p < n) { v.x = xyz[3 * p]; v.y = xyz[3 * p + 1]; v.z = xyz[3 * p + 2]; }
            *reinterpret_cast<float4*>(xs + r * Cfg::LD) = v;
        }
        __syncthreads();
        tile_forward<Cfg, false>(H, M.w, sW, sw_cap, resident, plan, st, o);
        for (int r = g; r < 8; r += TPI) {
            const long long p = tile * per_tile + item * 2 + r / 4;
            const int kind = r % 4;
            if (p >= n) continue;
            if (kind == 0) { if (val) val[p] = o[item * 8 + r]; }
            else grad[3 * p + kind - 1] = o[item * 8 + r];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- box classification
// Builds an item's input rows for a general box (center, vecs[v]) in affine or slope
// layout (src/affine.py:109-117, src/slope_interval.py:192-197).  Threads g = 0..3 of
// the item each own input column g (column 3 is the zero pad).
template <class Cfg, bool C, bool SLOPE>
__device__ __forceinline__ void build_box_rows(float* xs, int g, bool valid, const float* c, const float* vv, int v,
                                               bool interval, float gamma0) {
    constexpr int LD = Cfg::LD, R = Cfg::R;
    if (g >= 4) return;
    const int k = g;
    for (int r = 0; r < R; ++r) xs[r * LD + k] = 0.f;
    if (!valid || k == 3) return;
    if (!SLOPE) {
        xs[k] = c[k];
        if (interval) {
            float e = 0.f;  // err = sum |vecs| (src/affine.py:111-113)
            for (int r = 0; r < v; ++r) e = add_up<C>(e, fabsf(vv[3 * r + k]));
            xs[(R - 1) * LD + k] = C ? __fmaf_ru(gamma0, fabsf(c[k]), e) : e;
        } else {
            float S = fabsf(c[k]);
            for (int r = 0; r < v; ++r) {
                xs[(1 + r) * LD + k] = vv[3 * r + k];
                S = __fadd_ru(S, fabsf(vv[3 * r + k]));
            }
            xs[(R - 1) * LD + k] = C ? __fmul_ru(gamma0, S) : 0.f;
        }
    } else {
        xs[k] = c[k];
        for (int r = 0; r < v; ++r) {
            xs[(1 + r) * LD + k] = vv[3 * r + k];
            xs[(5 + r) * LD + k] = C ? __fmul_ru(gamma0, fabsf(vv[3 * r + k])) : 0.f;
        }
        xs[4 * LD + k] = C ? __fmul_ru(gamma0, fabsf(c[k])) : 0.f;
    }
}

template <int TPI, bool C, bool SLOPE>
__global__ void __launch_bounds__(kNT) k_classify(NiqModelRef M, long long n, const float* __restrict__ center,
                                                  const float* __restrict__ vecs, int v, int interval, float offset,
                                                  int* __restrict__ sign_out, float* __restrict__ lohi_out,
                                                  int fixed_floats, int sw_cap, int resident) {
    using Cfg = typename std::conditional<SLOPE, TileCfg<8, 4, TPI, kNT>, TileCfg<5, 1, TPI, kNT>>::type;
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    float* st = smem;
    float* o = st + Cfg::STATE_FLOATS;
    float* sW = smem + fixed_floats;
    __shared__ NiqSpecHeader H;
    load_header(H, M.hdr);
    __syncthreads();
    if (resident) stage_floats(sW, M.w, H.n_weight_floats);
    const RowPlan plan{SLOPE ? ROWS_SLOPE : ROWS_AFFINE, interval ? 0 : v, 0};
    const int item = threadIdx.x / TPI, g = threadIdx.x % TPI;
    const float gamma0 = H.layers[0].gamma;
    for (long long tile = blockIdx.x; tile * Cfg::ITEMS < n; tile += gridDim.x) {
        const long long b = tile * Cfg::ITEMS + item;
        const bool valid = b < n;
        float* xs = st + item * Cfg::R * Cfg::LD;
        const float* c = valid ? center + 3 * b : center;
        const float* vv = valid ? vecs + 3 * v * b : vecs;
        build_box_rows<Cfg, C, SLOPE>(xs, g, valid, c, vv, v, interval != 0, gamma0);
        __syncthreads();
        tile_forward<Cfg, C>(H, M.w, sW, sw_cap, resident, plan, st, o);
        if (g == 0 && valid) {
            float lo, hi;
            if (SLOPE) slope_out_bounds<C>(o + item * Cfg::R, plan.v, lo, hi);
            else affine_out_bounds<Cfg::R, C>(o + item * Cfg::R, plan.v, lo, hi);
            sign_out[b] = sign_of_bounds(lo, hi, offset);
            if (lohi_out) { lohi_out[2 * b] = lo; lohi_out[2 * b + 1] = hi; }
        }
        __syncthreads();
    }
}

template <class K>
static int launch_tile_kernel(K kernel, int R, int TPI, const niq_model* m, long long work_tiles, cudaStream_t s,
                              SmemPlan& p, int& grid) {
    const int items = kNT / TPI;
    const int W = TPI * 8;
    const int state = items * R * (W + 4) + ((items * R + 3) & ~3);
    p = plan_smem(state, m->hdr.n_weight_floats, max_layer_floats(m->hdr), smem_budget(kernel, kNT));
    int rc = prepare_kernel(kernel, p.bytes);
    if (rc) return rc;
    return persistent_grid(kernel, kNT, p.bytes, work_tiles, &grid);
}

}  // namespace niq

using namespace niq;

extern "C" {

int niq_eval_points(const niq_model* model, int64_t n, const float* xyz, float* out, void* stream) {
    NIQ_REQUIRE(model && (n == 0 || (xyz && out)), NIQ_ERR_INVALID_ARG, "null argument");
    NIQ_REQUIRE(n >= 0, NIQ_ERR_INVALID_ARG, "negative count");
    if (n == 0) return NIQ_OK;
    const int tpi = tpi_for_width(model->hdr.max_width);
    cudaStream_t s = as_stream(stream);
    int rc = NIQ_OK;
    NIQ_DISPATCH_TPI(tpi, {
        auto kern = k_eval_points<TPI>;
        SmemPlan p;
        int grid = 0;
        const long long tiles = (n + (kNT / TPI) * 8 - 1) / ((kNT / TPI) * 8);
        rc = launch_tile_kernel(kern, 8, TPI, model, tiles, s, p, grid);
        if (rc) return rc;
        kern<<<grid, kNT, p.bytes, s>>>(model->ref(), n, xyz, out, p.fixed_floats, p.sw_cap, p.resident);
    });
    NIQ_CUDA(cudaGetLastError());
    return rc;
}

int niq_eval_gradients(const niq_model* model, int64_t n, const float* xyz, float* val_out, float* grad_out,
                       void* stream) {
    NIQ_REQUIRE(model && (n == 0 || (xyz && grad_out)), NIQ_ERR_INVALID_ARG, "null argument");
    NIQ_REQUIRE(n >= 0, NIQ_ERR_INVALID_ARG, "negative count");
    if (n == 0) return NIQ_OK;
    const int tpi = tpi_for_width(model->hdr.max_width);
    cudaStream_t s = as_stream(stream);
    int rc = NIQ_OK;
    NIQ_DISPATCH_TPI(tpi, {
        auto kern = k_eval_grad<TPI>;
        SmemPlan p;
        int grid = 0;
        const long long tiles = (n + (kNT / TPI) * 2 - 1) / ((kNT / TPI) * 2);
        rc = launch_tile_kernel(kern, 8, TPI, model, tiles, s, p, grid);
        if (rc) return rc;
        kern<<<grid, kNT, p.bytes, s>>>(model->ref(), n, xyz, val_out, grad_out, p.fixed_floats, p.sw_cap, p.resident);
    });
    NIQ_CUDA(cudaGetLastError());
    return rc;
}

size_t niq_classify_workspace_size(const niq_model* model, const niq_bound_opts* opts, int64_t n, int32_t v) {
    if (!model || !opts) return 0;
    if (opts->mode == NIQ_MODE_AFFINE_FIXED || opts->mode == NIQ_MODE_INTERVAL || opts->mode == NIQ_MODE_SLOPE_INTERVAL)
        return 0;
    return wide_workspace_bytes(model->hdr, *opts, v);
}

int niq_classify_boxes(const niq_model* model, const niq_bound_opts* opts, int64_t n, const float* center,
                       const float* vecs, int32_t v, float offset, int32_t* sign_out, float* lo_hi_out,
                       void* workspace, size_t workspace_bytes, void* stream) {
    NIQ_REQUIRE(model && opts, NIQ_ERR_INVALID_ARG, "null argument");
    NIQ_REQUIRE(n >= 0 && v >= 1 && v <= 3, NIQ_ERR_INVALID_ARG, "need n >= 0 and 1 <= v <= 3 (v=%d)", v);
    NIQ_REQUIRE(n == 0 || (center && vecs && sign_out), NIQ_ERR_INVALID_ARG, "null array");
    if (n == 0) return NIQ_OK;
    cudaStream_t s = as_stream(stream);
    const int mode = opts->mode;
    if (mode != NIQ_MODE_AFFINE_FIXED && mode != NIQ_MODE_INTERVAL && mode != NIQ_MODE_SLOPE_INTERVAL)
        return wide_classify(model, *opts, n, center, vecs, v, offset, sign_out, lo_hi_out, workspace, workspace_bytes, s);
    const int tpi = tpi_for_width(model->hdr.max_width);
    const bool slope = mode == NIQ_MODE_SLOPE_INTERVAL;
    const bool cons = opts->conservative != 0;
    const int interval = mode == NIQ_MODE_INTERVAL;
    int rc = NIQ_OK;
#define NIQ_LAUNCH_CLASSIFY(CC, SL)                                                                          \
    NIQ_DISPATCH_TPI(tpi, {                                                                                  \
        auto kern = k_classify<TPI, CC, SL>;                                                                 \
        SmemPlan p;                                                                                          \
        int grid = 0;                                                                                        \
        const long long tiles = (n + kNT / TPI - 1) / (kNT / TPI);                                           \
        rc = launch_tile_kernel(kern, SL ? 8 : 5, TPI, model, tiles, s, p, grid);                            \
        if (rc) return rc;                                                                                   \
        kern<<<grid, kNT, p.bytes, s>>>(model->ref(), n, center, vecs, v, interval, offset, sign_out,        \
                                        lo_hi_out, p.fixed_floats, p.sw_cap, p.resident);                    \
    })
    if (slope) {
        if (cons) { NIQ_LAUNCH_CLASSIFY(true, true); } else { NIQ_LAUNCH_CLASSIFY(false, true); }
    } else {
        if (cons) { NIQ_LAUNCH_CLASSIFY(true, false); } else { NIQ_LAUNCH_CLASSIFY(false, false); }
    }
#undef NIQ_LAUNCH_CLASSIFY
    NIQ_CUDA(cudaGetLastError());
    return rc;
}

}  // extern "C"
