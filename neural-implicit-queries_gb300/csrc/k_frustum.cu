// k_frustum.cu -- queries.cast_rays_frustum (src/queries.py:178-587) on the GPU.
//
// A frustum is an integer pixel range [x0, x1) x [y0, y1) of the image marching like a
// ray along its central direction.  Per step (src/queries.py:202-267), for each function:
//   the box enclosing the frustum between t and the step's end (center plus three
//   vectors: along the central ray, and the half extents across and up at the far end)
//   is classified; the step is safe when every function is POSITIVE or NEGATIVE; the
//   sign test at t and t + hit_eps along the central ray detects a hit.
// After n_substeps steps a frustum terminates on a hit (single pixels only), t > max_dist
// or the global step count; a frustum whose step has fallen behind its width (or that
// demands it) splits in half along its wider pixel axis (src/queries.py:340-467).
// Finished frusta write their t, hit_id and count to every pixel they cover
// (src/queries.py:469-587).
//
// One launch per iteration over the live list (the reference's loop: survivors and
// children append to the next list, finished frusta to the result list) and one device
// to host count read.  The bound and the two hit-test points of a step share one fused
// forward pass for 'interval' and 'affine_fixed' (8 rows: center, three vectors, two
// points, err); 'slope_interval' uses a bound pass and a point pass.
#include <cmath>
#include <vector>
#include "cast_common.cuh"
#include "wide_engine.cuh"

namespace niq {

struct FrustCam {
    float root[3], look[3], up[3], left[3];
    float tan_x, tan_y;      // tan(deg2rad(fov) / 2)
    float half_x, half_y;    // deg2rad(fov) / 2
    float rx1, ry1;          // res + 1
    int res_x, res_y;
};

struct FrustWs {
    unsigned long long n_next;  // live frusta appended this iteration
    unsigned long long n_fin;   // finished frusta
    int err;
    int pad;
};

struct FrustList {
    int4* rng;      // x0, y0, x1, y1
    float* t;
    float* size;
    float* count;
};

// src/render.py:17-23: normalize(look + left (a tan_x) + up (b tan_y)), float32 op by op
__device__ __forceinline__ void frust_ray(const FrustCam& c, float a, float b, float* r) {
    const float sa = __fmul_rn(a, c.tan_x), sb = __fmul_rn(b, c.tan_y);
    float p[3];
    for (int k = 0; k < 3; ++k) p[k] = __fadd_rn(__fadd_rn(c.look[k], __fmul_rn(c.left[k], sa)), __fmul_rn(c.up[k], sb));
    const float n = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(p[0], p[0]), __fmul_rn(p[1], p[1])), __fmul_rn(p[2], p[2])));
    for (int k = 0; k < 3; ++k) r[k] = __fdiv_rn(p[k], n);
}

template <int TPI, bool C, bool SLOPE>
__global__ void __launch_bounds__(kNT) k_frust(ModelSet S, int mode_interval, FrustCam cam, CastDev o, float refine_fac,
                                               int iter, FrustList in, long long n_live, FrustList out, FrustList fin,
                                               int* __restrict__ fin_hit, FrustWs* ws, long long cap,
                                               unsigned long long* __restrict__ n_evals, int fixed_floats, int sw_cap,
                                               int resident) {
    // affine/interval: one pass of 8 rows; slope: 8-row bound pass, then an 8-row point pass
    using CB = typename std::conditional<SLOPE, TileCfg<8, 4, TPI, kNT>, TileCfg<8, 1, TPI, kNT>>::type;
    using CP = TileCfg<8, 0, TPI, kNT>;
    constexpr int ITEMS = CB::ITEMS, R = CB::R, LD = CB::LD;
    static_assert(CP::ITEMS == ITEMS && CP::LD == LD, "same tile");
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    float* st = smem;
    float* ob = st + CB::STATE_FLOATS;
    float* sW = smem + fixed_floats;
    __shared__ NiqSpecHeader H;
    __shared__ int4 s_rng[ITEMS];
    __shared__ float s_t[ITEMS], s_size[ITEMS], s_count[ITEMS], s_expand[ITEMS];
    __shared__ float s_mid[ITEMS][3], s_d1[ITEMS][3], s_d2[ITEMS][3];
    __shared__ int s_alive[ITEMS], s_single[ITEMS], s_hit[ITEMS], s_hitid[ITEMS], s_can[ITEMS], s_steps[ITEMS];
    __shared__ int s_act[ITEMS], s_demand[ITEMS];
    __shared__ unsigned long long s_evals[kMaxFuncs];

    const int item = threadIdx.x / TPI, g = threadIdx.x % TPI;
    if (threadIdx.x < kMaxFuncs) s_evals[threadIdx.x] = 0ull;
    if (resident)
        for (int f = 0; f < S.n; ++f) {
            load_header(H, S.m[f].hdr);
            __syncthreads();
            stage_floats(sW + S.woff[f], S.m[f].w, H.n_weight_floats);
            __syncthreads();
        }
    if (S.n == 1) load_header(H, S.m[0].hdr);
    const int v = mode_interval ? 0 : 3;
    const RowPlan pb{SLOPE ? ROWS_SLOPE : ROWS_AFFINE, v, SLOPE ? 0 : 2};
    const RowPlan pp{ROWS_POINTS, 0, 8};
    const int rp0 = SLOPE ? 0 : v + 1;   // rows of the two points (in the point pass for slope)

    for (long long base = (long long)blockIdx.x * ITEMS; base < n_live; base += (long long)gridDim.x * ITEMS) {
        if (g == 0) {
            const long long id = base + item;
            s_alive[item] = id < n_live;
            if (id < n_live) {
                const int4 rg = in.rng[id];
                s_rng[item] = rg;
                s_t[item] = in.t[id];
                s_size[item] = in.size[id];
                s_count[item] = in.count[id];
                // frustum geometry (src/queries.py:272-306)
                s_single[item] = (rg.x + 1 == rg.z) && (rg.y + 1 == rg.w);
                const float xl = __fsub_rn(__fdiv_rn(__fmul_rn(2.f, (float)rg.x), cam.rx1), 1.f);
                const float xu = __fsub_rn(__fdiv_rn(__fmul_rn(2.f, (float)(rg.z - 1)), cam.rx1), 1.f);
                const float yl = __fsub_rn(__fdiv_rn(__fmul_rn(2.f, (float)rg.y), cam.ry1), 1.f);
                const float yu = __fsub_rn(__fdiv_rn(__fmul_rn(2.f, (float)(rg.w - 1)), cam.ry1), 1.f);
                float uu[3], lu[3], ul[3], ll[3];
                frust_ray(cam, xu, yu, uu);
                frust_ray(cam, xl, yu, lu);
                frust_ray(cam, xu, yl, ul);
                frust_ray(cam, xl, yl, ll);
                float m[3];
                for (int k = 0; k < 3; ++k) m[k] = __fmul_rn(0.5f, __fadd_rn(uu[k], ll[k]));
                const float ml = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], m[0]), __fmul_rn(m[1], m[1])), __fmul_rn(m[2], m[2])));
                for (int k = 0; k < 3; ++k) {
                    s_mid[item][k] = __fdiv_rn(m[k], ml);
                    s_d1[item][k] = __fsub_rn(uu[k], lu[k]);
                    s_d2[item][k] = __fsub_rn(uu[k], ul[k]);
                }
                s_expand[item] = __fdiv_rn(1.f, ml);
            }
            s_hit[item] = 0;
            s_hitid[item] = 0;
            s_steps[item] = 0;
            s_demand[item] = 0;
        }
        __syncthreads();
        for (int sub = 0; sub < o.n_substeps; ++sub) {
            if (g == 0) {
                s_can[item] = !s_hit[item];
                s_act[item] = s_alive[item] && !s_hit[item];
                s_steps[item] += s_act[item] ? 1 : 0;
            }
            __syncthreads();
            for (int f = 0; f < S.n; ++f) {
                if (S.n > 1) load_header(H, S.m[f].hdr);
                const bool active = s_act[item];
                float* xs = st + item * R * LD;
                const float gam0 = C ? __ldg(&S.m[f].hdr->layers[0].gamma) : 0.f;
                float p0 = 0.f, p1 = 0.f;   // this thread's coordinate of the two points
                if (g < 4) {
                    const int k = g;
                    for (int r = 0; r < R; ++r) xs[r * LD + k] = 0.f;
                    if (active && k < 3) {
                        // src/queries.py:206-244
                        const float t = s_t[item], sz = s_size[item];
                        const float tadj = __fmul_rn(__fadd_rn(t, sz), s_expand[item]);
                        const float mk = s_mid[item][k], rt = cam.root[k];
                        const float rfr = __fdiv_rn(__fmul_rn(s_d1[item][k], tadj), 2.f);
                        const float ufr = __fdiv_rn(__fmul_rn(s_d2[item][k], tadj), 2.f);
                        const float cen = __fadd_rn(rt, __fmul_rn(__fmul_rn(0.5f, __fadd_rn(t, tadj)), mk));
                        const float cv = __fmul_rn(__fmul_rn(0.5f, __fsub_rn(tadj, t)), mk);
                        p0 = __fadd_rn(rt, __fmul_rn(t, mk));
                        p1 = __fadd_rn(rt, __fmul_rn(__fadd_rn(t, o.hit_eps), mk));
                        const float av = fabsf(cv), ar = fabsf(rfr), au = fabsf(ufr);
                        xs[k] = cen;
                        if (SLOPE) {
                            xs[1 * LD + k] = cv;
                            xs[2 * LD + k] = rfr;
                            xs[3 * LD + k] = ufr;
                            xs[4 * LD + k] = C ? __fmul_ru(gam0, fabsf(cen)) : 0.f;
                            xs[5 * LD + k] = C ? __fmul_ru(gam0, av) : 0.f;
                            xs[6 * LD + k] = C ? __fmul_ru(gam0, ar) : 0.f;
                            xs[7 * LD + k] = C ? __fmul_ru(gam0, au) : 0.f;
                        } else if (mode_interval) {
                            // src/affine.py:111-113: err = sum over the vectors of |vec|
                            const float e = C ? __fadd_ru(__fadd_ru(av, ar), au) : __fadd_rn(__fadd_rn(av, ar), au);
                            xs[(R - 1) * LD + k] = C ? __fmaf_ru(gam0, fabsf(cen), e) : e;
                            xs[(rp0) * LD + k] = p0;
                            xs[(rp0 + 1) * LD + k] = p1;
                        } else {
                            xs[1 * LD + k] = cv;
                            xs[2 * LD + k] = rfr;
                            xs[3 * LD + k] = ufr;
                            xs[(rp0) * LD + k] = p0;
                            xs[(rp0 + 1) * LD + k] = p1;
                            xs[(R - 1) * LD + k] =
                                C ? __fmul_ru(gam0, __fadd_ru(__fadd_ru(__fadd_ru(fabsf(cen), av), ar), au)) : 0.f;
                        }
                    }
                }
                __syncthreads();
                const int woff = resident ? S.woff[f] : 0;
                tile_forward<CB, C>(H, S.m[f].w, sW + woff, sw_cap, resident, pb, st, ob);
                int bt = NIQ_SIGN_UNKNOWN;
                if (g == 0 && active) {
                    float lo, hi;
                    if (SLOPE) slope_out_bounds<C>(ob + item * R, pb.v, lo, hi);
                    else affine_out_bounds<CB::R, C>(ob + item * R, pb.v, lo, hi);
                    bt = sign_of_bounds(lo, hi, 0.f);
                }
                float v0 = 0.f, v1 = 0.f;
                if (SLOPE) {
                    // point pass: rows 0 and 1 hold the two points
                    __syncthreads();
                    if (g < 4) {
                        for (int r = 0; r < R; ++r) xs[r * LD + g] = 0.f;
                        if (active && g < 3) { xs[g] = p0; xs[LD + g] = p1; }
                    }
                    __syncthreads();
                    tile_forward<CP, false>(H, S.m[f].w, sW + woff, sw_cap, resident, pp, st, ob);
                }
                if (g == 0 && active) {
                    v0 = ob[item * R + rp0];
                    v1 = ob[item * R + rp0 + 1];
                    if (bt == NIQ_SIGN_UNKNOWN) s_can[item] = 0;
                    const int sg0 = (v0 > 0.f) - (v0 < 0.f), sg1 = (v1 > 0.f) - (v1 < 0.f);
                    if ((v0 != v0) || (v1 != v1) || sg0 != sg1) { s_hitid[item] = f + 1; s_hit[item] = 1; }
                    atomicAdd(&s_evals[f], 1ull);
                }
                __syncthreads();
            }
            if (g == 0 && s_alive[item]) {
                // src/queries.py:249-267
                const bool can = s_can[item];
                const float sz = s_size[item];
                const float this_step = can ? sz : __fmul_rn(o.hit_eps, s_single[item] ? 1.f : 0.f);
                if (!s_hit[item]) s_t[item] = __fadd_rn(s_t[item], __fmul_rn(this_step, o.safety));
                const float ns = can ? __fmul_rn(sz, o.grow) : __fmul_rn(sz, o.shrink);
                if (ns < o.hit_eps || s_hit[item]) s_demand[item] = 1;
                s_size[item] = fmaxf(ns, o.hit_eps);
            }
            __syncthreads();
        }
        // ---- count, termination, refinement (src/queries.py:323-360)
        bool term = false, refine = false;
        int4 rg = make_int4(0, 0, 0, 0);
        if (g == 0 && s_alive[item]) {
            rg = s_rng[item];
            const int area = (rg.z - rg.x) * (rg.w - rg.y);
            s_count[item] = __fadd_rn(s_count[item], __fmul_rn((float)s_steps[item], __fdiv_rn(1.f, (float)area)));
            const bool hit = s_hit[item] && area == 1;
            term = hit || (s_t[item] > o.max_dist) || (iter >= o.n_max_step);
            if (!term) {
                const float t = s_t[item];
                const float wx = __fmul_rn(__fmul_rn(2.f, sinf(__fdiv_rn(__fmul_rn(cam.half_x, (float)(rg.z - rg.x)), (float)cam.res_x))), t);
                const float wy = __fmul_rn(__fmul_rn(2.f, sinf(__fdiv_rn(__fmul_rn(cam.half_y, (float)(rg.w - rg.y)), (float)cam.res_y))), t);
                const bool can_subd = (rg.z > rg.x + 1) || (rg.w > rg.y + 1);
                const float lim = __fmul_rn(refine_fac, s_size[item]);
                refine = can_subd && (wx > lim || wy > lim || s_demand[item]);
            }
        }
        const bool keep = (g == 0) && s_alive[item] && !term && !refine;
        const long long pf = niq_warp_reserve(&ws->n_fin, term, 1);
        const long long pk = niq_warp_reserve(&ws->n_next, keep, 1);
        const long long pr = niq_warp_reserve(&ws->n_next, refine, 2);
        if (term) {
            if (pf < cap) {
                fin.rng[pf] = rg;
                fin.t[pf] = s_t[item];
                fin.count[pf] = s_count[item];
                fin_hit[pf] = s_hitid[item];
            } else {
                niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
            }
        }
        if (keep) {
            if (pk < cap) {
                out.rng[pk] = rg;
                out.t[pk] = s_t[item];
                out.size[pk] = s_size[item];
                out.count[pk] = s_count[item];
            } else {
                niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
            }
        }
        if (refine) {
            if (pr + 1 < cap) {
                // split along the wider pixel axis at the floored midpoint (src/queries.py:409-467)
                const bool sx = (rg.z - rg.x) >= (rg.w - rg.y);
                const int xm = (rg.x + rg.z) / 2, ym = (rg.y + rg.w) / 2;
                const int4 a = make_int4(rg.x, rg.y, sx ? xm : rg.z, sx ? rg.w : ym);
                const int4 b = make_int4(sx ? xm : rg.x, sx ? rg.y : ym, rg.z, rg.w);
                out.rng[pr] = a;
                out.rng[pr + 1] = b;
                for (int q = 0; q < 2; ++q) {
                    out.t[pr + q] = s_t[item];
                    out.size[pr + q] = s_size[item];
                    out.count[pr + q] = s_count[item];
                }
            } else {
                niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
            }
        }
        __syncthreads();
    }
    __syncthreads();
    if (threadIdx.x < S.n && s_evals[threadIdx.x]) atomicAdd(&n_evals[threadIdx.x], s_evals[threadIdx.x]);
}

// ---------------------------------------------------------------- growing-term modes
// 'affine_truncate', 'affine_all', 'affine_append': each substep's boxes are bounded by
// the growing-term engine (wide_classify, v = 3) and the hit-test points by the point
// kernel, between per-frustum kernels that hold k_frust's arithmetic op by op.
struct WFrust {
    float* geo;    // per live frustum: mid[3], d1[3], d2[3], expand (10 floats)
    int* single;   // single-pixel frustum
    int* hit;      // hit flag, hit id, steps taken, demands subdivision
    int* hitid;
    int* steps;
    int* demand;
    float* center; // (n, 3) box centers
    float* vecs;   // (n, 3, 3): along the central ray, across, up
    float* pts;    // (n, 2, 3): the two hit-test points
    int* sign;     // (nfunc, n)
    float* vals;   // (nfunc, n, 2)
};

// Frustum geometry (src/queries.py:272-306) of every live frustum, state cleared.
__global__ void k_wfr_setup(FrustCam cam, FrustList in, long long n_live, WFrust W) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_live; i += (long long)gridDim.x * blockDim.x) {
        const int4 rg = in.rng[i];
        W.single[i] = (rg.x + 1 == rg.z) && (rg.y + 1 == rg.w);
        const float xl = __fsub_rn(__fdiv_rn(__fmul_rn(2.f, (float)rg.x), cam.rx1), 1.f);
        const float xu = __fsub_rn(__fdiv_rn(__fmul_rn(2.f, (float)(rg.z - 1)), cam.rx1), 1.f);
        const float yl = __fsub_rn(__fdiv_rn(__fmul_rn(2.f, (float)rg.y), cam.ry1), 1.f);
        const float yu = __fsub_rn(__fdiv_rn(__fmul_rn(2.f, (float)(rg.w - 1)), cam.ry1), 1.f);
        float uu[3], lu[3], ul[3], ll[3];
        frust_ray(cam, xu, yu, uu);
        frust_ray(cam, xl, yu, lu);
        frust_ray(cam, xu, yl, ul);
        frust_ray(cam, xl, yl, ll);
        float m[3];
        for (int k = 0; k < 3; ++k) m[k] = __fmul_rn(0.5f, __fadd_rn(uu[k], ll[k]));
        const float ml = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], m[0]), __fmul_rn(m[1], m[1])), __fmul_rn(m[2], m[2])));
        float* g = W.geo + 10 * i;
        for (int k = 0; k < 3; ++k) {
            g[k] = __fdiv_rn(m[k], ml);
            g[3 + k] = __fsub_rn(uu[k], lu[k]);
            g[6 + k] = __fsub_rn(uu[k], ul[k]);
        }
        g[9] = __fdiv_rn(1.f, ml);
        W.hit[i] = 0;
        W.hitid[i] = 0;
        W.steps[i] = 0;
        W.demand[i] = 0;
    }
}

// One substep's boxes and hit-test points (src/queries.py:206-244).
__global__ void k_wfr_prep(FrustCam cam, CastDev o, FrustList in, long long n_live, WFrust W) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_live; i += (long long)gridDim.x * blockDim.x) {
        const float* g = W.geo + 10 * i;
        const float t = in.t[i], sz = in.size[i];
        const float tadj = __fmul_rn(__fadd_rn(t, sz), g[9]);
        for (int k = 0; k < 3; ++k) {
            const float mk = g[k], rt = cam.root[k];
            const float rfr = __fdiv_rn(__fmul_rn(g[3 + k], tadj), 2.f);
            const float ufr = __fdiv_rn(__fmul_rn(g[6 + k], tadj), 2.f);
            const float cen = __fadd_rn(rt, __fmul_rn(__fmul_rn(0.5f, __fadd_rn(t, tadj)), mk));
            const float cv = __fmul_rn(__fmul_rn(0.5f, __fsub_rn(tadj, t)), mk);
            W.center[3 * i + k] = cen;
            W.vecs[9 * i + k] = cv;
            W.vecs[9 * i + 3 + k] = rfr;
            W.vecs[9 * i + 6 + k] = ufr;
            W.pts[6 * i + k] = __fadd_rn(rt, __fmul_rn(t, mk));
            W.pts[6 * i + 3 + k] = __fadd_rn(rt, __fmul_rn(__fadd_rn(t, o.hit_eps), mk));
        }
    }
}

// The substep's decisions from the signs and point values, then the step rule
// (src/queries.py:245-267), as k_frust takes them.
__global__ void k_wfr_update(CastDev o, FrustList in, long long n_live, int nfunc, WFrust W) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_live; i += (long long)gridDim.x * blockDim.x) {
        const bool hit_before = W.hit[i] != 0;
        bool can = !hit_before;
        bool hit = hit_before;
        int hid = W.hitid[i];
        if (!hit_before) {
            W.steps[i] += 1;
            for (int f = 0; f < nfunc; ++f) {
                if (W.sign[(long long)f * n_live + i] == NIQ_SIGN_UNKNOWN) can = false;
                const float v0 = W.vals[((long long)f * n_live + i) * 2], v1 = W.vals[((long long)f * n_live + i) * 2 + 1];
                const int sg0 = (v0 > 0.f) - (v0 < 0.f), sg1 = (v1 > 0.f) - (v1 < 0.f);
                if ((v0 != v0) || (v1 != v1) || sg0 != sg1) { hid = f + 1; hit = true; }
            }
        }
        const float sz = in.size[i];
        const float this_step = can ? sz : __fmul_rn(o.hit_eps, W.single[i] ? 1.f : 0.f);
        if (!hit) in.t[i] = __fadd_rn(in.t[i], __fmul_rn(this_step, o.safety));
        const float ns = can ? __fmul_rn(sz, o.grow) : __fmul_rn(sz, o.shrink);
        if (ns < o.hit_eps || hit) W.demand[i] = 1;
        in.size[i] = fmaxf(ns, o.hit_eps);
        W.hit[i] = hit;
        W.hitid[i] = hid;
    }
}

// Count, termination, refinement and the appends of one iteration (src/queries.py:323-467),
// as the tail of k_frust.  Every lane of a warp joins the warp-aggregated reservations.
__global__ void k_wfr_finish(FrustCam cam, CastDev o, float refine_fac, int iter, FrustList in, long long n_live,
                             FrustList out, FrustList fin, int* __restrict__ fin_hit, FrustWs* ws, long long cap,
                             WFrust W) {
    for (long long i0 = blockIdx.x * (long long)blockDim.x; i0 < n_live; i0 += (long long)gridDim.x * blockDim.x) {
        const long long i = i0 + threadIdx.x;
        bool term = false, refine = false;
        int4 rg = make_int4(0, 0, 0, 0);
        float cnt = 0.f, t = 0.f, sz = 0.f;
        if (i < n_live) {
            rg = in.rng[i];
            t = in.t[i];
            sz = in.size[i];
            const int area = (rg.z - rg.x) * (rg.w - rg.y);
            cnt = __fadd_rn(in.count[i], __fmul_rn((float)W.steps[i], __fdiv_rn(1.f, (float)area)));
            const bool hit = W.hit[i] && area == 1;
            term = hit || (t > o.max_dist) || (iter >= o.n_max_step);
            if (!term) {
                const float wx = __fmul_rn(__fmul_rn(2.f, sinf(__fdiv_rn(__fmul_rn(cam.half_x, (float)(rg.z - rg.x)), (float)cam.res_x))), t);
                const float wy = __fmul_rn(__fmul_rn(2.f, sinf(__fdiv_rn(__fmul_rn(cam.half_y, (float)(rg.w - rg.y)), (float)cam.res_y))), t);
                const bool can_subd = (rg.z > rg.x + 1) || (rg.w > rg.y + 1);
                const float lim = __fmul_rn(refine_fac, sz);
                refine = can_subd && (wx > lim || wy > lim || W.demand[i]);
            }
        }
        const bool keep = i < n_live && !term && !refine;
        const long long pf = niq_warp_reserve(&ws->n_fin, term, 1);
        const long long pk = niq_warp_reserve(&ws->n_next, keep, 1);
        const long long pr = niq_warp_reserve(&ws->n_next, refine, 2);
        if (term) {
            if (pf < cap) {
                fin.rng[pf] = rg;
                fin.t[pf] = t;
                fin.count[pf] = cnt;
                fin_hit[pf] = W.hitid[i];
            } else {
                niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
            }
        }
        if (keep) {
            if (pk < cap) {
                out.rng[pk] = rg;
                out.t[pk] = t;
                out.size[pk] = sz;
                out.count[pk] = cnt;
            } else {
                niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
            }
        }
        if (refine) {
            if (pr + 1 < cap) {
                const bool sx = (rg.z - rg.x) >= (rg.w - rg.y);
                const int xm = (rg.x + rg.z) / 2, ym = (rg.y + rg.w) / 2;
                out.rng[pr] = make_int4(rg.x, rg.y, sx ? xm : rg.z, sx ? rg.w : ym);
                out.rng[pr + 1] = make_int4(sx ? xm : rg.x, sx ? rg.y : ym, rg.z, rg.w);
                for (int q = 0; q < 2; ++q) {
                    out.t[pr + q] = t;
                    out.size[pr + q] = sz;
                    out.count[pr + q] = cnt;
                }
            } else {
                niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
            }
        }
    }
}

// Initial frusta: an n_side x n_side grid of pixel tiles (src/queries.py:506-517).
__global__ void k_frust_init(FrustList L, const int* xt, const int* yt, int ns, float init_size) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ns * ns) return;
    const int xi = i % ns, yi = i / ns;
    L.rng[i] = make_int4(xt[xi], yt[yi], xt[xi + 1], yt[yi + 1]);
    L.t[i] = 0.f;
    L.size[i] = init_size;
    L.count[i] = 0.f;
}

// Every pixel of a finished frustum takes its t, hit_id and count (the reference splits
// finished frusta down to single pixels, each inheriting them).  Outputs are [x][y].
__global__ void k_frust_fill(FrustList fin, const int* fin_hit, long long n_fin, int res_y, float* t_out, int* hit_out,
                             int* count_out) {
    for (long long i = blockIdx.x; i < n_fin; i += gridDim.x) {
        const int4 rg = fin.rng[i];
        const float t = fin.t[i];
        const int h = fin_hit[i];
        const int c = (int)fin.count[i];   // the reference stores the float count into an int array
        const int w = rg.w - rg.y, np = (rg.z - rg.x) * w;
        for (int p = threadIdx.x; p < np; p += blockDim.x) {
            const long long idx = (long long)(rg.x + p / w) * res_y + (rg.y + p % w);
            t_out[idx] = t;
            hit_out[idx] = h;
            count_out[idx] = c;
        }
    }
}

struct FrustLayout {
    size_t hdr, ticks, evals, list[3], hit, total;
    long long cap;
};

static FrustLayout frust_layout(int res_x, int res_y, int ns) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    FrustLayout L;
    L.cap = (long long)res_x * res_y;
    if (L.cap < (long long)ns * ns) L.cap = (long long)ns * ns;
    const size_t one = al(16 * L.cap) + 3 * al(4 * L.cap);
    L.hdr = 0;
    L.ticks = al(sizeof(FrustWs));
    L.evals = L.ticks + al(8 * (size_t)(ns + 1));
    size_t off = L.evals + al(8 * kMaxFuncs);
    for (int i = 0; i < 3; ++i) { L.list[i] = off; off += one; }
    L.hit = off;
    off += al(4 * L.cap);
    L.total = off + 256;
    return L;
}

static FrustList frust_list(char* base, size_t off, long long cap) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    FrustList L;
    L.rng = reinterpret_cast<int4*>(base + off);
    off += al(16 * cap);
    L.t = reinterpret_cast<float*>(base + off);
    off += al(4 * cap);
    L.size = reinterpret_cast<float*>(base + off);
    off += al(4 * cap);
    L.count = reinterpret_cast<float*>(base + off);
    return L;
}

// Extra workspace of the growing-term path: the per-frustum state and step buffers of up
// to `cap` live frusta, then the growing-term engine's own slots (the largest over the
// functions).
struct WFrustLayout {
    size_t geo, single, hit, hitid, steps, demand, center, vecs, pts, sign, vals, wide, total;
};

static WFrustLayout wfr_layout(const niq_model* const* models, int nfunc, const niq_bound_opts& o, long long cap,
                               size_t base) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    WFrustLayout W;
    const size_t n = (size_t)cap;
    W.geo = base;
    W.single = W.geo + al(40 * n);
    W.hit = W.single + al(4 * n);
    W.hitid = W.hit + al(4 * n);
    W.steps = W.hitid + al(4 * n);
    W.demand = W.steps + al(4 * n);
    W.center = W.demand + al(4 * n);
    W.vecs = W.center + al(12 * n);
    W.pts = W.vecs + al(36 * n);
    W.sign = W.pts + al(24 * n);
    W.vals = W.sign + al(4 * n * (size_t)nfunc);
    W.wide = W.vals + al(8 * n * (size_t)nfunc);
    size_t wmax = 0;
    for (int f = 0; f < nfunc; ++f)
        if (models && models[f]) {
            const size_t b = wide_workspace_bytes(models[f]->hdr, o, 3);
            wmax = wmax > b ? wmax : b;
        }
    W.total = W.wide + al(wmax) + 256;
    return W;
}

static int wfr_grid(long long n) {
    const long long g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

}  // namespace niq

using namespace niq;

extern "C" {

size_t niq_cast_frustum_growing_workspace_size(const niq_model* const* models, int32_t nfunc,
                                               const niq_bound_opts* opts, int32_t res_x, int32_t res_y,
                                               int32_t n_side_init) {
    if (!models || !opts || nfunc < 1 || nfunc > kMaxFuncs || res_x < 1 || res_y < 1 || n_side_init < 1) return 0;
    const FrustLayout FL = frust_layout(res_x, res_y, n_side_init);
    return wfr_layout(models, nfunc, *opts, FL.cap, FL.total).total;
}

size_t niq_cast_frustum_workspace_size(int32_t res_x, int32_t res_y, int32_t n_side_init) {
    if (res_x < 1 || res_y < 1 || n_side_init < 1) return 0;
    return frust_layout(res_x, res_y, n_side_init).total;
}

int niq_cast_frustum(const niq_model* const* models, int32_t nfunc, const niq_bound_opts* opts,
                     const niq_frustum_camera* camera, const niq_cast_opts* cast, float refine_width_fac,
                     int32_t n_side_init, float* t_out, int32_t* hit_id_out, int32_t* count_out, int64_t* n_evals_out,
                     void* workspace, size_t workspace_bytes, void* stream) {
    NIQ_REQUIRE(opts && camera && cast && t_out && hit_id_out && count_out && n_evals_out, NIQ_ERR_INVALID_ARG,
                "null argument");
    const int mode = opts->mode;
    const bool growing = mode == NIQ_MODE_AFFINE_TRUNCATE || mode == NIQ_MODE_AFFINE_ALL || mode == NIQ_MODE_AFFINE_APPEND;
    NIQ_REQUIRE(growing || mode == NIQ_MODE_AFFINE_FIXED || mode == NIQ_MODE_INTERVAL || mode == NIQ_MODE_SLOPE_INTERVAL,
                NIQ_ERR_UNSUPPORTED, "unknown bound mode %d", mode);
    const int rx = camera->res_x, ry = camera->res_y, ns = n_side_init;
    NIQ_REQUIRE(rx >= 1 && ry >= 1 && (long long)rx * ry < (1ll << 31), NIQ_ERR_INVALID_ARG, "bad resolution");
    NIQ_REQUIRE(ns >= 1 && ns <= rx && ns <= ry, NIQ_ERR_INVALID_ARG, "n_side_init must be in [1, min(res_x, res_y)]");
    NIQ_REQUIRE(cast->n_substeps >= 1 && cast->hit_eps > 0.f, NIQ_ERR_INVALID_ARG, "n_substeps >= 1 and hit_eps > 0 required");
    ModelSet S;
    int maxw, wfloats, maxlayer;
    int rc = make_set(models, nfunc, S, maxw, wfloats, maxlayer);
    if (rc) return rc;
    const FrustLayout FL = frust_layout(rx, ry, ns);
    const size_t need = growing ? wfr_layout(models, nfunc, *opts, FL.cap, FL.total).total : FL.total;
    NIQ_REQUIRE(workspace && workspace_bytes >= need, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed", need);
    cudaStream_t s = as_stream(stream);
    char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
    FrustWs* ws = reinterpret_cast<FrustWs*>(base + FL.hdr);
    int* ticks = reinterpret_cast<int*>(base + FL.ticks);
    FrustList lists[3] = {frust_list(base, FL.list[0], FL.cap), frust_list(base, FL.list[1], FL.cap),
                          frust_list(base, FL.list[2], FL.cap)};
    FrustList& fin = lists[2];
    int* fin_hit = reinterpret_cast<int*>(base + FL.hit);

    FrustCam cam;
    for (int k = 0; k < 3; ++k) {
        cam.root[k] = camera->root[k];
        cam.look[k] = camera->look[k];
        cam.up[k] = camera->up[k];
        cam.left[k] = camera->left[k];
    }
    // jnp.deg2rad multiplies by pi/180 in float32; then / 2 and tan, sin in float32
    const float d2r = (float)(3.14159265358979323846 / 180.0);
    cam.half_x = (camera->fov_x * d2r) / 2.f;
    cam.half_y = (camera->fov_y * d2r) / 2.f;
    cam.tan_x = (float)std::tan((double)cam.half_x);
    cam.tan_y = (float)std::tan((double)cam.half_y);
    cam.res_x = rx;
    cam.res_y = ry;
    cam.rx1 = (float)rx + 1.f;
    cam.ry1 = (float)ry + 1.f;
    const CastDev cd = to_dev(*cast);

    // initial tiles: jnp.linspace(0, res, n_side + 1, dtype=int), computed in float32
    NIQ_REQUIRE(ns <= 64, NIQ_ERR_INVALID_ARG, "n_side_init must be <= 64");
    int th[2 * 65];
    for (int a = 0; a < 2; ++a)
        for (int i = 0; i <= ns; ++i) {
            const float sv = (float)i / (float)ns;
            const float val = 0.f * (1.f - sv) + (float)(a == 0 ? rx : ry) * sv;
            th[a * (ns + 1) + i] = (int)val;
        }
    NIQ_CUDA(cudaMemsetAsync(ws, 0, sizeof(FrustWs), s));
    NIQ_CUDA(cudaMemcpyAsync(ticks, th, sizeof(int) * 2 * (ns + 1), cudaMemcpyHostToDevice, s));
    k_frust_init<<<(ns * ns + 255) / 256, 256, 0, s>>>(lists[0], ticks, ticks + ns + 1, ns, cd.init_step);
    NIQ_CUDA(cudaGetLastError());
    // per-function counts of bounded frustum steps
    unsigned long long* d_evals = reinterpret_cast<unsigned long long*>(base + FL.evals);
    NIQ_CUDA(cudaMemsetAsync(d_evals, 0, sizeof(unsigned long long) * kMaxFuncs, s));

    const bool cons = opts->conservative != 0;
    const bool slope = mode == NIQ_MODE_SLOPE_INTERVAL;
    const int interval = mode == NIQ_MODE_INTERVAL;
    const int tpi = tpi_for_width(maxw);
    long long steps_total = 0;
    auto run = [&](auto kern, int TPIv) -> int {
        const int items = kNT / TPIv;
        const int state = items * 8 * (TPIv * 8 + 4) + ((items * 8 + 3) & ~3);
        SmemPlan p = plan_smem(state, wfloats, maxlayer, smem_budget(kern, kNT));
        NIQ_REQUIRE(p.resident || p.sw_cap >= 5 * maxw, NIQ_ERR_UNSUPPORTED, "shared memory too small for width %d", maxw);
        int r2 = prepare_kernel(kern, p.bytes);
        if (r2) return r2;
        int grid_max = 0;
        r2 = persistent_grid(kern, kNT, p.bytes, (FL.cap + items - 1) / items, &grid_max);
        if (r2) return r2;
        long long n_live = (long long)ns * ns;
        int cur = 0, it = 0;
        while (n_live > 0) {
            NIQ_CUDA(cudaMemsetAsync(&ws->n_next, 0, sizeof(unsigned long long), s));
            const long long tiles = (n_live + items - 1) / items;
            const int grid = (int)(tiles < grid_max ? tiles : grid_max);
            kern<<<grid, kNT, p.bytes, s>>>(S, interval, cam, cd, refine_width_fac, it, lists[cur], n_live,
                                            lists[1 - cur], fin, fin_hit, ws, FL.cap, d_evals, p.fixed_floats,
                                            p.sw_cap, p.resident);
            NIQ_CUDA(cudaGetLastError());
            steps_total += n_live;
            unsigned long long next = 0;
            NIQ_CUDA(cudaMemcpyAsync(&next, &ws->n_next, sizeof(next), cudaMemcpyDeviceToHost, s));
            NIQ_CUDA(cudaStreamSynchronize(s));
            int err = 0;
            NIQ_CUDA(cudaMemcpyAsync(&err, &ws->err, sizeof(int), cudaMemcpyDeviceToHost, s));
            NIQ_CUDA(cudaStreamSynchronize(s));
            NIQ_REQUIRE(err == 0, err, "frustum kernel error %d", err);
            n_live = (long long)next;
            it += cast->n_substeps;
            cur = 1 - cur;
        }
        return NIQ_OK;
    };
    // the growing-term modes: per iteration the geometry, then per substep the boxes and
    // points, the growing-term engine and the point kernel per function, the step rule;
    // then the iteration's appends -- one host read of the live count per iteration
    auto run_growing = [&]() -> int {
        const WFrustLayout WL = wfr_layout(models, nfunc, *opts, FL.cap, FL.total);
        WFrust W;
        W.geo = reinterpret_cast<float*>(base + WL.geo);
        W.single = reinterpret_cast<int*>(base + WL.single);
        W.hit = reinterpret_cast<int*>(base + WL.hit);
        W.hitid = reinterpret_cast<int*>(base + WL.hitid);
        W.steps = reinterpret_cast<int*>(base + WL.steps);
        W.demand = reinterpret_cast<int*>(base + WL.demand);
        W.center = reinterpret_cast<float*>(base + WL.center);
        W.vecs = reinterpret_cast<float*>(base + WL.vecs);
        W.pts = reinterpret_cast<float*>(base + WL.pts);
        W.sign = reinterpret_cast<int*>(base + WL.sign);
        W.vals = reinterpret_cast<float*>(base + WL.vals);
        void* wws = base + WL.wide;
        const size_t wws_bytes = workspace_bytes - (size_t)(base - reinterpret_cast<char*>(workspace)) - WL.wide;
        long long n_live = (long long)ns * ns;
        int cur = 0, it = 0;
        while (n_live > 0) {
            NIQ_CUDA(cudaMemsetAsync(&ws->n_next, 0, sizeof(unsigned long long), s));
            const int blocks = wfr_grid(n_live);
            k_wfr_setup<<<blocks, 256, 0, s>>>(cam, lists[cur], n_live, W);
            NIQ_CUDA(cudaGetLastError());
            for (int sub = 0; sub < cd.n_substeps; ++sub) {
                k_wfr_prep<<<blocks, 256, 0, s>>>(cam, cd, lists[cur], n_live, W);
                NIQ_CUDA(cudaGetLastError());
                for (int f = 0; f < nfunc; ++f) {
                    int r2 = wide_classify(models[f], *opts, n_live, W.center, W.vecs, 3, 0.f,
                                           W.sign + (long long)f * n_live, nullptr, wws, wws_bytes, s);
                    if (r2) return r2;
                    r2 = niq_eval_points(models[f], 2 * n_live, W.pts, W.vals + (long long)f * 2 * n_live, s);
                    if (r2) return r2;
                }
                k_wfr_update<<<blocks, 256, 0, s>>>(cd, lists[cur], n_live, nfunc, W);
                NIQ_CUDA(cudaGetLastError());
            }
            k_wfr_finish<<<blocks, 256, 0, s>>>(cam, cd, refine_width_fac, it, lists[cur], n_live, lists[1 - cur], fin,
                                                fin_hit, ws, FL.cap, W);
            NIQ_CUDA(cudaGetLastError());
            steps_total += n_live;
            unsigned long long next = 0;
            int err = 0;
            NIQ_CUDA(cudaMemcpyAsync(&next, &ws->n_next, sizeof(next), cudaMemcpyDeviceToHost, s));
            NIQ_CUDA(cudaMemcpyAsync(&err, &ws->err, sizeof(int), cudaMemcpyDeviceToHost, s));
            NIQ_CUDA(cudaStreamSynchronize(s));
            NIQ_REQUIRE(err == 0, err, "frustum kernel error %d", err);
            n_live = (long long)next;
            it += cast->n_substeps;
            cur = 1 - cur;
        }
        return NIQ_OK;
    };
#define NIQ_FRUST(CC, SL) NIQ_DISPATCH_TPI(tpi, { rc = run(k_frust<TPI, CC, SL>, TPI); })
    if (growing) { rc = run_growing(); }
    else if (slope) { if (cons) { NIQ_FRUST(true, true); } else { NIQ_FRUST(false, true); } }
    else { if (cons) { NIQ_FRUST(true, false); } else { NIQ_FRUST(false, false); } }
#undef NIQ_FRUST
    if (rc) return rc;
    unsigned long long n_fin = 0;
    NIQ_CUDA(cudaMemcpyAsync(&n_fin, &ws->n_fin, sizeof(n_fin), cudaMemcpyDeviceToHost, s));
    NIQ_CUDA(cudaStreamSynchronize(s));
    if (n_fin > 0) {
        const int grid = (int)(n_fin < 4096 ? n_fin : 4096);
        k_frust_fill<<<grid, 256, 0, s>>>(fin, fin_hit, (long long)n_fin, ry, t_out, hit_id_out, count_out);
        NIQ_CUDA(cudaGetLastError());
    }
    const long long ev = steps_total;
    NIQ_CUDA(cudaMemcpyAsync(n_evals_out, &ev, sizeof(ev), cudaMemcpyHostToDevice, s));
    NIQ_CUDA(cudaStreamSynchronize(s));
    return NIQ_OK;
}

}  // extern "C"
