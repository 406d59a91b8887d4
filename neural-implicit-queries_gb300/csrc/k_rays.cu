// k_rays.cu -- queries.cast_rays (src/queries.py:39-175) on the GPU.
//
// Per ray and step (src/queries.py:44-92), for each function of funcs_tuple:
//   pos_start = root + t dir; half = 0.5 step dir; pos_mid = pos_start + half
//   box_type  = classify_general_box(pos_mid, [half])       (one noise row)
//   val_start = f(pos_start); val_eps = f(root + (t + hit_eps) dir)
//   hit when sign(val_start) != sign(val_eps)
// then t advances by step*safety when every function classified the segment, else by
// hit_eps*safety; step grows or shrinks and is clipped at hit_eps.  A ray terminates on
// a hit, t > max_dist or count >= n_max_step, checked after n_substeps steps
// (src/queries.py:113-120).
//
// The bound and the two point values of one step are three row groups of a single
// tile-engine item, so one fused forward pass serves all three.
//
// k_rays<PERSISTENT=true>: CTA slots refill from a global ray counter until every ray
// has terminated (one launch).  k_rays<PERSISTENT=false>: one reference iteration over a
// list of live rays, appending survivors to the next list (the plain form).
#include <vector>
#include "cast_common.cuh"
#include "wide_engine.cuh"

namespace niq {

struct RayWs {                      // device workspace header
    unsigned long long next_ray;    // persistent: next unclaimed ray
    unsigned long long n_live_next; // plain: survivors appended this iteration
    int err;
    int pad;
};

template <int TPI, int COLS, bool C, bool SLOPE, bool PERSISTENT>
__global__ void __launch_bounds__(kNT) k_rays(ModelSet S, int mode_interval, long long n, const float* __restrict__ roots,
                                               const float* __restrict__ dirs, CastDev o, float* __restrict__ t_out,
                                               int* __restrict__ hit_out, int* __restrict__ count_out,
                                               unsigned long long* __restrict__ n_evals, RayWs* ws,
                                               // plain-form state (full-size arrays indexed by ray id)
                                               float* __restrict__ st_t, float* __restrict__ st_step,
                                               int* __restrict__ st_count, const int* __restrict__ live_in,
                                               long long n_live, int* __restrict__ live_out,
                                               int fixed_floats, int sw_cap, int resident) {
    using Cfg = typename std::conditional<SLOPE, TileCfg<8, 4, TPI, kNT, COLS>, TileCfg<5, 1, TPI, kNT, COLS>>::type;
    constexpr int ITEMS = Cfg::ITEMS, R = Cfg::R, LD = Cfg::LD;
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    float* st = smem;
    float* ob = st + Cfg::STATE_FLOATS;
    float* sW = smem + fixed_floats;
    __shared__ NiqSpecHeader H;
    __shared__ long long s_id[ITEMS];
    __shared__ float s_t[ITEMS], s_step[ITEMS], s_root[ITEMS][3], s_dir[ITEMS][3];
    __shared__ int s_count[ITEMS], s_alive[ITEMS], s_hit[ITEMS], s_hitid[ITEMS], s_can[ITEMS], s_inner[ITEMS];
    __shared__ int s_act[ITEMS];   // evaluating in this substep: alive and not hit before it
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
    const RowPlan plan{SLOPE ? ROWS_SLOPE : ROWS_AFFINE, mode_interval ? 0 : 1, 2};
    // rows of the two points: affine v+1, v+2; slope 2, 3
    const int rp0 = SLOPE ? 2 : plan.v + 1;
    const int rerr = SLOPE ? 4 : R - 1;

    // ---- slot (re)fill by the owner thread of each item
    auto claim = [&](int it) {
        long long id = -1;
        if (PERSISTENT) {
            const unsigned long long k = atomicAdd(&ws->next_ray, 1ull);
            if ((long long)k < n) id = (long long)k;
        }
        s_id[it] = id;
        s_alive[it] = id >= 0;
        if (id >= 0) {
            s_t[it] = 0.f;
            s_step[it] = o.init_step;
            s_count[it] = 0;
            for (int k = 0; k < 3; ++k) { s_root[it][k] = roots[3 * id + k]; s_dir[it][k] = dirs[3 * id + k]; }
        }
    };
    long long tile_base = (long long)blockIdx.x * ITEMS;
    if (PERSISTENT) {
        if (g == 0) claim(item);
    }
    __syncthreads();

    // WM (warp mode): one function with its weights resident -- each warp steps its own
    // items with warp-level syncs only, refills its own slots and leaves when they are all
    // done, so warps whose rays ended free their issue slots for the others.  (An item's
    // threads share a warp.)  Otherwise the CTA steps in lock-step with block barriers.
    auto run = [&](auto wm_tag) {
    constexpr bool WM = decltype(wm_tag)::value;
    auto sync = [&]() {
        if constexpr (WM) __syncwarp();
        else __syncthreads();
    };
    while (true) {
        if (!PERSISTENT) {
            if (tile_base >= n_live) break;
            if (g == 0) {
                const long long li = tile_base + item;
                long long id = li < n_live ? (long long)live_in[li] : -1;
                s_id[item] = id;
                s_alive[item] = id >= 0;
                if (id >= 0) {
                    s_t[item] = st_t[id];
                    s_step[item] = st_step[id];
                    s_count[item] = st_count[id];
                    for (int k = 0; k < 3; ++k) { s_root[item][k] = roots[3 * id + k]; s_dir[item][k] = dirs[3 * id + k]; }
                }
            }
            sync();
        } else if constexpr (WM) {
            if (!__any_sync(0xffffffffu, s_alive[item] && g == 0)) break;
        } else {
            if (!__syncthreads_or(s_alive[item] && g == 0)) break;
        }
        if (g == 0) { s_hit[item] = 0; s_hitid[item] = 0; s_inner[item] = 0; }
        for (int sub = 0; sub < o.n_substeps; ++sub) {
            if (g == 0) {
                s_can[item] = !s_hit[item];
                s_act[item] = s_alive[item] && !s_hit[item];
                s_inner[item] += s_act[item] ? 1 : 0;
            }
            sync();
            for (int f = 0; f < S.n; ++f) {
                if (S.n > 1) load_header(H, S.m[f].hdr);
                // build rows: thread g < 4 owns input column g
                const bool active = s_act[item];
                float* xs = st + item * R * LD;
                if (g < 4) {
                    const int k = g;
                    for (int r = 0; r < R; ++r) xs[r * LD + k] = 0.f;
                    if (active && k < 3) {
                        const float t = s_t[item], sz = s_step[item];
                        const float rt = s_root[item][k], d = s_dir[item][k];
                        const float ps = __fadd_rn(rt, __fmul_rn(t, d));
                        const float hv = __fmul_rn(__fmul_rn(0.5f, sz), d);
                        const float pm = __fadd_rn(ps, hv);
                        const float pe = __fadd_rn(rt, __fmul_rn(__fadd_rn(t, o.hit_eps), d));
                        xs[k] = pm;
                        xs[rp0 * LD + k] = ps;
                        xs[(rp0 + 1) * LD + k] = pe;
                        // gamma of this function's first layer (read from global: H may be in flux)
                        const float gam0 = C ? __ldg(&S.m[f].hdr->layers[0].gamma) : 0.f;
                        if (SLOPE) {
                            xs[LD + k] = hv;
                            xs[5 * LD + k] = C ? __fmul_ru(gam0, fabsf(hv)) : 0.f;
                            xs[4 * LD + k] = C ? __fmul_ru(gam0, fabsf(pm)) : 0.f;
                        } else if (mode_interval) {
                            xs[rerr * LD + k] = C ? __fmaf_ru(gam0, fabsf(pm), fabsf(hv)) : fabsf(hv);
                        } else {
                            xs[LD + k] = hv;
                            xs[rerr * LD + k] = C ? __fmul_ru(gam0, __fadd_ru(fabsf(pm), fabsf(hv))) : 0.f;
                        }
                    }
                }
                sync();
                const int woff = resident ? S.woff[f] : 0;
                tile_forward<Cfg, C, WM>(H, S.m[f].w, sW + woff, sw_cap, resident, plan, st, ob);
                if (g == 0 && active) {
                    const float* out = ob + item * R;
                    float lo, hi;
                    if (SLOPE) slope_out_bounds<C>(out, plan.v, lo, hi);
                    else affine_out_bounds<Cfg::R, C>(out, plan.v, lo, hi);
                    const int bt = sign_of_bounds(lo, hi, 0.f);
                    if (bt == NIQ_SIGN_UNKNOWN) s_can[item] = 0;
                    const float v0 = out[rp0], v1 = out[rp0 + 1];
                    const int sg0 = (v0 > 0.f) - (v0 < 0.f), sg1 = (v1 > 0.f) - (v1 < 0.f);
                    const bool this_hit = (v0 != v0) || (v1 != v1) || sg0 != sg1;  // NaN != NaN
                    if (this_hit) { s_hitid[item] = f + 1; s_hit[item] = 1; }
                    atomicAdd(&s_evals[f], 1ull);
                }
                sync();
            }
            if (g == 0 && s_alive[item]) {
                // src/queries.py:79-90
                const bool can = s_can[item];
                const float sz = s_step[item];
                const float this_step = can ? sz : o.hit_eps;
                if (!s_hit[item]) s_t[item] = __fadd_rn(s_t[item], __fmul_rn(this_step, o.safety));
                float ns = can ? __fmul_rn(sz, o.grow) : __fmul_rn(sz, o.shrink);
                s_step[item] = fmaxf(ns, o.hit_eps);
            }
            sync();
        }
        // ---- termination (src/queries.py:113-126) and slot refill
        if (g == 0 && s_alive[item]) {
            const long long id = s_id[item];
            const int cnt = s_count[item] + s_inner[item];
            s_count[item] = cnt;
            const float t = s_t[item];
            const bool term = s_hit[item] || (t > o.max_dist) || (cnt >= o.n_max_step);
            if (term) {
                t_out[id] = t;
                hit_out[id] = s_hitid[item];
                count_out[id] = cnt;
                if (PERSISTENT) claim(item);
                else s_alive[item] = 0;
            } else if (!PERSISTENT) {
                st_t[id] = t;
                st_step[id] = s_step[item];
                st_count[id] = cnt;
            }
        }
        if (!PERSISTENT) {
            // append survivors to the next live list (warp-aggregated)
            const bool keep = (g == 0) && s_alive[item];
            const long long pos = niq_warp_append(&ws->n_live_next, keep);
            if (keep) live_out[pos] = (int)s_id[item];
            sync();
            tile_base += (long long)gridDim.x * ITEMS;
        }
        sync();
    }
    };
    if constexpr (PERSISTENT) {
        if (resident && S.n == 1) run(std::integral_constant<bool, true>());
        else run(std::integral_constant<bool, false>());
    } else {
        run(std::integral_constant<bool, false>());
    }
    __syncthreads();
    if (threadIdx.x < S.n && s_evals[threadIdx.x]) atomicAdd(&n_evals[threadIdx.x], s_evals[threadIdx.x]);
}

__global__ void k_ray_init(float* step, int* live, long long n, float init_step) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        step[i] = init_step;
        live[i] = (int)i;
    }
}

static void fill_ray_init(float* step, int* live, long long n, float init_step, cudaStream_t s) {
    long long blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_ray_init<<<(int)blocks, 256, 0, s>>>(step, live, n, init_step);
}

}  // namespace niq

using namespace niq;

namespace {

struct RayLayout {
    size_t hdr = 0, t = 0, step = 0, count = 0, live0 = 0, live1 = 0, total = 0;
};

RayLayout ray_layout(long long n) {
    RayLayout L;
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    L.hdr = 0;
    L.t = al(sizeof(RayWs));
    L.step = L.t + al(4 * n);
    L.count = L.step + al(4 * n);
    L.live0 = L.count + al(4 * n);
    L.live1 = L.live0 + al(4 * n);
    L.total = L.live1 + al(4 * n) + 256;
    return L;
}

bool growing_mode(int mode) {
    return mode == NIQ_MODE_AFFINE_TRUNCATE || mode == NIQ_MODE_AFFINE_ALL || mode == NIQ_MODE_AFFINE_APPEND;
}

// Extra workspace of the growing-term path: per live ray a segment (center, vec), two
// hit-test points, per function a sign and two values, and the substep state; then the
// growing-term engine's own slots (the largest over the functions).
struct WideRayLayout {
    size_t center, vec, pts, sign, vals, hit, hitid, can, inner, wide, total;
};

WideRayLayout wide_ray_layout(const niq_model* const* models, int nfunc, const niq_bound_opts& o, long long n,
                              size_t base) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    WideRayLayout W;
    W.center = base;
    W.vec = W.center + al(12 * n);
    W.pts = W.vec + al(12 * n);
    W.sign = W.pts + al(24 * n);
    W.vals = W.sign + al(4 * n * (size_t)nfunc);
    W.hit = W.vals + al(8 * n * (size_t)nfunc);
    W.hitid = W.hit + al(4 * n);
    W.can = W.hitid + al(4 * n);
    W.inner = W.can + al(4 * n);
    W.wide = W.inner + al(4 * n);
    size_t wmax = 0;
    for (int f = 0; f < nfunc; ++f)
        if (models && models[f]) {
            const size_t b = wide_workspace_bytes(models[f]->hdr, o, 1);
            wmax = wmax > b ? wmax : b;
        }
    W.total = W.wide + al(wmax) + 256;
    return W;
}

__global__ void k_wray_prep(long long n_live, const int* live, const float* roots, const float* dirs, const float* st_t,
                            const float* st_step, float hit_eps, float* center, float* vec, float* pts) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_live; i += (long long)gridDim.x * blockDim.x) {
        const int id = live[i];
        const float t = st_t[id], sz = st_step[id];
        for (int k = 0; k < 3; ++k) {
            const float rt = roots[3 * id + k], d = dirs[3 * id + k];
            const float ps = __fadd_rn(rt, __fmul_rn(t, d));
            const float hv = __fmul_rn(__fmul_rn(0.5f, sz), d);
            center[3 * i + k] = __fadd_rn(ps, hv);
            vec[3 * i + k] = hv;
            pts[6 * i + k] = ps;
            pts[6 * i + 3 + k] = __fadd_rn(rt, __fmul_rn(__fadd_rn(t, hit_eps), d));
        }
    }
}

// One substep for every live ray (src/queries.py:44-92) from the per-function signs and
// point values; substep 0 also resets the outer iteration's hit state.
__global__ void k_wray_update(long long n_live, const int* live, int nfunc, const int* sign, const float* vals,
                              int first_substep, CastDev o, float* st_t, float* st_step, int* hit, int* hitid,
                              int* inner) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n_live; i += (long long)gridDim.x * blockDim.x) {
        const int id = live[i];
        if (first_substep) { hit[i] = 0; hitid[i] = 0; inner[i] = 0; }
        const bool hit_before = hit[i] != 0;
        bool can = !hit_before;
        bool is_hit = hit_before;
        int hid = hitid[i];
        inner[i] += hit_before ? 0 : 1;
        for (int f = 0; f < nfunc; ++f) {
            const int bt = sign[(long long)f * n_live + i];
            if (bt == NIQ_SIGN_UNKNOWN) can = false;
            const float v0 = vals[(long long)f * 2 * n_live + 2 * i], v1 = vals[(long long)f * 2 * n_live + 2 * i + 1];
            const int s0 = (v0 > 0.f) - (v0 < 0.f), s1 = (v1 > 0.f) - (v1 < 0.f);
            if ((v0 != v0) || (v1 != v1) || s0 != s1) { hid = f + 1; is_hit = true; }
        }
        const float sz = st_step[id];
        const float this_step = can ? sz : o.hit_eps;
        if (!is_hit) st_t[id] = __fadd_rn(st_t[id], __fmul_rn(this_step, o.safety));
        st_step[id] = fmaxf(can ? __fmul_rn(sz, o.grow) : __fmul_rn(sz, o.shrink), o.hit_eps);
        hit[i] = is_hit;
        hitid[i] = hid;
    }
}

__global__ void k_wray_finish(long long n_live, const int* live, const int* hit, const int* hitid, const int* inner,
                              CastDev o, const float* st_t, int* st_count, float* t_out, int* hit_out, int* count_out,
                              int* live_next, unsigned long long* n_next) {
    for (long long i0 = blockIdx.x * (long long)blockDim.x; i0 < n_live; i0 += (long long)gridDim.x * blockDim.x) {
        const long long i = i0 + threadIdx.x;
        bool keep = false;
        int id = 0;
        if (i < n_live) {
            id = live[i];
            const int cnt = st_count[id] + inner[i];
            st_count[id] = cnt;
            const float t = st_t[id];
            const bool term = hit[i] || (t > o.max_dist) || (cnt >= o.n_max_step);
            if (term) { t_out[id] = t; hit_out[id] = hitid[i]; count_out[id] = cnt; }
            keep = !term;
        }
        const long long pos = niq_warp_append(n_next, keep);
        if (keep) live_next[pos] = id;
    }
}

template <bool PERSISTENT>
int launch_rays(const niq_model* const* models, int nfunc, const niq_bound_opts* opts, long long n, const float* roots,
                const float* dirs, const niq_cast_opts* cast, float* t_out, int* hit_out, int* count_out,
                unsigned long long* n_evals, void* workspace, size_t ws_bytes, cudaStream_t s);

// The growing-term modes: a host loop over the reference's iterations, each substep
// bounding every live segment with the growing-term engine (v = 1) and evaluating the
// two hit-test points, then the reference's step rule and a compaction.
int launch_rays_wide(const niq_model* const* models, int nfunc, const niq_bound_opts* opts, long long n,
                     const float* roots, const float* dirs, const niq_cast_opts* cast, float* t_out, int* hit_out,
                     int* count_out, unsigned long long* n_evals, void* workspace, size_t ws_bytes, cudaStream_t s) {
    NIQ_REQUIRE(models && nfunc >= 1 && nfunc <= kMaxFuncs, NIQ_ERR_INVALID_ARG, "nfunc must be in [1, %d]", kMaxFuncs);
    for (int f = 0; f < nfunc; ++f) NIQ_REQUIRE(models[f], NIQ_ERR_INVALID_ARG, "null model %d", f);
    const RayLayout RL = ray_layout(n);
    const WideRayLayout W = wide_ray_layout(models, nfunc, *opts, n, RL.total);
    NIQ_REQUIRE(workspace && ws_bytes >= W.total, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed", W.total);
    NIQ_REQUIRE(n == 0 || (roots && dirs && t_out && hit_out && count_out && n_evals), NIQ_ERR_INVALID_ARG, "null array");
    NIQ_CUDA(cudaMemsetAsync(n_evals, 0, sizeof(unsigned long long) * nfunc, s));
    if (n == 0) return NIQ_OK;
    char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
    RayWs* ws = reinterpret_cast<RayWs*>(base + RL.hdr);
    float* st_t = reinterpret_cast<float*>(base + RL.t);
    float* st_step = reinterpret_cast<float*>(base + RL.step);
    int* st_count = reinterpret_cast<int*>(base + RL.count);
    int* live[2] = {reinterpret_cast<int*>(base + RL.live0), reinterpret_cast<int*>(base + RL.live1)};
    float* center = reinterpret_cast<float*>(base + W.center);
    float* vec = reinterpret_cast<float*>(base + W.vec);
    float* pts = reinterpret_cast<float*>(base + W.pts);
    int* sign = reinterpret_cast<int*>(base + W.sign);
    float* vals = reinterpret_cast<float*>(base + W.vals);
    int* hit = reinterpret_cast<int*>(base + W.hit);
    int* hitid = reinterpret_cast<int*>(base + W.hitid);
    int* inner = reinterpret_cast<int*>(base + W.inner);
    void* wws = base + W.wide;
    const size_t wws_bytes = ws_bytes - (size_t)(base - reinterpret_cast<char*>(workspace)) - W.wide;
    const CastDev cd = to_dev(*cast);
    NIQ_CUDA(cudaMemsetAsync(ws, 0, sizeof(RayWs), s));
    NIQ_CUDA(cudaMemsetAsync(st_t, 0, 4 * n, s));
    NIQ_CUDA(cudaMemsetAsync(st_count, 0, 4 * n, s));
    fill_ray_init(st_step, live[0], n, cd.init_step, s);
    long long n_live = n;
    int cur = 0;
    std::vector<unsigned long long> evals(nfunc, 0ull);
    while (n_live > 0) {
        const int blocks = (int)((n_live + 255) / 256 < 4096 ? (n_live + 255) / 256 : 4096);
        for (int sub = 0; sub < cd.n_substeps; ++sub) {
            k_wray_prep<<<blocks, 256, 0, s>>>(n_live, live[cur], roots, dirs, st_t, st_step, cd.hit_eps, center, vec, pts);
            NIQ_CUDA(cudaGetLastError());
            for (int f = 0; f < nfunc; ++f) {
                int rc = wide_classify(models[f], *opts, n_live, center, vec, 1, 0.f, sign + (long long)f * n_live,
                                       nullptr, wws, wws_bytes, s);
                if (rc) return rc;
                rc = niq_eval_points(models[f], 2 * n_live, pts, vals + (long long)f * 2 * n_live, s);
                if (rc) return rc;
                evals[f] += (unsigned long long)n_live;
            }
            k_wray_update<<<blocks, 256, 0, s>>>(n_live, live[cur], nfunc, sign, vals, sub == 0, cd, st_t, st_step, hit,
                                                 hitid, inner);
            NIQ_CUDA(cudaGetLastError());
        }
        NIQ_CUDA(cudaMemsetAsync(&ws->n_live_next, 0, sizeof(unsigned long long), s));
        k_wray_finish<<<blocks, 256, 0, s>>>(n_live, live[cur], hit, hitid, inner, cd, st_t, st_count, t_out, hit_out,
                                             count_out, live[1 - cur], &ws->n_live_next);
        NIQ_CUDA(cudaGetLastError());
        unsigned long long next = 0;
        NIQ_CUDA(cudaMemcpyAsync(&next, &ws->n_live_next, sizeof(next), cudaMemcpyDeviceToHost, s));
        NIQ_CUDA(cudaStreamSynchronize(s));
        n_live = (long long)next;
        cur = 1 - cur;
    }
    NIQ_CUDA(cudaMemcpyAsync(n_evals, evals.data(), sizeof(unsigned long long) * nfunc, cudaMemcpyHostToDevice, s));
    NIQ_CUDA(cudaStreamSynchronize(s));
    return NIQ_OK;
}

template <bool PERSISTENT>
int launch_rays(const niq_model* const* models, int nfunc, const niq_bound_opts* opts, long long n, const float* roots,
                const float* dirs, const niq_cast_opts* cast, float* t_out, int* hit_out, int* count_out,
                unsigned long long* n_evals, void* workspace, size_t ws_bytes, cudaStream_t s) {
    NIQ_REQUIRE(opts && cast, NIQ_ERR_INVALID_ARG, "null options");
    NIQ_REQUIRE(n >= 0 && n < (1ll << 31), NIQ_ERR_INVALID_ARG, "ray count %lld out of range", n);
    NIQ_REQUIRE(cast->n_substeps >= 1 && cast->hit_eps > 0.f, NIQ_ERR_INVALID_ARG, "n_substeps >= 1 and hit_eps > 0 required");
    const int mode = opts->mode;
    if (growing_mode(mode))
        return launch_rays_wide(models, nfunc, opts, n, roots, dirs, cast, t_out, hit_out, count_out, n_evals, workspace,
                                ws_bytes, s);
    NIQ_REQUIRE(mode == NIQ_MODE_AFFINE_FIXED || mode == NIQ_MODE_INTERVAL || mode == NIQ_MODE_SLOPE_INTERVAL,
                NIQ_ERR_UNSUPPORTED, "unknown mode %d", mode);
    ModelSet S;
    int maxw, wfloats, maxlayer;
    int rc = make_set(models, nfunc, S, maxw, wfloats, maxlayer);
    if (rc) return rc;
    const RayLayout RL = ray_layout(n);
    NIQ_REQUIRE(workspace && ws_bytes >= RL.total, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed", RL.total);
    NIQ_REQUIRE(n == 0 || (roots && dirs && t_out && hit_out && count_out && n_evals), NIQ_ERR_INVALID_ARG, "null array");
    NIQ_CUDA(cudaMemsetAsync(n_evals, 0, sizeof(unsigned long long) * nfunc, s));
    if (n == 0) return NIQ_OK;
    char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
    RayWs* ws = reinterpret_cast<RayWs*>(base + RL.hdr);
    float* st_t = reinterpret_cast<float*>(base + RL.t);
    float* st_step = reinterpret_cast<float*>(base + RL.step);
    int* st_count = reinterpret_cast<int*>(base + RL.count);
    int* live[2] = {reinterpret_cast<int*>(base + RL.live0), reinterpret_cast<int*>(base + RL.live1)};
    NIQ_CUDA(cudaMemsetAsync(ws, 0, sizeof(RayWs), s));
    const CastDev cd = to_dev(*cast);
    const bool cons = opts->conservative != 0;
    const bool slope = mode == NIQ_MODE_SLOPE_INTERVAL;
    const int interval = mode == NIQ_MODE_INTERVAL;
    const int tpi = tpi_for_width(maxw);
    // The narrow tile (4 columns per thread, 8 lanes per ray; same results) for models at
    // most 32 wide: in slope_interval always (its 8-column tile needs more than 128
    // registers and fits one CTA per SM: 1.9x faster at 128^2 and 1024^2 rays on the
    // 3->32x3->1 model), otherwise when the rays are few enough that the cast is bound by
    // its slowest rays' step latency rather than by throughput (up to 512 rays per SM,
    // about four resident waves of the 8-column tile: 1.37x faster at 128^2; at 1024^2
    // the 8-column tile is 2% faster).  The tuning parameter overrides the choice.
    const int cols_tuned = tune_value(kTuneRayColumns);
    const bool few = n <= 512ll * device_info().sm_count;
    const bool narrow = maxw <= 32 && (cols_tuned == 4 || (cols_tuned == 0 && (slope || few)));
    rc = NIQ_OK;
    auto run = [&](auto kern, int R, int TPIv, int COLSv) -> int {
        const int items = kNT / TPIv;
        const int state = items * R * (TPIv * COLSv + 4) + ((items * R + 3) & ~3);
        SmemPlan p = plan_smem(state, wfloats, maxlayer, smem_budget(kern, kNT));
        NIQ_REQUIRE(p.resident || p.sw_cap >= 5 * maxw, NIQ_ERR_UNSUPPORTED, "shared memory too small for width %d", maxw);
        int r2 = prepare_kernel(kern, p.bytes);
        if (r2) return r2;
        if (PERSISTENT) {
            int grid = 0;
            r2 = persistent_grid(kern, kNT, p.bytes, (n + items - 1) / items, &grid);
            if (r2) return r2;
            kern<<<grid, kNT, p.bytes, s>>>(S, interval, n, roots, dirs, cd, t_out, hit_out, count_out, n_evals, ws,
                                            nullptr, nullptr, nullptr, nullptr, 0, nullptr, p.fixed_floats, p.sw_cap,
                                            p.resident);
            NIQ_CUDA(cudaGetLastError());
            return NIQ_OK;
        }
        // plain: host loop over iterations with a device->host count read each time
        long long n_live = n;
        NIQ_CUDA(cudaMemsetAsync(st_t, 0, 4 * n, s));
        NIQ_CUDA(cudaMemsetAsync(st_count, 0, 4 * n, s));
        fill_ray_init(st_step, live[0], n, cd.init_step, s);
        int cur = 0;
        int grid_max = 0;
        r2 = persistent_grid(kern, kNT, p.bytes, (n + items - 1) / items, &grid_max);
        if (r2) return r2;
        while (n_live > 0) {
            NIQ_CUDA(cudaMemsetAsync(&ws->n_live_next, 0, sizeof(unsigned long long), s));
            long long tiles = (n_live + items - 1) / items;
            const int grid = (int)(tiles < grid_max ? tiles : grid_max);
            kern<<<grid, kNT, p.bytes, s>>>(S, interval, n, roots, dirs, cd, t_out, hit_out, count_out, n_evals, ws,
                                            st_t, st_step, st_count, live[cur], n_live, live[1 - cur], p.fixed_floats,
                                            p.sw_cap, p.resident);
            NIQ_CUDA(cudaGetLastError());
            unsigned long long next = 0;
            NIQ_CUDA(cudaMemcpyAsync(&next, &ws->n_live_next, sizeof(next), cudaMemcpyDeviceToHost, s));
            NIQ_CUDA(cudaStreamSynchronize(s));
            n_live = (long long)next;
            cur = 1 - cur;
        }
        return NIQ_OK;
    };
#define NIQ_RAYS(CC, SL)                                                                    \
    if (narrow) rc = run(k_rays<8, 4, CC, SL, PERSISTENT>, SL ? 8 : 5, 8, 4);                   \
    else NIQ_DISPATCH_TPI(tpi, { rc = run(k_rays<TPI, 8, CC, SL, PERSISTENT>, SL ? 8 : 5, TPI, 8); })
    if (slope) { if (cons) { NIQ_RAYS(true, true); } else { NIQ_RAYS(false, true); } }
    else { if (cons) { NIQ_RAYS(true, false); } else { NIQ_RAYS(false, false); } }
#undef NIQ_RAYS
    return rc;
}

}  // namespace

extern "C" {

size_t niq_cast_rays_workspace_size(const niq_model* const* models, int32_t nfunc, const niq_bound_opts* opts,
                                    int64_t n) {
    const RayLayout RL = ray_layout(n);
    if (opts && growing_mode(opts->mode)) return wide_ray_layout(models, nfunc, *opts, n, RL.total).total;
    return RL.total;
}

int niq_cast_rays(const niq_model* const* models, int32_t nfunc, const niq_bound_opts* opts, int64_t n,
                  const float* roots, const float* dirs, const niq_cast_opts* cast, float* t_out, int32_t* hit_id_out,
                  int32_t* count_out, int64_t* n_evals_out, void* workspace, size_t workspace_bytes, void* stream) {
    return launch_rays<true>(models, nfunc, opts, n, roots, dirs, cast, t_out, hit_id_out, count_out,
                             reinterpret_cast<unsigned long long*>(n_evals_out), workspace, workspace_bytes,
                             as_stream(stream));
}

int niq_cast_rays_plain(const niq_model* const* models, int32_t nfunc, const niq_bound_opts* opts, int64_t n,
                        const float* roots, const float* dirs, const niq_cast_opts* cast, float* t_out,
                        int32_t* hit_id_out, int32_t* count_out, int64_t* n_evals_out, void* workspace,
                        size_t workspace_bytes, void* stream) {
    return launch_rays<false>(models, nfunc, opts, n, roots, dirs, cast, t_out, hit_id_out, count_out,
                              reinterpret_cast<unsigned long long*>(n_evals_out), workspace, workspace_bytes,
                              as_stream(stream));
}

}  // extern "C"
