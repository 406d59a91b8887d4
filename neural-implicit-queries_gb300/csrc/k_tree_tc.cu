// k_tree_tc.cu -- construct_uniform_unknown_levelset_tree (src/kd_tree.py:19-218) with the
// hidden layers' dense products on the tensor cores.
//
// Same level loop, node claims, appends and split rule as k_tree.cu; what changes is how
// a node's affine_fixed bound (src/affine.py:109-193, src/affine_layers.py:11-56) is
// computed.  A CTA (8 warps, one per SM: the operands fill the shared memory) takes 32
// nodes at a time.  Their four signed rows each -- base and the three noise rows -- form
// the M = 128 rows of one GEMM per hidden layer,
//     D[4 b + kind][n] = sum_k X[4 b + kind][k] A[k][n],
// issued by one thread as tcgen05.mma kind::tf32 split-precision products
// Xhi Ahi + Xhi Alo + Xlo Ahi accumulated in fp32 in tensor memory (TMEM lane = row).
// The err row (err @ |A|, one row per node) runs on the CUDA cores at the same time.
// The first layer (3 inputs) and the last (one output) are computed on the CUDA cores.
//
// Epilogue (src/affine.py:164-193, the ReLU/ELU/TanH linearisations of tile_engine.cuh):
// warp w reads TMEM lane quadrant w % 4 (nodes 8 (w % 4) .. + 7, lane 4 i + kind) and
// the 32 columns of half w / 4.  The four lanes of a node trade values in 4 x 4
// transposes so that each lane holds the four rows of one column, applies the
// linearisation to it, and transposes back to store the next layer's operand (hi, lo)
// as 16-byte rows.
//
// Outward rounding (every bound contains the exact range of the network over the box):
// a split-precision product of n terms differs from the exact dot product by at most
// gamma_tc(n) sum |x||a| (the hi parts are exact in tf32, the lo parts lose at most 2^-10
// of themselves, the dropped lo*lo term is below 2^-20 |x||a|, and the fp32 accumulation
// is charged 2^-21 per addition); as in the FP32 engine that bound is folded into the
// err row before the layer, err' = err + gamma_tc (|base| + sum |aff|), and travels
// through |A|.  The err row's own FP32 dot product is scaled by 1 + 2 gamma(n); the bias
// add is charged 2^-23 |base|; underflow gets a fixed absolute allowance.
#include "tree_common.cuh"
#include "tc_sm100.cuh"

namespace niq {

constexpr int kTtNT = 256;            // threads per CTA
constexpr int kTtBoxes = 32;          // nodes per group: 4 rows each fill one M = 128 tile
constexpr int kTtMaxW = 64;           // widest layer input or output
constexpr int kTtEst = kTtMaxW + 4;   // err row stride (floats)
#define NIQ_TC_TINY 7.888609052210118e-31f   // 2^-100: absolute allowance per product (underflow)

NIQ_HOST_DEVICE int tt_round16(int x) { return (x + 15) & ~15; }

// Dynamic shared-memory plan (float offsets).
struct TtPlan {
    int b_off[NIQ_MAX_LAYERS];   // split operand (hi block, lo block after it) of hidden layer l
    int x_off;                   // node-row operand: hi half, lo half at x_off + 128 * kmax
    int kmax;                    // widest K of the node-row operand
    int e_off;                   // err rows [32][kTtEst]
    int total;                   // floats in all
};

static bool tt_plan(const NiqSpecHeader& H, TtPlan& p) {
    const int nL = H.n_layers;
    if (nL < 3 || nL > NIQ_MAX_LAYERS) return false;
    const NiqLayer& L0 = H.layers[0];
    const NiqLayer& LL = H.layers[nL - 1];
    if (L0.in != 3 || L0.act == NIQ_ACT_NONE || tt_round16(L0.out) > kTtMaxW) return false;
    if (LL.out != 1 || LL.act != NIQ_ACT_NONE || tt_round16(LL.in) > kTtMaxW) return false;
    int off = (H.n_weight_floats + 31) & ~31;
    int kmax = tt_round16(L0.out);
    for (int l = 1; l + 1 < nL; ++l) {
        const NiqLayer& L = H.layers[l];
        if (L.act == NIQ_ACT_NONE) return false;
        const int K = tt_round16(L.in), N = tt_round16(L.out);
        if (K > kTtMaxW || N > kTtMaxW) return false;
        p.b_off[l] = off;
        off += 2 * N * K;
        kmax = kmax > N ? kmax : N;
    }
    p.kmax = kmax;
    p.x_off = off;
    off += 2 * 128 * kmax;
    p.e_off = off;
    off += kTtBoxes * kTtEst;
    p.total = off;
    return true;
}

// Relative bound of one split-precision tensor-core dot product of n terms.
__device__ __forceinline__ float tt_gamma_tc(int n) {
    const float nu = (float)(n + 2) * 4.76837158203125e-07f;         // (n + 2) 2^-21
    return __fadd_ru(__fdiv_ru(nu, 1.f - nu), 3.814697265625e-06f);  // + 2^-18 for the splits
}

// 4 x 4 transpose among the four lanes of a node: lane k of the quad holds v = row k,
// columns 0..3; afterwards it holds column k, rows 0..3.  The same call transposes back.
__device__ __forceinline__ void quad_transpose(float& v0, float& v1, float& v2, float& v3, int lane) {
    const bool b1 = (lane & 2) != 0, b0 = (lane & 1) != 0;
    const float r0 = __shfl_xor_sync(0xffffffffu, b1 ? v0 : v2, 2);
    const float r1 = __shfl_xor_sync(0xffffffffu, b1 ? v1 : v3, 2);
    // 2 x 2 block: rows (lane & 1) and (lane & 1) | 2, columns 2 b1 and 2 b1 + 1
    const float m00 = b1 ? r0 : v0, m01 = b1 ? r1 : v1;
    const float m10 = b1 ? v2 : r0, m11 = b1 ? v3 : r1;
    const float u0 = __shfl_xor_sync(0xffffffffu, b0 ? m00 : m01, 1);
    const float u1 = __shfl_xor_sync(0xffffffffu, b0 ? m10 : m11, 1);
    v0 = b0 ? u0 : m00;
    v1 = b0 ? m01 : u0;
    v2 = b0 ? u1 : m10;
    v3 = b0 ? m11 : u1;
}

// One column of an activated layer, conservative (the phased epilogue of tile_forward):
// pre-activation rows in, the next layer's rows out with its dot-product rounding
// (gam_next) folded into err.
struct TtCol { float base, a0, a1, a2, err; };

__device__ __forceinline__ TtCol tt_activate(int act, float base, float a0, float a1, float a2, float err,
                                             float gam_next) {
    const float S = __fadd_ru(__fadd_ru(fabsf(a0), fabsf(a1)), fabsf(a2));
    const float rad = __fadd_ru(S, err);
    const float lo = __fsub_rd(base, rad), hi = __fadd_ru(base, rad);
    const Lin z = linearize<true>(act, lo, hi);
    const float nb = fmaf(z.a, base, z.b);
    const float aS = __fmul_ru(z.a, S);
    float e = __fmaf_ru(z.a, err, z.d);
    e = __fmaf_ru(__fadd_ru(fabsf(nb), aS), NIQ_ULP_REL, e);
    e = __fmaf_ru(gam_next, __fadd_ru(fabsf(nb), __fmul_ru(aS, 1.f + NIQ_ULP_REL)), e);
    TtCol o;
    o.base = nb;
    o.a0 = __fmul_rn(z.a, a0);
    o.a1 = __fmul_rn(z.a, a1);
    o.a2 = __fmul_rn(z.a, a2);
    o.err = e;
    return o;
}

template <bool COOP>
__global__ void __launch_bounds__(kTtNT, 1) k_tree_tc(NiqModelRef M, TreeParams P, TreeWs* ws, TreeBufs B, int level0,
                                                      TtPlan pl) {
    extern __shared__ __align__(1024) float smem[];
    __shared__ NiqSpecHeader H;
    __shared__ float s_lo[kTtBoxes][3], s_hi[kTtBoxes][3];
    __shared__ int s_type[kTtBoxes];
    __shared__ long long s_base;
    __shared__ unsigned long long s_boxes;
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t s_tmem;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    load_header(H, M.hdr);
    if (warp == 0) tc::tmem_alloc(&s_tmem, 64);
    if (tid == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_mbar_init();
        s_boxes = 0;
    }
    __syncthreads();
    float* sWf = smem;                       // the model's fp32 weight area
    float* sXh = smem + pl.x_off;            // node-row operand, hi and lo
    float* sXl = sXh + 128 * pl.kmax;
    float* sE = smem + pl.e_off;             // err rows
    stage_floats(sWf, M.w, H.n_weight_floats);
    __syncthreads();
    const int nL = H.n_layers;
    // split operands of the hidden layers: rows n, K-major (D = X * B^T)
    for (int l = 1; l + 1 < nL; ++l) {
        const NiqLayer Ly = H.layers[l];
        const int K = tt_round16(Ly.in), N = tt_round16(Ly.out);
        float* bh = smem + pl.b_off[l];
        float* bl = bh + N * K;
        for (int i = tid; i < N * K; i += kTtNT) {
            const int n = i / K, k = i - n * K;
            const float w = (n < Ly.out && k < Ly.in) ? sWf[Ly.a_off + k * Ly.out_pad + n] : 0.f;
            const float wh = tc::tf32_hi(w);
            const int o = (int)(tc::kmajor_offset(n, k, K) >> 2);
            bh[o] = wh;
            bl[o] = w - wh;
        }
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = s_tmem;
    uint32_t phase = 0;
    unsigned int epoch = 0;
    bool fail = false;
    bool mma_out = false;     // a commit this thread has not seen complete (after a failed wait)

    // epilogue roles: TMEM quadrant q, column half h, node i of the quadrant, row kind
    const int q = warp & 3, hh = warp >> 2, qi = lane >> 2, kind = lane & 3;
    const int eb = 8 * q + qi;                               // this lane's node
    const uint32_t t_row = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(32 * hh);
    // err GEMV roles: n-group of 4 columns and a pair of nodes
    const int gng = 2 * warp + (lane >> 4), gbp = lane & 15;
    // last-layer roles: node and k slice
    const int lb = tid >> 3, ls = tid & 7;

    // Writes one column's rows of node eb: err in place, the four signed rows (transposed
    // back to 16-byte rows of the K-major operand, hi and lo) for the layer with K = Kn.
    auto store_col = [&](TtCol o, int c, int outw, int Kn) {
        if (c >= outw) o = TtCol{0.f, 0.f, 0.f, 0.f, 0.f};
        if (c < Kn) sE[eb * kTtEst + c] = o.err;
        float v0 = o.base, v1 = o.a0, v2 = o.a1, v3 = o.a2;
        quad_transpose(v0, v1, v2, v3, lane);     // lane `kind` now holds row kind, 4 columns
        const int k0 = c & ~3;
        if (k0 < Kn) {
            const float4 h4 = make_float4(tc::tf32_hi(v0), tc::tf32_hi(v1), tc::tf32_hi(v2), tc::tf32_hi(v3));
            const float4 l4 = make_float4(v0 - h4.x, v1 - h4.y, v2 - h4.z, v3 - h4.w);
            const int o4 = (int)(tc::kmajor_offset(4 * eb + kind, k0, Kn) >> 2);
            *reinterpret_cast<float4*>(sXh + o4) = h4;
            *reinterpret_cast<float4*>(sXl + o4) = l4;
        }
    };

    for (int L = level0; L < kTreeMaxLevels && !fail; ++L) {
        const long long n_in = (long long)*((volatile unsigned long long*)&ws->level_count[L]);
        if (n_in > B.cap) {
            niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
            break;
        }
        const bool quit = (n_in >= P.thresh) || (L + 1 >= P.n_rounds) || (n_in == 0) || (L + 1 == kTreeMaxLevels);
        const long long n_lim = n_in < P.batch_end ? n_in : P.batch_end;
        const float* in_lo = B.lvl_lo[L & 1];
        const float* in_hi = B.lvl_hi[L & 1];
        float* out_lo = B.lvl_lo[(L + 1) & 1];
        float* out_hi = B.lvl_hi[(L + 1) & 1];
        while (!fail) {
            __syncthreads();
            if (tid == 0) s_base = P.batch_start + (long long)atomicAdd(&ws->grab[L], (unsigned long long)kTtBoxes);
            __syncthreads();
            const long long nbase = s_base;
            if (nbase >= n_lim) break;
            if (tid < 3 * kTtBoxes) {
                const int b = tid / 3, k = tid - 3 * b;
                const long long nid = nbase + b;
                const bool ok = nid < n_lim;
                s_lo[b][k] = ok ? in_lo[3 * nid + k] : 0.f;
                s_hi[b][k] = ok ? in_hi[3 * nid + k] : 0.f;
            }
            __syncthreads();
            // ---------------- layer 0 (3 inputs) on the CUDA cores: center and diagonal
            // half extents (src/implicit_function.py:33-37), the FP32 tile engine's rules
            {
                const NiqLayer Ly = H.layers[0];
                const float gam0 = Ly.gamma;
                float cc[3], hx[3], ef[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float lo = s_lo[eb][k], hi = s_hi[eb][k];
                    cc[k] = __fmul_rn(0.5f, __fadd_rn(lo, hi));
                    hx[k] = fmaxf(__fsub_ru(hi, cc[k]), __fsub_ru(cc[k], lo));
                    ef[k] = __fmul_ru(gam0, __fadd_ru(fabsf(cc[k]), hx[k]));
                }
                const int N0 = tt_round16(Ly.out);
                const float scale = 1.f + 2.f * gam0, tiny = (float)(Ly.in + 2) * NIQ_TINY;
                const float gl = tt_gamma_tc(tt_round16(H.layers[1].in));
                const float* A = sWf + Ly.a_off;
#pragma unroll 1
                for (int g = 0; g < 8; ++g) {
                    const int c = 32 * hh + 4 * g + kind;
                    if (32 * hh + 4 * g >= N0) break;   // uniform across the warp
                    TtCol o{0.f, 0.f, 0.f, 0.f, 0.f};
                    if (c < Ly.out) {
                        const float a0 = A[c], a1 = A[Ly.out_pad + c], a2 = A[2 * Ly.out_pad + c];
                        float db = fmaf(cc[0], a0, 0.f);
                        db = fmaf(cc[1], a1, db);
                        db = fmaf(cc[2], a2, db);
                        float de = fmaf(ef[0], fabsf(a0), 0.f);
                        de = fmaf(ef[1], fabsf(a1), de);
                        de = fmaf(ef[2], fabsf(a2), de);
                        const float bj = sWf[Ly.b_off + c];
                        const float base = __fadd_rn(db, bj);
                        const float err = __fadd_ru(__fmaf_ru(de, scale, __fmul_ru(gam0, fabsf(bj))), tiny);
                        o = tt_activate(Ly.act, base, __fmul_rn(hx[0], a0), __fmul_rn(hx[1], a1),
                                        __fmul_rn(hx[2], a2), err, gl);
                    }
                    store_col(o, c, Ly.out, N0);
                }
            }
            tc::fence_async_smem();
            __syncthreads();
            // ---------------- hidden layers: signed rows on the tensor cores
            for (int l = 1; l + 1 < nL; ++l) {
                const NiqLayer Ly = H.layers[l];
                const int K = tt_round16(Ly.in), N = tt_round16(Ly.out);
                if (tid == 0) {
                    tc::fence_after_sync();
                    const uint32_t xh = tc::smem_addr(sXh), xl = tc::smem_addr(sXl);
                    const uint32_t bh = tc::smem_addr(smem + pl.b_off[l]), bl = bh + (uint32_t)(N * K * 4);
                    const uint32_t sbo = (uint32_t)(K / 4) * 128u;
                    const uint32_t idesc = tc::idesc_tf32(128, N);
                    for (int ks = 0; ks < K / 8; ++ks) {
                        const uint64_t ah = tc::smem_desc(xh + ks * 256, 128, sbo);
                        const uint64_t al = tc::smem_desc(xl + ks * 256, 128, sbo);
                        const uint64_t wh = tc::smem_desc(bh + ks * 256, 128, sbo);
                        const uint64_t wl = tc::smem_desc(bl + ks * 256, 128, sbo);
                        tc::mma_tf32(tmem, ah, wh, idesc, ks > 0 ? 1u : 0u);
                        tc::mma_tf32(tmem, ah, wl, idesc, 1u);
                        tc::mma_tf32(tmem, al, wh, idesc, 1u);
                    }
                    tc::mma_commit(&bar);
                }
                mma_out = true;
                // err @ |A| on the CUDA cores (src/affine_layers.py:24-26) while the MMAs run
                float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
                const bool gon = 4 * gng < Ly.out_pad;
                if (gon) {
                    const float* A = sWf + Ly.a_off + 4 * gng;
                    const float* e0p = sE + (2 * gbp) * kTtEst;
                    const float* e1p = e0p + kTtEst;
#pragma unroll 2
                    for (int k = 0; k < Ly.in_pad; k += 4) {
                        const float4 x0 = *reinterpret_cast<const float4*>(e0p + k);
                        const float4 x1 = *reinterpret_cast<const float4*>(e1p + k);
                        const float xa[4] = {x0.x, x0.y, x0.z, x0.w}, xb[4] = {x1.x, x1.y, x1.z, x1.w};
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk) {
                            const float4 a = *reinterpret_cast<const float4*>(A + (k + kk) * Ly.out_pad);
                            const float aa[4] = {fabsf(a.x), fabsf(a.y), fabsf(a.z), fabsf(a.w)};
#pragma unroll
                            for (int j = 0; j < 4; ++j) {
                                acc[0][j] = fmaf(xa[kk], aa[j], acc[0][j]);
                                acc[1][j] = fmaf(xb[kk], aa[j], acc[1][j]);
                            }
                        }
                    }
                }
                __syncthreads();   // every err row read before it is overwritten
                if (4 * gng < N) {
                    const float gam = Ly.gamma, scale = 1.f + 2.f * gam;
#pragma unroll
                    for (int r = 0; r < 2; ++r) {
                        float4 o;
                        o.x = gon ? __fmul_ru(acc[r][0], scale) : 0.f;
                        o.y = gon ? __fmul_ru(acc[r][1], scale) : 0.f;
                        o.z = gon ? __fmul_ru(acc[r][2], scale) : 0.f;
                        o.w = gon ? __fmul_ru(acc[r][3], scale) : 0.f;
                        *reinterpret_cast<float4*>(sE + (2 * gbp + r) * kTtEst + 4 * gng) = o;
                    }
                }
                // the layer's MMAs complete before TMEM is read
                if (!tc::mbar_wait(&bar, phase, P.mbar_polls)) fail = true;
                else mma_out = false;
                phase ^= 1u;
                tc::fence_after_sync();
                fail = __syncthreads_or(fail ? 1 : 0) != 0;   // also: the err rows are written
                if (fail) break;
                // ---------------- epilogue: bias, rounding terms, activation, next operand
                const bool last_hidden = (l + 2 == nL);
                const NiqLayer Ln = H.layers[l + 1];
                const int Kn = tt_round16(Ln.in);
                const float gnext = last_hidden ? Ln.gamma : tt_gamma_tc(Kn);
                const float tiny = (float)(Ly.in + 2) * NIQ_TINY + (float)(4 * K + 8) * NIQ_TC_TINY;
                if (32 * hh < N) {
                    float v[32];
                    tc::tmem_ld32(t_row, v);
#pragma unroll
                    for (int g = 0; g < 8; ++g) {
                        if (32 * hh + 4 * g >= N) break;   // warp-uniform
                        const int c = 32 * hh + 4 * g + kind;
                        float d0 = v[4 * g], d1 = v[4 * g + 1], d2 = v[4 * g + 2], d3 = v[4 * g + 3];
                        quad_transpose(d0, d1, d2, d3, lane);   // d0 base, d1..d3 noise rows, column c
                        TtCol o{0.f, 0.f, 0.f, 0.f, 0.f};
                        if (c < Ly.out) {
                            const float bj = sWf[Ly.b_off + c];
                            const float base = __fadd_rn(d0, bj);
                            float err = sE[eb * kTtEst + c];
                            err = __fadd_ru(err, __fmaf_ru(fabsf(base), NIQ_ULP_REL, tiny));
                            o = tt_activate(Ly.act, base, d1, d2, d3, err, gnext);
                        }
                        store_col(o, c, Ly.out, Kn);
                    }
                }
                tc::fence_before_sync();   // TMEM reads done before the next layer's MMAs
                tc::fence_async_smem();    // operand writes visible to the tensor cores
                __syncthreads();
            }
            if (fail) break;
            // ---------------- last layer (one output) on the CUDA cores, bounds, sign
            {
                const NiqLayer Ly = H.layers[nL - 1];
                const int K = tt_round16(Ly.in);
                const int per = K / 8;
                float sb = 0.f, s0 = 0.f, s1 = 0.f, s2 = 0.f, se = 0.f;
                for (int k = ls * per; k < ls * per + per; ++k) {
                    if (k >= Ly.in) break;
                    const float a = sWf[Ly.a_off + k * Ly.out_pad];
                    const int r0 = (int)(tc::kmajor_offset(4 * lb, k, K) >> 2);
                    // rows 4 lb .. 4 lb + 3 sit 16 bytes (4 floats) apart in the operand
                    const float x0 = sXh[r0] + sXl[r0], x1 = sXh[r0 + 4] + sXl[r0 + 4];
                    const float x2 = sXh[r0 + 8] + sXl[r0 + 8], x3 = sXh[r0 + 12] + sXl[r0 + 12];
                    sb = fmaf(x0, a, sb);
                    s0 = fmaf(x1, a, s0);
                    s1 = fmaf(x2, a, s1);
                    s2 = fmaf(x3, a, s2);
                    se = fmaf(sE[lb * kTtEst + k], fabsf(a), se);
                }
#pragma unroll
                for (int off = 4; off > 0; off >>= 1) {
                    sb += __shfl_xor_sync(0xffffffffu, sb, off);
                    s0 += __shfl_xor_sync(0xffffffffu, s0, off);
                    s1 += __shfl_xor_sync(0xffffffffu, s1, off);
                    s2 += __shfl_xor_sync(0xffffffffu, s2, off);
                    se += __shfl_xor_sync(0xffffffffu, se, off);
                }
                if (ls == 0) {
                    const float gam = Ly.gamma, bj = sWf[Ly.b_off];
                    const float base = __fadd_rn(sb, bj);
                    const float err = __fadd_ru(__fmaf_ru(se, 1.f + 2.f * gam, __fmul_ru(gam, fabsf(bj))),
                                                (float)(Ly.in + 2) * NIQ_TINY);
                    const float S = __fadd_ru(__fadd_ru(fabsf(s0), fabsf(s1)), fabsf(s2));
                    const float rad = __fadd_ru(S, err);
                    s_type[lb] = sign_of_bounds(__fsub_rd(base, rad), __fadd_ru(base, rad), P.offset);
                }
            }
            __syncthreads();
            // ---------------- results and children (warp 0, lane = node)
            if (warp == 0) {
                const long long nid = nbase + lane;
                const bool valid = nid < n_lim;
                const int type = valid ? s_type[lane] : -1;
                const bool is_unknown = type == NIQ_SIGN_UNKNOWN;
                const bool is_int = P.with_interior && type == NIQ_SIGN_NEGATIVE;
                const bool is_ext = P.with_exterior && type == NIQ_SIGN_POSITIVE;
                const long long pi = niq_warp_reserve(&ws->n_interior, is_int, 1);
                const long long pe = niq_warp_reserve(&ws->n_exterior, is_ext, 1);
                const long long pu = quit ? niq_warp_reserve(&ws->n_unknown, is_unknown, 1) : -1;
                const long long pc = quit ? -1 : niq_warp_reserve(&ws->level_count[L + 1], is_unknown, 2);
                if (valid) {
                    const float* lo = s_lo[lane];
                    const float* hi = s_hi[lane];
                    if (is_int) { if (pi < B.cap) put_node(B.res_lo[1], B.res_hi[1], pi, lo, hi); else niq_flag_error(&ws->err, NIQ_ERR_CAPACITY); }
                    if (is_ext) { if (pe < B.cap) put_node(B.res_lo[2], B.res_hi[2], pe, lo, hi); else niq_flag_error(&ws->err, NIQ_ERR_CAPACITY); }
                    if (is_unknown) {
                        if (quit) {
                            if (pu < B.cap) put_node(B.res_lo[0], B.res_hi[0], pu, lo, hi);
                            else niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
                        } else if (pc + 1 < B.cap) {
                            // split along the first longest axis (src/kd_tree.py:38,70-77)
                            const float l0 = lo[0], l1 = lo[1], l2 = lo[2], h0 = hi[0], h1 = hi[1], h2 = hi[2];
                            const float e0 = __fsub_rn(h0, l0), e1 = __fsub_rn(h1, l1), e2 = __fsub_rn(h2, l2);
                            int d = 0;
                            float em = e0;
                            if (e1 > em) { d = 1; em = e1; }
                            if (e2 > em) { d = 2; }
                            const float mid = d == 0 ? __fmul_rn(0.5f, __fadd_rn(l0, h0))
                                            : d == 1 ? __fmul_rn(0.5f, __fadd_rn(l1, h1))
                                                     : __fmul_rn(0.5f, __fadd_rn(l2, h2));
                            const float alo[3] = {l0, l1, l2};
                            const float ahi[3] = {d == 0 ? mid : h0, d == 1 ? mid : h1, d == 2 ? mid : h2};
                            const float blo[3] = {d == 0 ? mid : l0, d == 1 ? mid : l1, d == 2 ? mid : l2};
                            const float bhi[3] = {h0, h1, h2};
                            put_node(out_lo, out_hi, pc, alo, ahi);
                            put_node(out_lo, out_hi, pc + 1, blo, bhi);
                        } else {
                            niq_flag_error(&ws->err, NIQ_ERR_CAPACITY);
                        }
                    }
                }
                const unsigned int nv = __popc(__ballot_sync(0xffffffffu, valid));
                if (lane == 0) s_boxes += nv;
            }
        }
        if (fail) break;
        if (!COOP) {
            if (tid == 0 && quit) atomicMax(&ws->last_level, L);
            break;
        }
        if (quit) {
            if (blockIdx.x == 0 && tid == 0) ws->last_level = L;
            break;
        }
        if (!niq_grid_barrier(&ws->barrier, gridDim.x, epoch, &ws->err, P.barrier_polls)) break;
    }
    if (fail) {
        if (tid == 0) niq_flag_error(&ws->err, NIQ_ERR_TIMEOUT);
        // the commit that did not arrive in time: wait for it once more, with the built-in
        // limit, before the tensor memory it writes is released
        if (mma_out) tc::mbar_wait(&bar, phase ^ 1u, kMbarPollsDefault);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0 && s_boxes) atomicAdd(&ws->n_boxes, s_boxes);
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, 64);
        tc::tmem_relinquish();
    }
}

static int tt_static_smem(int* bytes) {
    cudaFuncAttributes fa;
    NIQ_CUDA(cudaFuncGetAttributes(&fa, k_tree_tc<true>));
    *bytes = (int)fa.sharedSizeBytes;
    return NIQ_OK;
}

bool tree_tc_eligible(const NiqSpecHeader& H) {
    TtPlan p;
    if (!tt_plan(H, p)) return false;
    int st = 0;
    if (tt_static_smem(&st) != NIQ_OK) return false;
    return (long long)p.total * 4 + st <= (long long)device_info().smem_optin;
}

int run_tree_tc(const TreeLaunch& T) {
    TtPlan pl;
    NIQ_REQUIRE(tt_plan(*T.host_hdr, pl), NIQ_ERR_UNSUPPORTED, "model outside the tensor-core tree");
    const size_t bytes = (size_t)pl.total * 4;
    auto run = [&](auto kern) -> int {
        int r = prepare_kernel(kern, bytes);
        if (r) return r;
        int per_sm = 0;
        NIQ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTtNT, bytes));
        NIQ_REQUIRE(per_sm >= 1, NIQ_ERR_UNSUPPORTED, "tensor-core tree kernel does not fit on an SM");
        const int grid = device_info().sm_count;
        NiqModelRef M = T.M;
        TreeParams P = T.P;
        TreeWs* ws = T.ws;
        TreeBufs B = T.B;
        int level0 = 0;
        if (T.coop) {
            void* args[] = {&M, &P, &ws, &B, &level0, &pl};
            NIQ_CUDA(cudaLaunchCooperativeKernel((const void*)kern, grid, kTtNT, args, bytes, T.s));
            return NIQ_OK;
        }
        // plain: one launch per level (or per batch of T.batch nodes), the host reading
        // each level's size (src/kd_tree.py:137-198)
        for (int L = 0; L < kTreeMaxLevels; ++L) {
            unsigned long long cnt = 0;
            NIQ_CUDA(cudaMemcpyAsync(&cnt, &ws->level_count[L], 8, cudaMemcpyDeviceToHost, T.s));
            NIQ_CUDA(cudaStreamSynchronize(T.s));
            const long long n_in = (long long)cnt;
            const bool quit = (n_in >= P.thresh) || (L + 1 >= P.n_rounds) || (n_in == 0) || (L + 1 == kTreeMaxLevels);
            const long long step = T.batch > 0 ? T.batch : (n_in > 0 ? n_in : 1);
            for (long long b0 = 0; b0 < (n_in > 0 ? n_in : 1); b0 += step) {
                TreeParams Pb = P;
                Pb.batch_start = b0;
                Pb.batch_end = b0 + step;
                if (b0 > 0) NIQ_CUDA(cudaMemsetAsync(&ws->grab[L], 0, sizeof(unsigned long long), T.s));
                const long long nb = (n_in - b0 < step ? n_in - b0 : step);
                const long long tiles = (nb + kTtBoxes - 1) / kTtBoxes;
                const int g = (int)(tiles < grid ? (tiles < 1 ? 1 : tiles) : grid);
                kern<<<g, kTtNT, bytes, T.s>>>(M, Pb, ws, B, L, pl);
                NIQ_CUDA(cudaGetLastError());
            }
            if (quit) break;
        }
        return NIQ_OK;
    };
    return T.coop ? run(k_tree_tc<true>) : run(k_tree_tc<false>);
}

}  // namespace niq
