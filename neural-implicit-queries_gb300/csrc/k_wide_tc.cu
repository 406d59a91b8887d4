// k_wide_tc.cu -- the growing-term engine ('affine_truncate', 'affine_all';
// src/affine.py:127-193) with its dense products on the tensor cores.
//
// One CTA (8 warps, one per SM) propagates one box at a time.  A box's noise rows are the
// M dimension of a GEMM  D[rows x out] = X[rows x in] * A[in x out]  with up to 256 rows
// (two M = 128 tiles), computed by tcgen05.mma kind::tf32 as three split-precision
// products  Xhi*Ahi + Xhi*Alo + Xlo*Ahi  accumulated in fp32 in tensor memory (TMEM,
// 512 columns: tile t at columns 256 t).  X (split on the way in) and the split weights are
// streamed through a three-stage shared-memory ring in K chunks of 16 (weights by
// cp.async, two chunks ahead), the MMAs issued by one
// thread and tracked with an mbarrier per stage.  The base and err rows (one vector
// each) are computed on the CUDA cores.
//
// The activation epilogue reads D straight from TMEM, thread per row:
//   1. column sums S_j = sum_r |D_rj| (transposed through shared memory),
//   2. the linearisation per column (alpha, beta, delta), exactly as the FP32 engine,
//   3. row magnitudes sum_j alpha_j |D_rj| and the new rows' delta_j,
//   4. the stable descending rank of every candidate row (src/affine.py:144-162),
//   5. kept rows, scaled by alpha, written in fp32 to the CTA's scratch as the next
//      layer's X, in rank order (split into hi and lo as each K chunk is staged); dropped
//      rows folded into err.
// The first layer (3 inputs) and the last (1 output) are computed on the CUDA cores.
// TMEM lanes past the box's rows and columns past the layer's width hold stale values;
// every epilogue read masks them.
//
// Conservative mode.  A tensor-core product of split operands differs from the exact
// product sum_k x_k a_k by at most gamma_tc(n) sum_k |x_k||a_k|: the hi parts are exact
// in tf32, the lo parts lose at most 2^-10 of themselves (2^-20 of x or a), the dropped
// lo*lo term is below 2^-20 |x||a|, and the fp32 accumulation is charged 2^-21 per
// addition (four times the unit of a truncating fp32 adder).  As in the FP32 engine the
// per-neuron bound rho_j = (gamma |base| + gamma_tc sum_r |X_r|) @ |A| (sum_r |X_rk| is
// bounded by alpha_k S_k + delta_k) widens the bounds that choose the linearisation and
// joins neuron j's new noise row, so it travels through later layers with A, not |A|.
#include <mutex>
#include "wide_engine.cuh"
#include "tc_sm100.cuh"

namespace niq {

constexpr int kTcNT = 256;
constexpr int kTcKC = 16;                      // K per pipeline stage
constexpr int kTcRows = 256;                   // noise rows one GEMM holds
constexpr int kTcTrLD = 17;                    // transpose buffer row stride (16 columns)
constexpr int kTcStages = 3;                   // shared-memory pipeline depth
constexpr int kTcStage = 4 * kTcRows * kTcKC;  // floats: X hi, X lo, W hi, W lo
constexpr int kTcXFloats = kTcRows * NIQ_MAX_WIDTH;  // a CTA's X scratch (fp32, split while staging)

// dynamic shared memory (floats)
constexpr int kTcOffTr = kTcStages * kTcStage;
constexpr int kTcOffPart = kTcOffTr + kTcRows * kTcTrLD;
constexpr int kTcOffVec = kTcOffPart + 256;
constexpr int kTcOffMag = kTcOffVec + 8 * 256;
constexpr int kTcOffRank = kTcOffMag + 512;
constexpr int kTcSmemFloats = kTcOffRank + 512;
constexpr size_t kTcSmemBytes = (size_t)kTcSmemFloats * 4;

struct TcArgs {
    NiqModelRef M;
    const float* tcw;                  // split transposed weights of layers 1 .. L-2
    long long tc_off[NIQ_MAX_LAYERS];  // float offset of a layer's hi block (lo follows)
    niq_bound_opts opts;
    long long n;
    const float* center;
    const float* vecs;
    int v;
    float offset;
    int* sign_out;
    float* lohi_out;
    float* xs;                         // per CTA: kTcXFloats (the next layer's X in fp32)
    int* status;
    long long mbar_polls;              // poll limit of the waits on the MMAs
};

NIQ_HOST_DEVICE int round16(int x) { return (x + 15) & ~15; }

// Relative bound of one split-precision tensor-core dot product of length n.
__device__ __forceinline__ float gamma_tc(int n) {
    const float nu = (float)(n + 2) * 4.76837158203125e-07f;  // (n + 2) 2^-21
    return __fadd_ru(__fdiv_ru(nu, 1.f - nu), 3.814697265625e-06f);  // + 2^-18 for the splits
}

// Float offset of element (r, k) of a split half in the chunked K-major layout: chunk
// k / 16 holds kTcRows rows x 16 (or out_p16 rows for weights) as core matrices.
__device__ __forceinline__ int x_index(int r, int k) {
    return (k >> 4) * (kTcRows * kTcKC) + (int)(tc::kmajor_offset(r, k & 15, kTcKC) >> 2);
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc::smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// every committed group but the most recent one complete
__device__ __forceinline__ void cp_async_wait_but_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Stable descending rank of value v at index me among s[0..n):
//   #{i : s_i > v} + #{i < me : s_i == v}   (the order of a stable descending argsort).
// Below the calling warp's window [w0, w0 + 32) every index is < me, so the test is
// s_i >= v; above it every index is > me, so it is s_i > v.  Those two ranges go in
// float4 steps; only the window compares indices.  s is 16-byte aligned, w0 <= me < n.
__device__ __forceinline__ int stable_rank(const float* s, int n, float v, int me, int w0) {
    const int lo = w0 & ~3;
    int hi = (w0 + 32 + 3) & ~3;
    if (hi > n) hi = n;
    int rk = 0;
    for (int i = 0; i < lo; i += 4) {
        const float4 q = *reinterpret_cast<const float4*>(s + i);
        rk += (q.x >= v) + (q.y >= v) + (q.z >= v) + (q.w >= v);
    }
    for (int i = lo; i < hi; ++i) rk += (s[i] > v) || (s[i] == v && i < me);
    const int n4 = n & ~3;
    int i = hi;
    for (; i < n4; i += 4) {
        const float4 q = *reinterpret_cast<const float4*>(s + i);
        rk += (q.x > v) + (q.y > v) + (q.z > v) + (q.w > v);
    }
    for (i = (i > hi ? i : hi); i < n; ++i) rk += s[i] > v;
    return rk;
}

// Column sums over the CTA's rows of one 16-column group: every thread contributes
// val[i] for its row; thread t < 16 receives the sum of column t.
template <bool C>
__device__ __forceinline__ float column_sum16(const float* val, int row, float* tr, float* part) {
    const int tid = threadIdx.x;
#pragma unroll
    for (int i = 0; i < 16; ++i) tr[row * kTcTrLD + i] = val[i];
    __syncthreads();
    const int col = tid & 15, pr = tid >> 4;
    float s = 0.f;
#pragma unroll 8
    for (int q = 0; q < 16; ++q) s = add_up<C>(s, tr[(pr * 16 + q) * kTcTrLD + col]);
    part[pr * 16 + col] = s;
    __syncthreads();
    float t = 0.f;
    if (tid < 16)
        for (int p = 0; p < kTcNT / 16; ++p) t = add_up<C>(t, part[p * 16 + tid]);
    return t;
}

template <bool C>
__global__ void __launch_bounds__(kTcNT, 1) k_wide_tc(TcArgs a) {
    extern __shared__ __align__(1024) float smem[];
    float* tr = smem + kTcOffTr;
    float* part = smem + kTcOffPart;
    float* s_base = smem + kTcOffVec;
    float* s_err = s_base + 256;
    float* s_S = s_err + 256;
    float* s_alpha = s_S + 256;
    float* s_delta = s_alpha + 256;
    float* s_drop = s_delta + 256;
    float* s_rho = s_drop + 256;    // rounding bound of the layer's dot products, per neuron
    float* s_fold = s_rho + 256;    // per input k: the bound's share before |A| (conservative)
    float* s_mag = smem + kTcOffMag;
    int* s_rank = reinterpret_cast<int*>(smem + kTcOffRank);
    __shared__ NiqSpecHeader H;
    __shared__ __align__(8) uint64_t bar[kTcStages];
    __shared__ uint32_t s_tmem;
    __shared__ float red[40];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    load_header(H, a.M.hdr);
    if (warp == 0) tc::tmem_alloc(&s_tmem, 512);
    if (tid == 0) {
        for (int i = 0; i < kTcStages; ++i) tc::mbar_init(&bar[i], 1);
        tc::fence_mbar_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = s_tmem;
    // A stage has at most one MMA commit outstanding (it is waited for before reuse):
    // bit s of `pending` marks it, bit s of `phase` is the parity of its next completion.
    // Register bit masks, not arrays indexed by the stage, which would live in local memory.
    uint32_t pending = 0u, phase = 0u;
    float* xs = a.xs + (size_t)blockIdx.x * kTcXFloats;
    const int tile = warp >> 2;
    const int row = tile * 128 + (warp & 3) * 32 + lane;  // this thread's noise row
    const uint32_t t_row = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(tile * 256);
    const int nL = H.n_layers;
    const int mode = a.opts.mode;
    const int K = mode == NIQ_MODE_AFFINE_TRUNCATE ? a.opts.truncate_count : kTcRows;
    bool fail = false;

    // A wait that gives up leaves the stage pending, so the unwind below waits for it again
    // (with the built-in limit) before the tensor memory is released.
    auto wait_stage = [&](int s, long long limit) -> bool {
        if (!((pending >> s) & 1u)) return true;
        const bool ok = tc::mbar_wait(&bar[s], (phase >> s) & 1u, limit);
        if (ok) {
            phase ^= 1u << s;
            pending &= ~(1u << s);
        }
        return ok;
    };

    for (long long b = blockIdx.x; b < a.n && !fail; b += gridDim.x) {
        const int v = a.v;
        // ---------------- layer 0 (3 inputs) on the CUDA cores (src/affine.py:109-117)
        {
            const NiqLayer L = H.layers[0];
            const float* A = a.M.w + L.a_off;
            const float g0 = C ? L.gamma : 0.f;
            float c[3], fo[3];
            for (int k = 0; k < 3; ++k) {
                c[k] = a.center[3 * b + k];
                float S = fabsf(c[k]);
                for (int r = 0; r < v; ++r) S = __fadd_ru(S, fabsf(a.vecs[3 * v * b + 3 * r + k]));
                fo[k] = C ? __fmul_ru(g0, S) : 0.f;
            }
            if (tid < NIQ_MAX_WIDTH) {
                const int j = tid;
                float bs = 0.f, rho = 0.f;
                if (j < L.out) {
                    for (int k = 0; k < 3; ++k) {
                        const float w = A[k * L.out_pad + j];
                        bs = fmaf(c[k], w, bs);
                        if (C) rho = __fmaf_ru(fo[k], fabsf(w), rho);
                    }
                    const float bj = a.M.w[L.b_off + j];
                    bs = __fadd_rn(bs, bj);
                    if (C) rho = __fadd_ru(__fmaf_ru(rho, 1.f + 2.f * g0, __fmul_ru(g0, fabsf(bj))), 5.f * NIQ_TINY);
                }
                s_base[j] = bs;
                s_err[j] = 0.f;   // the input box has no err term
                s_rho[j] = rho;
            }
            // noise rows r < v: D_rj = vecs_r . A[:, j] into TMEM lane r (warp 0, tile 0)
            if (warp == 0) {
                const int o16 = round16(L.out);
                for (int c0 = 0; c0 < o16; c0 += 32) {
                    uint32_t u[32];
#pragma unroll
                    for (int i = 0; i < 32; ++i) {
                        const int j = c0 + i;
                        float d = 0.f;
                        if (lane < v && j < L.out)
                            for (int k = 0; k < 3; ++k) d = fmaf(a.vecs[3 * v * b + 3 * lane + k], A[k * L.out_pad + j], d);
                        u[i] = __float_as_uint(d);
                    }
                    asm volatile(
                        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
                        "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
                        "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(tmem + (uint32_t)c0),
                        "r"(u[0]), "r"(u[1]), "r"(u[2]), "r"(u[3]), "r"(u[4]), "r"(u[5]), "r"(u[6]), "r"(u[7]),
                        "r"(u[8]), "r"(u[9]), "r"(u[10]), "r"(u[11]), "r"(u[12]), "r"(u[13]), "r"(u[14]), "r"(u[15]),
                        "r"(u[16]), "r"(u[17]), "r"(u[18]), "r"(u[19]), "r"(u[20]), "r"(u[21]), "r"(u[22]), "r"(u[23]),
                        "r"(u[24]), "r"(u[25]), "r"(u[26]), "r"(u[27]), "r"(u[28]), "r"(u[29]), "r"(u[30]), "r"(u[31])
                        : "memory");
                }
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            }
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
        }
        int nrows = v;

        for (int li = 0; li + 1 < nL && !fail; ++li) {
            const NiqLayer L = H.layers[li];
            const int out = L.out, o16 = round16(out);
            // ---------------- dense: noise rows on the tensor cores, base/err on CUDA cores
            if (li > 0) {
                const int i16 = round16(L.in);
                const int chunks = i16 / kTcKC;
                const int mt = (nrows + 127) >> 7;
                const float* whi = a.tcw + a.tc_off[li];
                const float* wlo = whi + (long long)chunks * o16 * kTcKC;
                const uint32_t idesc = tc::idesc_tf32(128, o16);
                float g_bs = 0.f, g_es = 0.f, g_rho = 0.f;   // column tid of the base, err, rounding rows
                // chunk c goes to stage c % kTcStages; loads run two chunks ahead of the MMAs
                auto load_chunk = [&](int c) {
                    if (c < chunks) {
                        const int s = c % kTcStages;
                        if (!wait_stage(s, a.mbar_polls)) fail = true;   // the MMAs that last read this stage
                    }
                    if (c < chunks && !fail) {   // no copy into a stage whose MMAs may still read it
                        const int s = c % kTcStages;
                        float* stg = smem + s * kTcStage;
                        const int xf4 = mt * 128 * kTcKC / 4, wf4 = o16 * kTcKC / 4;
                        const float* xsrc = xs + c * kTcRows * kTcKC;
                        const float* wsrc_h = whi + (long long)c * o16 * kTcKC;
                        const float* wsrc_l = wlo + (long long)c * o16 * kTcKC;
                        // X is kept once in fp32 and split here: half the scratch traffic of
                        // keeping hi and lo (the split weights stream with cp.async)
                        for (int i = tid; i < xf4; i += kTcNT) {
                            const float4 v = __ldcg(reinterpret_cast<const float4*>(xsrc) + i);
                            const float4 h = make_float4(tc::tf32_hi(v.x), tc::tf32_hi(v.y), tc::tf32_hi(v.z),
                                                         tc::tf32_hi(v.w));
                            *reinterpret_cast<float4*>(stg + 4 * i) = h;
                            *reinterpret_cast<float4*>(stg + kTcRows * kTcKC + 4 * i) =
                                make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
                        }
                        for (int i = tid; i < wf4; i += kTcNT) {
                            cp_async16(stg + 2 * kTcRows * kTcKC + 4 * i, wsrc_h + 4 * i);
                            cp_async16(stg + 3 * kTcRows * kTcKC + 4 * i, wsrc_l + 4 * i);
                        }
                    }
                    cp_async_commit();   // an empty group past the last chunk keeps the count
                };
                load_chunk(0);
                load_chunk(1);
                for (int c = 0; c < chunks; ++c) {
                    const int s = c % kTcStages;
                    float* stg = smem + s * kTcStage;
                    cp_async_wait_but_one();   // chunk c has landed (chunk c + 1 may be in flight)
                    tc::fence_async_smem();
                    // also: every thread is done with iteration c - 1, and all agree on `fail`
                    fail = __syncthreads_or(fail ? 1 : 0) != 0;
                    if (tid == 0 && !fail) {
                        tc::fence_after_sync();
                        const uint32_t xh = tc::smem_addr(stg), xl = xh + kTcRows * kTcKC * 4;
                        const uint32_t wh = xh + 2 * kTcRows * kTcKC * 4, wl = xh + 3 * kTcRows * kTcKC * 4;
                        const uint32_t sbo = (kTcKC / 4) * 128;
#pragma unroll
                        for (int ks = 0; ks < kTcKC / 8; ++ks) {
                            const uint64_t bh = tc::smem_desc(wh + ks * 256, 128, sbo);
                            const uint64_t bl = tc::smem_desc(wl + ks * 256, 128, sbo);
                            for (int t = 0; t < mt; ++t) {
                                const uint32_t toff = (uint32_t)t * 128 / 8 * sbo + ks * 256;
                                const uint64_t ah = tc::smem_desc(xh + toff, 128, sbo);
                                const uint64_t al = tc::smem_desc(xl + toff, 128, sbo);
                                const uint32_t d = tmem + (uint32_t)(t * 256);
                                tc::mma_tf32(d, ah, bh, idesc, (c > 0 || ks > 0) ? 1u : 0u);
                                tc::mma_tf32(d, ah, bl, idesc, 1u);
                                tc::mma_tf32(d, al, bh, idesc, 1u);
                            }
                        }
                        tc::mma_commit(&bar[s]);
                    }
                    if (!fail) pending |= 1u << s;
                    // the stage of chunk c + 2 held chunk c - 1: every thread finished with it
                    // (the barrier above); its MMAs are waited for inside load_chunk
                    load_chunk(c + 2);
                    // base, err and rounding rows while the tensor cores work
                    // (src/affine_layers.py:11-31): column j of the staged weight chunk,
                    // hi + lo = the fp32 weight exactly, against the chunk's 16 inputs
                    if (tid < out) {
                        const float* wh = stg + 2 * kTcRows * kTcKC;
                        const float* wl = stg + 3 * kTcRows * kTcKC;
#pragma unroll
                        for (int q = 0; q < kTcKC / 4; ++q) {
                            const int off = (int)(tc::kmajor_offset(tid, 4 * q, kTcKC) >> 2);
                            const float4 h = *reinterpret_cast<const float4*>(wh + off);
                            const float4 l = *reinterpret_cast<const float4*>(wl + off);
                            const float w4[4] = {h.x + l.x, h.y + l.y, h.z + l.z, h.w + l.w};
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                const int k = c * kTcKC + 4 * q + e;
                                g_bs = fmaf(s_base[k], w4[e], g_bs);
                                g_es = fmaf(s_err[k], fabsf(w4[e]), g_es);
                                if (C) g_rho = __fmaf_ru(s_fold[k], fabsf(w4[e]), g_rho);
                            }
                        }
                    }
                }
                // every MMA of the layer complete before TMEM is read; a wait that gave up
                // anywhere in the CTA ends the kernel for every thread
                for (int s = 0; s < kTcStages; ++s)
                    if (!wait_stage(s, a.mbar_polls)) fail = true;
                tc::fence_after_sync();
                fail = __syncthreads_or(fail ? 1 : 0) != 0;   // also: every thread read the old vectors
                if (fail) {
                    if (tid == 0) niq_flag_error(a.status, NIQ_ERR_TIMEOUT);
                    break;
                }
                if (tid < out) {
                    const float gam = C ? L.gamma : 0.f;
                    const float bj = a.M.w[L.b_off + tid];
                    g_bs = __fadd_rn(g_bs, bj);
                    if (C) {
                        g_es = __fmul_ru(g_es, 1.f + 2.f * gam);
                        g_rho = __fadd_ru(__fmaf_ru(g_rho, 1.f + 2.f * gam, __fmul_ru(gam, fabsf(bj))),
                                          (float)(L.in + 2) * NIQ_TINY);
                    }
                }
                if (tid < NIQ_MAX_WIDTH) {
                    s_base[tid] = tid < out ? g_bs : 0.f;
                    s_err[tid] = tid < out ? g_es : 0.f;
                    s_rho[tid] = tid < out ? g_rho : 0.f;
                }
            }
            // ---------------- activation epilogue (src/affine.py:164-193)
            const bool row_ok = row < nrows;
            const bool warp_on = (tile * 128 + (warp & 3) * 32) < nrows;
            const int nch = (o16 + 31) / 32;
            // 1. column sums of |D|
            for (int ch = 0; ch < nch; ++ch) {
                float val[32];
                if (warp_on) tc::tmem_ld32(t_row + (uint32_t)(ch * 32), val);
#pragma unroll
                for (int i = 0; i < 32; ++i) val[i] = (warp_on && row_ok && ch * 32 + i < out) ? fabsf(val[i]) : 0.f;
                const float t0 = column_sum16<C>(val, row, tr, part);
                if (tid < 16) s_S[ch * 32 + tid] = t0;
                const float t1 = column_sum16<C>(val + 16, row, tr, part);
                if (tid < 16) s_S[ch * 32 + 16 + tid] = t1;
            }
            __syncthreads();
            // 2. linearisation per column
            const int j = tid;
            float nb = 0.f, e = 0.f, aS = 0.f, alpha = 0.f, delta = 0.f;
            if (j < out) {
                const float base = s_base[j], err = s_err[j], S = s_S[j];
                const float rad = add_up<C>(add_up<C>(S, err), s_rho[j]);
                const float lo = sub_dn<C>(base, rad), hi = add_up<C>(base, rad);
                const Lin z = linearize<C>(L.act, lo, hi);
                alpha = z.a;
                delta = fabsf(z.d);
                nb = C ? fmaf(z.a, base, z.b) : __fadd_rn(__fmul_rn(z.a, base), z.b);
                aS = C ? __fmul_ru(__fmul_ru(z.a, S), 1.f + NIQ_ULP_REL) : 0.f;
                e = C ? __fmul_ru(z.a, err) : __fmul_rn(z.a, err);
                if (C) {
                    // neuron j's symbol: linearisation, the layer's rounding, alpha*base + beta, alpha*aff
                    delta = __fmaf_ru(z.a, s_rho[j], delta);
                    delta = __fmaf_ru(__fadd_ru(fabsf(nb), aS), NIQ_ULP_REL, delta);
                }
            }
            if (j < NIQ_MAX_WIDTH) { s_alpha[j] = alpha; s_delta[j] = delta; }
            __syncthreads();
            // 3. magnitudes of the candidate rows: scaled old rows, then the new rows
            const int ncand = nrows + out;
            const bool truncate = mode == NIQ_MODE_AFFINE_TRUNCATE && ncand > K;
            if (truncate) {
                float m = 0.f;
                for (int ch = 0; ch < nch; ++ch) {
                    float val[32];
                    if (warp_on) tc::tmem_ld32(t_row + (uint32_t)(ch * 32), val);
#pragma unroll
                    for (int i = 0; i < 32; ++i)
                        m += (warp_on && ch * 32 + i < out) ? fabsf(__fmul_rn(s_alpha[ch * 32 + i], val[i])) : 0.f;
                }
                if (row_ok) s_mag[row] = m;
                if (j < out) s_mag[nrows + j] = delta;
                __syncthreads();
                // 4. stable descending rank
                if (row_ok) s_rank[row] = stable_rank(s_mag, ncand, m, row, row - lane);
                if (j < out) s_rank[nrows + j] = stable_rank(s_mag, ncand, delta, nrows + j, nrows + j - lane);
            } else {
                if (row_ok) s_rank[row] = row;
                if (j < out) s_rank[nrows + j] = nrows + j;
            }
            __syncthreads();
            const int keep = truncate ? K : ncand;
            // 5. write the kept rows as the next X (split), fold the dropped ones
            const int my_rank = row_ok ? s_rank[row] : kTcRows;
            const bool kept = row_ok && my_rank < keep;
            for (int ch = 0; ch < nch; ++ch) {
                float val[32];
                if (warp_on) tc::tmem_ld32(t_row + (uint32_t)(ch * 32), val);
#pragma unroll
                for (int i = 0; i < 32; ++i)
                    val[i] = (warp_on && ch * 32 + i < out) ? __fmul_rn(s_alpha[ch * 32 + i], val[i]) : 0.f;
                if (kept) {
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const int k = ch * 32 + 4 * q;
                        if (k >= o16) break;
                        *reinterpret_cast<float4*>(xs + x_index(my_rank, k)) =
                            make_float4(val[4 * q], val[4 * q + 1], val[4 * q + 2], val[4 * q + 3]);
                    }
                }
#pragma unroll
                for (int i = 0; i < 32; ++i) val[i] = (row_ok && !kept) ? fabsf(val[i]) : 0.f;
                const float t0 = column_sum16<C>(val, row, tr, part);
                if (tid < 16) s_drop[ch * 32 + tid] = t0;
                const float t1 = column_sum16<C>(val + 16, row, tr, part);
                if (tid < 16) s_drop[ch * 32 + 16 + tid] = t1;
            }
            // new rows diag(delta): kept ones become rows of X, dropped ones go to err
            if (j < out) {
                const int rk = s_rank[nrows + j];
                if (rk < keep) {
                    for (int k = 0; k < o16; k += 4)
                        *reinterpret_cast<float4*>(xs + x_index(rk, k)) =
                            make_float4(j == k ? delta : 0.f, j == k + 1 ? delta : 0.f, j == k + 2 ? delta : 0.f,
                                        j == k + 3 ? delta : 0.f);
                } else {
                    e = add_up<C>(e, delta);
                }
            }
            __syncthreads();
            // 6. err of the activation output, with the next layer's rounding folded in
            float fold = 0.f;
            if (j < out) {
                e = add_up<C>(e, s_drop[j]);
                if (C) {
                    const NiqLayer& Ln = H.layers[li + 1];
                    if (li + 2 < nL)  // next layer: noise rows on the tensor cores, base on the CUDA cores
                        fold = __fmaf_ru(gamma_tc(Ln.in), __fadd_ru(aS, delta), __fmul_ru(Ln.gamma, fabsf(nb)));
                    else
                        fold = __fmul_ru(Ln.gamma, __fadd_ru(__fadd_ru(fabsf(nb), aS), delta));
                }
            }
            if (j < NIQ_MAX_WIDTH) {
                s_base[j] = j < out ? nb : 0.f;
                s_err[j] = j < out ? e : 0.f;
                s_fold[j] = fold;
            }
            nrows = keep;
            // X written by this layer visible to the next layer's copies; TMEM reads done
            // before the next layer's MMAs overwrite it
            __threadfence_block();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
        }
        if (fail) break;
        // ---------------- last layer (one output) on the CUDA cores
        {
            const NiqLayer L = H.layers[nL - 1];
            const float* A = a.M.w + L.a_off;
            const float gam = C ? L.gamma : 0.f;
            float part_s = 0.f;
            if (row < nrows) {
                float d = 0.f;
                for (int k = 0; k < L.in; k += 4) {
                    const int xi = x_index(row, k);
                    const float4 xv = *reinterpret_cast<const float4*>(xs + xi);
                    const float x4[4] = {xv.x, xv.y, xv.z, xv.w};
                    for (int q = 0; q < 4 && k + q < L.in; ++q) d = fmaf(x4[q], A[(k + q) * L.out_pad], d);
                }
                part_s = fabsf(d);
            }
            const float S = wide_block_sum<C>(part_s, red);
            if (tid == 0) {
                float bs = 0.f, es = 0.f, rho = 0.f;
                for (int k = 0; k < L.in; ++k) {
                    const float w = A[k * L.out_pad];
                    bs = fmaf(s_base[k], w, bs);
                    es = fmaf(s_err[k], fabsf(w), es);
                    if (C) rho = __fmaf_ru(s_fold[k], fabsf(w), rho);
                }
                const float bj = a.M.w[L.b_off];
                bs = __fadd_rn(bs, bj);
                if (C) {
                    es = __fmul_ru(es, 1.f + 2.f * gam);
                    rho = __fadd_ru(__fmaf_ru(rho, 1.f + 2.f * gam, __fmul_ru(gam, fabsf(bj))), (float)(L.in + 2) * NIQ_TINY);
                }
                const float rad = add_up<C>(add_up<C>(S, es), rho);
                const float lo = sub_dn<C>(bs, rad), hi = add_up<C>(bs, rad);
                a.sign_out[b] = sign_of_bounds(lo, hi, a.offset);
                if (a.lohi_out) { a.lohi_out[2 * b] = lo; a.lohi_out[2 * b + 1] = hi; }
            }
            __syncthreads();
        }
    }
    // unwind: wait (bounded) for MMAs still in flight, then free TMEM
    for (int s = 0; s < kTcStages; ++s)
        if (!wait_stage(s, kMbarPollsDefault) && tid == 0) niq_flag_error(a.status, NIQ_ERR_TIMEOUT);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::tmem_relinquish();
        tc::tmem_dealloc(tmem, 512);
    }
}

// Split transposed weights: for a layer, hi then lo, each [chunk][o16 rows][16] in the
// K-major core-matrix layout; zero beyond the layer's in/out.
__global__ void k_tc_split_weights(NiqModelRef M, int li, float* dst) {
    const NiqLayer L = M.hdr->layers[li];
    const int o16 = round16(L.out), i16 = round16(L.in);
    const int chunks = i16 / kTcKC;
    const long long half = (long long)chunks * o16 * kTcKC;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)o16 * i16;
         e += (long long)gridDim.x * blockDim.x) {
        const int n = (int)(e / i16), k = (int)(e % i16);
        const float w = (n < L.out && k < L.in) ? M.w[L.a_off + k * L.out_pad + n] : 0.f;
        const float h = tc::tf32_hi(w);
        const long long at = (long long)(k / kTcKC) * o16 * kTcKC + (tc::kmajor_offset(n, k % kTcKC, kTcKC) >> 2);
        dst[at] = h;
        dst[half + at] = w - h;
    }
}

static std::mutex g_tc_mu;

// The model's split weights, built on first use.
static int tc_weights(const niq_model* cm, cudaStream_t s) {
    niq_model* m = const_cast<niq_model*>(cm);
    std::lock_guard<std::mutex> lk(g_tc_mu);
    if (m->d_tc) return NIQ_OK;
    long long off = 0;
    for (int li = 0; li < m->hdr.n_layers; ++li) {
        const NiqLayer& L = m->hdr.layers[li];
        m->tc_off[li] = off;
        if (li == 0 || li + 1 == m->hdr.n_layers) continue;
        off += 2ll * round16(L.in) * round16(L.out);
    }
    void* p = nullptr;
    NIQ_CUDA(cudaMalloc(&p, (size_t)(off > 0 ? off : 1) * 4));
    for (int li = 1; li + 1 < m->hdr.n_layers; ++li) {
        k_tc_split_weights<<<64, 256, 0, s>>>(m->ref(), li, reinterpret_cast<float*>(p) + m->tc_off[li]);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) { cudaFree(p); return cuda_fail(e, "k_tc_split_weights"); }
    }
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { cudaFree(p); return cuda_fail(e, "split weights"); }
    m->d_tc = p;
    return NIQ_OK;
}

bool wide_tc_eligible(const NiqSpecHeader& H, const niq_bound_opts& o, int v) {
    if (o.mode == NIQ_MODE_AFFINE_TRUNCATE) {
        if (o.truncate_count < 1 || o.truncate_count > kTcRows) return false;
    } else if (o.mode == NIQ_MODE_AFFINE_ALL) {
        if (wide_rows_cap(H, o, v) > kTcRows) return false;
    } else {
        return false;
    }
    if (v < 1 || v > 32 || H.n_layers < 3) return false;
    if (H.layers[0].in != 3 || H.layers[H.n_layers - 1].out != 1) return false;
    for (int i = 0; i + 1 < H.n_layers; ++i)
        if (H.layers[i].act == NIQ_ACT_NONE || round16(H.layers[i].out) > NIQ_MAX_WIDTH) return false;
    return true;
}

bool wide_use_tc(const NiqSpecHeader& H, const niq_bound_opts& o, int v) {
    if (o.products == NIQ_PRODUCTS_FP32 || !wide_tc_eligible(H, o, v)) return false;
    if (o.products == NIQ_PRODUCTS_3XTF32) return true;
    // automatic: the tensor cores pay off when rows x width is dense (measured 5.3x the FP32
    // engine on 256 rows of a 256-wide network)
    const int rows = o.mode == NIQ_MODE_AFFINE_TRUNCATE ? o.truncate_count : wide_rows_cap(H, o, v);
    return H.max_width >= 128 && rows >= 64;
}

size_t wide_tc_workspace_bytes() {
    return (size_t)device_info().sm_count * kTcXFloats * 4 + 256 + 256;
}

int wide_tc_classify(const niq_model* m, const niq_bound_opts& o, long long n, const float* center, const float* vecs,
                     int v, float offset, int* sign_out, float* lohi_out, void* ws, size_t ws_bytes, cudaStream_t s) {
    NIQ_REQUIRE(wide_tc_eligible(m->hdr, o, v), NIQ_ERR_UNSUPPORTED, "model or mode not supported by the 3xTF32 engine");
    const size_t need = wide_tc_workspace_bytes();
    NIQ_REQUIRE(ws && ws_bytes >= need, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed, %zu given", need, ws_bytes);
    int rc = tc_weights(m, s);
    if (rc) return rc;
    TcArgs a;
    a.M = m->ref();
    a.tcw = reinterpret_cast<const float*>(m->d_tc);
    for (int i = 0; i < NIQ_MAX_LAYERS; ++i) a.tc_off[i] = m->tc_off[i];
    a.opts = o;
    a.n = n;
    a.center = center;
    a.vecs = vecs;
    a.v = v;
    a.offset = offset;
    a.sign_out = sign_out;
    a.lohi_out = lohi_out;
    char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~uintptr_t(255));
    a.status = reinterpret_cast<int*>(base);
    a.mbar_polls = mbar_polls();
    a.xs = reinterpret_cast<float*>(base + 256);
    NIQ_CUDA(cudaMemsetAsync(a.status, 0, sizeof(int), s));
    long long grid = device_info().sm_count;
    if (grid > n) grid = n;
    auto kern = o.conservative ? k_wide_tc<true> : k_wide_tc<false>;
    NIQ_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmemBytes));
    kern<<<(int)grid, kTcNT, kTcSmemBytes, s>>>(a);
    NIQ_CUDA(cudaGetLastError());
    int st = 0;
    NIQ_CUDA(cudaMemcpyAsync(&st, a.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    NIQ_CUDA(cudaStreamSynchronize(s));
    NIQ_REQUIRE(st == 0, st, "3xTF32 engine: a tensor-core wait timed out");
    return NIQ_OK;
}

}  // namespace niq
