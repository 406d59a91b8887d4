// k_wide_tc.cu -- the growing-term engine ('affine_truncate', 'affine_all';
// src/affine.py:127-193) with its dense products on the tensor cores.
//
// One CTA (8 warps, one per SM) propagates one box at a time.  A box's noise rows are the
// M dimension of a GEMM  D[rows x out] = X[rows x in] * A[in x out]  with up to 256 rows
// (two M = 128 tiles), computed by tcgen05.mma kind::tf32 as three split-precision
// products  Xhi*Ahi + Xhi*Alo + Xlo*Ahi  accumulated in fp32 in tensor memory (TMEM,
// 512 columns: tile t at columns 256 t).  X (split on the way in) and the split weights are
// streamed through a three-stage shared-memory ring in K chunks of 16, two chunks ahead:
// a chunk's weights (hi and lo, contiguous in global memory) by two bulk copies of the
// tensor memory accelerator that one thread issues, counted on the stage's "full"
// mbarrier.  The MMAs are issued by one thread and tracked with a second mbarrier per
// stage.  The base and err rows (one vector
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
constexpr int kTcOffTr = kTcStages * kTcStage;           // per-warp 32 x 17 transpose tiles
constexpr int kTcOffVec = kTcOffTr + kTcRows * kTcTrLD;     // per-neuron vectors
constexpr int kTcOffOut = kTcOffVec + 8 * 256;             // output layer's column, scan counts, select digit
constexpr int kTcOffNew = kTcOffOut + 512;                 // kept new rows: neuron, delta
constexpr int kTcSmemFloats = kTcOffNew + 512;
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

// Column sums over a warp's 32 rows (lane = row) of 32 values per lane: lane l receives
// the sum of column l.  The values go through the warp's own 32 x 17 shared-memory tile,
// 16 columns at a time (conflict-free rows and columns), with warp-level sync only.
template <bool C>
__device__ __forceinline__ float warp_column_sum32(const float* val, float* wt, int lane) {
    float res = 0.f;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
#pragma unroll
        for (int i = 0; i < 16; ++i) wt[lane * kTcTrLD + i] = val[16 * h + i];
        __syncwarp();
        const int col = lane & 15, r0 = (lane >> 4) * 16;
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < 16; ++q) s = add_up<C>(s, wt[(r0 + q) * kTcTrLD + col]);
        s = add_up<C>(s, __shfl_xor_sync(0xffffffffu, s, 16));
        if ((lane >> 4) == h) res = s;
        __syncwarp();
    }
    return res;
}

// Radix-select step for one lane of the searching warp.  The lane owns the 8 digits
// 255 - 8 lane - e (e = 0..7, descending) of the 256-bin histogram h; `above` keys have a
// larger digit.  If the kk-th largest key has one of the lane's digits, the lane writes
// that digit to sel[0] and the number of keys with a larger digit to sel[1].
__device__ __forceinline__ void kth_digit_in_lane(const int* h, int lane, int above, int kk, int* sel) {
    for (int e = 0; e < 8; ++e) {
        const int d = 255 - 8 * lane - e;
        if (above < kk && kk <= above + h[d]) {
            sel[0] = d;
            sel[1] = above;
            return;
        }
        above += h[d];
    }
}

// The K-th largest (1 <= K <= number of valid keys) of the block's keys, two per thread
// (k0 if v0, k1 if v1): nonnegative floats as bit patterns, whose unsigned order is their
// order (a NaN counts as the largest).  Four passes over 8-bit digits, most significant
// first.  A pass histograms the digit of the keys that match the digits found so far
// (lanes with the same digit add once), then one warp finds the digit that holds the
// K-th largest: each lane owns 8 digits in descending order and a shuffle scan gives the
// number of keys above them.  Two histogram buffers alternate, so clearing the next one
// overlaps the search.  Returns the key; *n_gt receives the number of keys above it.
__device__ uint32_t block_kth_largest(uint32_t k0, bool v0, uint32_t k1, bool v1, int K, int* hist, int* sel,
                                      int* n_gt) {
    const int tid = threadIdx.x, lane = tid & 31;
    hist[tid] = 0;   // buffer 0 (kTcNT == 256 bins)
    __syncthreads();
    uint32_t prefix = 0u, mask = 0u;
    int kk = K;
#pragma unroll 1
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = 24 - 8 * pass;
        int* h = hist + 256 * (pass & 1);
        const bool m0 = v0 && (k0 & mask) == prefix, m1 = v1 && (k1 & mask) == prefix;
        {
            const uint32_t d = m0 ? (k0 >> shift) & 255u : 256u + (uint32_t)lane;   // unmatched: a group of one
            const uint32_t grp = __match_any_sync(0xffffffffu, d);
            if (m0 && lane == __ffs(grp) - 1) atomicAdd(&h[d], __popc(grp));
        }
        {
            const uint32_t d = m1 ? (k1 >> shift) & 255u : 256u + (uint32_t)lane;
            const uint32_t grp = __match_any_sync(0xffffffffu, d);
            if (m1 && lane == __ffs(grp) - 1) atomicAdd(&h[d], __popc(grp));
        }
        __syncthreads();
        if (tid < 32) {
            int tot = 0;
#pragma unroll
            for (int e = 0; e < 8; ++e) tot += h[255 - 8 * lane - e];
            int incl = tot;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= off) incl += y;
            }
            kth_digit_in_lane(h, lane, incl - tot, kk, sel);
        } else {
            int* hn = hist + 256 * ((pass + 1) & 1);
            for (int i = tid - 32; i < 256; i += kTcNT - 32) hn[i] = 0;
        }
        __syncthreads();
        kk -= sel[1];
        prefix |= (uint32_t)sel[0] << shift;
        mask |= 255u << shift;
    }
    *n_gt = K - kk;
    return prefix;
}

// Exclusive prefix counts of two flags in candidate order: f0 of candidate tid (an old
// row) and f1 of the new-row candidate tid, which follows every old row.  p0 / p1: the set
// flags before this thread's candidates; t0: the set f0 flags; t: all set flags.
__device__ __forceinline__ void block_scan_pair(bool f0, bool f1, int* cnt, int& p0, int& p1, int& t0, int& t) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t b0 = __ballot_sync(0xffffffffu, f0), b1 = __ballot_sync(0xffffffffu, f1);
    if (lane == 0) {
        cnt[warp] = __popc(b0);
        cnt[8 + warp] = __popc(b1);
    }
    __syncthreads();
    int a0 = 0, a1 = 0, c0 = 0, c1 = 0;
#pragma unroll
    for (int w = 0; w < kTcNT / 32; ++w) {
        const int x0 = cnt[w], x1 = cnt[8 + w];
        a0 += w < warp ? x0 : 0;
        a1 += w < warp ? x1 : 0;
        c0 += x0;
        c1 += x1;
    }
    const uint32_t lt = (1u << lane) - 1u;
    p0 = a0 + __popc(b0 & lt);
    p1 = c0 + a1 + __popc(b1 & lt);
    t0 = c0;
    t = c0 + c1;
    __syncthreads();   // the counts may be rewritten by the next call
}

template <bool C>
__global__ void __launch_bounds__(kTcNT, 1) k_wide_tc(TcArgs a) {
    extern __shared__ __align__(1024) float smem[];
    float* tr = smem + kTcOffTr;
    float* s_base = smem + kTcOffVec;
    float* s_err = s_base + 256;
    float* s_alpha = s_err + 256;
    float* s_rho = s_alpha + 256;   // rounding bound of the layer's dot products, per neuron
    float* s_fold = s_rho + 256;    // per input k: the bound's share before |A| (conservative)
    float* s_aout = smem + kTcOffOut;                                   // output layer's column
    int* s_cnt = reinterpret_cast<int*>(smem + kTcOffOut + 256);        // 16 scan counts
    int* s_sel = s_cnt + 16;                                            // select: digit, keys above
    int* s_newj = reinterpret_cast<int*>(smem + kTcOffNew);             // kept new rows: neuron
    float* s_newd = smem + kTcOffNew + 256;                             //                delta
    int* hist = reinterpret_cast<int*>(smem + 2048);                    // in the idle stage buffers
    __shared__ NiqSpecHeader H;
    __shared__ __align__(8) uint64_t bar[kTcStages];    // the stage's MMAs completed
    __shared__ __align__(8) uint64_t full[kTcStages];   // the stage's weight copies landed
    __shared__ uint32_t s_tmem;
    __shared__ float red[40];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    load_header(H, a.M.hdr);
    if (warp == 0) tc::tmem_alloc(&s_tmem, 512);
    if (tid == 0) {
        for (int i = 0; i < kTcStages; ++i) {
            tc::mbar_init(&bar[i], 1);
            tc::mbar_init(&full[i], 1);
        }
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
    // The same for the weight copies: bit s of `fphase` is the parity of full[s]'s next
    // completion; bit s of `fpend` (kept by the thread that issues the copies, lane 0 of warp
    // 1, so the MMA issuer's warp is not held up by them) marks a copy in flight.
    uint32_t fphase = 0u, fpend = 0u;
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
        int nrows = v;      // noise rows of the layer input: n_old from the scratch, then the new ones
        int n_old = v;      // rows of X held in the scratch (the rest are diag(delta) rows, built while staging)
        float out_part = 0.f;   // |output-layer product| of this thread's kept rows (last hidden layer)

        for (int li = 0; li + 1 < nL && !fail; ++li) {
            const NiqLayer L = H.layers[li];
            const int out = L.out, o16 = round16(out);
            const bool last_hidden = (li + 2 == nL);
            // ---------------- dense: noise rows on the tensor cores, base/err on CUDA cores
            if (li > 0) {
                const int i16 = round16(L.in);
                const int chunks = i16 / kTcKC;
                const int mt = (nrows + 127) >> 7;
                const float* whi = a.tcw + a.tc_off[li];
                const float* wlo = whi + (long long)chunks * o16 * kTcKC;
                const uint32_t idesc = tc::idesc_tf32(128, o16);
                float g_bs = 0.f, g_es = 0.f, g_rho = 0.f;   // column tid of the base, err, rounding rows
                // X of a chunk in this thread's float4 slots q (the chunk's float4 tid + 256 q):
                // row 8 (tid / 32) + tid % 8 + 64 q, inputs 16 c + 4 ((tid / 8) % 4) .. + 3 (the
                // K-major core-matrix layout).  Rows below n_old come from the scratch, fetched into
                // registers one chunk ahead; the new rows diag(delta) are built from their neuron
                // and delta; rows past nrows are zero.
                float4 pf[4];
                const int slots = 2 * mt;
                auto row_of = [&](int q) { return 8 * (tid >> 5) + (tid & 7) + 64 * q; };
                auto fetch_x = [&](int c) {
                    if (c >= chunks) return;
                    const float4* src = reinterpret_cast<const float4*>(xs + c * kTcRows * kTcKC);
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (q < slots && row_of(q) < n_old) pf[q] = __ldcg(src + tid + 256 * q);
                };
                // chunk c goes to stage c % kTcStages; staging runs two chunks ahead of the MMAs
                auto load_chunk = [&](int c) {
                    if (c < chunks) {
                        const int s = c % kTcStages;
                        if (!wait_stage(s, a.mbar_polls)) fail = true;   // the MMAs that last read this stage
                    }
                    if (c < chunks && !fail) {   // no copy into a stage whose MMAs may still read it
                        const int s = c % kTcStages;
                        float* stg = smem + s * kTcStage;
                        if (tid == 32) {   // the chunk's split weights: o16 x 16 floats each, 1 KB aligned
                            const uint32_t wbytes = (uint32_t)(o16 * kTcKC * 4);
                            tc::mbar_arrive_expect_tx(&full[s], 2 * wbytes);
                            tc::bulk_g2s(stg + 2 * kTcRows * kTcKC, whi + (long long)c * o16 * kTcKC, wbytes, &full[s]);
                            tc::bulk_g2s(stg + 3 * kTcRows * kTcKC, wlo + (long long)c * o16 * kTcKC, wbytes, &full[s]);
                            fpend |= 1u << s;
                        }
                        const int k0 = c * kTcKC + 4 * ((tid >> 3) & 3);
                        // X is kept once in fp32 and split here
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            if (q >= slots) break;
                            const int r = row_of(q);
                            float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
                            if (r < n_old) {
                                x = pf[q];
                            } else if (r < nrows) {
                                const int jn = s_newj[r - n_old];
                                const float dn = s_newd[r - n_old];
                                x = make_float4(jn == k0 ? dn : 0.f, jn == k0 + 1 ? dn : 0.f, jn == k0 + 2 ? dn : 0.f,
                                                jn == k0 + 3 ? dn : 0.f);
                            }
                            const float4 h = make_float4(tc::tf32_hi(x.x), tc::tf32_hi(x.y), tc::tf32_hi(x.z),
                                                         tc::tf32_hi(x.w));
                            const int i = tid + 256 * q;
                            *reinterpret_cast<float4*>(stg + 4 * i) = h;
                            *reinterpret_cast<float4*>(stg + kTcRows * kTcKC + 4 * i) =
                                make_float4(x.x - h.x, x.y - h.y, x.z - h.z, x.w - h.w);
                        }
                    }
                };
                fetch_x(0);
                load_chunk(0);
                fetch_x(1);
                load_chunk(1);
                fetch_x(2);
                for (int c = 0; c < chunks; ++c) {
                    const int s = c % kTcStages;
                    float* stg = smem + s * kTcStage;
                    if (!fail) {   // chunk c's weights have landed (chunk c + 1's may be in flight)
                        if (tc::mbar_wait(&full[s], (fphase >> s) & 1u, a.mbar_polls)) {
                            fphase ^= 1u << s;
                            fpend &= ~(1u << s);
                        } else {
                            fail = true;
                        }
                    }
                    tc::fence_async_smem();   // this thread's X stores, before the MMAs read them
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
                    // (the barrier above); its MMAs are waited for inside load_chunk.  The X of
                    // chunk c + 2 was fetched an iteration ago; the next fetch covers the MMAs.
                    load_chunk(c + 2);
                    fetch_x(c + 3);
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
            // Thread tid owns noise row tid (TMEM lane tid % 128 of tile tid / 128) and neuron tid.
            // The stage buffers are idle until the next layer's first copy: they hold the
            // per-warp column sums and the selection histograms meanwhile.
            const bool row_ok = row < nrows;
            const bool warp_on = warp * 32 < nrows;   // warp-uniform: the warp holds rows of the box
            const int nw_on = (nrows + 31) >> 5;
            const int nch = (o16 + 31) / 32;
            float* wsum = smem;                        // [8 warps][256 columns]
            float* wt = tr + warp * 32 * kTcTrLD;      // this warp's transpose tile
            if (last_hidden && tid < out) s_aout[tid] = a.M.w[H.layers[li + 1].a_off + tid * H.layers[li + 1].out_pad];
            // 1. column sums of |D|: per warp over its 32 rows, then over the warps
            if (warp_on) {
                for (int ch = 0; ch < nch; ++ch) {
                    float val[32];
                    tc::tmem_ld32(t_row + (uint32_t)(ch * 32), val);
#pragma unroll
                    for (int i = 0; i < 32; ++i) val[i] = (row_ok && ch * 32 + i < out) ? fabsf(val[i]) : 0.f;
                    wsum[warp * 256 + ch * 32 + lane] = warp_column_sum32<C>(val, wt, lane);
                }
            }
            __syncthreads();
            // 2. linearisation per column
            const int j = tid;
            float nb = 0.f, e = 0.f, aS = 0.f, alpha = 0.f, delta = 0.f;
            if (j < out) {
                float S = 0.f;
                for (int w = 0; w < nw_on; ++w) S = add_up<C>(S, wsum[w * 256 + j]);
                const float base = s_base[j], err = s_err[j];
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
            if (j < NIQ_MAX_WIDTH) s_alpha[j] = alpha;   // 0 past the layer's width
            __syncthreads();
            // 3. magnitudes of the candidate rows (src/affine.py:141-142): the scaled old rows
            //    (thread = row) and the new rows diag(delta) (thread = neuron)
            const int ncand = nrows + out;
            const bool truncate = mode == NIQ_MODE_AFFINE_TRUNCATE && ncand > K;
            bool keep0 = row_ok, keep1 = j < out;
            if (truncate) {
                float m = 0.f;
                if (warp_on) {
                    for (int ch = 0; ch < nch; ++ch) {
                        float val[32];
                        tc::tmem_ld32(t_row + (uint32_t)(ch * 32), val);
#pragma unroll
                        for (int i = 0; i < 32; i += 4) {
                            const float4 al = *reinterpret_cast<const float4*>(s_alpha + ch * 32 + i);
                            const float a4[4] = {al.x, al.y, al.z, al.w};
#pragma unroll
                            for (int u = 0; u < 4; ++u)
                                m += (ch * 32 + i + u < out) ? fabsf(__fmul_rn(a4[u], val[i + u])) : 0.f;
                        }
                    }
                }
                // 4. keep the K largest (src/affine.py:150-155): the K-th largest magnitude T by a
                //    radix select; every candidate above T and the first candidates equal to T, in
                //    candidate order (old rows, then new rows), as a stable descending sort keeps them
                const uint32_t k0 = __float_as_uint(m), k1 = __float_as_uint(delta);
                int n_gt;
                const uint32_t T = block_kth_largest(k0, row_ok, k1, j < out, K, hist, s_sel, &n_gt);
                int q0, q1, t0, tt;
                block_scan_pair(row_ok && k0 == T, j < out && k1 == T, s_cnt, q0, q1, t0, tt);
                keep0 = row_ok && (k0 > T || (k0 == T && q0 < K - n_gt));
                keep1 = j < out && (k1 > T || (k1 == T && q1 < K - n_gt));
            }
            // kept rows are packed in candidate order: old rows to 0 .. n_keep_old - 1, new after
            int p0, p1, n_keep_old, keep;
            block_scan_pair(keep0, keep1, s_cnt, p0, p1, n_keep_old, keep);
            // 5. kept old rows, scaled by alpha, become the next X (or, after the last hidden
            //    layer, their products with the output layer's column); dropped rows go to err
            //    as column sums of |alpha D| (src/affine.py:157-160)
            float d_out = 0.f;
            if (warp_on) {
                const bool any_drop = __any_sync(0xffffffffu, row_ok && !keep0);
                for (int ch = 0; ch < nch; ++ch) {
                    float val[32];
                    tc::tmem_ld32(t_row + (uint32_t)(ch * 32), val);
#pragma unroll
                    for (int i = 0; i < 32; i += 4) {
                        const float4 al = *reinterpret_cast<const float4*>(s_alpha + ch * 32 + i);
                        const float a4[4] = {al.x, al.y, al.z, al.w};
#pragma unroll
                        for (int u = 0; u < 4; ++u)
                            val[i + u] = (ch * 32 + i + u < out) ? __fmul_rn(a4[u], val[i + u]) : 0.f;
                    }
                    if (keep0) {
                        if (last_hidden) {
#pragma unroll
                            for (int i = 0; i < 32; ++i)
                                if (ch * 32 + i < out) d_out = fmaf(val[i], s_aout[ch * 32 + i], d_out);
                        } else {
#pragma unroll
                            for (int q = 0; q < 8; ++q) {
                                const int k = ch * 32 + 4 * q;
                                if (k >= o16) break;
                                *reinterpret_cast<float4*>(xs + x_index(p0, k)) =
                                    make_float4(val[4 * q], val[4 * q + 1], val[4 * q + 2], val[4 * q + 3]);
                            }
                        }
                    }
                    if (any_drop) {
#pragma unroll
                        for (int i = 0; i < 32; ++i) val[i] = (row_ok && !keep0) ? fabsf(val[i]) : 0.f;
                        wsum[warp * 256 + ch * 32 + lane] = warp_column_sum32<C>(val, wt, lane);
                    } else {
                        wsum[warp * 256 + ch * 32 + lane] = 0.f;
                    }
                }
            }
            // new rows diag(delta): kept ones are built into X while the next layer stages it,
            // dropped ones go to err
            float d_new = 0.f;
            if (j < out) {
                if (keep1) {
                    if (last_hidden) d_new = __fmul_rn(delta, s_aout[j]);
                    else {
                        s_newj[p1 - n_keep_old] = j;
                        s_newd[p1 - n_keep_old] = delta;
                    }
                } else {
                    e = add_up<C>(e, delta);
                }
            }
            if (last_hidden) out_part = add_up<C>(keep0 ? fabsf(d_out) : 0.f, keep1 ? fabsf(d_new) : 0.f);
            __syncthreads();
            // 6. err of the activation output, with the next layer's rounding folded in
            float fold = 0.f;
            if (j < out) {
                float drop = 0.f;
                for (int w = 0; w < nw_on; ++w) drop = add_up<C>(drop, wsum[w * 256 + j]);
                e = add_up<C>(e, drop);
                if (C) {
                    const NiqLayer& Ln = H.layers[li + 1];
                    if (!last_hidden)  // next layer: noise rows on the tensor cores, base on the CUDA cores
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
            n_old = n_keep_old;
            // X written by this layer visible to the next layer's copies; TMEM reads done
            // before the next layer's MMAs overwrite it; the stage buffers' use as sums and
            // histograms ordered before the next layer's bulk copies into them
            __threadfence_block();
            tc::fence_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
        }
        if (fail) break;
        // ---------------- last layer (one output) on the CUDA cores: its noise-row products
        // came out of the last hidden layer's epilogue (out_part); base, err and rounding
        // rows as dot products over the layer's inputs
        {
            const NiqLayer L = H.layers[nL - 1];
            const float* A = a.M.w + L.a_off;
            const float gam = C ? L.gamma : 0.f;
            float pb = 0.f, pe = 0.f, pr = 0.f;
            if (tid < L.in) {
                const float w = A[tid * L.out_pad];
                pb = __fmul_rn(s_base[tid], w);
                pe = C ? __fmul_ru(s_err[tid], fabsf(w)) : __fmul_rn(s_err[tid], fabsf(w));
                if (C) pr = __fmul_ru(s_fold[tid], fabsf(w));
            }
            // warp sums, then thread 0 adds the warps' (rounded up where conservative; the base
            // row is rounded to nearest, its rounding is in rho)
            float v4[4] = {out_part, pb, pe, pr};
#pragma unroll
            for (int off = 16; off > 0; off >>= 1)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float y = __shfl_down_sync(0xffffffffu, v4[q], off);
                    v4[q] = q == 1 ? v4[q] + y : add_up<C>(v4[q], y);
                }
            if (lane == 0) {
#pragma unroll
                for (int q = 0; q < 4; ++q) red[8 * q + warp] = v4[q];
            }
            __syncthreads();
            if (tid == 0) {
                float S = 0.f, bs0 = 0.f, es0 = 0.f, rho0 = 0.f;
                for (int w = 0; w < kTcNT / 32; ++w) {
                    S = add_up<C>(S, red[w]);
                    bs0 += red[8 + w];
                    es0 = add_up<C>(es0, red[16 + w]);
                    rho0 = add_up<C>(rho0, red[24 + w]);
                }
                const float bj = a.M.w[L.b_off];
                const float bs = __fadd_rn(bs0, bj);
                float es = es0, rho = rho0;
                if (C) {
                    es = __fmul_ru(es, 1.f + 2.f * gam);
                    rho = __fadd_ru(__fmaf_ru(rho, 1.f + 2.f * gam, __fmul_ru(gam, fabsf(bj))), (float)(L.in + 2) * NIQ_TINY);
                }
                const float rad = add_up<C>(add_up<C>(S, es), rho);
                const float lo = sub_dn<C>(bs, rad), hi = add_up<C>(bs, rad);
                a.sign_out[b] = sign_of_bounds(lo, hi, a.offset);
                if (a.lohi_out) { a.lohi_out[2 * b] = lo; a.lohi_out[2 * b + 1] = hi; }
            }
            __syncthreads();   // red is rewritten by the next box
        }
    }
    // unwind: wait (bounded) for MMAs and weight copies still in flight, then free TMEM
    for (int s = 0; s < kTcStages; ++s) {
        if (!wait_stage(s, kMbarPollsDefault) && tid == 0) niq_flag_error(a.status, NIQ_ERR_TIMEOUT);
        if (((fpend >> s) & 1u) && !tc::mbar_wait(&full[s], (fphase >> s) & 1u, kMbarPollsDefault))
            niq_flag_error(a.status, NIQ_ERR_TIMEOUT);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::tmem_relinquish();
        tc::tmem_dealloc(tmem, 512);
    }
}

// ---------------------------------------------------------------- roofline calibration
// The dense step alone: per 16-deep chunk, the three split products of two M = 128 tiles
// at N = 256 from the three-stage ring, exactly as k_wide_tc issues them, with no
// staging and no epilogue.  One CTA per SM; the rate is the tensor pipe's tf32 ceiling
// for this instruction sequence on this GPU.
__device__ int g_tc_rate_status;

__global__ void __launch_bounds__(kTcNT, 1) k_tc_rate(int chunks, long long polls) {
    extern __shared__ __align__(1024) float smem[];
    __shared__ __align__(8) uint64_t bar[kTcStages];
    __shared__ uint32_t s_tmem;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < kTcStages * kTcStage; i += kTcNT) smem[i] = 1e-3f * (float)(i & 7);
    if (warp == 0) tc::tmem_alloc(&s_tmem, 512);
    if (tid == 0) {
        for (int i = 0; i < kTcStages; ++i) tc::mbar_init(&bar[i], 1);
        tc::fence_mbar_init();
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = s_tmem;
    if (tid == 0) {
        const uint32_t idesc = tc::idesc_tf32(128, 256);
        const uint32_t sbo = (kTcKC / 4) * 128;
        uint32_t phase = 0u;
        bool ok = true;
        int issued = 0, waited = 0;   // commits made, commits waited for (in order)
        for (int c = 0; c < chunks && ok; ++c) {
            const int s = c % kTcStages;
            if (c >= kTcStages) {   // the stage's previous MMAs, as before a restage
                ok = tc::mbar_wait(&bar[s], (phase >> s) & 1u, polls);
                if (!ok) break;
                phase ^= 1u << s;
                ++waited;
            }
            const uint32_t xh = tc::smem_addr(smem + s * kTcStage), xl = xh + kTcRows * kTcKC * 4;
            const uint32_t wh = xh + 2 * kTcRows * kTcKC * 4, wl = xh + 3 * kTcRows * kTcKC * 4;
#pragma unroll
            for (int ks = 0; ks < kTcKC / 8; ++ks) {
                const uint64_t bh = tc::smem_desc(wh + ks * 256, 128, sbo);
                const uint64_t bl = tc::smem_desc(wl + ks * 256, 128, sbo);
#pragma unroll
                for (int t = 0; t < 2; ++t) {
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
            ++issued;
        }
        // the commits not yet waited for, in order; with the built-in limit after a
        // give-up, so no MMA is in flight when the tensor memory is released
        for (; waited < issued; ++waited) {
            const int s = waited % kTcStages;
            if (!tc::mbar_wait(&bar[s], (phase >> s) & 1u, ok ? polls : kMbarPollsDefault)) {
                ok = false;
                if (!tc::mbar_wait(&bar[s], (phase >> s) & 1u, kMbarPollsDefault)) break;
            }
            phase ^= 1u << s;
        }
        if (!ok) atomicExch(&g_tc_rate_status, NIQ_ERR_TIMEOUT);
    }
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

using namespace niq;

extern "C" int niq_tc_tf32_rate(int32_t chunks, float* tflops_out, void* stream) {
    NIQ_REQUIRE(tflops_out && chunks >= 1 && chunks <= (1 << 20), NIQ_ERR_INVALID_ARG, "need 1 <= chunks <= 2^20");
    cudaStream_t s = as_stream(stream);
    const int grid = device_info().sm_count;
    const size_t smem = (size_t)kTcStages * kTcStage * 4;
    NIQ_CUDA(cudaFuncSetAttribute(k_tc_rate, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int zero = 0;
    NIQ_CUDA(cudaMemcpyToSymbolAsync(g_tc_rate_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s));
    k_tc_rate<<<grid, kTcNT, smem, s>>>(chunks < 64 ? chunks : 64, mbar_polls());   // warm-up
    NIQ_CUDA(cudaGetLastError());
    cudaEvent_t e0, e1;
    NIQ_CUDA(cudaEventCreate(&e0));
    NIQ_CUDA(cudaEventCreate(&e1));
    NIQ_CUDA(cudaEventRecord(e0, s));
    k_tc_rate<<<grid, kTcNT, smem, s>>>(chunks, mbar_polls());
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_fail(e, "k_tc_rate");
    int st = 0;
    NIQ_CUDA(cudaMemcpyFromSymbol(&st, g_tc_rate_status, sizeof(int)));
    NIQ_REQUIRE(st == 0, st, "tensor-core rate probe: an MMA wait timed out");
    const double flop = 2.0 * 128 * 256 * kTcKC * 2 * 3 * (double)chunks * grid;
    *tflops_out = (float)(flop / (ms * 1e-3) / 1e12);
    return NIQ_OK;
}
