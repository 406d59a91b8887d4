// niq_common.cuh -- shared definitions of the GB300 range-analysis kernels.
//
// Packed spec ("NIQ1"): the reference's dict spec (src/mlp.py:14-24) flattened by the host
// layer into a fixed header followed by fp32 weights.  Each dense layer stores A as
// (in_pad x out_pad) row-major (A is applied as x @ A + b, src/mlp.py:253-257) and b as
// out_pad floats, both zero-padded to multiples of 4 and 16-byte aligned; the activation
// that follows the dense op is fused into the layer record.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/niq.h"

#define NIQ_HOST_DEVICE __host__ __device__ __forceinline__

struct NiqLayer {
    int32_t in, out;          // logical dims
    int32_t in_pad, out_pad;  // multiples of 4
    int32_t act;              // NIQ_ACT_*
    int32_t a_off;            // float offset of A in the weight area
    int32_t b_off;            // float offset of b (always present, zeros if the spec had none)
    float   gamma;            // (in+1)u / (1-(in+1)u) rounded up, u = 2^-24
};

struct NiqSpecHeader {
    uint32_t magic;
    int32_t  version;
    int32_t  n_layers;
    int32_t  in_dim;
    int32_t  out_dim;
    int32_t  max_width;       // max over layers of out_pad (and in_pad)
    int32_t  n_weight_floats; // size of the weight area
    int32_t  reserved;
    NiqLayer layers[NIQ_MAX_LAYERS];
};
static_assert(sizeof(NiqLayer) == 32, "layer record is 32 bytes");
static_assert(sizeof(NiqSpecHeader) % 16 == 0, "header keeps the weights 16B aligned");

// A model as the kernels see it: header and weights in device memory.
struct NiqModelRef {
    const NiqSpecHeader* hdr;
    const float* w;
};

// Host-side handle (opaque to C callers).
struct niq_model {
    NiqSpecHeader hdr;        // host copy
    void* d_blob;             // device: header + weights
    size_t bytes;
    int device;
    void* d_tc = nullptr;     // device: split transposed weights for the tensor cores (built on first use)
    long long tc_off[NIQ_MAX_LAYERS] = {};
    NiqModelRef ref() const {
        NiqModelRef r;
        r.hdr = reinterpret_cast<const NiqSpecHeader*>(d_blob);
        r.w = reinterpret_cast<const float*>(reinterpret_cast<const char*>(d_blob) + sizeof(NiqSpecHeader));
        return r;
    }
};

// ---------------------------------------------------------------------------------
// Directed rounding.  With `C` false the helpers round to nearest, which reproduces the
// reference's arithmetic; with `C` true they round outward so enclosures stay valid.
// ---------------------------------------------------------------------------------
template <bool C> __device__ __forceinline__ float add_up(float a, float b) { return C ? __fadd_ru(a, b) : a + b; }
template <bool C> __device__ __forceinline__ float add_dn(float a, float b) { return C ? __fadd_rd(a, b) : a + b; }
template <bool C> __device__ __forceinline__ float sub_up(float a, float b) { return C ? __fsub_ru(a, b) : a - b; }
template <bool C> __device__ __forceinline__ float sub_dn(float a, float b) { return C ? __fsub_rd(a, b) : a - b; }
template <bool C> __device__ __forceinline__ float mul_up(float a, float b) { return C ? __fmul_ru(a, b) : a * b; }
template <bool C> __device__ __forceinline__ float fma_up(float a, float b, float c) { return C ? __fmaf_ru(a, b, c) : fmaf(a, b, c); }
template <bool C> __device__ __forceinline__ float fma_dn(float a, float b, float c) { return C ? __fmaf_rd(a, b, c) : fmaf(a, b, c); }

// Relative bound on one round-to-nearest operation, doubled for headroom: 2^-23.
#define NIQ_ULP_REL 1.1920928955078125e-07f
// Absolute allowance for underflow in one product (2^-148).
#define NIQ_TINY 2.802596928649634e-45f

// ---------------------------------------------------------------------------------
// Error reporting from kernels: the first error code wins.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ void niq_flag_error(int* flag, int code) {
    if (flag) atomicCAS(flag, 0, code);
}

// Grid-wide barrier for cooperative launches (all CTAs co-resident).  `ctr` counts
// arrivals monotonically; `epoch` is the number of barriers this CTA has passed.  The
// spin is bounded: after max_polls polls (2^28 by default, seconds) it records
// NIQ_ERR_TIMEOUT in `err` and returns false so the caller can unwind instead of
// hanging; max_polls = 0 gives up without polling.
__device__ __forceinline__ bool niq_grid_barrier(unsigned int* ctr, unsigned int nblocks,
                                                 unsigned int& epoch, int* err, unsigned int max_polls) {
    __syncthreads();
    bool ok = true;
    if (threadIdx.x == 0) {
        epoch += 1;
        const unsigned int target = epoch * nblocks;
        __threadfence();
        atomicAdd(ctr, 1u);
        unsigned int polls = 0;
        while (true) {
            if (polls++ >= max_polls) { niq_flag_error(err, NIQ_ERR_TIMEOUT); ok = false; break; }
            unsigned int v = *((volatile unsigned int*)ctr);
            if (v >= target) break;
            if (err && *((volatile int*)err) != 0) { ok = false; break; }
            __nanosleep(64);
        }
        __threadfence();
    } else {
        epoch += 1;
    }
    ok = __syncthreads_and(ok ? 1 : 0);
    return ok;
}

// Warp-aggregated append: every lane with `want` gets a distinct slot of *counter.
__device__ __forceinline__ long long niq_warp_append(unsigned long long* counter, bool want) {
    const unsigned int mask = __ballot_sync(__activemask(), want);
    if (!want) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    const int rank = __popc(mask & ((1u << lane) - 1u));
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    return (long long)(base + rank);
}

// Warp-aggregated reservation of `per` consecutive slots for each lane with `want`; all
// 32 lanes of the warp must call it.  Returns the first slot or -1.
__device__ __forceinline__ long long niq_warp_reserve(unsigned long long* counter, bool want, int per) {
    const unsigned int mask = __ballot_sync(0xffffffffu, want);
    if (!want) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    const int rank = __popc(mask & ((1u << lane) - 1u));
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned long long)(__popc(mask) * per));
    base = __shfl_sync(mask, base, leader);
    return (long long)base + (long long)rank * per;
}
