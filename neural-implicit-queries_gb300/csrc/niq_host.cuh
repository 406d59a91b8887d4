// niq_host.cuh -- host-side helpers shared by the entry points: error state, launch
// planning (shared-memory split between item state and weights), width dispatch.
#pragma once
#include <cstdio>
#include <cstring>
#include <string>
#include "niq_common.cuh"
#include "tile_engine.cuh"

namespace niq {

void set_error(const char* fmt, ...);
// Launch parameters an autotuner may set (niq_tune_set); 0 means the built-in choice.
enum TuneParam : int {
    kTuneBatchedChunk = 0, kTuneBatchedCtasPerSm = 1, kTuneTreeCtasPerSm = 2, kTuneBarrierPolls = 3,
    kTuneMbarPolls = 4, kTuneRayColumns = 5, kTuneCount = 6
};
int tune_value(int param);
// Poll limits of the bounded device-side waits: the tuned value minus one, or the
// built-in limits (grid barrier 2^28 polls, mbarrier 2^24) when it is 0.
constexpr unsigned int kBarrierPollsDefault = 1u << 28;
constexpr long long kMbarPollsDefault = 1ll << 24;
inline unsigned int barrier_polls() {
    const int v = tune_value(kTuneBarrierPolls);
    return v > 0 ? (unsigned int)(v - 1) : kBarrierPollsDefault;
}
inline long long mbar_polls() {
    const int v = tune_value(kTuneMbarPolls);
    return v > 0 ? (long long)(v - 1) : kMbarPollsDefault;
}
// Checks a packed spec header against its byte size (capi.cu).
int validate_spec(const NiqSpecHeader& H, size_t bytes);
int cuda_fail(cudaError_t e, const char* where);

#define NIQ_CUDA(call)                                                 \
    do {                                                               \
        cudaError_t _e = (call);                                       \
        if (_e != cudaSuccess) return ::niq::cuda_fail(_e, #call);     \
    } while (0)

#define NIQ_REQUIRE(cond, code, ...)                                   \
    do {                                                               \
        if (!(cond)) { ::niq::set_error(__VA_ARGS__); return (code); } \
    } while (0)

struct DeviceInfo {
    int device = -1;
    int sm_count = 0;
    int smem_optin = 0;      // max dynamic shared memory per block (bytes)
    int smem_per_sm = 0;
};
const DeviceInfo& device_info();

// Shared-memory budget per CTA used when planning (2 CTAs per SM).
constexpr int kSmemBudget = 110 * 1024;
constexpr int kNT = 256;

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int max_layer_floats(const NiqSpecHeader& H) {
    int m = 0;
    for (int i = 0; i < H.n_layers; ++i) m = m > layer_floats(H.layers[i]) ? m : layer_floats(H.layers[i]);
    return m;
}

// Width class -> threads per item (8 columns per thread).
inline int tpi_for_width(int w) { return w <= 32 ? 4 : w <= 64 ? 8 : w <= 128 ? 16 : 32; }

struct SmemPlan {
    size_t bytes = 0;     // dynamic shared memory per CTA
    int fixed_floats = 0; // floats before the weight buffer
    int sw_cap = 0;       // weight buffer capacity (floats)
    bool resident = false;
};

// fixed_floats: item state + outputs + caller scratch (floats, multiple of 4).
// weight_floats: total floats of all models that should be resident together.
inline SmemPlan plan_smem(int fixed_floats, int weight_floats, int max_layer, int budget = kSmemBudget) {
    SmemPlan p;
    fixed_floats = (fixed_floats + 3) & ~3;
    p.fixed_floats = fixed_floats;
    const int avail = budget / 4 - fixed_floats;
    if (weight_floats <= avail) {
        p.resident = true;
        p.sw_cap = weight_floats;
    } else {
        p.resident = false;
        // at least 4 rows of the widest layer plus its bias
        const int want = max_layer < avail ? max_layer : avail;
        p.sw_cap = want;
    }
    p.bytes = (size_t)(fixed_floats + p.sw_cap) * 4;
    const DeviceInfo& d = device_info();
    if (d.smem_optin > 0 && p.bytes > (size_t)d.smem_optin) p.bytes = d.smem_optin;
    return p;
}

// Shared-memory budget of one CTA of `nt` threads: kSmemBudget while the kernel's
// registers let two CTAs share an SM, else (one CTA per SM anyway) the per-block maximum,
// so that the weights can stay resident instead of being restaged every layer.
template <class K>
inline int smem_budget(K kernel, int nt) {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return kSmemBudget;
    const int warp_regs = (fa.numRegs * 32 + 255) / 256 * 256;   // allocated per warp in units of 256
    if (2 * warp_regs * (nt / 32) <= 65536) return kSmemBudget;
    const DeviceInfo& d = device_info();
    const int b = d.smem_optin - (int)fa.sharedSizeBytes;
    return b > kSmemBudget ? b : kSmemBudget;
}

template <class K>
inline int prepare_kernel(K kernel, size_t smem) {
    NIQ_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return NIQ_OK;
}

template <class K>
inline int persistent_grid(K kernel, int nt, size_t smem, long long work_tiles, int* grid, int max_per_sm = 0) {
    int per_sm = 0;
    NIQ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, nt, smem));
    if (per_sm < 1) { set_error("kernel does not fit on an SM (smem %zu)", smem); return NIQ_ERR_UNSUPPORTED; }
    if (max_per_sm > 0 && per_sm > max_per_sm) per_sm = max_per_sm;
    long long g = (long long)per_sm * device_info().sm_count;
    if (work_tiles < g) g = work_tiles;
    if (g < 1) g = 1;
    *grid = (int)g;
    return NIQ_OK;
}

// Copy of the model header into shared memory by the whole CTA.
__device__ __forceinline__ void load_header(NiqSpecHeader& H, const NiqSpecHeader* g) {
    const int4* s = reinterpret_cast<const int4*>(g);
    int4* d = reinterpret_cast<int4*>(&H);
    for (int i = threadIdx.x; i < (int)(sizeof(NiqSpecHeader) / 16); i += blockDim.x) d[i] = __ldg(s + i);
}

}  // namespace niq

// Width dispatch: instantiates BODY with TPI = 4, 8, 16, 32.
#define NIQ_DISPATCH_TPI(tpi, ...)                               \
    switch (tpi) {                                               \
        case 4: { constexpr int TPI = 4; __VA_ARGS__; } break;   \
        case 8: { constexpr int TPI = 8; __VA_ARGS__; } break;   \
        case 16: { constexpr int TPI = 16; __VA_ARGS__; } break; \
        default: { constexpr int TPI = 32; __VA_ARGS__; } break; \
    }
