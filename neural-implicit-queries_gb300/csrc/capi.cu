// capi.cu -- library-level entry points: errors, device info, model upload.
#include <cstdarg>
#include <cmath>
#include <atomic>
#include <mutex>
#include "niq_host.cuh"

namespace niq {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_fail(cudaError_t e, const char* where) {
    set_error("CUDA error %s (%d) in %s", cudaGetErrorString(e), (int)e, where);
    return NIQ_ERR_CUDA;
}

static std::atomic<int> g_tune[kTuneCount];

int tune_value(int param) { return (param >= 0 && param < kTuneCount) ? g_tune[param].load() : 0; }

static DeviceInfo g_info[64];
static std::mutex g_info_mu;

const DeviceInfo& device_info() {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    std::lock_guard<std::mutex> lk(g_info_mu);
    DeviceInfo& d = g_info[dev];
    if (d.device != dev) {
        d.device = dev;
        cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&d.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaDeviceGetAttribute(&d.smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    }
    return d;
}

// Validates a packed spec.  Mirrors the checks the reference performs while walking
// the dict (src/mlp.py:117-144): every op resolvable, shapes chained.
int validate_spec(const NiqSpecHeader& H, size_t bytes) {
    NIQ_REQUIRE(H.magic == NIQ_SPEC_MAGIC, NIQ_ERR_BAD_SPEC, "bad spec magic 0x%08x", H.magic);
    NIQ_REQUIRE(H.n_layers >= 1 && H.n_layers <= NIQ_MAX_LAYERS, NIQ_ERR_BAD_SPEC, "bad layer count %d", H.n_layers);
    NIQ_REQUIRE(H.in_dim == 3, NIQ_ERR_BAD_SPEC, "input dimension must be 3, got %d", H.in_dim);
    NIQ_REQUIRE(H.out_dim == 1, NIQ_ERR_BAD_SPEC, "output dimension must be 1, got %d", H.out_dim);
    NIQ_REQUIRE(H.n_weight_floats >= 0 && bytes == sizeof(NiqSpecHeader) + (size_t)H.n_weight_floats * 4,
                NIQ_ERR_BAD_SPEC, "spec size %zu does not match %d weights", bytes, H.n_weight_floats);
    int prev = 3;
    int maxw = 0;
    for (int i = 0; i < H.n_layers; ++i) {
        const NiqLayer& L = H.layers[i];
        NIQ_REQUIRE(L.in == prev, NIQ_ERR_BAD_SPEC, "layer %d input %d does not match previous output %d", i, L.in, prev);
        NIQ_REQUIRE(L.out >= 1 && L.out <= NIQ_MAX_WIDTH, NIQ_ERR_UNSUPPORTED, "layer %d width %d outside [1, %d]", i, L.out, NIQ_MAX_WIDTH);
        NIQ_REQUIRE(L.in_pad == ((L.in + 3) & ~3) && L.out_pad == ((L.out + 3) & ~3), NIQ_ERR_BAD_SPEC, "layer %d padding", i);
        NIQ_REQUIRE(L.act >= NIQ_ACT_NONE && L.act <= NIQ_ACT_TANH, NIQ_ERR_BAD_SPEC, "layer %d activation %d", i, L.act);
        NIQ_REQUIRE(L.a_off % 4 == 0 && L.b_off % 4 == 0 && L.a_off >= 0 && L.b_off >= 0 &&
                        L.a_off + L.in_pad * L.out_pad <= H.n_weight_floats && L.b_off + L.out_pad <= H.n_weight_floats,
                    NIQ_ERR_BAD_SPEC, "layer %d weight offsets out of range", i);
        NIQ_REQUIRE(L.gamma >= 0.f && L.gamma < 0.01f, NIQ_ERR_BAD_SPEC, "layer %d rounding factor", i);
        maxw = maxw > L.out_pad ? maxw : L.out_pad;
        maxw = maxw > L.in_pad ? maxw : L.in_pad;
        prev = L.out;
    }
    NIQ_REQUIRE(prev == 1, NIQ_ERR_BAD_SPEC, "last layer must have one output");
    NIQ_REQUIRE(H.layers[H.n_layers - 1].act == NIQ_ACT_NONE, NIQ_ERR_BAD_SPEC, "last layer must be linear");
    NIQ_REQUIRE(H.max_width == maxw, NIQ_ERR_BAD_SPEC, "max width %d != %d", H.max_width, maxw);
    return NIQ_OK;
}

// FP32 FMA ceiling: every thread of two 256-thread CTAs per SM runs eight independent chains
// of packed fp32x2 FMAs (the tile engine's dense instruction) on registers, no memory.
__global__ void __launch_bounds__(256) k_fma_rate(int iters, float seed, float* sink) {
    float2 a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = make_float2(seed + (float)(threadIdx.x + i), seed - (float)i);
    const float2 m = make_float2(0.999999f, 1.000001f), c = make_float2(1e-7f, -1e-7f);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < 16; ++u)
#pragma unroll
            for (int i = 0; i < 8; ++i) a[i] = __ffma2_rn(a[i], m, c);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += a[i].x + a[i].y;
    if (s == 1234.5f) sink[blockIdx.x] = s;   // keeps the chains live; never true for these values
}

}  // namespace niq

using namespace niq;

extern "C" {

const char* niq_last_error(void) { return g_err; }

int niq_version(void) { return 1; }

int niq_tune_set(int32_t param, int32_t value) {
    NIQ_REQUIRE(param >= 0 && param < kTuneCount, NIQ_ERR_INVALID_ARG, "unknown tuning parameter %d", param);
    NIQ_REQUIRE(value >= 0, NIQ_ERR_INVALID_ARG, "tuning values are >= 0 (0: built-in choice)");
    NIQ_REQUIRE(param != kTuneBatchedChunk || value == 0 || (value >= 32 && value <= 4096), NIQ_ERR_INVALID_ARG,
                "batched chunk must be in [32, 4096]");
    NIQ_REQUIRE(param != kTuneRayColumns || value == 0 || value == 4 || value == 8, NIQ_ERR_INVALID_ARG,
                "ray-cast columns per thread must be 4 or 8 (0: built-in choice)");
    g_tune[param].store(value);
    return NIQ_OK;
}

int niq_tune_get(int32_t param, int32_t* value) {
    NIQ_REQUIRE(param >= 0 && param < kTuneCount && value, NIQ_ERR_INVALID_ARG, "bad argument");
    *value = g_tune[param].load();
    return NIQ_OK;
}

int niq_device_info(int32_t* sm_count, int32_t* max_smem_per_block) {
    const DeviceInfo& d = device_info();
    if (sm_count) *sm_count = d.sm_count;
    if (max_smem_per_block) *max_smem_per_block = d.smem_optin;
    return d.sm_count > 0 ? NIQ_OK : NIQ_ERR_CUDA;
}

int niq_model_create(const void* packed_spec, size_t bytes, niq_model** out) {
    NIQ_REQUIRE(packed_spec && out, NIQ_ERR_INVALID_ARG, "null argument");
    NIQ_REQUIRE(bytes >= sizeof(NiqSpecHeader), NIQ_ERR_BAD_SPEC, "spec too short (%zu bytes)", bytes);
    NiqSpecHeader H;
    memcpy(&H, packed_spec, sizeof(H));
    int rc = validate_spec(H, bytes);
    if (rc) return rc;
    niq_model* m = new niq_model();
    m->hdr = H;
    m->bytes = bytes;
    cudaGetDevice(&m->device);
    cudaError_t e = cudaMalloc(&m->d_blob, bytes);
    if (e != cudaSuccess) { delete m; return cuda_fail(e, "cudaMalloc(model)"); }
    e = cudaMemcpy(m->d_blob, packed_spec, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { cudaFree(m->d_blob); delete m; return cuda_fail(e, "cudaMemcpy(model)"); }
    *out = m;
    return NIQ_OK;
}

int niq_model_destroy(niq_model* model) {
    if (!model) return NIQ_OK;
    if (model->d_tc) cudaFree(model->d_tc);
    cudaError_t e = cudaFree(model->d_blob);
    delete model;
    return e == cudaSuccess ? NIQ_OK : cuda_fail(e, "cudaFree(model)");
}

int niq_model_info(const niq_model* model, int32_t* max_width, int32_t* n_layers) {
    NIQ_REQUIRE(model, NIQ_ERR_INVALID_ARG, "null model");
    if (max_width) *max_width = model->hdr.max_width;
    if (n_layers) *n_layers = model->hdr.n_layers;
    return NIQ_OK;
}

}  // extern "C"

extern "C" int niq_fp32_fma_rate(int32_t iters, float* tflops_out, void* stream) {
    NIQ_REQUIRE(tflops_out && iters >= 1 && iters <= (1 << 22), NIQ_ERR_INVALID_ARG, "need 1 <= iters <= 2^22");
    cudaStream_t s = as_stream(stream);
    const int grid = 2 * device_info().sm_count;
    k_fma_rate<<<grid, 256, 0, s>>>(iters < 64 ? iters : 64, 1.f, nullptr);   // warm-up
    NIQ_CUDA(cudaGetLastError());
    cudaEvent_t e0, e1;
    NIQ_CUDA(cudaEventCreate(&e0));
    NIQ_CUDA(cudaEventCreate(&e1));
    NIQ_CUDA(cudaEventRecord(e0, s));
    k_fma_rate<<<grid, 256, 0, s>>>(iters, 1.f, nullptr);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_fail(e, "k_fma_rate");
    // 2 FMAs per packed instruction, 2 FLOP per FMA
    const double flop = 4.0 * 8 * 16 * (double)iters * 256 * grid;
    *tflops_out = (float)(flop / (ms * 1e-3) / 1e12);
    return NIQ_OK;
}
