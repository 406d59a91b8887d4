// k_sample.cu -- kd_tree.sample_surface and kd_tree.bulk_properties
// (src/kd_tree.py:220-292, 804-863): Monte Carlo over the nodes of a level-set tree.
//
// Candidates: node index uniform over the nodes, position uniform inside the node
// (jax.random.randint / uniform in the reference).  The random numbers come from a
// counter-based generator: the splitmix64 finaliser (Steele, Lea and Flood 2014) of
// (seed, stream, index), so every candidate is reproducible from the seed alone and
// rounds need no state.  The reference draws from JAX's threefry stream instead, so
// individual samples differ; the distributions are the same.
//
// sample_surface keeps candidates with |f| < width, appended with a warp-aggregated
// counter up to the requested count; bulk_properties sums, over candidates with f < 0,
// the count and the positions, and adds the interior nodes' exact volume and moments.
#include "niq_host.cuh"

namespace niq {

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// uniform on [0, 1) with 24 random bits
__device__ __forceinline__ float u01(unsigned long long seed, unsigned long long stream, unsigned long long i) {
    const unsigned long long h = mix64(seed ^ mix64(stream * 0x100000001B3ull + i));
    return (float)(h >> 40) * 5.9604644775390625e-08f;   // 2^-24
}

// n candidates of round `round`: node uniform over [0, n_nodes), point uniform in it
__global__ void k_sample_candidates(long long n_nodes, const float* __restrict__ lo, const float* __restrict__ hi,
                                    long long n, unsigned long long seed, unsigned long long round,
                                    float* __restrict__ xyz) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long base = round * 4;
        long long node = (long long)(u01(seed, base, i) * (float)n_nodes);
        if (node >= n_nodes) node = n_nodes - 1;
        for (int k = 0; k < 3; ++k) {
            const float l = lo[3 * node + k], h = hi[3 * node + k];
            xyz[3 * i + k] = __fadd_rn(l, __fmul_rn(u01(seed, base + 1 + k, i), __fsub_rn(h, l)));
        }
    }
}

// appends candidates with |f| < width to out (capacity cap) through *count
__global__ void k_sample_keep(long long n, const float* __restrict__ xyz, const float* __restrict__ val, float width,
                              float* __restrict__ out, unsigned long long* count, long long cap) {
    for (long long i0 = blockIdx.x * (long long)blockDim.x; i0 < n; i0 += (long long)gridDim.x * blockDim.x) {
        const long long i = i0 + threadIdx.x;
        const bool want = i < n && fabsf(val[i]) < width;
        const long long pos = niq_warp_append(count, want);
        if (want && pos < cap)
            for (int k = 0; k < 3; ++k) out[3 * pos + k] = xyz[3 * i + k];
    }
}

// sums (in double) over candidates with f < 0: count and positions -> acc[0..3]
__global__ void k_mass_boundary(long long n, const float* __restrict__ xyz, const float* __restrict__ val,
                                double* acc) {
    double c = 0.0, s[3] = {0.0, 0.0, 0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (val[i] < 0.f) {
            c += 1.0;
            for (int k = 0; k < 3; ++k) s[k] += xyz[3 * i + k];
        }
    for (int off = 16; off > 0; off >>= 1) {
        c += __shfl_xor_sync(0xffffffffu, c, off);
        for (int k = 0; k < 3; ++k) s[k] += __shfl_xor_sync(0xffffffffu, s[k], off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(acc, c);
        for (int k = 0; k < 3; ++k) atomicAdd(acc + 1 + k, s[k]);
    }
}

// sums over nodes: volume and volume * center -> acc[0..3]
__global__ void k_node_moments(long long n, const float* __restrict__ lo, const float* __restrict__ hi, double* acc) {
    double m = 0.0, s[3] = {0.0, 0.0, 0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double w0 = (double)hi[3 * i] - lo[3 * i], w1 = (double)hi[3 * i + 1] - lo[3 * i + 1],
                     w2 = (double)hi[3 * i + 2] - lo[3 * i + 2];
        const double v = w0 * w1 * w2;
        m += v;
        for (int k = 0; k < 3; ++k) s[k] += v * 0.5 * ((double)lo[3 * i + k] + hi[3 * i + k]);
    }
    for (int off = 16; off > 0; off >>= 1) {
        m += __shfl_xor_sync(0xffffffffu, m, off);
        for (int k = 0; k < 3; ++k) s[k] += __shfl_xor_sync(0xffffffffu, s[k], off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(acc, m);
        for (int k = 0; k < 3; ++k) atomicAdd(acc + 1 + k, s[k]);
    }
}

static int grid_of(long long n) {
    long long g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

}  // namespace niq

using namespace niq;

extern "C" {

size_t niq_sample_workspace_size(int64_t n_candidates) {
    return (size_t)(n_candidates > 0 ? n_candidates : 0) * 16 + 1024;
}

int niq_sample_surface(const niq_model* model, int64_t n_nodes, const float* node_lower, const float* node_upper,
                       int64_t n_samples, float width, uint64_t seed, int64_t n_per_round, int32_t max_rounds,
                       float* samples_out, int64_t* n_found_out, void* workspace, size_t workspace_bytes, void* stream) {
    NIQ_REQUIRE(model && node_lower && node_upper && samples_out && n_found_out, NIQ_ERR_INVALID_ARG, "null argument");
    NIQ_REQUIRE(n_nodes >= 1 && n_samples >= 0 && n_per_round >= 1 && max_rounds >= 1, NIQ_ERR_INVALID_ARG,
                "need nodes, a sample count >= 0, a round size >= 1 and max_rounds >= 1");
    const size_t need = niq_sample_workspace_size(n_per_round);
    NIQ_REQUIRE(workspace && workspace_bytes >= need, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed", need);
    cudaStream_t s = as_stream(stream);
    char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
    unsigned long long* count = reinterpret_cast<unsigned long long*>(base);
    float* xyz = reinterpret_cast<float*>(base + 256);
    float* val = xyz + 3 * n_per_round;
    NIQ_CUDA(cudaMemsetAsync(count, 0, sizeof(unsigned long long), s));
    unsigned long long found = 0;
    for (int r = 0; r < max_rounds && (long long)found < n_samples; ++r) {
        k_sample_candidates<<<grid_of(n_per_round), 256, 0, s>>>(n_nodes, node_lower, node_upper, n_per_round, seed,
                                                               (unsigned long long)r, xyz);
        NIQ_CUDA(cudaGetLastError());
        int rc = niq_eval_points(model, n_per_round, xyz, val, stream);
        if (rc) return rc;
        k_sample_keep<<<grid_of(n_per_round), 256, 0, s>>>(n_per_round, xyz, val, width, samples_out, count, n_samples);
        NIQ_CUDA(cudaGetLastError());
        NIQ_CUDA(cudaMemcpyAsync(&found, count, sizeof(found), cudaMemcpyDeviceToHost, s));
        NIQ_CUDA(cudaStreamSynchronize(s));
    }
    *n_found_out = (long long)found < n_samples ? (long long)found : n_samples;
    NIQ_REQUIRE((long long)found >= n_samples, NIQ_ERR_TIMEOUT, "%lld of %lld samples after %d rounds",
                (long long)found, (long long)n_samples, max_rounds);
    return NIQ_OK;
}

int niq_bulk_properties(const niq_model* model, int64_t n_interior, const float* interior_lower,
                        const float* interior_upper, int64_t n_boundary, const float* boundary_lower,
                        const float* boundary_upper, int64_t n_sample, uint64_t seed, double* mass_centroid_out,
                        void* workspace, size_t workspace_bytes, void* stream) {
    NIQ_REQUIRE(model && mass_centroid_out, NIQ_ERR_INVALID_ARG, "null argument");
    NIQ_REQUIRE(n_interior >= 0 && n_boundary >= 0 && n_sample >= 0, NIQ_ERR_INVALID_ARG, "negative size");
    const size_t need = niq_sample_workspace_size(n_sample);
    NIQ_REQUIRE(workspace && workspace_bytes >= need, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed", need);
    cudaStream_t s = as_stream(stream);
    char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
    double* acc = reinterpret_cast<double*>(base);   // [interior m, mx, my, mz, boundary c, sx, sy, sz, boundary volume ...]
    float* xyz = reinterpret_cast<float*>(base + 256);
    float* val = xyz + 3 * n_sample;
    NIQ_CUDA(cudaMemsetAsync(acc, 0, 16 * sizeof(double), s));
    if (n_interior > 0) {
        NIQ_REQUIRE(interior_lower && interior_upper, NIQ_ERR_INVALID_ARG, "null interior arrays");
        k_node_moments<<<grid_of(n_interior), 256, 0, s>>>(n_interior, interior_lower, interior_upper, acc);
        NIQ_CUDA(cudaGetLastError());
    }
    if (n_boundary > 0 && n_sample > 0) {
        NIQ_REQUIRE(boundary_lower && boundary_upper, NIQ_ERR_INVALID_ARG, "null boundary arrays");
        k_node_moments<<<grid_of(n_boundary), 256, 0, s>>>(n_boundary, boundary_lower, boundary_upper, acc + 8);
        k_sample_candidates<<<grid_of(n_sample), 256, 0, s>>>(n_boundary, boundary_lower, boundary_upper, n_sample,
                                                            seed, 0ull, xyz);
        NIQ_CUDA(cudaGetLastError());
        int rc = niq_eval_points(model, n_sample, xyz, val, stream);
        if (rc) return rc;
        k_mass_boundary<<<grid_of(n_sample), 256, 0, s>>>(n_sample, xyz, val, acc + 4);
        NIQ_CUDA(cudaGetLastError());
    }
    double h[16];
    NIQ_CUDA(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s));
    NIQ_CUDA(cudaStreamSynchronize(s));
    // src/kd_tree.py:826-862: boundary volume / n_sample per accepted sample
    const double vps = n_sample > 0 ? h[8] / (double)n_sample : 0.0;
    const double mass = h[0] + vps * h[4];
    mass_centroid_out[0] = mass;
    for (int k = 0; k < 3; ++k) mass_centroid_out[1 + k] = mass > 0 ? (h[1 + k] + vps * h[5 + k]) / mass : 0.0;
    return NIQ_OK;
}

}  // extern "C"
