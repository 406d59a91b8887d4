// tree_common.cuh -- state shared by the level-set tree kernels (k_tree.cu: FP32 tile
// engine; k_tree_tc.cu: tensor-core products): the workspace header of per-level
// counters, the node buffers and the launch parameters.
#pragma once
#include "niq_host.cuh"

namespace niq {

constexpr int kTreeMaxLevels = 64;

struct TreeWs {
    unsigned long long level_count[kTreeMaxLevels + 1];  // nodes of level L (append counter)
    unsigned long long grab[kTreeMaxLevels + 1];         // claim counter of level L
    unsigned long long n_unknown, n_interior, n_exterior, n_boxes;
    unsigned int barrier;
    int err;
    int last_level;
    int pad;
};

struct TreeBufs {
    float* lvl_lo[2];
    float* lvl_hi[2];
    float* res_lo[3];   // unknown, interior, exterior
    float* res_hi[3];
    long long cap;
};

struct TreeParams {
    int n_rounds;               // split_depth + 1, or kTreeMaxLevels
    long long thresh;           // node_terminate_thresh (huge when unset)
    float offset;
    int with_interior, with_exterior;
    int mode_interval;
    long long batch_start, batch_end;   // node range of the level this launch covers
    unsigned int barrier_polls;         // grid-barrier poll limit
    long long mbar_polls;               // mbarrier poll limit (tensor-core form)
};

__device__ __forceinline__ void put_node(float* lo, float* hi, long long i, const float* a, const float* b) {
    lo[3 * i] = a[0]; lo[3 * i + 1] = a[1]; lo[3 * i + 2] = a[2];
    hi[3 * i] = b[0]; hi[3 * i + 1] = b[1]; hi[3 * i + 2] = b[2];
}

// Launch parameters of one tree build (shared by the FP32 and tensor-core kernels).
struct TreeLaunch {
    NiqModelRef M;
    const NiqSpecHeader* host_hdr;  // host copy of the model header (launch planning)
    TreeParams P;
    TreeWs* ws;
    TreeBufs B;
    cudaStream_t s;
    bool coop;                      // one cooperative launch for every level
    long long batch;                // plain form: nodes per launch (0: whole level)
};

// The tensor-core tree (k_tree_tc.cu): affine_fixed with outward rounding, ReLU/ELU/TanH
// hidden layers of width <= 64 and a scalar output.  tree_tc_eligible says whether a
// model qualifies (and fits the shared memory); run_tree_tc launches it (all levels
// cooperatively, or the plain per-level form) and returns an NIQ status.
bool tree_tc_eligible(const NiqSpecHeader& H);
int run_tree_tc(const TreeLaunch& T);

}  // namespace niq
