/*
 * niq.h -- C ABI of the GB300 range-analysis query engine (libniq.so).
 *
 * Drop-in boundary for the range-analysis hot path of nmwsharp/neural-implicit-queries.
 * The reference is pure Python/JAX and has no FFI of its own; each entry point below
 * replaces one reference function (cited as src/<file>:<line> inside that project).
 * A Python host layer re-exposes the reference's names and signatures on top of it.
 *
 * Conventions
 *  - Every function returns an int status: NIQ_OK (0) or a negative NIQ_ERR_* code;
 *    niq_last_error() gives a one-line message for the calling thread.
 *  - All array arguments are DEVICE pointers owned by the caller (float32, int32 or
 *    int64 as typed), row-major; points and box centers are (n, 3).
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).  Calls
 *    are asynchronous on that stream unless documented otherwise ("syncs").
 *  - Scratch memory is caller-provided (`workspace`, `workspace_bytes`); each query has a
 *    *_workspace_size() helper.  A workspace too small for the work found at run time
 *    returns NIQ_ERR_CAPACITY and leaves outputs undefined.
 *  - A model handle is immutable after niq_model_create and may be shared by streams;
 *    one workspace must not be used by two calls in flight at once.
 */
#ifndef NIQ_H
#define NIQ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------- */
#define NIQ_OK                 0
#define NIQ_ERR_INVALID_ARG   -1  /* bad pointer, size or option                      */
#define NIQ_ERR_BAD_SPEC      -2  /* packed spec malformed (src/mlp.py:131,142)       */
#define NIQ_ERR_CUDA          -3  /* CUDA runtime error                               */
#define NIQ_ERR_CAPACITY      -4  /* workspace / output capacity exceeded             */
#define NIQ_ERR_TIMEOUT       -5  /* a bounded device-side wait gave up               */
#define NIQ_ERR_UNSUPPORTED   -6  /* mode / width / depth outside the built kernels   */

/* ---- sign codes: src/implicit_function.py:11-13 --------------------------------- */
#define NIQ_SIGN_UNKNOWN   0
#define NIQ_SIGN_POSITIVE  1
#define NIQ_SIGN_NEGATIVE  2

/* ---- range-arithmetic modes: src/implicit_mlp_utils.py:12-64, src/affine.py:62-76 -- */
#define NIQ_MODE_INTERVAL         0
#define NIQ_MODE_AFFINE_FIXED     1
#define NIQ_MODE_AFFINE_TRUNCATE  2
#define NIQ_MODE_AFFINE_APPEND    3
#define NIQ_MODE_AFFINE_ALL       4
#define NIQ_MODE_SLOPE_INTERVAL   5

/* ---- activation codes inside a packed spec ---------------------------------------- */
#define NIQ_ACT_NONE  0
#define NIQ_ACT_RELU  1   /* src/affine_layers.py:34-56   */
#define NIQ_ACT_ELU   2   /* src/affine_layers.py:59-97   */
#define NIQ_ACT_TANH  3   /* no reference rule: new        */

#define NIQ_MAX_LAYERS 32
#define NIQ_MAX_WIDTH  256
#define NIQ_SPEC_MAGIC 0x3151494eu /* "NIQ1" */

typedef struct niq_model niq_model;

/* How the growing-term modes (AFFINE_TRUNCATE, AFFINE_ALL) form their dense products:
 * AUTO picks the tensor cores where the noise rows x layer width are dense (hidden
 * widths >= 128 and >= 64 rows), FP32 forces FP32 FMA, 3XTF32 forces the tensor cores
 * (split-precision tf32 products; needs every hidden layer activated, widths <= 256 and
 * at most 256 noise rows).  3XTF32 also puts the level-set tree in affine_fixed with
 * outward rounding on the tensor cores (niq_tree_engine); the other modes and queries
 * use FP32 FMA. */
#define NIQ_PRODUCTS_AUTO    0
#define NIQ_PRODUCTS_FP32    1
#define NIQ_PRODUCTS_3XTF32  2

/* Options of one range-analysis evaluation (the reference's AffineContext,
 * src/affine.py:62-76).  truncate_count is used by AFFINE_TRUNCATE, n_append by
 * AFFINE_APPEND.  conservative != 0 adds the outward rounding-error terms.  products:
 * NIQ_PRODUCTS_*. */
typedef struct niq_bound_opts {
    int32_t mode;
    int32_t truncate_count;
    int32_t n_append;
    int32_t conservative;
    int32_t products;
} niq_bound_opts;

/* The cast options dict of src/queries.py:23-36. */
typedef struct niq_cast_opts {
    float   hit_eps;
    float   max_dist;
    int32_t n_max_step;
    int32_t n_substeps;
    float   safety_factor;
    float   interval_grow_fac;
    float   interval_shrink_fac;
    float   interval_init_size;
} niq_cast_opts;

/* ---- library ---------------------------------------------------------------------- */
const char* niq_last_error(void);
int niq_version(void);
/* Launch parameters an autotuner may set for the whole process (0 = the built-in
 * choice): NIQ_TUNE_BATCHED_CHUNK queries per work chunk of niq_batched_closest_point
 * (32..4096, default 128); NIQ_TUNE_BATCHED_CTAS_PER_SM and NIQ_TUNE_TREE_CTAS_PER_SM cap
 * the resident CTAs per SM of those persistent kernels.  No counterpart in the
 * reference (its batch sizes are arguments, its launches XLA's). */
#define NIQ_TUNE_BATCHED_CHUNK        0
#define NIQ_TUNE_BATCHED_CTAS_PER_SM  1
#define NIQ_TUNE_TREE_CTAS_PER_SM     2
/* Limits of the bounded device-side waits, as 1 + the number of polls a wait may make
 * before it gives up with NIQ_ERR_TIMEOUT (0 = the built-in limit: 2^28 polls of a grid
 * barrier, 2^24 of an mbarrier on tensor-core work; 1 = give up at once).  The waits are
 * those of the persistent tree and intersection kernels (grid barrier between levels)
 * and of the tensor-core kernels (completion of their MMAs; a kernel that gave up still
 * waits for its MMAs with the built-in limit before it releases tensor memory). */
#define NIQ_TUNE_BARRIER_POLLS        3
#define NIQ_TUNE_MBAR_POLLS           4
/* Output columns per thread of the per-ray cast's tile (niq_cast_rays and
 * niq_cast_rays_plain in interval, affine_fixed and slope_interval): 8, or 4 (the narrow
 * tile: twice the lanes per ray, each with half the work, for models at most 32 wide).
 * 0 = the built-in choice: 4 for models at most 32 wide in slope_interval, or when the
 * cast has at most 512 rays per SM.  Results are identical either way. */
#define NIQ_TUNE_RAY_COLUMNS          5
int niq_tune_set(int32_t param, int32_t value);
int niq_tune_get(int32_t param, int32_t* value);
/* Number of SMs and resident-CTA counts of the current device (for workspace sizing). */
int niq_device_info(int32_t* sm_count, int32_t* max_smem_per_block);
/* The tensor-core ceiling of the 3xTF32 engine on the current device (no counterpart in
 * the reference: it calibrates the roofline of the tensor-core kernels).  One CTA per SM
 * issues, per 16-deep chunk, the engine's dense step -- the three split products of two
 * M = 128 tiles at N = 256 from its three-stage shared-memory ring -- for `chunks` chunks
 * with no staging and no epilogue; *tflops_out receives the measured rate in tf32
 * TFLOP/s.  Synchronises `stream`; allocates no device memory. */
int niq_tc_tf32_rate(int32_t chunks, float* tflops_out, void* stream);
/* The FP32 FMA ceiling of the current device (no counterpart in the reference: it
 * calibrates the roofline of the FP32 tile engine).  Two 256-thread CTAs per SM run eight
 * independent chains of packed fp32x2 FMAs per thread, 128 per iteration, for `iters`
 * iterations on registers only; *tflops_out receives the measured rate in fp32 TFLOP/s
 * (2 FLOP per FMA).  Synchronises `stream`; allocates no device memory. */
int niq_fp32_fma_rate(int32_t iters, float* tflops_out, void* stream);

/* ---- models: the dict spec of src/mlp.py:14-24,117-144 packed by the host layer ---- */
/* Validates and uploads a packed spec (host memory) to the current device.
 * Replaces the trace-time spec walk of src/mlp.py:96-113 (func_from_spec/eval_spec). */
int niq_model_create(const void* packed_spec, size_t bytes, niq_model** out);
int niq_model_destroy(niq_model* model);
/* Widest layer and number of dense layers of a model. */
int niq_model_info(const niq_model* model, int32_t* max_width, int32_t* n_layers);

/* ---- point evaluation: ImplicitFunction.__call__ (src/affine.py:26-28,
 *      src/mlp.py:253-347) --------------------------------------------------------- */
int niq_eval_points(const niq_model* model, int64_t n, const float* xyz, float* out,
                    void* stream);
/* Value (val_out (n), may be NULL) and gradient (grad_out (n,3)) of the MLP at n points:
 * the derivative jax.jacfwd takes of the point function for outward_normal(...,
 * method='autodiff') (src/render.py:61-63), by forward-mode tangents with JAX's
 * activation derivatives (relu' = 0 at x <= 0, elu' = exp(x) at x <= 0). */
int niq_eval_gradients(const niq_model* model, int64_t n, const float* xyz, float* val_out,
                       float* grad_out, void* stream);

/* ---- range bounds: classify_general_box (src/affine.py:34-55,
 *      src/slope_interval.py:29-51).  center (n,3), vecs (n,v,3) with 1 <= v <= 3.
 *      sign_out (n) gets NIQ_SIGN_*, lo_hi_out (n,2) optional (may be NULL).
 *      Growing-term modes (TRUNCATE/APPEND/ALL) need a workspace of
 *      niq_classify_workspace_size() bytes; the fixed modes accept NULL. ---------- */
size_t niq_classify_workspace_size(const niq_model* model, const niq_bound_opts* opts,
                                   int64_t n, int32_t v);
int niq_classify_boxes(const niq_model* model, const niq_bound_opts* opts, int64_t n,
                       const float* center, const float* vecs, int32_t v, float offset,
                       int32_t* sign_out, float* lo_hi_out,
                       void* workspace, size_t workspace_bytes, void* stream);

/* ---- ray casting: queries.cast_rays (src/queries.py:39-175) ------------------------ *
 * models[nfunc] are the functions of funcs_tuple; hit_id is 1-based (0 = no hit).
 * Persistent kernel: every ray steps on the device until it terminates; no host
 * round trip per iteration.  n_evals_out (device int64) counts ray-steps evaluated
 * per function.  workspace: niq_cast_rays_workspace_size() bytes.
 * The growing-term modes (TRUNCATE/APPEND/ALL) run the reference's iteration loop on
 * the host for both entry points: per substep every live segment is bounded by the
 * growing-term engine, then the step rule and a compaction run on the device; syncs. */
size_t niq_cast_rays_workspace_size(const niq_model* const* models, int32_t nfunc,
                                    const niq_bound_opts* opts, int64_t n);
int niq_cast_rays(const niq_model* const* models, int32_t nfunc, const niq_bound_opts* opts,
                  int64_t n, const float* roots, const float* dirs, const niq_cast_opts* cast,
                  float* t_out, int32_t* hit_id_out, int32_t* count_out, int64_t* n_evals_out,
                  void* workspace, size_t workspace_bytes, void* stream);
/* The plain form: one launch per iteration over the live rays with a host-side
 * compaction step between iterations, the structure of the reference's loop
 * (src/queries.py:158-173).  Syncs the stream. */
int niq_cast_rays_plain(const niq_model* const* models, int32_t nfunc, const niq_bound_opts* opts,
                        int64_t n, const float* roots, const float* dirs, const niq_cast_opts* cast,
                        float* t_out, int32_t* hit_id_out, int32_t* count_out, int64_t* n_evals_out,
                        void* workspace, size_t workspace_bytes, void* stream);

/* ---- queries.cast_rays_frustum (src/queries.py:178-587) ------------------------------
 * The camera tuple (root_pos, look_dir, up_dir, left_dir, fov_x, fov_y, res_x, res_y) of
 * the reference; fov in degrees. */
typedef struct niq_frustum_camera {
    float root[3];
    float look[3];
    float up[3];
    float left[3];
    float fov_x, fov_y;
    int32_t res_x, res_y;
} niq_frustum_camera;
/* Frusta start as an n_side_init^2 grid of pixel tiles, march like rays with a box
 * enclosing each step, split in half along the wider pixel axis when the step falls
 * behind the frustum's width (refine_width_fac) and hit only as single pixels.  Outputs
 * are (res_x, res_y) arrays indexed [x][y] as the reference returns them: t_out, hit_id
 * (1-based function index, 0 = none) and count (steps per pixel, truncated);
 * n_evals_out (device int64) counts frustum steps.  One launch per iteration with a
 * host read of the live count, as the reference's loop.  Every mode: interval,
 * affine_fixed and slope_interval in one fused kernel per iteration (workspace:
 * niq_cast_frustum_workspace_size() bytes); affine_truncate, affine_all and
 * affine_append bound each substep's boxes with the growing-term engine between
 * per-frustum kernels (workspace: niq_cast_frustum_growing_workspace_size() bytes). */
size_t niq_cast_frustum_workspace_size(int32_t res_x, int32_t res_y, int32_t n_side_init);
size_t niq_cast_frustum_growing_workspace_size(const niq_model* const* models, int32_t nfunc,
                                               const niq_bound_opts* opts, int32_t res_x, int32_t res_y,
                                               int32_t n_side_init);
int niq_cast_frustum(const niq_model* const* models, int32_t nfunc, const niq_bound_opts* opts,
                     const niq_frustum_camera* camera, const niq_cast_opts* cast, float refine_width_fac,
                     int32_t n_side_init, float* t_out, int32_t* hit_id_out, int32_t* count_out,
                     int64_t* n_evals_out, void* workspace, size_t workspace_bytes, void* stream);

/* ---- kd_tree.sample_surface / bulk_properties (src/kd_tree.py:220-292, 804-863) --------
 * Monte Carlo over the nodes of a level-set tree (device arrays (n, 3) of lower and upper
 * corners): candidates pick a node uniformly and a point uniformly inside it, from a
 * counter-based generator seeded by `seed` (the reference draws from JAX's threefry
 * stream: the same distribution, other samples).
 * niq_sample_surface keeps points with |f| < width until n_samples are found
 * (samples_out: device (n_samples, 3)), drawing n_per_round candidates per round for at
 * most max_rounds rounds (NIQ_ERR_TIMEOUT with *n_found_out < n_samples after that).
 * niq_bulk_properties: mass and centroid of {f < 0}: the interior nodes exactly, the
 * boundary nodes by n_sample candidates; mass_centroid_out (host, 4 doubles) = mass,
 * centroid.  workspace: niq_sample_workspace_size(n_per_round or n_sample) bytes. */
size_t niq_sample_workspace_size(int64_t n_candidates);
int niq_sample_surface(const niq_model* model, int64_t n_nodes, const float* node_lower, const float* node_upper,
                       int64_t n_samples, float width, uint64_t seed, int64_t n_per_round, int32_t max_rounds,
                       float* samples_out, int64_t* n_found_out, void* workspace, size_t workspace_bytes,
                       void* stream);
int niq_bulk_properties(const niq_model* model, int64_t n_interior, const float* interior_lower,
                        const float* interior_upper, int64_t n_boundary, const float* boundary_lower,
                        const float* boundary_upper, int64_t n_sample, uint64_t seed, double* mass_centroid_out,
                        void* workspace, size_t workspace_bytes, void* stream);

/* ---- render.outward_normals / shade_image (src/render.py:53-90,152-224) ----------------
 * Normals by the reference's tetrahedron central differences at the hit positions, for
 * the function each pixel hit (hit_id 1-based; zero normal for no hit).  hit_pos,
 * hit_id and normals_out are device arrays of n rows.  workspace:
 * niq_outward_normals_workspace_size(n) bytes. */
size_t niq_outward_normals_workspace_size(int64_t n);
int niq_outward_normals(const niq_model* const* models, int32_t nfunc, int64_t n, const float* hit_pos,
                        const int32_t* hit_id, float eps, float* normals_out, void* workspace,
                        size_t workspace_bytes, void* stream);
/* outward_normals(..., method='autodiff') (src/render.py:61-63,81-90): the normalised
 * gradient (niq_eval_gradients) of the function each point hit, zeros where none; a
 * workspace of niq_outward_normals_autodiff_workspace_size(n) bytes. */
size_t niq_outward_normals_autodiff_workspace_size(int64_t n);
int niq_outward_normals_autodiff(const niq_model* const* models, int32_t nfunc, int64_t n,
                                 const float* hit_pos, const int32_t* hit_id, float* normals_out,
                                 void* workspace, size_t workspace_bytes, void* stream);
/* Shading into a device RGB buffer (n, 3): shading 0 = 'normal', 1 = 'matcap_color' with
 * matcaps a device array (4, matcap_h, matcap_w, 3) of the r, g, b, k images and colors
 * a host array (ncolors, 3), one per function.  up_dir is host (3).  Pixels without a
 * hit are white; tonemap != 0 applies tonemap_image (src/render.py:152-158). */
int niq_shade_image(int32_t shading, int64_t n, const float* ray_dirs, const float* normals, const int32_t* hit_id,
                    const float* up_dir, const float* matcaps, int32_t matcap_h, int32_t matcap_w,
                    const float* colors, int32_t ncolors, int32_t tonemap, float* rgb_out, void* stream);
/* 'matcap_color' shading with a color per pixel: pixel_colors a device array (n, 3), the
 * values of the reference's shading_color_func at the hit positions
 * (src/render.py:193-206), in place of the per-function colors. */
int niq_shade_image_pixel_colors(int64_t n, const float* ray_dirs, const float* normals, const int32_t* hit_id,
                                 const float* up_dir, const float* matcaps, int32_t matcap_h, int32_t matcap_w,
                                 const float* pixel_colors, int32_t tonemap, float* rgb_out, void* stream);

/* ---- level-set kd-tree: construct_uniform_unknown_levelset_tree
 *      (src/kd_tree.py:19-218) ------------------------------------------------------ *
 * Breadth-first bisection of the box [lower, upper] (host float[3] each) for
 * split_depth+1 classify rounds (split_depth < 0: none) or until a round starts with
 * >= node_terminate_thresh nodes (<= 0: none).  Results land in the workspace; the
 * counts are written to the device int64 array counts_out[4] =
 * {n_unknown, n_interior, n_exterior, n_boxes_classified} and the node arrays are read
 * back with niq_tree_result().  flags: bit0 with_interior_nodes, bit1
 * with_exterior_nodes.  Persistent cooperative kernel, one launch for all levels. */
#define NIQ_TREE_WITH_INTERIOR 1
#define NIQ_TREE_WITH_EXTERIOR 2
size_t niq_tree_workspace_size(int64_t node_capacity, int32_t flags);
int niq_levelset_tree(const niq_model* model, const niq_bound_opts* opts,
                      const float* lower, const float* upper, int32_t split_depth,
                      int64_t node_terminate_thresh, float offset, int32_t flags,
                      int64_t node_capacity, int64_t* counts_out,
                      void* workspace, size_t workspace_bytes, void* stream);
/* The plain form: one launch + host sync per level (src/kd_tree.py:137-198). */
int niq_levelset_tree_plain(const niq_model* model, const niq_bound_opts* opts,
                            const float* lower, const float* upper, int32_t split_depth,
                            int64_t node_terminate_thresh, float offset, int32_t flags,
                            int64_t node_capacity, int64_t* counts_out,
                            void* workspace, size_t workspace_bytes, void* stream);
/* The level-set tree for callers that cannot allocate device memory when they call:
 * hosts whose device memory comes from a fixed pool or arena they cannot grow (the
 * allocator would fail or fragment it), plug-ins that are handed only pre-allocated
 * buffers, and latency-critical loops that must not enter the allocator (a device
 * allocation can synchronise the whole device).  No counterpart in the reference (it
 * has no allocation-free path).
 * - No device memory is allocated, by this call or by a model handle: the caller passes
 *   the packed spec twice, a host copy (validated and used for launch planning) and a
 *   16-byte-aligned device copy that the kernels read.  The two must hold the same
 *   bytes; the call compares their headers and fails with NIQ_ERR_BAD_SPEC otherwise.
 * - Scratch (level counters and two level buffers) is a static device array of the
 *   library, NIQ_STATIC_TREE_NODES nodes per level (about 3 MB), which every GPU that
 *   loads the library holds until the process exits.  A level, or a result list, larger
 *   than NIQ_STATIC_TREE_NODES nodes fails with NIQ_ERR_CAPACITY.
 * - Results go to the caller's arrays, each (NIQ_STATIC_TREE_NODES, 3) float32 (interior
 *   and exterior only when requested in flags); counts_out as for niq_levelset_tree.
 * - The first call on a device looks up the scratch array's device address and keeps it
 *   for the process; make no call after a cudaDeviceReset of that device.  Every call
 *   clears the counters it needs.
 * - All calls share the one scratch array: calls that overlap on the GPU (two streams,
 *   or two host threads) race and corrupt each other's results.  Syncs the stream. */
#define NIQ_STATIC_TREE_NODES 65536
int niq_levelset_tree_static(const void* packed_spec_host, const void* packed_spec_device,
                             size_t spec_bytes, const niq_bound_opts* opts,
                             const float* lower, const float* upper, int32_t split_depth,
                             int64_t node_terminate_thresh, float offset, int32_t flags,
                             float* unknown_lower, float* unknown_upper,
                             float* interior_lower, float* interior_upper,
                             float* exterior_lower, float* exterior_upper,
                             int64_t* counts_out, void* stream);
/* The plain form on the reference's schedule: each level in launches of at most
 * batch_process_size nodes (one XLA call per batch in src/kd_tree.py:161-172), one host
 * read of the level size per level.  Same results as niq_levelset_tree_plain. */
int niq_levelset_tree_batches(const niq_model* model, const niq_bound_opts* opts, const float* lower,
                              const float* upper, int32_t split_depth, int64_t node_terminate_thresh, float offset,
                              int32_t flags, int64_t batch_process_size, int64_t node_capacity,
                              int64_t* counts_out, void* workspace, size_t workspace_bytes, void* stream);
/* The tree in every mode, including the growing-term ones (affine_truncate,
 * affine_append, affine_all), which the kernels above reject: the reference's level loop
 * (src/kd_tree.py:137-198) with each level classified by niq_classify_boxes in chunks of
 * 65,536 nodes and the results and children appended on the device; one host read of
 * the level size per level.  Syncs.  Its workspace (niq_tree_growing_workspace_size) has
 * the layout of niq_tree_workspace_size's followed by the chunk scratch, so
 * niq_tree_result reads its nodes. */
size_t niq_tree_growing_workspace_size(const niq_model* model, const niq_bound_opts* opts, int64_t node_capacity,
                                       int32_t flags);
int niq_levelset_tree_growing(const niq_model* model, const niq_bound_opts* opts, const float* lower,
                              const float* upper, int32_t split_depth, int64_t node_terminate_thresh, float offset,
                              int32_t flags, int64_t node_capacity, int64_t* counts_out,
                              void* workspace, size_t workspace_bytes, void* stream);
/* Which engine the level-set tree entry points use for a model and options:
 * NIQ_TREE_ENGINE_TENSOR -- hidden layers' products on the tensor cores (3xTF32, affine_fixed
 *   with outward rounding, products 3XTF32, hidden widths <= 64, a scalar output; slower
 *   than the FP32 engine on the models measured, with wider bounds, so not the default);
 * NIQ_TREE_ENGINE_FP32 -- the FP32 tile engine (the other fixed-mode cases);
 * NIQ_TREE_ENGINE_GROWING -- the growing-term modes, through niq_levelset_tree_growing.
 * Pure host code; the reference has one engine (XLA), so no counterpart. */
#define NIQ_TREE_ENGINE_FP32     0
#define NIQ_TREE_ENGINE_TENSOR   1
#define NIQ_TREE_ENGINE_GROWING  2
int niq_tree_engine(const niq_model* model, const niq_bound_opts* opts, int32_t* engine_out);
/* Device pointers into a finished tree workspace: kind 0 unknown, 1 interior,
 * 2 exterior; lower/upper are (node_capacity, 3) arrays whose first count rows hold
 * the result. */
int niq_tree_result(void* workspace, int64_t node_capacity, int32_t flags, int32_t kind,
                    float** lower, float** upper);

/* ---- hierarchical marching cubes: hierarchical_marching_cubes
 *      (src/kd_tree.py:338-399, src/extract_cell.py:306-421) ------------------------ *
 * Extracts triangles (n_tris_out[0] of them, <= tri_capacity) from the n_leaves
 * boxes (lower/upper (n_leaves,3), e.g. niq_tree_result kind 0) on a
 * (2^n_subcell_depth)^3 subgrid each.  tris_out is (tri_capacity, 3, 3). */
size_t niq_hmc_workspace_size(void);
int niq_hmc_extract(const niq_model* model, int64_t n_leaves, const float* leaf_lower,
                    const float* leaf_upper, int32_t n_subcell_depth,
                    float* tris_out, int64_t tri_capacity, int64_t* n_tris_out,
                    void* workspace, size_t workspace_bytes, void* stream);
/* The 256x16 triangle table used by niq_hmc_extract (host int32 out[256*16]; -1 pads).
 * Same polygons and orientation as src/extract_cell.py:12-268 for every case; pure
 * host code, no device needed. */
int niq_mc_table(int32_t* out);
/* The n_subcell_depth = 0 extraction for the leaves of a uniform tree of split_depth
 * bisections of [root_lower, root_upper]: corners shared by neighbouring leaves are
 * evaluated once (the leaves are cells of one lattice; a split plane is the same float
 * in both children), then every leaf is polygonised as niq_hmc_extract does, with the
 * same arithmetic and the same triangles (in another order).  workspace:
 * niq_hmc_lattice_workspace_size() bytes. */
size_t niq_hmc_lattice_workspace_size(const float* root_lower, const float* root_upper, int32_t split_depth,
                                      int64_t n_leaves);
int niq_hmc_extract_lattice(const niq_model* model, int64_t n_leaves, const float* leaf_lower,
                            const float* leaf_upper, const float* root_lower, const float* root_upper,
                            int32_t split_depth, float* tris_out, int64_t tri_capacity, int64_t* n_tris_out,
                            void* workspace, size_t workspace_bytes, void* stream);

/* ---- pairwise intersection: find_any_intersection (src/kd_tree.py:402-655) ---------- *
 * found_out (device int32[1]) = 1 when an intersection is found, loc_out (device
 * float[3]) its witness, (-777,-777,-777) otherwise.  Persistent kernel over all depths;
 * counts_out (device int64[2]) = {nodes processed, depth reached}. */
size_t niq_intersect_workspace_size(const niq_model* model_a, const niq_model* model_b,
                                    const niq_bound_opts* opts, int64_t node_capacity);
int niq_find_any_intersection(const niq_model* model_a, const niq_model* model_b,
                              const niq_bound_opts* opts, const float* lower, const float* upper,
                              float eps, int64_t node_capacity, int32_t* found_out, float* loc_out,
                              int64_t* counts_out, void* workspace, size_t workspace_bytes,
                              void* stream);

/* ---- closest point: closest_point (src/kd_tree.py:659-802) -------------------------- *
 * The reference schedule: one global LIFO stack, batch pops of batch_process_size
 * nodes, scatter-min of candidate distances.  Host loop with one sync per batch.
 * Every mode: in the growing-term ones (affine_truncate, affine_append, affine_all)
 * each popped batch is classified by the growing-term engine first, and the workspace
 * must have niq_closest_point_growing_workspace_size() bytes. */
size_t niq_closest_point_workspace_size(int64_t n_queries, int32_t batch_process_size,
                                        int64_t stack_capacity);
size_t niq_closest_point_growing_workspace_size(const niq_model* model, const niq_bound_opts* opts,
                                                int64_t n_queries, int32_t batch_process_size,
                                                int64_t stack_capacity);
int niq_closest_point(const niq_model* model, const niq_bound_opts* opts, const float* lower,
                      const float* upper, int64_t n_queries, const float* query_points,
                      float eps, int32_t batch_process_size, int64_t stack_capacity,
                      float* min_dist_out, float* min_loc_out,
                      void* workspace, size_t workspace_bytes, void* stream);
/* Persistent form: every query traverses its own depth-first stack on the device,
 * nearer child first; one launch.  Same candidate and pruning tests as the reference;
 * Nodes are pruned when the query-to-box distance (a true lower bound) is within eps of
 * the best candidate, so the result is never larger than the reference schedule's by more
 * than eps (candidates already carry a leaf diagonal, <= eps, of slack).  node_budget
 * (<= 0: none) caps the nodes
 * one query may visit; a query that reaches it keeps its best distance so far (still an
 * upper bound) and the call returns NIQ_ERR_TIMEOUT after writing every result. */
size_t niq_closest_point_persistent_workspace_size(int64_t n_queries);
int niq_closest_point_persistent(const niq_model* model, const niq_bound_opts* opts,
                                 const float* lower, const float* upper, int64_t n_queries,
                                 const float* query_points, float eps, int64_t node_budget,
                                 float* min_dist_out, float* min_loc_out,
                                 void* workspace, size_t workspace_bytes, void* stream);

/* ---- many models in one launch (closest point over a model table) ------------------ *
 * Job j runs query_count[j] closest-point queries starting at row query_offset[j] of
 * query_points against models[job_model[j]]; all jobs run in one persistent launch.
 * Arrays job_model/query_offset/query_count are host arrays of n_jobs entries.
 * status_out: optional device int32; when given the call does not sync and the
 * traversal's status (NIQ_OK or NIQ_ERR_CAPACITY) is written there; when NULL the call
 * syncs the stream and returns that status. */
size_t niq_batched_closest_point_workspace_size(int64_t total_queries, int32_t n_jobs);
int niq_batched_closest_point(const niq_model* const* models, int32_t n_models,
                              const niq_bound_opts* opts, int32_t n_jobs,
                              const int32_t* job_model, const int64_t* query_offset,
                              const int64_t* query_count, const float* query_points,
                              const float* lower, const float* upper, float eps,
                              float* min_dist_out, float* min_loc_out, int64_t node_budget,
                              int32_t* status_out,
                              void* workspace, size_t workspace_bytes, void* stream);
/* Counters of the last niq_batched_closest_point call on this workspace: the queries that
 * stopped at node_budget (each keeps its best candidate so far, an upper bound on its
 * distance) and the nodes bounded (a box bound and its sign samples each).  Either output
 * may be NULL.  Read after that call's work completed; syncs `stream`. */
int niq_batched_closest_point_stats(const void* workspace, int64_t* budget_spent_out, int64_t* nodes_out,
                                    void* stream);

/* ---- serving: continuous batching of mixed requests ---------------------------------
 * No counterpart in the reference (it has no server; its queries are called one at a
 * time).  A server owns n_lanes lanes: a lane is a host worker thread with its own CUDA
 * stream and lane_scratch_bytes of device scratch, allocated once by niq_server_create,
 * so submitting and running requests allocates nothing.  niq_batch_submit cuts a request
 * into slices -- ray tiles of at most slice_rays rays, closest-point slices of at most
 * slice_queries queries, one slice per intersection -- queues them and returns a ticket
 * at once.  Free lanes take ray tiles first, then the other slices, and run each on
 * their stream, so requests that arrive while others run overlap them on the device and
 * a short ray tile never waits behind a long closest-point batch.  niq_batch_poll
 * reports, without blocking, whether a request is done and its status (NIQ_OK,
 * NIQ_ERR_TIMEOUT when a closest-point query spent its node budget -- every result is
 * still written, an upper bound -- or another error); niq_batch_wait blocks up to a
 * timeout.  A done ticket is reported once.  Inputs and outputs are the caller's device
 * arrays and must stay valid until the request is done; models are borrowed. */
#define NIQ_REQ_RAYS       0   /* queries.cast_rays (src/queries.py:134-175) on a tile      */
#define NIQ_REQ_CLOSEST    1   /* kd_tree.closest_point (src/kd_tree.py:766-802), persistent */
#define NIQ_REQ_INTERSECT  2   /* kd_tree.find_any_intersection (src/kd_tree.py:567-655)   */
typedef struct niq_request {
    int32_t kind;                 /* NIQ_REQ_*                                              */
    const niq_model* model;       /* the model (intersection: model A)                      */
    const niq_model* model_b;     /* intersection: model B                                  */
    niq_bound_opts opts;
    niq_cast_opts cast;           /* rays                                                   */
    int64_t n;                    /* rays or query points                                   */
    const float* in0;             /* rays: roots (n,3); closest point: points (n,3)         */
    const float* in1;             /* rays: dirs (n,3)                                       */
    float* out_f;                 /* rays: t (n); closest point: distance (n)              */
    float* out_f2;                /* closest point: location (n,3); intersection: loc (3)  */
    int32_t* out_i;               /* rays: hit_id (n); intersection: found (1)             */
    int32_t* out_i2;              /* rays: count (n)                                        */
    float eps;                    /* closest point and intersection                         */
    int64_t node_budget;          /* closest point: nodes per query (<= 0: none)            */
    int64_t node_capacity;        /* intersection: nodes per level (<= 0: 2^20)             */
    float lower[3], upper[3];     /* root box of closest point and intersection             */
} niq_request;
typedef struct niq_server_opts {
    int32_t n_lanes;
    int64_t slice_rays;
    int64_t slice_queries;
    int64_t lane_scratch_bytes;
} niq_server_opts;
typedef struct niq_server niq_server;
int niq_server_create(const niq_server_opts* opts, niq_server** out);
/* Finishes the queued work, stops the lanes and frees their scratch. */
int niq_server_destroy(niq_server* server);
int niq_batch_submit(niq_server* server, const niq_request* request, int64_t* ticket_out);
int niq_batch_poll(niq_server* server, int64_t ticket, int32_t* done_out, int32_t* status_out);
int niq_batch_wait(niq_server* server, int64_t ticket, double timeout_s, int32_t* status_out);
int niq_server_stats(niq_server* server, int64_t* completed, int64_t* in_flight);

#ifdef __cplusplus
}
#endif
#endif /* NIQ_H */
