// k_shade.cu -- render.outward_normals and render.shade_image (src/render.py:53-90,
// 152-224) into device buffers; no graphics API.
//
// Normals: the reference's 'tetrahedron' central differences.  f is sampled at the hit
// point plus the four offsets (+e,-e,-e), (-e,-e,+e), (-e,+e,-e), (+e,+e,+e); the gradient
// is sum_i offset_i f_i, normalised; a pixel takes the normal of the function it hit
// (zero when it hit none).  The samples run through the point-evaluation kernel.
//
// Shading: 'normal' maps the normal to [0, 1]; 'matcap_color' looks the normal up in four
// matcap images (r, g, b, k) with bilinear interpolation clamped at the edges
// (map_coordinates, order 1, mode 'nearest') and mixes them with the hit function's color
// (c_r, c_g, c_b, 1 - c_r - c_g - c_b).  Pixels without a hit are white.
#include "niq_host.cuh"

namespace niq {

__constant__ float c_tet[4][3] = {{1.f, -1.f, -1.f}, {-1.f, -1.f, 1.f}, {-1.f, 1.f, -1.f}, {1.f, 1.f, 1.f}};

__global__ void k_normal_samples(long long n, const float* __restrict__ pos, float eps, float* __restrict__ pts) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < 4 * n; i += (long long)gridDim.x * blockDim.x) {
        const long long p = i >> 2;
        const int q = (int)(i & 3);
        for (int k = 0; k < 3; ++k) pts[3 * i + k] = __fadd_rn(pos[3 * p + k], __fmul_rn(c_tet[q][k], eps));
    }
}

// grad = sum_i offset_i * f_i (offsets are +-eps), normalised; kept where hit_id == f + 1
__global__ void k_normal_combine(long long n, int f, const float* __restrict__ vals, const int* __restrict__ hit_id,
                                 float eps, float* __restrict__ normals) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        if (f == 0) normals[3 * p] = normals[3 * p + 1] = normals[3 * p + 2] = 0.f;
        if (hit_id[p] != f + 1) continue;
        float g[3];
        for (int k = 0; k < 3; ++k) {
            float s = 0.f;
            for (int q = 0; q < 4; ++q) s = __fadd_rn(s, __fmul_rn(__fmul_rn(c_tet[q][k], eps), vals[4 * p + q]));
            g[k] = s;
        }
        const float nrm = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(g[0], g[0]), __fmul_rn(g[1], g[1])), __fmul_rn(g[2], g[2])));
        for (int k = 0; k < 3; ++k) normals[3 * p + k] = __fdiv_rn(g[k], nrm);
    }
}

// Normals from gradients (method 'autodiff'): where the point hit function f + 1, its
// normalised gradient (geometry.normalize, src/geometry.py:12-13).
__global__ void k_grad_combine(long long n, int f, const float* __restrict__ grad, const int* __restrict__ hit_id,
                               float* __restrict__ normals) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        if (f == 0) normals[3 * p] = normals[3 * p + 1] = normals[3 * p + 2] = 0.f;
        if (hit_id[p] != f + 1) continue;
        const float* g = grad + 3 * p;
        const float nrm = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(g[0], g[0]), __fmul_rn(g[1], g[1])), __fmul_rn(g[2], g[2])));
        for (int k = 0; k < 3; ++k) normals[3 * p + k] = __fdiv_rn(g[k], nrm);
    }
}

struct ShadeArgs {
    int shading;          // 0 normal, 1 matcap_color
    float up[3];          // up direction as the caller gives it
    const float* matcaps; // (4, H, W, 3): r, g, b, k
    int mh, mw;
    float colors[8][3];   // per function (1-based hit id)
    int ncolors;
    int tonemap;
    const float* pix;     // per-pixel colors (n, 3) of shading_color_func, or null
};

// one channel of a matcap at (x, y): bilinear, indices clamped to the image (src/render.py:184-187)
__device__ __forceinline__ float matcap_sample(const float* img, int H, int W, int ch, float x, float y) {
    const float x0f = floorf(x), y0f = floorf(y);
    const float wx1 = __fsub_rn(x, x0f), wy1 = __fsub_rn(y, y0f);
    const float wx0 = __fsub_rn(1.f, wx1), wy0 = __fsub_rn(1.f, wy1);
    const int x0 = (int)x0f, y0 = (int)y0f;
    const int xi[2] = {min(max(x0, 0), H - 1), min(max(x0 + 1, 0), H - 1)};
    const int yi[2] = {min(max(y0, 0), W - 1), min(max(y0 + 1, 0), W - 1)};
    const float wx[2] = {wx0, wx1}, wy[2] = {wy0, wy1};
    float acc = 0.f;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            acc = __fadd_rn(acc, __fmul_rn(img[((long long)xi[a] * W + yi[b]) * 3 + ch], __fmul_rn(wx[a], wy[b])));
    return acc;
}

__global__ void k_shade(long long n, ShadeArgs a, const float* __restrict__ dirs, const float* __restrict__ normals,
                        const int* __restrict__ hit_id, float* __restrict__ rgb) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const float nx = normals[3 * p], ny = normals[3 * p + 1], nz = normals[3 * p + 2];
        float c[3];
        if (a.shading == 0) {
            c[0] = __fdiv_rn(__fadd_rn(nx, 1.f), 2.f);
            c[1] = __fdiv_rn(__fadd_rn(ny, 1.f), 2.f);
            c[2] = __fdiv_rn(__fadd_rn(nz, 1.f), 2.f);
        } else {
            // matcap coordinates (src/render.py:168-181): ray_up = orthogonal_dir(up, dir),
            // ray_left = dir x ray_up, u = -ray_left . n, v = ray_up . n
            const float d[3] = {dirs[3 * p], dirs[3 * p + 1], dirs[3 * p + 2]};
            const float dn = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2])));
            const float r[3] = {__fdiv_rn(d[0], dn), __fdiv_rn(d[1], dn), __fdiv_rn(d[2], dn)};
            const float du = __fadd_rn(__fadd_rn(__fmul_rn(a.up[0], r[0]), __fmul_rn(a.up[1], r[1])), __fmul_rn(a.up[2], r[2]));
            float u[3];
            for (int k = 0; k < 3; ++k) u[k] = __fsub_rn(a.up[k], __fmul_rn(du, r[k]));
            const float un = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(u[0], u[0]), __fmul_rn(u[1], u[1])), __fmul_rn(u[2], u[2])));
            for (int k = 0; k < 3; ++k) u[k] = __fdiv_rn(u[k], un);
            const float l[3] = {__fsub_rn(__fmul_rn(d[1], u[2]), __fmul_rn(d[2], u[1])),
                                __fsub_rn(__fmul_rn(d[2], u[0]), __fmul_rn(d[0], u[2])),
                                __fsub_rn(__fmul_rn(d[0], u[1]), __fmul_rn(d[1], u[0]))};
            float mu = __fadd_rn(__fadd_rn(__fmul_rn(-l[0], nx), __fmul_rn(-l[1], ny)), __fmul_rn(-l[2], nz));
            float mv = __fadd_rn(__fadd_rn(__fmul_rn(u[0], nx), __fmul_rn(u[1], ny)), __fmul_rn(u[2], nz));
            mu = __fmul_rn(mu, 0.98f);
            mv = __fmul_rn(mv, 0.98f);
            const float x = __fmul_rn(__fdiv_rn(__fadd_rn(mu, 1.f), 2.f), (float)a.mh);
            const float y = __fmul_rn(__fdiv_rn(__fadd_rn(-mv, 1.f), 2.f), (float)a.mw);
            const int h = hit_id[p];
            float col[3] = {1.f, 1.f, 1.f};
            if (a.pix)
                for (int k = 0; k < 3; ++k) col[k] = a.pix[3 * p + k];
            else if (h >= 1 && h <= a.ncolors)
                for (int k = 0; k < 3; ++k) col[k] = a.colors[h - 1][k];
            const float ck = __fsub_rn(1.f, __fadd_rn(__fadd_rn(col[0], col[2]), col[1]));
            const long long plane = (long long)a.mh * a.mw * 3;
            for (int ch = 0; ch < 3; ++ch) {
                const float mr = matcap_sample(a.matcaps, a.mh, a.mw, ch, x, y);
                const float mg = matcap_sample(a.matcaps + plane, a.mh, a.mw, ch, x, y);
                const float mb = matcap_sample(a.matcaps + 2 * plane, a.mh, a.mw, ch, x, y);
                const float mk = matcap_sample(a.matcaps + 3 * plane, a.mh, a.mw, ch, x, y);
                // c_r m_r + c_b m_b + c_g m_g + c_k m_k, summed left to right
                c[ch] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(col[0], mr), __fmul_rn(col[2], mb)), __fmul_rn(col[1], mg)),
                                  __fmul_rn(ck, mk));
            }
        }
        // pixels without a hit are white (src/render.py:139)
        if (hit_id[p] == 0) c[0] = c[1] = c[2] = 1.f;
        if (a.tonemap) {
            // src/render.py:152-158 with gamma 2.2, white level 0.75, exposure 1
            for (int k = 0; k < 3; ++k) {
                const float x = c[k];
                const float num = __fmul_rn(x, __fadd_rn(1.f, __fdiv_rn(x, __fmul_rn(0.75f, 0.75f))));
                const float den = __fadd_rn(1.f, x);
                c[k] = powf(__fdiv_rn(num, den), __fdiv_rn(1.f, 2.2f));
            }
        }
        rgb[3 * p] = c[0];
        rgb[3 * p + 1] = c[1];
        rgb[3 * p + 2] = c[2];
    }
}

static int grid_for(long long n) {
    long long g = (n + 255) / 256;
    return (int)(g < 1 ? 1 : (g > 8 * 1024 ? 8 * 1024 : g));
}

}  // namespace niq

using namespace niq;

extern "C" {

size_t niq_outward_normals_workspace_size(int64_t n) {
    return (size_t)(n > 0 ? n : 0) * (12 * 4 + 4 * 4) + 512;
}

int niq_outward_normals(const niq_model* const* models, int32_t nfunc, int64_t n, const float* hit_pos,
                        const int32_t* hit_id, float eps, float* normals_out, void* workspace, size_t workspace_bytes,
                        void* stream) {
    NIQ_REQUIRE(models && nfunc >= 1 && nfunc <= 8, NIQ_ERR_INVALID_ARG, "nfunc must be in [1, 8]");
    NIQ_REQUIRE(n >= 0, NIQ_ERR_INVALID_ARG, "n < 0");
    if (n == 0) return NIQ_OK;
    NIQ_REQUIRE(hit_pos && hit_id && normals_out, NIQ_ERR_INVALID_ARG, "null array");
    const size_t need = niq_outward_normals_workspace_size(n);
    NIQ_REQUIRE(workspace && workspace_bytes >= need, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed", need);
    cudaStream_t s = as_stream(stream);
    char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
    float* pts = reinterpret_cast<float*>(base);
    float* vals = pts + 12 * n;
    k_normal_samples<<<grid_for(4 * n), 256, 0, s>>>(n, hit_pos, eps, pts);
    NIQ_CUDA(cudaGetLastError());
    for (int f = 0; f < nfunc; ++f) {
        NIQ_REQUIRE(models[f], NIQ_ERR_INVALID_ARG, "null model %d", f);
        int rc = niq_eval_points(models[f], 4 * n, pts, vals, stream);
        if (rc) return rc;
        k_normal_combine<<<grid_for(n), 256, 0, s>>>(n, f, vals, hit_id, eps, normals_out);
        NIQ_CUDA(cudaGetLastError());
    }
    return NIQ_OK;
}

size_t niq_outward_normals_autodiff_workspace_size(int64_t n) {
    return (size_t)(n > 0 ? n : 0) * 3 * 4 + 512;
}

int niq_outward_normals_autodiff(const niq_model* const* models, int32_t nfunc, int64_t n, const float* hit_pos,
                                 const int32_t* hit_id, float* normals_out, void* workspace, size_t workspace_bytes,
                                 void* stream) {
    NIQ_REQUIRE(models && nfunc >= 1 && nfunc <= 8, NIQ_ERR_INVALID_ARG, "nfunc must be in [1, 8]");
    NIQ_REQUIRE(n >= 0, NIQ_ERR_INVALID_ARG, "n < 0");
    if (n == 0) return NIQ_OK;
    NIQ_REQUIRE(hit_pos && hit_id && normals_out, NIQ_ERR_INVALID_ARG, "null array");
    const size_t need = niq_outward_normals_autodiff_workspace_size(n);
    NIQ_REQUIRE(workspace && workspace_bytes >= need, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed", need);
    cudaStream_t s = as_stream(stream);
    float* grad = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
    for (int f = 0; f < nfunc; ++f) {
        NIQ_REQUIRE(models[f], NIQ_ERR_INVALID_ARG, "null model %d", f);
        int rc = niq_eval_gradients(models[f], n, hit_pos, nullptr, grad, stream);
        if (rc) return rc;
        k_grad_combine<<<grid_for(n), 256, 0, s>>>(n, f, grad, hit_id, normals_out);
        NIQ_CUDA(cudaGetLastError());
    }
    return NIQ_OK;
}

static int shade(int32_t shading, int64_t n, const float* ray_dirs, const float* normals, const int32_t* hit_id,
                 const float* up_dir, const float* matcaps, int32_t matcap_h, int32_t matcap_w, const float* colors,
                 int32_t ncolors, const float* pixel_colors, int32_t tonemap, float* rgb_out, void* stream) {
    NIQ_REQUIRE(shading == 0 || shading == 1, NIQ_ERR_INVALID_ARG, "shading must be 0 (normal) or 1 (matcap_color)");
    NIQ_REQUIRE(n >= 0, NIQ_ERR_INVALID_ARG, "n < 0");
    if (n == 0) return NIQ_OK;
    NIQ_REQUIRE(ray_dirs && normals && hit_id && rgb_out, NIQ_ERR_INVALID_ARG, "null array");
    ShadeArgs a;
    a.shading = shading;
    a.tonemap = tonemap != 0;
    a.matcaps = matcaps;
    a.mh = matcap_h;
    a.mw = matcap_w;
    a.ncolors = 0;
    a.pix = pixel_colors;
    if (shading == 1) {
        NIQ_REQUIRE(up_dir && matcaps && matcap_h >= 1 && matcap_w >= 1, NIQ_ERR_INVALID_ARG, "matcap shading needs up_dir and matcaps");
        NIQ_REQUIRE(pixel_colors || (colors && ncolors >= 1 && ncolors <= 8), NIQ_ERR_INVALID_ARG, "1 to 8 colors needed");
        // orthogonal_dir(up_dir, ray_dir) removes the ray's component from up_dir as given
        // (src/geometry.py:15-19)
        for (int k = 0; k < 3; ++k) a.up[k] = up_dir[k];
        a.ncolors = ncolors;
        for (int i = 0; i < ncolors; ++i)
            for (int k = 0; k < 3; ++k) a.colors[i][k] = colors[3 * i + k];
    }
    k_shade<<<grid_for(n), 256, 0, as_stream(stream)>>>(n, a, ray_dirs, normals, hit_id, rgb_out);
    NIQ_CUDA(cudaGetLastError());
    return NIQ_OK;
}

int niq_shade_image(int32_t shading, int64_t n, const float* ray_dirs, const float* normals, const int32_t* hit_id,
                    const float* up_dir, const float* matcaps, int32_t matcap_h, int32_t matcap_w,
                    const float* colors, int32_t ncolors, int32_t tonemap, float* rgb_out, void* stream) {
    return shade(shading, n, ray_dirs, normals, hit_id, up_dir, matcaps, matcap_h, matcap_w, colors, ncolors, nullptr,
                 tonemap, rgb_out, stream);
}

int niq_shade_image_pixel_colors(int64_t n, const float* ray_dirs, const float* normals, const int32_t* hit_id,
                                 const float* up_dir, const float* matcaps, int32_t matcap_h, int32_t matcap_w,
                                 const float* pixel_colors, int32_t tonemap, float* rgb_out, void* stream) {
    NIQ_REQUIRE(n == 0 || pixel_colors, NIQ_ERR_INVALID_ARG, "null pixel colors");
    return shade(1, n, ray_dirs, normals, hit_id, up_dir, matcaps, matcap_h, matcap_w, nullptr, 0, pixel_colors,
                 tonemap, rgb_out, stream);
}

}  // extern "C"
