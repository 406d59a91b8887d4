// k_hmc.cu -- hierarchical marching cubes extraction (src/kd_tree.py:338-399,
// src/extract_cell.py:306-421).
//
// For each leaf box, the (2^k+1)^3 grid of jnp.linspace points (lo*(1-s) + hi*s,
// s = i/(2^k)) is evaluated, and every one of the (2^k)^3 subcells is polygonised:
// corner values come from the grid, corner positions from subcell_lower + {0, delta}
// (src/extract_cell.py:402-409), edge crossings t = -vA/(vB-vA) with NaN -> 0 and
// clip [0, 1], case bit i set when corner i is negative, up to five triangles from the
// table (src/extract_cell.py:335-362).
//
// One CTA claims a group of leaves, evaluates all their grid points with the tile
// engine into shared memory, then polygonises the group's subcells from there, so no
// scratch memory is needed.  Triangles are appended with warp-aggregated atomics; their
// order is not the reference's.
//
// The triangle table.  The reference ships a third-party table (src/extract_cell.py:
// 12-268).  This file derives an equivalent one from the reference's corner and edge
// numbering (src/extract_cell.py:274-302): on every cube face the cut edges are joined
// into segments (an ambiguous face keeps its inside corners apart), segments chain into
// loops, each loop is oriented with its normal from inside (< 0) to outside corners, and
// fan-triangulated from its lowest edge id.  Every case has the reference's polygons and
// orientation; polygons of four or more vertices may be split into different triangles.
#include <mutex>
#include <vector>
#include <algorithm>
#include "niq_host.cuh"

namespace niq {

__constant__ signed char c_tri[256][16];

__device__ __constant__ int c_vert[8][3] = {{0, 1, 0}, {1, 1, 0}, {1, 0, 0}, {0, 0, 0},
                                            {0, 1, 1}, {1, 1, 1}, {1, 0, 1}, {0, 0, 1}};
__device__ __constant__ int c_edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                             {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

static const int kVert[8][3] = {{0, 1, 0}, {1, 1, 0}, {1, 0, 0}, {0, 0, 0}, {0, 1, 1}, {1, 1, 1}, {1, 0, 1}, {0, 0, 1}};
static const int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
// faces as corner 4-cycles (x=0, x=1, y=0, y=1, z=0, z=1)
static const int kFace[6][4] = {{3, 0, 4, 7}, {2, 1, 5, 6}, {3, 2, 6, 7}, {0, 1, 5, 4}, {3, 2, 1, 0}, {7, 6, 5, 4}};

static int edge_id(int a, int b) {
    for (int e = 0; e < 12; ++e)
        if ((kEdge[e][0] == a && kEdge[e][1] == b) || (kEdge[e][0] == b && kEdge[e][1] == a)) return e;
    return -1;
}

void build_mc_table(signed char T[256][16]) {
    for (int c = 0; c < 256; ++c) {
        for (int i = 0; i < 16; ++i) T[c][i] = -1;
        int inside[8];
        for (int i = 0; i < 8; ++i) inside[i] = (c >> i) & 1;
        std::vector<std::pair<int, int>> segs;
        for (int f = 0; f < 6; ++f) {
            std::vector<int> cut;
            for (int k = 0; k < 4; ++k) {
                const int a = kFace[f][k], b = kFace[f][(k + 1) % 4];
                if (inside[a] != inside[b]) cut.push_back(edge_id(a, b));
            }
            if (cut.size() == 2) segs.push_back({cut[0], cut[1]});
            else if (cut.size() == 4)
                for (int k = 0; k < 4; ++k) {
                    const int cc = kFace[f][k];
                    if (inside[cc]) segs.push_back({edge_id(kFace[f][(k + 3) % 4], cc), edge_id(cc, kFace[f][(k + 1) % 4])});
                }
        }
        std::vector<std::vector<int>> adj(12);
        for (auto& s : segs) { adj[s.first].push_back(s.second); adj[s.second].push_back(s.first); }
        bool seen[12] = {false};
        int n_out = 0;
        for (int start = 0; start < 12; ++start) {
            if (adj[start].empty() || seen[start]) continue;
            std::vector<int> loop{start};
            seen[start] = true;
            int prev = -1, cur = start;
            while (true) {
                int nxt = -1;
                for (int x : adj[cur]) {
                    if (x == prev) continue;
                    if (!seen[x]) { nxt = x; break; }
                }
                if (nxt < 0) break;
                loop.push_back(nxt);
                seen[nxt] = true;
                prev = cur;
                cur = nxt;
            }
            // orientation from the Newell normal of the edge midpoints
            double n[3] = {0, 0, 0}, d[3] = {0, 0, 0};
            const int L = (int)loop.size();
            for (int i = 0; i < L; ++i) {
                double p[3], q[3];
                for (int k = 0; k < 3; ++k) {
                    p[k] = 0.5 * (kVert[kEdge[loop[i]][0]][k] + kVert[kEdge[loop[i]][1]][k]);
                    q[k] = 0.5 * (kVert[kEdge[loop[(i + 1) % L]][0]][k] + kVert[kEdge[loop[(i + 1) % L]][1]][k]);
                }
                n[0] += p[1] * q[2] - p[2] * q[1];
                n[1] += p[2] * q[0] - p[0] * q[2];
                n[2] += p[0] * q[1] - p[1] * q[0];
                const int a = kEdge[loop[i]][0], b = kEdge[loop[i]][1];
                const int in = inside[a] ? a : b, out = inside[a] ? b : a;
                for (int k = 0; k < 3; ++k) d[k] += (double)(kVert[out][k] - kVert[in][k]);
            }
            if (n[0] * d[0] + n[1] * d[1] + n[2] * d[2] < 0) std::reverse(loop.begin(), loop.end());
            const int kmin = (int)(std::min_element(loop.begin(), loop.end()) - loop.begin());
            std::rotate(loop.begin(), loop.begin() + kmin, loop.end());
            for (int i = 1; i + 1 < L; ++i) {
                T[c][3 * n_out + 0] = (signed char)loop[0];
                T[c][3 * n_out + 1] = (signed char)loop[i];
                T[c][3 * n_out + 2] = (signed char)loop[i + 1];
                ++n_out;
            }
        }
    }
}

static signed char g_table[256][16];
static std::once_flag g_table_once;
static bool g_uploaded[64] = {false};
static std::mutex g_upload_mu;

static int ensure_table() {
    std::call_once(g_table_once, [] { build_mc_table(g_table); });
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_upload_mu);
    if (dev >= 0 && dev < 64 && !g_uploaded[dev]) {
        NIQ_CUDA(cudaMemcpyToSymbol(c_tri, g_table, sizeof(g_table)));
        g_uploaded[dev] = true;
    }
    return NIQ_OK;
}

struct HmcArgs {
    long long n_leaves;
    const float* lo;
    const float* hi;
    int k;            // n_subcell_depth
    int npts_side;    // 2^k + 1
    int npts;         // npts_side^3
    int group;        // leaves per CTA group
    float* tris;
    long long cap;
    unsigned long long* counter;
    int* err;
};

template <int TPI>
__global__ void __launch_bounds__(kNT) k_hmc(NiqModelRef M, HmcArgs a, unsigned long long* grab, int fixed_floats,
                                             int sw_cap, int resident) {
    using Cfg = TileCfg<8, 0, TPI, kNT>;
    constexpr int ITEMS = Cfg::ITEMS, R = Cfg::R, LD = Cfg::LD;
    constexpr int PPASS = ITEMS * 8;
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    float* st = smem;
    float* ob = st + Cfg::STATE_FLOATS;
    float* sW = smem + fixed_floats;
    __shared__ NiqSpecHeader H;
    __shared__ float s_vals[1024];       // grid values of the group (<= max(PPASS, 729))
    __shared__ float s_box[64][6];
    __shared__ long long s_base;
    load_header(H, M.hdr);
    __syncthreads();
    if (resident) stage_floats(sW, M.w, H.n_weight_floats);
    const RowPlan plan{ROWS_POINTS, 0, 8};
    const int item = threadIdx.x / TPI, g = threadIdx.x % TPI;
    const int ns = 1 << a.k;
    const int np = a.npts_side;
    while (true) {
        __syncthreads();
        if (threadIdx.x == 0) s_base = (long long)atomicAdd(grab, (unsigned long long)a.group);
        __syncthreads();
        const long long leaf0 = s_base;
        if (leaf0 >= a.n_leaves) break;
        const int gl = (int)min((long long)a.group, a.n_leaves - leaf0);
        for (int i = threadIdx.x; i < gl * 6; i += blockDim.x) {
            const int l = i / 6, c = i % 6;
            s_box[l][c] = c < 3 ? a.lo[3 * (leaf0 + l) + c] : a.hi[3 * (leaf0 + l) + c - 3];
        }
        __syncthreads();
        const int total = gl * a.npts;
        for (int p0 = 0; p0 < total; p0 += PPASS) {
            float* xs = st + item * R * LD;
            for (int r = g; r < 8; r += TPI) {
                const int p = p0 + item * 8 + r;
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (p < total) {
                    const int l = p / a.npts, li = p % a.npts;
                    const int i0 = li / (np * np), i1 = (li / np) % np, i2 = li % np;
                    const int ii[3] = {i0, i1, i2};
                    float c[3];
                    for (int k = 0; k < 3; ++k) {
                        const float s = __fdiv_rn((float)ii[k], (float)(np - 1));
                        c[k] = __fadd_rn(__fmul_rn(s_box[l][k], __fsub_rn(1.f, s)), __fmul_rn(s_box[l][3 + k], s));
                    }
                    v.x = c[0]; v.y = c[1]; v.z = c[2];
                }
                *reinterpret_cast<float4*>(xs + r * LD) = v;
            }
            __syncthreads();
            tile_forward<Cfg, false>(H, M.w, sW, sw_cap, resident, plan, st, ob);
            for (int r = g; r < 8; r += TPI) {
                const int p = p0 + item * 8 + r;
                if (p < total) s_vals[p] = ob[item * 8 + r];
            }
            __syncthreads();
        }
        // ---- polygonise every subcell of the group (lane-uniform loop for the warp votes)
        const int n_cells = gl * ns * ns * ns;
        for (int c0 = 0; c0 < n_cells; c0 += blockDim.x) {
            const int cid = c0 + threadIdx.x;
            const bool valid = cid < n_cells;
            int n_tri = 0;
            float ep[12][3];
            signed char row[16];
            if (valid) {
                const int l = cid / (ns * ns * ns), sc = cid % (ns * ns * ns);
                const int j0 = sc / (ns * ns), j1 = (sc / ns) % ns, j2 = sc % ns;
                const int jj[3] = {j0, j1, j2};
                float lo[3], hi[3];
                for (int k = 0; k < 3; ++k) {
                    const float delta = __fdiv_rn(__fsub_rn(s_box[l][3 + k], s_box[l][k]), (float)ns);
                    lo[k] = __fadd_rn(s_box[l][k], __fmul_rn((float)jj[k], delta));
                    hi[k] = __fadd_rn(lo[k], delta);
                }
                float vv[8];
                int cs = 0;
                for (int i = 0; i < 8; ++i) {
                    const int gi = ((j0 + c_vert[i][0]) * np + (j1 + c_vert[i][1])) * np + (j2 + c_vert[i][2]);
                    vv[i] = s_vals[l * a.npts + gi];
                    cs |= (vv[i] < 0.f) << i;
                }
                for (int e = 0; e < 12; ++e) {
                    const int ia = c_edge[e][0], ib = c_edge[e][1];
                    float t = __fdiv_rn(-vv[ia], __fsub_rn(vv[ib], vv[ia]));
                    if (t != t) t = 0.f;
                    t = fminf(fmaxf(t, 0.f), 1.f);
                    for (int k = 0; k < 3; ++k) {
                        const float pa = c_vert[ia][k] ? hi[k] : lo[k];
                        const float pb = c_vert[ib][k] ? hi[k] : lo[k];
                        ep[e][k] = __fadd_rn(__fmul_rn(__fsub_rn(1.f, t), pa), __fmul_rn(t, pb));
                    }
                }
                for (int i = 0; i < 16; ++i) row[i] = c_tri[cs][i];
                for (int tI = 0; tI < 5; ++tI) n_tri += row[3 * tI] != -1;
            }
            // warp-aggregated reservation of n_tri slots
            int incl = n_tri;
            const int lane = threadIdx.x & 31;
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, off);
                if (lane >= off) incl += y;
            }
            const int wsum = __shfl_sync(0xffffffffu, incl, 31);
            unsigned long long wbase = 0;
            if (lane == 31 && wsum > 0) wbase = atomicAdd(a.counter, (unsigned long long)wsum);
            wbase = __shfl_sync(0xffffffffu, wbase, 31);
            long long pos = (long long)wbase + (incl - n_tri);
            for (int tI = 0, w = 0; tI < 5 && w < n_tri; ++tI) {
                if (row[3 * tI] == -1) continue;
                if (pos + w < a.cap) {
                    float* dst = a.tris + 9 * (pos + w);
                    for (int vI = 0; vI < 3; ++vI)
                        for (int k = 0; k < 3; ++k) dst[3 * vI + k] = ep[row[3 * tI + vI]][k];
                } else {
                    niq_flag_error(a.err, NIQ_ERR_CAPACITY);
                }
                ++w;
            }
        }
    }
}

// ---------------------------------------------------------------------------------
// Shared corners (n_subcell_depth = 0 on a uniform tree).  The leaves of a uniform tree
// are cells of one lattice, and neighbouring leaves share their corner points exactly
// (a split plane is one float for both children), so each lattice vertex is evaluated
// once instead of once per leaf touching it.  k_lattice_mark gives every distinct corner
// a slot (the first leaf to reach it stores its coordinates), the point kernel evaluates
// the slots, and k_lattice_cells polygonises each leaf from its corners' slots with the
// same arithmetic as k_hmc.
// ---------------------------------------------------------------------------------
struct Lattice {
    float L[3], h[3];   // lower corner of the root, cell size
    int n[3];           // vertices per axis (cells + 1)
};

__device__ __forceinline__ long long lattice_index(const Lattice& G, const float* p) {
    long long idx = 0;
    for (int k = 0; k < 3; ++k) {
        int i = (int)rintf((p[k] - G.L[k]) / G.h[k]);
        i = min(max(i, 0), G.n[k] - 1);
        idx = idx * G.n[k] + i;
    }
    return idx;
}

__global__ void k_lattice_mark(long long n_leaves, const float* __restrict__ lo, const float* __restrict__ hi, Lattice G,
                               int* __restrict__ slot, unsigned long long* __restrict__ n_unique, float* __restrict__ pts,
                               long long cap, int* err) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 8 * n_leaves;
         t += (long long)gridDim.x * blockDim.x) {
        const long long l = t >> 3;
        const int c = (int)(t & 7);
        float p[3];
        for (int k = 0; k < 3; ++k) p[k] = c_vert[c][k] ? hi[3 * l + k] : lo[3 * l + k];
        const long long idx = lattice_index(G, p);
        if (atomicCAS(&slot[idx], -1, -2) == -1) {
            const unsigned long long pos = atomicAdd(n_unique, 1ull);
            if ((long long)pos < cap) {
                for (int k = 0; k < 3; ++k) pts[3 * pos + k] = p[k];
                slot[idx] = (int)pos;
            } else {
                niq_flag_error(err, NIQ_ERR_CAPACITY);
            }
        }
    }
}

__global__ void k_lattice_cells(long long n_leaves, const float* __restrict__ blo, const float* __restrict__ bhi,
                                Lattice G, const int* __restrict__ slot, const float* __restrict__ vals,
                                float* __restrict__ tris, long long cap, unsigned long long* counter, int* err) {
    for (long long l0 = blockIdx.x * (long long)blockDim.x; l0 < n_leaves; l0 += (long long)gridDim.x * blockDim.x) {
        const long long l = l0 + threadIdx.x;
        const bool valid = l < n_leaves;
        int n_tri = 0;
        float ep[12][3];
        signed char row[16];
        if (valid) {
            // the leaf is the only subcell: lower + {0, (upper - lower) / 1} as in k_hmc
            float lo[3], hi[3];
            for (int k = 0; k < 3; ++k) {
                const float delta = __fdiv_rn(__fsub_rn(bhi[3 * l + k], blo[3 * l + k]), 1.f);
                lo[k] = __fadd_rn(blo[3 * l + k], __fmul_rn(0.f, delta));
                hi[k] = __fadd_rn(lo[k], delta);
            }
            float vv[8];
            int cs = 0;
            for (int i = 0; i < 8; ++i) {
                float p[3];
                for (int k = 0; k < 3; ++k) p[k] = c_vert[i][k] ? bhi[3 * l + k] : blo[3 * l + k];
                const int sl = slot[lattice_index(G, p)];
                vv[i] = sl >= 0 ? vals[sl] : __int_as_float(0x7fffffff);   // every corner was marked
                cs |= (vv[i] < 0.f) << i;
            }
            for (int e = 0; e < 12; ++e) {
                const int ia = c_edge[e][0], ib = c_edge[e][1];
                float t = __fdiv_rn(-vv[ia], __fsub_rn(vv[ib], vv[ia]));
                if (t != t) t = 0.f;
                t = fminf(fmaxf(t, 0.f), 1.f);
                for (int k = 0; k < 3; ++k) {
                    const float pa = c_vert[ia][k] ? hi[k] : lo[k];
                    const float pb = c_vert[ib][k] ? hi[k] : lo[k];
                    ep[e][k] = __fadd_rn(__fmul_rn(__fsub_rn(1.f, t), pa), __fmul_rn(t, pb));
                }
            }
            for (int i = 0; i < 16; ++i) row[i] = c_tri[cs][i];
            for (int tI = 0; tI < 5; ++tI) n_tri += row[3 * tI] != -1;
        }
        int incl = n_tri;
        const int lane = threadIdx.x & 31;
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += y;
        }
        const int wsum = __shfl_sync(0xffffffffu, incl, 31);
        unsigned long long wbase = 0;
        if (lane == 31 && wsum > 0) wbase = atomicAdd(counter, (unsigned long long)wsum);
        wbase = __shfl_sync(0xffffffffu, wbase, 31);
        long long pos = (long long)wbase + (incl - n_tri);
        for (int tI = 0, w = 0; tI < 5 && w < n_tri; ++tI) {
            if (row[3 * tI] == -1) continue;
            if (pos + w < cap) {
                float* dst = tris + 9 * (pos + w);
                for (int vI = 0; vI < 3; ++vI)
                    for (int k = 0; k < 3; ++k) dst[3 * vI + k] = ep[row[3 * tI + vI]][k];
            } else {
                niq_flag_error(err, NIQ_ERR_CAPACITY);
            }
            ++w;
        }
    }
}

}  // namespace niq

using namespace niq;

extern "C" {

int niq_mc_table(int32_t* out) {
    NIQ_REQUIRE(out, NIQ_ERR_INVALID_ARG, "null argument");
    std::call_once(g_table_once, [] { build_mc_table(g_table); });
    for (int c = 0; c < 256; ++c)
        for (int i = 0; i < 16; ++i) out[16 * c + i] = g_table[c][i];
    return NIQ_OK;
}

size_t niq_hmc_workspace_size(void) { return 512; }

// The uniform tree's lattice: simulate split_depth bisections of the root (first longest
// axis, midpoint, float32 as the tree kernel does) to get the cell size per axis.
static int lattice_of(const float* root_lower, const float* root_upper, int split_depth, Lattice& G) {
    float lo[3] = {root_lower[0], root_lower[1], root_lower[2]}, hi[3] = {root_upper[0], root_upper[1], root_upper[2]};
    int splits[3] = {0, 0, 0};
    for (int s = 0; s < split_depth; ++s) {
        const float e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
        int d = 0;
        float em = e0;
        if (e1 > em) { d = 1; em = e1; }
        if (e2 > em) d = 2;
        hi[d] = 0.5f * (lo[d] + hi[d]);
        ++splits[d];
    }
    for (int k = 0; k < 3; ++k) {
        NIQ_REQUIRE(splits[k] < 24, NIQ_ERR_UNSUPPORTED, "lattice too fine");
        G.L[k] = root_lower[k];
        G.h[k] = hi[k] - lo[k];
        G.n[k] = (1 << splits[k]) + 1;
    }
    return NIQ_OK;
}

size_t niq_hmc_lattice_workspace_size(const float* root_lower, const float* root_upper, int32_t split_depth,
                                      int64_t n_leaves) {
    Lattice G;
    if (!root_lower || !root_upper || lattice_of(root_lower, root_upper, split_depth, G)) return 0;
    const size_t nv = (size_t)G.n[0] * G.n[1] * G.n[2];
    const size_t nu = (size_t)(8 * (n_leaves > 0 ? n_leaves : 0));   // distinct corners, at most 8 per leaf
    return 512 + ((nv * 4 + 255) & ~size_t(255)) + ((nu * 12 + 255) & ~size_t(255)) + ((nu * 4 + 255) & ~size_t(255));
}

int niq_hmc_extract_lattice(const niq_model* model, int64_t n_leaves, const float* leaf_lower, const float* leaf_upper,
                            const float* root_lower, const float* root_upper, int32_t split_depth, float* tris_out,
                            int64_t tri_capacity, int64_t* n_tris_out, void* workspace, size_t workspace_bytes,
                            void* stream) {
    NIQ_REQUIRE(model && n_tris_out && root_lower && root_upper && n_leaves >= 0 && tri_capacity >= 0,
                NIQ_ERR_INVALID_ARG, "bad argument");
    NIQ_REQUIRE(n_leaves == 0 || (leaf_lower && leaf_upper), NIQ_ERR_INVALID_ARG, "null leaf arrays");
    NIQ_REQUIRE(tri_capacity == 0 || tris_out, NIQ_ERR_INVALID_ARG, "null triangle array");
    Lattice G;
    int rc = lattice_of(root_lower, root_upper, split_depth, G);
    if (rc) return rc;
    const size_t need = niq_hmc_lattice_workspace_size(root_lower, root_upper, split_depth, n_leaves);
    NIQ_REQUIRE(workspace && workspace_bytes >= need, NIQ_ERR_CAPACITY, "workspace of %zu bytes needed", need);
    cudaStream_t s = as_stream(stream);
    rc = ensure_table();
    if (rc) return rc;
    NIQ_CUDA(cudaMemsetAsync(n_tris_out, 0, sizeof(int64_t), s));
    if (n_leaves == 0) return NIQ_OK;
    char* b = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
    unsigned long long* n_unique = reinterpret_cast<unsigned long long*>(b);
    int* err = reinterpret_cast<int*>(b + 8);
    const size_t nv = (size_t)G.n[0] * G.n[1] * G.n[2];
    const long long nu_cap = 8 * n_leaves;
    int* slot = reinterpret_cast<int*>(b + 256);
    float* pts = reinterpret_cast<float*>(b + 256 + ((nv * 4 + 255) & ~size_t(255)));
    float* vals = pts + (((size_t)nu_cap * 12 + 255) & ~size_t(255)) / 4;
    NIQ_CUDA(cudaMemsetAsync(b, 0, 16, s));
    NIQ_CUDA(cudaMemsetAsync(slot, 0xFF, nv * 4, s));   // -1: not yet claimed
    const int grid = (int)std::min<long long>((8 * n_leaves + 255) / 256, 8 * 1024);
    k_lattice_mark<<<grid, 256, 0, s>>>(n_leaves, leaf_lower, leaf_upper, G, slot, n_unique, pts, nu_cap, err);
    NIQ_CUDA(cudaGetLastError());
    unsigned long long nu = 0;
    NIQ_CUDA(cudaMemcpyAsync(&nu, n_unique, 8, cudaMemcpyDeviceToHost, s));
    NIQ_CUDA(cudaStreamSynchronize(s));
    NIQ_REQUIRE((long long)nu <= nu_cap, NIQ_ERR_CAPACITY, "distinct corners overflow");
    rc = niq_eval_points(model, (int64_t)nu, pts, vals, stream);
    if (rc) return rc;
    const int grid2 = (int)std::min<long long>((n_leaves + 255) / 256, 8 * 1024);
    k_lattice_cells<<<grid2, 256, 0, s>>>(n_leaves, leaf_lower, leaf_upper, G, slot, vals, tris_out, tri_capacity,
                                          reinterpret_cast<unsigned long long*>(n_tris_out), err);
    NIQ_CUDA(cudaGetLastError());
    long long n = 0;
    int e = 0;
    NIQ_CUDA(cudaMemcpyAsync(&n, n_tris_out, 8, cudaMemcpyDeviceToHost, s));
    NIQ_CUDA(cudaMemcpyAsync(&e, err, 4, cudaMemcpyDeviceToHost, s));
    NIQ_CUDA(cudaStreamSynchronize(s));
    NIQ_REQUIRE(n <= tri_capacity, NIQ_ERR_CAPACITY, "%lld triangles exceed the capacity %lld", n, (long long)tri_capacity);
    NIQ_REQUIRE(e == 0, e, "lattice extraction error %d", e);
    return NIQ_OK;
}

int niq_hmc_extract(const niq_model* model, int64_t n_leaves, const float* leaf_lower, const float* leaf_upper,
                    int32_t n_subcell_depth, float* tris_out, int64_t tri_capacity, int64_t* n_tris_out,
                    void* workspace, size_t workspace_bytes, void* stream) {
    NIQ_REQUIRE(model && n_tris_out && n_leaves >= 0 && tri_capacity >= 0, NIQ_ERR_INVALID_ARG, "bad argument");
    NIQ_REQUIRE(n_subcell_depth >= 0 && n_subcell_depth <= 3, NIQ_ERR_UNSUPPORTED, "n_subcell_depth must be in [0, 3]");
    NIQ_REQUIRE(n_leaves == 0 || (leaf_lower && leaf_upper), NIQ_ERR_INVALID_ARG, "null leaf arrays");
    NIQ_REQUIRE(tri_capacity == 0 || tris_out, NIQ_ERR_INVALID_ARG, "null triangle array");
    cudaStream_t s = as_stream(stream);
    int rc = ensure_table();
    if (rc) return rc;
    NIQ_REQUIRE(workspace && workspace_bytes >= niq_hmc_workspace_size(), NIQ_ERR_CAPACITY, "workspace too small");
    // n_tris_out doubles as the append counter; overflow shows in the final count
    NIQ_CUDA(cudaMemsetAsync(n_tris_out, 0, sizeof(int64_t), s));
    if (n_leaves == 0) return NIQ_OK;
    // workspace: the leaf claim counter and the error flag
    unsigned long long* d_aux =
        reinterpret_cast<unsigned long long*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
    NIQ_CUDA(cudaMemsetAsync(d_aux, 0, 16, s));
    HmcArgs a;
    a.n_leaves = n_leaves;
    a.lo = leaf_lower;
    a.hi = leaf_upper;
    a.k = n_subcell_depth;
    a.npts_side = (1 << n_subcell_depth) + 1;
    a.npts = a.npts_side * a.npts_side * a.npts_side;
    a.tris = tris_out;
    a.cap = tri_capacity;
    a.counter = reinterpret_cast<unsigned long long*>(n_tris_out);
    a.err = reinterpret_cast<int*>(d_aux + 1);
    const int tpi = tpi_for_width(model->hdr.max_width);
    NIQ_DISPATCH_TPI(tpi, {
        auto kern = k_hmc<TPI>;
        const int items = kNT / TPI;
        const int ppass = items * 8;
        a.group = a.npts <= ppass ? (ppass / a.npts < 64 ? ppass / a.npts : 64) : 1;
        const int state = items * 8 * (TPI * 8 + 4) + ((items * 8 + 3) & ~3);
        SmemPlan p = plan_smem(state, model->hdr.n_weight_floats, max_layer_floats(model->hdr), 96 * 1024);
        rc = prepare_kernel(kern, p.bytes);
        if (rc) return rc;
        int grid = 0;
        rc = persistent_grid(kern, kNT, p.bytes, (n_leaves + a.group - 1) / a.group, &grid);
        if (rc) return rc;
        kern<<<grid, kNT, p.bytes, s>>>(model->ref(), a, d_aux, p.fixed_floats, p.sw_cap, p.resident);
    });
    NIQ_CUDA(cudaGetLastError());
    long long n = 0;
    NIQ_CUDA(cudaMemcpyAsync(&n, n_tris_out, 8, cudaMemcpyDeviceToHost, s));
    NIQ_CUDA(cudaStreamSynchronize(s));
    NIQ_REQUIRE(n <= tri_capacity, NIQ_ERR_CAPACITY, "%lld triangles exceed the capacity %lld", n, (long long)tri_capacity);
    return NIQ_OK;
}

}  // extern "C"
