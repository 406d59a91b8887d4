/* cpu_tree.c -- CPU restatement of the level-set tree (src/kd_tree.py:19-218) over
 * affine_fixed bounds (src/affine.py:109-193, src/affine_layers.py:11-56) and of the
 * marching-cubes extraction on its leaves (src/kd_tree.py:357-399 with n_subcell_depth
 * 0, src/extract_cell.py:314-421), in C with OpenMP, for the CPU baseline of the
 * benchmark and as a second checker of the tree.
 *
 * Test infrastructure: only the tests and the benchmark's CPU-baseline leg call it.
 *
 * Each node's box (center, three axis half-extents as noise rows, err 0) goes through
 * the dense layers (base <- base A + b, aff <- aff A, err <- err |A|) and the ReLU/ELU
 * linearisations applied as 'affine_fixed' (err <- alpha err + delta) in float32 with
 * round-to-nearest and no contraction, the reference's arithmetic (other activations are
 * rejected).  A node is UNKNOWN when its bound straddles the offset band; UNKNOWN nodes
 * split at the midpoint of their first longest axis; the last round keeps them as
 * leaves.  Each level classifies its nodes in parallel (OpenMP), then builds the children
 * in node order, so the leaf set and its order match the reference's schedule.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXW 256
#define MAXL 32

typedef struct {
    int n_layers;
    int in[MAXL], out[MAXL], act[MAXL];   /* act: 0 none, 1 relu, 2 elu */
    const float* A[MAXL];                /* (in, out) row-major */
    const float* b[MAXL];
} Net;

static float eluf_(float x) { return x > 0.f ? x : expm1f(x); }

/* alpha, beta, delta of src/affine_layers.py:34-97 (ReLU, ELU) */
static void linearize(int act, float l, float u, float* a, float* be, float* d) {
    if (act == 1) {
        float al;
        if (l >= 0.f) al = 1.f;
        else if (u < 0.f) al = 0.f;
        else al = (fmaxf(u, 0.f) - fmaxf(l, 0.f)) / (u - l);
        if (al != al) al = 0.f;
        al = fminf(fmaxf(al, 0.f), 1.f);
        *a = al;
        *be = (fmaxf(l, 0.f) - al * l) * 0.5f;
        *d = fabsf(*be);
        return;
    }
    if (act == 2) {
        const float lF = eluf_(l), uF = eluf_(u);
        const float lS = fminf(expf(l), 1.f), uS = fminf(expf(u), 1.f);
        float al = (uF - lF) / (u - l);
        if (l >= 0.f) al = 1.f;
        if (al != al) al = 0.f;
        al = fminf(fmaxf(al, lS), uS);
        if (l >= 0.f) { *a = 1.f; *be = 0.f; *d = 0.f; return; }
        const float r_upper = lF - al * l;
        const float xl = fminf(fmaxf(logf(al), l), u);
        const float r_lower = (al - 1.f) - al * xl;
        *a = al;
        *be = 0.5f * (r_upper + r_lower);
        *d = 0.5f * fabsf(r_upper - r_lower);
        return;
    }
    /* other activations are not restated here */
    *a = 0.f;
    *be = 0.f;
    *d = INFINITY;
}

/* sign of the affine_fixed bound of the box: 1 positive, -1 negative, 0 unknown */
static int classify(const Net* N, const float* lo, const float* hi, float offset) {
    float base[MAXW], aff[3][MAXW], err[MAXW];
    float nb[MAXW], na[3][MAXW], ne[MAXW];
    int w = 3;
    for (int k = 0; k < 3; ++k) {
        const float c = 0.5f * (lo[k] + hi[k]);
        base[k] = c;
        err[k] = 0.f;
        for (int r = 0; r < 3; ++r) aff[r][k] = (r == k) ? hi[k] - c : 0.f;
    }
    for (int li = 0; li < N->n_layers; ++li) {
        const int in = N->in[li], out = N->out[li];
        const float* A = N->A[li];
        for (int j = 0; j < out; ++j) { nb[j] = 0.f; ne[j] = 0.f; na[0][j] = na[1][j] = na[2][j] = 0.f; }
        for (int k = 0; k < in; ++k) {
            const float* row = A + (size_t)k * out;
            const float bk = base[k], ek = err[k], a0 = aff[0][k], a1 = aff[1][k], a2 = aff[2][k];
            for (int j = 0; j < out; ++j) {
                const float x = row[j];
                nb[j] += bk * x;
                na[0][j] += a0 * x;
                na[1][j] += a1 * x;
                na[2][j] += a2 * x;
                ne[j] += ek * fabsf(x);
            }
        }
        for (int j = 0; j < out; ++j) {
            float bj = nb[j] + (N->b[li] ? N->b[li][j] : 0.f);
            float e = ne[j];
            float a0 = na[0][j], a1 = na[1][j], a2 = na[2][j];
            if (N->act[li]) {
                const float rad = fabsf(a0) + fabsf(a1) + fabsf(a2) + e;
                float al, be, de;
                linearize(N->act[li], bj - rad, bj + rad, &al, &be, &de);
                bj = al * bj + be;
                a0 *= al; a1 *= al; a2 *= al;
                e = al * e + fabsf(de);
            }
            base[j] = bj; err[j] = e; aff[0][j] = a0; aff[1][j] = a1; aff[2][j] = a2;
        }
        w = out;
    }
    (void)w;
    const float rad = fabsf(aff[0][0]) + fabsf(aff[1][0]) + fabsf(aff[2][0]) + err[0];
    if (base[0] - rad > offset) return 1;
    if (base[0] + rad < -offset) return -1;
    return 0;
}

/* Builds the tree to split_depth bisections; returns the number of unknown leaves and
 * writes the number of classified boxes to *n_boxes.  If leaves is not NULL it receives
 * up to cap leaves as (lower[3], upper[3]). */
int64_t cpu_levelset_tree(int n_layers, const int* in, const int* out, const int* act, const float* const* A,
                          const float* const* b, const float* lower, const float* upper, int split_depth, float offset,
                          int threads, int64_t* n_boxes, float* leaves, int64_t cap) {
    Net N;
    if (n_layers < 1 || n_layers > MAXL) return -1;
    N.n_layers = n_layers;
    for (int i = 0; i < n_layers; ++i) {
        if (in[i] > MAXW || out[i] > MAXW || act[i] < 0 || act[i] > 2) return -1;
        N.in[i] = in[i]; N.out[i] = out[i]; N.act[i] = act[i]; N.A[i] = A[i]; N.b[i] = b[i];
    }
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    int64_t n = 1, boxes = 0, n_leaves = 0;
    float* cur = (float*)malloc(6 * sizeof(float));
    for (int k = 0; k < 3; ++k) { cur[k] = lower[k]; cur[3 + k] = upper[k]; }
    for (int level = 0; level <= split_depth && n > 0; ++level) {
        const int last = level == split_depth;
        unsigned char* type = (unsigned char*)malloc((size_t)n);
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) type[i] = (unsigned char)(classify(&N, cur + 6 * i, cur + 6 * i + 3, offset) == 0);
        boxes += n;
        int64_t m = 0;
        for (int64_t i = 0; i < n; ++i) m += type[i];
        if (last) {
            if (leaves) {
                int64_t o = 0;
                for (int64_t i = 0; i < n && o < cap; ++i)
                    if (type[i]) { memcpy(leaves + 6 * o, cur + 6 * i, 6 * sizeof(float)); ++o; }
            }
            n_leaves = m;
            free(type);
            break;
        }
        float* nxt = (float*)malloc((size_t)(2 * m > 0 ? 2 * m : 1) * 6 * sizeof(float));
        int64_t o = 0;
        /* the reference's order: per batch of 2048 nodes (src/kd_tree.py:141-172), the
         * A children of its unknown nodes, then their B children */
        for (int64_t b0 = 0; b0 < n; b0 += 2048) {
            const int64_t b1 = b0 + 2048 < n ? b0 + 2048 : n;
            for (int half = 0; half < 2; ++half)
                for (int64_t i = b0; i < b1; ++i) {
                    if (!type[i]) continue;
                    const float* lo = cur + 6 * i;
                    const float* hi = lo + 3;
                    const float e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
                    int d = 0;
                    float em = e0;
                    if (e1 > em) { d = 1; em = e1; }
                    if (e2 > em) d = 2;
                    const float mid = 0.5f * (lo[d] + hi[d]);
                    float* c = nxt + 6 * o;
                    memcpy(c, lo, 6 * sizeof(float));
                    if (half == 0) c[3 + d] = mid;   /* A: upper[d] = mid */
                    else c[d] = mid;                 /* B: lower[d] = mid */
                    ++o;
                }
        }
        free(type);
        free(cur);
        cur = nxt;
        n = o;
    }
    free(cur);
    if (n_boxes) *n_boxes = boxes;
    return n_leaves;
}


/* Plain forward pass of one point (src/mlp.py:253-347, float32, no contraction). */
static float eval_point(const Net* N, const float* x) {
    float a[MAXW], b[MAXW];
    float* cur = a;
    float* nxt = b;
    cur[0] = x[0]; cur[1] = x[1]; cur[2] = x[2];
    for (int li = 0; li < N->n_layers; ++li) {
        const int in = N->in[li], out = N->out[li];
        const float* A = N->A[li];
        for (int j = 0; j < out; ++j) nxt[j] = 0.f;
        for (int k = 0; k < in; ++k) {
            const float xk = cur[k];
            const float* row = A + (size_t)k * out;
            for (int j = 0; j < out; ++j) nxt[j] += xk * row[j];
        }
        for (int j = 0; j < out; ++j) {
            float v = nxt[j] + (N->b[li] ? N->b[li][j] : 0.f);
            if (N->act[li] == 1) v = fmaxf(v, 0.f);
            else if (N->act[li] == 2) v = eluf_(v);
            nxt[j] = v;
        }
        float* t = cur; cur = nxt; nxt = t;
    }
    return cur[0];
}

/* Marching cubes on each leaf box as one cell (n_subcell_depth 0): the 8 corners
 * (corner i at vert[i] in {0,1}^3: upper where 1, lower where 0), case bit i set when
 * the value at corner i is negative, and for every triangle of tri_table[case] (256 x
 * 16, -1 padded) the vertices on edges (edge[e] = corners a, b) at
 * t = clip(nan_to_num(-va / (vb - va)), 0, 1), p = (1 - t) pa + t pb.  Returns the number
 * of triangles; writes up to cap of them to tris (T, 3, 3) in leaf order. */
int64_t cpu_hmc_leaves(int n_layers, const int* in, const int* out, const int* act, const float* const* A,
                       const float* const* b, const float* leaves, int64_t n, const int* tri_table, const int* edge,
                       const int* vert, int threads, float* tris, int64_t cap) {
    Net N;
    if (n_layers < 1 || n_layers > MAXL) return -1;
    N.n_layers = n_layers;
    for (int i = 0; i < n_layers; ++i) {
        if (in[i] > MAXW || out[i] > MAXW || act[i] < 0 || act[i] > 2) return -1;
        N.in[i] = in[i]; N.out[i] = out[i]; N.act[i] = act[i]; N.A[i] = A[i]; N.b[i] = b[i];
    }
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    float* vals = (float*)malloc((size_t)(n > 0 ? n : 1) * 8 * sizeof(float));
    int64_t* first = (int64_t*)malloc((size_t)(n + 1) * sizeof(int64_t));
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        const float* lo = leaves + 6 * i;
        const float* hi = lo + 3;
        int cs = 0;
        for (int c = 0; c < 8; ++c) {
            float p[3];
            for (int k = 0; k < 3; ++k) p[k] = vert[3 * c + k] ? hi[k] : lo[k];
            const float v = eval_point(&N, p);
            vals[8 * i + c] = v;
            if (v < 0.f) cs |= 1 << c;
        }
        int nt = 0;
        while (nt < 5 && tri_table[16 * cs + 3 * nt] != -1) ++nt;
        first[i + 1] = nt;
    }
    first[0] = 0;
    for (int64_t i = 0; i < n; ++i) first[i + 1] += first[i];
    const int64_t total = first[n];
    if (tris) {
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            const float* lo = leaves + 6 * i;
            const float* hi = lo + 3;
            const float* v = vals + 8 * i;
            int cs = 0;
            for (int c = 0; c < 8; ++c) if (v[c] < 0.f) cs |= 1 << c;
            int64_t o = first[i];
            for (int t = 0; t < 5 && o < cap; ++t, ++o) {
                const int* e3 = tri_table + 16 * cs + 3 * t;
                if (e3[0] == -1) break;
                for (int q = 0; q < 3; ++q) {
                    const int ca = edge[2 * e3[q]], cb = edge[2 * e3[q] + 1];
                    const float va = v[ca], vb = v[cb];
                    float tc = -va / (vb - va);
                    if (tc != tc) tc = 0.f;
                    if (tc > 3.4028234663852886e38f) tc = 3.4028234663852886e38f;
                    if (tc < -3.4028234663852886e38f) tc = -3.4028234663852886e38f;
                    tc = fminf(fmaxf(tc, 0.f), 1.f);
                    for (int k = 0; k < 3; ++k) {
                        const float pa = vert[3 * ca + k] ? hi[k] : lo[k];
                        const float pb = vert[3 * cb + k] ? hi[k] : lo[k];
                        tris[9 * o + 3 * q + k] = (1.f - tc) * pa + tc * pb;
                    }
                }
            }
        }
    }
    free(vals);
    free(first);
    return total;
}
