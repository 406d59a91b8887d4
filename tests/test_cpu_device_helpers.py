"""Host checks of branch-free / windowed device helpers, compiled from the CUDA sources.

The helper's text is cut from the .cu file and compiled with g++ under small shims for
the CUDA qualifiers, so the test exercises the exact code the kernel runs, on the CPU.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), 'neural-implicit-queries_gb300', 'csrc')

SHIM = r'''
#include <cmath>
#include <cstdio>
#include <cstdlib>
struct float4 { float x, y, z, w; };
#define __device__
#define __forceinline__ inline
'''

MAIN = r'''
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
// The selection of k_wide_tc on the host: the device's 4-pass radix select (histograms
// of 8-bit digits, the per-lane digit search over lanes whose 'above' counts are the
// exclusive prefix over lanes), then the tie rule and the candidate-order packing.
static uint32_t bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
int main() {
    srand(7);
    long bad = 0, tot = 0;
    for (int trial = 0; trial < 3000; ++trial) {
        const int n = 2 + rand() % 512;
        std::vector<float> key(n);
        const int style = trial % 4;
        for (int i = 0; i < n; ++i) {
            if (style == 0) key[i] = (rand() % 4 == 0) ? 0.f : (float)(rand() % 9);            // many ties
            else if (style == 1) key[i] = ldexpf((float)rand() / RAND_MAX, -(rand() % 60));    // spread exponents
            else if (style == 2) key[i] = 1.f + (rand() % 3) * 1e-7f;                          // one top digit
            else key[i] = (float)rand() / RAND_MAX;
        }
        if (trial % 97 == 0) key[rand() % n] = INFINITY;
        const int K = 1 + rand() % (n - 1);
        // device algorithm
        uint32_t prefix = 0, mask = 0;
        int kk = K;
        for (int pass = 0; pass < 4; ++pass) {
            const int shift = 24 - 8 * pass;
            int h[256] = {0};
            for (int i = 0; i < n; ++i)
                if ((bits(key[i]) & mask) == prefix) h[(bits(key[i]) >> shift) & 255u]++;
            int sel[2] = {-1, -1}, above = 0;
            for (int lane = 0; lane < 32; ++lane) {
                int t = 0;
                for (int e = 0; e < 8; ++e) t += h[255 - 8 * lane - e];
                kth_digit_in_lane(h, lane, above, kk, sel);
                above += t;
            }
            if (sel[0] < 0) { ++bad; break; }
            kk -= sel[1];
            prefix |= (uint32_t)sel[0] << shift;
            mask |= 255u << shift;
        }
        const uint32_t T = prefix;
        const int n_gt = K - kk;
        std::vector<int> kept(n, 0);
        int ties = 0;
        for (int i = 0; i < n; ++i) {
            const uint32_t b = bits(key[i]);
            kept[i] = b > T || (b == T && ties < K - n_gt);
            ties += b == T;
        }
        // reference: stable descending argsort, first K
        std::vector<int> idx(n);
        for (int i = 0; i < n; ++i) idx[i] = i;
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return key[a] > key[b]; });
        std::vector<int> ref(n, 0);
        for (int r = 0; r < K; ++r) ref[idx[r]] = 1;
        int nk = 0;
        for (int i = 0; i < n; ++i) { bad += kept[i] != ref[i]; nk += kept[i]; }
        bad += nk != K;
        ++tot;
    }
    printf("%ld %ld\n", bad, tot);
    return 0;
}
'''


def _function_text(path, signature):
    src = open(path).read()
    i = src.index(signature)
    j = src.index('\n}\n', i) + 3
    return src[i:j]


def test_radix_select_keeps_the_stable_top_k(tmp_path):
    """k_wide_tc.cu's per-lane digit search (kth_digit_in_lane), driven through the four
    8-bit passes of its block radix select and the tie rule, keeps exactly the rows a stable
    descending argsort keeps first (src/affine.py:150-155): ties, zeros, spread exponents
    and infinities included."""
    if shutil.which('g++') is None:
        pytest.skip('g++ not available')
    fn = _function_text(os.path.join(CSRC, 'k_wide_tc.cu'), '__device__ __forceinline__ void kth_digit_in_lane')
    cpp = tmp_path / 'select.cpp'
    cpp.write_text(SHIM + fn + MAIN)
    exe = tmp_path / 'select'
    subprocess.run(['g++', '-O2', '-o', str(exe), str(cpp)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    bad, tot = int(out[0]), int(out[1])
    assert tot == 3000
    assert bad == 0
