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
int main() {
    alignas(16) float s[512];
    long bad = 0, tot = 0;
    srand(7);
    for (int trial = 0; trial < 300; ++trial) {
        const int n = 1 + rand() % 512;
        for (int i = 0; i < n; ++i) s[i] = (rand() % 4 == 0) ? 0.f : (float)(rand() % 9);  // many ties
        if (trial % 50 == 0) s[rand() % n] = NAN;
        for (int me = 0; me < n; ++me)
            for (int lane = 0; lane < 32 && lane <= me; lane += 5) {
                const float v = s[me];
                int ref = 0;   // stable descending argsort position
                for (int i = 0; i < n; ++i) ref += (s[i] > v) || (s[i] == v && i < me);
                bad += stable_rank(s, n, v, me, me - lane) != ref;
                ++tot;
            }
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


def test_stable_rank_matches_naive_count(tmp_path):
    """k_wide_tc.cu's stable_rank (float4 steps outside the warp's index window) gives the
    same rank as counting every element with the index tie rule, ties and NaN included."""
    if shutil.which('g++') is None:
        pytest.skip('g++ not available')
    fn = _function_text(os.path.join(CSRC, 'k_wide_tc.cu'), '__device__ __forceinline__ int stable_rank')
    cpp = tmp_path / 'rank.cpp'
    cpp.write_text(SHIM + fn + MAIN)
    exe = tmp_path / 'rank'
    subprocess.run(['g++', '-O2', '-o', str(exe), str(cpp)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    bad, tot = int(out[0]), int(out[1])
    assert tot > 100000
    assert bad == 0
