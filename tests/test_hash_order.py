"""CPU: the device-side model of libstdc++'s unordered-container iteration order (sb_common.cuh) against
the live library, compiled as host code."""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = "/usr/local/cuda/include"

PROG = r"""
#include <unordered_set>
#include <vector>
#include <random>
#include <cstdio>
#include "sb_common.cuh"
int main() {
  // bucket schedule against the library
  std::unordered_set<size_t> s; size_t prev = 0; int bad = 0;
  for (size_t n = 1; n <= 3000000; ++n) { s.insert(n * 7); if (s.bucket_count() != sbg::hash_bucket_count((uint32_t)n)) { bad++; break; } }
  // iteration order on random sequences
  std::mt19937_64 rng(3);
  for (int t = 0; t < 4000 && !bad; ++t) {
    int n = rng() % 700 + 1; size_t range = (t % 3 == 0) ? 40 : (t % 3 == 1 ? 3000 : 1000000000);
    std::unordered_set<size_t> u; std::vector<uint64_t> keys;
    for (int i = 0; i < n; ++i) { size_t k = rng() % range; if (u.insert(k).second) keys.push_back(k); }
    std::vector<int> next(keys.size() + 1), order(keys.size() + 1), bucket(sbg::hash_bucket_count((uint32_t)keys.size() + 1));
    sbg::hash_iteration_order(keys.data(), (int)keys.size(), next.data(), bucket.data(), order.data());
    size_t i = 0; for (size_t k : u) { if (keys[order[i++]] != k) { bad++; break; } }
  }
  printf("%d\n", bad); return bad;
}
"""


def test_hash_iteration_order_matches_libstdcxx():
    if not os.path.isdir(CUDA_INC):
        pytest.skip("CUDA headers not present")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "h.cpp")
        open(src, "w").write(PROG)
        exe = os.path.join(d, "h")
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "solidboolean_gb300", "csrc"),
                               "-I", CUDA_INC, src, "-o", exe])
        assert subprocess.run([exe]).returncode == 0
