"""CPU: the integer division by three used for the reference tree's box centres (sb_common.cuh div3_rn)
against IEEE double division, compiled as host code."""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = "/usr/local/cuda/include"

PROG = r"""
#include <cstdio>
#include <cmath>
#include <random>
#include "sb_common.cuh"
static int check(double x) {
  double a = sbg::div3_rn(x), b = x / 3.0;
  if (std::isnan(b)) return std::isnan(a) ? 0 : 1;
  return sbg::dbl_bits(a) == sbg::dbl_bits(b) ? 0 : 1;
}
int main() {
  std::mt19937_64 rng(11);
  long bad = 0;
  // random bit patterns (every exponent, sign, subnormals, infinities and NaNs)
  for (long i = 0; i < 4000000; ++i) bad += check(sbg::bits_dbl(rng()));
  // sums of three coordinates, as the centres are formed
  std::uniform_real_distribution<double> U(-10.0, 10.0);
  for (long i = 0; i < 2000000; ++i) { double s = 0.0; s = s + U(rng); s = s + U(rng); s = s + U(rng); bad += check(s); }
  // neighbourhoods of exact multiples of three and of powers of two (ties, carries into the exponent)
  for (int e = -1070; e < 1024; ++e) {
    double p = std::ldexp(1.0, e);
    for (int k = -4; k <= 4; ++k) { bad += check(std::nextafter(p, k < 0 ? 0.0 : INFINITY)); bad += check(3 * p + k * std::ldexp(p, -52)); }
  }
  for (long m = 1; m < 200000; ++m) { bad += check((double)m); bad += check(-(double)(3 * m)); bad += check((double)m * 0.75); }
  bad += check(0.0) + check(-0.0) + check(INFINITY) + check(-INFINITY) + check(NAN) + check(DBL_MAX) + check(DBL_MIN) + check(-DBL_MIN * 3);
  printf("%ld\n", bad); return bad != 0;
}
"""


def test_div3_matches_ieee_division():
    if not os.path.isdir(CUDA_INC):
        pytest.skip("CUDA headers not present")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "d3.cpp")
        open(src, "w").write(PROG)
        exe = os.path.join(d, "d3")
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                               os.path.join(ROOT, "solidboolean_gb300", "csrc"), "-I", CUDA_INC, src, "-o", exe])
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout
