"""The invariant-divisor division of the generic kernels' cell coordinates
(hd::divu64 in hyperdeal_gb300/csrc/hd_ecl.cuh, Granlund-Montgomery 1994,
Figure 4.1 with 64-bit words).

Its host branch (the same formula with a 128-bit multiply-high in place of
__umul64hi) is compiled by nvcc into a small host program and checked against
the hardware division for divisors 1..2000, powers of two and their
neighbours and large divisors, at the edges of every quotient and at random
dividends up to 2^64 - 1.  No GPU involved.
"""
import os
import shutil
import subprocess

import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "hyperdeal_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include <random>
#include "hd_ecl.cuh"

static int check(unsigned long long d, unsigned long long n, const hd::DivU64& v) {
  const unsigned long long q = hd::divu64(n, v);
  if (q != n / d) {
    std::printf("d=%llu n=%llu q=%llu want %llu\n", d, n, q, n / d);
    return 1;
  }
  return 0;
}

int main() {
  std::vector<unsigned long long> ds;
  for (unsigned long long d = 1; d <= 2000; ++d) ds.push_back(d);
  for (int k = 1; k < 64; ++k) {
    const unsigned long long p = 1ULL << k;
    ds.push_back(p - 1);
    ds.push_back(p);
    ds.push_back(p + 1);
  }
  ds.push_back(4096ULL * 4096ULL * 3ULL);
  ds.push_back(0xFFFFFFFFFFFFFFFFULL);
  std::mt19937_64 rng(7);
  for (int i = 0; i < 200; ++i) ds.push_back(rng() >> (rng() % 64) | 1ULL);
  long long bad = 0, n_checked = 0;
  for (unsigned long long d : ds) {
    const hd::DivU64 v = hd::make_divu64(d);
    const unsigned long long edge[] = {0ULL, 1ULL, d - 1, d, d + 1, 2 * d - 1, 2 * d, 0xFFFFFFFFULL,
                                       0xFFFFFFFFFFFFFFFFULL, 0xFFFFFFFFFFFFFFFFULL - d,
                                       (0xFFFFFFFFFFFFFFFFULL / d) * d, (0xFFFFFFFFFFFFFFFFULL / d) * d - 1};
    for (unsigned long long n : edge) { bad += check(d, n, v); ++n_checked; }
    for (int i = 0; i < 2000; ++i) {
      const unsigned long long n = rng() >> (rng() % 64);
      bad += check(d, n, v);
      const unsigned long long q = n / d;
      if (q > 0) bad += check(d, q * d - 1, v) + check(d, q * d, v);
      n_checked += 3;
      if (bad > 10) return 1;
    }
  }
  std::printf("checked %lld bad %lld\n", n_checked, bad);
  return bad ? 1 : 0;
}
"""


def test_divu64_matches_hardware_division(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "divu64_check.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "divu64_check"
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-I", CSRC, str(src), "-o", str(exe)], capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout
