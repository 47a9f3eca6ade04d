"""CPU: pgx_half_signed (pypde_gb300/csrc/pgx_exact.cuh) equals x * (+-0.5) bit for bit.

The DCT kernels scale by +-1/2 on the bit pattern (integer instructions) instead of an FP64
multiply.  The same header compiles for the host; this test builds a small harness with g++ and
compares it with the host's IEEE multiply on random 64-bit patterns (every exponent, subnormals
included) and on the edge cases: signed zeros, the smallest subnormals, the normal/subnormal
boundary with ties, the largest finite numbers and infinities.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "pypde_gb300", "csrc")

HARNESS = r"""
#include <stdio.h>
#include <stdint.h>
#include <string.h>
#include "pgx_exact.cuh"

static uint64_t state = 0x9E3779B97F4A7C15ULL;
static uint64_t next64(void) {  /* splitmix64 */
  uint64_t z = (state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static int check(uint64_t bits, long* bad) {
  double x, want, got;
  memcpy(&x, &bits, 8);
  if (x != x) return 0;                       /* NaN: only NaN-ness is promised */
  for (int neg = 0; neg < 2; ++neg) {
    volatile double h = neg ? -0.5 : 0.5;
    want = x * h;
    got = pgx_half_signed(x, neg != 0);
    if (memcmp(&want, &got, 8) != 0) {
      if (*bad < 5) printf("mismatch %016llx neg=%d\n", (unsigned long long)bits, neg);
      ++*bad;
    }
  }
  return 1;
}
int main(void) {
  long bad = 0, n = 0;
  for (long i = 0; i < 4000000; ++i) n += check(next64(), &bad);
  /* low exponents densely: subnormals and the first normal binades, both signs */
  for (long i = 0; i < 2000000; ++i) {
    uint64_t b = next64();
    b = (b & 0x800FFFFFFFFFFFFFULL) | ((uint64_t)(i % 4) << 52);
    n += check(b, &bad);
  }
  const uint64_t edge[] = {0x0ULL, 0x8000000000000000ULL, 0x1ULL, 0x8000000000000001ULL, 0x2ULL, 0x3ULL,
                           0x000FFFFFFFFFFFFFULL, 0x0010000000000000ULL, 0x0010000000000001ULL,
                           0x001FFFFFFFFFFFFFULL, 0x0020000000000000ULL, 0x7FEFFFFFFFFFFFFFULL,
                           0x7FF0000000000000ULL, 0xFFF0000000000000ULL, 0x3FF0000000000000ULL};
  for (unsigned i = 0; i < sizeof edge / sizeof edge[0]; ++i) n += check(edge[i], &bad);
  printf("checked %ld mismatches %ld\n", n, bad);
  return bad != 0;
}
"""


def test_half_signed_equals_the_fp64_multiply():
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "h.cpp"), os.path.join(d, "h")
        with open(src, "w") as f:
            f.write(HARNESS)
        r = subprocess.run([cxx, "-O2", "-ffp-contract=off", "-I", CSRC, src, "-o", exe], capture_output=True,
                           text=True)
        assert r.returncode == 0, r.stderr
        r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout
        assert "mismatches 0" in r.stdout
