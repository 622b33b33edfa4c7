"""The integer-pipe FP64 <-> FP32 conversions of the nodal update (ci_fpconv.h) against
the host's IEEE conversions, bit for bit for every input: the FP32 normal range with its
ties and mantissa carries, signed zeros, and the ranges that fall back to the hardware
conversion (subnormals, overflow, infinities, NaNs)."""
import os
import subprocess

import pytest

from conftest import ROOT

SRC = r'''
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <random>
#include <initializer_list>
#include "ci_fpconv.h"
using namespace ci;
static bool same32(float a, float b) { return fp_bits(a) == fp_bits(b); }
static bool same64(double a, double b) { return fp_bits(a) == fp_bits(b); }
int main() {
  std::mt19937_64 g(20261203);
  long bad_d2f = 0, bad_f2d = 0, n = 0;
  auto check_d = [&](double x) {
    const float ref = (float)x;
    if (std::isnan(x)) { if (!std::isnan(f64_to_f32(x))) bad_d2f++; return; }
    if (!same32(f64_to_f32(x), ref)) { if (bad_d2f < 5) std::printf("d2f %.17g\n", x); bad_d2f++; }
    n++;
  };
  auto check_f = [&](float f) {
    const double ref = (double)f;
    if (std::isnan(f)) { if (!std::isnan(f32_to_f64(f))) bad_f2d++; return; }
    if (!same64(f32_to_f64(f), ref)) { if (bad_f2d < 5) std::printf("f2d %.9g\n", f); bad_f2d++; }
  };
  // random bit patterns over the whole double range and a log-uniform sweep
  for (int i = 0; i < 2000000; i++) {
    check_d(fp_f64(g()));
    const double m = std::ldexp((double)(g() >> 11) / 9007199254740992.0 + 0.5, (int)(g() % 300) - 150);
    check_d((g() & 1) ? m : -m);
    check_f(fp_f32((uint32_t)g()));
  }
  // exact ties, ties +- 1 ulp of the dropped bits, mantissa carry into the exponent
  for (int i = 0; i < 200000; i++) {
    const uint64_t e = 897 + g() % 254, mant = g() & 0xfffffffffffffull;
    const uint64_t base = (e << 52) | (mant & ~0x1fffffffull);
    for (uint64_t r : {0x10000000ull, 0x0fffffffull, 0x10000001ull, 0x1fffffffull, 0ull})
      check_d(fp_f64(base | r));
    check_d(fp_f64((e << 52) | 0xfffffffffffffull));
  }
  for (double x : std::initializer_list<double>{0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38,
                   3.4028235677973362e38, 1e39, -1e300, INFINITY, -INFINITY, NAN,
                   1.1754943508222875e-38, 1.1754942106924411e-38, 1e-45, 5e-324})
    check_d(x);
  for (float f : std::initializer_list<float>{0.0f, -0.0f, 1.0f, 1.17549435e-38f, 1e-45f, 3.40282347e38f, INFINITY, -INFINITY, NAN})
    check_f(f);
  std::printf("%ld %ld %ld\n", n, bad_d2f, bad_f2d);
  return 0;
}
'''


def test_integer_conversions_match_ieee(tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text(SRC)
    exe = tmp_path / "t"
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                        "-I", os.path.join(ROOT, "cppimpact_gb300", "csrc"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120).stdout.split()
    n, bad_d2f, bad_f2d = (int(x) for x in out[-3:])
    assert n > 4_000_000
    assert bad_d2f == 0 and bad_f2d == 0, " ".join(out)
