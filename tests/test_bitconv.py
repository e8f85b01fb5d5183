"""Host check of the integer-pipe FP32 <-> FP64 conversions (ampe_gb300/
csrc/bitconv.h) against the C casts: f2d exact for all normal floats (and
signed zero for subnormals), d2f round-to-nearest-even for the normal float
range, ties included, overflow to inf, NaN kept, underflow to signed zero."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include "bitconv.h"
static uint64_t dbits(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static uint32_t fbits(float x) { uint32_t u; memcpy(&u, &x, 4); return u; }
int main() {
  std::mt19937_64 rng(3);
  unsigned long long bad = 0, n = 0;
  // f2d over random float bit patterns
  for (int r = 0; r < 2000000; r++) {
    uint32_t u = (uint32_t)rng();
    float x; memcpy(&x, &u, 4);
    double got = ampe::f2d(x);
    uint32_t e = (u >> 23) & 0xff;
    double want = e == 0 ? std::copysign(0.0, x) : (double)x;
    if (std::isnan(want) ? !std::isnan(got) : dbits(got) != dbits(want)) bad++;
    n++;
  }
  // d2f over doubles spread across the float range, plus exact ties
  std::uniform_real_distribution<double> ex(-130.0, 130.0);
  for (int r = 0; r < 2000000; r++) {
    double x = std::ldexp(1.0 + (double)(rng() >> 11) / 9007199254740992.0, (int)ex(rng));
    if (rng() & 1) x = -x;
    if (r % 7 == 0) {  // exact tie between two floats
      float f = (float)x;
      double nf = (double)std::nextafter(f, 2.0f * f);
      x = 0.5 * ((double)f + nf);
    }
    float got = ampe::d2f(x);
    float want = std::fabs(x) < 1.1754943508222875e-38 ? (float)std::copysign(0.0, x) : (float)x;
    if (fbits(got) != fbits(want)) bad++;
    n++;
  }
  const double specials[] = {0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 3.4028235677973366e38,
                             1e300, -1e300, INFINITY, -INFINITY, 1e-300, -1e-300};
  for (double x : specials) {
    float got = ampe::d2f(x);
    float want = std::fabs(x) < 1.1754943508222875e-38 ? (float)std::copysign(0.0, x) : (float)x;
    if (fbits(got) != fbits(want)) bad++;
    n++;
  }
  if (!std::isnan(ampe::d2f(NAN))) bad++;
  std::printf("%llu %llu\n", bad, n);
  return bad != 0;
}
"""


def test_bit_conversions(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "bc.cc"
    src.write_text(PROG)
    exe = tmp_path / "bc"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "ampe_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    bad, n = map(int, out.stdout.split())
    assert out.returncode == 0 and bad == 0 and n > 3_000_000, out.stdout
