"""Host check of the kernels' 31-bit index division (ampe_gb300/csrc/
fastdiv.h): quotient by every divisor 1..2100 (every grid extent and
extent+1 up to 2048^2 levels) and by large ones, for the numerators at both
ends of [0, 2^31) and seeded random ones, against plain integer division."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = r"""
#include <cstdio>
#include <random>
#include "fastdiv.h"
int main() {
  std::mt19937 rng(7);
  unsigned long long bad = 0, n = 0;
  auto check = [&](unsigned d) {
    ampe::FastDiv f(d);
    for (unsigned r = 0; r < 3000; r++) {
      unsigned x;
      if (r < 1000) x = r;
      else if (r < 2000) x = 0x7fffffffu - (r - 1000);
      else x = rng() & 0x7fffffffu;
      if (f.div(x) != x / d) bad++;
      n++;
    }
  };
  for (unsigned d = 1; d <= 2100; d++) check(d);
  const unsigned big[] = {65535u, 65536u, 65537u, 1u << 20, (1u << 20) + 1, 4194305u,
                          (1u << 30) - 1, 1u << 30, (1u << 30) + 1, 0x7fffffffu};
  for (unsigned d : big) check(d);
  std::printf("%llu %llu\n", bad, n);
  return bad != 0;
}
"""


def test_fastdiv_matches_division(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "fd.cc"
    src.write_text(PROG)
    exe = tmp_path / "fd"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "ampe_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    bad, n = map(int, out.stdout.split())
    assert out.returncode == 0 and bad == 0 and n > 6_000_000
