"""The FFT stage loops divide by multiply-high constants that the host sets
with the plans (make_fastdiv in hosnwt_internal.h); the kernels form
x / d = (mulhi(x, m) + x) >> s.  A host program built from the same header
checks the constants against plain division for every divisor up to 65536
(plan divisors are at most the longest transform, 12400) and sampled
dividends up to 2^31 - 1."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cstdio>
#include <cstdint>
#include "hosnwt_internal.h"
static unsigned umulhi(unsigned a, unsigned b) { return (unsigned)(((unsigned long long)a * b) >> 32); }
int main() {
  unsigned long long bad = 0, n = 0, seed = 12345;
  for (unsigned d = 1; d <= 65536; ++d) {
    const hos::FastDivC f = hos::make_fastdiv(d);
    unsigned xs[8] = {0u, 1u, d - 1u, d, d + 1u, 2u * d - 1u, 0x7fffffffu, 0x7ffffffeu};
    for (int k = 0; k < 40; ++k) {
      seed = seed * 6364136223846793005ULL + 1442695040888963407ULL;
      const unsigned x = (unsigned)(seed >> 33);
      const unsigned q = (unsigned)(((unsigned long long)umulhi(x, f.m) + x) >> f.s);
      bad += (q != x / d);
      ++n;
    }
    for (unsigned x : xs) {
      const unsigned q = (unsigned)(((unsigned long long)umulhi(x, f.m) + x) >> f.s);
      bad += (q != x / d);
      ++n;
    }
  }
  std::printf("%llu %llu\n", bad, n);
  return bad != 0;
}
"""


def test_fastdiv_constants(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    cuda_inc = "/usr/local/cuda/include"
    if cxx is None or not os.path.isdir(cuda_inc):
        pytest.skip("needs a C++ compiler and the CUDA headers")
    src = tmp_path / "fastdiv.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "fastdiv"
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-I", cuda_inc, "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "hos-nwt_gb300", "csrc"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    bad, n = map(int, r.stdout.split())
    assert n > 3_000_000
    assert bad == 0
