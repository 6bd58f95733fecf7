"""The sampler's integer-only float uniforms (u53f in smc_device.cuh) equal
the FP64 route (float)u53 bit for bit: random words and the rounding edge
cases, on the host (no GPU)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "supermc_gb300", "csrc")

PROGRAM = r'''
#include <cstdio>
#include <cstring>
#include "smc_device.cuh"
static uint64_t sm64(uint64_t &s) {   // splitmix64
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static int check(uint64_t v) {
  const uint32_t lo = (uint32_t)v, hi = (uint32_t)(v >> 32);
  const float a = (float)smc::u53(lo, hi), b = smc::u53f(lo, hi);
  uint32_t ia, ib;
  std::memcpy(&ia, &a, 4);
  std::memcpy(&ib, &b, 4);
  if (ia != ib) { std::printf("mismatch %016llx %a %a\n", (unsigned long long)v, a, b); return 1; }
  return 0;
}
int main() {
  int bad = 0;
  uint64_t s = 12345;
  for (int i = 0; i < 20000000; i++) bad += check(sm64(s));
  // ties and near-ties at the double and float rounding positions, tiny and
  // largest values
  for (int sh = 0; sh < 64; sh++)
    for (uint64_t d = 0; d < 4; d++) {
      bad += check(1ull << sh);
      bad += check((1ull << sh) - d);
      bad += check((1ull << sh) + d);
      bad += check(~0ull - (d << sh));
      bad += check(((sm64(s) >> sh) << sh) | (d << 11));
    }
  for (uint64_t m = 0; m < 100000; m++) bad += check(m << 11);
  std::printf("%d\n", bad);
  return bad != 0;
}
'''


def test_float_uniforms_round_like_the_fp64_route(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "u.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "u"
    subprocess.check_call([nvcc, "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off", "-I", CSRC, str(src),
                           "-o", str(exe)])
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
