"""The integer-pipe float -> double conversion of the float-pair header (km_ff.cuh: f2d_bits,
f2d_exact) against the host's conversion, bit for bit: every subnormal, zeros, infinities, the
exponent boundaries and a stride through all 2^32 patterns.  The header is compiled for the host
with nvcc (no GPU needed); NaNs only have to stay NaNs."""
import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "kernelmatrices.jl_gb300" / "csrc"

PROG = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include "km_ff.cuh"

static unsigned long long host_bits(unsigned u) {
  float f;
  std::memcpy(&f, &u, 4);
  const double d = (double)f;
  unsigned long long b;
  std::memcpy(&b, &d, 8);
  return b;
}

static long long bad = 0, checked = 0;
static void check(unsigned u) {
  ++checked;
  float f;
  std::memcpy(&f, &u, 4);
  const double got = km::f2d_exact(f);
  if (std::isnan(f)) {
    if (!std::isnan(got)) ++bad;
    return;
  }
  unsigned long long g;
  std::memcpy(&g, &got, 8);
  if (g != host_bits(u)) {
    if (bad < 5) std::printf("mismatch %08x\n", u);
    ++bad;
  }
}

int main() {
  for (unsigned s = 0; s < 2; ++s) {
    const unsigned sign = s << 31;
    for (unsigned m = 0; m < (1u << 23); ++m) check(sign | m);                 // zero and subnormals
    for (unsigned e = 1; e < 256; ++e)                                         // every exponent
      for (unsigned m : {0u, 1u, 2u, 7u, 8u, 0x3fffffu, 0x400000u, 0x7ffff8u, 0x7fffffu}) check(sign | (e << 23) | m);
  }
  for (unsigned long long u = 0; u < (1ull << 32); u += 4099) check((unsigned)u);  // a stride through all
  std::printf("checked %lld bad %lld\n", checked, bad);
  return bad != 0;
}
"""


def test_f2d_exact_matches_host_conversion(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if Path("/usr/local/cuda/bin/nvcc").exists() else None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    src = tmp_path / "f2d.cu"
    src.write_text(PROG)
    exe = tmp_path / "f2d"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", str(CSRC), "-o", str(exe), str(src)], check=True,
                   capture_output=True, timeout=300)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " bad 0" in r.stdout
