"""The double-word (FP32 pair) arithmetic of the FP64-accurate hopping operator, checked on the
CPU: the integer split of FP64 values, and addition, multiplication and fused multiply-add
against exact results (80-bit long double holds every exact sum / product of the pairs here to
far below the bounds), at the error bounds the header states."""
import os
import shutil
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

PROG = r"""
#include "dsfloat.cuh"
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <random>
using gbdw::dsf;
static long double ex(dsf a) { return (long double)a.h + (long double)a.l; }
int main() {
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex_d(-48, 48);
  double split_err = 0, add_err = 0, mul_err = 0, fma_err = 0;
  int not_normal = 0;
  // magnitudes in [2^-48, 2^50): products stay above 2^-100, where their trailing parts are
  // still normal FP32 numbers
  auto rnd = [&]() { const double v = u(rng); return std::ldexp(std::copysign(1.0 + std::fabs(v), v), ex_d(rng)); };
  for (int i = 0; i < 200000; ++i) {
    const double d = rnd();
    const dsf a = dsf(d);
    if (a.h != a.h + a.l) ++not_normal;  // h = RN(h + l)
    if (d != 0) split_err = std::fmax(split_err, (double)(std::fabs(ex(a) - (long double)d) / std::fabs(d)));
    const dsf b = dsf(rnd()), c = dsf(rnd());
    const long double sa = ex(a), sb = ex(b), sc = ex(c);
    const dsf s = a + b;
    add_err = std::fmax(add_err, (double)(std::fabs(ex(s) - (sa + sb)) / (std::fabs(sa) + std::fabs(sb))));
    const dsf m = a * b;
    if (sa * sb != 0) mul_err = std::fmax(mul_err, (double)(std::fabs(ex(m) - sa * sb) / std::fabs(sa * sb)));
    const dsf f = gbdw::fma(a, b, c);
    fma_err = std::fmax(fma_err, (double)(std::fabs(ex(f) - (sa * sb + sc)) / (std::fabs(sa * sb) + std::fabs(sc))));
  }
  // zero, signs, flushing below 2^-126 and saturation above FP32 range
  const dsf z = dsf(0.0), nz = dsf(-0.0), tiny = dsf(1e-40), big = dsf(1e300), neg = dsf(-3.0);
  // below 2^-74 the trailing part is dropped: 24 bits remain
  const double small = 0x1.23456789abcdep-80;
  const dsf sm = dsf(small);
  const int specials = (z.h == 0 && z.l == 0) + (nz.h == 0 && std::signbit(nz.h)) + (tiny.h == 0) +
                       (std::isinf(big.h) != 0) + (neg.h == -3.0f && neg.l == 0) +
                       (std::fabs((double)sm.h - small) <= 0x1p-23 * small);
  std::printf("%.3e %.3e %.3e %.3e %d %d\n", split_err, add_err, mul_err, fma_err, not_normal, specials);
  return 0;
}
"""


def test_double_word_arithmetic_bounds(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    src = tmp_path / "ds_test.cc"
    src.write_text(PROG)
    exe = tmp_path / "ds_test"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "gridbench_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    split_err, add_err, mul_err, fma_err = (float(v) for v in out[:4])
    not_normal, specials = int(out[4]), int(out[5])
    assert split_err <= 2.0 ** -47, split_err
    assert add_err <= 2.0 ** -46, add_err
    assert mul_err <= 2.0 ** -44, mul_err
    assert fma_err <= 2.0 ** -45, fma_err
    assert not_normal == 0
    assert specials == 6
