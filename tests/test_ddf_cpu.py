"""The bit-level conversions between FP64 fields and double-float values (csrc/ddf.cuh), checked on the
host: the split d = hi + lo keeps 48 significand bits (relative error <= 2^-48) and is normalised
(|lo| <= ulp(hi)); the widening float -> double is exact; zero and tiny values take the FP64
conversion (values from 2^128 up are beyond the format's FP32 exponent range).  The header's host
path is the device path's arithmetic with memcpy bit casts."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "soerenpragya3dglasma_gb300", "csrc")

PROGRAM = r"""
#include <cmath>
#include <cstdio>
#include <random>
#include "ddf.cuh"
using namespace glasma;
int main() {
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> u(-1.0, 1.0), ex(-90.0, 127.0);  // double-float's range ends at 2^128
  double worst = 0.0;
  long not_normalised = 0, widen_mismatch = 0, merge_mismatch = 0;
  for (long i = 0; i < 400000; i++) {
    double d = u(rng) * std::pow(2.0, ex(rng));
    if (i % 97 == 0) d = 0.0;
    ddf a = ddf_from_double(d);
    const double back = (double)a.hi + (double)a.lo;
    const double rel = d != 0.0 ? std::fabs(back - d) / std::fabs(d) : std::fabs(back);
    if (rel > worst) worst = rel;
    if (std::fabs(a.lo) > std::ldexp(std::fabs(a.hi), -23)) not_normalised++;
    const float f = (float)(u(rng) * std::pow(2.0, ex(rng) / 2.0));
    if (ddf_widen(f) != (double)f) widen_mismatch++;
    if (to_double(a) != back) merge_mismatch++;
  }
  std::printf("%.6e %ld %ld %ld\n", worst, not_normalised, widen_mismatch, merge_mismatch);
  return 0;
}
"""


def test_double_float_conversions_on_the_host():
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "ddf_check.cu")
        exe = os.path.join(tmp, "ddf_check")
        with open(src, "w") as fh:
            fh.write(PROGRAM)
        subprocess.run([nvcc, "-std=c++17", "-O2", "-I", CSRC, "-o", exe, src], check=True, capture_output=True,
                       timeout=300)
        out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=120).stdout.split()
    worst, not_normalised, widen_mismatch, merge_mismatch = float(out[0]), int(out[1]), int(out[2]), int(out[3])
    assert worst <= 2.0 ** -48 * 1.0000001
    assert not_normalised == 0
    assert widen_mismatch == 0
    assert merge_mismatch == 0
