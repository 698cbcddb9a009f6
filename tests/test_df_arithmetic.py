"""Double-float arithmetic of the fast form's FP64-accurate kernels (micropp_gb300/csrc/df.cuh), on the CPU.

The header compiles as plain C++ with the same sequence of correctly rounded FP32 operations that the GPU
kernels use (built here without floating-point contraction, which the device code forbids with its
explicit-rounding intrinsics).  A small harness checks every operator against long double on seeded random
operands over twelve decades, and the two composite steps of the kernels: the refinement residual's row
f - sum k x (df_sub_prod, FP32 k, double-float x and f) on rows that cancel to 1e-7 of their terms, and the
accumulation X += D (df_add).  Bars: 2^-44 relative for the operators, 1e-12 of sum |k x| for a row.
"""
import pathlib
import shutil
import subprocess

import pytest

CSRC = pathlib.Path(__file__).resolve().parents[1] / "micropp_gb300" / "csrc"

HARNESS = r"""
#include <cmath>
#include <cstdio>
#include <random>
#include "df.cuh"
using namespace mgb;
typedef long double LD;
static LD ld(dfl a) { return (LD)a.h + (LD)a.l; }
static LD ldabs(LD x) { return x < 0 ? -x : x; }
int main() {
  std::mt19937_64 g(20241204);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  std::normal_distribution<double> N(0.0, 1.0);
  double e_add = 0, e_mul = 0, e_mulf = 0, e_div = 0, e_sqrt = 0, e_split = 0;
  for (int it = 0; it < 200000; ++it) {
    const double x = U(g) * std::pow(10.0, 6.0 * U(g)), y = U(g) * std::pow(10.0, 6.0 * U(g));
    const dfl a = df_of(x), b = df_of(y);
    const LD A = ld(a), B = ld(b);
    e_split = std::fmax(e_split, (double)(ldabs(A - (LD)x) / ldabs((LD)x)));
    e_add = std::fmax(e_add, (double)(ldabs(ld(a + b) - (A + B)) / (ldabs(A) + ldabs(B))));
    e_mul = std::fmax(e_mul, (double)(ldabs(ld(a * b) - A * B) / ldabs(A * B)));
    const float f = (float)y;
    e_mulf = std::fmax(e_mulf, (double)(ldabs(ld(a * f) - A * (LD)f) / ldabs(A * (LD)f)));
    e_div = std::fmax(e_div, (double)(ldabs(ld(a / b) - A / B) / ldabs(A / B)));
    const dfl p = df_of(std::fabs(x));
    const LD P = ld(p), R = std::sqrt((long double)P);
    e_sqrt = std::fmax(e_sqrt, (double)(ldabs(ld(df_sqrt(p)) - R) / R));
  }
  // refinement-residual rows: f - sum_j k_j x_j with 81 terms cancelling to ~1e-7 of their size
  double e_row = 0;
  for (int row = 0; row < 20000; ++row) {
    float k[81];
    double x[81];
    LD exact = 0;
    for (int j = 0; j < 81; ++j) {
      k[j] = (float)(N(g) * 2e5);
      x[j] = N(g) * 0.3;
      exact += (LD)k[j] * (LD)x[j];
    }
    float h, l;
    df_split((double)exact * (1.0 + 1e-7 * N(g)), h, l);
    LD ref = (LD)h + (LD)l, scale = 0;
    for (int j = 0; j < 81; ++j) {
      float xh, xl;
      df_split(x[j], xh, xl);
      df_sub_prod(h, l, k[j], xh, xl);
      ref -= (LD)k[j] * ((LD)xh + (LD)xl);
      scale += ldabs((LD)k[j] * (LD)x[j]);
    }
    e_row = std::fmax(e_row, (double)(ldabs((LD)h + (LD)l - ref) / scale));
  }
  // X += D over 50 FP32 corrections of decreasing size (the sweeps of a refined solve)
  double e_acc = 0;
  for (int it = 0; it < 20000; ++it) {
    float h = 0.f, l = 0.f;
    LD ref = 0, scale = 0;
    for (int s = 0; s < 50; ++s) {
      const float d = (float)(N(g) * std::pow(10.0, -0.2 * s));
      df_add(h, l, d);
      ref += (LD)d;
      scale += ldabs((LD)d);
    }
    e_acc = std::fmax(e_acc, (double)(ldabs((LD)h + (LD)l - ref) / scale));
  }
  std::printf("split %.3e add %.3e mul %.3e mulf %.3e div %.3e sqrt %.3e row %.3e acc %.3e\n", e_split, e_add, e_mul,
              e_mulf, e_div, e_sqrt, e_row, e_acc);
  return 0;
}
"""


def test_double_float_operators_and_kernel_steps(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    src = tmp_path / "df_check.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "df_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(CSRC), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    err = {out[i]: float(out[i + 1]) for i in range(0, len(out), 2)}
    print(err)
    bar = 2.0 ** -44
    for op in ("split", "add", "mul", "mulf", "div", "sqrt", "acc"):
        assert err[op] <= bar, (op, err[op])
    assert err["row"] <= 1e-12, err["row"]
