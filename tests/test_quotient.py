"""The interface Riemann solver's shared-reciprocal quotients (Markstein's
method, m2cg_device.cuh: quot_of / qdiv) must equal IEEE division bit for bit,
so that the device solver follows the oracle's operations exactly.  The check
runs on the device over 2^32 operand pairs of every class the self-test draws
(random bit patterns, wide and physical exponent ranges, all-ones significands,
zeros, subnormals, infinities, NaNs, exponent-limit and exact quotients)."""
import ctypes as C

import pytest

from m2c_gb300 import abi

INVALID_ARG = 1   # M2CG_ERR_INVALID_ARG


def test_selftest_entry_rejects_bad_arguments():
    lib = abi.load()
    bad = C.c_int64(-1)
    assert lib.m2cg_selftest_quotient(0, 1, C.byref(bad), None) == INVALID_ARG
    assert lib.m2cg_selftest_quotient(1 << 37, 1, C.byref(bad), None) == INVALID_ARG
    assert lib.m2cg_selftest_quotient(16, 1, None, None) == INVALID_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [1, 20261204])
def test_shared_reciprocal_quotients_equal_ieee_division(seed):
    lib = abi.load()
    bad, fast = C.c_int64(-1), C.c_int64(-1)
    n = 1 << 32
    abi.check(lib, lib.m2cg_selftest_quotient(n, seed, C.byref(bad), C.byref(fast)), "m2cg_selftest_quotient")
    assert bad.value == 0
    # most operand classes are inside the shared-reciprocal path's range
    assert 0.4 * n < fast.value < n


MARKSTEIN_C = r"""
/* The device's shared-reciprocal quotient (m2cg_device.cuh: quot_of / qdiv)
   restated on the CPU with C99 fma(): a reciprocal seed within one ulp
   (here a binary32 reciprocal refined by the same third-order step), the
   Markstein correction to RN(1/b), then two remainder steps per quotient;
   operands outside the range fall back to a / b.  Counts results that
   differ from IEEE a / b, and from 1 / b for the reciprocal itself. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
static uint64_t s = 0x9e3779b97f4a7c15ull;
static uint64_t nx(void) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
static double bits2d(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static uint64_t d2bits(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }
static int ef(double x) { return (int)((d2bits(x) >> 52) & 0x7ff); }
static double with_exp(uint64_t r, int e) { return bits2d((r & 0x800fffffffffffffull) | ((uint64_t)(e & 0x7ff) << 52)); }
int main(int argc, char** argv) {
  long n = 2000000, bad = 0, fast = 0;
  for (long i = 0; i < n; i++) {
    uint64_t r1 = nx(), r2 = nx(), r3 = nx();
    double a, b;
    switch (i & 3) {
      case 0: a = with_exp(r1, 1023 - 60 + (int)(r3 % 121)); b = with_exp(r2, 1023 - 60 + (int)((r3 >> 16) % 121)); break;
      case 1: b = with_exp(r2, 1023 - 20 + (int)(r3 % 41)); a = b * (double)(1 + (int)((r3 >> 16) % 4096)); break;
      case 2: b = bits2d((r2 & 0x8000000000000000ull) | ((uint64_t)(1000 + (int)(r3 % 40)) << 52) | 0xfffffffffffffull);
              a = with_exp(r1, 1000 + (int)((r3 >> 20) % 40)); break;
      default: a = with_exp(r1, (r3 & 1) ? 128 + (int)((r3 >> 1) % 5) - 2 : 1920 + (int)((r3 >> 1) % 5) - 2);
               b = with_exp(r2, 1023 + (int)((r3 >> 8) % 200) - 100); break;
    }
    const int eb = ef(b);
    const int ok_b = (unsigned)(eb - 128) <= 1792u && (d2bits(b) & 0xfffffffffffffull) != 0xfffffffffffffull;
    double y = 0.0;
    if (ok_b) {
      double r = (double)(1.0f / (float)b);
      double e = fma(-b, r, 1.0);
      double y1 = fma(r, fma(e, e, e), r);
      y = fma(fma(-b, y1, 1.0), y1, y1);
      if (d2bits(y) != d2bits(1.0 / b)) bad++;
    }
    const int ea = ef(a), eq = ea - eb + 1023;
    double q;
    if (!ok_b || (unsigned)(ea - 128) > 1792u || (unsigned)(eq - 128) > 1792u) q = a / b;
    else {
      fast++;
      q = a * y;
      q = fma(fma(-b, q, a), y, q);
      q = fma(fma(-b, q, a), y, q);
    }
    if (d2bits(q) != d2bits(a / b)) bad++;
  }
  printf("%ld %ld\n", bad, fast);
  return 0;
}
"""


def test_markstein_quotient_sequence_on_cpu(tmp_path):
    """The same operation sequence with a binary32 seed, on the host's correctly
    rounded fma(): every quotient in range equals IEEE a / b (the method, apart
    from the device's reciprocal seed, which the GPU test covers)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "markstein.c"
    src.write_text(MARKSTEIN_C)
    exe = tmp_path / "markstein"
    r = subprocess.run([cc, "-O2", "-std=c99", "-ffp-contract=off", str(src), "-o", str(exe), "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300).stdout.split()
    bad, fast = int(out[0]), int(out[1])
    assert bad == 0
    assert fast > 1000000
