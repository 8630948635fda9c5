"""The division of the convective adjustment's merges (no GPU).

k_co_decide and k_co_mix divide a merge's sums by its summed thickness b with the reciprocal
y = RN(1/b) computed once per merge: q0 = a*y, then two residual corrections
q <- fma(fma(-b, q, a), y, q).  By Markstein's theorem (the first correction makes q
faithful, the second correctly rounded) the result is RN(a/b), the IEEE quotient co takes.
The same operation sequence in C (round-to-nearest doubles, libm's correctly rounded fma)
is checked against a/b on random operands and on quotients placed at and next to rounding
midpoints."""
import os
import shutil
import subprocess
import tempfile

import pytest

SRC = r"""
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
static uint64_t st = 88172645463325252ull;
static uint64_t rnd(void) { st ^= st << 13; st ^= st >> 7; st ^= st << 17; return st; }
static double bits(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static double co_div(double a, double b, double y)
{
    double q0 = a * y;
    double q1 = fma(fma(-b, q0, a), y, q0);
    return fma(fma(-b, q1, a), y, q1);
}
int main(int argc, char **argv)
{
    long n = atol(argv[1]), bad = 0;
    for (long i = 0; i < n; ++i) {
        double a = bits(((uint64_t)(1023 + (int)(rnd() % 81) - 40) << 52) | (rnd() >> 12));
        double b = bits(((uint64_t)(1023 + (int)(rnd() % 17) - 12) << 52) | (rnd() >> 12));
        if (rnd() & 1) a = -a;
        switch (i % 4) {
        case 1: {   /* exact products: quotients that are doubles, and their neighbours */
            double q = bits(((uint64_t)1023 << 52) | (rnd() >> 12));
            a = b * q;
            break;
        }
        case 2: {   /* a = b * (q + ulp/2) rounded: quotients next to midpoints */
            double q = bits(((uint64_t)1023 << 52) | (rnd() >> 12));
            a = fma(b, q, b * ldexp(1.0, -53));
            break;
        }
        case 3:     /* divisors with long runs of ones */
            b = bits(((uint64_t)1020 << 52) | (rnd() >> 12) | 0xffffffff0000ull);
            break;
        }
        double y = 1.0 / b;
        if (co_div(a, b, y) != a / b) ++bad;
    }
    printf("%ld\n", bad);
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_markstein_division_is_the_ieee_quotient():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "div.c")
        exe = os.path.join(d, "div")
        with open(src, "w") as f:
            f.write(SRC.replace("#include <string.h>", "#include <string.h>\n#include <stdlib.h>"))
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-o", exe, src, "-lm"], check=True)
        out = subprocess.run([exe, "20000000"], check=True, capture_output=True, text=True).stdout
        assert int(out.strip()) == 0
