"""The hole fill divides by a neighbour count w in {1, 2, 3, 4} as a reciprocal product with one residual
correction, q = v * (1/w); q + (1/w) * fma(-q, w, v) (Markstein's method). With the reciprocal rounded to
nearest, this is the correctly rounded quotient, i.e. the division's result bit for bit. Checked here in C
(float arithmetic, fmaf, no contraction) over every mantissa of one binade for each w and over random values of
all magnitudes the images reach and beyond."""
import shutil
import subprocess

import pytest

SRC = r"""
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
static int same(float a, float b) { return memcmp(&a, &b, sizeof a) == 0; }
int main(void) {
    unsigned long long bad = 0, n = 0;
    srand(7);
    for (int k = 1; k <= 4; ++k) {
        volatile float w = (float)k;
        const float rw = 1.0f / w;
        for (unsigned m = 0; m < (1u << 23); ++m) {       /* every mantissa of [1, 2) */
            unsigned u = 0x3f800000u | m;
            float v;
            memcpy(&v, &u, 4);
            const float q = v * rw, qc = fmaf(fmaf(-q, w, v), rw, q);
            bad += !same(qc, v / w);
            ++n;
        }
        for (long i = 0; i < 2000000; ++i) {               /* random values in [-1e6, 1e6] */
            const float v = ((float)rand() / RAND_MAX - 0.5f) * 2e6f * ((float)rand() / RAND_MAX);
            const float q = v * rw, qc = fmaf(fmaf(-q, w, v), rw, q);
            bad += !same(qc, v / w);
            ++n;
        }
    }
    printf("%llu %llu\n", bad, n);
    return 0;
}
"""


def test_corrected_reciprocal_equals_division(tmp_path):
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "markstein.c"
    exe = tmp_path / "markstein"
    src.write_text(SRC)
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-o", str(exe), str(src), "-lm"], check=True)
    bad, n = map(int, subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split())
    assert n > 4 * (1 << 23)
    assert bad == 0
