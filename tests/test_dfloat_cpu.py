"""The double-float kernel's adjoint flush, restated on the host.

`gput` of lammps-mlip-package_gb300/csrc/kernel_impl.cuh (double-float
path) splits a scaled flush y = yh + yl (two FP32 values, |yh| < 2^70,
|yl| <= ulp(yh) / 2) into four int32 words, multiples of 2^48, 2^32, 2^16 and
1, by magic-number roundings whose remainders must be exact, so that the
words' sum equals y to within half a unit of the last word.  This file
replays those FP32 steps in numpy (an FP32 FMA is the FP64 product rounded
once, exact for these operands) over random flushes of every magnitude and
checks each remainder and the reconstruction exactly, and the per-flush word
bounds that the host's overflow bound on flushes per entry relies on.
"""
from fractions import Fraction

import numpy as np

F32 = np.float32
MAGIC = F32(12582912.0)           # 1.5 * 2^23


def fma32(a, b, c):
    return F32(np.float64(a) * np.float64(b) + np.float64(c))


def mi(t):
    return int(t) - 12582912


def split(yh, yl):
    th3 = fma32(yh, F32(2.0 ** -48), MAGIC)
    r2 = fma32(-(th3 - MAGIC), F32(2.0 ** 48), yh)
    th2 = fma32(r2, F32(2.0 ** -32), MAGIC)
    r1 = fma32(-(th2 - MAGIC), F32(2.0 ** 32), r2)
    th1 = fma32(r1, F32(2.0 ** -16), MAGIC)
    r0 = fma32(-(th1 - MAGIC), F32(65536.0), r1)
    sh2 = fma32(yl, F32(2.0 ** -32), MAGIC)
    q1 = fma32(-(sh2 - MAGIC), F32(2.0 ** 32), yl)
    sh1 = fma32(q1, F32(2.0 ** -16), MAGIC)
    q0 = fma32(-(sh1 - MAGIC), F32(65536.0), q1)
    t0 = (r0 + q0) + MAGIC
    rem = [(r2, yh, th3, 48), (r1, r2, th2, 32), (r0, r1, th1, 16), (q1, yl, sh2, 32),
           (q0, q1, sh1, 16)]
    words = (mi(th3), mi(th2) + mi(sh2), mi(th1) + mi(sh1), mi(t0))
    return words, rem


def test_four_word_split_is_exact():
    rng = np.random.default_rng(3)
    worst = Fraction(0)
    for _ in range(20000):
        yh = F32(rng.uniform(-1, 1) * 2.0 ** int(rng.integers(-12, 70)))
        yl = F32(rng.uniform(-0.5, 0.5) * float(np.spacing(yh)))
        (w3, w2, w1, w0), rem = split(yh, yl)
        for r, src, t, sc in rem:
            assert Fraction(float(r)) == Fraction(float(src)) - mi(t) * 2 ** sc
        assert abs(w2) <= 2 ** 15 + 2 ** 14 + 1
        assert abs(w1) <= 2 ** 16 + 2 and abs(w0) <= 2 ** 16 + 1
        exact = Fraction(float(yh)) + Fraction(float(yl))
        worst = max(worst, abs(Fraction(w3 * 2 ** 48 + w2 * 2 ** 32 + w1 * 2 ** 16 + w0) - exact))
    assert worst <= Fraction(1, 2) + Fraction(1, 256)
