"""The residual-change terms of the Gram-blocked sweep are rounded to the
fixed-point grid E = value * 2^50 by two float-to-int64 conversions
(round to nearest even) of the scaled high and low parts of a double-float
pair (`df_to_fix_near`, csrc/brr_block.cu).  This restates that rounding in
numpy float32 arithmetic and checks its bound against the exact rational
value: the nearest integer whenever the scaled high part reaches 2^23 (it is
then an integer), within one unit otherwise.  The residual update it feeds
follows src/densebayesrkernel.cpp:10-20 (epsilon += (beta_old - beta) * x).
"""
from fractions import Fraction

import numpy as np

SCALE = np.float32(2.0 ** 50)


def near(h: np.float32, l: np.float32) -> int:
    sh, sl = np.float32(h * SCALE), np.float32(l * SCALE)
    return int(np.rint(np.float64(sh))) + int(np.rint(np.float64(sl)))


def exact_nearest(h: np.float32, l: np.float32) -> Fraction:
    return (Fraction(float(h)) + Fraction(float(l))) * 2 ** 50


def split_df(x: float):
    h = np.float32(x)
    l = np.float32(x - float(h))
    return h, l


def test_near_rounding_is_exact_for_large_terms_and_within_one_unit_below():
    rng = np.random.default_rng(7)
    # magnitudes of dBeta * x from 1e-18 to 10 (the residual's range is far below 2^11)
    mags = 10.0 ** rng.uniform(-18, 1, 20000)
    vals = mags * rng.choice([-1.0, 1.0], mags.size)
    for x in vals:
        h, l = split_df(float(x))
        e = near(h, l)
        v = exact_nearest(h, l)
        assert abs(e - v) <= 1, (x, e, float(v))
        if abs(float(h) * 2 ** 50) >= 2 ** 23:
            # the scaled high part is an integer, so the sum rounds once
            assert abs(e - v) <= Fraction(1, 2), (x, e, float(v))


def test_scaled_high_part_is_an_integer_from_two_to_the_23():
    rng = np.random.default_rng(3)
    for x in 2.0 ** rng.uniform(-27, 10, 5000):
        h = np.float32(x)
        sh = float(np.float32(h * SCALE))
        assert sh == float(h) * 2 ** 50            # scaling by a power of two is exact
        if abs(sh) >= 2 ** 23:
            assert sh == int(sh)
