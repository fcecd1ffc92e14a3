"""The exponent of tupan's power-of-two step, int(log2(min_ts) - 1)
(integrator/__init__.py:59-78), as the device drivers form it
(quantised_power in tupan_gb300/csrc/tg_common.cuh): the exponent from
frexp, only the mantissa's logarithm from log2.  The device log2 may be one
ulp off; these tests emulate that error on the host and check that the
frexp form still reproduces numpy's value, where log2(min_ts) alone does not
at exact powers of two."""

import math

import numpy as np


def numpy_power(x):
    return int(np.log2(x) - 1)


def frexp_power(x, log2):
    m, e = math.frexp(x)            # x = m 2^e, m in [0.5, 1)
    if m < 0.70710678118654752:
        l = float(e - 1) + log2(2.0 * m)
    else:
        l = float(e) + log2(m)
    return int(l - 1.0)


def naive_power(x, log2):
    return int(log2(x) - 1.0)


def exact(v):
    return math.log2(v)


def ulp_up(v):
    return np.nextafter(math.log2(v), np.inf)


def ulp_down(v):
    return np.nextafter(math.log2(v), -np.inf)


def test_powers_of_two_exact_under_a_one_ulp_log2():
    for k in range(-60, 11):
        x = 2.0 ** k
        want = numpy_power(x)
        for f in (exact, ulp_up, ulp_down):
            # here 2m = 1: a log2(1) one ulp off zero is lost in the sum
            assert frexp_power(x, f) == want, (k, f.__name__)


def test_naive_form_misses_powers_of_two_by_a_factor_of_two():
    # the failure the frexp form avoids: log2(2^-6) one ulp above -6
    # truncates to -6 instead of -7
    x = 2.0 ** -6
    assert numpy_power(x) == -7
    assert naive_power(x, ulp_up) == -6


def test_random_steps_match_numpy_under_a_one_ulp_log2():
    rng = np.random.default_rng(5)
    xs = np.concatenate([
        10.0 ** rng.uniform(-12, 1, 20000),
        # a few ulps above and below powers of two
        [2.0 ** k * (1 + d * 2.0 ** -52) for k in range(-40, 4)
         for d in (-4, -3, -2, -1, 1, 2, 3, 4)],
    ])
    for x in xs:
        want = numpy_power(float(x))
        for f in (exact, ulp_up, ulp_down):
            assert frexp_power(float(x), f) == want, (x, f.__name__)
