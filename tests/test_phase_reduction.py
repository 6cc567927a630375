"""Error bound of the FP32 forms' phase reduction (CPU).

The FP32 kernels reduce cycles = phi nu / c to [-1/2, 1/2] from FP32 pairs
(hi, lo) of the FP64 path length phi and of nu / c (``frac_cycles_df`` in
``montblanc_gb300/csrc/mb_common.cuh``).  This restates those FP32 steps with
NumPy float32 (each FMA rounded once from its exact value) and checks the
error against exact rational arithmetic: at most 1.25 |cycles| 2^-47 plus the
final FP32 rounding.  The GPU parity tests check the kernels themselves.
"""
from fractions import Fraction

import numpy as np

C = 299792458.0
f32 = np.float32


def _fma(a, b, c):
    return f32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def _split(x):
    h = f32(x)
    return h, f32(x - float(h))


def frac_cycles_df(phi, nu_over_c):
    ph, pl = _split(phi)
    nh, nl = _split(nu_over_c)
    p = f32(ph * nh)
    e = _fma(ph, nh, -p)
    e = _fma(ph, nl, e)
    e = _fma(pl, nh, e)
    return f32(f32(p - np.rint(p)) + e)


def test_double_float_phase_reduction_bound():
    rng = np.random.default_rng(7)
    worst = 0.0
    for _ in range(600):
        phi = rng.uniform(-3e4, 3e4) * rng.choice([1e-6, 1e-3, 1.0, 30.0])
        nu_over_c = rng.uniform(5e7, 3e10) / C
        got = frac_cycles_df(phi, nu_over_c)
        exact = Fraction(phi) * Fraction(nu_over_c)
        d = float(Fraction(float(got)) - (exact - round(exact)))
        d -= round(d)  # a tie may come out as +1/2 or -1/2
        cycles = abs(float(exact))
        bound = 1.25 * cycles * 2.0 ** -47 + 2.0 ** -25
        worst = max(worst, abs(d) / bound)
        assert abs(d) <= bound, (phi, nu_over_c, d, bound)
        # reduced to within 3 |cycles| 2^-24 of [-1/2, 1/2] (the sincospi
        # that takes it reduces the rest exactly)
        assert abs(float(got)) <= 0.5 + 3.0 * cycles * 2.0 ** -24 + 2.0 ** -20
    assert worst > 0.0
