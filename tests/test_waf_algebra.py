"""The division-free WAF flux used by the GPU kernels equals the reference's
flux formula to rounding.

Reference (Main/mod_moloch.F90:877-883 and the horizontal passes):
  r = local_flow_param(num, den);  b = max(0, min(2, max(r, min(2r, 1))))
  phi = is + zamu*b - is*b;        F = hvel*((1+phi)*a + (1-phi)*c)
with den = c - a.  The kernels form (a+c) - (is*den + (zamu-is)*B), B = b*den
chosen by the region of r, without dividing.
"""
from __future__ import annotations

import numpy as np


def ref_flux(hvel, is_, zamu, a, c, num):
    den = c - a
    minden, minnum = 1.0e-30, float(np.float32(1.0e-30))
    if abs(den) < minden:
        r = 1.0 if abs(num) < minnum else 0.0
    else:
        r = num / den
    b = max(0.0, min(2.0, max(r, min(2.0 * r, 1.0))))
    phi = is_ + zamu * b - is_ * b
    return hvel * ((1.0 + phi) * a + (1.0 - phi) * c)


def new_flux(hvel, is_, zamu, a, c, num):
    den = c - a
    aden = abs(den)
    if aden < 1.0e-30:
        B = den if abs(num) < float(np.float32(1.0e-30)) else 0.0
    else:
        q = -num if den < 0 else num
        if q <= 0:
            B = 0.0
        elif q < 0.5 * aden:
            B = num + num
        elif q <= aden:
            B = den
        elif q < 2.0 * aden:
            B = num
        else:
            B = den + den
    return hvel * ((a + c) - (is_ * den + (zamu - is_) * B))


def test_division_free_flux_matches_reference():
    rng = np.random.default_rng(42)
    worst = 0.0
    for _ in range(20000):
        base = rng.uniform(200.0, 400.0)
        a = base + rng.normal() * 10 ** rng.uniform(-6, 0)
        c = base + rng.normal() * 10 ** rng.uniform(-6, 0)
        num = (c - a) * rng.choice([-3.0, -0.7, 0.0, 0.2, 0.5, 0.9, 1.0, 1.5, 2.0, 3.0]) \
            + rng.normal() * 1e-9
        zamu = rng.uniform(-0.9, 0.9)
        is_ = 1.0 if zamu > 0 else -1.0
        hvel = 0.5 * rng.uniform(-20, 20)
        f0 = ref_flux(hvel, is_, zamu, a, c, num)
        f1 = new_flux(hvel, is_, zamu, a, c, num)
        scale = abs(hvel) * (abs(a) + abs(c))
        worst = max(worst, abs(f0 - f1) / scale)
    assert worst < 1e-15, worst


def test_region_ties_and_tiny_denominators():
    # r exactly at the limiter's breakpoints and |den| below 1e-30
    for num_over_den in (0.0, 0.5, 1.0, 2.0, -1.0):
        a, c = 1.0, 1.25
        num = (c - a) * num_over_den
        for zamu in (-0.4, 0.3):
            is_ = 1.0 if zamu > 0 else -1.0
            assert abs(ref_flux(3.0, is_, zamu, a, c, num) - new_flux(3.0, is_, zamu, a, c, num)) \
                <= 1e-15 * 3.0 * 2.25
    for num in (0.0, 1e-31, 1e-3):
        assert ref_flux(2.0, 1.0, 0.2, 5.0, 5.0, num) == new_flux(2.0, 1.0, 0.2, 5.0, 5.0, num)
