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
    """The kernels' form: B = sign(den) * max(0, min(2d, max(q, min(2q, d))))
    with d = |den|, q = num*sign(den); no division, no branch on r."""
    den = c - a
    d = abs(den)
    q = -num if den < 0 else num
    bd = max(0.0, min(d + d, max(q, min(q + q, d))))
    B = -bd if den < 0 else bd
    if d < 1.0e-30:
        B = den if abs(num) < float(np.float32(1.0e-30)) else 0.0
    return hvel * ((a + c) - (is_ * den + (zamu - is_) * B))


def wind_flux(hvel, is_, zamu, a, c, num):
    """The kernels' present form vel*(x - zmih*B): vel = 2*hvel, x = a when
    is = +1 else c, zmih = (zamu - is)/2 (per interface, for every field)."""
    den = c - a
    d = abs(den)
    q = -num if den < 0 else num
    bd = max(0.0, min(d + d, max(q, min(q + q, d))))
    B = -bd if den < 0 else bd
    if d < 1.0e-30:
        B = den if abs(num) < float(np.float32(1.0e-30)) else 0.0
    x = a if is_ > 0 else c
    zmih = (zamu - is_) * 0.5
    return (2.0 * hvel) * (x - zmih * B)


def branch_b(num, den):
    """B = b*den by region of r = num/den (the earlier form, kept as a check)."""
    aden = abs(den)
    if aden < 1.0e-30:
        return den if abs(num) < float(np.float32(1.0e-30)) else 0.0
    q = -num if den < 0 else num
    if q <= 0:
        return 0.0
    if q < 0.5 * aden:
        return num + num
    if q <= aden:
        return den
    if q < 2.0 * aden:
        return num
    return den + den


def test_clamp_limiter_equals_region_form_exactly():
    rng = np.random.default_rng(3)
    for _ in range(20000):
        den = rng.normal() * 10 ** rng.uniform(-3, 3)
        num = den * rng.choice([-1.0, 0.0, 0.25, 0.5, 0.75, 1.0, 1.5, 2.0, 3.0, rng.uniform(-3, 3)])
        d = abs(den)
        q = -num if den < 0 else num
        bd = max(0.0, min(d + d, max(q, min(q + q, d))))
        B = -bd if den < 0 else bd
        assert B == branch_b(num, den), (num, den)


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
        f2 = wind_flux(hvel, is_, zamu, a, c, num)
        scale = abs(hvel) * (abs(a) + abs(c))
        worst = max(worst, abs(f0 - f1) / scale, abs(f0 - f2) / scale)
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
            assert abs(ref_flux(3.0, is_, zamu, a, c, num) - wind_flux(3.0, is_, zamu, a, c, num)) \
                <= 1e-15 * 3.0 * 2.25
    for num in (0.0, 1e-31, 1e-3):
        assert ref_flux(2.0, 1.0, 0.2, 5.0, 5.0, num) == new_flux(2.0, 1.0, 0.2, 5.0, 5.0, num)


# ---- increment form (the FP64 fields of a mixed member) --------------------
# The kernels advect theta_v and Exner relative to each cell's own value:
# fluxes from neighbour differences, moved between the two cells of an
# interface by -2*hvel*(difference), constant parts kept apart where the
# scheme does not preserve a constant (model top; non-uniform map factors).
# Evaluated in FP64, the increment form equals the direct form to rounding.

def vertical_direct(v, s, zu, zd, dtrdz):
    kz = len(v)
    col = v.copy()
    for _ in range(2):
        flx = np.zeros(kz + 1)
        for k in range(1, kz):            # interface k+1 (1-based), flx index k
            skp = s[k]                     # s(k+1)
            zamu = skp * dtrdz
            if zamu >= 0:
                is_, k1, k1p1 = 1.0, k + 1, min(k + 2, kz)
            else:
                is_, k1, k1p1 = -1.0, max(k - 1, 1), k
            flx[k] = ref_flux(0.5 * skp, is_, zamu, col[k], col[k - 1], col[k1 - 1] - col[k1p1 - 1])
        new = col.copy()
        for k in range(kz):
            pk = col[k]
            zdv = (s[k] * zu[k] - s[k + 1] * zd[k]) * pk
            new[k] = pk - flx[k] * zu[k] + flx[k + 1] * zd[k] + zdv
        col = new
    return col


def vertical_increment(v, s, zu, zd, dtrdz):
    kz = len(v)
    dz = np.diff(v)                        # dz[k-1] = v(k+1) - v(k)
    e = np.zeros(kz)
    eb32 = et32 = hb = ht = 0.0
    for _ in range(2):
        fb = 0.0
        new = e.copy()
        for k in range(1, kz + 1):
            sk, skp = s[k - 1], s[k]
            fa = fup = 0.0
            if k <= kz - 1:
                zamu = skp * dtrdz
                ek, ekp1 = e[k - 1], e[k]
                if zamu >= 0:
                    is_ = 1.0
                    num = (ekp1 - e[k + 1]) - dz[k] if k + 2 <= kz else 0.0
                else:
                    is_ = -1.0
                    num = (e[k - 2] - ek) - dz[k - 2] if k >= 2 else 0.0
                fa = new_flux(0.5 * skp, is_, zamu, dz[k - 1] + ekp1, ek, num)
                fup = fa - skp * dz[k - 1]
            upd = -fb * zu[k - 1] + fa * zd[k - 1] + (sk * zu[k - 1] - skp * zd[k - 1]) * e[k - 1]
            if k == kz:
                et32 += upd
                ht += v[k - 1] * (-skp * zd[k - 1])
                new[k - 1] = et32 + ht
            elif k == 1:
                eb32 += upd
                hb += v[0] * (sk * zu[0])
                new[0] = eb32 + hb
            else:
                new[k - 1] = e[k - 1] + upd
            fb = fup
        e = new
    return v + e


def test_vertical_increment_form_equals_direct():
    rng = np.random.default_rng(7)
    worst = 0.0
    for _ in range(300):
        kz = int(rng.integers(4, 14))
        v = 300.0 + np.cumsum(rng.uniform(0.0, 8.0, kz)) + rng.normal(0, 0.5, kz)
        s = rng.normal(0, 0.4, kz + 1)
        s[0] = 0.0 if rng.uniform() < 0.7 else s[0]   # s(1) = 0 in the interior
        zu = rng.uniform(0.02, 0.3, kz)
        zd = rng.uniform(0.02, 0.3, kz)
        dtrdz = rng.uniform(0.05, 0.6)
        a = vertical_direct(v, s, zu, zd, dtrdz)
        b = vertical_increment(v, s, zu, zd, dtrdz)
        worst = max(worst, float(np.max(np.abs(a - b)) / np.max(np.abs(v))))
    assert worst < 1e-13, worst


def horizontal_direct(pp, wz, u, v, msfu, msfv, mx2, rmu, rmv, zfac, rot, dtr):
    """Meridional then zonal WAF on (ny, nx) cross points, 1-based rows i and
    columns j as the kernels; zfac stands for fmz*rfmz* (one per point)."""
    ny, nx = pp.shape
    iy, jx = ny + 1, nx + 1
    imin, imax, jmin, jmax = 1, iy - 1, 1, jx - 1
    P = lambda a, j, i: a[i - 1, j - 1]
    zpby = np.zeros((iy + 1, jx + 1))
    for i in range(2, iy):
        for j in range(1, jx):
            vv = v[i - 1, j - 1]
            zamu = vv * dtr if rot else vv * msfv[i - 1, j - 1] * dtr
            if zamu > 0:
                is_, ih = 1.0, i - 1
            else:
                is_, ih = -1.0, min(i + 1, imax)
            ihm1 = max(ih - 1, imin)
            zpby[i, j] = ref_flux(0.5 * vv, is_, zamu, P(wz, j, i - 1), P(wz, j, i),
                                  P(wz, j, ih) - P(wz, j, ihm1))
    p0 = np.zeros((iy + 1, jx + 1))
    for i in range(2, iy - 1):
        for j in range(1, jx):
            zn, zs = dtr * zfac[i, j - 1], dtr * zfac[i - 1, j - 1]
            vs, vn = v[i - 1, j - 1], v[i, j - 1]
            if rot:
                zdv = (vn * zn - vs * zs) * P(pp, j, i)
                p0[i, j] = P(wz, j, i) + (zpby[i, j] * zs - zpby[i + 1, j] * zn + zdv)
            else:
                zdv = (vn * rmv[i, j - 1] * zn - vs * rmv[i - 1, j - 1] * zs) * P(pp, j, i)
                p0[i, j] = P(wz, j, i) + mx2[i - 1, j - 1] * (zpby[i, j] * zs - zpby[i + 1, j] * zn + zdv)
    out = pp.copy()
    zpbw = np.zeros((iy + 1, jx + 1))
    for i in range(2, iy - 1):
        for j in range(2, jx):
            uu = u[i - 1, j - 1]
            zamu = uu * msfu[i - 1, j - 1] * dtr
            if zamu > 0:
                is_, jh = 1.0, j - 1
            else:
                is_, jh = -1.0, min(j + 1, jmax)
            jhm1 = max(jh - 1, jmin)
            zpbw[i, j] = ref_flux(0.5 * uu, is_, zamu, p0[i, j - 1], p0[i, j], p0[i, jh] - p0[i, jhm1])
        for j in range(2, jx - 1):
            zw, ze = dtr * zfac[i - 1, j - 1], dtr * zfac[i - 1, j]
            uw, ue = u[i - 1, j - 1], u[i - 1, j]
            if rot:
                zdv = (ue * ze - uw * zw) * P(pp, j, i)
                out[i - 1, j - 1] = p0[i, j] + zpbw[i, j] * zw - zpbw[i, j + 1] * ze + zdv
            else:
                zdv = (ue * rmu[i - 1, j] * ze - uw * rmu[i - 1, j - 1] * zw) * P(pp, j, i)
                out[i - 1, j - 1] = p0[i, j] + mx2[i - 1, j - 1] * (zpbw[i, j] * zw - zpbw[i, j + 1] * ze + zdv)
    return out


def horizontal_increment(pp, wz, u, v, msfu, msfv, mx2, rmu, rmv, zfac, rot, dtr):
    ny, nx = pp.shape
    iy, jx = ny + 1, nx + 1
    imin, imax, jmin, jmax = 1, iy - 1, 1, jx - 1
    P = lambda a, j, i: a[i - 1, j - 1]
    dz = wz - pp
    dy = lambda j, i: P(pp, j, i + 1) - P(pp, j, i)
    dx = lambda j, i: P(pp, j + 1, i) - P(pp, j, i)
    fy = np.zeros((iy + 1, jx + 1))            # relative to pp(i-1)
    for i in range(2, iy):
        for j in range(1, jx):
            vv = v[i - 1, j - 1]
            zamu = vv * dtr if rot else vv * msfv[i - 1, j - 1] * dtr
            if zamu > 0:
                is_, ih = 1.0, i - 1
            else:
                is_, ih = -1.0, min(i + 1, imax)
            ihm1 = max(ih - 1, imin)
            dpp = dy(j, ihm1) if ih != ihm1 else 0.0
            num = (P(dz, j, ih) - P(dz, j, ihm1)) + dpp
            fy[i, j] = new_flux(0.5 * vv, is_, zamu, P(dz, j, i - 1), P(dz, j, i) + dy(j, i - 1), num)
    hy = np.zeros((iy + 1, jx + 1))
    ey = np.zeros((iy + 1, jx + 1))
    for i in range(2, iy - 1):
        for j in range(1, jx):
            zn, zs = dtr * zfac[i, j - 1], dtr * zfac[i - 1, j - 1]
            vs, vn = v[i - 1, j - 1], v[i, j - 1]
            fs = fy[i, j] - vs * dy(j, i - 1)
            fn = fy[i + 1, j]
            if rot:
                h = fs * zs - fn * zn
            else:
                m, rs, rn = mx2[i - 1, j - 1], rmv[i - 1, j - 1], rmv[i, j - 1]
                h = m * (fs * zs - fn * zn) + P(pp, j, i) * (m * (vs * zs * (1 - rs) - vn * zn * (1 - rn)))
            hy[i, j] = h
            ey[i, j] = P(dz, j, i) + h
    out = pp.copy()
    for i in range(2, iy - 1):
        fx = np.zeros(jx + 1)
        for j in range(2, jx):
            uu = u[i - 1, j - 1]
            zamu = uu * msfu[i - 1, j - 1] * dtr
            if zamu > 0:
                is_, jh = 1.0, j - 1
            else:
                is_, jh = -1.0, min(j + 1, jmax)
            jhm1 = max(jh - 1, jmin)
            dpp = dx(jhm1, i) if jh != jhm1 else 0.0
            num = (ey[i, jh] - ey[i, jhm1]) + dpp
            fx[j] = new_flux(0.5 * uu, is_, zamu, ey[i, j - 1], ey[i, j] + dx(j - 1, i), num)
        for j in range(2, jx - 1):
            zw, ze = dtr * zfac[i - 1, j - 1], dtr * zfac[i - 1, j]
            uw, ue = u[i - 1, j - 1], u[i - 1, j]
            fw = fx[j] - uw * dx(j - 1, i)
            fe = fx[j + 1]
            if rot:
                h = fw * zw - fe * ze
            else:
                m, rw, re = mx2[i - 1, j - 1], rmu[i - 1, j - 1], rmu[i - 1, j]
                h = m * (fw * zw - fe * ze) + P(pp, j, i) * (m * (uw * zw * (1 - rw) - ue * ze * (1 - re)))
            out[i - 1, j - 1] = P(pp, j, i) + P(dz, j, i) + (hy[i, j] + h)
    return out


def test_horizontal_increment_form_equals_direct():
    rng = np.random.default_rng(11)
    worst = 0.0
    for trial in range(24):
        ny, nx = int(rng.integers(5, 11)), int(rng.integers(5, 11))
        pp = 300.0 + rng.normal(0, 3.0, (ny, nx)) + np.linspace(0, 5, nx)[None, :]
        wz = pp + rng.normal(0, 0.2, (ny, nx))
        shp = (ny + 1, nx + 1)
        u, v = rng.normal(0, 8, shp), rng.normal(0, 8, shp)
        uniform = trial % 3 == 0
        msfu = np.ones(shp) if uniform else rng.uniform(0.97, 1.03, shp)
        msfv = np.ones(shp) if uniform else rng.uniform(0.97, 1.03, shp)
        mx2 = np.ones(shp) if uniform else rng.uniform(0.95, 1.05, shp)
        rmu, rmv = 1.0 / msfu, 1.0 / msfv
        zfac = rng.uniform(0.9, 1.1, shp)
        rot = trial % 4 == 1
        dtr = rng.uniform(0.002, 0.01)
        a = horizontal_direct(pp, wz, u, v, msfu, msfv, mx2, rmu, rmv, zfac, rot, dtr)
        b = horizontal_increment(pp, wz, u, v, msfu, msfv, mx2, rmu, rmv, zfac, rot, dtr)
        worst = max(worst, float(np.max(np.abs(a - b)) / 300.0))
    assert worst < 1e-13, worst
