"""The library's host setup helpers against the oracle's own restatement of
RegCM's setup routines, bit for bit (both are FP64 host code without FMA
contraction, run in the same process)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle import oracle as orc
from regcm_gb300 import abi
from regcm_gb300 import case as cs


def _dims(jx, iy, kz, nqx=2, ntr=0):
    return abi.mlc_dims(jx, iy, kz, nqx, ntr)


@pytest.mark.parametrize("kz,ztop", [(4, 25000.0), (30, 25000.0), (41, 25000.0), (60, 30000.0)])
def test_levels(kz, ztop):
    lib, ol = abi.load(), orc.load()
    a, b = np.zeros(kz + 1), np.zeros(kz)
    c, d = np.zeros(kz + 1), np.zeros(kz)
    assert lib.mlc_setup_levels(kz, ztop, abi.dptr(a), abi.dptr(b)) == 0
    ol.orc_setup_levels(kz, ztop, abi.dptr(c), abi.dptr(d))
    assert np.array_equal(a, c) and np.array_equal(b, d)
    assert a[0] == ztop and a[-1] == 0.0 and np.all(np.diff(a) < 0)


@pytest.mark.parametrize("np_,lo,hi", [(1, 0.1, 1.0), (2, 0.025, 0.75), (8, 0.025, 0.75),
                                      (16, 0.0333, 0.999), (32, 0.001, 0.999)])
def test_relax_coefficients(np_, lo, hi):
    lib, ol = abi.load(), orc.load()
    a, b = np.zeros(np_), np.zeros(np_)
    assert lib.mlc_relax_coefficients(np_, lo, hi, abi.dptr(a)) == 0
    assert ol.orc_relax_coefficients(np_, lo, hi, abi.dptr(b)) == 0
    assert np.array_equal(a, b)
    assert np.all((a > 0) & (a < 1))


def test_relax_coefficients_known_answer():
    # np = 1: the recursion is empty, k = p(1)/q(0) = 1, weight = s/(1+s)
    # with s = sqrt(gmmin*gmmax) (Main/mpplib/mod_runparams.F90:689-700)
    a = np.zeros(1)
    assert abi.load().mlc_relax_coefficients(1, 0.25, 0.64, abi.dptr(a)) == 0
    s = np.sqrt(0.25 * 0.64)
    assert a[0] == s / (1.0 + s)
    # not a power of two is rejected like the reference's fatal()
    b = np.zeros(6)
    assert abi.load().mlc_relax_coefficients(6, 0.1, 1.0, abi.dptr(b)) == abi.MLC_ERR_INVALID


@pytest.mark.parametrize("jx,iy,nx,ny", [(25, 21, 10, 10), (65, 65, 10, 10), (33, 33, 18, 18),
                                         (40, 30, 6, 8)])
def test_boundaries(jx, iy, nx, ny):
    lib, ol = abi.load(), orc.load()
    for lx, ly in ((0, 0), (1, 0), (0, 1)):
        a = np.zeros((jx, iy), dtype=np.int32, order="F")
        b = np.zeros((jx, iy), dtype=np.int32, order="F")
        assert lib.mlc_setup_boundaries(jx, iy, lx, ly, nx, ny, abi.iptr(a)) == 0
        ol.orc_setup_boundaries(jx, iy, lx, ly, nx, ny, abi.iptr(b))
        assert np.array_equal(a, b)
        assert a.max() <= max(nx, ny) - 1 and (a[a > 0] >= 2).all()


def test_nspg_lehmann():
    lib = abi.load()
    gx, gd = C.c_int(), C.c_int()
    # ds = 12 km -> nint(20*12^-0.35)+1 = 9 -> power of two 8 + 2 = 10
    lib.mlc_setup_nspg(65, 65, 12.0, 1, 0, 0, C.byref(gx), C.byref(gd))
    assert (gx.value, gd.value) == (10, 10)
    # ds = 3 km -> 15 -> 16 + 2 = 18
    lib.mlc_setup_nspg(513, 513, 3.0, 1, 0, 0, C.byref(gx), C.byref(gd))
    assert (gx.value, gd.value) == (18, 18)


@pytest.mark.parametrize("moist,lrot", [(False, False), (True, False), (False, True)])
def test_metric_relaxation_pai(moist, lrot):
    c = cs.build(22, 18, 12, dx=12000.0, dt=60.0, nsound=3, moist=moist, seed=5,
                 hills=[(9 * 12000.0, 8 * 12000.0, 900.0)], lrotllr=lrot)
    ol = orc.load()
    d, p = c.dims, c.params
    jx, iy, kz = d.jx, d.iy, d.kz
    st = c.static
    names = ["hx", "hy", "zeta", "fmz", "rfmzu", "rfmzv", "fmzf", "zetaf", "dz"]
    out = {n: np.zeros_like(st[n], order="F") for n in names}
    ol.orc_setup_metric(C.byref(d), C.byref(p), *[abi.dptr(st[n]) for n in (
        "ht", "htu", "htv", "msfu", "msfv", "zita", "zitah")], *[abi.dptr(out[n]) for n in names])
    for n in names:
        assert np.array_equal(out[n], st[n]), n
    hefc = np.zeros_like(st["hefc"], order="F")
    fcx = np.zeros(p.nspgx)
    tn, ff = np.zeros(kz), np.zeros(kz)
    nz = C.c_int()
    ol.orc_setup_relaxation(C.byref(d), C.byref(p), abi.dptr(st["zeta"]), abi.dptr(hefc),
                            abi.dptr(fcx), abi.dptr(tn), abi.dptr(ff), C.byref(nz))
    assert np.array_equal(hefc, st["hefc"])
    assert np.array_equal(fcx, st["fcx"])
    assert np.array_equal(tn, st["tnudge"]) and np.array_equal(ff, st["ffilt"])
    assert nz.value == p.nztop
    # spectral nudging weights from the level-mean heights
    cn_lib, cn_orc = np.zeros(kz), np.zeros(kz)
    assert abi.load().mlc_setup_spectral(C.byref(p), kz, abi.dptr(st["gmeanz"]), abi.dptr(cn_lib)) == 0
    ol.orc_setup_spectral(C.byref(p), kz, abi.dptr(st["gmeanz"]), abi.dptr(cn_orc))
    assert np.array_equal(cn_lib, cn_orc)
    assert np.all(cn_lib >= 0) and cn_lib.max() <= p.dtrad / p.dtbdys
    # paicompute on the case's own inputs
    t = c.bdy["xtb"][0]
    qv = c.bdy["xqb"][0]
    ps = c.bdy["xpsb"][0]
    pai = np.zeros_like(t, order="F")
    ol.orc_paicompute(C.byref(d), abi.dptr(ps), abi.dptr(st["zeta"]), abi.dptr(np.asfortranarray(
        cs.isa(np.asfortranarray(c.static["ht"][: jx - 1, : iy - 1, None] / cs.GRAV + st["zeta"]))[0])),
        abi.dptr(qv), abi.dptr(st["fmzf"]), st["zita"][kz - 1], abi.dptr(pai))
    mine = np.zeros_like(pai, order="F")
    tis = np.asfortranarray(cs.isa(np.asfortranarray(
        c.static["ht"][: jx - 1, : iy - 1, None] / cs.GRAV + st["zeta"]))[0])
    assert abi.load().mlc_paicompute(C.byref(d), C.byref(p), abi.dptr(ps), abi.dptr(st["zeta"]),
                                     abi.dptr(tis), abi.dptr(qv), abi.dptr(st["fmzf"]),
                                     abi.dptr(st["zita"]), abi.dptr(mine)) == 0
    assert np.array_equal(mine, pai)
    assert np.all((pai > 0.3) & (pai < 1.1))


def test_pfwsat_known_answer():
    # at 0 C the polynomial is its constant term a0 = 611.213476 Pa
    t = np.asfortranarray([273.15, 273.15, 300.0])
    p = np.asfortranarray([1.0e5, 3.0e3, 1.0e5])
    q = cs.pfwsat(t, p)
    ep2 = 18.01528 / 28.96454
    assert q[0] == ep2 * (0.611213476e3 / (1.0e5 - 0.611213476e3))
    # the 0.15 p cap (Share/pfwsat.inc:36-41)
    assert q[1] == ep2 * ((0.15 * 3.0e3) / (3.0e3 - 0.15 * 3.0e3))
    assert 0.02 < q[2] < 0.03


@pytest.mark.parametrize("jx,iy,ds,leh", [(65, 65, 12.0, 1), (513, 513, 3.0, 1), (65, 65, 12.0, 0),
                                          (30, 200, 50.0, 0), (401, 97, 2.0, 0), (49, 49, 25.0, 1)])
def test_nspg_oracle(jx, iy, ds, leh):
    a, b, c, d = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    assert abi.load().mlc_setup_nspg(jx, iy, ds, leh, 0, 0, C.byref(a), C.byref(b)) == 0
    assert orc.load().orc_setup_nspg(jx, iy, ds, leh, 0, 0, C.byref(c), C.byref(d)) == 0
    assert (a.value, b.value) == (c.value, d.value)


@pytest.mark.parametrize("make", [
    lambda su: cs.config0(nx=32, ny=28, kz=20, setup=su),
    lambda su: cs.config1(nx=40, ny=36, kz=24, setup=su),
    lambda su: cs.build(24, 22, 12, dx=12000.0, dt=60.0, nsound=3, moist=True, seed=2,
                        spectral=True, setup=su),
])
def test_case_from_oracle_setup_is_identical(make):
    """A case built through the oracle's setup (how the CPU reference timing
    builds its input without loading the GPU library) holds exactly the
    bytes of the case the library's setup builds."""
    a = make(None)
    b = make(orc.OracleSetup())
    for f, _ in abi.mlc_params._fields_:
        assert getattr(a.params, f) == getattr(b.params, f), f
    assert a.dims.as_tuple() == b.dims.as_tuple()
    for part in ("static", "state"):
        da, db = getattr(a, part), getattr(b, part)
        assert da.keys() == db.keys()
        for n in da:
            assert np.array_equal(da[n], db[n]), (part, n)
    for n in a.bdy:
        for x, y in zip(a.bdy[n], b.bdy[n]):
            assert np.array_equal(x, y), n


@pytest.mark.parametrize("kz,ztop,hml", [(30, 25000.0, (3.0, 2.0, 1.0)), (41, 25000.0, (3.0, 2.0, 1.0)),
                                         (18, 30000.0, (5.0, 1.5, 0.5)), (60, 20000.0, (2.0, 2.5, 1.0))])
def test_exponential_nudging(kz, ztop, hml):
    lib, ol = abi.load(), orc.load()
    a, b = np.zeros(kz), np.zeros(kz)
    assert lib.mlc_exponential_nudging(kz, ztop, *hml, abi.dptr(a)) == 0
    assert ol.orc_exponential_nudging(kz, ztop, *hml, abi.dptr(b)) == 0
    assert np.array_equal(a, b)
    assert np.all(a > 0)


def test_exponential_nudging_known_answers():
    lib = abi.load()
    # equal strengths: the spline is the constant
    a = np.zeros(30)
    assert lib.mlc_exponential_nudging(30, 25000.0, 2.0, 2.0, 2.0, abi.dptr(a)) == 0
    assert np.all(a == 2.0)
    # the reference's strengths 3, 2, 1 fall from the top (k = 1) to the surface
    assert lib.mlc_exponential_nudging(30, 25000.0, 3.0, 2.0, 1.0, abi.dptr(a)) == 0
    assert np.all(np.diff(a) < 0) and 2.9 < a[0] <= 3.0 and 1.0 <= a[-1] < 1.1


@pytest.mark.parametrize("moist", [False, True])
def test_exponential_relaxation_weights(moist):
    """hefc with bdy_use_lehmann = .false.: the library's setup equals the
    oracle's bit for bit, and the weights are exp(-(n-1)/anudge(k))."""
    c = cs.build(30, 26, 20, dx=12000.0, dt=60.0, nsound=3, moist=moist, seed=6, lehmann=False)
    d, p, st = c.dims, c.params, c.static
    assert p.bdy_use_lehmann == 0 and p.nspgx >= 6
    hefc = np.zeros_like(st["hefc"], order="F")
    fcx = np.zeros(p.nspgx)
    tn, ff = np.zeros(d.kz), np.zeros(d.kz)
    nz = C.c_int()
    orc.load().orc_setup_relaxation(C.byref(d), C.byref(p), abi.dptr(st["zeta"]), abi.dptr(hefc),
                                    abi.dptr(fcx), abi.dptr(tn), abi.dptr(ff), C.byref(nz))
    assert np.array_equal(hefc, st["hefc"])
    an = np.zeros(d.kz)
    abi.load().mlc_exponential_nudging(d.kz, p.mo_ztop, 3.0, 2.0, 1.0, abi.dptr(an))
    n = np.arange(2, p.nspgx)
    assert np.allclose(st["hefc"][1:-1, :], np.exp(-(n - 1)[:, None] / an[None, :]), rtol=1e-15)
    assert np.all(st["hefc"][0] == 1.0) and np.all(st["hefc"][-1] == 0.0)
