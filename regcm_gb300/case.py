"""Synthetic MOLOCH domains: the stand-in for RegCM's terrain and ICBC input.

RegCM reads its terrain and initial/boundary conditions from netCDF files made
by its preprocessors; none exist here, so a ``Case`` builds the same arrays in
memory from a seeded recipe:

* Cartesian grid, map factors 1, f-plane at 45N, model top 25 km, uniform
  zita spacing (Share/mod_zita.F90:54-86), mo_h = 8 km, mo_a0 = 0.
* Gaussian hills h0*exp(-ln2*(r/(10 dx))^2) sampled at cross, u and v points
  and stored as geopotential (Main/mod_params.F90:2436-2440).
* US standard atmosphere T(z) and hydrostatic pressure (Share/mod_isaatm.F90:
  27-69) at the terrain-following levels, Exner function by paicompute
  (Main/mod_bdycod.F90:3762-3796), theta_v perturbed by seeded uniform noise.
* Boundary data b0 = b1 = the initial state; the prognostic state is derived
  from b0 the way init does (Main/mod_init.F90:155-219).
* Lehmann relaxation weights (bdy_use_lehmann = .true.), top nudging on,
  spectral nudging off, divergence damping and filter on.

Static fields come from a setup backend: by default the library's own host
setup (moloch_gb300_setup.h, ``LibrarySetup``); any object with the same
methods may stand in for it (a caller that must not load the GPU library
passes its own).  Every array is a Fortran-ordered float64 numpy array with the extents of
include/moloch_gb300.h.  Random numbers come from SplitMix64 so any consumer
(the GPU library, the CPU oracle) sees identical bytes.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import abi

# Share/mod_constants.F90 (non-RCEMIP), the values of mlc_constants.h
GRAV = 9.80665
RGAS = ((6.02214076e23 * 1.3806490e-23) / 28.96454) * 1000.0
CPD = 3.5 * RGAS
EP1 = 28.96454 / 18.01528 - 1.0
P00 = 1.0e5
STDP = 1.013250e5
STDT = 288.15
LRATE = 0.00649
CPOVR = CPD / RGAS


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n uniform doubles in [0, 1) from SplitMix64 started at `seed`."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + \
            np.arange(1, n + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def isa(height):
    """US standard atmosphere T [K], p [Pa] for heights 0-32 km (mod_isaatm)."""
    h = np.asarray(height, dtype=np.float64)
    g_rl = GRAV / (RGAS * LRATE)
    t11 = STDT - LRATE * 11000.0
    p11 = STDP * (t11 / STDT) ** g_rl
    p20 = p11 * np.exp(-GRAV * (20000.0 - 11000.0) / (RGAS * t11))
    t = np.where(h <= 11000.0, STDT - LRATE * h,
                 np.where(h <= 20000.0, t11, t11 + 0.001 * (h - 20000.0)))
    p_low = STDP * (np.maximum(t, 1.0) / STDT) ** g_rl
    p_mid = p11 * np.exp(-GRAV * (h - 11000.0) / (RGAS * t11))
    p_up = p20 * (t / t11) ** (-(GRAV / (RGAS * 0.001)))
    p = np.where(h <= 11000.0, p_low, np.where(h <= 20000.0, p_mid, p_up))
    return t, p


class LibrarySetup:
    """The library's host setup helpers (include/moloch_gb300_setup.h) as a
    case-building backend: levels, nspgx, metric, relaxation weights,
    boundary masks, spectral weights, paicompute and pfwsat."""

    def __init__(self):
        self.lib = abi.load()

    def nspg(self, jx, iy, ds_km, lehmann=True):
        gx, gd = C.c_int(), C.c_int()
        abi.check(self.lib.mlc_setup_nspg(jx, iy, ds_km, 1 if lehmann else 0, 0, 0,
                                          C.byref(gx), C.byref(gd)), "mlc_setup_nspg")
        return gx.value, gd.value

    def levels(self, kz, ztop, zita, zitah):
        abi.check(self.lib.mlc_setup_levels(kz, ztop, abi.dptr(zita), abi.dptr(zitah)),
                  "mlc_setup_levels")

    def metric(self, dims, params, arrays):
        abi.check(self.lib.mlc_setup_metric(C.byref(dims), C.byref(params),
                                            *[abi.dptr(a) for a in arrays]), "mlc_setup_metric")

    def relaxation(self, dims, params, zeta, hefc, fcx, tnudge, ffilt, gmeanz):
        abi.check(self.lib.mlc_setup_relaxation(C.byref(dims), C.byref(params), abi.dptr(zeta),
                                                abi.dptr(hefc), abi.dptr(fcx), abi.dptr(tnudge),
                                                abi.dptr(ffilt), abi.dptr(gmeanz)),
                  "mlc_setup_relaxation")

    def boundaries(self, jx, iy, lx, ly, nspgx, nspgd, out):
        abi.check(self.lib.mlc_setup_boundaries(jx, iy, lx, ly, nspgx, nspgd, abi.iptr(out)),
                  "mlc_setup_boundaries")

    def spectral(self, params, kz, gmeanz, cnudge):
        abi.check(self.lib.mlc_setup_spectral(C.byref(params), kz, abi.dptr(gmeanz),
                                              abi.dptr(cnudge)), "mlc_setup_spectral")

    def paicompute(self, dims, params, ps, zeta, t, qv, fmzf, zita, pai):
        abi.check(self.lib.mlc_paicompute(C.byref(dims), C.byref(params), abi.dptr(ps),
                                          abi.dptr(zeta), abi.dptr(t), abi.dptr(qv),
                                          abi.dptr(fmzf), abi.dptr(zita), abi.dptr(pai)),
                  "mlc_paicompute")

    def pfwsat(self, t, p):
        t = np.asfortranarray(t, dtype=np.float64)
        p = np.asfortranarray(p, dtype=np.float64)
        out = np.empty_like(t, order="F")
        abi.check(self.lib.mlc_pfwsat(t.size, abi.dptr(t), abi.dptr(p), abi.dptr(out)),
                  "mlc_pfwsat")
        return out


def pfwsat(t, p, setup=None):
    """Saturation mixing ratio (Share/pfwsat.inc) through the setup backend."""
    return (setup or LibrarySetup()).pfwsat(t, p)


def _f(shape):
    return np.zeros(shape, dtype=np.float64, order="F")


@dataclass
class Case:
    """One domain: extents, run parameters, static fields, state, boundary."""
    name: str
    dims: abi.mlc_dims
    params: abi.mlc_params
    static: dict = field(default_factory=dict)
    state: dict = field(default_factory=dict)
    bdy: dict = field(default_factory=dict)
    xbctime: float = 0.0

    @property
    def points(self) -> int:
        """Cross points x levels: the grid points one model step advances."""
        d = self.dims
        return (d.jx - 1) * (d.iy - 1) * d.kz

    # -- pointer structs (arrays stay owned by this object) ---------------
    def static_ptrs(self) -> abi.mlc_static_ptrs:
        s = abi.mlc_static_ptrs()
        for n in abi.STATIC_FIELDS + abi.SPECTRAL_FIELDS:
            setattr(s, n, abi.dptr(self.static.get(n)))
        for n in abi.IBND_FIELDS:
            setattr(s, n, abi.iptr(self.static[n]))
        return s

    @staticmethod
    def state_ptrs_of(state: dict) -> abi.mlc_state_ptrs:
        s = abi.mlc_state_ptrs()
        for n in abi.STATE_FIELDS:
            setattr(s, n, abi.dptr(state.get(n)))
        return s

    def state_ptrs(self) -> abi.mlc_state_ptrs:
        return self.state_ptrs_of(self.state)

    def bdy_ptrs(self) -> abi.mlc_bdy_ptrs:
        b = abi.mlc_bdy_ptrs()
        for n in abi.BDY_FIELDS:
            pair = self.bdy.get(n, (None, None))
            arr = (C.POINTER(C.c_double) * 2)(abi.dptr(pair[0]), abi.dptr(pair[1]))
            setattr(b, n, arr)
        return b

    def tendencies(self, seed: int = 0) -> dict:
        """Synthetic physics tendencies on the interior jci x ici, Fortran
        arrays (jx-3, iy-3, kz[, n]) as mo_atm%tten/uten/vten/qxten/chiten:
        heating and wind forcing of a few K/day and m/s/h, small species
        sources, and at one point in twenty a sink of 1.5 times the initial
        amount per step, which drives q below its floor there."""
        d = self.dims
        rng = np.random.default_rng(seed)
        shp = (d.jx - 3, d.iy - 3, d.kz)
        f = lambda a: np.asfortranarray(a, dtype=np.float64)
        out = {"tten": f(rng.normal(0.0, 1e-4, shp)), "uten": f(rng.normal(0.0, 3e-4, shp)),
               "vten": f(rng.normal(0.0, 3e-4, shp))}
        dt = self.params.dtsec

        def species(q0, scale):
            ten = rng.normal(0.0, scale, q0.shape)
            sink = rng.random(q0.shape) < 0.05
            ten[sink] = -1.5 * q0[sink] / dt - scale
            return f(ten)

        out["qxten"] = species(self.state["qx"][1:-1, 1:-1], 1e-9)
        if d.ntr:
            out["chiten"] = species(self.state["trac"][1:-1, 1:-1], 1e-7)
        if self.params.ibltyp == 2:
            out["tketen"] = species(self.state["tke"][1:-1, 1:-1], 1e-4)
        return out

    def empty_sav(self) -> dict:
        """Arrays for the MOLOCH variables of a SAV file."""
        out = {n: np.zeros_like(self.state[n], order="F")
               for n in ("u", "v", "w", "t", "pai", "qx", "ps")}
        if self.dims.ntr:
            out["trac"] = np.zeros_like(self.state["trac"], order="F")
        if "tke" in self.state:
            out["tke"] = np.zeros_like(self.state["tke"], order="F")
        return out

    @staticmethod
    def sav_ptrs_of(sav: dict) -> abi.mlc_sav_fields:
        f = abi.mlc_sav_fields()
        for n in abi.SAV_FIELDS:
            setattr(f, n, abi.dptr(sav.get(n)))
        return f

    @staticmethod
    def tend_ptrs_of(tend: dict) -> abi.mlc_tend_ptrs:
        t = abi.mlc_tend_ptrs()
        for n in abi.TEND_FIELDS:
            setattr(t, n, abi.dptr(tend.get(n)))
        return t

    def empty_state(self) -> dict:
        """Arrays shaped like the state, for downloads."""
        return {k: np.zeros_like(v, order="F") for k, v in self.state.items()}

    def copy_state(self) -> dict:
        return {k: np.array(v, order="F", copy=True) for k, v in self.state.items()}


def _zero_params() -> abi.mlc_params:
    """A parameter block with every field zero; build() sets each one."""
    return abi.mlc_params()


def build(nx: int, ny: int, kz: int, *, dx: float, dt: float, nsound: int, nadv: int = 1,
          moist: bool = False, seed: int = 0, hills=None, wind=10.0, jet: bool = False,
          theta_noise: float = 0.1, tracer: bool = False, precision: int = abi.MLC_PREC_FP64,
          name: str = "case", debug_level: int = 1, lrotllr: bool = False,
          apply_bdy: bool = True, spectral: bool = False, dtrad: float = 1800.0,
          lehmann: bool = True, ipptls: int | None = None, tke: bool = False,
          setup=None) -> Case:
    """Build one synthetic domain of nx x ny cross points and kz levels.
    `lehmann` picks Lehmann's relaxation weights (else exponential nudging
    with the reference's default strengths 3, 2, 1); `ipptls` the
    microphysics class of a moist domain (default 2; 3-5 add species that
    start at zero); `tke` runs the UW PBL's TKE (ibltyp = 2: a boundary-
    layer profile at the interfaces, advected by the step); `setup` is the
    backend of the static fields (default: the library's)."""
    su = setup or LibrarySetup()
    jx, iy = nx + 1, ny + 1
    if ipptls is None:
        ipptls = 2 if moist else 0
    nqx = {0: 2, 1: 2, 2: 5, 3: 5, 4: 7, 5: 10}[ipptls]
    ntr = 1 if tracer else 0
    dims = abi.mlc_dims(jx, iy, kz, nqx, ntr)
    p = _zero_params()
    p.dtsec, p.dx = float(dt), float(dx)
    p.mo_ztop, p.mo_h, p.mo_a0 = 25000.0, 8000.0, 0.0
    p.mo_nadv, p.mo_nsound = nadv, nsound
    p.mo_divdamp = p.mo_divfilter = p.mo_top_nudge = 1
    p.mo_spectral_nudge = 1 if spectral else 0
    p.dtrad = float(dtrad)
    p.do_apply_bdy = 1 if apply_bdy else 0
    p.lrotllr = 1 if lrotllr else 0
    p.ipptls = ipptls
    p.present_qc = 1 if moist else 0
    p.present_qi = 1 if moist else 0
    p.debug_level = debug_level
    p.precision = precision
    p.dtbdys = 6.0 * 3600.0
    p.bdy_use_lehmann = 1 if lehmann else 0
    p.ibltyp = 2 if tke else 1
    p.high_nudge, p.medium_nudge, p.low_nudge = 3.0, 2.0, 1.0
    p.nspgx, p.nspgd = su.nspg(jx, iy, dx / 1000.0, lehmann)

    # ---- terrain (geopotential) at cross / u / v positions on (jx, iy) ----
    xc = (np.arange(1, jx + 1) - 0.5) * dx
    xd = (np.arange(1, jx + 1) - 1.0) * dx
    yc = (np.arange(1, iy + 1) - 0.5) * dx
    yd = (np.arange(1, iy + 1) - 1.0) * dx
    if hills is None:
        hills = [(0.5 * nx * dx, 0.5 * ny * dx, 500.0)]

    def terrain(x, y):
        X, Y = np.meshgrid(x, y, indexing="ij")
        h = np.zeros_like(X)
        for (cx, cy, h0) in hills:
            r = np.hypot(X - cx, Y - cy)
            h += h0 * np.exp(-math.log(2.0) * (r / (10.0 * dx)) ** 2)
        return np.asfortranarray(h)

    h_cross = terrain(xc, yc)
    st = {}
    st["ht"] = np.asfortranarray(h_cross * GRAV)
    st["htu"] = np.asfortranarray(terrain(xd, yc) * GRAV)
    st["htv"] = np.asfortranarray(terrain(xc, yd) * GRAV)
    for n in ("msfu", "msfv", "msfx"):
        st[n] = np.ones((jx, iy), dtype=np.float64, order="F")
    st["ulat"] = np.full((jx, iy - 1), 45.0, order="F")
    st["vlat"] = np.full((jx - 1, iy), 45.0, order="F")
    st["rlat"] = np.full((iy,), 45.0, order="F")
    zita, zitah = np.zeros(kz + 1), np.zeros(kz)
    su.levels(kz, p.mo_ztop, zita, zitah)
    st["zita"], st["zitah"] = zita, zitah
    for n, shp in (("hx", (jx, iy - 1)), ("hy", (jx - 1, iy)), ("zeta", (jx - 1, iy - 1, kz)),
                   ("fmz", (jx - 1, iy - 1, kz)), ("rfmzu", (jx, iy - 1, kz)),
                   ("rfmzv", (jx - 1, iy, kz)), ("fmzf", (jx - 1, iy - 1, kz + 1)),
                   ("zetaf", (jx - 1, iy - 1, kz + 1)), ("dz", (jx - 1, iy - 1, kz))):
        st[n] = _f(shp)
    su.metric(dims, p, [st[n] for n in (
        "ht", "htu", "htv", "msfu", "msfv", "zita", "zitah", "hx", "hy", "zeta", "fmz",
        "rfmzu", "rfmzv", "fmzf", "zetaf", "dz")])
    st["hefc"] = _f((p.nspgx, kz))
    st["fcx"] = _f((p.nspgx,))
    st["tnudge"] = _f((kz,))
    st["ffilt"] = _f((kz,))
    st["gmeanz"] = _f((kz,))
    su.relaxation(dims, p, st["zeta"], st["hefc"], st["fcx"], st["tnudge"], st["ffilt"],
                  st["gmeanz"])
    for n, (lx, ly) in (("ibnd_cr", (0, 0)), ("ibnd_ud", (1, 0)), ("ibnd_vd", (0, 1))):
        st[n] = np.zeros((jx, iy), dtype=np.int32, order="F")
        su.boundaries(jx, iy, lx, ly, p.nspgx, p.nspgd, st[n])
    if spectral:
        st["cnudge"] = _f((kz,))
        su.spectral(p, kz, st["gmeanz"], st["cnudge"])

    # ---- atmosphere on cross points ----
    rng_n = 0
    cshape = (jx - 1, iy - 1, kz)
    zabs = np.asfortranarray(h_cross[: jx - 1, : iy - 1, None] + st["zeta"])
    t_isa, p_isa = isa(zabs)
    t_isa = np.asfortranarray(t_isa)
    _, ps_isa = isa(h_cross[: jx - 1, : iy - 1])
    ps_isa = np.asfortranarray(ps_isa)
    if moist:
        noise = splitmix64(seed * 7919 + 1, int(np.prod(cshape))).reshape(cshape, order="F")
        qv = 0.7 * su.pfwsat(t_isa, np.asfortranarray(p_isa)) * (1.0 + 0.1 * (noise - 0.5))
        qv = np.asfortranarray(qv)
    else:
        qv = np.full(cshape, 1.0e-8, order="F")
    pai = _f(cshape)
    su.paicompute(dims, p, ps_isa, st["zeta"], t_isa, qv, st["fmzf"], zita, pai)
    thv = t_isa * (1.0 + EP1 * qv) / pai
    noise = splitmix64(seed * 7919 + 2, int(np.prod(cshape))).reshape(cshape, order="F")
    inner = np.zeros(cshape, dtype=bool)
    inner[1:-1, 1:-1, :] = True
    thv = np.where(inner, thv + theta_noise * (2.0 * noise - 1.0), thv)
    t_b = np.asfortranarray(thv * pai / (1.0 + EP1 * qv))

    # winds: u on (jx, iy-1), v on (jx-1, iy)
    if jet:
        ly = (iy - 1) * dx
        prof = 15.0 * np.sin(math.pi * yc[: iy - 1] / ly)
        u_b = np.asfortranarray(np.broadcast_to(prof[None, :, None], (jx, iy - 1, kz)).copy())
    else:
        u_b = np.full((jx, iy - 1, kz), float(wind), order="F")
    v_b = _f((jx - 1, iy, kz))

    qx = _f((jx - 1, iy - 1, kz, nqx))
    qx[..., 0] = qv
    qc_b = None
    qi_b = None
    kk = np.arange(1, kz + 1)
    J, I = np.meshgrid(np.arange(1, jx), np.arange(1, iy), indexing="ij")
    if moist:
        cen = splitmix64(seed * 7919 + 3, 3)
        cj = 1 + p.nspgx + cen[0] * (nx - 2 * p.nspgx)
        ci = 1 + p.nspgx + cen[1] * (ny - 2 * p.nspgx)
        ck = kz - 4 - int(cen[2] * max(1, kz // 3))
        patch = np.exp(-((J - cj) ** 2 + (I - ci) ** 2)[..., None] / (2 * 5.0 ** 2)
                       - ((kk - ck) ** 2)[None, None, :] / (2 * 2.0 ** 2))
        qc_b = np.asfortranarray(1.0e-4 * patch)
        qi_b = _f(cshape)
        qx[..., 1] = qc_b
        # the classes with more species: graupel and hail in the same patch,
        # number concentrations (ipptls 5) above their floors
        if ipptls >= 4:
            qx[..., 5] = 5.0e-5 * patch
            qx[..., 6] = 2.0e-5 * patch
        if ipptls == 5:
            qx[..., 7] = 1.0e10 * (1.0 + patch)
            qx[..., 8] = 1.0e2 * (1.0 + patch)
            qx[..., 9] = 1.0e-2 * (1.0 + patch)
    trac = None
    chib = None
    if tracer:
        cj, ci, ck = 0.5 * (jx - 1) + 0.5, 0.5 * (iy - 1) + 0.5, kz // 2
        blob = np.exp(-((J - cj) ** 2 + (I - ci) ** 2)[..., None] / (2 * 5.0 ** 2)
                      - ((kk - ck) ** 2)[None, None, :] / (2 * 2.0 ** 2))
        trac = np.asfortranarray(blob[..., None])
        chib = np.asfortranarray(trac.copy())

    # ---- boundary data: b0 = b1 = initial fields ----
    bdy = {
        "xtb": (t_b, t_b), "xqb": (qv, qv), "xpaib": (pai, pai), "dub": (u_b, u_b),
        "dvb": (v_b, v_b), "xpsb": (ps_isa, ps_isa),
    }
    if moist:
        bdy["xlb"] = (qc_b, qc_b)
        bdy["xib"] = (qi_b, qi_b)
    if tracer:
        bdy["chib"] = (chib, chib)

    # ---- initial state from b0, Main/mod_init.F90:155-219 ----
    tvirt = np.asfortranarray(t_b * (1.0 + EP1 * qv))
    pres = np.asfortranarray(pai ** CPOVR * P00)
    rho = np.asfortranarray(pres / (RGAS * t_b))
    zk = st["zeta"][..., kz - 1]
    psa = np.asfortranarray(pres[..., kz - 1] * np.exp(GRAV * zk / (RGAS * tvirt[..., kz - 1])))
    state = {
        "u": np.array(u_b, order="F"), "v": np.array(v_b, order="F"),
        "w": _f((jx - 1, iy - 1, kz + 1)), "pai": np.array(pai, order="F"),
        "tetav": np.asfortranarray(tvirt / pai), "t": np.array(t_b, order="F"),
        "tvirt": tvirt, "ux": _f(cshape), "vx": _f(cshape), "p": pres, "rho": rho,
        "qsat": su.pfwsat(t_b, pres), "qx": qx, "ps": psa,
    }
    if tracer:
        state["trac"] = np.array(trac, order="F")
    if tke:
        # TKE at the interfaces (jx-1, iy-1, kz+1): a boundary-layer profile
        # decaying over 600 m above the ground, seeded +-10 % noise, over the
        # UW floor 1e-3 m2/s2
        zf = st["zetaf"]
        noise = splitmix64(seed * 7919 + 5, int(zf.size)).reshape(zf.shape, order="F")
        state["tke"] = np.asfortranarray(1.0e-3 + np.exp(-zf / 600.0) * (0.9 + 0.2 * noise))
    keep = {k: v for k, v in st.items()}
    case = Case(name=name, dims=dims, params=p, static=keep, state=state, bdy=bdy)
    return case


# ---- the configurations of the benchmark suite ---------------------------

def config0(nx=64, ny=64, kz=30, seed=0, **kw) -> Case:
    """Plain dry dynamics: 64x64x30, dx 12 km, dt 60 s, 3 substeps, hill 500 m,
    u = 10 m/s, theta noise +-0.1 K, one passive tracer blob."""
    return build(nx, ny, kz, dx=12000.0, dt=60.0, nsound=3, moist=False, seed=seed,
                 hills=[(0.5 * nx * 12000.0, 0.5 * ny * 12000.0, 500.0)], wind=10.0,
                 theta_noise=0.1, tracer=True, name=f"c0_{nx}x{ny}x{kz}", **kw)


def _moist(nx, ny, kz, seed, dx, dt, nsound, name, **kw) -> Case:
    r = splitmix64(seed * 104729 + 11, 9)
    hills = []
    for h in range(3):
        cx = (0.2 + 0.6 * r[3 * h]) * nx * dx
        cy = (0.2 + 0.6 * r[3 * h + 1]) * ny * dx
        hills.append((cx, cy, 200.0 + 1800.0 * r[3 * h + 2]))
    return build(nx, ny, kz, dx=dx, dt=dt, nsound=nsound, moist=True, seed=seed, hills=hills,
                 jet=True, theta_noise=0.1, tracer=False, name=name, **kw)


def config1(nx=512, ny=512, kz=41, seed=1, **kw) -> Case:
    """Moist convection-permitting: 512x512x41, dx 3 km, dt 20 s, 4 substeps,
    3 seeded hills of 200-2000 m, qv at 70% RH, a qc patch, u jet 15 sin(y)."""
    return _moist(nx, ny, kz, seed, 3000.0, 20.0, 4, f"c1_{nx}x{ny}x{kz}", **kw)


def log_uniform_int(u: float, lo: int, hi: int) -> int:
    return int(round(math.exp(math.log(lo) + u * (math.log(hi) - math.log(lo)))))


def config3_dims(m: int):
    """Extents of uneven-batch domain m: nx, ny log-uniform in 48-384
    (independently), kz from {23, 30, 41}."""
    r = splitmix64(3000 + m, 3)
    nx = log_uniform_int(float(r[0]), 48, 384)
    ny = log_uniform_int(float(r[1]), 48, 384)
    kz = (23, 30, 41)[min(2, int(r[2] * 3))]
    return nx, ny, kz


def config3_member(m: int, scale: float = 1.0, **kw) -> Case:
    """Uneven-batch domain m: the moist recipe at dx 12 km, dt 60 s, 3
    substeps with its own seed; `scale` shrinks the horizontal extents (for
    tests) with a floor of 24 cells."""
    nx, ny, kz = config3_dims(m)
    nx = max(24, int(round(nx * scale)))
    ny = max(24, int(round(ny * scale)))
    return _moist(nx, ny, kz, 3000 + m, 12000.0, 60.0, 3, f"c3_m{m}_{nx}x{ny}x{kz}", **kw)


def config4_shape(r: int, scale: float = 1.0):
    """(n, steps) of serving request r: nx = ny log-uniform in 32-512 (scaled
    by `scale`, floor 24 cells), steps uniform in 6-240."""
    u = splitmix64(4000 + r, 2)
    n = max(24, int(round(log_uniform_int(float(u[0]), 32, 512) * scale)))
    return n, 6 + min(234, int(u[1] * 235))


def config4_request(r: int, scale: float = 1.0, **kw):
    """Serving request r: (case, steps).  nx = ny log-uniform in 32-512,
    kz 30, steps uniform in 6-240, the moist recipe of the 3 km domain with
    the request's seed; `scale` shrinks the extents (floor 24 cells)."""
    n, steps = config4_shape(r, scale)
    return _moist(n, n, 30, 4000 + r, 3000.0, 20.0, 4, f"c4_r{r}_{n}", **kw), steps


def config2_member(m: int, nx=128, ny=128, kz=30, **kw) -> Case:
    """Ensemble member m: config-0 recipe, theta noise +-0.5 K, wind U(5, 20)."""
    wind = 5.0 + 15.0 * float(splitmix64(1000 + m, 1)[0])
    return build(nx, ny, kz, dx=12000.0, dt=60.0, nsound=3, moist=False, seed=m,
                 hills=[(0.5 * nx * 12000.0, 0.5 * ny * 12000.0, 500.0)], wind=wind,
                 theta_noise=0.5, tracer=True, name=f"c2_m{m}", **kw)
