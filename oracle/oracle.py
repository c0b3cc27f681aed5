"""TEST INFRASTRUCTURE ONLY: ctypes access to the CPU oracle.

The oracle is a C++ FP64 restatement of RegCM's MOLOCH step
(oracle/moloch_oracle.cpp) and of its setup routines (oracle/oracle_setup.cpp).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
as the checker; the product library never loads it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from regcm_gb300 import abi

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libmoloch_oracle.so"
_lib = None


def load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
        lib = C.CDLL(str(LIB))
        P = C.POINTER
        dp = P(C.c_double)
        lib.orc_create.restype = C.c_void_p
        lib.orc_create.argtypes = [P(abi.mlc_dims), P(abi.mlc_params)]
        lib.orc_destroy.argtypes = [C.c_void_p]
        lib.orc_bind_static.argtypes = [C.c_void_p, P(abi.mlc_static_ptrs)]
        lib.orc_set_state.argtypes = [C.c_void_p, P(abi.mlc_state_ptrs)]
        lib.orc_get_state.argtypes = [C.c_void_p, P(abi.mlc_state_ptrs)]
        lib.orc_set_boundary.argtypes = [C.c_void_p, P(abi.mlc_bdy_ptrs), C.c_double, C.c_double]
        lib.orc_step.argtypes = [C.c_void_p, C.c_int, P(abi.mlc_diag)]
        lib.orc_step_dynamics.argtypes = [C.c_void_p]
        lib.orc_set_tendencies.argtypes = [C.c_void_p, P(abi.mlc_tend_ptrs)]
        lib.orc_step_finish.argtypes = [C.c_void_p, P(abi.mlc_diag)]
        lib.orc_restart_state.argtypes = [P(abi.mlc_dims), P(abi.mlc_sav_fields), P(abi.mlc_state_ptrs)]
        lib.orc_sound_only.argtypes = [C.c_void_p]
        lib.orc_get_work.argtypes = [C.c_void_p, C.c_int, dp]
        lib.orc_setup_levels.argtypes = [C.c_int, C.c_double, dp, dp]
        lib.orc_setup_metric.argtypes = [P(abi.mlc_dims), P(abi.mlc_params)] + [dp] * 16
        lib.orc_relax_coefficients.argtypes = [C.c_int, C.c_double, C.c_double, dp]
        lib.orc_setup_relaxation.argtypes = [P(abi.mlc_dims), P(abi.mlc_params), dp, dp, dp, dp,
                                             dp, P(C.c_int)]
        lib.orc_setup_boundaries.argtypes = [C.c_int] * 6 + [P(C.c_int32)]
        lib.orc_setup_spectral.argtypes = [P(abi.mlc_params), C.c_int, dp, dp]
        lib.orc_paicompute.argtypes = [P(abi.mlc_dims)] + [dp] * 5 + [C.c_double, dp]
        lib.orc_setup_nspg.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int,
                                       P(C.c_int), P(C.c_int)]
        lib.orc_gmeanz.argtypes = [P(abi.mlc_dims), dp, dp]
        lib.orc_exponential_nudging.argtypes = [C.c_int] + [C.c_double] * 4 + [dp]
        lib.orc_pfwsat.argtypes = [C.c_size_t, dp, dp, dp]
        lib.orc_set_threads.argtypes = [C.c_int]
        _lib = lib
    return _lib


class Oracle:
    """One domain stepped by the CPU oracle."""

    def __init__(self, case):
        self.case = case
        self.lib = load()
        self.h = self.lib.orc_create(C.byref(case.dims), C.byref(case.params))
        if not self.h:
            raise RuntimeError("orc_create rejected the domain")
        self._sp = case.static_ptrs()
        assert self.lib.orc_bind_static(self.h, C.byref(self._sp)) == 0
        self._st = case.state_ptrs()
        assert self.lib.orc_set_state(self.h, C.byref(self._st)) == 0
        self._bp = case.bdy_ptrs()
        if case.params.do_apply_bdy:
            assert self.lib.orc_set_boundary(self.h, C.byref(self._bp), case.xbctime,
                                             case.params.dtbdys) == 0

    def set_boundary(self, bdy_ptrs, xbctime: float, dtbdys: float):
        self._bp = bdy_ptrs
        assert self.lib.orc_set_boundary(self.h, C.byref(bdy_ptrs), xbctime, dtbdys) == 0

    def step(self, n=1):
        d = abi.mlc_diag()
        st = self.lib.orc_step(self.h, n, C.byref(d))
        return st, d

    def step_dynamics(self):
        return self.lib.orc_step_dynamics(self.h)

    def set_tendencies(self, tend_ptrs):
        return self.lib.orc_set_tendencies(self.h, C.byref(tend_ptrs))

    def step_finish(self):
        d = abi.mlc_diag()
        st = self.lib.orc_step_finish(self.h, C.byref(d))
        return st, d

    def sound_only(self):
        self.lib.orc_sound_only(self.h)

    def state(self) -> dict:
        out = self.case.empty_state()
        sp = self.case.state_ptrs_of(out)
        self.lib.orc_get_state(self.h, C.byref(sp))
        return out

    def work(self, which: int, shape):
        a = np.zeros(shape, order="F")
        self.lib.orc_get_work(self.h, which, abi.dptr(a))
        return a

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def set_threads(n: int) -> int:
    """Threads of the oracle's OpenMP loops; returns the count in effect."""
    return int(load().orc_set_threads(int(n)))


class OracleSetup:
    """The oracle's restatement of RegCM's setup routines behind the
    interface of regcm_gb300.case's setup backends, so a case can be built
    without loading the GPU library (the CPU reference timing)."""

    def __init__(self):
        self.lib = load()

    @staticmethod
    def _ok(st, where):
        if st != 0:
            raise RuntimeError(f"{where}: status {st}")

    def nspg(self, jx, iy, ds_km, lehmann=True):
        gx, gd = C.c_int(), C.c_int()
        self._ok(self.lib.orc_setup_nspg(jx, iy, ds_km, 1 if lehmann else 0, 0, 0,
                                         C.byref(gx), C.byref(gd)), "orc_setup_nspg")
        return gx.value, gd.value

    def levels(self, kz, ztop, zita, zitah):
        self._ok(self.lib.orc_setup_levels(kz, ztop, abi.dptr(zita), abi.dptr(zitah)),
                 "orc_setup_levels")

    def metric(self, dims, params, arrays):
        self._ok(self.lib.orc_setup_metric(C.byref(dims), C.byref(params),
                                           *[abi.dptr(a) for a in arrays]), "orc_setup_metric")

    def relaxation(self, dims, params, zeta, hefc, fcx, tnudge, ffilt, gmeanz):
        nz = C.c_int()
        self._ok(self.lib.orc_setup_relaxation(C.byref(dims), C.byref(params), abi.dptr(zeta),
                                               abi.dptr(hefc), abi.dptr(fcx), abi.dptr(tnudge),
                                               abi.dptr(ffilt), C.byref(nz)),
                 "orc_setup_relaxation")
        params.nztop = nz.value
        self._ok(self.lib.orc_gmeanz(C.byref(dims), abi.dptr(zeta), abi.dptr(gmeanz)), "orc_gmeanz")

    def boundaries(self, jx, iy, lx, ly, nspgx, nspgd, out):
        self._ok(self.lib.orc_setup_boundaries(jx, iy, lx, ly, nspgx, nspgd, abi.iptr(out)),
                 "orc_setup_boundaries")

    def spectral(self, params, kz, gmeanz, cnudge):
        self._ok(self.lib.orc_setup_spectral(C.byref(params), kz, abi.dptr(gmeanz),
                                             abi.dptr(cnudge)), "orc_setup_spectral")

    def paicompute(self, dims, params, ps, zeta, t, qv, fmzf, zita, pai):
        self._ok(self.lib.orc_paicompute(C.byref(dims), abi.dptr(ps), abi.dptr(zeta), abi.dptr(t),
                                         abi.dptr(qv), abi.dptr(fmzf), float(zita[dims.kz - 1]),
                                         abi.dptr(pai)), "orc_paicompute")

    def pfwsat(self, t, p):
        t = np.asfortranarray(t, dtype=np.float64)
        p = np.asfortranarray(p, dtype=np.float64)
        out = np.empty_like(t, order="F")
        self._ok(self.lib.orc_pfwsat(t.size, abi.dptr(t), abi.dptr(p), abi.dptr(out)), "orc_pfwsat")
        return out
