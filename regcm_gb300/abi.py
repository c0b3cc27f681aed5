"""ctypes mirror of include/moloch_gb300.h and include/moloch_gb300_setup.h.

The structures here are field-for-field copies of the C declarations; the
library handle is loaded from the in-tree build (``regcm_gb300/_build``) and
there is no fallback: a missing or stale build raises ``MolochLibraryError``.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
BUILD_DIR = PKG_DIR / "_build"
LIB_NAME = "libmoloch_gb300.so"

MLC_OK = 0
MLC_ERR_INVALID = -1
MLC_ERR_UNSUPPORTED = -2
MLC_ERR_CUDA = -3
MLC_ERR_NOMEM = -4
MLC_ERR_STATE = -5
MLC_ERR_NONFINITE = -6
MLC_ERR_NODEVICE = -7
MLC_ERR_BUDGET = -8
MLC_ERR_TOO_LARGE = -9

MLC_PREC_FP64 = 0
MLC_PREC_MIXED = 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class MolochLibraryError(RuntimeError):
    """The compiled library is missing or does not export what is needed."""


class mlc_dims(C.Structure):
    _fields_ = [("jx", C.c_int32), ("iy", C.c_int32), ("kz", C.c_int32),
                ("nqx", C.c_int32), ("ntr", C.c_int32)]

    def as_tuple(self):
        return (self.jx, self.iy, self.kz, self.nqx, self.ntr)


class mlc_params(C.Structure):
    _fields_ = [("dtsec", C.c_double), ("dx", C.c_double), ("mo_ztop", C.c_double),
                ("mo_h", C.c_double), ("mo_a0", C.c_double), ("dtbdys", C.c_double),
                ("mo_nadv", C.c_int32), ("mo_nsound", C.c_int32),
                ("mo_divdamp", C.c_int32), ("mo_divfilter", C.c_int32),
                ("mo_top_nudge", C.c_int32), ("mo_spectral_nudge", C.c_int32),
                ("do_apply_bdy", C.c_int32), ("lrotllr", C.c_int32),
                ("ipptls", C.c_int32), ("present_qc", C.c_int32), ("present_qi", C.c_int32),
                ("nspgx", C.c_int32), ("nspgd", C.c_int32), ("nztop", C.c_int32),
                ("debug_level", C.c_int32), ("precision", C.c_int32), ("dtrad", C.c_double),
                ("bdy_use_lehmann", C.c_int32), ("ibltyp", C.c_int32), ("high_nudge", C.c_double),
                ("medium_nudge", C.c_double), ("low_nudge", C.c_double)]


STATIC_FIELDS = ["msfu", "msfv", "msfx", "ulat", "vlat", "rlat", "hx", "hy", "fmz", "fmzf",
                 "rfmzu", "rfmzv", "zeta", "dz", "zita", "zitah", "ffilt", "hefc", "fcx",
                 "tnudge"]
IBND_FIELDS = ["ibnd_cr", "ibnd_ud", "ibnd_vd"]


# read only when mo_spectral_nudge is set
SPECTRAL_FIELDS = ["cnudge"]


class mlc_static_ptrs(C.Structure):
    _fields_ = ([(n, _dp) for n in STATIC_FIELDS] + [(n, _ip) for n in IBND_FIELDS] +
                [(n, _dp) for n in SPECTRAL_FIELDS])


STATE_FIELDS = ["u", "v", "w", "pai", "tetav", "t", "tvirt", "ux", "vx", "p", "rho", "qsat",
                "qx", "trac", "ps", "tke"]


class mlc_state_ptrs(C.Structure):
    _fields_ = [(n, _dp) for n in STATE_FIELDS]


BDY_FIELDS = ["xtb", "xqb", "xpaib", "xlb", "xib", "dub", "dvb", "xpsb", "chib"]


class mlc_bdy_ptrs(C.Structure):
    _fields_ = [(n, _dp * 2) for n in BDY_FIELDS]


# physics tendencies on the interior jci x ici, (jx-3, iy-3, kz[, n])
TEND_FIELDS = ["tten", "uten", "vten", "qxten", "chiten", "tketen"]


class mlc_tend_ptrs(C.Structure):
    _fields_ = [(n, _dp) for n in TEND_FIELDS]


# the MOLOCH variables of a SAV restart file
SAV_FIELDS = ["u", "v", "w", "t", "pai", "qx", "ps", "trac", "tke"]


class mlc_sav_fields(C.Structure):
    _fields_ = [(n, _dp) for n in SAV_FIELDS]


class mlc_tune_report(C.Structure):
    _fields_ = [("col_x", C.c_int32), ("col_y", C.c_int32), ("solve_x", C.c_int32),
                ("solve_y", C.c_int32), ("vert_x", C.c_int32), ("vert_y", C.c_int32),
                ("htile", C.c_int32), ("ms_fixed", C.c_double), ("ms_tuned", C.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class mlc_diag(C.Structure):
    _fields_ = [("ps_max", C.c_double), ("ps_min", C.c_double), ("nonfinite", C.c_int32),
                ("steps_done", C.c_int32), ("drymass", C.c_double), ("dryadv", C.c_double),
                ("qmass", C.c_double), ("qadv", C.c_double), ("xbctime", C.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


def dptr(a):
    """double* of a C-contiguous float64 array (or NULL for None)."""
    if a is None:
        return _dp()
    if a.dtype != np.float64 or not a.flags["F_CONTIGUOUS"]:
        raise TypeError("expected a Fortran-ordered float64 array")
    return a.ctypes.data_as(_dp)


def iptr(a):
    if a is None:
        return _ip()
    if a.dtype != np.int32 or not a.flags["F_CONTIGUOUS"]:
        raise TypeError("expected a Fortran-ordered int32 array")
    return a.ctypes.data_as(_ip)


_LIB = None


def _declare(lib):
    P = C.POINTER
    sigs = {
        "mlc_default_params": (None, [P(mlc_params)]),
        "mlc_create": (C.c_int, [P(mlc_dims), P(mlc_params), P(C.c_void_p)]),
        "mlc_bind_static": (C.c_int, [C.c_void_p, P(mlc_static_ptrs)]),
        "mlc_upload_state": (C.c_int, [C.c_void_p, P(mlc_state_ptrs)]),
        "mlc_download_state": (C.c_int, [C.c_void_p, P(mlc_state_ptrs)]),
        "mlc_set_boundary": (C.c_int, [C.c_void_p, P(mlc_bdy_ptrs), C.c_double, C.c_double]),
        "mlc_step": (C.c_int, [C.c_void_p, C.c_int, P(mlc_diag)]),
        "mlc_destroy": (None, [C.c_void_p]),
        "mlc_strerror": (C.c_char_p, [C.c_int]),
        "mlc_last_error": (C.c_char_p, []),
        "mlc_footprint_bytes": (C.c_size_t, [P(mlc_dims), C.c_int]),
        "mlc_setup_levels": (C.c_int, [C.c_int, C.c_double, _dp, _dp]),
        "mlc_setup_nspg": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int,
                                     P(C.c_int), P(C.c_int)]),
        "mlc_setup_metric": (C.c_int, [P(mlc_dims), P(mlc_params)] + [_dp] * 16),
        "mlc_relax_coefficients": (C.c_int, [C.c_int, C.c_double, C.c_double, _dp]),
        "mlc_exponential_nudging": (C.c_int, [C.c_int] + [C.c_double] * 4 + [_dp]),
        "mlc_setup_relaxation": (C.c_int, [P(mlc_dims), P(mlc_params), _dp, _dp, _dp, _dp, _dp,
                                           _dp]),
        "mlc_setup_boundaries": (C.c_int, [C.c_int] * 6 + [_ip]),
        "mlc_setup_spectral": (C.c_int, [P(mlc_params), C.c_int, _dp, _dp]),
        "mlc_paicompute": (C.c_int, [P(mlc_dims), P(mlc_params)] + [_dp] * 7),
        "mlc_pfwsat": (C.c_int, [C.c_size_t, _dp, _dp, _dp]),
        "mlc_create_batch": (C.c_int, [P(mlc_dims), P(mlc_params), C.c_int, P(C.c_void_p)]),
        "mlc_members": (C.c_int, [C.c_void_p]),
        "mlc_member_bind_static": (C.c_int, [C.c_void_p, C.c_int, P(mlc_static_ptrs)]),
        "mlc_member_upload_state": (C.c_int, [C.c_void_p, C.c_int, P(mlc_state_ptrs)]),
        "mlc_member_download_state": (C.c_int, [C.c_void_p, C.c_int, P(mlc_state_ptrs)]),
        "mlc_member_set_boundary": (C.c_int, [C.c_void_p, C.c_int, P(mlc_bdy_ptrs), C.c_double,
                                              C.c_double]),
        "mlc_step_batch": (C.c_int, [C.c_void_p, C.c_int, P(mlc_diag)]),
        "mlc_launches_per_step": (C.c_int, [C.c_void_p]),
        "mlc_set_graphs": (C.c_int, [C.c_void_p, C.c_int]),
        "mlc_fp64_peak": (C.c_int, [C.c_int, P(C.c_double)]),
        "mlc_set_solve_precision": (C.c_int, [C.c_void_p, C.c_int]),
        "mlc_member_test_stall": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
        "mlc_autotune": (C.c_int, [C.c_void_p, C.c_int, P(mlc_tune_report)]),
        "mlc_set_launch_shapes": (C.c_int, [C.c_void_p, P(mlc_tune_report)]),
        "mlc_create_multi": (C.c_int, [P(mlc_dims), P(mlc_params), C.c_int, P(C.c_void_p)]),
        "mlc_create_pool": (C.c_int, [P(mlc_params), C.c_int, C.c_size_t, P(C.c_void_p)]),
        "mlc_pool_add": (C.c_int, [C.c_void_p, P(mlc_dims), P(C.c_int)]),
        "mlc_pool_remove": (C.c_int, [C.c_void_p, C.c_int]),
        "mlc_pool_bytes": (C.c_size_t, [C.c_void_p]),
        "mlc_member_footprint": (C.c_size_t, [P(mlc_dims), P(mlc_params)]),
        "mlc_sav_write": (C.c_int, [C.c_char_p, P(mlc_dims), P(mlc_sav_fields), C.c_char_p,
                                    C.c_char_p]),
        "mlc_sav_read": (C.c_int, [C.c_char_p, P(mlc_dims), P(mlc_sav_fields), C.c_char_p,
                                   C.c_size_t]),
        "mlc_sav_restart_state": (C.c_int, [P(mlc_dims), P(mlc_sav_fields), P(mlc_state_ptrs)]),
        "mlc_member_write_sav": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p, C.c_char_p, C.c_char_p]),
        "mlc_member_read_sav": (C.c_int, [C.c_void_p, C.c_int, C.c_char_p]),
        "mlc_step_dynamics": (C.c_int, [C.c_void_p]),
        "mlc_member_set_tendencies": (C.c_int, [C.c_void_p, C.c_int, P(mlc_tend_ptrs)]),
        "mlc_step_finish": (C.c_int, [C.c_void_p, P(mlc_diag)]),
    }
    for name, (res, args) in sigs.items():
        try:
            fn = getattr(lib, name)
        except AttributeError as e:
            raise MolochLibraryError(f"{LIB_NAME} does not export {name}") from e
        fn.restype = res
        fn.argtypes = args
    return lib


def lib_path() -> Path:
    return Path(os.environ.get("MOLOCH_GB300_LIB", BUILD_DIR / LIB_NAME))


def load():
    """Load the in-tree CUDA library; raise when it has not been built."""
    global _LIB
    if _LIB is None:
        path = lib_path()
        if not path.exists():
            raise MolochLibraryError(
                f"{path} not found: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        _LIB = _declare(C.CDLL(str(path)))
    return _LIB


class MolochError(RuntimeError):
    """A negative status from the library (the reference calls fatal())."""

    def __init__(self, status: int, where: str):
        self.status = status
        msg = load().mlc_strerror(status).decode()
        if status in (MLC_ERR_CUDA, MLC_ERR_NOMEM):
            msg += f" [{load().mlc_last_error().decode()}]"
        super().__init__(f"{where}: {msg} (status {status})")


def check(status: int, where: str):
    if status != MLC_OK:
        raise MolochError(status, where)
    return status
