"""Host mirror of RegCM's MOLOCH module interface over the C ABI.

RegCM's module exposes three argument-less procedures,
``public :: allocate_moloch, init_moloch, moloch`` (Main/mod_moloch.F90:127),
called from param (Main/mod_params.F90:1979-1980), init
(Main/mod_init.F90:922-923) and once per model step from RCM_run
(Main/mod_regcm_interface.F90:274-275).  ``MolochDomain`` keeps the same three
phases with the state passed explicitly, and the module-level functions of the
same names drive one default domain the way the Fortran globals do.  Failures
raise ``MolochError`` where the reference calls fatal(); a non-finite surface
pressure raises ``CFLViolation`` ("CFL VIOLATION", Main/mod_moloch.F90:407-422).
There is no CPU fallback: without the compiled library or a GPU every call
raises.
"""
from __future__ import annotations

import ctypes as C

from . import abi
from .abi import MolochError

__all__ = ["MolochDomain", "MolochBatch", "MolochPool", "MolochError", "CFLViolation", "allocate_moloch",
           "init_moloch", "moloch"]


class CFLViolation(MolochError):
    """Surface pressure became NaN or Inf (the reference stops the model)."""


class MolochDomain:
    """One MOLOCH domain resident on the GPU."""

    def __init__(self, dims: abi.mlc_dims, params: abi.mlc_params):
        self.lib = abi.load()
        self.dims = dims
        self.params = params
        self._ctx = C.c_void_p()
        abi.check(self.lib.mlc_create(C.byref(dims), C.byref(params), C.byref(self._ctx)),
                  "allocate_moloch")
        self._keep = []

    # -- init_moloch -------------------------------------------------------
    def bind_static(self, static_ptrs: abi.mlc_static_ptrs):
        self._keep.append(static_ptrs)
        abi.check(self.lib.mlc_bind_static(self._ctx, C.byref(static_ptrs)), "init_moloch(static)")

    def upload(self, state_ptrs: abi.mlc_state_ptrs):
        abi.check(self.lib.mlc_upload_state(self._ctx, C.byref(state_ptrs)), "init_moloch(state)")

    def set_boundary(self, bdy_ptrs: abi.mlc_bdy_ptrs, xbctime: float, dtbdys: float):
        self._keep.append(bdy_ptrs)
        abi.check(self.lib.mlc_set_boundary(self._ctx, C.byref(bdy_ptrs), xbctime, dtbdys),
                  "bdyin")

    # -- moloch ------------------------------------------------------------
    def step(self, nsteps: int = 1) -> abi.mlc_diag:
        d = abi.mlc_diag()
        st = self.lib.mlc_step(self._ctx, nsteps, C.byref(d))
        if st == abi.MLC_ERR_NONFINITE:
            raise CFLViolation(st, "moloch")
        abi.check(st, "moloch")
        return d

    def download(self, state_ptrs: abi.mlc_state_ptrs):
        abi.check(self.lib.mlc_download_state(self._ctx, C.byref(state_ptrs)), "download")

    # -- SAV restart files (Main/mod_savefile.F90, Main/mod_init.F90) ------
    def write_sav(self, path: str, idatex: str | None = None, calendar: str | None = None):
        """Snapshot the device state into the MOLOCH variables of a SAV file."""
        enc = lambda x: None if x is None else x.encode()
        abi.check(self.lib.mlc_member_write_sav(self._ctx, 0, str(path).encode(), enc(idatex),
                                                enc(calendar)), "write_savefile")

    def read_sav(self, path: str):
        """Restart the device state from a SAV file (read_savefile + init)."""
        abi.check(self.lib.mlc_member_read_sav(self._ctx, 0, str(path).encode()), "read_savefile")

    # -- the step split at the physics (Main/mod_moloch.F90:354-376) --------
    def step_dynamics(self):
        """Dynamics, boundary and mkslice's edits: the state the physics reads."""
        abi.check(self.lib.mlc_step_dynamics(self._ctx), "moloch(dynamics)")

    def set_tendencies(self, tend_ptrs: abi.mlc_tend_ptrs):
        """The physics' tendencies for the open step (NULL fields are zero)."""
        abi.check(self.lib.mlc_member_set_tendencies(self._ctx, 0, C.byref(tend_ptrs)),
                  "physics tendencies")

    def step_finish(self) -> abi.mlc_diag:
        """status_update with the tendencies, mass budget and ps check."""
        d = abi.mlc_diag()
        st = self.lib.mlc_step_finish(self._ctx, C.byref(d))
        if st == abi.MLC_ERR_NONFINITE:
            raise CFLViolation(st, "moloch")
        abi.check(st, "moloch(status_update)")
        return d

    def launches_per_step(self) -> int:
        return self.lib.mlc_launches_per_step(self._ctx)

    def set_graphs(self, on: bool):
        abi.check(self.lib.mlc_set_graphs(self._ctx, 1 if on else 0), "mlc_set_graphs")

    def set_solve_precision(self, df_recurrence: bool):
        """Mixed precision: the w-Exner recurrence in double-float (True,
        the default) or FP32 (False)."""
        abi.check(self.lib.mlc_set_solve_precision(self._ctx, 1 if df_recurrence else 0),
                  "mlc_set_solve_precision")

    def autotune(self, steps_per_trial: int = 2) -> dict:
        return _autotune(self.lib, self._ctx, steps_per_trial)

    def set_launch_shapes(self, shapes: dict):
        """Apply launch shapes (a dict as autotune returns; ms fields ignored)."""
        _set_launch_shapes(self.lib, self._ctx, shapes)

    def close(self):
        if self._ctx:
            self.lib.mlc_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _autotune(lib, ctx, steps_per_trial):
    rep = abi.mlc_tune_report()
    abi.check(lib.mlc_autotune(ctx, steps_per_trial, C.byref(rep)), "autotune")
    return rep.as_dict()


# the fixed configuration the autotuner compares against
DEFAULT_SHAPES = {"col_x": 32, "col_y": 4, "solve_x": 32, "solve_y": 2, "vert_x": 32, "vert_y": 4,
                  "htile": 0}


def _set_launch_shapes(lib, ctx, shapes):
    rep = abi.mlc_tune_report()
    for n, _ in rep._fields_:
        if not n.startswith("ms_"):
            setattr(rep, n, shapes.get(n, DEFAULT_SHAPES[n]))
    abi.check(lib.mlc_set_launch_shapes(ctx, C.byref(rep)), "mlc_set_launch_shapes")


_SHARED_PARAMS = ("dtsec", "dx", "mo_ztop", "mo_h", "mo_a0", "mo_nadv", "mo_nsound",
                  "mo_divdamp", "mo_divfilter", "mo_top_nudge", "mo_spectral_nudge",
                  "do_apply_bdy", "lrotllr", "ipptls", "present_qc", "present_qi", "nspgx",
                  "nspgd", "debug_level", "precision", "dtrad", "bdy_use_lehmann", "ibltyp",
                  "high_nudge", "medium_nudge", "low_nudge")


def _same_params(a: abi.mlc_params, b: abi.mlc_params) -> bool:
    """Members of one context share every parameter but the per-domain ones
    (nztop follows each domain's levels, dtbdys comes with its boundary)."""
    return all(getattr(a, f) == getattr(b, f) for f in _SHARED_PARAMS)


def _load_member(lib, ctx, m, c, keep):
    sp, bp = c.static_ptrs(), c.bdy_ptrs()
    keep += [sp, bp]
    abi.check(lib.mlc_member_bind_static(ctx, m, C.byref(sp)), "init_moloch")
    abi.check(lib.mlc_member_upload_state(ctx, m, C.byref(c.state_ptrs())), "init_moloch(state)")
    if c.params.do_apply_bdy:
        abi.check(lib.mlc_member_set_boundary(ctx, m, C.byref(bp), c.xbctime, c.params.dtbdys),
                  "bdyin")


class MolochBatch:
    """Domains advanced by the same kernel launches (one launch per kernel
    stage for all members).  Members share the run parameters; their extents
    may differ (an uneven batch), in which case each launch covers the
    largest member and smaller members' blocks return at once."""

    def __init__(self, cases):
        if not cases:
            raise ValueError("empty ensemble")
        self.lib = abi.load()
        self.cases = list(cases)
        c0 = self.cases[0]
        for c in self.cases[1:]:
            if not _same_params(c.params, c0.params):
                raise ValueError(f"member {c.name} does not share the run parameters of {c0.name}")
        self.dims, self.params = c0.dims, c0.params
        self._ctx = C.c_void_p()
        n = len(self.cases)
        same = all(tuple(c.dims.as_tuple()) == tuple(c0.dims.as_tuple()) for c in self.cases)
        if same:
            st = self.lib.mlc_create_batch(C.byref(c0.dims), C.byref(c0.params), n,
                                           C.byref(self._ctx))
        else:
            arr = (abi.mlc_dims * n)(*[c.dims for c in self.cases])
            st = self.lib.mlc_create_multi(arr, C.byref(c0.params), n, C.byref(self._ctx))
        abi.check(st, "allocate_moloch(batch)")
        self._keep = []
        for m, c in enumerate(self.cases):
            _load_member(self.lib, self._ctx, m, c, self._keep)

    @classmethod
    def lazy(cls, dims, params, make):
        """A batch of len(dims) members whose cases are built one at a time by
        make(m), loaded and dropped (bounded host memory for large batches).
        ``cases`` holds None for every member."""
        self = cls.__new__(cls)
        self.lib = abi.load()
        n = len(dims)
        self.cases = [None] * n
        self.dims, self.params = dims[0], params
        self._ctx = C.c_void_p()
        arr = (abi.mlc_dims * n)(*dims)
        abi.check(self.lib.mlc_create_multi(arr, C.byref(params), n, C.byref(self._ctx)),
                  "allocate_moloch(batch)")
        self._keep = []
        for m in range(n):
            c = make(m)
            if c.dims.as_tuple() != dims[m].as_tuple() or not _same_params(c.params, params):
                raise ValueError(f"member {m} does not match its declared extents/parameters")
            keep = []
            _load_member(self.lib, self._ctx, m, c, keep)
        return self

    @property
    def nmem(self) -> int:
        return len(self.cases)

    def step(self, nsteps: int = 1):
        diags = (abi.mlc_diag * self.nmem)()
        st = self.lib.mlc_step_batch(self._ctx, nsteps, diags)
        if st == abi.MLC_ERR_NONFINITE:
            raise CFLViolation(st, "moloch(batch)")
        abi.check(st, "moloch(batch)")
        return list(diags)

    def step_timed(self, nsteps: int = 1) -> float:
        """Steps every member; returns the device milliseconds of the steps."""
        ms = C.c_float()
        d = abi.mlc_diag()
        abi.check(self.lib.mlc_step_timed(self._ctx, nsteps, C.byref(d), C.byref(ms)), "moloch")
        return ms.value

    def download(self, m: int, state_ptrs: abi.mlc_state_ptrs):
        abi.check(self.lib.mlc_member_download_state(self._ctx, m, C.byref(state_ptrs)),
                  "download")

    def step_dynamics(self):
        abi.check(self.lib.mlc_step_dynamics(self._ctx), "moloch(dynamics)")

    def set_tendencies(self, m: int, tend_ptrs: abi.mlc_tend_ptrs):
        abi.check(self.lib.mlc_member_set_tendencies(self._ctx, m, C.byref(tend_ptrs)),
                  "physics tendencies")

    def step_finish(self):
        diags = (abi.mlc_diag * self.nmem)()
        st = self.lib.mlc_step_finish(self._ctx, diags)
        if st == abi.MLC_ERR_NONFINITE:
            raise CFLViolation(st, "moloch(batch)")
        abi.check(st, "moloch(status_update)")
        return list(diags)

    def upload(self, m: int, state_ptrs: abi.mlc_state_ptrs):
        abi.check(self.lib.mlc_member_upload_state(self._ctx, m, C.byref(state_ptrs)), "upload")

    def set_graphs(self, on: bool):
        abi.check(self.lib.mlc_set_graphs(self._ctx, 1 if on else 0), "mlc_set_graphs")

    def set_solve_precision(self, df_recurrence: bool):
        """Mixed precision: the w-Exner recurrence in double-float (True,
        the default) or FP32 (False)."""
        abi.check(self.lib.mlc_set_solve_precision(self._ctx, 1 if df_recurrence else 0),
                  "mlc_set_solve_precision")

    def launches_per_step(self) -> int:
        return self.lib.mlc_launches_per_step(self._ctx)

    def autotune(self, steps_per_trial: int = 2) -> dict:
        return _autotune(self.lib, self._ctx, steps_per_trial)

    def set_launch_shapes(self, shapes: dict):
        """Apply launch shapes (a dict as autotune returns; ms fields ignored)."""
        _set_launch_shapes(self.lib, self._ctx, shapes)

    def close(self):
        if self._ctx:
            self.lib.mlc_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MolochPool:
    """A serving pool: `capacity` member slots whose domains join and leave
    between steps (continuous batching), under a bound on the device bytes
    all member arenas hold.  ``join`` returns the slot or None when the
    budget or the slots are exhausted."""

    def __init__(self, params: abi.mlc_params, capacity: int, budget_bytes: int = 0):
        self.lib = abi.load()
        self.params = params
        self._ctx = C.c_void_p()
        abi.check(self.lib.mlc_create_pool(C.byref(params), capacity, budget_bytes,
                                           C.byref(self._ctx)), "mlc_create_pool")
        self.capacity = capacity
        self.cases = {}
        self._keep = {}

    def footprint(self, dims: abi.mlc_dims) -> int:
        return self.lib.mlc_member_footprint(C.byref(dims), C.byref(self.params))

    def bytes_in_use(self) -> int:
        return self.lib.mlc_pool_bytes(self._ctx)

    def join(self, case):
        if not _same_params(case.params, self.params):
            raise ValueError(f"{case.name} does not share the pool's run parameters")
        slot = C.c_int(-1)
        st = self.lib.mlc_pool_add(self._ctx, C.byref(case.dims), C.byref(slot))
        if st == abi.MLC_ERR_BUDGET:
            return None
        abi.check(st, "mlc_pool_add")
        keep = []
        try:
            _load_member(self.lib, self._ctx, slot.value, case, keep)
        except Exception:
            self.lib.mlc_pool_remove(self._ctx, slot.value)
            raise
        # the uploads are synchronous: the pool keeps the member's extents,
        # not its host arrays
        self.cases[slot.value] = case.dims
        self._keep[slot.value] = keep
        return slot.value

    def leave(self, slot: int):
        abi.check(self.lib.mlc_pool_remove(self._ctx, slot), "mlc_pool_remove")
        self.cases.pop(slot, None)
        self._keep.pop(slot, None)

    def step(self, nsteps: int = 1):
        diags = (abi.mlc_diag * self.capacity)()
        st = self.lib.mlc_step_batch(self._ctx, nsteps, diags)
        if st == abi.MLC_ERR_NONFINITE:
            raise CFLViolation(st, "moloch(pool)")
        abi.check(st, "moloch(pool)")
        return list(diags)

    def download(self, slot: int, state_ptrs: abi.mlc_state_ptrs):
        abi.check(self.lib.mlc_member_download_state(self._ctx, slot, C.byref(state_ptrs)),
                  "download")

    def launches_per_step(self) -> int:
        return self.lib.mlc_launches_per_step(self._ctx)

    def close(self):
        if self._ctx:
            self.lib.mlc_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def domain_from_case(case) -> MolochDomain:
    """allocate_moloch + init_moloch for a synthetic ``Case``."""
    dom = MolochDomain(case.dims, case.params)
    dom.bind_static(case.static_ptrs())
    dom.upload(case.state_ptrs())
    if case.params.do_apply_bdy:
        dom.set_boundary(case.bdy_ptrs(), case.xbctime, case.params.dtbdys)
    dom._case = case
    return dom


# ---- module-level entry points with the reference's names -----------------
_default: MolochDomain | None = None
_default_case = None


def allocate_moloch(case) -> MolochDomain:
    """Main/mod_moloch.F90:159-199: create the default domain for `case`."""
    global _default, _default_case
    if _default is not None:
        _default.close()
    _default = MolochDomain(case.dims, case.params)
    _default_case = case
    return _default


def init_moloch() -> None:
    """Main/mod_moloch.F90:201-308: bind static fields, state and boundary."""
    if _default is None:
        raise MolochError(abi.MLC_ERR_STATE, "init_moloch before allocate_moloch")
    c = _default_case
    _default.bind_static(c.static_ptrs())
    _default.upload(c.state_ptrs())
    if c.params.do_apply_bdy:
        _default.set_boundary(c.bdy_ptrs(), c.xbctime, c.params.dtbdys)


def moloch() -> abi.mlc_diag:
    """Main/mod_moloch.F90:312-446: advance the default domain by one dt and
    copy the state back into the case's arrays (the Fortran globals)."""
    if _default is None:
        raise MolochError(abi.MLC_ERR_STATE, "moloch before allocate_moloch")
    d = _default.step(1)
    _default.download(_default_case.state_ptrs())
    return d
