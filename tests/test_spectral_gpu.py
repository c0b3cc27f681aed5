"""Spectral nudging of t, u and v toward the boundary data's large scales
(Main/mod_bdycod.F90:3844-3960, called from Main/mod_moloch.F90:499-506)
on the GPU against the CPU oracle.

FP64 members are held to the path's tolerances (relative L2 <= 1e-12 after
one step, <= 1e-10 after ten); each case also checks that the nudging moves
the state by far more than the tolerance, so the comparison is not vacuous.
The domains give 2x2 modes (24x22 at 12 km) and 4x6 modes (200x160 at
12 km).  With dtrad a multiple of dtsec the nudging runs every few steps
only, which the ten-step case with dtrad = 3*dtsec covers.  A mixed member
is compared point by point with the FP64 oracle after one step and in
relative L2 after twenty.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle.oracle import Oracle
from regcm_gb300 import abi
from regcm_gb300 import case as cs
from regcm_gb300.moloch import domain_from_case

from .conftest import rel_l2
from .test_parity_gpu import field_errors, run_pair

pytestmark = pytest.mark.gpu


def small_dry(**kw):
    return cs.build(24, 22, 12, dx=12000.0, dt=60.0, nsound=3, moist=False, seed=3,
                    hills=[(12 * 12000.0, 11 * 12000.0, 600.0)], wind=10.0, theta_noise=0.3,
                    tracer=True, name="small_dry_spectral", spectral=True, **kw)


def wide_moist(**kw):
    return cs.build(200, 160, 16, dx=12000.0, dt=60.0, nsound=3, moist=True, seed=11,
                    hills=[(100 * 12000.0, 80 * 12000.0, 900.0)], jet=True, theta_noise=0.3,
                    name="wide_moist_spectral", spectral=True, **kw)


def oracle_state(case, nsteps):
    orc = Oracle(case)
    st, _ = orc.step(nsteps)
    assert st == 0
    out = orc.state()
    orc.close()
    return out


@pytest.mark.parametrize("name,make,nsteps,tol", [
    ("dry_every_step", lambda **kw: small_dry(dtrad=60.0, **kw), 1, 1e-12),
    ("wide_every_step", lambda **kw: wide_moist(dtrad=60.0, **kw), 1, 1e-12),
    ("dry_every_third_step", lambda **kw: small_dry(dtrad=180.0, **kw), 10, 1e-10),
])
def test_spectral_parity(name, make, nsteps, tol):
    case = make()
    g, o, dg, do = run_pair(case, nsteps)
    err = field_errors(g, o, case)
    bad = {k: v for k, v in err.items() if not v <= tol}
    assert not bad, f"{name}: {bad}"
    # the nudging changed the state by far more than the tolerance
    off = make()
    off.params.mo_spectral_nudge = 0
    ref_off = oracle_state(off, nsteps)
    assert rel_l2(ref_off["v"], o["v"]) > 1e3 * tol, name


def test_spectral_mixed():
    """A mixed member with spectral nudging every step against the FP64
    oracle: after one step point by point (FP32 rounding size, as the other
    mixed members), after twenty in relative L2 (scope: 1e-4)."""
    def make(prec):
        return small_dry(dtrad=60.0, precision=prec)

    for nsteps in (1, 20):
        cm, cf = make(abi.MLC_PREC_MIXED), make(abi.MLC_PREC_FP64)
        dom = domain_from_case(cm)
        dom.step(nsteps)
        got = cm.empty_state()
        dom.download(cm.state_ptrs_of(got))
        dom.close()
        ref = oracle_state(cf, nsteps)
        if nsteps == 1:
            vel = max(np.abs(ref["u"]).max(), np.abs(ref["v"]).max())
            for n, scale, tol in (("u", vel, 1e-5), ("v", vel, 1e-5),
                                  ("tetav", np.abs(ref["tetav"]).max(), 1e-6),
                                  ("pai", np.abs(ref["pai"]).max(), 1e-7)):
                d = np.abs(got[n] - ref[n]).max() / scale
                assert d <= tol, (n, d)
        else:
            for n in ("u", "v", "w", "tetav"):
                assert rel_l2(got[n], ref[n]) <= 3e-5, (n, rel_l2(got[n], ref[n]))
