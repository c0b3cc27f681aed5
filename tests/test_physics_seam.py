"""The step split at the physics on the CPU oracle (no GPU).

Main/mod_moloch.F90:354-376 runs mkslice and the physics between the
dynamics and status_update; status_update (:1403-1443) adds dtsec times the
tendencies to t, ux, vx, qx and the tracers on the interior and applies the
species floors.  These tests pin the oracle's split: without tendencies it
equals the whole step bit for bit, and with tendencies the interior t moves
by exactly dtsec * tten while the species respect their floors.
"""
from __future__ import annotations

import numpy as np

from oracle.oracle import Oracle
from regcm_gb300 import abi
from regcm_gb300 import case as cs

# qxcheckval / qxzeroval of qv, qc, qi, qr, qs (Main/mpplib/mod_runparams.F90:184-192)
QX_CHECK = (1.0e-8, 1.0e-16, 1.0e-16, 1.0e-16, 1.0e-16)
QX_ZERO = (1.0e-8, 0.0, 0.0, 0.0, 0.0)


def small_case():
    return cs.build(24, 22, 10, dx=12000.0, dt=60.0, nsound=3, moist=True, seed=5,
                    hills=[(12 * 12000.0, 11 * 12000.0, 600.0)], wind=10.0, theta_noise=0.3,
                    tracer=True, name="seam")


def test_split_without_tendencies_is_the_step():
    c = small_case()
    a, b = Oracle(c), Oracle(c)
    assert a.step(3)[0] == 0
    for _ in range(3):
        assert b.step_dynamics() == 0
        assert b.step_finish()[0] == 0
    sa, sb = a.state(), b.state()
    for n in sa:
        assert np.array_equal(sa[n], sb[n]), n


def test_tendencies_enter_status_update():
    c = small_case()
    o = Oracle(c)
    assert o.step_dynamics() == 0
    mid = o.state()
    ten = c.tendencies(seed=1)
    assert o.set_tendencies(c.tend_ptrs_of(ten)) == 0
    assert o.step_finish()[0] == 0
    end = o.state()
    dt = c.params.dtsec
    inner = (slice(1, -1), slice(1, -1))
    # t gains dtsec * tten on jci x ici and nothing elsewhere
    assert np.array_equal(end["t"][inner], mid["t"][inner] + dt * ten["tten"])
    assert np.array_equal(end["t"][0], mid["t"][0])
    # the floors: after status_update no interior species is below its check value
    # unless it was set to its zero value; the tracer is non-negative
    q = end["qx"][inner]
    for n in range(q.shape[-1]):
        assert np.all((q[..., n] >= QX_CHECK[n]) | (q[..., n] == QX_ZERO[n])), n
    assert np.all(end["trac"][inner] >= 0.0)
    # the sinks drove some points to the floor
    assert np.any(end["trac"][inner] == 0.0)
    assert np.any(q[..., 0] == QX_ZERO[0])


def test_mkslice_tracer_floor():
    """After the dynamics half, interior tracer values are 0 or >= 1e-50
    (Main/mod_slice.F90:141-147)."""
    c = small_case()
    c.state["trac"][1:-1, 1:-1] = np.where(c.state["trac"][1:-1, 1:-1] > 0.5, 1e-60,
                                           c.state["trac"][1:-1, 1:-1])
    o = Oracle(c)
    assert o.step_dynamics() == 0
    tr = o.state()["trac"][1:-1, 1:-1]
    assert np.all((tr == 0.0) | (tr >= 1e-50))
    assert o.step_finish()[0] == 0


def test_open_step_refuses_a_whole_step():
    o = Oracle(small_case())
    assert o.set_tendencies(abi.mlc_tend_ptrs()) == abi.MLC_ERR_STATE
    assert o.step_finish()[0] == abi.MLC_ERR_STATE
    assert o.step_dynamics() == 0
    assert o.step(1)[0] == abi.MLC_ERR_STATE
    assert o.step_dynamics() == abi.MLC_ERR_STATE
    assert o.step_finish()[0] == 0


def test_tke_status_update_and_ring():
    """ibltyp = 2: the interior TKE gains dtsec * tketen and is floored at
    tkemin = 1e-3 (Main/mod_moloch.F90:1419-1424); on the boundary ring the
    top interface holds tkemin (Main/mod_bdycod.F90:1684-1869); a constant
    TKE above the floor in a resting, flat domain stays constant in the
    interior (the advection of a constant field is exact)."""
    c = cs.build(24, 22, 10, dx=12000.0, dt=60.0, nsound=3, moist=True, seed=5,
                 hills=[(12 * 12000.0, 11 * 12000.0, 600.0)], wind=10.0, theta_noise=0.3,
                 tke=True, name="seam_tke")
    o = Oracle(c)
    assert o.step_dynamics() == 0
    mid = o.state()
    ten = c.tendencies(seed=2)
    assert o.set_tendencies(c.tend_ptrs_of(ten)) == 0
    assert o.step_finish()[0] == 0
    end = o.state()
    inner = (slice(1, -1), slice(1, -1))
    exp = mid["tke"][inner] + c.params.dtsec * ten["tketen"]
    exp = np.where(exp < 1.0e-3, 1.0e-3, exp)
    assert np.array_equal(end["tke"][inner], exp)
    assert np.any(end["tke"][inner] == 1.0e-3)
    assert np.all(end["tke"][0, 1:-1, 0] == 1.0e-3) and np.all(end["tke"][:, 0, 0] == 1.0e-3)
