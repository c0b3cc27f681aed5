"""Boundary refresh in mid-run (bdyin, Main/mod_bdycod.F90:1079-1200): new b0/b1
and xbctime = 0 after some steps, as RegCM does every ibdyfrq hours.  The GPU
keeps its step counter and buffer roles across the refresh and stays at the
oracle's state, in FP64 and in a batch."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle.oracle import Oracle
from regcm_gb300 import abi
from regcm_gb300 import case as cs
from regcm_gb300.moloch import MolochBatch, domain_from_case

from .conftest import rel_l2

pytestmark = pytest.mark.gpu


def refreshed_boundary(c, scale0: float, scale1: float):
    """b0' = b0 * scale0 and b1' = b0 * scale1 for t, q, winds; Exner and ps
    shifted by the same relative amounts (a smooth change of the driving data)."""
    new = {}
    for name, (b0, b1) in c.bdy.items():
        if b0 is None:
            new[name] = (None, None)
            continue
        new[name] = (np.asfortranarray(b0 * scale0), np.asfortranarray(b0 * scale1))
    keep = c.bdy
    c.bdy = new
    ptrs = c.bdy_ptrs()
    c.bdy = keep
    return ptrs, new


@pytest.mark.parametrize("make", [
    lambda: cs.config0(nx=40, ny=36, kz=14),
    lambda: cs.config1(nx=40, ny=40, kz=20),
])
def test_refresh_matches_oracle(make):
    c = make()
    dom = domain_from_case(c)
    orc = Oracle(make())
    dom.step(5)
    orc.step(5)
    ptrs, arrays = refreshed_boundary(c, 1.0005, 0.9995)
    dom.set_boundary(ptrs, 0.0, c.params.dtbdys)
    orc.set_boundary(ptrs, 0.0, c.params.dtbdys)
    d = dom.step(6)
    st, do = orc.step(6)
    assert st == 0
    assert abs(d.xbctime - 6 * c.params.dtsec) < 1e-9 and abs(do.xbctime - d.xbctime) < 1e-9
    got = c.empty_state()
    dom.download(c.state_ptrs_of(got))
    ref = orc.state()
    dom.close()
    orc.close()
    for n in ("u", "v", "w", "tetav", "pai", "t", "qx"):
        assert rel_l2(got[n], ref[n]) <= 1e-11, n


def test_refresh_in_batch_same_as_alone():
    cases = [cs.config2_member(m, nx=36, ny=32, kz=12) for m in range(3)]
    b = MolochBatch(cases)
    b.step(4)
    ptrs, _ = refreshed_boundary(cases[1], 1.001, 0.999)
    abi.check(b.lib.mlc_member_set_boundary(b._ctx, 1, C.byref(ptrs), 0.0, cases[1].params.dtbdys),
              "refresh")
    b.step(3)
    alone = cs.config2_member(1, nx=36, ny=32, kz=12)
    d = domain_from_case(alone)
    d.step(4)
    ptrs2, _ = refreshed_boundary(alone, 1.001, 0.999)
    d.set_boundary(ptrs2, 0.0, alone.params.dtbdys)
    d.step(3)
    ga = alone.empty_state()
    d.download(alone.state_ptrs_of(ga))
    gb = cases[1].empty_state()
    b.download(1, cases[1].state_ptrs_of(gb))
    for n in ga:
        assert np.array_equal(ga[n], gb[n]), n
