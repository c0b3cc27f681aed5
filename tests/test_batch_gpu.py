"""Ensembles: members advanced together by one launch per kernel stage give
exactly the states the same members reach one at a time."""
from __future__ import annotations

import numpy as np
import pytest

from regcm_gb300 import abi
from regcm_gb300 import case as cs
from regcm_gb300.moloch import MolochBatch, domain_from_case

pytestmark = pytest.mark.gpu


def members(prec, n=3):
    return [cs.config2_member(m, nx=40, ny=36, kz=14, precision=prec) for m in range(n)]


@pytest.mark.parametrize("prec", [abi.MLC_PREC_FP64, abi.MLC_PREC_MIXED])
def test_batch_equals_members_alone(prec):
    batch_cases = members(prec)
    alone_cases = members(prec)
    b = MolochBatch(batch_cases)
    db = b.step(5)
    for m, c in enumerate(alone_cases):
        d = domain_from_case(c)
        da = d.step(5)
        ga = c.empty_state()
        d.download(c.state_ptrs_of(ga))
        d.close()
        gb = batch_cases[m].empty_state()
        b.download(m, batch_cases[m].state_ptrs_of(gb))
        for n in ga:
            assert np.array_equal(ga[n], gb[n]), (m, n)
        assert db[m].drymass == da.drymass and db[m].ps_max == da.ps_max
    b.close()


def test_batch_members_differ_and_graph_matches_eager():
    a = MolochBatch(members(abi.MLC_PREC_MIXED, 4))
    e = MolochBatch(members(abi.MLC_PREC_MIXED, 4))
    e.set_graphs(False)
    a.step(3)
    e.step(3)
    states = []
    for m in range(4):
        ga = a.cases[m].empty_state()
        a.download(m, a.cases[m].state_ptrs_of(ga))
        ge = e.cases[m].empty_state()
        e.download(m, e.cases[m].state_ptrs_of(ge))
        for n in ga:
            assert np.array_equal(ga[n], ge[n]), (m, n)
        states.append(ga)
    # members carry their own winds and noise
    assert not np.array_equal(states[0]["u"], states[1]["u"])


def test_autotune_keeps_state_and_results():
    tuned = MolochBatch(members(abi.MLC_PREC_MIXED, 3))
    plain = MolochBatch(members(abi.MLC_PREC_MIXED, 3))
    rep = tuned.autotune(1)
    assert rep["ms_tuned"] > 0 and rep["ms_fixed"] > 0
    assert rep["col_x"] * rep["col_y"] <= 1024 and rep["htile"] in (0, 1, 2, 3)
    tuned.step(4)
    plain.step(4)
    for m in range(3):
        a = tuned.cases[m].empty_state()
        tuned.download(m, tuned.cases[m].state_ptrs_of(a))
        b = plain.cases[m].empty_state()
        plain.download(m, plain.cases[m].state_ptrs_of(b))
        for n in a:
            # the tuned tile shapes may round FP32 fields differently at a
            # few points (tests/test_shapes_gpu.py); the state must be kept
            d = np.abs(a[n] - b[n]).max()
            assert d <= 2e-5 * np.abs(b[n]).max(), (m, n, d)
