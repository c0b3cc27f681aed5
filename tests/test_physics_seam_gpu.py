"""The step split at the physics (mlc_step_dynamics, mlc_member_set_tendencies,
mlc_step_finish) on the GPU against the CPU oracle's split.

* Without tendencies the split step equals mlc_step: bit for bit in FP64,
  within FP32 rounding for a mixed member (the split path runs the scalar
  step-end kernels, the whole step the four-column ones).
* The state after the dynamics half (what mkslice and the physics read) and
  the state after status_update with synthetic tendencies match the oracle
  to the path's FP64 tolerance, for three consecutive coupled steps with new
  tendencies each; the tendencies move the state by far more than that.
* A mixed member with tendencies stays within FP32 rounding of the oracle.
* The same with the UW PBL's TKE (ibltyp = 2) and its tendency tketen.
* An open step refuses whole steps, uploads and a second dynamics half.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle.oracle import Oracle
from regcm_gb300 import abi
from regcm_gb300 import case as cs
from regcm_gb300.moloch import MolochBatch, domain_from_case

from .conftest import rel_l2
from .test_parity_gpu import field_errors

pytestmark = pytest.mark.gpu


def seam_case(precision=abi.MLC_PREC_FP64, **kw):
    return cs.build(40, 38, 14, dx=3000.0, dt=20.0, nsound=4, moist=True, seed=4,
                    hills=[(20 * 3000.0, 18 * 3000.0, 1200.0)], jet=True, theta_noise=0.2,
                    tracer=True, name="seam_moist", precision=precision, **kw)


def download(dom, case):
    g = case.empty_state()
    dom.download(case.state_ptrs_of(g))
    return g


@pytest.mark.parametrize("prec", [abi.MLC_PREC_FP64, abi.MLC_PREC_MIXED])
def test_split_without_tendencies_is_the_step(prec):
    c = seam_case(prec)
    a, b = domain_from_case(c), domain_from_case(c)
    a.step(3)
    for _ in range(3):
        b.step_dynamics()
        b.step_finish()
    ga, gb = download(a, c), download(b, c)
    a.close()
    b.close()
    for n in ga:
        if prec == abi.MLC_PREC_FP64:
            assert np.array_equal(ga[n], gb[n]), n
        else:
            d = np.abs(ga[n] - gb[n]).max()
            assert d <= 2e-6 * max(np.abs(ga[n]).max(), 1e-30), (n, d)


@pytest.mark.parametrize("tke", [False, True])
def test_coupled_steps_match_oracle(tke):
    c = seam_case(tke=tke)
    dom, orc = domain_from_case(c), Oracle(c)
    keep = []
    for step in range(3):
        dom.step_dynamics()
        assert orc.step_dynamics() == 0
        mid_g, mid_o = download(dom, c), orc.state()
        err = field_errors(mid_g, mid_o, c)
        bad = {k: v for k, v in err.items() if not v <= 1e-12}
        assert not bad, (step, "mkslice state", bad)
        ten = c.tendencies(seed=10 + step)
        tp = c.tend_ptrs_of(ten)
        keep.append((ten, tp))
        dom.set_tendencies(tp)
        assert orc.set_tendencies(tp) == 0
        dg = dom.step_finish()
        st, do = orc.step_finish()
        assert st == 0
        end_g, end_o = download(dom, c), orc.state()
        err = field_errors(end_g, end_o, c)
        bad = {k: v for k, v in err.items() if not v <= 1e-12}
        assert not bad, (step, "status_update", bad)
        assert abs(dg.xbctime - do.xbctime) == 0.0
    # the tendencies changed the state by far more than the tolerance
    ref = Oracle(c)
    assert ref.step(3)[0] == 0
    plain = ref.state()
    assert rel_l2(plain["t"], end_o["t"]) > 1e-9
    assert rel_l2(plain["u"], end_o["u"]) > 1e-9
    dom.close()
    orc.close()
    ref.close()


@pytest.mark.parametrize("tke", [False, True])
def test_coupled_mixed_member(tke):
    cm, cf = seam_case(abi.MLC_PREC_MIXED, tke=tke), seam_case(tke=tke)
    dom, orc = domain_from_case(cm), Oracle(cf)
    keep = []
    for step in range(5):
        ten = cf.tendencies(seed=20 + step)
        tp = cf.tend_ptrs_of(ten)
        keep.append((ten, tp))
        dom.step_dynamics()
        dom.set_tendencies(tp)
        dom.step_finish()
        assert orc.step_dynamics() == 0
        assert orc.set_tendencies(tp) == 0
        assert orc.step_finish()[0] == 0
    got, ref = download(dom, cm), orc.state()
    for n in ("u", "v", "w", "tetav", "t"):
        assert rel_l2(got[n], ref[n]) <= 3e-5, (n, rel_l2(got[n], ref[n]))
    assert rel_l2(got["qx"][..., 0], ref["qx"][..., 0]) <= 3e-5
    assert rel_l2(got["trac"], ref["trac"]) <= 3e-5
    if tke:
        assert rel_l2(got["tke"], ref["tke"]) <= 3e-5, rel_l2(got["tke"], ref["tke"])
    dom.close()
    orc.close()


def test_batch_member_tendencies_stay_with_their_member():
    """Tendencies set for member 1 of a batch change member 1 only."""
    cases = [seam_case(), seam_case()]
    b = MolochBatch(cases)
    b.step_dynamics()
    ten = cases[1].tendencies(seed=3)
    tp = cases[1].tend_ptrs_of(ten)
    b.set_tendencies(1, tp)
    b.step_finish()
    g = [cases[m].empty_state() for m in range(2)]
    for m in range(2):
        b.download(m, cases[m].state_ptrs_of(g[m]))
    b.close()
    solo = domain_from_case(cases[0])
    solo.step(1)
    ref0 = download(solo, cases[0])
    solo.close()
    for n in ref0:
        assert np.array_equal(g[0][n], ref0[n]), n
    assert not np.array_equal(g[1]["t"], ref0["t"])


def test_open_step_state_machine():
    c = seam_case()
    dom = domain_from_case(c)
    lib, ctx = dom.lib, dom._ctx
    tp = abi.mlc_tend_ptrs()
    d = abi.mlc_diag()
    import ctypes as C
    assert lib.mlc_member_set_tendencies(ctx, 0, C.byref(tp)) == abi.MLC_ERR_STATE
    assert lib.mlc_step_finish(ctx, C.byref(d)) == abi.MLC_ERR_STATE
    assert lib.mlc_step_dynamics(ctx) == 0
    assert lib.mlc_step_dynamics(ctx) == abi.MLC_ERR_STATE
    assert lib.mlc_step(ctx, 1, C.byref(d)) == abi.MLC_ERR_STATE
    assert lib.mlc_upload_state(ctx, C.byref(c.state_ptrs())) == abi.MLC_ERR_STATE
    assert lib.mlc_member_set_tendencies(ctx, 0, C.byref(tp)) == 0
    assert lib.mlc_step_finish(ctx, C.byref(d)) == 0
    assert lib.mlc_step(ctx, 1, C.byref(d)) == 0
    dom.close()
