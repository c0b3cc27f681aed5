"""Failure paths of the step, made without any GPU fault.

1. The stop on a non-finite state (Main/mod_moloch.F90:407-422: NaN or Inf in
the surface-pressure extrema is fatal "CFL VIOLATION").

The failure is made on the host: a NaN in one interior Exner value of the
uploaded state is ordinary data to the GPU (no fault is involved).  The
surface pressure extrapolated from that column is NaN after the step, the
library returns MLC_ERR_NONFINITE, the Python mirror raises CFLViolation,
and the oracle stops the same way.  The context stays usable: a clean state
uploaded afterwards steps normally.

2. The bounded waits of the copy-engine pipelines: a test hook makes the
horizontal WAF's blocks wait on an mbarrier that nothing completes (before
any copy is issued), so the wait runs out after a few polls; the kernel
records the fault and leaves, and the step reports it as a status.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle.oracle import Oracle
from regcm_gb300 import abi
from regcm_gb300.moloch import CFLViolation, domain_from_case

from .test_parity_gpu import small_dry, small_moist

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("make,prec", [(small_dry, abi.MLC_PREC_FP64),
                                       (small_moist, abi.MLC_PREC_FP64),
                                       (small_moist, abi.MLC_PREC_MIXED)])
def test_nan_in_state_is_a_cfl_violation(make, prec):
    case = make(precision=prec)
    kz = case.dims.kz
    bad = case.copy_state()
    bad["pai"][9, 8, kz - 1] = np.nan
    dom = domain_from_case(case)
    dom.upload(case.state_ptrs_of(bad))
    d = abi.mlc_diag()
    st = dom.lib.mlc_step(dom._ctx, 1, C.byref(d))
    assert st == abi.MLC_ERR_NONFINITE
    assert d.nonfinite == 1
    assert not (np.isfinite(d.ps_max) and np.isfinite(d.ps_min))
    # the Python mirror of moloch() raises the reference's fatal as CFLViolation
    with pytest.raises(CFLViolation):
        dom.step(1)
    # the oracle given the same state stops too
    if prec == abi.MLC_PREC_FP64:
        bc = make()
        bc.state = bad
        orc = Oracle(bc)
        ost, od = orc.step(1)
        orc.close()
        assert ost == abi.MLC_ERR_NONFINITE and od.nonfinite == 1
    dom.close()
    # the device is fine afterwards: a fresh domain with the clean state steps
    ok = domain_from_case(make(precision=prec))
    dg = ok.step(2)
    assert dg.nonfinite == 0 and np.isfinite(dg.ps_max)
    ok.close()


@pytest.mark.parametrize("prec", [abi.MLC_PREC_FP64, abi.MLC_PREC_MIXED])
def test_bounded_wait_gives_up_and_reports(prec):
    from regcm_gb300.moloch import MolochBatch
    cases = [small_dry(precision=prec), small_dry(precision=prec)]
    b = MolochBatch(cases)
    b.step(1)
    lib = b.lib
    assert lib.mlc_member_test_stall(b._ctx, 1, 64) == abi.MLC_OK
    d = (abi.mlc_diag * 2)()
    st = lib.mlc_step_batch(b._ctx, 1, d)
    assert st == abi.MLC_ERR_CUDA
    assert b"bounded device wait" in lib.mlc_last_error()
    b.close()
    # the device still answers: a fresh domain steps normally
    ok = domain_from_case(small_dry(precision=prec))
    dg = ok.step(1)
    assert dg.nonfinite == 0 and np.isfinite(dg.ps_max)
    ok.close()
