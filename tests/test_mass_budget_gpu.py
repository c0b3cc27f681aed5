"""The mass budget of the GPU step (Main/mod_massck.F90:57-200) against exact
sums of the state it reports on.

drymass = dx^2 * sum(dz * rho) and qmass = dx^2 * sum_n sum(qx_n * dz * rho)
over the interior jci x ici x kz, summed exactly (math.fsum of the FP64 products)
from the downloaded state, agree with the step's reported sums to 1e-12
relative, for FP64 members and for mixed members, whose FP32 state is summed
with exact products and double-float accumulation: the column mass of a mixed
member is accounted to FP64 accuracy.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from regcm_gb300 import abi
from regcm_gb300 import case as cs
from regcm_gb300.moloch import domain_from_case

pytestmark = pytest.mark.gpu


def exact_sums(case, st):
    dx2 = case.params.dx ** 2
    dz = case.static["dz"][1:-1, 1:-1, :]
    rho = st["rho"][1:-1, 1:-1, :]
    w = dz * rho  # exact in FP64 for FP32 inputs (24 x 24 bits)
    dry = dx2 * math.fsum(w.ravel())
    q = st["qx"][1:-1, 1:-1, :, :]
    # qx*dz*rho: 24 x 48 bits, within 2^-53 of the exact product per term
    qm = dx2 * math.fsum((q * w[..., None]).ravel())
    return dry, qm


@pytest.mark.parametrize("prec", [abi.MLC_PREC_FP64, abi.MLC_PREC_MIXED])
@pytest.mark.parametrize("make", [
    lambda p: cs.config1(nx=96, ny=80, kz=30, precision=p),
    lambda p: cs.build(40, 38, 14, dx=3000.0, dt=20.0, nsound=4, moist=True, seed=4, jet=True,
                       hills=[(20 * 3000.0, 18 * 3000.0, 1200.0)], tracer=True, name="budget",
                       precision=p),
])
def test_budget_sums_are_exact(prec, make):
    c = make(prec)
    assert c.params.debug_level > 0
    dom = domain_from_case(c)
    for _ in range(3):
        d = dom.step(1)
        st = c.empty_state()
        dom.download(c.state_ptrs_of(st))
        dry, qm = exact_sums(c, st)
        assert abs(d.drymass - dry) <= 1e-12 * abs(dry), (d.drymass, dry)
        assert abs(d.qmass - qm) <= 1e-12 * abs(qm), (d.qmass, qm)
    dom.close()
