"""The allocation-free mass budget against the budget mlc_step reports.

Callers that manage device memory themselves (and so cannot let the library
call cudaMalloc) use mlc_mass_budget_noalloc on their own device arrays; it
must give the sums that the normal step gives for the same fields.  Two
calls in a row, a larger domain and then a smaller one, check that the
shared scratch array carries nothing over from one call to the next.  This
file is collected last on purpose.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from regcm_gb300 import abi
from regcm_gb300 import case as cs
from regcm_gb300.moloch import domain_from_case

pytestmark = pytest.mark.gpu


def _fn():
    lib = abi.load()
    f = lib.mlc_mass_budget_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(abi.mlc_dims), C.c_double, C.c_double] + [C.c_void_p] * 8
    return f


def _budget_of(f, case, st, dev, out):
    """mlc_mass_budget_noalloc on device copies of a downloaded state."""
    import torch
    on = {n: torch.from_numpy(np.ravel(st[n], order="F").copy()).to(dev)
          for n in ("rho", "qx", "u", "v", "ps")}
    dz = torch.from_numpy(np.ravel(case.static["dz"], order="F").copy()).to(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = f(C.byref(case.dims), case.params.dx, case.params.dtsec, on["rho"].data_ptr(),
           dz.data_ptr(), on["qx"].data_ptr(), on["u"].data_ptr(), on["v"].data_ptr(),
           on["ps"].data_ptr(), out.data_ptr(), C.c_void_p(stream))
    assert rc == abi.MLC_OK
    torch.cuda.synchronize(dev)
    return out.cpu().numpy()


def test_noalloc_budget_matches_step_budget_twice():
    """A larger domain first (more partial records in the shared array), then
    a smaller one: the second result must be the smaller domain's own budget,
    with nothing read from the records the first call left behind."""
    import torch
    f = _fn()
    big = cs.build(64, 60, 20, dx=3000.0, dt=20.0, nsound=4, moist=True, seed=5, jet=True,
                   name="noalloc_big")
    small = cs.build(40, 38, 14, dx=3000.0, dt=20.0, nsound=4, moist=True, seed=4, jet=True,
                     name="noalloc_small")
    dev = torch.device("cuda", torch.cuda.current_device())
    out = torch.full((7,), -1.0, dtype=torch.float64, device=dev)
    for call, case in enumerate((big, small)):
        dom = domain_from_case(case)
        d = dom.step(1)
        st = case.empty_state()
        dom.download(case.state_ptrs_of(st))
        dom.close()
        got = _budget_of(f, case, st, dev, out)
        scale = abs(d.drymass)
        assert abs(got[0] - d.drymass) <= 1e-12 * abs(d.drymass), call
        assert abs(got[2] - d.qmass) <= 1e-12 * abs(d.qmass), call
        assert abs(got[1] - d.dryadv) <= 1e-12 * max(abs(d.dryadv), 1e-6 * scale), call
        assert abs(got[3] - d.qadv) <= 1e-12 * max(abs(d.qadv), 1e-6 * abs(d.qmass)), call
        assert got[4] == d.ps_max and got[5] == d.ps_min and got[6] == 0.0, call


def test_noalloc_flags_non_finite_surface_pressure():
    """A NaN in one interior ps value (host data, copied to the device) sets
    the non-finite flag and NaN extrema, as the step's own check does."""
    import torch
    f = _fn()
    case = cs.build(40, 38, 14, dx=3000.0, dt=20.0, nsound=4, moist=True, seed=4, jet=True,
                    name="noalloc_nan")
    st = case.copy_state()
    st["ps"][10, 12] = np.nan
    dev = torch.device("cuda", torch.cuda.current_device())
    out = torch.full((7,), -1.0, dtype=torch.float64, device=dev)
    got = _budget_of(f, case, st, dev, out)
    assert got[6] == 1.0 and np.isnan(got[4]) and np.isnan(got[5])
    assert np.isfinite(got[0]) and got[0] > 0


def test_noalloc_rejects_domains_beyond_its_scratch():
    f = _fn()
    big = abi.mlc_dims(65, 2049, 20, 2, 0)   # 2048 * 20 rows > 32768
    one = C.c_void_p(8)  # never dereferenced: the size check comes first
    rc = f(C.byref(big), 1.0, 1.0, one, one, one, one, one, one, one, None)
    assert rc == abi.MLC_ERR_TOO_LARGE
