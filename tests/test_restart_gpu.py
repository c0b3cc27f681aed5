"""SAV restart on the GPU: a snapshot of the device state written as the
MOLOCH variables of a SAV file holds exactly the state mlc_download_state
returns (read back with scipy's netCDF reader), and a domain restarted from
that file (mlc_member_read_sav: read_savefile + the restart state of
Main/mod_init.F90:421-450,941-966) steps like the oracle restarted from the
same fields, to the path's FP64 tolerance.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle.oracle import Oracle
from oracle.oracle import load as load_oracle
from regcm_gb300 import abi
from regcm_gb300 import case as cs
from regcm_gb300.moloch import MolochDomain, domain_from_case

from .test_parity_gpu import field_errors

pytestmark = pytest.mark.gpu
netcdf = pytest.importorskip("scipy.io").netcdf_file

NAMES = {"atm_u": "u", "atm_v": "v", "atm_w": "w", "atm_t": "t", "atm_pai": "pai",
         "atm_qx": "qx", "ps": "ps", "trac": "trac"}


def moist_tracer(precision=abi.MLC_PREC_FP64, tke=False):
    return cs.build(40, 38, 14, dx=3000.0, dt=20.0, nsound=4, moist=True, seed=4,
                    hills=[(20 * 3000.0, 18 * 3000.0, 1200.0)], jet=True, theta_noise=0.2,
                    tracer=True, name="restart", precision=precision, tke=tke)


@pytest.mark.parametrize("prec,tke", [(abi.MLC_PREC_FP64, False), (abi.MLC_PREC_MIXED, False),
                                      (abi.MLC_PREC_FP64, True)])
def test_snapshot_is_the_device_state(tmp_path, prec, tke):
    c = moist_tracer(prec, tke)
    dom = domain_from_case(c)
    dom.step(4)
    path = tmp_path / "SAV.nc"
    dom.write_sav(str(path), "2000010100", "gregorian")
    g = c.empty_state()
    dom.download(c.state_ptrs_of(g))
    dom.close()
    with netcdf(str(path), "r", mmap=False) as f:
        assert f.idatex == b"2000010100"
        for v, n in NAMES.items():
            assert np.array_equal(np.asarray(f.variables[v].data).T, g[n]), v
        # atm_tke only with the UW PBL (Main/mod_savefile.F90:884-887)
        assert ("atm_tke" in f.variables) == tke
        if tke:
            assert np.array_equal(np.asarray(f.variables["atm_tke"].data).T, g["tke"])


@pytest.mark.parametrize("tke", [False, True])
def test_restart_steps_like_the_oracle(tmp_path, tke):
    c = moist_tracer(tke=tke)
    dom = domain_from_case(c)
    d4 = dom.step(4)
    path = tmp_path / "SAV.nc"
    dom.write_sav(str(path))
    dom.close()
    # a new domain restarted from the file; boundary data and clock from bdyin
    r = MolochDomain(c.dims, c.params)
    r.bind_static(c.static_ptrs())
    r.read_sav(str(path))
    bp = c.bdy_ptrs()
    r.set_boundary(bp, d4.xbctime, c.params.dtbdys)
    # the oracle restarted from the same fields
    sav = c.empty_sav()
    assert abi.load().mlc_sav_read(str(path).encode(), C.byref(c.dims), C.byref(c.sav_ptrs_of(sav)),
                                   None, 0) == 0
    rs = c.empty_state()
    assert load_oracle().orc_restart_state(C.byref(c.dims), C.byref(c.sav_ptrs_of(sav)),
                                           C.byref(c.state_ptrs_of(rs))) == 0
    orc = Oracle(c)
    sp = c.state_ptrs_of(rs)
    assert orc.lib.orc_set_state(orc.h, C.byref(sp)) == 0
    orc.set_boundary(bp, d4.xbctime, c.params.dtbdys)
    # the restart state itself, then three steps
    g0 = c.empty_state()
    r.download(c.state_ptrs_of(g0))
    err = field_errors(g0, orc.state(), c)
    assert max(err.values()) <= 1e-15, err
    r.step(3)
    st, _ = orc.step(3)
    assert st == 0
    g = c.empty_state()
    r.download(c.state_ptrs_of(g))
    err = field_errors(g, orc.state(), c)
    bad = {k: v for k, v in err.items() if not v <= 1e-12}
    assert not bad, bad
    r.close()
    orc.close()
