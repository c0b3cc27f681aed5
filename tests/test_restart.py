"""SAV restart files without a GPU: the netCDF classic writer and reader of
the library (mlc_sav_write / mlc_sav_read) checked against scipy's
independent netCDF-3 implementation in both directions (and a CDF-5 file
written by hand from the format's definition), their error paths,
and the restart state (Main/mod_init.F90:421-450,941-960) against the
oracle's restatement.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle.oracle import load as load_oracle
from regcm_gb300 import abi
from regcm_gb300 import case as cs

netcdf = pytest.importorskip("scipy.io").netcdf_file

# (name, Fortran dimension names) of the MOLOCH variables, Main/mod_savefile.F90:867-883
VARS = {"atm_u": ("jdot", "icross", "khalf"), "atm_v": ("jcross", "idot", "khalf"),
        "atm_w": ("jcross", "icross", "kfull"), "atm_t": ("jcross", "icross", "khalf"),
        "atm_pai": ("jcross", "icross", "khalf"), "atm_qx": ("jcross", "icross", "khalf", "nqx"),
        "ps": ("jcross", "icross"), "trac": ("jcross", "icross", "khalf", "ntr")}
KEYS = {"atm_u": "u", "atm_v": "v", "atm_w": "w", "atm_t": "t", "atm_pai": "pai",
        "atm_qx": "qx", "ps": "ps", "trac": "trac"}


def small(tracer=True):
    return cs.build(17, 13, 6, dx=12000.0, dt=60.0, nsound=3, moist=True, seed=8,
                    tracer=tracer, name="sav")


def random_sav(c, seed=0):
    rng = np.random.default_rng(seed)
    sav = c.empty_sav()
    for n, a in sav.items():
        a[...] = rng.normal(size=a.shape)
    return sav


@pytest.mark.parametrize("tracer", [False, True])
def test_written_file_reads_back_in_scipy(tmp_path, tracer):
    c = small(tracer)
    sav = random_sav(c)
    path = tmp_path / "SAV.2020010100.nc"
    lib = abi.load()
    assert lib.mlc_sav_write(str(path).encode(), C.byref(c.dims), C.byref(c.sav_ptrs_of(sav)),
                             b"2020010100", b"gregorian") == 0
    with netcdf(str(path), "r", mmap=False) as f:
        assert f.version_byte == 2
        d = c.dims
        assert f.dimensions["jcross"] == d.jx - 1 and f.dimensions["jdot"] == d.jx
        assert f.dimensions["icross"] == d.iy - 1 and f.dimensions["idot"] == d.iy
        assert f.dimensions["khalf"] == d.kz and f.dimensions["kfull"] == d.kz + 1
        assert f.dimensions["nqx"] == d.nqx
        assert f.idatex == b"2020010100" and f.calendar == b"gregorian"
        for name, fdims in VARS.items():
            if name == "trac" and not tracer:
                assert name not in f.variables
                continue
            var = f.variables[name]
            assert var.dimensions == tuple(reversed(fdims)), name
            assert var.data.dtype == np.dtype(">f8")
            # netCDF lists dimensions slowest first: the Fortran array is its transpose
            assert np.array_equal(np.asarray(var.data).T, sav[KEYS[name]]), name


@pytest.mark.parametrize("version,dtype", [(1, "f8"), (2, "f8"), (2, "f4")])
def test_scipy_file_reads_in_library(tmp_path, version, dtype):
    c = small()
    sav = random_sav(c, seed=1)
    path = tmp_path / "SAV.nc"
    d = c.dims
    with netcdf(str(path), "w", version=version) as f:
        f.idatex = "1999123118"
        f.createDimension("jcross", d.jx - 1)
        f.createDimension("icross", d.iy - 1)
        f.createDimension("jdot", d.jx)
        f.createDimension("idot", d.iy)
        f.createDimension("khalf", d.kz)
        f.createDimension("kfull", d.kz + 1)
        f.createDimension("nqx", d.nqx)
        f.createDimension("ntr", d.ntr)
        f.createDimension("month", 12)  # a dimension of other SAV variables
        f.createVariable("other", "f8", ("month",))[:] = np.arange(12.0)
        for name, fdims in VARS.items():
            v = f.createVariable(name, dtype, tuple(reversed(fdims)))
            v[...] = sav[KEYS[name]].T
    got = c.empty_sav()
    buf = C.create_string_buffer(32)
    assert abi.load().mlc_sav_read(str(path).encode(), C.byref(d), C.byref(c.sav_ptrs_of(got)),
                                   buf, 32) == 0
    assert buf.value == b"1999123118"
    for n, a in sav.items():
        want = a.astype(np.float32).astype(np.float64) if dtype == "f4" else a
        assert np.array_equal(got[n], want), n


def test_read_errors(tmp_path):
    c = small()
    sav = random_sav(c)
    lib = abi.load()
    path = tmp_path / "a.nc"
    assert lib.mlc_sav_write(str(path).encode(), C.byref(c.dims), C.byref(c.sav_ptrs_of(sav)),
                             None, None) == 0
    got = c.empty_sav()
    # other extents than the file's
    other = small()
    other.dims.jx += 1
    assert lib.mlc_sav_read(str(path).encode(), C.byref(other.dims),
                            C.byref(other.sav_ptrs_of(other.empty_sav())), None, 0) == abi.MLC_ERR_INVALID
    # a missing file, an HDF5 (netCDF-4) file, a truncated file
    assert lib.mlc_sav_read(str(tmp_path / "none.nc").encode(), C.byref(c.dims),
                            C.byref(c.sav_ptrs_of(got)), None, 0) == abi.MLC_ERR_INVALID
    h5 = tmp_path / "h5.nc"
    h5.write_bytes(b"\x89HDF\r\n\x1a\n" + bytes(64))
    assert lib.mlc_sav_read(str(h5).encode(), C.byref(c.dims), C.byref(c.sav_ptrs_of(got)),
                            None, 0) == abi.MLC_ERR_UNSUPPORTED
    cut = tmp_path / "cut.nc"
    cut.write_bytes(path.read_bytes()[:2000])
    assert lib.mlc_sav_read(str(cut).encode(), C.byref(c.dims), C.byref(c.sav_ptrs_of(got)),
                            None, 0) == abi.MLC_ERR_INVALID


def test_restart_state_matches_oracle():
    c = small()
    sav = {n: np.array(c.state[n], order="F", copy=True) for n in ("u", "v", "w", "t", "pai", "qx",
                                                                      "ps", "trac")}
    a, b = c.empty_state(), c.empty_state()
    assert abi.load().mlc_sav_restart_state(C.byref(c.dims), C.byref(c.sav_ptrs_of(sav)),
                                            C.byref(c.state_ptrs_of(a))) == 0
    assert load_oracle().orc_restart_state(C.byref(c.dims), C.byref(c.sav_ptrs_of(sav)),
                                           C.byref(c.state_ptrs_of(b))) == 0
    for n in a:
        assert np.array_equal(a[n], b[n]), n
    # the diagnostics follow from t, pai and qv alone
    assert np.allclose(a["tvirt"], sav["t"] * (1 + 0.6077 * sav["qx"][..., 0]), rtol=1e-4)
    assert not np.any(a["ux"]) and not np.any(a["vx"])


def _cdf5_bytes(dims, atts, vars_):
    """A netCDF CDF-5 (64-bit data) file written by hand: header of 64-bit
    counts and lengths, then each variable's big-endian values at its offset."""
    import struct
    u32 = lambda v: struct.pack(">I", v)
    u64 = lambda v: struct.pack(">Q", v)

    def name(s):
        b = s.encode()
        return u64(len(b)) + b + b"\0" * ((4 - len(b) % 4) % 4)

    def header(begins):
        h = b"CDF\x05" + u64(0)
        h += u32(10) + u64(len(dims))
        for n, ln in dims:
            h += name(n) + u64(ln)
        h += u32(12) + u64(len(atts))
        for n, txt in atts:
            b = txt.encode()
            h += name(n) + u32(2) + u64(len(b)) + b + b"\0" * ((4 - len(b) % 4) % 4)
        h += u32(11) + u64(len(vars_))
        for (n, dimids, data), beg in zip(vars_, begins):
            h += name(n) + u64(len(dimids)) + b"".join(u64(d) for d in dimids)
            h += u32(0) + u64(0) + u32(6) + u64(data.size * 8) + u64(beg)
        return h

    size = len(header([0] * len(vars_)))
    begins, off = [], size
    for _, _, data in vars_:
        begins.append(off)
        off += data.size * 8
    out = header(begins)
    for _, _, data in vars_:
        out += np.asarray(data, dtype=">f8").tobytes()
    return out


def test_cdf5_file_reads_in_library(tmp_path):
    """A CDF-5 file (RegCM built with NETCDF_CDF5, or a variable above 4 GiB)
    reads like the classic formats."""
    c = small()
    sav = random_sav(c, seed=2)
    d = c.dims
    names = ["jcross", "icross", "jdot", "idot", "khalf", "kfull", "nqx", "ntr"]
    lens = [d.jx - 1, d.iy - 1, d.jx, d.iy, d.kz, d.kz + 1, d.nqx, d.ntr]
    did = {n: q for q, n in enumerate(names)}
    vars_ = []
    for v, fdims in VARS.items():
        # Fortran order in memory = netCDF dimensions listed slowest first
        vars_.append((v, [did[n] for n in reversed(fdims)], sav[KEYS[v]].ravel(order="F")))
    path = tmp_path / "SAV.cdf5.nc"
    path.write_bytes(_cdf5_bytes(list(zip(names, lens)), [("idatex", "2001020300")], vars_))
    got = c.empty_sav()
    buf = C.create_string_buffer(16)
    assert abi.load().mlc_sav_read(str(path).encode(), C.byref(d), C.byref(c.sav_ptrs_of(got)),
                                   buf, 16) == 0
    assert buf.value == b"2001020300"
    for n, a in sav.items():
        assert np.array_equal(got[n], a), n
