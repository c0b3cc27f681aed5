"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares; error paths that need no device behave like the
reference's fatal() checks."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import pytest

from regcm_gb300 import abi

HEADERS = sorted((Path(__file__).resolve().parent.parent / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
        for m in re.finditer(r"\b(?:int|void|size_t|const char\s*\*)\s*(mlc_\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_entry_points():
    names = declared_functions()
    for n in ("mlc_create", "mlc_bind_static", "mlc_upload_state", "mlc_download_state",
              "mlc_set_boundary", "mlc_step", "mlc_destroy", "mlc_strerror"):
        assert n in names


@pytest.mark.parametrize("name", declared_functions())
def test_library_exports(name):
    lib = C.CDLL(str(abi.lib_path()))
    assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_strerror_and_defaults():
    lib = abi.load()
    assert lib.mlc_strerror(abi.MLC_ERR_NONFINITE).decode().startswith("CFL VIOLATION")
    p = abi.mlc_params()
    lib.mlc_default_params(C.byref(p))
    # reference defaults, Share/mod_dynparam.F90:203-211
    assert (p.mo_ztop, p.mo_h, p.mo_a0, p.mo_nadv, p.mo_nsound) == (30000.0, 8000.0, 0.0, 2, 5)
    assert p.mo_divdamp == p.mo_divfilter == p.mo_top_nudge == 1


def test_create_rejects_bad_input_before_touching_the_device():
    lib = abi.load()
    p = abi.mlc_params()
    lib.mlc_default_params(C.byref(p))
    ctx = C.c_void_p()
    # too few levels / spectral nudging without an interval / no output pointer
    assert lib.mlc_create(C.byref(abi.mlc_dims(65, 65, 2, 2, 0)), C.byref(p), C.byref(ctx)) == \
        abi.MLC_ERR_INVALID
    p.mo_spectral_nudge = 1
    p.dtrad = 0.0
    assert lib.mlc_create(C.byref(abi.mlc_dims(65, 65, 30, 2, 0)), C.byref(p), C.byref(ctx)) == \
        abi.MLC_ERR_INVALID
    p.mo_spectral_nudge = 0
    p.dtrad = 1800.0
    p.ipptls = 2
    assert lib.mlc_create(C.byref(abi.mlc_dims(65, 65, 30, 2, 0)), C.byref(p), C.byref(ctx)) == \
        abi.MLC_ERR_INVALID  # ipptls 2 needs qv..qs


def test_footprint_grows_with_domain():
    lib = abi.load()
    a = lib.mlc_footprint_bytes(C.byref(abi.mlc_dims(65, 65, 30, 2, 1)), abi.MLC_PREC_FP64)
    b = lib.mlc_footprint_bytes(C.byref(abi.mlc_dims(513, 513, 41, 5, 0)), abi.MLC_PREC_FP64)
    c = lib.mlc_footprint_bytes(C.byref(abi.mlc_dims(513, 513, 41, 5, 0)), abi.MLC_PREC_MIXED)
    assert 0 < a < b and c < b


def test_struct_layouts_match_the_headers(tmp_path):
    """Every ctypes structure of the bindings has the size and field offsets
    the C compiler gives the header's structure (guards against drift)."""
    import ctypes as C
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = [abi.mlc_dims, abi.mlc_params, abi.mlc_static_ptrs, abi.mlc_state_ptrs,
               abi.mlc_bdy_ptrs, abi.mlc_diag, abi.mlc_tune_report, abi.mlc_tend_ptrs,
               abi.mlc_sav_fields]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "moloch_gb300.h"',
             '#include "moloch_gb300_setup.h"', '#include "moloch_gb300_restart.h"',
             'int main(void) {']
    for st in structs:
        n = st.__name__
        lines.append(f'  printf("{n} size %zu\\n", sizeof({n}));')
        for f, _ in st._fields_:
            lines.append(f'  printf("{n} {f} %zu\\n", offsetof({n}, {f}));')
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = Path(__file__).resolve().parent.parent / "include"
    subprocess.run([cc, "-std=c99", "-I", str(inc), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        a, b, v = line.split()
        got[(a, b)] = int(v)
    for st in structs:
        n = st.__name__
        assert got[(n, "size")] == C.sizeof(st), n
        for f, _ in st._fields_:
            assert got[(n, f)] == getattr(st, f).offset, (n, f)


def test_fortran_shim_types_follow_the_headers():
    """The bind(c) derived types of the Fortran shim list the same fields, in
    the same order and of matching kinds, as the ctypes structures (the shim
    is not compiled here: no Fortran compiler)."""
    import ctypes as C

    src = (Path(__file__).resolve().parent.parent / "regcm_gb300" / "fortran" /
           "mod_moloch_gb300.F90").read_text()
    kinds = {"real(c_double)": "d", "integer(c_int32_t)": "i", "type(c_ptr)": "p"}
    types = {}
    for m in re.finditer(r"type, bind\(c\) :: (\w+)\n(.*?)end type", src, re.S):
        fields = []
        for line in m.group(2).splitlines():
            line = line.strip()
            if not line:
                continue
            decl, names = line.split("::")
            k = kinds[decl.strip()]
            for nm in names.split(","):
                nm = nm.strip()
                cnt = 1
                mm = re.match(r"(\w+)\((\d+)\)", nm)
                if mm:
                    nm, cnt = mm.group(1), int(mm.group(2))
                fields.append((nm, k, cnt))
        types[m.group(1)] = fields

    def kind_of(t):
        if isinstance(t, type) and issubclass(t, C.Array):
            return kind_of(t._type_)[0], t._length_
        if t is C.c_double:
            return "d", 1
        if t in (C.c_int32, C.c_int):
            return "i", 1
        return "p", 1

    for st in (abi.mlc_dims, abi.mlc_params, abi.mlc_static_ptrs, abi.mlc_state_ptrs,
               abi.mlc_bdy_ptrs, abi.mlc_diag, abi.mlc_tend_ptrs):
        want = [(n,) + kind_of(t) for n, t in st._fields_]
        assert types[st.__name__] == want, st.__name__


def _gpu_present() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_gpu_present(), reason="checks the behaviour on a host without a GPU")
def test_no_gpu_means_an_error_not_a_fallback():
    """Without a device the library refuses to create a domain (there is no
    CPU path behind the ABI), and the Python mirror raises."""
    from regcm_gb300 import case as cs
    from regcm_gb300.moloch import domain_from_case
    lib = abi.load()
    c = cs.build(24, 22, 12, dx=12000.0, dt=60.0, nsound=3, moist=False, seed=1, name="nogpu")
    ctx = C.c_void_p()
    st = lib.mlc_create(C.byref(c.dims), C.byref(c.params), C.byref(ctx))
    assert st != abi.MLC_OK and not ctx.value
    with pytest.raises(abi.MolochError):
        domain_from_case(c)
