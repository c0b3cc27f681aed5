"""The benchmark's roofline arithmetic on the CPU: the algorithmic bytes and
FP64 operations per launch that the bench line divides by, for the default
workload (moist 512 x 512 x 41, 10 advected fields) and the dry domain with
a tracer, and the count of advected fields for every option that adds one
(Main/mod_moloch.F90:781-807)."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

from regcm_gb300 import abi
from regcm_gb300 import case as cs

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
import bench  # noqa: E402


@pytest.fixture(scope="module")
def c1():
    return cs.config1()


def test_advected_fields(c1):
    assert bench.n_adv_fields(c1) == 10                              # theta_v .. wx, 5 species
    assert bench.n_adv_fields(cs.config0()) == 7                     # dry: 6 and the tracer
    c = cs.config0()
    c.params.ipptls, c.dims.nqx, c.dims.ntr = 2, 5, 0
    assert bench.n_adv_fields(c) == 10
    c.params.ibltyp = 2
    assert bench.n_adv_fields(c) == 11                               # TKE
    c.params.ipptls = 0
    assert bench.n_adv_fields(c) == 7                                # qv only, TKE


def test_algorithmic_bytes_per_point(c1):
    c = c1
    d = c.dims
    pts = (d.jx - 1) * (d.iy - 1) * d.kz
    inner = (d.jx - 3) * (d.iy - 3) * d.kz
    nf = bench.n_adv_fields(c)
    # FP64: every advected field of type R = 8 bytes
    assert bench.kernel_bytes("adv_horizontal", c, nf, 8) == 272 * pts   # (3*10 + 4) * 8
    assert bench.kernel_bytes("sound_solve", c, nf, 8) == 88 * inner     # (4 + 7) * 8
    # mixed: 8 FP32 fields and theta_v, Exner as double-float pairs
    assert bench.kernel_bytes("sound_solve", c, nf, 4) == 72 * inner     # 4*4 + 7*8
    assert bench.kernel_bytes("adv_horizontal", c, nf, 4) == 112 * pts   # (3*8 + 4) * 4
    assert bench.kernel_bytes("adv_horizontal_inc", c, nf, 4) == 64 * pts  # 3*2*8 + 4*4
    assert bench.kernel_bytes("adv_horizontal_inc", c, nf, 8) is None  # no such launch in FP64
    assert bench.kernel_bytes("no_such_kernel", c, nf, 8) is None


def test_algorithmic_fp64_operations(c1):
    c = c1
    d = c.dims
    pts = (d.jx - 1) * (d.iy - 1) * d.kz
    nf = bench.n_adv_fields(c)
    assert bench.kernel_fp64_ops("adv_horizontal", c, nf) == (50 * 10 + 24) * pts
    assert bench.kernel_fp64_ops("adv_vertical", c, nf) == (48 * 10 + 18) * pts
    assert bench.kernel_fp64_ops("sound_div", c, nf) is None


@pytest.mark.parametrize("prec", [abi.MLC_PREC_FP64, abi.MLC_PREC_MIXED])
def test_captured_traffic_keys_match_the_dominant_kernels(prec):
    """The constants the line labels as captured belong to the kernel group
    that dominates each precision's step on the default workload."""
    name = "adv_horizontal" if prec == abi.MLC_PREC_FP64 else "sound_solve"
    key = (name, "fp64" if prec == abi.MLC_PREC_FP64 else "mixed", 10)
    per_point, build = bench.CAPTURED_TRAFFIC_PER_POINT[key]
    assert per_point > 0 and build
