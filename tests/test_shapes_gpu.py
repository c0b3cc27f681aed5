"""Launch shapes do not change results.

Every horizontal WAF tile shape and the other block shapes the autotuner may
pick must give the state of the fixed configuration: the tiles of the
horizontal WAF overlap and split rows differently for each shape, so this
exercises their edges, the overlap of consecutive tiles along j (a member
wider than one tile) and the partial last tile along i (tests/test_mixed_gpu.py
checks each shape pointwise against the oracle).  FP64 members agree bit for
bit.  The FP32 fields of a mixed member may differ by a few FP32
roundings at a few points (the compiler may fuse a multiply-add differently
in each tile shape's instantiation; measured after one step: at most 1.6e-7
of the field's largest value, at under 0.1 % of the points, with theta_v and
Exner bit for bit), and later steps carry such differences into the other
fields; an indexing error would show as differences of order the increments
themselves.  Shapes outside the autotuner's candidates are refused.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from regcm_gb300 import abi
from regcm_gb300 import case as cs
from regcm_gb300.moloch import DEFAULT_SHAPES, MolochBatch

pytestmark = pytest.mark.gpu

SHAPES = [dict(DEFAULT_SHAPES, htile=h) for h in (1, 2, 3)] + [
    dict(DEFAULT_SHAPES, vert_x=64, vert_y=2, col_x=64, col_y=4, solve_x=64, solve_y=1),
    dict(DEFAULT_SHAPES, vert_x=128, vert_y=1, col_x=128, col_y=1, solve_x=16, solve_y=4, htile=2),
]


def members(prec):
    # 30x55, 24x71 and 56x25 points at scale 0.25; 224x100 (four 64-column
    # tiles, eight 32-column tiles) at scale 1
    return ([cs.config3_member(m, scale=0.25, precision=prec) for m in (0, 2)] +
            [cs.config3_member(6, scale=1.0, precision=prec)])


def run(prec, shapes, nsteps=3):
    cases = members(prec)
    b = MolochBatch(cases)
    if shapes is not None:
        b.set_launch_shapes(shapes)
    b.step(nsteps)
    out = []
    for m, c in enumerate(cases):
        g = c.empty_state()
        b.download(m, c.state_ptrs_of(g))
        out.append(g)
    b.close()
    return out


@pytest.mark.parametrize("prec", [abi.MLC_PREC_FP64, abi.MLC_PREC_MIXED])
def test_shapes_same_state(prec):
    ref = run(prec, None)
    for sh in SHAPES:
        got = run(prec, sh)
        for m in range(len(ref)):
            for n in ref[m]:
                a, b = ref[m][n], got[m][n]
                if prec == abi.MLC_PREC_FP64:
                    assert np.array_equal(a, b), (sh, m, n)
                else:
                    # well inside the mixed precision's own distance from FP64
                    # (after one step up to 4e-5 of the largest v)
                    d = np.abs(a - b).max()
                    assert d <= 2e-5 * np.abs(a).max(), (sh, m, n, d)


def test_unknown_shapes_refused():
    c = cs.config3_member(0, scale=0.25, precision=abi.MLC_PREC_MIXED)
    b = MolochBatch([c])
    rep = abi.mlc_tune_report(col_x=48, col_y=4, solve_x=32, solve_y=2, vert_x=32, vert_y=4, htile=0)
    assert b.lib.mlc_set_launch_shapes(b._ctx, C.byref(rep)) == abi.MLC_ERR_INVALID
    rep = abi.mlc_tune_report(col_x=32, col_y=4, solve_x=32, solve_y=2, vert_x=32, vert_y=4, htile=4)
    assert b.lib.mlc_set_launch_shapes(b._ctx, C.byref(rep)) == abi.MLC_ERR_INVALID
    b.close()
