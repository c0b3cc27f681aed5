"""Uneven batches and the serving pool.

Domains of different extents and level counts advance together, one launch
per kernel stage whose blocks come from a work list of the members' own
tiles; each one must reach exactly the state it reaches alone (where the
plain grids serve it), and stay at the FP64 oracle's state.  In a pool,
members join and leave between steps: a member's result is the same whether
it ran alone or in the mix, and the byte budget and slot count are enforced.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle.oracle import Oracle
from regcm_gb300 import abi
from regcm_gb300 import case as cs
from regcm_gb300.moloch import MolochBatch, MolochPool, domain_from_case

from .conftest import rel_l2

pytestmark = pytest.mark.gpu


def uneven(prec, ids=(0, 2, 6, 7), scale=0.25):
    # extents (30x55, 24x71, 56x25, 50x24) and 30, 41, 23, 41 levels
    return [cs.config3_member(m, scale=scale, precision=prec) for m in ids]


def alone_state(c, nsteps):
    d = domain_from_case(c)
    d.step(nsteps)
    g = c.empty_state()
    d.download(c.state_ptrs_of(g))
    d.close()
    return g


def member_state(ctx, m, c):
    g = c.empty_state()
    ctx.download(m, c.state_ptrs_of(g))
    return g


def test_uneven_extents_differ():
    dims = {c.dims.as_tuple() for c in uneven(abi.MLC_PREC_FP64)}
    assert len(dims) == 4
    assert len({d[2] for d in dims}) == 3  # level counts differ too


@pytest.mark.parametrize("prec", [abi.MLC_PREC_FP64, abi.MLC_PREC_MIXED])
def test_uneven_batch_equals_members_alone(prec):
    cases = uneven(prec)
    b = MolochBatch(cases)
    b.step(4)
    for m, c in enumerate(uneven(prec)):
        ga = alone_state(c, 4)
        gb = member_state(b, m, cases[m])
        for n in ga:
            assert np.array_equal(ga[n], gb[n]), (c.name, n)
    b.close()


def test_uneven_batch_against_oracle_fp64():
    cases = uneven(abi.MLC_PREC_FP64)
    b = MolochBatch(cases)
    b.step(3)
    for m, c in enumerate(uneven(abi.MLC_PREC_FP64)):
        orc = Oracle(c)
        st, _ = orc.step(3)
        assert st == 0
        ref = orc.state()
        orc.close()
        got = member_state(b, m, cases[m])
        for n in ("u", "v", "w", "tetav", "pai", "qx"):
            assert rel_l2(got[n], ref[n]) <= 1e-12, (c.name, n)
    b.close()


@pytest.mark.parametrize("col,vert,htile", [((32, 4), (32, 4), 0), ((64, 2), (64, 2), 1),
                                            ((64, 4), (32, 8), 2), ((16, 8), (128, 1), 3),
                                            ((128, 1), (32, 2), 0), ((32, 8), (32, 4), 1)])
def test_uneven_batch_every_launch_shape_fp64(col, vert, htile):
    """The work lists follow the launch shapes: with every point, column and
    tile shape an FP64 uneven batch equals its members run alone."""
    from regcm_gb300.moloch import DEFAULT_SHAPES
    cases = uneven(abi.MLC_PREC_FP64)
    b = MolochBatch(cases)
    b.set_launch_shapes(dict(DEFAULT_SHAPES, col_x=col[0], col_y=col[1], vert_x=vert[0],
                             vert_y=vert[1], htile=htile))
    b.step(2)
    for m, c in enumerate(uneven(abi.MLC_PREC_FP64)):
        ga = alone_state(c, 2)
        gb = member_state(b, m, cases[m])
        for n in ga:
            assert np.array_equal(ga[n], gb[n]), (c.name, n, col, vert, htile)
    b.close()


def test_uneven_batch_graph_matches_eager():
    a = MolochBatch(uneven(abi.MLC_PREC_MIXED))
    e = MolochBatch(uneven(abi.MLC_PREC_MIXED))
    e.set_graphs(False)
    a.step(3)
    e.step(3)
    for m in range(a.nmem):
        ga = member_state(a, m, a.cases[m])
        ge = member_state(e, m, e.cases[m])
        for n in ga:
            assert np.array_equal(ga[n], ge[n]), (m, n)


@pytest.mark.parametrize("graphs", [True, False])
def test_pool_join_leave_same_as_alone(graphs):
    prec = abi.MLC_PREC_MIXED

    def mk(r):
        return cs.config4_request(r, scale=0.12, precision=prec)[0]

    A, B, C = mk(0), mk(1), mk(2)
    pool = MolochPool(A.params, capacity=4)
    if not graphs:
        abi.check(pool.lib.mlc_set_graphs(pool._ctx, 0), "mlc_set_graphs")
    sa = pool.join(A)
    sb = pool.join(B)
    pool.step(3)
    sc = pool.join(C)
    pool.step(4)
    ga = member_state(pool, sa, A)
    pool.leave(sa)
    pool.step(2)
    gb = member_state(pool, sb, B)
    gc = member_state(pool, sc, C)
    pool.close()
    for r, got, n in ((0, ga, 7), (1, gb, 9), (2, gc, 6)):
        ref = alone_state(mk(r), n)
        for f in ref:
            assert np.array_equal(ref[f], got[f]), (r, f)


def test_pool_budget_and_slots():
    A, B = (cs.config4_request(r, scale=0.12)[0] for r in (0, 1))
    probe = MolochPool(A.params, capacity=1)
    fa, fb = probe.footprint(A.dims), probe.footprint(B.dims)
    probe.close()
    assert fa > 0 and fb > 0
    pool = MolochPool(A.params, capacity=3, budget_bytes=fa + fb - 1)
    assert pool.join(A) is not None
    assert pool.bytes_in_use() == fa
    assert pool.join(B) is None          # over the byte budget
    assert pool.bytes_in_use() == fa
    pool.leave(0)
    assert pool.bytes_in_use() == 0
    assert pool.join(B) is not None
    pool.close()
    full = MolochPool(A.params, capacity=1)
    assert full.join(A) is not None
    assert full.join(A) is None          # no free slot
    full.close()


def test_serve_stream_results_match_alone():
    from regcm_gb300.serve import Request, serve_stream
    prec = abi.MLC_PREC_MIXED

    def mk(r):
        return cs.config4_request(r, scale=0.1, precision=prec)[0]

    steps = [min(8, cs.config4_request(r, scale=0.1)[1]) for r in range(6)]
    reqs = [Request(r, 0.002 * r, steps[r], (lambda r=r: mk(r))) for r in range(6)]
    c0 = mk(0)
    probe = MolochPool(c0.params, capacity=1)
    budget = 2 * max(probe.footprint(mk(r).dims) for r in range(6))
    probe.close()
    summ = serve_stream(reqs, c0.params, budget, capacity=4, keep_results=True, workers=2)
    assert summ["requests"] == 6 and summ["max_resident"] <= 4
    assert summ["gp_steps"] == sum(mk(r).points * steps[r] for r in range(6))
    for r in reqs:
        ref = alone_state(mk(r.rid), r.steps)
        for f in ref:
            assert np.array_equal(ref[f], r.result[f]), (r.rid, f)
        assert r.t_done >= r.t_admit >= 0.0
