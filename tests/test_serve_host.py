"""Host logic of the serving loop (regcm_gb300/serve.py) without a GPU.

The pool and the plain single-domain path are replaced by fakes that keep
the same interface (join / step / download / leave, and a domain's step /
download / close), and the loop's clock by a fake time that the fakes
advance by a fixed cost a grid-point-step.  The tests then check the
scheduling itself:

* every request is advanced by exactly its number of steps while resident
  (the continuous batch never overshoots a member that finishes earlier);
* admission is first come, first served, within the byte budget and the
  slot count;
* the throughput and latency accounting of the service clock, and the
  first-come-first-served queue of the one-at-a-time baseline,
  finish(n) = max(arrival(n), finish(n-1)) + service(n).
"""
from __future__ import annotations

import types

import numpy as np
import pytest

from regcm_gb300 import abi
from regcm_gb300 import serve
from regcm_gb300.case import Case

STEP_COST = 1e-9      # fake seconds a grid-point-step
JOIN_COST = 2e-3      # fake seconds an upload and bind
BYTES_PER_POINT = 100


class FakeTime:
    def __init__(self):
        self.t = 0.0

    def perf_counter(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 0.0)


def fake_case(rid, nx, ny, kz):
    dims = abi.mlc_dims(nx + 1, ny + 1, kz, 5, 0)
    ps = np.zeros((nx, ny), order="F")
    return types.SimpleNamespace(
        name=f"r{rid}", rid=rid, dims=dims, points=nx * ny * kz, params=None,
        state={"ps": ps}, empty_state=lambda: {"ps": np.zeros_like(ps, order="F")},
        state_ptrs_of=Case.state_ptrs_of)


class FakePool:
    """The pool's interface on the host: byte budget and slots enforced as
    mlc_pool_add does, steps counted per resident member."""
    instances = []

    def __init__(self, params, capacity, budget_bytes):
        self.capacity, self.budget = capacity, budget_bytes
        self.res = {}          # slot -> [case, steps while resident]
        self.joined = []       # request ids in join order
        self.finished = {}     # request id -> steps while resident
        self.max_bytes = 0
        FakePool.instances.append(self)

    @staticmethod
    def bytes_of(dims):
        return dims.jx * dims.iy * dims.kz * BYTES_PER_POINT

    def footprint(self, dims):
        return self.bytes_of(dims)

    def used(self):
        return sum(self.bytes_of(c.dims) for c, _ in self.res.values())

    def join(self, case):
        serve.time.sleep(JOIN_COST)
        if len(self.res) == self.capacity or self.used() + self.bytes_of(case.dims) > self.budget:
            return None
        slot = min(set(range(self.capacity)) - set(self.res))
        self.res[slot] = [case, 0]
        self.joined.append(case.rid)
        self.max_bytes = max(self.max_bytes, self.used())
        return slot

    def step(self, n):
        assert n >= 1
        serve.time.sleep(n * STEP_COST * sum(c.points for c, _ in self.res.values()))
        for v in self.res.values():
            v[1] += n

    def download(self, slot, ptrs):
        assert isinstance(ptrs, abi.mlc_state_ptrs) and slot in self.res

    def leave(self, slot):
        case, steps = self.res.pop(slot)
        self.finished[case.rid] = steps

    def close(self):
        pass


@pytest.fixture
def fake_env(monkeypatch):
    ft = FakeTime()
    monkeypatch.setattr(serve, "time", types.SimpleNamespace(perf_counter=ft.perf_counter,
                                                             sleep=ft.sleep))
    monkeypatch.setattr(serve, "MolochPool", FakePool)
    FakePool.instances.clear()
    return ft


def make_stream(n, rate, seed, nmax=96):
    rng = np.random.default_rng(seed)
    arr = serve.poisson_arrivals(rate, n, seed)
    reqs = []
    for rid in range(n):
        nx, ny = (int(x) for x in rng.integers(16, nmax, 2))
        kz, steps = int(rng.choice([12, 20])), int(rng.integers(2, 40))
        reqs.append(serve.Request(rid, float(arr[rid]), steps,
                                  (lambda r=rid, a=nx, b=ny, k=kz: fake_case(r, a, b, k))))
    return reqs


@pytest.mark.parametrize("rate,capacity", [(2.0, 4), (50.0, 4), (500.0, 16)])
def test_stream_steps_admission_and_budget(fake_env, rate, capacity):
    reqs = make_stream(40, rate, seed=int(rate))
    budget = 3 * 97 * 97 * 20 * BYTES_PER_POINT   # about three of the largest requests
    out = serve.serve_stream(reqs, None, budget_bytes=budget, capacity=capacity, prefetch=4,
                             workers=2, max_chunk=8)
    pool = FakePool.instances[-1]
    # every request ran exactly its steps while resident, and left
    assert pool.finished == {r.rid: r.steps for r in reqs}
    assert not pool.res
    # first come, first served: joins in arrival order, admissions in order
    assert pool.joined == sorted(pool.joined)
    assert [r.t_admit for r in reqs] == sorted(r.t_admit for r in reqs)
    for r in reqs:
        assert r.arrival <= r.t_admit <= r.t_done
    # the budget and the slots held at every join
    assert pool.max_bytes <= budget
    assert out["max_resident"] <= capacity
    # accounting
    gp = sum(r.points * r.steps for r in reqs)
    assert out["gp_steps"] == gp and out["joins"] == len(reqs)
    assert out["makespan_s"] >= reqs[-1].arrival
    assert out["value"] == pytest.approx(gp / out["makespan_s"])
    lat = np.array([r.t_done - r.arrival for r in reqs])
    assert out["p50_s"] == pytest.approx(float(np.percentile(lat, 50)))
    assert out["p99_s"] == pytest.approx(float(np.percentile(lat, 99)))


def test_stream_service_clock_skips_idle_time(fake_env):
    """One request at a time (arrivals far apart): on the service clock a
    request's latency is its own join, steps and copy-back, and the makespan
    is the last arrival plus that."""
    reqs = [serve.Request(i, 100.0 * i, 5, (lambda r=i: fake_case(r, 32, 32, 10)))
            for i in range(3)]
    out = serve.serve_stream(reqs, None, budget_bytes=10 ** 9, capacity=4, prefetch=2, workers=1)
    service = JOIN_COST + 5 * STEP_COST * 32 * 32 * 10
    for r in reqs:
        assert r.t_done - r.arrival == pytest.approx(service)
    assert out["makespan_s"] == pytest.approx(200.0 + service)


def test_request_larger_than_the_budget_is_refused(fake_env):
    reqs = [serve.Request(0, 0.0, 3, lambda: fake_case(0, 64, 64, 20))]
    with pytest.raises(ValueError, match="more than the budget"):
        serve.serve_stream(reqs, None, budget_bytes=1000, capacity=2, prefetch=1, workers=1)


class FakeDomain:
    def __init__(self, case):
        self.case = case

    def step(self, n):
        serve.time.sleep(n * STEP_COST * self.case.points)

    def download(self, ptrs):
        assert isinstance(ptrs, abi.mlc_state_ptrs)

    def close(self):
        pass


def test_one_at_a_time_queue(fake_env, monkeypatch):
    monkeypatch.setattr(serve, "domain_from_case", FakeDomain)
    reqs = make_stream(25, 20.0, seed=7)
    out = serve.serve_one_at_a_time(reqs, lambda r: r.make, workers=2, prefetch=3)
    finish, lat, busy, gp = 0.0, [], 0.0, 0
    for r in reqs:
        c = r.make()
        service = r.steps * STEP_COST * c.points
        finish = max(r.arrival, finish) + service
        lat.append(finish - r.arrival)
        busy += service
        gp += c.points * r.steps
    assert out["makespan_s"] == pytest.approx(finish)
    assert out["service_s"] == pytest.approx([r.steps * STEP_COST * r.make().points for r in reqs])
    assert out["service_rate"] == pytest.approx(gp / busy)
    assert out["p50_s"] == pytest.approx(float(np.percentile(lat, 50)))
    assert out["p99_s"] == pytest.approx(float(np.percentile(lat, 99)))


def test_poisson_arrivals():
    a = serve.poisson_arrivals(8.0, 4000, seed=3)
    assert np.all(np.diff(a) > 0)
    assert len(a) / a[-1] == pytest.approx(8.0, rel=0.05)
    assert np.array_equal(a, serve.poisson_arrivals(8.0, 4000, seed=3))
