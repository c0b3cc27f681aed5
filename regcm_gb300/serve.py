"""Serving MOLOCH integrations: admission by device-memory footprint and
continuous batching over one ``MolochPool``.

A request is an initial state (a ``Case``) and a number of model steps.
Requests wait in arrival order; the head of the queue joins the pool as soon
as its arena fits the byte budget and a slot is free (first come, first
served: a large request at the head is not overtaken).  Every iteration
advances all resident members by one model step with one graph launch; a
member that has done its steps is copied back to the host and leaves, and its
bytes go to the next request in the queue.  A member's result does not
depend on the other members, so a request gets the same answer alone and in
the mix.

No counterpart in the reference, where each integration is a separate run of
the model executable (Main/mod_regcm_interface.F90).
"""
from __future__ import annotations

import time
from collections import deque
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .case import Case
from .moloch import MolochPool, domain_from_case


@dataclass
class Request:
    rid: int
    arrival: float            # seconds after the start of the stream
    steps: int
    make: object              # callable returning the request's Case
    case: object = None
    slot: int = -1
    done_steps: int = 0
    t_admit: float = 0.0
    t_done: float = 0.0
    result: dict = field(default_factory=dict)
    points: int = 0           # grid points of the request's domain (kept after its payload is released)
    ps_like: object = None    # the surface-pressure array's shape and type, for the result

    @property
    def latency(self) -> float:
        return self.t_done - self.arrival


def poisson_arrivals(rate: float, n: int, seed: int) -> np.ndarray:
    """n arrival times of a Poisson stream of `rate` per second."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, n))


def _prefetch(reqs, pool_exec, depth):
    """Build the next `depth` requests' cases in worker threads (the client
    preparing its payload before it arrives)."""
    futures = {}
    nxt = 0

    def fill():
        nonlocal nxt
        while nxt < len(reqs) and len(futures) < depth:
            r = reqs[nxt]
            futures[r.rid] = pool_exec.submit(r.make)
            nxt += 1

    def get(r):
        fill()
        c = futures.pop(r.rid).result()
        fill()
        return c

    fill()
    return get


class _Clock:
    """Server time.  'wall': seconds since the start.  'service': the sum of
    the durations of the server's own operations (joins, steps, result
    copies, departures), jumping forward to the next arrival when idle; the
    time the client takes to build a payload is not server time, so a load
    generator slower than the server does not thin the arrival stream."""

    def __init__(self, mode: str):
        if mode not in ("wall", "service"):
            raise ValueError(mode)
        self.mode = mode
        self.t0 = time.perf_counter()
        self.srv = 0.0

    def now(self) -> float:
        return time.perf_counter() - self.t0 if self.mode == "wall" else self.srv

    def run(self, fn, *a):
        t = time.perf_counter()
        out = fn(*a)
        self.srv += time.perf_counter() - t
        return out

    def idle_until(self, t: float):
        if self.mode == "wall":
            dt = t - self.now()
            if dt > 0:
                time.sleep(dt)
        else:
            self.srv = max(self.srv, t)


def serve_stream(reqs, params, budget_bytes: int, capacity: int = 256,
                 keep_results: bool = False, prefetch: int = 8, workers: int = 8,
                 clock: str = "service", max_chunk: int = 16):
    """Serve `reqs` (sorted by arrival).  Returns a summary dict; each request
    gets t_admit, t_done and (keep_results) its final state.

    Resident members advance together in chunks of steps: a chunk ends when
    the first member finishes, or about when the next request arrives (from
    the last measured step time), and is at most `max_chunk` steps."""
    pool = MolochPool(params, capacity, budget_bytes)
    queue = deque()
    active = {}
    pending = deque(reqs)
    ex = ThreadPoolExecutor(max_workers=workers)
    get_case = _prefetch(reqs, ex, prefetch)
    clk = _Clock(clock)
    steps_run = 0
    gp_steps = 0
    max_resident = 0
    step_s = 0.0
    joins = 0

    while pending or queue or active:
        t = clk.now()
        while pending and pending[0].arrival <= t:
            queue.append(pending.popleft())
        # admission in arrival order while the head fits; a request's payload
        # is taken from the prefetcher only when it reaches the head, so the
        # host holds the prefetched payloads and the head's, not the queue's
        while queue:
            r = queue[0]
            if r.case is None:
                r.case = get_case(r)
            slot = clk.run(pool.join, r.case)
            if slot is None:
                if not active:
                    raise ValueError(f"request {r.rid} needs {pool.footprint(r.case.dims)} bytes, "
                                     f"more than the budget of {budget_bytes}")
                break
            joins += 1
            queue.popleft()
            r.slot = slot
            r.t_admit = clk.now()
            r.points = r.case.points
            r.ps_like = r.case.state["ps"]
            if not keep_results:
                r.case = None  # the member's data is on the device now
            active[slot] = r
        if not active:
            if pending:
                clk.idle_until(pending[0].arrival)
            continue
        chunk = min(max_chunk, min(r.steps - r.done_steps for r in active.values()))
        if pending and step_s > 0:
            ahead = pending[0].arrival - clk.now()
            chunk = max(1, min(chunk, int(ahead / step_s) + 1))
        t = time.perf_counter()
        clk.run(pool.step, chunk)
        step_s = (time.perf_counter() - t) / chunk
        steps_run += chunk
        max_resident = max(max_resident, len(active))
        for slot in list(active):
            r = active[slot]
            r.done_steps += chunk
            gp_steps += r.points * chunk
            if r.done_steps >= r.steps:
                out = r.case.empty_state() if keep_results else {"ps": np.zeros_like(r.ps_like, order="F")}
                clk.run(pool.download, slot, Case.state_ptrs_of(out))
                clk.run(pool.leave, slot)
                r.t_done = clk.now()
                if keep_results:
                    r.result = out
                del active[slot]
                r.case = None  # release the host arrays
                r.ps_like = None
    makespan = clk.now()
    ex.shutdown()
    pool.close()
    lat = np.array([r.latency for r in reqs])
    return {"requests": len(reqs), "clock": clock, "makespan_s": makespan, "gp_steps": gp_steps,
            "value": gp_steps / makespan, "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "mean_s": float(lat.mean()),
            "pool_steps": steps_run, "joins": joins, "max_resident": max_resident}


def serve_one_at_a_time(reqs, make_fp64, workers: int = 8, prefetch: int = 4):
    """The same stream served by the plain FP64 single-domain path, one
    request after another in arrival order: each request's service time is
    measured (create, load, steps, result copy, release) and the first-come
    first-served queue gives its latency."""
    ex = ThreadPoolExecutor(max_workers=workers)
    fp64_reqs = [Request(r.rid, r.arrival, r.steps, make_fp64(r)) for r in reqs]
    get_case = _prefetch(fp64_reqs, ex, prefetch)
    finish = 0.0
    lat = []
    svc = []
    gp = 0
    busy = 0.0
    for r in fp64_reqs:
        c = get_case(r)
        t = time.perf_counter()
        d = domain_from_case(c)
        d.step(r.steps)
        out = {"ps": c.empty_state()["ps"]}
        d.download(c.state_ptrs_of(out))
        d.close()
        service = time.perf_counter() - t
        svc.append(service)
        start = max(r.arrival, finish)
        finish = start + service
        lat.append(finish - r.arrival)
        gp += c.points * r.steps
        busy += service
    ex.shutdown()
    lat = np.array(lat)
    return {"requests": len(reqs), "makespan_s": finish, "busy_s": busy, "gp_steps": gp,
            "value": gp / finish, "service_rate": gp / busy, "service_s": svc,
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean())}
