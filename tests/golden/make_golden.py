"""Regression fixtures of the CPU oracle (tests/golden/oracle_fixtures.json).

RegCM ships no golden vectors for the MOLOCH step and its Fortran cannot be
built here, so these fixtures do not come from the reference: they record the
oracle's own results on small seeded cases, so that any later change to the
oracle (or to the case builder) that moves its output shows up in
tests/test_golden.py.  Per case and field: the shape, the sum and the sum of
squares, and the values at 24 seeded points.

    python tests/golden/make_golden.py        # rewrites the fixture file
"""
from __future__ import annotations

import json
import sys
import zlib
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from oracle.oracle import Oracle  # noqa: E402
from regcm_gb300 import case as cs  # noqa: E402

OUT = Path(__file__).resolve().parent / "oracle_fixtures.json"
FIELDS = ("u", "v", "w", "pai", "tetav", "t", "ps", "qx", "trac")


def cases():
    """Name -> (case builder, steps, tendency seeds per step or None)."""
    def dry(**kw):
        return cs.build(24, 22, 12, dx=12000.0, dt=60.0, nsound=3, moist=False, seed=3,
                        hills=[(12 * 12000.0, 11 * 12000.0, 600.0)], wind=10.0,
                        theta_noise=0.3, tracer=True, name="golden_dry", **kw)

    def moist(**kw):
        return cs.build(40, 38, 14, dx=3000.0, dt=20.0, nsound=4, moist=True, seed=4,
                        hills=[(20 * 3000.0, 18 * 3000.0, 1200.0)], jet=True,
                        theta_noise=0.2, tracer=True, name="golden_moist", **kw)

    return {
        "dry_tracer_5": (lambda: dry(), 5, None),
        "moist_3": (lambda: moist(), 3, None),
        "rotllr_3": (lambda: dry(lrotllr=True), 3, None),
        "spectral_every_step_3": (lambda: dry(spectral=True, dtrad=60.0), 3, None),
        "physics_tendencies_3": (lambda: moist(), 3, [31, 32, 33]),
    }


def run(make, steps, seeds):
    c = make()
    o = Oracle(c)
    if seeds is None:
        st, _ = o.step(steps)
        assert st == 0
    else:
        keep = []  # the arrays behind the pointers stay alive through the call
        for s in seeds:
            assert o.step_dynamics() == 0
            ten = c.tendencies(seed=s)
            tp = c.tend_ptrs_of(ten)
            keep.append((ten, tp))
            assert o.set_tendencies(tp) == 0
            assert o.step_finish()[0] == 0
    out = o.state()
    o.close()
    return out


def summary(a: np.ndarray, rng) -> dict:
    flat = np.asarray(a, dtype=np.float64).ravel(order="F")
    idx = sorted(int(i) for i in rng.choice(flat.size, size=min(24, flat.size), replace=False))
    return {"shape": list(a.shape), "sum": float(np.sum(flat)), "sumsq": float(np.sum(flat * flat)),
            "points": [[i, float(flat[i])] for i in idx]}


def build() -> dict:
    fx = {}
    for name, (make, steps, seeds) in cases().items():
        st = run(make, steps, seeds)
        rng = np.random.default_rng(zlib.crc32(name.encode()))
        fx[name] = {f: summary(st[f], rng) for f in FIELDS if f in st}
    return fx


if __name__ == "__main__":
    OUT.write_text(json.dumps(build(), separators=(",", ":")) + "\n")
    print(f"wrote {OUT}")
