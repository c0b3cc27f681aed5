#!/usr/bin/env python3
"""Benchmark of the MOLOCH step: grid-point-steps per second on one GB300.

Workload (default): the moist convection-permitting domain, 512 x 512 cross
points x 41 levels, dx 3 km, dt 20 s, 4 acoustic substeps, FP64, with the
seeded synthetic initial state of regcm_gb300.case.config1 (no netCDF input
exists here; the recipe stands in for RegCM's ICBC files).  A step is one full
MOLOCH model step (acoustic substeps, WAF advection of 10 fields, boundary
relaxation, diagnostics, status update, mass budget).

Our arm prints one JSON line with
  value      device-resident gp-steps/s (CUDA events on the library stream),
  e2e        the same metric through the C ABI with host buffers: per step
             upload of the prognostic inputs from pinned memory, the step,
             download of the full state,
  roofline   the dominant kernel against what bounds it: in FP64 the FP64
             pipe (algorithmic FP64 operations per launch / its average launch
             time, against the FP64 multiply-add rate measured in the same run
             by mlc_fp64_peak), with its HBM figures beside; in mixed
             precision HBM (algorithmic bytes / launch time against the
             measured copy bandwidth),
  cpu_baseline  the CPU oracle (FP64 C++ restatement of the reference, OpenMP
             on all host cores, and on one core) timed on a bounded sample of
             the same domain.
`--impl reference` times that CPU implementation alone (the reference's own
Fortran cannot be built here: no Fortran compiler, MPI or netCDF).  Its input
is built through the oracle's own setup routines, so that arm never loads the
GPU library.

Multi-GPU: replicas only (each rank advances its own domain; no data-path
collective); value = all ranks' gp-steps / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import resource
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "grid-point-steps/s"
UNIT = "gp-steps/s"


def peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


# ---- clocks during the timed region ---------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not Path(self.path).exists():
            return None
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- algorithmic bytes per launch of each kernel group ---------------------
def kernel_bytes(name: str, case, nadv_fields: int, wbytes: int) -> float | None:
    """Compulsory HBM bytes each launch must move.

    Counts follow the fusion contract 'each kernel reads its inputs and writes
    its outputs once'; 2-D and 1-D arrays are ignored.  Per point (cross
    point x level) of the launch's domain, with R the field type (wbytes) and
    D = 8 bytes (the Exner function and theta_v: FP64, or a double-float pair
    of FP32 planes in a mixed member; the FP64 solve also reads fmz, fmzf):
      sound_div           u, v, rfmzu, rfmzv, fmz -> zdiv2, s               7 R
      sound_solve         zdiv2, s, w -> w                                  4 R
                          pai, tetav, tetavf, fmz, fmzf -> pai, tetavf      7 D
      sound_momentum      u, v, zdiv2 -> u, v                               5 R
                          pai, tetav                                        2 D
      adv_vertical        per field of type R: field -> wz (2 R); shared s, zrfmu, zrfmd (3 R)
      adv_horizontal      per field of type R: field, wz -> out (3 R); shared u, v, fmz, rfmzu (4 R)
      adv_vertical_inc    theta_v, Exner of a mixed member: field -> increment (2 D each); 3 R shared
      adv_horizontal_inc  the same two: field, increment -> out (3 D each); 4 R shared
    In an FP64 member every advected field is of type R.
    """
    d = case.dims
    pts = (d.jx - 1) * (d.iy - 1) * d.kz
    inner = (d.jx - 3) * (d.iy - 3) * d.kz
    r, w = wbytes, 8
    nd = 2 if wbytes == 4 else 0     # double-float fields of a mixed member
    nr = nadv_fields - nd            # fields of type R
    by = {
        "sound_div": 7 * r * pts,
        "sound_solve": (4 * r + 7 * w) * inner,
        "sound_momentum": (5 * r + 2 * w) * pts,
        "adv_vertical": (2 * nr + 3) * r * pts,
        "adv_horizontal": (3 * nr + 4) * r * pts,
        "adv_vertical_inc": (2 * nd * w + 3 * r) * pts if nd else None,
        "adv_horizontal_inc": (3 * nd * w + 4 * r) * pts if nd else None,
    }.get(name)
    return None if by is None else float(by)


# DRAM bytes per point of a launch (dram__bytes_read.sum + dram__bytes_write.sum)
# from one ncu capture of the same kernel and precision on the quarter-size
# case (moist 256x256x41, 10 advected fields), scaled to the bench case by its
# points.  These are constants from that capture, not measured by this run:
# the line prints them with that label and the kernel build they were taken
# on.  Keyed by (kernel group, precision, advected fields).
CAPTURED_TRAFFIC_PER_POINT = {
    ("adv_horizontal", "fp64", 10): (733.3e6 / (256 * 256 * 41), "b130abd"),
    ("sound_solve", "mixed", 10): (243.0e6 / (256 * 256 * 41), "b130abd"),
}
# What limits the dominant kernel besides its roofline, from the same captures.
CAPTURED_LIMITER = {
    ("adv_horizontal", "fp64"): {
        "pipe": "fp64", "active": 0.84, "counter": "sm__inst_executed_pipe_fp64"},
    ("sound_solve", "mixed"): {
        "stall": "block barrier (one a level, freeing a copy stage)", "warps_active": 0.21},
}


def kernel_fp64_ops(name: str, case, nadv_fields: int) -> float | None:
    """Algorithmic FP64 operations of one launch of an FP64 member's kernel
    group: the arithmetic the reference performs for the same results,
    counted from Main/mod_moloch.F90 with each add, multiply, divide, min
    and max one operation (a multiply-add is two), and the factors that do
    not depend on the advected field counted once per point.

      adv_horizontal  (wafone :949-1040, per direction) limiter flux of a
                      field: 2 differences, r = num/den, 2r, 4 min/max,
                      zphi (2 products, 2 sums), 1 +- zphi, the two products,
                      their sum and the product by 0.5 v = 18; update of p0
                      or pp: zdv's product by pp, the flux terms (2 products,
                      2 sums), mx2 * (...) and the sum = 7.  Field-independent
                      per point and direction: zamu (2), 0.5 v (1), zrfmn/s
                      (4), zdv's factor (5) = 12.  Both directions:
                      50 F + 24 per point.
      adv_vertical    (:862-922, do_vadvtwice) per pass and field: the same
                      flux (18) and update (zdv's product, 2 products, 3
                      sums = 6); field-independent: zamu (1), 0.5 s (1),
                      zrfmu/zrfmd (4), zdv's factor (3) = 9.  Two passes:
                      48 F + 18 per point.
      sound_solve     (:627-671) per interior point: tetavf (5), zrom1w (2),
                      zwexpl (13), zu/zd (8), zrapp (5, one divide), w and
                      wwkw (4), back substitution (2), Exner update (7),
                      filtered divergence (5-point Laplacian, 7), its
                      vertical term (5) = 58.
    """
    d = case.dims
    pts = (d.jx - 1) * (d.iy - 1) * d.kz
    inner = (d.jx - 3) * (d.iy - 3) * d.kz
    f = nadv_fields
    ops = {
        "adv_horizontal": (50 * f + 24) * pts,
        "adv_vertical": (48 * f + 18) * pts,
        "sound_solve": 58 * inner,
    }.get(name)
    return None if ops is None else float(ops)


def n_adv_fields(case) -> int:
    """Advected fields of a member: theta_v, Exner, ux, vx, wx, qv, the other
    species when ipptls > 0, TKE when ibltyp = 2, the tracers
    (Main/mod_moloch.F90:781-807)."""
    p, d = case.params, case.dims
    return 6 + (d.nqx - 1 if p.ipptls > 0 else 0) + (1 if p.ibltyp == 2 else 0) + d.ntr


def make_case(args, rank=0, setup=None):
    from regcm_gb300 import abi
    from regcm_gb300 import case as cs
    prec = abi.MLC_PREC_MIXED if args.precision == "mixed" else abi.MLC_PREC_FP64
    if args.config == "c1":
        n = args.size or 512
        return cs.config1(nx=n, ny=n, seed=1 + rank, precision=prec, setup=setup)
    if args.config == "c0":
        n = args.size or 64
        return cs.config0(nx=n, ny=n, seed=rank, precision=prec, setup=setup)
    raise SystemExit(f"unknown config {args.config}")


def config_of(args, world, points):
    """The workload description both arms print."""
    return {"workload": workload_name(args), "points_per_domain": points,
            "precision": args.precision, "parallelism": f"replicas{world}",
            "l2": "inputs larger than L2 (state > 1 GB)"}


def workload_name(args):
    if args.config == "c1":
        n = args.size or 512
        return f"moloch-moist-{n}x{n}x41-dx3km-dt20-ns4"
    n = args.size or 64
    return f"moloch-dry-{n}x{n}x30-dx12km-dt60-ns3"


# ---- CPU oracle timing -------------------------------------------------------
def time_oracle(case, steps: int, warmup: int = 1, budget_s: float = 30.0, threads: int = 0):
    """gp-steps/s of the CPU oracle on `case` (`threads` OpenMP threads; 0 =
    every host thread this process may use)."""
    from oracle.oracle import Oracle, set_threads
    set_threads(threads or cpu_threads())
    o = Oracle(case)
    t0 = time.perf_counter()
    for _ in range(warmup):
        o.step(1)
    t1 = time.perf_counter()
    per = (t1 - t0) / max(warmup, 1)
    n = max(1, min(steps, int(budget_s / max(per, 1e-6))))
    t0 = time.perf_counter()
    st, _ = o.step(n)
    dt = time.perf_counter() - t0
    o.close()
    return case.points * n / dt, n, dt


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# ---- the reference arm -------------------------------------------------------
def run_reference(args, rank, world):
    """The CPU oracle alone on the same workload.  The domain is built by the
    oracle's restatement of the setup routines (bit-identical to the
    library's, tests/test_setup_parity.py), so this arm never maps the GPU
    library."""
    if rank != 0:
        return
    from oracle.oracle import OracleSetup
    threads = cpu_threads()
    case = make_case(args, setup=OracleSetup())
    value, n, dt = time_oracle(case, args.steps, warmup=max(1, min(args.warmup, 2)),
                               budget_s=150.0, threads=threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": n, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / n,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_of(args, world, case.points),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads,
                         "kind": "port",
                         "sample": f"{n} full steps of the {workload_name(args)} domain "
                                   "(CPU oracle: C++ FP64 restatement of Main/mod_moloch.F90; the "
                                   "reference Fortran needs gfortran, MPI and netCDF, absent here)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def max_over_ranks(seconds: float, world: int) -> float:
    """The slowest rank's time, which is the whole job's: an all-reduce over
    the process group on its own device (the GPU for NCCL, the host for
    gloo).  One process alone returns its own time."""
    if world <= 1:
        return seconds
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([seconds], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---- our arm -----------------------------------------------------------------
def pinned_like(arrays: dict) -> dict:
    import torch
    out = {}
    for k, v in arrays.items():
        t = torch.empty(v.size, dtype=torch.float64, pin_memory=True)
        a = t.numpy().reshape(v.shape, order="F")
        a[...] = v
        out[k] = (a, t)
    return out


def run_ours(args, rank, world):
    import torch
    from regcm_gb300 import abi
    from regcm_gb300.moloch import domain_from_case

    lib = abi.load()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    case = make_case(args, rank)
    dom = domain_from_case(case)
    ctx = dom._ctx
    lib.mlc_step_timed.argtypes = [C.c_void_p, C.c_int, C.POINTER(abi.mlc_diag),
                                   C.POINTER(C.c_float)]

    # warm-up (records the step graphs)
    dom.step(args.warmup)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    diag = abi.mlc_diag()
    ms = C.c_float()
    with ClockSampler(dev) as clk:
        st = lib.mlc_step_timed(ctx, args.steps, C.byref(diag), C.byref(ms))
    abi.check(st, "mlc_step_timed")
    torch.cuda.synchronize()
    t_dev = ms.value / 1000.0
    t_dev = max_over_ranks(t_dev, world)
    if world > 1:
        torch.distributed.barrier()
    pts = case.points
    value = pts * args.steps * world / t_dev
    launches = dom.launches_per_step()

    roofline = kernel_roofline(lib, ctx, case, args.precision)

    # end-to-end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        inputs = {k: case.state[k] for k in ("u", "v", "w", "pai", "tetav", "qx")}
        if case.dims.ntr:
            inputs["trac"] = case.state["trac"]
        pin_in = pinned_like(inputs)
        pin_out = pinned_like(case.empty_state())
        sp_in = case.state_ptrs_of({k: v[0] for k, v in pin_in.items()})
        sp_out = case.state_ptrs_of({k: v[0] for k, v in pin_out.items()})
        h2d = sum(v[0].nbytes for v in pin_in.values())
        d2h = sum(v[0].nbytes for v in pin_out.values())
        ne = max(2, min(args.steps, 10))
        dom.upload(sp_in)
        dom.step(1)
        dom.download(sp_out)
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(ne):
            dom.upload(sp_in)
            dom.step(1)
            dom.download(sp_out)
        te = time.perf_counter() - t0
        te = max_over_ranks(te, world)
        e2e = {"value": pts * ne * world / te, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "steps": ne, "ms_per_step": 1000.0 * te / ne}
    dom.close()

    side = None
    if args.precision == "fp64" and not args.no_mixed:
        side = run_mixed_side(args, rank)
    if args.precision == "fp64" and world == 1 and not args.no_ensemble and args.config == "c1":
        # the batched form the scope targets, measured in the same run: the
        # 64-member ensemble of 128x128x30 domains in mixed precision with
        # autotuned launch shapes, against the plain FP64 single-domain path
        import copy
        eargs = copy.copy(args)
        eargs.config, eargs.members, eargs.size, eargs.precision = "c2", 64, 0, "mixed"
        eargs.no_tune = False
        ens = ensemble_line(eargs, rank, world)
        if ens is not None:
            side = dict(side or {})
            side["ensemble"] = {
                "workload": ens["config"]["workload"], "value": ens["value"], "unit": UNIT,
                "ms_per_step": ens["ms_per_step"], "dtype": ens["dtype"],
                "plain_fp64_single_domain": ens["side_by_side"]["plain_fp64_single_domain"],
                "ratio_to_plain_fp64": ens["side_by_side"]["ratio_to_plain_fp64"],
                "autotune": ens["side_by_side"]["autotune"], "roofline": ens["roofline"],
                "gpu_launches": ens["gpu_launches"]}
    if rank != 0:
        return
    cpu = None
    if world == 1 and not args.no_cpu:
        threads = cpu_threads()
        cv, n, dt = time_oracle(case, steps=5, warmup=1, budget_s=20.0, threads=threads)
        c1, n1, dt1 = time_oracle(case, steps=1, warmup=0, budget_s=1.0, threads=1)
        cpu = {"value": cv, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{n} full steps of the same domain on the CPU oracle (C++ FP64, OpenMP)",
               "single_core": {"value": c1, "unit": UNIT, "cores": 1,
                               "sample": f"{n1} full step of the same domain, one thread",
                               "seconds": dt1}}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
        "config": config_of(args, world, pts),
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "side_by_side": side,
        "gpu_launches": launches * args.steps, "clocks": clk.summary(),
        "diag": {"ps_min": diag.ps_min, "ps_max": diag.ps_max, "drymass": diag.drymass},
    }
    print(json.dumps(line), flush=True)


def run_ensemble(args, rank, world):
    line = ensemble_line(args, rank, world)
    if rank == 0:
        print(json.dumps(line), flush=True)


def ensemble_line(args, rank, world):
    """Ensemble workload: members of the dry recipe (128x128x30, dx 12 km,
    dt 60 s, 3 substeps, theta noise +-0.5 K and wind U(5,20) per member)
    advanced by one launch per kernel stage, autotuned launch shapes; next to
    the plain single-domain FP64 path on one member.  Returns the JSON line
    (rank 0; None elsewhere)."""
    import torch
    from regcm_gb300 import abi
    from regcm_gb300 import case as cs
    from regcm_gb300.moloch import MolochBatch, domain_from_case

    class KT(C.Structure):
        _fields_ = [("name", C.c_char * 32), ("launches", C.c_int32), ("ms", C.c_double)]

    lib = abi.load()
    lib.mlc_step_timed.argtypes = [C.c_void_p, C.c_int, C.POINTER(abi.mlc_diag),
                                   C.POINTER(C.c_float)]
    lib.mlc_profile_steps.argtypes = [C.c_void_p, C.c_int, C.POINTER(KT), C.c_int,
                                      C.POINTER(C.c_int)]
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    n = args.size or 128
    nmem = args.members
    prec = abi.MLC_PREC_FP64 if args.precision == "fp64" else abi.MLC_PREC_MIXED
    cases = [cs.config2_member(rank * nmem + m, nx=n, ny=n, kz=30, precision=prec)
             for m in range(nmem)]
    pts = cases[0].points
    batch = MolochBatch(cases)
    batch.step(args.warmup)
    tune = None if args.no_tune else batch.autotune(2)
    batch.step(2)  # re-record graphs with the picked shapes
    if world > 1:
        torch.distributed.barrier()
    diag = abi.mlc_diag()
    ms = C.c_float()
    with ClockSampler(dev) as clk:
        abi.check(lib.mlc_step_timed(batch._ctx, args.steps, C.byref(diag), C.byref(ms)), "batch")
    t_dev = ms.value / 1000.0
    t_dev = max_over_ranks(t_dev, world)
    value = pts * nmem * args.steps * world / t_dev
    ktab = (KT * 32)()
    nk = C.c_int()
    abi.check(lib.mlc_profile_steps(batch._ctx, 1, ktab, 32, C.byref(nk)), "profile")
    kernels = {ktab[i].name.decode(): (ktab[i].launches, ktab[i].ms) for i in range(nk.value)}
    launches = batch.launches_per_step()
    batch.close()
    # plain single-domain FP64 path on member 0's recipe
    single = cs.config2_member(rank * nmem, nx=n, ny=n, kz=30, precision=abi.MLC_PREC_FP64)
    d = domain_from_case(single)
    d.step(args.warmup)
    ms1 = C.c_float()
    abi.check(lib.mlc_step_timed(d._ctx, args.steps, C.byref(diag), C.byref(ms1)), "single")
    d.close()
    plain = pts * args.steps / (ms1.value / 1000.0)
    if rank != 0:
        return None
    wbytes = 4 if prec == abi.MLC_PREC_MIXED else 8
    dom_name = max(kernels, key=lambda k: kernels[k][1])
    nl, kms = kernels[dom_name]
    bytes_per = kernel_bytes(dom_name, cases[0], n_adv_fields(cases[0]), wbytes)
    pk = peaks()
    hbm_peak = float(pk.get("hbm_gbs", 6800.0))
    roofline = {"kernel": dom_name, "bound": "hbm", "unit": "GB/s", "peak": hbm_peak,
                "peak_source": "measured" if "hbm_gbs" in pk else "fallback", "traffic": None,
                "share_of_step": kms / sum(v[1] for v in kernels.values()),
                "kernels_ms_per_step": {k: v[1] for k, v in sorted(kernels.items(),
                                                                     key=lambda kv: -kv[1][1])}}
    if bytes_per:
        ach = bytes_per * nmem / (kms / nl / 1000.0) / 1e9
        roofline.update({"achieved": ach, "frac": ach / hbm_peak})
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if prec == abi.MLC_PREC_MIXED else "f64", "data": "synthetic",
        "config": {"workload": f"moloch-ensemble-{nmem}x{n}x{n}x30-dx12km-dt60-ns3",
                   "members": nmem, "points_per_member": pts, "precision": args.precision,
                   "parallelism": f"replicas{world}", "l2": "inputs larger than L2"},
        "roofline": roofline, "gpu_launches": launches * args.steps,
        "side_by_side": {"plain_fp64_single_domain": {"value": plain, "unit": UNIT},
                         "ratio_to_plain_fp64": value / world / plain,
                         "autotune": tune},
        "clocks": clk.summary(),
    }
    return line


def rel_l2(a, b) -> float:
    import numpy as np
    d = np.linalg.norm((np.asarray(a) - np.asarray(b)).ravel())
    n = np.linalg.norm(np.asarray(b).ravel())
    return float(d / n) if n > 0 else float(d)


def run_uneven(args, rank, world):
    """Uneven batch: `members` domains with nx, ny log-uniform in 48-384 and kz
    from {23, 30, 41} (moist recipe, dx 12 km, dt 60 s, 3 substeps, own seeds)
    advanced together in mixed precision with autotuned launch shapes.  A
    sample of every 10th domain is run alone on the plain FP64 path: its
    throughput is the comparison, its final state the per-domain error
    reference (the FP64 path matches the CPU oracle to 1e-12 in the tests)."""
    import numpy as np
    import torch
    from regcm_gb300 import abi
    from regcm_gb300 import case as cs
    from regcm_gb300.moloch import MolochBatch, domain_from_case

    lib = abi.load()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    nmem = args.members or 200
    ids = [rank * nmem + m for m in range(nmem)]
    prec = abi.MLC_PREC_FP64 if args.precision == "fp64" else abi.MLC_PREC_MIXED

    def mk(i, p=prec):
        return cs.config3_member(i, precision=p)

    dims, pts = [], []
    for i in ids:
        nx, ny, kz = cs.config3_dims(i)
        dims.append(abi.mlc_dims(nx + 1, ny + 1, kz, 5, 0))
        pts.append(nx * ny * kz)
    params = mk(ids[0]).params
    t_build = time.perf_counter()
    batch = MolochBatch.lazy(dims, params, lambda m: mk(ids[m]))
    t_build = time.perf_counter() - t_build
    batch.step(args.warmup)
    tune = None if args.no_tune else batch.autotune(1)  # state is kept
    if world > 1:
        torch.distributed.barrier()
    with ClockSampler(dev) as clk:
        ms = batch.step_timed(args.steps)
    t_dev = max_over_ranks(ms / 1000.0, world)
    value = sum(pts) * args.steps * world / t_dev
    launches = batch.launches_per_step()
    sample = list(range(0, nmem, 10))
    errs = {n: [] for n in ("tetav", "u", "v", "w", "qv")}
    plain_gp, plain_t = 0, 0.0
    for m in sample:
        c = mk(ids[m])
        got = c.empty_state()
        batch.download(m, c.state_ptrs_of(got))
        c64 = mk(ids[m], abi.MLC_PREC_FP64)
        d = domain_from_case(c64)
        d.step(args.warmup)
        ms1 = C.c_float()
        diag = abi.mlc_diag()
        abi.check(lib.mlc_step_timed(d._ctx, args.steps, C.byref(diag), C.byref(ms1)), "plain")
        ref = c64.empty_state()
        d.download(c64.state_ptrs_of(ref))
        d.close()
        plain_gp += c64.points * args.steps
        plain_t += ms1.value / 1000.0
        for n in ("tetav", "u", "v", "w"):
            errs[n].append(rel_l2(got[n], ref[n]))
        errs["qv"].append(rel_l2(got["qx"][..., 0], ref["qx"][..., 0]))
    # per-kernel-group times of one eager step (after the state comparison:
    # profiling advances the members) and the dominant group's roofline,
    # its algorithmic bytes summed over the uneven members
    KT = KernelTime
    lib.mlc_profile_steps.argtypes = [C.c_void_p, C.c_int, C.POINTER(KT), C.c_int, C.POINTER(C.c_int)]
    ktab = (KT * 32)()
    nk = C.c_int()
    abi.check(lib.mlc_profile_steps(batch._ctx, 1, ktab, 32, C.byref(nk)), "profile")
    kernels = {ktab[i].name.decode(): (ktab[i].launches, ktab[i].ms) for i in range(nk.value)}
    batch.close()
    if rank != 0:
        return
    import types
    wbytes = 4 if prec == abi.MLC_PREC_MIXED else 8
    dom_name = max(kernels, key=lambda k: kernels[k][1])
    nl, kms = kernels[dom_name]
    pk = peaks()
    hbm_peak = float(pk.get("hbm_gbs", 6800.0))
    roofline = {"kernel": dom_name, "bound": "hbm", "unit": "GB/s", "peak": hbm_peak,
                "peak_source": "measured" if "hbm_gbs" in pk else "fallback", "traffic": None,
                "share_of_step": kms / sum(v[1] for v in kernels.values()),
                "kernels_ms_per_step": {k: v[1] for k, v in sorted(kernels.items(),
                                                                     key=lambda kv: -kv[1][1])}}
    per = [kernel_bytes(dom_name, types.SimpleNamespace(dims=dm, params=params),
                        n_adv_fields(types.SimpleNamespace(dims=dm, params=params)), wbytes)
           for dm in dims]
    if all(b is not None for b in per):
        ach = sum(per) / (kms / nl / 1000.0) / 1e9
        roofline.update({"achieved": ach, "frac": ach / hbm_peak, "algorithmic_bytes": sum(per)})
    plain = plain_gp / plain_t
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if prec == abi.MLC_PREC_MIXED else "f64", "data": "synthetic",
        "config": {"workload": f"moloch-uneven-{nmem}-domains-nx,ny~logU(48,384)-kz{{23,30,41}}"
                               "-dx12km-dt60-ns3",
                   "members": nmem, "points_total": sum(pts), "points_min": min(pts),
                   "points_max": max(pts), "precision": args.precision,
                   "parallelism": f"replicas{world}", "l2": "inputs larger than L2"},
        "roofline": roofline, "gpu_launches": launches * args.steps,
        "side_by_side": {"plain_fp64_one_domain_at_a_time": {"value": plain, "unit": UNIT,
                                                             "sample_domains": len(sample)},
                         "ratio_to_plain_fp64": value / world / plain, "autotune": tune},
        "per_domain_rel_l2_vs_fp64": {n: {"max": max(v), "median": float(np.median(v))}
                                      for n, v in errs.items()},
        "host_load_s": t_build,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def run_serving(args, rank, world):
    """Serving stream: Poisson arrivals at each rate, `requests` requests of
    nx = ny log-uniform in 32-512, kz 30, 6-240 steps, the moist 3 km recipe
    with the request's seed, admitted by arena bytes under the budget and
    batched per step in mixed precision; next to the same stream served one
    request at a time by the plain FP64 path (service times measured once,
    first-come first-served latencies per rate)."""
    import torch
    from regcm_gb300 import abi
    from regcm_gb300 import case as cs
    from regcm_gb300.serve import Request, poisson_arrivals, serve_one_at_a_time, serve_stream

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    rates = [float(r) for r in args.rates.split(",")]
    nreq = args.requests
    budget = int(args.budget_gb * 1e9)
    prec = abi.MLC_PREC_FP64 if args.precision == "fp64" else abi.MLC_PREC_MIXED
    params = cs.config4_request(0, scale=0.05, precision=prec)[0].params
    steps = [cs.config4_shape(r)[1] for r in range(nreq)]
    workers = max(4, min(16, cpu_threads()))
    out, wall = {}, {}
    with ClockSampler(dev) as clk:
        for lam in rates:
            arr = poisson_arrivals(lam, nreq, seed=int(lam * 1000) + 7)
            reqs = [Request(r, float(arr[r]), steps[r],
                            (lambda r=r: cs.config4_request(r, precision=prec)[0]))
                    for r in range(nreq)]
            out[lam] = serve_stream(reqs, params, budget, capacity=args.capacity,
                                    workers=workers, prefetch=min(16, 2 * workers))
        # the same stream's first `wall_requests` requests on the wall clock:
        # payloads built before the stream starts (the client's preparation is
        # not in the latency), arrivals in real time
        if args.wall_requests:
            from concurrent.futures import ThreadPoolExecutor
            nw = min(args.wall_requests, nreq)
            for lam in rates:
                arr = poisson_arrivals(lam, nreq, seed=int(lam * 1000) + 7)
                with ThreadPoolExecutor(max_workers=workers) as ex:
                    built = list(ex.map(lambda r: cs.config4_request(r, precision=prec)[0],
                                        range(nw)))
                reqs = [Request(r, float(arr[r]), steps[r], (lambda c=built[r]: c))
                        for r in range(nw)]
                del built
                wall[lam] = serve_stream(reqs, params, budget, capacity=args.capacity,
                                         clock="wall", prefetch=nw, workers=1)
        # one request at a time, plain FP64 (service times do not depend on the rate)
        arr = poisson_arrivals(rates[0], nreq, seed=int(rates[0] * 1000) + 7)
        base_reqs = [Request(r, float(arr[r]), steps[r], None) for r in range(nreq)]
        one = serve_one_at_a_time(
            base_reqs, lambda r: (lambda rid=r.rid: cs.config4_request(rid)[0]),
            workers=workers, prefetch=min(16, 2 * workers))
    if rank != 0:
        return
    # the FP64 queue's latencies at every rate from the measured service times
    base = {}
    svc = one.pop("service_s")
    for lam in rates:
        arr = poisson_arrivals(lam, nreq, seed=int(lam * 1000) + 7)
        fin, lat = 0.0, []
        for a, s in zip(arr, svc):
            fin = max(a, fin) + s
            lat.append(fin - a)
        import numpy as np
        lat = np.array(lat)
        base[lam] = {"value": one["gp_steps"] / fin, "p50_s": float(np.percentile(lat, 50)),
                     "p99_s": float(np.percentile(lat, 99))}
    head = out[rates[-1]]
    line = {
        "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world,
        "steps": int(sum(steps)), "warmup": 0, "ms_per_step": None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if prec == abi.MLC_PREC_MIXED else "f64", "data": "synthetic",
        "config": {"workload": f"moloch-serving-poisson-{nreq}req-nx~logU(32,512)-kz30-steps~U(6,240)",
                   "rates_per_s": rates, "budget_bytes": budget, "capacity": args.capacity,
                   "precision": args.precision, "requests_per_rate": nreq,
                   "parallelism": f"replicas{world}"},
        "serving": {str(l): v for l, v in out.items()},
        "serving_wall_clock": {str(l): v for l, v in wall.items()} or None,
        "plain_fp64_one_at_a_time": {"service_rate": one["service_rate"],
                                     "per_rate": {str(l): v for l, v in base.items()}},
        "ratio_to_plain_fp64": {str(l): out[l]["value"] / base[l]["value"] for l in rates},
        "clocks": clk.summary(),
        "host_peak_rss_gb": resource.getrusage(resource.RUSAGE_SELF).ru_maxrss / 1e6,
    }
    print(json.dumps(line), flush=True)


class KernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_int32), ("ms", C.c_double)]


_FP64_PEAK = None


def fp64_peak(lib) -> float:
    """FP64 multiply-add throughput of this GPU in FLOP/s, measured once per
    run by the library's probe (mlc_fp64_peak: independent FMA chains on
    every SM, best of 5 launches)."""
    global _FP64_PEAK
    if _FP64_PEAK is None:
        v = C.c_double()
        from regcm_gb300 import abi
        abi.check(lib.mlc_fp64_peak(5, C.byref(v)), "mlc_fp64_peak")
        _FP64_PEAK = v.value
    return _FP64_PEAK


def kernel_roofline(lib, ctx, case, precision):
    """Per-kernel-group device times of two eager steps (CUDA events around
    each group on the library stream) and the roofline of the dominant group.
    Mixed precision: its algorithmic bytes per launch over its mean launch
    time, against the measured HBM copy bandwidth.  FP64: its algorithmic
    FP64 operations per launch over the mean launch time, against the FP64
    rate measured in this run (the FP64 kernels are FP64-pipe bound on
    GB300); the HBM figures follow in `hbm`."""
    lib.mlc_profile_steps.argtypes = [C.c_void_p, C.c_int, C.POINTER(KernelTime), C.c_int,
                                      C.POINTER(C.c_int)]
    ktab = (KernelTime * 32)()
    nk = C.c_int()
    from regcm_gb300 import abi
    abi.check(lib.mlc_profile_steps(ctx, 2, ktab, 32, C.byref(nk)), "mlc_profile_steps")
    kernels = {ktab[i].name.decode(): (ktab[i].launches, ktab[i].ms) for i in range(nk.value)}
    total_k = sum(v[1] for v in kernels.values())
    wbytes = 4 if precision == "mixed" else 8
    nf = n_adv_fields(case)
    dom_name = max(kernels, key=lambda k: kernels[k][1])
    pk = peaks()
    hbm_peak = float(pk.get("hbm_gbs", 6800.0))
    hbm_src = "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in pk else "fallback"
    bytes_per = kernel_bytes(dom_name, case, nf, wbytes)
    nl, kms = kernels[dom_name]
    t_launch = kms / nl / 1000.0
    hbm = {"unit": "GB/s", "peak": hbm_peak, "peak_source": hbm_src}
    if bytes_per:
        ach = bytes_per / t_launch / 1e9
        hbm.update({"achieved": ach, "frac": ach / hbm_peak, "algorithmic_bytes": bytes_per})
    traffic = None
    cap = CAPTURED_TRAFFIC_PER_POINT.get((dom_name, precision, nf))
    if cap:
        traffic = cap[0] * case.points
    ops = kernel_fp64_ops(dom_name, case, nf) if precision == "fp64" else None
    if ops:
        peak = fp64_peak(lib) / 1e12
        ach = ops / t_launch / 1e12
        roofline = {"kernel": dom_name, "bound": "fp64", "unit": "TFLOP/s", "achieved": ach,
                    "peak": peak,
                    "peak_source": "measured in this run (mlc_fp64_peak, FP64 FMA chains)",
                    "frac": ach / peak, "algorithmic_fp64_ops": ops, "traffic": traffic,
                    "hbm": hbm,
                    "note": ("achieved counts the reference's FP64 operations for the same "
                             "results (its limiter's divides, min/max and compares included); "
                             "the kernel tests the limiter's regions on the integer pipe and "
                             "divides nowhere, so fewer FP64 instructions do that work and the "
                             "fraction can exceed 1")}
    else:
        roofline = {"kernel": dom_name, "bound": "hbm", "unit": "GB/s", "peak": hbm_peak,
                    "peak_source": hbm_src, "traffic": traffic}
        if "achieved" in hbm:
            roofline.update({"achieved": hbm["achieved"], "frac": hbm["frac"],
                             "algorithmic_bytes": bytes_per})
    roofline["share_of_step"] = kms / total_k
    if cap:
        roofline["traffic_source"] = (f"constant: ncu DRAM bytes of this kernel on moist "
                                      f"256x256x41 at build {cap[1]}, scaled by points; "
                                      "not measured by this run")
    lim = CAPTURED_LIMITER.get((dom_name, precision))
    if lim:
        roofline["limiter"] = dict(lim, source="constant from the same ncu capture")
    roofline["kernels_ms_per_step"] = {k: v[1] / 2.0 for k, v in sorted(
        kernels.items(), key=lambda kv: -kv[1][1])}
    return roofline


def run_mixed_side(args, rank):
    """The same workload in mixed precision (FP32 fields, FP64 solve/Exner/theta),
    timed the same way, for the FP64-and-FP32 side-by-side report."""
    import torch
    from regcm_gb300 import abi
    from regcm_gb300.moloch import domain_from_case
    lib = abi.load()
    import copy
    margs = copy.copy(args)
    margs.precision = "mixed"
    case = make_case(margs, rank)
    dom = domain_from_case(case)
    dom.step(args.warmup)
    diag = abi.mlc_diag()
    ms = C.c_float()
    abi.check(lib.mlc_step_timed(dom._ctx, args.steps, C.byref(diag), C.byref(ms)), "mixed")
    roofline = kernel_roofline(lib, dom._ctx, case, "mixed")
    dom.close()
    torch.cuda.synchronize()
    t = ms.value / 1000.0
    return {"mixed": {"value": case.points * args.steps / t, "unit": UNIT,
                      "ms_per_step": 1000.0 * t / args.steps, "dtype": "f32+f64",
                      "roofline": roofline}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c1", choices=["c0", "c1", "c2", "c3", "c4"])
    ap.add_argument("--members", type=int, default=0,
                    help="ensemble members (c2: 64) or domains (c3: 200)")
    ap.add_argument("--rates", default="2,8,32", help="arrival rates per second (c4)")
    ap.add_argument("--requests", type=int, default=200, help="requests per rate (c4)")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="arena budget (c4)")
    ap.add_argument("--wall-requests", type=int, default=0,
                    help="c4: also serve the first N requests of each stream on the wall clock")
    ap.add_argument("--capacity", type=int, default=256, help="member slots (c4)")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--precision", default=None, choices=["fp64", "mixed"],
                    help="default: fp64 for c0/c1 (mixed side by side), mixed for c2-c4")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision side run")
    ap.add_argument("--no-ensemble", action="store_true",
                    help="skip the 64-member ensemble side run of the default line")
    ap.add_argument("--size", type=int, default=0, help="cross points per side (profiling runs)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.precision is None:
        args.precision = "mixed" if args.config in ("c2", "c3", "c4") else "fp64"
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.init_process_group("nccl")
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.config == "c2":
        args.members = args.members or 64
        run_ensemble(args, rank, world)
    elif args.config == "c3":
        run_uneven(args, rank, world)
    elif args.config == "c4":
        run_serving(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
