"""Benchmark of the fv3d hydro step on GB300.

Workload (one JSON line): the plain FP64 Rayleigh-Taylor configuration,
512 x 1536 cells in the x-z plane, HLL, PLM, RK2, CFL 0.8, gravity -0.1,
periodic x / reflecting z (seeded synthetic initial state).  One step = one
RK2 step of the whole grid: the control kernel (CFL dt from the reduction
fused into the previous step), stage 1 and stage 2.

  value     Mcell-updates/s with the state resident in HBM, CUDA events on
            the library's stream around each step, L2 flushed (256 MiB
            write) between timed steps because the state fits in L2.
  e2e       the same metric through the C ABI with host buffers: per step
            set_prim from pinned host arrays, the step, get_prim back.
  roofline  the stage kernels (dominant) against measured HBM bandwidth:
            algorithmic bytes 5 state passes x 4 fields x 8 B = 160 B per
            cell-update, over their CUDA-event durations.
  cpu_baseline  the CPU oracle port of the reference algorithm on all host
            cores, a bounded sample of the same workload.

--impl reference times the reference's CPU implementation of the path
(oracle/_ref when it is loadable here, else the C port of it) on the same
workload and prints the same line with "impl": "reference".

Multi-GPU (torchrun, one rank per GPU): independent replicas, no collective
on the data path; value = total cell-updates of all ranks / max rank time.
"""
import argparse
import math
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-updates/s: FP64 plain vs mixed/batched at stated L1 err; HBM % of peak"
UNIT = "Mcell-updates/s"
WORKLOAD = "rayleigh_taylor_512x1536_fp64"
ALGO_BYTES_PER_CELL_UPDATE = 160  # 5 passes x 4 fields x 8 B (F = 4, inviscid 2-D)
# dram__bytes_read.sum + dram__bytes_write.sum of the two stage launches of one
# RK2 step of this workload, from one ncu --set full capture
# (profiles/stage2d_fp64_rt512x1536.md: stage 1 50.70+2.03 MB -- the
# primitive copy of U^n for its halo plus U^n at its own cells --, stage 2
# 50.55+3.58 MB).
NCU_TRAFFIC_BYTES_PER_STEP = 106.86e6
# FP64 arithmetic lane operations (DADD + DMUL + DFMA thread instructions)
# per cell-update of this workload from the same capture (stage 1: 364.4,
# stage 2: 425.5).  The FP64 kernel is bound by the FP64 pipe: its roofline
# against the FP64 FMA rate measured live by fvgpu_probe_fp64_rate.
FP64_OPS_PER_CELL_UPDATE = 790


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def problem(parse=None):
    from fv3d_gb300 import problems
    return problems.rayleigh_taylor(512, 1536, parse=parse)


def config_dict(pr, l2):
    return {"workload": WORKLOAD, "cells": pr.cells, "grid": [pr.params.Nx, pr.params.Nz],
            "riemann": "hll", "reconstruction": "plm", "time_stepping": "rk2", "precision": "fp64",
            "l2": l2, "parallelism": "replicas", "build": os.environ.get("FV3D_LIB_VARIANT", "default")}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self, gpu_index=0):
        try:
            rows = [r.split(",") for r in open(self.path).read().strip().splitlines()]
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = [[c.strip() for c in r] for r in rows if len(r) >= 9 and r[0].strip() == str(gpu_index)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_info():
    from fv3d_gb300 import replicas
    return replicas.dist_info()


def cpu_sample(pr, seconds=15.0, max_steps=20, use_ref=False):
    """Time the CPU reference path on the same workload (all host cores)."""
    from oracle import pyoracle
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    kind = "port"
    if use_ref:
        try:
            path = os.path.join(tempfile.mkdtemp(), "bench.ini")
            with open(path, "w") as f:
                f.write(pr.ini)
            o = pyoracle.RefOracle(path)
            kind = "reference"
        except Exception:
            o = pyoracle.Oracle(pr.params)
    else:
        o = pyoracle.Oracle(pr.params)
    o.set_prim(*pr.prim)
    o.step(o.compute_dt())  # warm-up (first touch)
    n, t0 = 0, time.perf_counter()
    while n < max_steps and (n == 0 or time.perf_counter() - t0 < seconds):
        o.step(o.compute_dt())
        n += 1
    el = time.perf_counter() - t0
    return {"value": pr.cells * n / el / 1e6, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": "%d RK2 steps (dt each step) of %s on %d threads, %.2f s" % (n, WORKLOAD, threads, el)}


def run_reference(args):
    world, rank, _ = dist_info()
    if rank != 0:
        return 0
    from oracle import pyoracle
    # the oracle's own readInifile: this arm loads no library of the GPU path
    pr = problem(parse=pyoracle.parse_ini)
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    kind = "port"
    o = None
    if pyoracle.reference_available():
        try:  # the reference's own headers, where they could be compiled here
            path = os.path.join(tempfile.mkdtemp(), "bench.ini")
            with open(path, "w") as f:
                f.write(pr.ini)
            o = pyoracle.RefOracle(path)
            kind = "reference"
        except Exception:
            o = None
    if o is None:
        o = pyoracle.Oracle(pr.params)
    o.set_prim(*pr.prim)
    t_all = time.perf_counter()
    for _ in range(args.warmup):
        o.step(o.compute_dt())
    per_step = []
    for _ in range(args.steps):  # one RK2 step (computeDt + update) of the whole grid each
        t0 = time.perf_counter()
        o.step(o.compute_dt())
        per_step.append((time.perf_counter() - t0) * 1e3)
    value = pr.cells * args.steps / (sum(per_step) / 1e3) / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(per_step)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": config_dict(pr, "n/a (CPU)"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": "%d timed RK2 steps (after %d warm-up) of %s on %d threads"
                                       % (args.steps, args.warmup, WORKLOAD, threads)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t_all}
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import torch
    import fv3d_gb300 as fv

    from fv3d_gb300 import replicas
    world, rank, local = dist_info()
    torch.cuda.set_device(local)
    replicas.init("nccl")
    pr = problem()
    sim = fv.Simulation(pr.params)
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    sim.set_prim(*pr.prim)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)

    for _ in range(args.warmup):
        sim.enqueue_steps(1)
    sim.synchronize()
    launches0 = sim.launch_count()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    replicas.barrier()
    torch.cuda.synchronize()
    # the raw clock samples go to $FV3D_BENCH_OUT when set (the JSON line
    # carries their summary either way)
    clk = Clocks(os.path.join(os.environ.get("FV3D_BENCH_OUT") or tempfile.mkdtemp(), "bench_clocks.csv"))
    with clk:
        for k in range(args.steps):
            flush_l2()
            evs[k][0].record(stream)
            sim.enqueue_steps(1)
            evs[k][1].record(stream)
        torch.cuda.synchronize()
    launches = sim.launch_count() - launches0
    ms = [a.elapsed_time(b) for a, b in evs]
    rate, slowest_s = replicas.aggregate_rate(pr.cells * args.steps, world, float(sum(ms)) / 1e3, device="cuda")
    total_ms = slowest_s * 1e3
    value = rate / 1e6
    sim.get_prim()  # surfaces any error of the timed steps

    # Dominant kernel: per-launch CUDA events (profile mode), L2 flushed per step.
    sim.profile(True)
    nprof = max(4, min(args.steps, 20))
    for _ in range(nprof):
        flush_l2()
        sim.enqueue_steps(1)
    kt = sim.kernel_times()
    sim.profile(False)
    stage_n, stage_ms = kt["stage"]
    ms_per_step_stages = stage_ms / (stage_n / 2.0)
    hbm_peak, peak_kind = peaks()
    achieved = ALGO_BYTES_PER_CELL_UPDATE * pr.cells / (ms_per_step_stages / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": "stage2d_fp64, both launches of one RK2 step", "achieved": achieved,
                "peak": hbm_peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm_peak,
                "traffic": NCU_TRAFFIC_BYTES_PER_STEP, "traffic_unit": "bytes per RK2 step (ncu)",
                "algo_bytes": ALGO_BYTES_PER_CELL_UPDATE * pr.cells,
                "algo_bytes_per_cell_update": ALGO_BYTES_PER_CELL_UPDATE,
                "stage_ms_per_launch": stage_ms / stage_n, "dt_kernel_ms_per_launch": kt["dt"][1] / max(kt["dt"][0], 1)}
    fp64_peak = fv.probe_fp64_rate()
    fp64_achieved = FP64_OPS_PER_CELL_UPDATE * pr.cells / (ms_per_step_stages / 1e3)
    roofline["fp64_pipe"] = {"achieved": fp64_achieved, "peak": fp64_peak, "frac": fp64_achieved / fp64_peak,
                             "unit": "FP64 lane-ops/s", "peak_kind": "measured live (fvgpu_probe_fp64_rate)",
                             "ops_per_cell_update": FP64_OPS_PER_CELL_UPDATE}

    # e2e through the C ABI from and to pinned host buffers: one
    # fvgpu_step_host per step (primToCons of the host state, CFL dt, one RK2
    # step, consToPrim of the result into host memory; the kernels read and
    # write the host arrays over the CPU-GPU link themselves)
    host_in = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in pr.prim]
    host_in[2] = None  # v is identically zero in the x-z plane
    host_out = [torch.empty(pr.shape, dtype=torch.float64).pin_memory() for _ in range(5)]
    np_in = [None if a is None else a.numpy() for a in host_in]
    np_out = [a.numpy() for a in host_out]
    for _ in range(2):
        sim.step_host(np_in, out=np_out)
    e2e_ms = []
    for _ in range(max(3, args.steps // 2)):
        t0 = time.perf_counter()
        sim.step_host(np_in, out=np_out)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    # the same through the separate calls (set_prim, one step, get_prim)
    sep_ms = []
    for _ in range(max(3, args.steps // 2)):
        t0 = time.perf_counter()
        sim.set_prim(*np_in)
        sim.enqueue_steps(1)
        sim.get_prim(out=np_out)
        sep_ms.append((time.perf_counter() - t0) * 1e3)
    h2d = sum(a.numel() * 8 for a in host_in if a is not None)
    d2h = sum(a.numel() * 8 for a in host_out)
    e2e = {"value": pr.cells * world / (float(np.mean(e2e_ms)) / 1e3) / 1e6, "unit": UNIT,
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": float(np.mean(e2e_ms)),
           "api": "fvgpu_step_host (pinned host arrays)",
           "separate_calls": {"api": "fvgpu_set_prim + fvgpu_enqueue_steps(1) + fvgpu_get_prim",
                              "value": pr.cells * world / (float(np.mean(sep_ms)) / 1e3) / 1e6,
                              "ms_per_step": float(np.mean(sep_ms))}}

    # one-step parity against the oracle on the same state (stated L1 error)
    from oracle import pyoracle
    from fv3d_gb300 import problems
    chk = problems.rayleigh_taylor(512, 1536)
    o = pyoracle.Oracle(chk.params)
    o.set_prim(*chk.prim)
    g = fv.Simulation(chk.params)
    g.set_prim(*chk.prim)
    dt = o.compute_dt()
    o.step(dt)
    g.step(dt)
    l1 = []
    for a, b in zip(g.get_prim(), o.get_prim()):
        den = float(np.abs(b).sum())
        l1.append(float(np.abs(a - b).sum()) / den if den else 0.0)
    g.close()

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": config_dict(pr, "flushed (256 MiB write between timed steps)"),
            "roofline": roofline, "e2e": e2e, "gpu_launches": launches, "clocks": clk.summary(local),
            "rel_l1_vs_oracle_one_step": dict(zip(["rho", "u", "v", "w", "p"], l1))}
    if rank == 0:
        if not args.no_variants:
            line["variants"] = run_variants(torch, args, flush)
        line["cpu_baseline"] = cpu_sample(pr)
        print(json.dumps(line))
    sim.close()
    replicas.shutdown()
    return 0


def _mixed(params):
    import fv3d_gb300 as fv
    q = params.copy()
    q.precision = fv._abi.FV_PREC_FP32_MIXED
    return q


def _rel_l1(a, b):
    den = float(np.abs(b).sum())
    return float(np.abs(a - b).sum()) / den if den else 0.0


def time_batch(torch, params_list, prims, nsteps, warmup, flush_each=None):
    """Mcell-updates/s of a batch (CUDA events on its stream); with
    flush_each, the L2 is flushed before every timed step (small states)."""
    import fv3d_gb300 as fv
    b = fv.Batch(params_list)
    stream = torch.cuda.Stream()
    b.set_stream(stream.cuda_stream)
    for i, pr in enumerate(prims):
        b.set_prim(i, *pr)
    tiles = b.tiling()
    schedule = b.schedule()
    b.run(warmup)
    b.synchronize()
    l0 = b.launch_count()
    cells = sum(int(np.prod(pr[0].shape)) for pr in prims)
    if flush_each is None:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run(nsteps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
    else:
        ms = 0.0
        for _ in range(nsteps):
            with torch.cuda.stream(stream):
                flush_each.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            b.run(1)
            e1.record(stream)
            torch.cuda.synchronize()
            ms += e0.elapsed_time(e1)
    b.times()  # surfaces any error
    return b, {"mcell_updates_per_s": cells * nsteps / (ms / 1e3) / 1e6, "ms_per_step": ms / nsteps,
               "cells": cells, "instances": len(params_list), "tiles": tiles, "schedule": schedule,
               "gpu_launches": b.launch_count() - l0}


def time_sim(torch, pr, nsteps, warmup):
    """Mcell-updates/s of one problem through fvgpu_* (CUDA events on its
    stream, the state larger than L2 or the steps long enough to amortise)."""
    import fv3d_gb300 as fv
    sim = fv.Simulation(pr.params)
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    sim.set_prim(*pr.prim)
    sim.enqueue_steps(warmup)
    sim.synchronize()
    l0 = sim.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sim.enqueue_steps(nsteps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    sim.get_prim()  # surfaces any error
    out = {"mcell_updates_per_s": pr.cells * nsteps / (ms / 1e3) / 1e6, "ms_per_step": ms / nsteps,
           "cells": pr.cells, "gpu_launches": sim.launch_count() - l0}
    sim.close()
    return out


def l1_vs_fp64(torch, probs, nsteps, params_mixed):
    """Per-field relative L1 (worst instance) of the mixed batch against the
    bit-exact FP64 batch after nsteps steps."""
    import fv3d_gb300 as fv
    res = []
    for plist in ([p.params for p in probs], params_mixed):
        b = fv.Batch(plist)
        for i, pr in enumerate(probs):
            b.set_prim(i, *pr.prim)
        b.run(nsteps)
        res.append((b, b.times()))
    worst = [0.0] * 5
    drift = {"fp64": [0.0, 0.0], "mixed": [0.0, 0.0]}
    for i, pr in enumerate(probs):
        a = res[1][0].get_prim(i)
        r = res[0][0].get_prim(i)
        for k in range(5):
            worst[k] = max(worst[k], _rel_l1(a[k], r[k]))
        m0, e0 = _mass_energy(pr.prim, pr.params.gamma0)
        for key, st in (("fp64", r), ("mixed", a)):
            m1, e1 = _mass_energy(st, pr.params.gamma0)
            drift[key][0] = max(drift[key][0], abs(m1 - m0) / abs(m0))
            drift[key][1] = max(drift[key][1], abs(e1 - e0) / abs(e0))
    tdrift = float(np.max(np.abs(res[1][1] - res[0][1]) / np.maximum(res[0][1], 1e-300)))
    return {"steps": nsteps, "rel_l1_worst_instance": dict(zip(["rho", "u", "v", "w", "p"], worst)),
            "rel_time_diff_max": tdrift,
            "rel_drift_worst_instance": {k: {"mass": v[0], "energy": v[1]} for k, v in drift.items()}}


def _mass_energy(prim, gamma):
    """Sum over cells of rho and of E = p/(gamma-1) + rho |u|^2 / 2 (FP64,
    cell volume omitted: the drift is relative)."""
    rho, u, v, w, p = (np.asarray(a, dtype=np.float64) for a in prim)
    E = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v + w * w)
    return float(math.fsum(rho.ravel())), float(math.fsum(E.ravel()))


def random_3d(n):
    """n^3 periodic random state, HLLC, PLM, RK2, conduction + viscosity."""
    from fv3d_gb300 import problems
    return problems.random_problem("tc_visc_3d", problems._mesh(n, n, n),
                                   {"tend": 1.0, "boundaries_x": "periodic", "boundaries_y": "periodic",
                                    "boundaries_z": "periodic"},
                                   {"riemann_solver": "hllc", "reconstruction": "plm", "time_stepping": "RK2",
                                    "CFL": 0.4}, {"gamma0": 1.4}, seed=12345, wmag=0.5,
                                   extra={"thermal_conduction": {"active": True, "kappa": 1e-4},
                                          "viscosity": {"active": True, "mu": 1e-4}})


def run_variants(torch, args, flush):
    """The other benchmark configurations (Sedov, diffusion, shear layer,
    the two batches, two 3-D runs), timed on the same GPU."""
    from fv3d_gb300 import problems
    hbm_peak, _ = peaks()
    out = {}

    def add(name, r, bytes_per_cell_update, l1=None):
        achieved = bytes_per_cell_update * r["mcell_updates_per_s"] * 1e6 / 1e9
        r = dict(r)
        r["roofline"] = {"bound": "hbm", "algo_bytes_per_cell_update": bytes_per_cell_update,
                         "achieved_gbs": achieved, "frac": achieved / hbm_peak}
        if l1 is not None:
            r["vs_fp64"] = l1
        out[name] = r

    # FP32-mixed Rayleigh-Taylor 512x1536 (a batch of one)
    rt = problem()
    _, r = time_batch(torch, [_mixed(rt.params)], [rt.prim], args.steps, 5, flush_each=flush)
    add("rayleigh_taylor_512x1536_fp32_mixed", r, 128, l1_vs_fp64(torch, [rt], 100, [_mixed(rt.params)]))

    # config 3: 512 Sod / Sedov instances, sides 64..256, 200 steps, FP64 and mixed
    b3 = problems.batch_sod_sedov(512)
    _, r = time_batch(torch, [p.params for p in b3], [p.prim for p in b3], 16, 8)
    add("batch512_sod_sedov_fp64", r, 160)
    _, r = time_batch(torch, [_mixed(p.params) for p in b3], [p.prim for p in b3], 64, 8)
    add("batch512_sod_sedov_fp32_mixed", r, 128, l1_vs_fp64(torch, b3, 200, [_mixed(p.params) for p in b3]))

    # config 4: 64 Rayleigh-Taylor instances 256x768 .. 1024x3072 with kappa = mu = 1e-4
    b4 = problems.batch_rt(64)
    _, r = time_batch(torch, [p.params for p in b4], [p.prim for p in b4], 8, 3)
    add("batch64_rt_fp64", r, 200)
    _, r = time_batch(torch, [_mixed(p.params) for p in b4], [p.prim for p in b4], 32, 8)
    add("batch64_rt_fp32_mixed", r, 160, l1_vs_fp64(torch, b4, args.rt_batch_l1_steps,
                                                    [_mixed(p.params) for p in b4]))

    # Single problems: FP64 through the single-problem handle (fvgpu_create),
    # the FP32-mixed form as a batch of one.
    # config 0: Sedov 256^2 (HLLC, absorbing), FP64 and mixed
    se = problems.sedov(256)
    add("sedov_256_fp64", time_sim(torch, se, 64, 8), 160)
    _, r = time_batch(torch, [_mixed(se.params)], [se.prim], 64, 8)
    add("sedov_256_fp32_mixed", r, 128, l1_vs_fp64(torch, [se], 200, [_mixed(se.params)]))

    # config 1b: thermal pulse 1024^2 with conduction and viscosity, 200 fixed steps
    tp = problems.thermal_pulse(1024)
    add("thermal_pulse_1024_fp64", time_sim(torch, tp, 16, 4), 200)
    _, r = time_batch(torch, [_mixed(tp.params)], [tp.prim], 64, 8)
    add("thermal_pulse_1024_fp32_mixed", r, 160, l1_vs_fp64(torch, [tp], 200, [_mixed(tp.params)]))

    # the reference's 3-D blast (settings/blast.ini: PCM, HLLC, Euler) at 256^3,
    # and a 3-D PLM / RK2 / conduction + viscosity run at 192^3 (3-D kernel)
    bl = problems.blast(256)
    add("blast_3d_256_fp64", time_sim(torch, bl, 4, 2), 80)  # Euler: read + write 5 fields
    _, r = time_batch(torch, [_mixed(bl.params)], [bl.prim], 16, 4)
    # Euler in the mixed form: read U^n pairs, write U^n+1 pairs, 5 fields: 80 B
    add("blast_3d_256_fp32_mixed", r, 80, l1_vs_fp64(torch, [bl], 40, [_mixed(bl.params)]))
    r3 = random_3d(192)
    add("random_3d_192_plm_rk2_tc_visc_fp64", time_sim(torch, r3, 2, 1), 200)
    _, r = time_batch(torch, [_mixed(r3.params)], [r3.prim], 8, 2)
    add("random_3d_192_plm_rk2_tc_visc_fp32_mixed", r, 160, l1_vs_fp64(torch, [r3], 10, [_mixed(r3.params)]))

    # config 2: shear layer 4096^2 with conduction and viscosity, FP64 and mixed
    sh = problems.shear_layer(4096)
    add("shear_layer_4096_fp64", time_sim(torch, sh, 8, 3), 200)
    _, r = time_batch(torch, [_mixed(sh.params)], [sh.prim], 32, 8)
    add("shear_layer_4096_fp32_mixed", r, 160, l1_vs_fp64(torch, [sh], 50, [_mixed(sh.params)]))
    return out


def _single_pair(pr, nsteps=0):
    """The FP64 handle and the FP32-mixed handle on one problem: advanced to
    its tend (the main.cpp loop) or for nsteps fixed CFL steps."""
    import fv3d_gb300 as fv
    out = {}
    for key, params in (("fp64", pr.params), ("mixed", _mixed(pr.params))):
        sim = fv.Simulation(params)
        sim.set_prim(*pr.prim)
        t0 = time.perf_counter()
        t, n = sim.advance(1.0e30 if nsteps else pr.params.tend, max_steps=nsteps)
        out[key] = (sim.get_prim(), t, n, time.perf_counter() - t0)
        sim.close()
    return out


def accuracy_entry(prim0, gamma, runs):
    """Per-field relative L1 of the mixed result against the FP64 result, and
    the relative mass / energy drift of both."""
    (a, ta, na, wa), (m, tm, nm, wm) = runs["fp64"], runs["mixed"]
    m0, e0 = _mass_energy(prim0, gamma)
    drift = {}
    for key, st in (("fp64", a), ("mixed", m)):
        m1, e1 = _mass_energy(st, gamma)
        drift[key] = {"mass": abs(m1 - m0) / abs(m0), "energy": abs(e1 - e0) / abs(e0)}
    l1 = [_rel_l1(x, y) for x, y in zip(m, a)]
    return {"rel_l1": dict(zip(["rho", "u", "v", "w", "p"], l1)), "steps": {"fp64": na, "mixed": nm},
            "t_end": {"fp64": ta, "mixed": tm}, "rel_drift": drift, "wall_s": {"fp64": wa, "mixed": wm}}


def checkpointed_pair(pr, fractions, perturb):
    """The unstable configurations: the FP64 handle, the FP32-mixed handle
    and (perturb > 0) a second FP64 handle whose initial density carries
    seeded relative noise of amplitude `perturb`, advanced side by side to
    each fraction of tend.  At every checkpoint: the per-field relative L1 of
    mixed vs FP64 and of perturbed FP64 vs FP64 -- the latter measures how
    much the flow itself amplifies a difference of rounding size."""
    import fv3d_gb300 as fv
    from fv3d_gb300 import problems
    runs = {"fp64": pr.params, "mixed": _mixed(pr.params)}
    if perturb:
        runs["fp64_perturbed"] = pr.params
    sims, clocks = {}, {}
    for key, params in runs.items():
        sims[key] = fv.Simulation(params)
        prim = [a.copy() for a in pr.prim]
        if key == "fp64_perturbed":
            noise = problems.uniform(problems.MASTER_SEED, 99, prim[0].size).reshape(prim[0].shape)
            prim[0] = prim[0] * (1.0 + perturb * (2.0 * noise - 1.0))
        sims[key].set_prim(*prim)
        clocks[key] = [0.0, 0, 0.0]  # t, steps, wall
    out = []
    states = {}
    for f in fractions:
        tend = f * pr.params.tend
        for key, sim in sims.items():
            t0 = time.perf_counter()
            t, n = sim.advance(tend, t=clocks[key][0])
            clocks[key][0] = t
            clocks[key][1] += n
            clocks[key][2] += time.perf_counter() - t0
            states[key] = sim.get_prim()
        row = {"t_target": tend, "t": {k: c[0] for k, c in clocks.items()},
               "steps": {k: c[1] for k, c in clocks.items()},
               "mixed_vs_fp64": dict(zip(["rho", "u", "v", "w", "p"],
                                         [_rel_l1(a, b) for a, b in zip(states["mixed"], states["fp64"])]))}
        if perturb:
            row["fp64_perturbed_vs_fp64"] = dict(zip(["rho", "u", "v", "w", "p"], [
                _rel_l1(a, b) for a, b in zip(states["fp64_perturbed"], states["fp64"])]))
        out.append(row)
        print(pr.name, json.dumps(row), file=sys.stderr, flush=True)
    m0, e0 = _mass_energy(pr.prim, pr.params.gamma0)
    drift = {}
    for key in ("fp64", "mixed"):
        m1, e1 = _mass_energy(states[key], pr.params.gamma0)
        drift[key] = {"mass": abs(m1 - m0) / abs(m0), "energy": abs(e1 - e0) / abs(e0)}
    for sim in sims.values():
        sim.close()
    return {"checkpoints": out, "rel_l1": out[-1]["mixed_vs_fp64"], "rel_drift": drift,
            "perturbation": perturb, "wall_s": {k: c[2] for k, c in clocks.items()}}


def run_accuracy(args):
    """The FP32-mixed form against the bit-exact FP64 form at every
    configuration's stated horizon (not timed): Sedov 256^2 to t = 0.1,
    Rayleigh-Taylor 512x1536 to t = 5, the thermal pulse 1024^2 for 200 steps,
    the shear layer 4096^2 to t = 1, the 512-instance batch for 200 steps and
    the 64-instance Rayleigh-Taylor batch for 500 steps.  The Rayleigh-Taylor
    and shear-layer flows are unstable (the instabilities they are named for
    grow any difference exponentially): they are compared at checkpoints on
    the way, next to FP64 runs from an initial state perturbed by 1e-8.
    Prints one JSON line: per configuration the per-field relative L1 (worst
    instance for batches) and the mass / energy drift of both forms."""
    import torch
    from fv3d_gb300 import problems
    torch.cuda.set_device(0)
    only = set(args.accuracy_only.split(",")) if args.accuracy_only else None
    out = {}

    def want(name):
        return only is None or name in only

    for name, build, nsteps in (("sedov_256_to_t0.1", lambda: problems.sedov(256), 0),
                                ("thermal_pulse_1024_200_steps", lambda: problems.thermal_pulse(1024), 200)):
        if not want(name):
            continue
        pr = build()
        out[name] = accuracy_entry(pr.prim, pr.params.gamma0, _single_pair(pr, nsteps))
        print(name, json.dumps(out[name]), file=sys.stderr, flush=True)
    for name, build in (("rayleigh_taylor_512x1536_to_t5", problem),
                        ("shear_layer_4096_to_t1", lambda: problems.shear_layer(4096))):
        if not want(name):
            continue
        out[name] = checkpointed_pair(build(), (0.1, 0.25, 0.5, 1.0), 1e-8)
    for name, build, nsteps in (("batch512_sod_sedov_200_steps", lambda: problems.batch_sod_sedov(512), 200),
                                ("batch64_rt_500_steps", lambda: problems.batch_rt(64), 500)):
        if not want(name):
            continue
        probs = build()
        t0 = time.perf_counter()
        out[name] = l1_vs_fp64(torch, probs, nsteps, [_mixed(p.params) for p in probs])
        out[name]["wall_s"] = time.perf_counter() - t0
        print(name, json.dumps(out[name]), file=sys.stderr, flush=True)
    print(json.dumps({"accuracy": out, "metric": "relative L1 of FP32-mixed vs bit-exact FP64, per field"}))
    return 0


def run_profile_case(args):
    """Only a workload's steps (warm-up + steps), for launch lists and ncu
    captures: no timing, no CPU baseline, no e2e.  Cases: fp64_rt (the bench
    workload), mixed_rt (the same in the FP32-mixed form, a batch of one),
    sedov_mixed (Sedov 256^2 mixed: the multi-step launch),
    batch_sod_sedov_mixed / batch_sod_sedov_fp64 (64 instances of the
    512-instance set, to keep captures small), shear_mixed / shear_fp64 (the
    4096^2 shear layer, a state larger than L2; FP64 through fvgpu_create as
    the bench times it), fp64_3d / mixed_3d (a 160^3 random state, HLLC, PLM,
    RK2, conduction + viscosity: the 3-D kernels)."""
    import fv3d_gb300 as fv
    from fv3d_gb300 import problems
    case = args.profile_case
    n = args.warmup + args.steps
    if case in ("fp64_rt", "fp64_3d", "shear_fp64"):
        pr = {"fp64_rt": problem, "fp64_3d": lambda: random_3d(160),
              "shear_fp64": lambda: problems.shear_layer(4096)}[case]()
        sim = fv.Simulation(pr.params)
        sim.set_prim(*pr.prim)
        sim.enqueue_steps(n)
        sim.synchronize()
        sim.get_prim()
    else:
        if case == "mixed_rt":
            probs = [problem()]
        elif case == "sedov_mixed":
            probs = [problems.sedov(256)]
        elif case.startswith("shear"):
            probs = [problems.shear_layer(4096)]
        elif case == "mixed_3d":
            probs = [random_3d(160)]
        else:
            probs = problems.batch_sod_sedov(64)
        plist = [p.params if case.endswith("fp64") else _mixed(p.params) for p in probs]
        b = fv.Batch(plist)
        for i, p in enumerate(probs):
            b.set_prim(i, *p.prim)
        b.run(n)
        b.times()
    print("profile case done: %d steps of %s" % (n, case))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--profile-case", nargs="?", const="fp64_rt", default=None,
                    choices=["fp64_rt", "fp64_3d", "mixed_3d", "mixed_rt", "sedov_mixed", "batch_sod_sedov_mixed",
                             "batch_sod_sedov_fp64", "shear_mixed", "shear_fp64"],
                    help="run only a workload's steps (for ncu); prints no JSON")
    ap.add_argument("--no-variants", action="store_true",
                    help="skip the other configurations (mixed, batched, shear layer)")
    ap.add_argument("--rt-batch-l1-steps", type=int, default=50,
                    help="steps of the 64-instance Rayleigh-Taylor batch compared with FP64 in the timed "
                         "run's variants (--accuracy runs the configuration's 500)")
    ap.add_argument("--accuracy", action="store_true",
                    help="no timing: the mixed form against FP64 at every configuration's stated horizon "
                         "(about 20 minutes on one GB300)")
    ap.add_argument("--accuracy-only", default=None, help="comma-separated subset of the --accuracy cases")
    args = ap.parse_args()
    if args.profile_case:
        return run_profile_case(args)
    if args.accuracy:
        return run_accuracy(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
