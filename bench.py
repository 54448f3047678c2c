"""Benchmark: ms per ghost-fluid pressure projection at 1024^2 to relative residual 1e-8.

Workload (one "step" = one PROJECTION_2D::Solve): 1024 x 1024 pressure nodes on
[0,1]^2, level set = signed distance to 8 seeded circles (rho 1 inside, 1000
outside, sigma = 0.0728), MAC velocity U[-1,1] smoothed by 4 Jacobi passes,
dt = 0.5 dx, zero initial pressure; solve to ||b - A p|| / ||b|| <= 1e-8.
The timed path is the mixed-precision MG-PCG (FP64 CG with the reference's matrix
entries, preconditioned by FP32 multigrid V-cycles); the all-FP64 MG-PCG path is
timed beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference's CPU projection (the oracle restatement of
PROJECTION_2D::Solve with PCG-IC(0), which reproduces the reference's iterates bit for
bit; the reference's solve is single-threaded) on the same workload: ONE full solve
to the same relative residual, measured, its iterations sliced over the K timed
steps (the first step also assembles and factors, the last also updates the
velocity), so that the whole run takes about one solve (~1 min on the GPU host).
Prints one JSON line on rank 0.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 1024
TOL = 1e-8
SEED = 0
METRIC = "ms per projection at 1024^2 to rel. residual 1e-8 (mixed MG-PCG)"
WORKLOAD = "standalone ghost-fluid projection, 1024x1024 nodes, 8 circles rho 1:1000, sigma 0.0728, rel. residual 1e-8"
# The configuration both arms report (the workload; nothing measured).
CONFIG = {"workload": WORKLOAD, "grid": f"{N}x{N}", "domain": "[0,1]^2", "tolerance": TOL, "seed": SEED, "dt": "0.5 dx",
          "density_ratio": "1:1000", "surface_tension": 0.0728, "initial_pressure": "zero",
          "l2": "GPU arm: flushed by a 256 MB write before every step; CPU arm: not applicable"}
# PCG-IC(0) iterations of this workload to ||r||/||b|| <= 1e-8 (3019: the oracle's count, which
# is the reference's, deterministic on any host).  It only decides how the reference arm slices
# its one full solve over the timed steps, and scales the GPU arm's bounded CPU sample.
REF_ITERATIONS_PLAN = 3019
REF_SAMPLE_ITERATIONS = 600


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# Flops per node of one WENO5 advection sweep and one reinitialisation sweep in the
# reference's arithmetic (ADVECTION_METHOD_2D.h:508-663, 1401-1658): per one-sided
# derivative 5 differences (10), smoothness indicators (33), weights (17), the three
# candidate stencils and their blend (20); four of them per node in both sweeps.
LS_ADVECT_FLOPS = 4 * 80 + 4 + 5 + 3
LS_REINIT_FLOPS = 4 * 80 + 4 + 9 + 3
REINIT_SWEEPS = 25


def shard(n, rank, ws):
    """Instances of a batch that one rank runs: a host-side partition, no communication."""
    return [k for k in range(n) if k % ws == rank]


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(key="smooth_f32_level0_bytes_per_launch"):
    """A DRAM-traffic figure from the committed ncu summary (profiles/traffic.json), if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(key)
    except (OSError, ValueError):
        return None


def ncu_traffic_per_launch():
    """DRAM bytes per launch of the probed kernel from the committed ncu summary, if any."""
    return ncu_traffic()


TOL_ORACLE = 3e-10


def _load_oracle():
    import numpy as np
    with np.load(os.path.join(ROOT, "tests", "golden", "projection_1024.npz")) as z:
        return {k: z[k] for k in z.files}


ORACLE = None


def oracle_errors(c, gb):
    """Relative L2 of the context's p, U, V against the reference's projection of the
    workload, over the fixture's nodes (every 4th in each direction)."""
    import numpy as np
    st = int(ORACLE["stride"])
    out = {}
    for k, f in (("p", gb.FIELD_P), ("u", gb.FIELD_U), ("v", gb.FIELD_V)):
        a = c.get(f)[1::st, 1::st]
        out["rel_l2_" + k] = float(np.linalg.norm(a - ORACLE[k]) / np.linalg.norm(ORACLE[k]))
    return out


def make_case(n=N):
    from tests.golden.cases import bubbles_case
    return bubbles_case(n, seed=SEED)


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle2d
    oracle2d.build()
    return oracle2d


def _projection_run(oracle2d, case):
    """The reference's projection of the workload (oracle restatement), started: curvature,
    assembly, IC(0) factor; PCG to ||r||/||b|| <= 1e-8."""
    import numpy as np
    g = oracle2d.grid(N, N)
    pr = oracle2d.params(pcg_tolerance=0.0, pcg_max_iterations=1 << 30, pcg_rel_residual=TOL)
    arrays = [case[k].copy() for k in ("phi", "u", "v", "p")] + [np.zeros((N, N))]
    return oracle2d.ProjectionRun(g, pr, *arrays, 0.5 / (N - 1))


def cpu_baseline(case, sample_iterations):
    """Bounded sample of the reference's projection (oracle, one thread like the reference's
    solve): setup and `sample_iterations` PCG-IC(0) iterations timed, scaled to the
    REF_ITERATIONS_PLAN iterations of the full solve."""
    oracle2d = _oracle()
    t0 = time.perf_counter()
    run = _projection_run(oracle2d, case)
    t1 = time.perf_counter()
    it = run.iterate(sample_iterations)
    t2 = time.perf_counter()
    run.close()
    per_iter = (t2 - t1) / max(it, 1)
    return ((t1 - t0) + per_iter * REF_ITERATIONS_PLAN) * 1e3, per_iter * 1e3, it


BATCH_INSTANCES, BATCH_FRAMES, BATCH_SEED = 256, 10, 3


def run_rayleigh_taylor(gb, stream, n=2048, frames=500, every=50):
    """Rayleigh-Taylor on 2048 x 2048 nodes over [0,1] x [0,2] (dy = 2 dx, the reference's
    dx-only diagonal): interface y = 1 + 0.05 cos(2 pi x), densities 3 over 1, viscosity 1e-3,
    no surface tension; mixed precision (FP32 WENO5 / reinit / ENO3 fluxes, FP32 V-cycles),
    CFL time steps, 500 frames, each timed with CUDA events.  Every 50 frames the state is
    also restarted for one frame on the FP64 path (untimed) and the frame's results compared
    (tests/test_gpu_rt_long.py holds the FP64 path to the CPU oracle on the same trajectory
    at 512^2)."""
    import numpy as np
    import torch
    from tests.golden.cases import rayleigh_taylor_level_set
    mk = lambda prec: gb.Context(n, n, 0.0, 0.0, 1.0, 2.0, water_density=3.0, air_density=1.0, surface_tension=0.0,
                                 advection_precision=prec)
    c, c64 = mk(gb.PRECISION_MIXED), mk(gb.PRECISION_FP64)
    for x in (c, c64):
        x.set_stream(stream.cuda_stream)
        x.set_flow_params(water_viscosity=1e-3, air_viscosity=1e-3, gravity=(0.0, -9.8), viscosity=True, cfl_number=0.5)
    c.set(gb.FIELD_PHI, rayleigh_taylor_level_set(n, n))
    opts = gb.solve_opts(precision=gb.PRECISION_MIXED, tolerance=TOL)
    o64 = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=1e-10, max_iterations=2000)
    ids = (gb.FIELD_PHI, gb.FIELD_U, gb.FIELD_V, gb.FIELD_UA, gb.FIELD_VA, gb.FIELD_P)
    inner = (slice(2, 2 + n), slice(2, 2 + n))
    dt = 0.0
    ms, its, worst = [], [], {}
    for f in range(1, frames + 1):
        check = f % every == 0
        if check:
            for fid in ids:
                c64.set(fid, c.get(fid))
        with torch.cuda.stream(stream):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            dt_new, st = c.advance_frame(cfl=1.0, prev_dt=dt, opts=opts, allow_max_iters=True)
            e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
        its.append(st.iterations / 3.0)
        if check:
            c64.advance_frame(cfl=1.0, prev_dt=dt, opts=o64, allow_max_iters=True)
            for name, fid in (("phi", gb.FIELD_PHI), ("u", gb.FIELD_U), ("v", gb.FIELD_V), ("p", gb.FIELD_P)):
                a, b = c.get(fid), c64.get(fid)
                if name == "phi":
                    a, b = a[inner], b[inner]
                e = float(np.linalg.norm(a - b) / np.linalg.norm(b))
                worst[name] = max(worst.get(name, 0.0), e)
        dt = dt_new
    c.close()
    c64.close()
    return {"nodes": [n, n], "domain": [1.0, 2.0], "frames_timed": frames, "ms_per_frame": statistics.mean(ms),
            "ms_per_frame_first_50": statistics.mean(ms[:50]), "ms_per_frame_last_50": statistics.mean(ms[-50:]),
            "cg_iterations_per_projection": statistics.mean(its), "last_dt": dt, "precision": "mixed",
            "one_frame_restarts_every": every, "max_rel_l2_mixed_vs_fp64_frame": worst}


def run_batch(gb, n, frames, cpu=True, dist=None, rank=0, ws=1):
    """Independent rising bubbles of uneven sizes (64^2 to 512^2) advanced together by the
    batched runtime (mixed precision, relative residual 1e-8, autotuned V-cycle sweeps and
    tile plans): the whole run as one graph launch (gb2d_batch_run_graph; its capture timed
    apart), the same frames driven by host worker threads and by one worker for
    comparison, and the reference's solver (the oracle) timed for one frame of a sampled
    instance of every size."""
    import numpy as np
    from tests.golden.cases import batched_bubbles
    grids, phis, params, flows = batched_bubbles(n, seed=BATCH_SEED)
    for p in params:
        p["advection_precision"] = gb.PRECISION_MIXED
    mine = shard(n, rank, ws)  # with N ranks each GPU runs every N-th instance
    all_grids, all_phis, all_params, all_flows = grids, phis, params, flows
    grids, phis, params, flows = ([a[k] for k in mine] for a in (grids, phis, params, flows))
    n_all, n = n, len(mine)
    opts = gb.solve_opts(precision=gb.PRECISION_MIXED, tolerance=TOL)
    out = {"instances": n_all, "instances_per_rank": n, "frames": frames,
           "sizes": {str(N): sum(1 for g in all_grids if g[0] == N) for N in (64, 128, 256, 512)}}
    walls = {}
    for workers in (0, 1):
        t0 = time.perf_counter()
        b = gb.Batch(grids, params=params, flows=flows, workers=workers)
        for k in range(n):
            b.context(k).set(gb.FIELD_PHI, phis[k])
        t1 = time.perf_counter()
        smooth = b.autotune(cfl=1.0, opts=opts)
        t2 = time.perf_counter()
        f = frames if workers == 0 else max(1, frames // 5)
        barrier(dist)
        dts, st = b.advance(f, cfl=1.0, opts=opts, allow_max_iters=True)
        wall_ms = max_over_ranks(dist, st.wall_ms)
        walls[workers] = wall_ms / f
        if workers == 0:
            cells = sum(g[0] * g[1] for g in all_grids)
            out.update({"workers": b.workers, "create_s": t1 - t0, "autotune_s": t2 - t1,
                        "host_threads": {"wall_ms": wall_ms, "ms_per_frame_all_instances": wall_ms / f,
                                         "cg_iterations_per_projection": st.cg_iterations / (3.0 * n * f)},
                        "cells": cells,
                        "schedule_by_size": {str(g[0]): dict(zip(("sweeps", "tile_plan"), b.schedule(k)))
                                             for k, g in enumerate(grids)}})
            # the same instances continue as one graph launch per run: the first call captures
            # the graph (timed apart), the second reuses it
            t3 = time.perf_counter()
            dts, st = b.run_graph(f, cfl=1.0, dts=dts, opts=opts, allow_max_iters=True)
            capture_s = time.perf_counter() - t3 - st.wall_ms * 1e-3
            barrier(dist)
            dts, st = b.run_graph(f, cfl=1.0, dts=dts, opts=opts, allow_max_iters=True)
            gwall = max_over_ranks(dist, st.wall_ms)
            out.update({"graph_capture_s": capture_s, "wall_ms": gwall, "ms_per_frame_all_instances": gwall / f,
                        "instance_frames_per_s": n_all * f / (gwall * 1e-3), "cell_frames_per_s": cells * f / (gwall * 1e-3),
                        "cg_iterations_per_projection": st.cg_iterations / (3.0 * n * f),
                        "max_rel_residual": st.max_rel_residual,
                        "path": "gb2d_batch_run_graph: one graph launch per run, every instance a WHILE node over its frames"})
            per_cell = ncu_traffic("batch_graph_dram_bytes_per_cell_frame")
            if per_cell:
                peak, peak_kind = measured_peaks()
                gbs = per_cell * out["cell_frames_per_s"] / 1e9
                out["hbm"] = {"dram_gbs": gbs, "frac": gbs / peak, "peak_gbs": peak, "peak_source": peak_kind,
                              "dram_bytes_per_cell_frame": per_cell,
                              "source": "DRAM bytes per cell-frame from the whole-graph ncu capture of a 64-instance batch "
                                        "(profiles/batch_graph_64.md) times this run's cell-frames/s"}
        b.close()
    out["one_worker_ms_per_frame_all_instances"] = walls[1]
    out["graph_speedup_vs_one_worker"] = walls[1] / out["ms_per_frame_all_instances"]
    out["graph_speedup_vs_host_threads"] = walls[0] / out["ms_per_frame_all_instances"]
    if cpu:
        out["cpu_reference"] = batch_cpu_estimate(all_grids, all_phis, all_params, all_flows, frames)
    return out


def batch_cpu_estimate(grids, phis, params, flows, frames):
    """The reference's solver (the oracle: IC(0)-PCG to the same relative residual,
    single-threaded) timed for one frame of the first instance of every size in the batch
    (its level set, density and viscosity, from rest); the batch's CPU time is that
    per-size frame time summed over the batch's instances and frames."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle2d
    oracle2d.build()
    ms = {}
    for N in sorted({g[0] for g in grids}):
        k = next(i for i, g in enumerate(grids) if g[0] == N)
        gr = oracle2d.grid(N, N)
        pr = oracle2d.params(water_density=params[k]["water_density"], air_density=1.0, pcg_tolerance=0.0,
                             pcg_max_iterations=100000, pcg_rel_residual=TOL)
        fl = oracle2d.flow(water_viscosity=flows[k]["water_viscosity"], air_viscosity=flows[k]["air_viscosity"], viscosity=True)
        phi = phis[k].copy()
        u, v = np.zeros((N + 4, N + 5)), np.zeros((N + 5, N + 4))
        ua, va = np.zeros((N + 6, N + 7)), np.zeros((N + 7, N + 6))
        p, kap = np.zeros((N + 2, N + 2)), np.zeros((N, N))
        t0 = time.perf_counter()
        oracle2d.curvature(gr, phi, kap)
        dt, _ = oracle2d.cfl_time_step(gr, pr, fl, u, v, kap, 0.5)
        oracle2d.time_step(gr, pr, fl, phi, u, v, ua, va, p, kap, None, dt)
        ms[N] = (time.perf_counter() - t0) * 1e3
    total_ms = sum(ms[g[0]] for g in grids) * frames
    return {"kind": "port", "cores": 1, "ms_per_frame_by_size": {str(N): t for N, t in ms.items()},
            "estimated_s_for_batch": total_ms * 1e-3,
            "sample": "one oracle frame (level-set RK3, reinit, 3 SolveForRK with IC(0)-PCG to 1e-8) of the first "
                      "instance of each size, from rest, times the batch's instances of that size and its frames"}


def run_reference(args):
    """One full solve of the reference's projection, measured: the K timed steps are K
    consecutive slices of it (about REF_ITERATIONS_PLAN / K PCG iterations each; the first
    step also assembles and factors, the last runs whatever iterations remain and the
    velocity update).  The W warm-up steps are slices of the same size of a solve that is
    then dropped.  value = the sum of the K step times = ms for the whole projection."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    case = make_case()
    oracle2d = _oracle()
    per = -(-REF_ITERATIONS_PLAN // args.steps)
    run = _projection_run(oracle2d, case)
    for _ in range(args.warmup):
        run.iterate(per)
    run.close()
    times, run, st = [], None, None
    t_all = time.perf_counter()
    for k in range(args.steps):
        t0 = time.perf_counter()
        if k == 0:
            run = _projection_run(oracle2d, case)
        if k < args.steps - 1:
            run.iterate(per)
        else:
            st = run.finish()
        times.append((time.perf_counter() - t0) * 1e3)
    wall = time.perf_counter() - t_all
    ms = sum(times)
    cores = 1
    sample = (f"one full projection (assembly, IC(0) factor, {st.iterations} PCG-IC(0) iterations to rel. residual 1e-8, "
              f"velocity update) measured, sliced over the {args.steps} steps; oracle restatement of the reference's "
              f"PROJECTION_2D::Solve, single-threaded as the reference's solve")
    out = {"metric": METRIC, "value": ms, "unit": "ms", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": ms / args.steps, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic", "impl": "reference", "config": dict(CONFIG),
           "details": {"solver": "PCG-IC(0) (reference PCG_METHOD, restated by the oracle), CPU, 1 thread",
                       "iterations": st.iterations, "step_ms": times, "wall_s": wall,
                       "iterations_per_step": per, "host_threads": os.cpu_count()},
           "cpu_baseline": {"value": ms, "unit": "ms", "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_gb300(args):
    import numpy as np
    import torch
    import importlib
    gb = importlib.import_module("2d_engine_gb300")
    global ORACLE
    ORACLE = _load_oracle()

    ws, rank, local = dist_env()
    dist = init_dist(ws)
    torch.cuda.set_device(local)
    case = make_case()
    dt = 0.5 / (N - 1)
    stream = torch.cuda.Stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def setup(prec):
        c = gb.Context(N, N)
        c.set_stream(stream.cuda_stream)
        for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_P, "p"), (gb.FIELD_UA, "ua"), (gb.FIELD_VA, "va")):
            c.set(f, case[k])
        c.checkpoint_save()
        c.synchronize()
        return c

    def timed(c, opts, steps, warmup, probe=False):
        ms, iters, stats = [], [], None
        for step in range(warmup + steps):
            c.checkpoint_restore()
            with torch.cuda.stream(stream):
                flush.zero_()  # > L2 (129 MB): every step starts cold
                if probe and step == warmup:
                    c.probe(True)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                st = c.projection(dt, opts)
                e1.record(stream)
            e1.synchronize()
            if step >= warmup:
                ms.append(e0.elapsed_time(e1))
                iters.append(st.iterations)
                stats = st
        return ms, iters, stats

    mixed = gb.solve_opts(precision=gb.PRECISION_MIXED, tolerance=TOL)
    fp64 = gb.solve_opts(precision=gb.PRECISION_FP64, tolerance=TOL)
    alu_fp64, alu_fp32 = gb.alu_peaks()  # measured FMA peaks, outside every timed region
    cm = setup(gb.PRECISION_MIXED)
    c64 = setup(gb.PRECISION_FP64)
    timed(cm, mixed, 0, args.warmup)
    timed(c64, fp64, 0, min(args.warmup, 2))

    clocks = ClockSampler(local)
    clocks.start()
    barrier(dist)
    torch.cuda.synchronize()
    launches0 = gb.kernel_launches()
    t_wall0 = time.perf_counter()
    ms_m, it_m, st_m = timed(cm, mixed, args.steps, 0)
    t_wall = time.perf_counter() - t_wall0
    launches = gb.kernel_launches() - launches0
    torch.cuda.synchronize()
    barrier(dist)
    # Roofline kernel: one more projection of the same workload with the finest-level
    # sweeps bracketed by CUDA events (launched directly, not from the graphs).
    timed(cm, mixed, 1, 0, probe=True)
    nprobe, probe_ms, probe_bytes = cm.probe_read()
    cm.probe(False)
    ms_64, it_64, st_64 = timed(c64, fp64, max(1, min(args.steps, 3)), 0)

    p_mixed = cm.get(gb.FIELD_P)
    p_64 = c64.get(gb.FIELD_P)
    diff = float(np.linalg.norm(p_mixed - p_64) / np.linalg.norm(p_64))
    # Both against the reference's own projection of this workload (tests/golden/
    # projection_1024.npz, every 4th node), and the mixed solve at the tolerance where
    # it meets 1e-8 against the reference in p, u and v (3e-10: at 1e-8 the pressure's
    # near-constant mode, which the corner pin barely fixes, is left at ~1e-7).
    vs_oracle = {"noise_floor_p": float(ORACLE["resolve_rel_l2_p"]),
                 "mixed": oracle_errors(cm, gb), "fp64": oracle_errors(c64, gb)}
    tight = gb.solve_opts(precision=gb.PRECISION_MIXED, tolerance=TOL_ORACLE)
    ms_t, it_t, st_t = timed(cm, tight, max(1, min(args.steps, 5)), 0)
    vs_oracle["mixed_at_tolerance"] = dict(tolerance=TOL_ORACLE, ms=statistics.mean(ms_t), iterations=statistics.mean(it_t),
                                           rel_residual=st_t.rel_residual, **oracle_errors(cm, gb))

    # End to end through the C ABI with host buffers: one gb2d_projection_host call per
    # step copies the step's inputs (phi, U, V, warm-start p) in from page-locked host
    # memory, projects, and copies p, U, V out; all of it inside the timed region.
    pin = {k: torch.from_numpy(np.ascontiguousarray(case[k])).pin_memory().numpy() for k in ("phi", "u", "v", "p")}
    out = {k: torch.empty(case[k].shape, dtype=torch.float64).pin_memory().numpy() for k in ("p", "u", "v")}
    h2d = sum(pin[k].nbytes for k in pin)
    d2h = sum(out[k].nbytes for k in out)
    e2e = []
    for step in range(args.warmup + args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            cm.projection_host(dt, mixed, phi=pin["phi"], u=pin["u"], v=pin["v"], p=pin["p"], p_out=out["p"], u_out=out["u"],
                               v_out=out["v"])
            e1.record(stream)
        e1.synchronize()
        if step >= args.warmup:
            e2e.append(e0.elapsed_time(e1))
    # The machine's host-link throughput for the same copies made one by one (not timed as
    # e2e): blocking gb2d_set_field / gb2d_get_field calls of the four inputs and three
    # outputs, so that e2e can be read against the copy cost it overlaps.
    e2e_h2d, e2e_d2h = [], []
    for step in range(3):
        with torch.cuda.stream(stream):
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            ev[0].record(stream)
            cm.set(gb.FIELD_PHI, pin["phi"]); cm.set(gb.FIELD_U, pin["u"]); cm.set(gb.FIELD_V, pin["v"]); cm.set(gb.FIELD_P, pin["p"])
            ev[1].record(stream)
            cm.get(gb.FIELD_P, out["p"]); cm.get(gb.FIELD_U, out["u"]); cm.get(gb.FIELD_V, out["v"])
            ev[2].record(stream)
        ev[2].synchronize()
        e2e_h2d.append(ev[0].elapsed_time(ev[1]))
        e2e_d2h.append(ev[1].elapsed_time(ev[2]))

    # Level-set path of the same workload (not part of the metric): one level-set
    # TVD-RK3 step with its reinitialisation (3 WENO5 sweeps + 3 x 25 reinit sweeps),
    # for the bit-exact FP64 kernels and the FP32-flux variant.
    levelset = {}
    for name, aprec in (("fp64_exact", gb.PRECISION_FP64), ("fp32_flux", gb.PRECISION_MIXED)):
        cl = gb.Context(N, N, advection_precision=aprec)
        cl.set_stream(stream.cuda_stream)
        for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_UA, "ua"), (gb.FIELD_VA, "va")):
            cl.set(f, case[k])
        cl.checkpoint_save()
        cl.synchronize()
        ts = []
        for step in range(4):
            cl.checkpoint_restore()
            with torch.cuda.stream(stream):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                cl.levelset_rk3(dt)
                e1.record(stream)
            e1.synchronize()
            if step >= 1:
                ts.append(e0.elapsed_time(e1))
        levelset[name + "_rk3_ms"] = statistics.median(ts)
        cl.close()
    # Roofline of the level-set step: both bounds, from the reference's arithmetic and
    # arrays per node (one WENO5 advection sweep: 4 one-sided WENO5 derivatives of 80
    # flops, velocity averages, update, RK blend = 332 flops, reads phi, U, V and writes
    # phi = 32 B; one reinitialisation sweep: the same derivatives, Godunov selection and
    # update, RK blend = 336 flops, reads phi, S and writes phi = 24 B; a step = 3 + 75).
    ls_flops = (3 * LS_ADVECT_FLOPS + 3 * REINIT_SWEEPS * LS_REINIT_FLOPS) * float(N * N)
    ls_bytes = (3 * 32 + 3 * REINIT_SWEEPS * 24) * float(N * N)
    roof_ls = {"kernels": "level-set TVD-RK3 + reinit TVD-RK3 step at 1024^2 (3 WENO5 advection sweeps, 75 reinit sweeps)",
               "flops_per_node": ls_flops / (N * N), "bytes_per_node": ls_bytes / (N * N),
               "alu_peaks_tflops": {"fp64": alu_fp64, "fp32": alu_fp32, "source": "measured (gb2d_alu_peaks, FMA chains)"}}
    peak_hbm, _ = measured_peaks()
    for name, key, alu in (("fp64_exact", "fp64_exact_rk3_ms", alu_fp64), ("fp32_flux", "fp32_flux_rk3_ms", alu_fp32)):
        sec = levelset[key] * 1e-3
        tf, gbs = ls_flops / sec / 1e12, ls_bytes / sec / 1e9
        roof_ls[name] = {"ms": levelset[key], "achieved_tflops": tf, "alu_peak_tflops": alu, "alu_frac": tf / alu,
                         "achieved_gbs": gbs, "hbm_frac": gbs / peak_hbm,
                         "bound": "alu" if tf / alu >= gbs / peak_hbm else "hbm"}

    # One whole time step of the same workload (not part of the metric): level-set and
    # reinit RK3, then three SolveForRK stages (ENO3 velocity advection, gravity +
    # explicit viscosity + wall conditions, projection) and the velocity RK3 blends.
    time_step = {}
    for name, aprec, sopts in (("fp64", gb.PRECISION_FP64, fp64), ("mixed", gb.PRECISION_MIXED, mixed)):
        cs = gb.Context(N, N, advection_precision=aprec)
        cs.set_stream(stream.cuda_stream)
        cs.set_flow_params(water_viscosity=1.0, air_viscosity=0.01, gravity=(0.0, -9.8), viscosity=True)
        for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_P, "p"),
                     (gb.FIELD_UA, "ua"), (gb.FIELD_VA, "va")):
            cs.set(f, case[k])
        cs.checkpoint_save()
        cs.synchronize()
        ts, its = [], []
        for step in range(3):
            cs.checkpoint_restore()
            with torch.cuda.stream(stream):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                st_s = cs.advance_time_step(dt, sopts)
                e1.record(stream)
            e1.synchronize()
            if step >= 1:
                ts.append(e0.elapsed_time(e1))
                its.append(st_s.iterations)
        time_step[name + "_ms"] = statistics.median(ts)
        time_step[name + "_projection_iterations"] = statistics.mean(its)
        cs.close()

    batch = run_batch(gb, BATCH_INSTANCES, BATCH_FRAMES, cpu=not args.no_cpu and rank == 0, dist=dist, rank=rank, ws=ws)
    rt = run_rayleigh_taylor(gb, stream)
    clk = clocks.stop()
    clk["window"] = "every timed leg (projections, end to end, level set, time step, batch, Rayleigh-Taylor)"

    # Per-replica latency (each rank runs its own projection of the same workload): the max
    # over ranks; the aggregate throughput of all replicas is reported beside it.
    ms_step = max_over_ranks(dist, statistics.mean(ms_m))
    value = ms_step
    e2e_ms = max_over_ranks(dist, statistics.mean(e2e))
    peak, peak_kind = measured_peaks()
    achieved = (probe_bytes / (probe_ms / nprobe * 1e-3) / 1e9) if nprobe else None
    traffic = ncu_traffic_per_launch()

    # Whole-projection roofline from the per-node algorithmic bytes of the path (every array
    # a pass must read or write, once, at its storage width): setup (phi, U, V in; the face
    # weights, b, kappa out) 64 B; each FP64 true-residual pass 40 B (one before the CG, one
    # to confirm it); per CG iteration the FP64 vector work 13 x 8 B plus one V(2,2) cycle,
    # (4/3) [5 s (2 + 2) + 6.5 s] with s the preconditioner's storage width.
    def projection_bytes_per_node(iters, s):
        return 64 + 2 * 40 + iters * (13 * 8 + (4.0 / 3.0) * (5 * s * 4 + 6.5 * s))
    roof_proj = {"formula": "64 + 2*40 + iterations * (104 + (4/3)*(26.5 s)) B per node; s = 4 (mixed), 8 (FP64)",
                 "peak_gbs": peak}
    for name, its, ms_, s_w in (("mixed", statistics.mean(it_m), ms_step, 4), ("fp64", statistics.mean(it_64), statistics.mean(ms_64), 8)):
        bpn = projection_bytes_per_node(its, s_w)
        gbs = bpn * N * N / (ms_ * 1e-3) / 1e9
        roof_proj[name] = {"iterations": its, "bytes_per_node": bpn, "ms": ms_, "achieved_gbs": gbs, "frac": gbs / peak}

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        cms, per_iter, it = cpu_baseline(case, REF_SAMPLE_ITERATIONS)
        cpu = {"value": cms, "unit": "ms", "cores": 1, "kind": "port",
               "sample": f"oracle projection (the reference's PCG-IC(0) solve, single-threaded as in the reference): setup + "
                         f"{it} iterations at 1024^2 timed ({per_iter:.1f} ms/iteration), scaled to the {REF_ITERATIONS_PLAN} "
                         f"iterations of the full solve to 1e-8; bench.py --impl reference measures that full solve"}
    res = {
        "metric": METRIC, "value": value, "unit": "ms", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 CG / f32 preconditioner", "data": "synthetic",
        "config": dict(CONFIG),
        "details": {"solver": "FP64 CG (reference matrix entries) preconditioned by FP32 V-cycles (2+2 red-black GS)",
                   "projections_per_s_all_replicas": ws * 1e3 / ms_step,
                   "iterations_mixed": statistics.mean(it_m), "outer_iterations_mixed": st_m.outer_iterations,
                   "rel_residual_mixed": st_m.rel_residual,
                   "fp64_mgpcg_ms": statistics.mean(ms_64), "iterations_fp64": statistics.mean(it_64), "rel_residual_fp64": st_64.rel_residual,
                   "mixed_vs_fp64_rel_l2_p": diff, "vs_reference_projection": vs_oracle, "replicas": ws,
                   "roofline_projection": roof_proj, "levelset_rk3_1024": levelset, "roofline_levelset": roof_ls,
                   "time_step_1024": time_step,
                   "batched_rising_bubbles": batch,
                   "rayleigh_taylor_2048": rt},
        "clocks": clk,
        "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "call": "gb2d_projection_host (page-locked host buffers; copies overlap the assembly and the velocity update)",
                "separate_copies": {"h2d_ms": statistics.median(e2e_h2d), "d2h_ms": statistics.median(e2e_d2h),
                                    "h2d_gbs": h2d / statistics.median(e2e_h2d) / 1e6,
                                    "d2h_gbs": d2h / statistics.median(e2e_d2h) / 1e6}},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": "finest-level smoothing launch (k_pre_smooth / k_post_smooth: two red-black sweeps each, FP32)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                     "peak_source": peak_kind, "traffic": traffic, "launches_timed": nprobe,
                     "avg_launch_us": (probe_ms / nprobe * 1e3) if nprobe else None, "algorithmic_bytes_per_launch": probe_bytes},
        "cpu_baseline": cpu,
        "wall_s_timed": t_wall,
    }
    print(json.dumps(res))


def profile_step():
    """Two AdvanceOneFrame calls (curvature, CFL time step, order-3 time step) of the benchmark's
    1024^2 state in mixed precision with the viscous term on: the workload of the time-step
    launch list in profiles/."""
    import importlib
    gb = importlib.import_module("2d_engine_gb300")
    case = make_case()
    c = gb.Context(N, N, advection_precision=gb.PRECISION_MIXED)
    c.set_flow_params(water_viscosity=1.0, air_viscosity=0.01, viscosity=True)
    for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_P, "p"), (gb.FIELD_UA, "ua"),
                 (gb.FIELD_VA, "va")):
        c.set(f, case[k])
    opts = gb.solve_opts(precision=gb.PRECISION_MIXED, tolerance=TOL)
    dt = 0.0
    for _ in range(2):
        dt, st = c.advance_frame(cfl=1.0, prev_dt=dt, opts=opts)
    c.synchronize()
    print(json.dumps({"frames": 2, "dt": dt, "cg_iterations_last_frame": st.iterations}))


def profile_batch(n):
    """A batch of n rising bubbles of 64^2-512^2 (the batch leg's distributions) as one graph
    launch, one frame captured and run twice, mixed precision: the workload of the batch's
    whole-graph capture in profiles/ (kernel nodes under conditional nodes are profiled as
    the whole graph)."""
    import importlib
    from tests.golden.cases import batched_bubbles
    gb = importlib.import_module("2d_engine_gb300")
    grids, phis, params, flows = batched_bubbles(n, seed=BATCH_SEED)
    for p in params:
        p["advection_precision"] = gb.PRECISION_MIXED
    b = gb.Batch(grids, params=params, flows=flows)
    for k in range(len(grids)):
        b.context(k).set(gb.FIELD_PHI, phis[k])
    opts = gb.solve_opts(precision=gb.PRECISION_MIXED, tolerance=TOL)
    dts, st = b.run_graph(1, cfl=1.0, opts=opts, allow_max_iters=True)
    dts, st = b.run_graph(1, cfl=1.0, dts=dts, opts=opts, allow_max_iters=True)
    print(json.dumps({"instances": len(grids), "frames": 1, "wall_ms": st.wall_ms, "cg_iterations": st.cg_iterations,
                      "max_rel_residual": st.max_rel_residual}))
    b.close()


def profile_projection(n=N):
    """The headline workload alone: 4 mixed-precision projections of the 1024^2 state (3 warm-up,
    1 as timed), each restored from a device checkpoint, then 1 FP64 projection: the workload of
    the projection launch list and the smoothing-kernel capture in profiles/.  n: the same case
    on an n^2 grid."""
    import importlib
    gb = importlib.import_module("2d_engine_gb300")
    case = make_case(n)
    dt = 0.5 / (n - 1)
    out = {"n": n}
    for name, prec, reps in (("mixed", gb.PRECISION_MIXED, 4), ("fp64", gb.PRECISION_FP64, 1)):
        c = gb.Context(n, n)
        for f, k in ((gb.FIELD_PHI, "phi"), (gb.FIELD_U, "u"), (gb.FIELD_V, "v"), (gb.FIELD_P, "p")):
            c.set(f, case[k])
        c.checkpoint_save()
        opts = gb.solve_opts(precision=prec, tolerance=TOL)
        for _ in range(reps):
            c.checkpoint_restore()
            st = c.projection(dt, opts)
        c.synchronize()
        out[name + "_iterations"] = st.iterations
        c.close()
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--profile-projection", type=int, nargs="?", const=N, default=0, metavar="N",
                    help="only run the benchmark's projections (4 mixed, 1 FP64) on an N^2 grid (default 1024), for profilers")
    ap.add_argument("--profile-step", action="store_true",
                    help="only run two mixed-precision frames (CFL time steps, viscous term on) of the 1024^2 state, for profilers")
    ap.add_argument("--profile-batch", type=int, nargs="?", const=16, default=0, metavar="N",
                    help="only run an N-instance batch (default 16) as one graph launch (two one-frame runs), for profilers")
    args = ap.parse_args()
    if args.profile_batch:
        profile_batch(args.profile_batch)
        return
    if args.profile_projection:
        profile_projection(args.profile_projection)
        return
    if args.profile_step:
        profile_step()
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
