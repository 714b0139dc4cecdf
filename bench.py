"""Benchmark: Gcell-updates/s of the FDTD time step and its fraction of the HBM roofline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config 512|64|hbm]

Default workload: the 512^3 random-box scenario (64 seeded dielectric boxes, 65 materials in a
uint8 index, 10-cell CPML, 4 delayed 50-ohm lumped sources, 16 Ez/Hx probes). A step is one Yee
time step (E update with source injection, H update, CPML, probes) over all 134,217,728 cells.
The fields (3.2 GB) are far larger than L2, so no flush is needed between steps.

Our arm prints one JSON line with: value (device-timed Gcell-updates/s, inputs resident),
e2e (same metric through the C ABI from host buffers: handle creation, material/waveform
upload, the K steps and the probe read-back), roofline (algorithmic bytes per cell-update x
cells / measured step time, against MEASURED_PEAKS.json), cpu_baseline (the CPU oracle on a
bounded sample) and clocks. The reference arm runs the reference's own CUDA kernels (calc_e +
calc_h built from fdtdrav.h, oracle/_ref) on the same workload and GPU.

Multi-GPU: the path does not shard (one resident grid per GPU); with --gpus N each rank runs an
independent replica of the workload (weak scaling, no collective), value = total over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=["512", "256", "64", "hbm"], default="512")
    ap.add_argument("--schedule", type=int, default=0,
                    help="0 auto, 1 two-pass, 2 fused, 3 fused with the CPML sweep (not chosen by auto)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--adjoint-steps", type=int, default=4000,
                    help="steps of the adjoint workload (4000 is the workload; fewer for profiling)")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-hbm", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 error record (profiling runs)")
    return ap.parse_args()


def scenario_for(cfg: str):
    from fdtd_gb300 import scenario as S
    if cfg == "64":
        return S.config_small(), "vacuum 64^3, 10-cell CPML, 1 z-edge source, 1 Ez probe"
    if cfg == "256":
        return (S.random_boxes(256, 256, 256, 1000, seed=256, edge=(8, 64), name="boxes256"),
                "256^3 random boxes (64 boxes, uint8 index), 10-cell CPML, 4 sources, 16 probes")
    if cfg == "hbm":
        return S.config_hbm(), ("1024x1024x896 random boxes (64 boxes, 65 materials, uint8 index), "
                                "10-cell CPML, 4 sources, 16 probes")
    return S.config_512(), "512^3 random boxes (64 boxes, 65 materials, uint8 index), 10-cell CPML, 4 sources, 16 probes"


def algorithmic_bytes_per_cell(sc) -> float:
    """48 B (6 FP32 components read + written once) + 1 B material index + 8 B per CPML psi update
    (4 B read + 4 B write), psi counted exactly from the update masks."""
    nx, ny, nz = sc.nx, sc.ny, sc.nz
    pxn, pxp, pyn, pyp, pzn, pzp = sc.pml
    i = np.arange(nx); j = np.arange(ny); k = np.arange(nz)

    def slab(q, n, pn, pp):
        return (q < pn) | (q >= n - pp)

    xs, ys, zs = slab(i, nx, pxn, pxp), slab(j, ny, pyn, pyp), slab(k, nz, pzn, pzp)

    def count(mi, mj, mk, si, sj, sk):
        # number of nodes in mask (mi x mj x mk) and in the slab product
        return int((mi & si).sum()) * int((mj & sj).sum()) * int((mk & sk).sum())

    T = np.ones_like
    inner = lambda q, n: (q > 0) & (q < n - 1)
    lo = lambda q, n: q < n - 1
    # E components (masks of calc_e) and H components (masks of calc_h), each with its two psi axes
    ex = (lo(i, nx), inner(j, ny), inner(k, nz))
    ey = (inner(i, nx), lo(j, ny), inner(k, nz))
    ez = (inner(i, nx), inner(j, ny), lo(k, nz))
    hx = (T(i, bool), lo(j, ny), lo(k, nz))
    hy = (lo(i, nx), T(j, bool), lo(k, nz))
    hz = (lo(i, nx), lo(j, ny), T(k, bool))
    allx, ally, allz = T(i, bool), T(j, bool), T(k, bool)
    psi = 0
    psi += count(*ex, allx, ys, allz) + count(*ex, allx, ally, zs)
    psi += count(*ey, xs, ally, allz) + count(*ey, allx, ally, zs)
    psi += count(*ez, xs, ally, allz) + count(*ez, allx, ys, allz)
    psi += count(*hx, allx, ys, allz) + count(*hx, allx, ally, zs)
    psi += count(*hy, xs, ally, allz) + count(*hy, allx, ally, zs)
    psi += count(*hz, xs, ally, allz) + count(*hz, allx, ys, allz)
    return 48.0 + 1.0 + 8.0 * psi / (nx * ny * nz)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0])); mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_setup(n_gpus):
    import torch
    rank, world = 0, 1
    if n_gpus > 1 or "RANK" in os.environ:
        import torch.distributed as dist
        rank = int(os.environ.get("RANK", "0"))
        world = int(os.environ.get("WORLD_SIZE", "1"))
        local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(cells, steps, ms_per_rank, world):
    """Whole-job throughput of `world` independent replicas: every rank advances its own grid of
    `cells` by `steps` steps; the job takes as long as the slowest rank."""
    return world * cells * steps / (ms_per_rank * 1e-3) / 1e9


def cpu_baseline():
    """The CPU oracle (FP32 restatement of the reference's calc_e / calc_h, OpenMP over z-planes)
    on all host cores, time loop only (setup excluded): a 50-step window of a 512 x 512 x 64 z-slab
    of the 512^3 generator (same seed, boxes clipped to the slab), median of 3 runs, as the value;
    the 64^3 vacuum workload in full (1000 steps) beside it."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from fdtd_gb300 import scenario as S
    cores = os.cpu_count() or 1
    window = S.random_boxes(512, 512, 64, 50, seed=512, name="cpu_window")
    rates = []
    for _ in range(3):
        oracle.run(window, steps=50, threads=cores)
        rates.append(window.cells * 50 / oracle.last_step_seconds() / 1e9)
    small = S.config_small()
    oracle.run(small, threads=cores)
    t_small = oracle.last_step_seconds()
    return {"value": float(np.median(rates)), "unit": "Gcell-updates/s", "cores": cores, "kind": "port",
            "sample": "CPU oracle (FP32, OpenMP, all host cores), time loop only: 50 steps of a 512x512x64 "
                      "z-slab of the 512^3 random-box generator, median of 3 runs",
            "runs": [round(r, 4) for r in rates],
            "vacuum64_full": {"value": round(small.cells * small.steps / t_small / 1e9, 4),
                              "unit": "Gcell-updates/s", "steps": small.steps, "seconds": round(t_small, 3)}}


def fp64_error():
    """Error of the FP32 solver against an FP64 build of the same update at small size: the 64^3
    vacuum workload on the GPU (C ABI, AUTO) against the FP64 oracle. Relative L2 of the Ez probe
    series over the full 1000 steps, and of the final fields after 150 steps, while the pulse is
    still inside the grid (after 1000 steps the CPML has absorbed it and only residue of the order
    of the rounding is left)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from fdtd_gb300 import scenario as S, solver
    sc = S.config_small()
    cores = os.cpu_count() or 1

    def gpu(steps):
        with solver.Simulation.from_scenario(sc, probe_capacity=steps) as sim:
            sim.step(steps)
            sim.synchronize()
            return sim.read_probes(0, steps).astype(np.float64), sim.fields().astype(np.float64)

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))
    p, _ = gpu(sc.steps)
    p64, _ = oracle.run(sc, precision="f64", threads=cores)
    _, f = gpu(150)
    _, f64 = oracle.run(sc, steps=150, precision="f64", threads=cores)
    return {"workload": "64^3 vacuum, 10-cell CPML, 1 source, 1 Ez probe",
            "probes_rel_l2": rel(p, p64), "probe_steps": sc.steps,
            "e_fields_rel_l2": rel(f[:3], f64[:3]), "h_fields_rel_l2": rel(f[3:], f64[3:]), "field_steps": 150,
            "note": "the solver equals the reference's kernels bit for bit on this workload "
                    "(tests/golden/vacuum64.npz); this is the FP32 error of the scheme itself"}


# DRAM bytes per cell update of one two-pass step (k_update_e + k_update_h), from an ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum) of the 256^3 random-box case: 78.15 B. Larger
# grids are scaled by cells (an upper bound: their CPML share is smaller).
TWO_PASS_DRAM_BYTES_PER_CELL = 78.15


# DRAM bytes per cell update of one fused step (k_shell_e + k_sweep_interior + k_shell_h),
# dram__bytes_read.sum + dram__bytes_write.sum from ncu captures of these kernels (the launch-list
# commands in profiles/yee_step_boxes512_launch_list.md): 63.59 B on the 512^3 bench workload
# itself, 72.77 B at 256^3, where the shell share is larger. Refreshed whenever the kernels change.
FUSED_DRAM_BYTES_PER_CELL = {"512": 63.59, "256": 72.77}


def measured_traffic(schedule, cells, config):
    if schedule == 3:
        return None  # not profiled
    if schedule == 2:
        per_cell = FUSED_DRAM_BYTES_PER_CELL.get(config)
        if per_cell is None:
            return None  # no capture of this workload's DRAM bytes
    else:
        per_cell = TWO_PASS_DRAM_BYTES_PER_CELL
    return round(per_cell * cells)


def bench_ours(args, rank, world):
    import torch
    from fdtd_gb300 import solver
    sc, desc = scenario_for(args.config)
    B = algorithmic_bytes_per_cell(sc)
    N = sc.cells
    total_steps = args.warmup + args.steps
    if len(sc.sources[0].waveform) < total_steps:
        from fdtd_gb300 import scenario as S
        for s in sc.sources:
            s.waveform = np.resize(s.waveform, total_steps).astype(np.float32)
    mat = sc.material_index()
    stream = torch.cuda.Stream()
    sim = solver.Simulation.from_scenario(sc, args.schedule, material_index=mat, probe_capacity=total_steps)
    sim.set_stream(stream.cuda_stream)
    sim.prepare()
    sim.tune_schedule()  # AUTO: time both schedules on this grid (state kept) and keep the faster
    sim.step(args.warmup)
    sim.synchronize()
    active = sim.active_schedule
    # fused: shell E, sweep, shell H (and the CPML sweep); two-pass: E and H
    launches_per_step = {2: 3, 3: 4}.get(active, 2)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(torch.cuda.current_device())
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    e0.record(stream)
    sim.step(args.steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    ms = max_over_ranks(ms, world)
    probes = sim.read_probes(total_steps - 1, 1)
    assert np.all(np.isfinite(probes))
    sim.close()
    del sim
    value = replica_value(N, args.steps, ms, world)
    step_ms = ms / args.steps
    peak, peak_kind = measured_peak()
    achieved = B * N / (step_ms * 1e-3) / 1e9
    out = {"metric": "Gcell-updates/s", "value": round(value, 3), "unit": "Gcell-updates/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 4),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded random-box scenario)",
           "config": {"workload": desc, "cells": N, "grid": [sc.nx, sc.ny, sc.nz], "cpml": 10,
                      "schedule": {0: "auto", 1: "two-pass", 2: "fused", 3: "fused-cpml"}[args.schedule] +
                                  (" (fused)" if args.schedule == 0 and active == 2 else
                                   " (two-pass)" if args.schedule == 0 else ""),
                      "l2": f"inputs larger than L2 (fields 24 B/cell x {N / 1e6:.0f}M cells)",
                      "parallelism": f"replicas{world}"},
           "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(achieved / peak, 4), "traffic": measured_traffic(active, N, args.config),
                        "bytes_per_cell_update": round(B, 3), "peak_source": peak_kind,
                        "kernel": "one full time step (all update launches of the step)"},
           "gpu_launches": launches_per_step * args.steps, "clocks": clk}
    if not args.no_e2e:
        out["e2e"] = e2e_ours(args, sc, mat)
        out["e2e"]["value"] = round(world * out["e2e"]["value"], 3)
    return out


def e2e_ours(args, sc, mat):
    """Same metric through the C ABI from host buffers: handle creation, material table and index
    upload (pinned), waveform upload, K steps, probe read-back (the handle is destroyed after the
    timer stops). A second run times each phase with a synchronize after it, destroy included."""
    import torch
    from fdtd_gb300 import solver
    pinned = torch.from_numpy(mat).pin_memory()
    host_mat = pinned.numpy()
    steps = args.steps
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim = solver.Simulation.from_scenario(sc, args.schedule, material_index=host_mat, probe_capacity=steps)
    sim.step(steps)
    probes = sim.read_probes(0, steps)
    t1 = time.perf_counter()
    sim.close()  # after the result is on the host: not part of the timed job
    h2d = host_mat.nbytes + sum(s.waveform.nbytes for s in sc.sources)
    d2h = probes.nbytes
    out = {"value": sc.cells * steps / (t1 - t0) / 1e9, "unit": "Gcell-updates/s",
           "h2d_bytes_per_step": round(h2d / steps, 1), "d2h_bytes_per_step": round(d2h / steps, 1),
           "seconds": round(t1 - t0, 4), "steps": steps}
    # phase breakdown (separate run, synchronised between phases)
    ph = {}
    t = time.perf_counter()

    def mark(name):
        nonlocal t
        torch.cuda.synchronize()
        now = time.perf_counter()
        ph[name] = round((now - t) * 1e3, 2)
        t = now
    sim = solver.Simulation(sc.nx, sc.ny, sc.nz, sc.dx, sc.dy, sc.dz, sc.dt, sc.pml, sc.eps0, sc.mu0, sc.pi,
                            args.schedule)
    mark("create_ms")
    sim.set_materials(sc.material_table())
    sim.set_material_index(host_mat)
    for q in sc.sources:
        sim.add_source(q.box, q.resistance, q.waveform)
    for q in sc.probes:
        sim.add_probe(q.component, q.i, q.j, q.k)
    sim.set_probe_capacity(steps)
    mark("upload_ms")
    sim.prepare()
    sim.synchronize()
    mark("prepare_ms")
    first = min(8, steps)
    sim.step(first)
    sim.synchronize()
    mark("first_8_steps_ms")
    sim.step(steps - first)
    sim.synchronize()
    mark("other_steps_ms")
    sim.read_probes(0, steps)
    mark("readback_ms")
    sim.close()
    mark("destroy_ms")
    out["phases"] = ph
    return out


def bench_hbm(warmup=3, steps=20):
    """The 1024 x 1024 x 896 single domain (939.5 M cells, the same random-box generator, 10-cell
    CPML, 4 sources, 16 probes): device-timed steps with the grid resident, its own roofline."""
    import torch
    from fdtd_gb300 import solver
    sc, desc = scenario_for("hbm")
    B = algorithmic_bytes_per_cell(sc)
    mat = sc.material_index()
    stream = torch.cuda.Stream()
    sim = solver.Simulation.from_scenario(sc, 0, material_index=mat, probe_capacity=warmup + steps + 64)
    del mat
    sim.set_stream(stream.cuda_stream)
    sim.prepare()
    sim.tune_schedule()
    sim.step(warmup)
    sim.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    e0.record(stream)
    sim.step(steps)
    e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    active = sim.active_schedule
    dev_bytes = sim.device_bytes()
    sim.close()
    ms = e0.elapsed_time(e1) / steps
    peak, peak_kind = measured_peak()
    achieved = B * sc.cells / (ms * 1e-3) / 1e9
    return {"workload": desc, "grid": [sc.nx, sc.ny, sc.nz], "cells": sc.cells, "steps": steps, "warmup": warmup,
            "value": round(sc.cells / (ms * 1e-3) / 1e9, 3), "unit": "Gcell-updates/s", "ms_per_step": round(ms, 4),
            "schedule": {1: "two-pass", 2: "fused", 3: "fused-cpml"}.get(active, str(active)),
            "device_gb": round(dev_bytes / 1e9, 2),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "bytes_per_cell_update": round(B, 3),
                         "peak_source": peak_kind},
            "clocks": clk}


def bench_adjoint(steps=4000):
    """Adjoint cost on the 128^3 design problem (32x32x16 centred design region, eps_r ~ U[1,12],
    10-cell CPML, one source, one Ez probe, 4000 steps): plain forward, forward with checkpoints
    every 64 steps + backward with segment recompute, and the resident-history variant (K = 0).
    Wall-clock around the synchronous C calls; every run starts from a fresh handle."""
    import torch
    from fdtd_gb300 import scenario as S, solver
    d = S.design_problem(steps=steps)
    sc = d.scenario

    def fresh():
        sim = solver.Simulation.from_scenario(sc, probe_capacity=sc.steps)
        sim.set_design_region(d.box, d.eps)
        sim.prepare()
        sim.synchronize()
        return sim

    sim = fresh(); sim.step(64); sim.synchronize(); sim.close()  # warm-up
    sim = fresh()
    t0 = time.perf_counter(); sim.step(sc.steps); sim.synchronize(); t_plain = time.perf_counter() - t0
    sim.close()
    out = {"workload": "128^3 vacuum, 10-cell CPML, 32x32x16 design region eps_r~U[1,12], 1 source, 1 Ez probe, "
                       "FoM sum dt*Ez^2", "steps": sc.steps, "forward_ms": round(t_plain * 1e3, 2)}
    for K, key in ((64, "checkpoint64"), (0, "resident")):
        sim = fresh()
        t0 = time.perf_counter(); J = sim.adjoint_forward(sc.steps, d.probe, K); t1 = time.perf_counter()
        g = sim.adjoint_backward(); t2 = time.perf_counter()
        sim.close()
        out[key] = {"adjoint_forward_ms": round((t1 - t0) * 1e3, 2), "backward_ms": round((t2 - t1) * 1e3, 2),
                    "ratio": round((t2 - t0) / t_plain, 3), "backward_over_forward": round((t2 - t1) / t_plain, 3),
                    "J": J, "grad_l2": float(np.linalg.norm(g))}
    return out


def bench_batched(steps=2000):
    """256 independent instances (per-axis sizes U{32..96}, 8-cell CPML, 8 dielectric boxes, one
    source and one probe each): the same instances run one by one through fdtd_step, then together
    through the batched launch (autotuned over the chain, flat and persistent forms, CUDA graphs).
    Handle creation and setup are outside both timings; both advance every instance by `steps`
    steps."""
    import torch
    from fdtd_gb300 import scenario as S, solver
    scs = S.batch_instances(256, steps=2 * steps + 16)
    cells = sum(sc.cells for sc in scs)
    sims = [solver.Simulation.from_scenario(sc, probe_capacity=2 * steps + 16) for sc in scs]
    for s in sims:
        s.prepare()
        s.step(2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in sims:
        s.step(steps)
    for s in sims:
        s.synchronize()
    t_seq = time.perf_counter() - t0
    with solver.Batch(sims) as b:
        tune_ms = b.tune(5)
        # capture the graphs the timed run replays (a 32-step chunk and the remainder)
        b.step(32)
        if steps % 32:
            b.step(steps % 32)
        b.synchronize()
        t0 = time.perf_counter()
        b.step(steps)
        b.synchronize()
        t_bat = time.perf_counter() - t0
        cfg = b.config
    for s in sims:
        s.close()
    seq = cells * steps / t_seq / 1e9
    bat = cells * steps / t_bat / 1e9
    return {"workload": "256 instances, per-axis sizes U{32..96}, 8-cell CPML, 8 boxes eps_r~U[1,12], 1 source + "
                        "1 probe each", "instances": len(scs), "cells": cells, "steps": steps,
            "sequential": {"value": round(seq, 3), "unit": "Gcell-updates/s", "seconds": round(t_seq, 3),
                           "gpu_launches": 2 * steps * len(scs)},
            "batched": {"value": round(bat, 3), "unit": "Gcell-updates/s", "seconds": round(t_bat, 3),
                        "gpu_launches": {-1: 2 * steps * len(scs) + -(-steps // 32), 0: 3 * steps}.get(cfg["cluster"], 1),
                        "config": cfg,
                        "form": {-1: "chains (each instance's two-pass kernels, concurrent graph branches)",
                                 0: "flat (E, H, step-counter kernels per step)"}.get(cfg["cluster"], "persistent clusters"),
                        "tune_ms_5_steps": round(tune_ms, 2)},
            "speedup": round(bat / seq, 2)}


def bench_batched_adjoint(n_instances=64, steps=1000, K=64):
    """Forward + adjoint of independent design problems (cubes with per-instance sizes U{44..96},
    8-cell CPML, a centred 16x16x8 design region, eps_r ~ U[1,12], one source and one Ez probe
    each; checkpoints every K steps): the instances one after another through
    fdtd_adjoint_forward / fdtd_adjoint_backward, then all together through fdtd_batch_adjoint,
    each simulation on its own stream. Handle creation, setup and the adjoint buffers' allocation
    (one untimed batched run) are outside both timings."""
    import torch
    from fdtd_gb300 import scenario as S, solver
    rng = np.random.default_rng(21)
    probs = [S.design_problem(int(rng.integers(44, 97)), steps, (16, 16, 8), pml=8, seed=q) for q in range(n_instances)]
    streams = [torch.cuda.Stream() for _ in probs]
    sims = []
    for d, st in zip(probs, streams):
        sim = solver.Simulation.from_scenario(d.scenario, probe_capacity=1)
        sim.set_stream(st.cuda_stream)
        sim.set_design_region(d.box, d.eps)
        sim.prepare()
        sims.append(sim)
    try:
        # warm-up: every handle allocates its adjoint buffers once (later runs of the same length reuse them)
        solver.batch_adjoint(sims, steps, [d.probe for d in probs], K)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for sim, d in zip(sims, probs):
            sim.adjoint_forward(steps, d.probe, K)
            sim.adjoint_backward()
        t_seq = time.perf_counter() - t0
        t0 = time.perf_counter()
        solver.batch_adjoint(sims, steps, [d.probe for d in probs], K)
        t_bat = time.perf_counter() - t0
    finally:
        for sim in sims:
            sim.close()
    cells = sum(d.scenario.cells for d in probs)
    return {"workload": f"{n_instances} design instances, cube sizes U{{44..96}}, 8-cell CPML, 16x16x8 design region "
                        "eps_r~U[1,12], 1 source + 1 Ez probe each, forward + adjoint",
            "instances": n_instances, "cells": cells, "steps": steps, "checkpoint_every": K,
            "sequential_s": round(t_seq, 3), "batched_s": round(t_bat, 3), "speedup": round(t_seq / t_bat, 2)}


def bench_reference(args, rank, world):
    """The reference's own kernels (calc_e + calc_h from fdtdrav.h, built into oracle/_ref) on the
    same workload, single slab on this GPU."""
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref_harness"))
    import refharness
    sc, desc = scenario_for(args.config)
    if not refharness.available():
        return {"impl": "reference", "unavailable": "oracle/_ref (reference kernels) not built"}
    need = sc.cells * 84 * 4
    import torch
    free, _ = torch.cuda.mem_get_info()
    if need > free * 0.95:
        return {"impl": "reference", "unavailable": f"the reference layout needs {need / 1e9:.0f} GB (84 arrays x 4 B x "
                                                    f"{sc.cells} cells), more than this GPU holds"}
    h = refharness.RefHarness()
    h.setup(sc)
    sig = np.resize(sc.signal_per_node(0), args.warmup + args.steps + 1).astype(np.float32)
    h.run(args.warmup, 0, 0, sig)
    barrier(world)
    _, ms = h.run(args.steps, args.warmup, 0, sig)
    h.close()
    ms = max_over_ranks(ms, world)
    value = world * sc.cells * args.steps / (ms * 1e-3) / 1e9
    return {"impl": "reference", "metric": "Gcell-updates/s", "value": round(value, 3), "unit": "Gcell-updates/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded random-box scenario)",
            "config": {"workload": desc, "cells": sc.cells, "grid": [sc.nx, sc.ny, sc.nz],
                       "l2": "inputs larger than L2", "parallelism": f"replicas{world}",
                       "note": "reference kernels inject one source per launch; timing does not depend on it"},
            "cpu_baseline": {"value": round(value, 3), "unit": "Gcell-updates/s", "cores": 0, "kind": "reference",
                             "sample": "the reference's own CUDA kernels (calc_e + calc_h per step, fdtdrav.h "
                                       "built for sm_103a) timed with CUDA events on this GPU; the reference has "
                                       "no CPU implementation of the path"},
            "e2e": {"value": round(value, 3), "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "gpu_launches": 2 * args.steps}


def main():
    args = parse()
    import torch
    rank, world = dist_setup(args.gpus)
    if args.impl == "reference":
        if rank != 0:
            return
        out = bench_reference(args, rank, 1)
        print(json.dumps(out))
        return
    out = bench_ours(args, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline()
        if world == 1 and not args.no_fp64:
            out["fp64_error"] = fp64_error()
        if not args.no_adjoint and world == 1:
            out["adjoint"] = bench_adjoint(args.adjoint_steps)
        if not args.no_batched and world == 1:
            out["batched"] = bench_batched()
            out["batched_adjoint"] = bench_batched_adjoint()
        if not args.no_hbm and world == 1 and args.config != "hbm":
            out["hbm"] = bench_hbm()
        print(json.dumps(out))


if __name__ == "__main__":
    main()
