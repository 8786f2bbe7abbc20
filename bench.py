#!/usr/bin/env python
"""Coupled PSM lattice-step benchmark (MLUPS and HBM roofline fraction).

Workload: periodic 256^3 lattice, tau = 0.55, 2000 spheres of radius 8 at
seeded non-overlapping uniform random centres (solid fraction 0.256),
velocities N(0, 0.01), angular velocities N(0, 1e-3), prescribed kinematics
(x += v per step, periodic wrap, ghost images appended as LIGGGHTS would).
A step is one coupling cycle: voxelize the spheres, collide-stream the whole
lattice with the PSM dynamics, sum per-particle force and torque.

MLUPS = lattice cells x steps / seconds / 1e6 (all cells, solid included).

Windows.  Driven by random prescribed kinematics with no DEM feedback, the
reference's PSM update gains mass every step (its rest-population term) and
the run goes non-finite after about 400 steps, in the FP64 and the FP32 form
alike; prescriptions that keep the spheres near their seeded places only
delay it (near step 700).  The lattice is therefore put back to rest every
WINDOW steps (one equilibrium write, ~0.1 % of a window's time, inside the
timed region); every step still voxelizes, collide-streams and sums forces in
full.

Headline `value`: FP32-deviation form, particle tables already in HBM, timed
with CUDA events on the launching stream.  `fp64` carries the FP64 drop-in
form on the same inputs, and `force_rel_err_fp32_vs_fp64` the per-particle
force error between the two after the run.  `e2e` is the FP32 form through
the C ABI (lbdem_cycle) with host buffers: the particle table copy in, the
forces copy out and the per-step synchronisation are inside the timed region;
`fp64.e2e` is the same for the FP64 form over a bounded number of cycles.

`--impl reference` times the CPU oracle (a restatement of the reference's
path; the reference itself needs Palabos, LIGGGHTS and MPI) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "lbdemcoupling-public_gb300"
for _p in (str(ROOT), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "coupled PSM MLUPS & %HBM roofline, FP32 vs FP64 form at force err ≤1e-4"
SHAPE = (256, 256, 256)   # --edge changes it (profiling runs on smaller cubes)
TAU = 0.55
SEED = 2024
WORKLOAD = "monodisperse suspension, periodic 256^3, 2000 spheres r=8, tau=0.55, prescribed kinematics"
WINDOW = 300   # steps between returns of the lattice to rest (see the module docstring)
E2E_FP64_STEPS = 100   # cycles of the FP64 form's end-to-end leg (about 0.8 s at 256^3)
BYTES_PER_CELL = {"fp32": 2 * 19 * 4 + 4, "fp64": 2 * 19 * 8 + 4}  # 19 loads + 19 stores + voxel word


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """Per collide-stream launch, from the committed ncu summary
    (profiles/collide_stream_traffic.txt): DRAM bytes ("fp32", "fp64") and the FP64
    form's double-precision thread instructions ("fp64_dp_ops")."""
    p = ROOT / "profiles" / "collide_stream_traffic.txt"
    out = {}
    if p.exists():
        for line in p.read_text().splitlines():
            parts = line.split()
            if len(parts) >= 2 and parts[0] in ("fp32", "fp64", "fp64_dp_ops", "fp64_pipe_active"):
                try:
                    out[parts[0]] = float(parts[1])
                except ValueError:
                    pass
    return out


def sm_count(device):
    import torch
    return int(torch.cuda.get_device_properties(device).multi_processor_count)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def particles():
    """The benchmark's spheres: workloads.monodisperse_256 at 256^3; on a smaller cube
    (--edge) the same construction with the sphere count scaled to the volume
    (the same solid fraction)."""
    import workloads as W
    if SHAPE == (256, 256, 256):
        return W.monodisperse_256(SEED)[1]
    n = int(round(2000 * float(np.prod(SHAPE)) / 256 ** 3))
    return W.suspension(SHAPE, n_max=n, radius=8.0, seed=SEED)


def build_tables(n_steps: int):
    """Per-step particle tables (ghost images included) for prescribed kinematics."""
    import workloads as W
    import lbdem
    p = particles()
    recs, host = [], []
    for _ in range(n_steps):
        g = W.with_ghosts(p, SHAPE)
        recs.append(lbdem.pack_records(g.x, g.v, g.w, g.r, g.tag))
        host.append(g)
        p = W.advance(p, SHAPE)
    offs = np.cumsum([0] + [r.shape[0] for r in recs])
    return np.concatenate(recs), offs, host, p.n


def run_device(prec_name: str, table, offs, steps: int, warmup: int, max_n: int, max_tag: int, device: int):
    import torch
    import lbdem
    prec = lbdem.PREC_FP32_DEV if prec_name == "fp32" else lbdem.PREC_FP64
    lat = lbdem.Lattice(*SHAPE, 1.0 / TAU, precision=prec, max_particles=max_n, max_tag=max_tag,
                        max_radius=8.0, device=device)
    stream = torch.cuda.Stream(device=device)
    lat.set_stream(stream.cuda_stream)
    d_tab = torch.from_numpy(table).to(f"cuda:{device}")
    d_out = torch.zeros(6 * max_n, dtype=torch.float64, device=f"cuda:{device}")
    base = d_tab.data_ptr()
    torch.cuda.synchronize(device)

    def step(s):
        n = int(offs[s + 1] - offs[s])
        if s > 0 and s % WINDOW == 0:
            lat.init_equilibrium()
        lat.set_particles_device(n, base + int(offs[s]) * 12 * 8)
        lat.collide_and_stream()
        lat.get_forces_device(d_out.data_ptr())

    with torch.cuda.stream(stream):
        for s in range(warmup):
            step(s)
        torch.cuda.synchronize(device)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
               torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        l0 = lat.launch_count()
        with ClockSampler(device) as clk:
            torch.cuda.synchronize(device)
            t0.record(stream)
            for k in range(steps):
                s = warmup + k
                n = int(offs[s + 1] - offs[s])
                e_a, e_b, e_c = ev[k]
                if s > 0 and s % WINDOW == 0:
                    lat.init_equilibrium()
                e_a.record(stream)
                lat.set_particles_device(n, base + int(offs[s]) * 12 * 8)
                e_b.record(stream)
                lat.collide_and_stream()
                e_c.record(stream)
                lat.get_forces_device(d_out.data_ptr())
            t1.record(stream)
            torch.cuda.synchronize(device)
        launches = lat.launch_count() - l0
    total_ms = t0.elapsed_time(t1)
    k2 = [a.elapsed_time(b) for a, b, _ in ev]
    k1 = [b.elapsed_time(c) for _, b, c in ev]
    n_last = int(offs[warmup + steps] - offs[warmup + steps - 1])
    F = d_out[: 3 * n_last].cpu().numpy().reshape(n_last, 3)
    errs = lat.device_errors()
    lat.close()
    return {"total_ms": total_ms, "k1_ms": float(np.mean(k1)), "k2_ms": float(np.mean(k2)),
            "k1_ms_min": float(np.min(k1)), "launches": launches, "F": F, "clocks": clk.summary(),
            "device_errors": errs}


def run_e2e(host_tables, steps: int, warmup: int, max_n: int, max_tag: int, device: int, prec: str = "fp32"):
    """One form through the C ABI's lbdem_cycle with host buffers: the particle
    table copy in, the kernels, the force/torque copy out and the synchronisation
    are inside the timed region.  The ctypes argument tuples of every step are
    built before it, so the region holds the C-ABI calls themselves and not the
    Python binding's per-call argument marshalling (which a C or C++ caller of
    the ABI does not have)."""
    import ctypes as C

    import lbdem
    lat = lbdem.Lattice(*SHAPE, 1.0 / TAU,
                        precision=lbdem.PREC_FP32_DEV if prec == "fp32" else lbdem.PREC_FP64,
                        max_particles=max_n, max_tag=max_tag, max_radius=8.0, device=device)
    F = np.zeros((max_n, 3))
    T = np.zeros((max_n, 3))
    for s in range(warmup):
        g = host_tables[s]
        if s > 0 and s % WINDOW == 0:
            lat.init_equilibrium()
        lat.cycle(g.x, g.v, g.w, g.r, g.tag, F=F[: g.n], T=T[: g.n])
    dp = C.POINTER(C.c_double)
    keep, calls = [], []
    for k in range(steps):
        g = host_tables[warmup + k]
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (g.x, g.v, g.w, g.r)]
        tag = np.ascontiguousarray(g.tag, dtype=np.int32)
        keep.append((arrs, tag))
        calls.append((lat.h, g.n, *[a.ctypes.data_as(dp) for a in arrs],
                      tag.ctypes.data_as(C.POINTER(C.c_int32)), 0, F.ctypes.data_as(dp), T.ctypes.data_as(dp)))
    cycle = lat.lib.lbdem_cycle
    h2d = d2h = 0
    t0 = time.perf_counter()
    for k in range(steps):
        if (warmup + k) % WINDOW == 0:
            lat.init_equilibrium()
        st = cycle(*calls[k])
        if st != 0:
            lat._check(st)
        n = calls[k][1]
        h2d += n * 12 * 8
        d2h += n * 6 * 8 + 4
    dt = time.perf_counter() - t0
    lat.close()
    return dt, h2d / steps, d2h / steps


def cpu_oracle_mlups(host_tables, budget_s: float, max_cycles: int, threads: int):
    """Bounded sample of the same workload on the CPU oracle (full 256^3 cycles)."""
    from oracle import psm_oracle
    ol = psm_oracle.OracleLattice(*SHAPE, 1.0 / TAU, threads=threads)
    done = 0
    t0 = time.perf_counter()
    while done < max_cycles:
        g = host_tables[done % len(host_tables)]
        ol.set_particles(g.x, g.v, g.w, g.r, g.tag)
        ol.collide_and_stream()
        ol.get_forces()
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    N = int(np.prod(SHAPE))
    return N * done / dt / 1e6, done, dt


def run_batched(steps: int, warmup: int, single_steps: int, device: int, flow_axis: int = 2):
    """Batched pressure-driven channels (workloads.channels: 512 domains, FP32
    deviation form): aggregate MLUPS of the batch -- graph replay of one launch
    per stage over all domains -- through the host-buffer cycle call, of the
    replayed step alone, and of the same domains stepped one handle at a time
    (every stage launched per domain, one synchronization per cycle)."""
    import ctypes as C

    import lbdem
    import workloads as W
    ch = W.channels(flow_axis=flow_axis)
    doms = [d for d, _ in ch]
    cells = sum(int(np.prod(d["shape"])) for d in doms)
    nt = min(warmup + max(steps, single_steps), 16)
    per_step, per_dom = [], []
    q = [p for _, p in ch]
    for _ in range(nt):
        g = [W.with_ghosts(p, d["shape"], d["periodic"]) for d, p in zip(doms, q)]
        counts = np.array([x.n for x in g], dtype=np.int32)
        rec = np.concatenate([lbdem.pack_records(x.x, x.v, x.w, x.r, x.tag) for x in g])
        per_step.append((counts, rec))
        per_dom.append(g)
        q = [W.advance(p, d["shape"], d["periodic"]) for d, p in zip(doms, q)]

    B = lbdem.Batch(doms, precision=lbdem.PREC_FP32_DEV, max_tag=64, max_radius=8.0, device=device)
    for s in range(warmup):
        B.cycle(*per_step[s % nt], init_vel=False)
    B.synchronize()
    t0 = time.perf_counter()
    for s in range(steps):
        B.cycle(*per_step[(warmup + s) % nt])
    t_e2e = time.perf_counter() - t0
    t0 = time.perf_counter()
    for s in range(steps):
        B.step()
    B.synchronize()
    t_dev = time.perf_counter() - t0
    n0 = B.launch_count()
    B.step()
    B.synchronize()
    launches = B.launch_count() - n0
    bps, k1_ms = B.tuning()
    B.close()

    lib = lbdem.load()
    Ls = []
    for d in doms:
        L = lbdem.Lattice(*d["shape"], d["omega"], periodic=d["periodic"], precision=lbdem.PREC_FP32_DEV,
                          max_particles=d["max_particles"], max_tag=64, max_radius=8.0, device=device)
        dr = d["drop"]
        L.set_pressure_drop(dr["dimension"], dr["inlet"], dr["outlet"], dr["rho_in"], dr["rho_out"])
        Ls.append(L)
    D = C.POINTER(C.c_double)
    calls = []   # per table: per domain the pointer arguments of lbdem_set_particles
    keep = []
    for g in per_dom:
        row = []
        for x in g:
            arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x.x, x.v, x.w, x.r)]
            tag = np.ascontiguousarray(x.tag, dtype=np.int32)
            keep.append((arrs, tag))
            row.append((x.n, *[a.ctypes.data_as(D) for a in arrs], tag.ctypes.data_as(C.POINTER(C.c_int32))))
        calls.append(row)
    Fbuf = [np.zeros((max(L.cfg.max_particles, 1), 3)) for L in Ls]
    Tbuf = [np.zeros((max(L.cfg.max_particles, 1), 3)) for L in Ls]

    def cycle_all(s):
        row = calls[s % nt]
        for L, a in zip(Ls, row):
            lib.lbdem_set_particles(L.h, a[0], a[1], a[2], a[3], a[4], a[5], 0)
            lib.lbdem_collide_and_stream(L.h)
        for L, a, F, T in zip(Ls, row, Fbuf, Tbuf):
            lib.lbdem_get_forces(L.h, a[0], F.ctypes.data_as(D), T.ctypes.data_as(D))

    for s in range(2):
        cycle_all(s)
    t0 = time.perf_counter()
    for s in range(single_steps):
        cycle_all(2 + s)
    t_one = time.perf_counter() - t0
    for L in Ls:
        L.close()
    peak, _ = peaks()
    ach = BYTES_PER_CELL["fp32"] * cells / (k1_ms * 1e-3) / 1e9 if k1_ms > 0 else None
    return {
        "workload": f"{len(doms)} pressure-driven channels, length U[64,160] along the flow (stored along "
                    f"{'xyz'[flow_axis]}), square cross-section U[24,48] between walls, 1-40 spheres r U[3,6] each, "
                    f"tau 0.6, fp32 deviation form",
        "cells": cells, "particles_local": int(sum(p.n for _, p in ch)),
        "value": cells * steps / t_e2e / 1e6, "unit": "MLUPS",
        "note": "value: lbdem_batch_cycle with host buffers (upload of the particle table and download of the "
                "forces inside the replayed graph), wall clock over the timed cycles",
        "device_value": cells * steps / t_dev / 1e6,
        "one_at_a_time": cells * single_steps / t_one / 1e6,
        "one_at_a_time_steps": single_steps,
        "speedup_vs_one_at_a_time": (cells * steps / t_e2e) / (cells * single_steps / t_one),
        "launches_per_step": launches, "launches_per_step_one_at_a_time": 4 * len(doms),
        "collide_blocks_per_sm": bps, "k1_ms": k1_ms,
        "k1_roofline": None if ach is None else {"achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                                                   "bytes_per_cell": BYTES_PER_CELL["fp32"]},
    }


def run_adjoint():
    """A short adjoint window of the 128^3 adjoint workload in both forms: the cost of
    the backward pass against the forward pass (reports.py adjoint has the full
    200-step window with its accuracy checks)."""
    import reports
    out = {"workload": "periodic 128^3, 64 spheres r = 6, body force 1e-6, 40 steps, checkpoint every 10, "
                       "loss = sum of x-forces of every step"}
    for name, fp64 in (("fp32", False), ("fp64", True)):
        r = reports.window(steps=40, K=10, fp64=fp64)
        out[name] = {"forward_ms": r["forward_ms"], "backward_ms": r["backward_ms"],
                     "backward_over_forward": r["backward_ms"] / r["forward_ms"], "loss": r["loss"]}
    return out


def max_over_ranks(values, dist, device):
    """Element-wise maximum of per-rank timings over all ranks of the process group
    (a replica's time is the slowest rank's: every rank runs its own lattice)."""
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU-oracle work")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--forms", default="fp32,fp64", help="population forms to time (fp32 is the headline)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer C-ABI leg (profiling runs)")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-channels leg")
    ap.add_argument("--batched-steps", type=int, default=60)
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint-window leg")
    ap.add_argument("--edge", type=int, default=256,
                    help="cube edge of the workload (profiling on smaller cases; the benchmark is 256)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    global SHAPE, WORKLOAD
    if args.edge != 256:
        SHAPE = (args.edge,) * 3
        WORKLOAD = WORKLOAD.replace("256^3", f"{args.edge}^3").replace(
            "2000 spheres", f"{int(round(2000 * args.edge ** 3 / 256 ** 3))} spheres")

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    threads = os.cpu_count() or 1
    N = int(np.prod(SHAPE))

    if args.impl == "reference":
        if rank != 0:
            return
        import workloads as W
        p = particles()
        tables = []
        q = p
        for _ in range(min(args.warmup + args.steps, 64)):
            tables.append(W.with_ghosts(q, SHAPE))
            q = W.advance(q, SHAPE)
        from oracle import psm_oracle
        ol = psm_oracle.OracleLattice(*SHAPE, 1.0 / TAU, threads=threads)
        for s in range(min(args.warmup, 1)):
            g = tables[s]
            ol.set_particles(g.x, g.v, g.w, g.r, g.tag); ol.collide_and_stream(); ol.get_forces()
        budget = 120.0
        done = 0
        t0 = time.perf_counter()
        while done < args.steps and time.perf_counter() - t0 < budget:
            g = tables[(done + 1) % len(tables)]
            ol.set_particles(g.x, g.v, g.w, g.r, g.tag); ol.collide_and_stream(); ol.get_forces()
            done += 1
        dt = time.perf_counter() - t0
        mlups = N * done / dt / 1e6
        sample = f"{done} of {args.steps} coupling cycles on the full 256^3 workload (time-bounded)"
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": mlups, "unit": "MLUPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(done, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "form": "fp64 CPU oracle"},
            "cpu_baseline": {"value": mlups, "unit": "MLUPS", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": mlups, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }))
        return

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = local if world > 1 else 0
    table, offs, host, n_local = build_tables(args.warmup + args.steps)
    max_n = int(np.max(np.diff(offs)))
    max_tag = n_local + 1

    if dist:
        dist.barrier()
    forms = [f.strip() for f in args.forms.split(",") if f.strip()]
    if "fp32" not in forms:
        ap.error("--forms must include fp32 (the headline form)")
    r32 = run_device("fp32", table, offs, args.steps, args.warmup, max_n, max_tag, device)
    r64 = run_device("fp64", table, offs, args.steps, args.warmup, max_n, max_tag, device) if "fp64" in forms else None
    # the FP64 form's end-to-end leg runs a bounded number of the same cycles
    steps64_e2e = min(args.steps, E2E_FP64_STEPS)
    if args.no_e2e:
        e2e_s, h2d, d2h = float("nan"), 0, 0
        e2e64_s = float("nan")
    else:
        e2e_s, h2d, d2h = run_e2e(host, args.steps, args.warmup, max_n, max_tag, device)
        e2e64_s = (run_e2e(host, steps64_e2e, args.warmup, max_n, max_tag, device, "fp64")[0] if r64
                   else float("nan"))

    t32 = r32["total_ms"]
    if dist:
        t32, t64, e2e_s, e2e64_s = max_over_ranks([t32, r64["total_ms"] if r64 else 0.0, e2e_s, e2e64_s], dist,
                                                   f"cuda:{device}")
    else:
        t64 = r64["total_ms"] if r64 else float("nan")
    if rank != 0:
        dist.destroy_process_group()
        return

    peak, peak_kind = peaks()
    traffic = profiled_traffic()
    value = world * N * args.steps / (t32 * 1e-3) / 1e6
    v64 = world * N * args.steps / (t64 * 1e-3) / 1e6
    ach32 = BYTES_PER_CELL["fp32"] * N / (r32["k1_ms"] * 1e-3) / 1e9
    ach64 = BYTES_PER_CELL["fp64"] * N / (r64["k1_ms"] * 1e-3) / 1e9 if r64 else None
    # the coupled step against the same bytes: K1's algorithmic bytes per whole step
    step32 = BYTES_PER_CELL["fp32"] * N / (t32 / args.steps * 1e-3) / 1e9
    # FP64 form against its own ceiling: double-precision lanes per clock per SM (2 on
    # GB300) x SMs x the median SM clock sampled during its run
    fp64_pipe = None
    if r64 and traffic.get("fp64_dp_ops") and r64["clocks"].get("sm_mhz"):
        ops = traffic["fp64_dp_ops"]
        rate = ops / (r64["k1_ms"] * 1e-3) / 1e12
        peak_dp = 2.0 * sm_count(device) * r64["clocks"]["sm_mhz"] * 1e6 / 1e12
        fp64_pipe = {"bound": "fp64", "achieved": rate, "peak": peak_dp, "unit": "T DP lane-ops/s",
                     "frac": rate / peak_dp, "dp_ops_per_launch": ops, "dp_ops_per_cell": ops / N,
                     "peak_source": "2 FP64 lanes per clock per SM x SMs x median SM clock of the FP64 run",
                     "pipe_active_frac": (traffic["fp64_pipe_active"] / 100.0) if traffic.get("fp64_pipe_active")
                                         else None,
                     "pipe_note": "achieved/peak counts add/mul/fma only; pipe_active_frac (ncu) counts every "
                                  "FP64-pipe instruction (conversions, compares, the reciprocal sequence)",
                     "ops_source": "ncu smsp__sass_thread_inst_executed_op_d{add,mul,fma}_pred_on.sum, "
                                   "profiles/collide_stream_traffic.txt"}
    ferr = None
    if r64:
        F32, F64 = r32["F"], r64["F"]
        ferr = float(np.max(np.abs(F32 - F64)) / np.max(np.abs(F64)))

    batched = None
    if not args.no_batched and world == 1:
        batched = run_batched(args.batched_steps, args.warmup, 8, device)
    adjoint = None
    if not args.no_adjoint and world == 1:
        adjoint = run_adjoint()

    cpu = None
    if not args.no_cpu_baseline:
        mlups, cycles, secs = cpu_oracle_mlups(host, args.cpu_budget, 1000, threads)
        cpu = {"value": mlups, "unit": "MLUPS", "cores": threads, "kind": "port",
               "sample": f"{cycles} coupling cycles of the same 256^3 workload in {secs:.1f} s (FP64 oracle)"}

    out = {
        "metric": METRIC, "value": value, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t32 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "form": "fp32 deviation populations, fp64 force/torque sums",
                   "cells": N, "particles_local": n_local, "particles_with_ghosts_max": max_n,
                   "l2": "inputs larger than L2 (populations 1.27 GB fp32 / 2.55 GB fp64)",
                   "window_steps": WINDOW, "forces_finite": bool(np.isfinite(r32["F"]).all()),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": ach32, "peak": peak, "unit": "GB/s", "frac": ach32 / peak,
                     "traffic": traffic.get("fp32"), "kernel": "k_collide_staged<float> (all axes periodic)",
                     "bytes_per_cell": BYTES_PER_CELL["fp32"], "peak_source": peak_kind,
                     "k1_ms": r32["k1_ms"], "k2_voxelize_ms": r32["k2_ms"],
                     "step_achieved": step32, "step_frac": step32 / peak,
                     "step_note": "K1's algorithmic bytes per coupling step / ms_per_step (voxelization, "
                                  "collide-stream and force sums all inside the step)"},
        "fp64": None if r64 is None else {
            "value": v64, "unit": "MLUPS", "ms_per_step": t64 / args.steps,
            "vs_cpu": (v64 / cpu["value"]) if cpu else None,
            "vs_cpu_note": "FP64 form against the FP64 CPU oracle of cpu_baseline (same precision)",
            "clocks": r64["clocks"],
            "roofline": fp64_pipe if fp64_pipe else {"bound": "fp64", "achieved": None, "frac": None},
            "hbm": {"achieved": ach64, "peak": peak, "unit": "GB/s", "frac": ach64 / peak,
                    "traffic": traffic.get("fp64"), "kernel": "k_collide_staged<double> (all axes periodic)",
                    "bytes_per_cell": BYTES_PER_CELL["fp64"]},
            "k1_ms": r64["k1_ms"], "k2_voxelize_ms": r64["k2_ms"],
            "e2e": None if args.no_e2e else {
                "value": world * N * steps64_e2e / e2e64_s / 1e6, "unit": "MLUPS", "steps": steps64_e2e,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "vs_cpu": (world * N * steps64_e2e / e2e64_s / 1e6 / cpu["value"]) if cpu else None,
                "note": "FP64 form through lbdem_cycle with host buffers, against the FP64 CPU oracle"}},
        "force_rel_err_fp32_vs_fp64": ferr,
        "batched": batched,
        "adjoint": adjoint,
        "e2e": None if args.no_e2e else {"value": world * N * args.steps / e2e_s / 1e6, "unit": "MLUPS",
                                         "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "cpu_baseline": cpu,
        "clocks": r32["clocks"],
        "gpu_launches": r32["launches"],
        "device_errors": r32["device_errors"] | (r64["device_errors"] if r64 else 0),
    }
    print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
