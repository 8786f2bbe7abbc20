"""Accuracy and cost reports of the precision and adjoint forms on full-size workloads.

    python reports.py adjoint      # periodic 128^3, 64 spheres r = 6, 200 steps, checkpoint every 20
    python reports.py precision    # periodic 512x256x256, r ~ U[4, 10] to solid fraction 0.30, 2000 steps
    python reports.py window [--steps S --checkpoint K --fp64]   # one adjoint window of the 128^3 case, timed
    python reports.py channels [--steps S --flow-axis A --domains D]  # batched channels (512), S coupling cycles

Each prints one JSON object.  Inputs are seeded synthetic workloads
(workloads.py); the FP64 form is the reference of the FP32 deviation form.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import lbdem  # noqa: E402
import workloads as W  # noqa: E402


def _rel(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def adjoint(steps: int = 200, K: int = 20, seed: int = 2027, tau: float = 0.6, g=(1e-6, 0.0, 0.0)) -> dict:
    """Loss = sum of the particles' x-forces over the last 50 steps; gradients with
    respect to the per-step particle velocities and angular velocities, the body
    force and tau, from rest."""
    shape = (128, 128, 128)
    p = W.suspension(shape, n_max=64, radius=6.0, seed=seed)
    gh = W.with_ghosts(p, shape)
    m, nl = gh.n, p.n
    rec = np.repeat(lbdem.pack_records(gh.x, gh.v, gh.w, gh.r, gh.tag)[None], steps, axis=0)
    weights = np.zeros((steps, m, 6))
    weights[steps - 50:, :nl, 0] = 1.0

    def lattice(prec, tau_=tau, g_=g):
        return lbdem.Lattice(*shape, 1.0 / tau_, periodic=(1, 1, 1), precision=prec, body_force=g_,
                             max_particles=m, max_tag=nl + 1, max_radius=8.0)

    def window(prec, k):
        with lattice(prec) as L:
            out = L.adjoint_window(rec, weights, k)
            fwd, bwd = L.adjoint_timing()
        return out, fwd, bwd

    o64, f64, b64 = window(0, K)
    o32, f32, b32 = window(1, K)
    otape, ftape, btape = window(0, 1)

    def loss_of(rec_=rec, g_=g, tau_=tau):
        with lattice(0, tau_, g_) as L:
            s = 0.0
            for t in range(steps):
                r = rec_[t]
                L.set_particles(r[:, 0:3], r[:, 3:6], r[:, 6:9], r[:, 9], r[:, 10].astype(np.int32))
                L.collide_and_stream()
                if np.any(weights[t]):
                    F, T = L.get_forces()
                    s += float(np.sum(weights[t][:, :3] * F) + np.sum(weights[t][:, 3:] * T))
        return s

    h = 1e-6
    tags = rec[0][:, 10]
    fd = []
    for (t, k, q, name) in [(160, 0, 0, "v_x of particle 0 at step 160"), (100, 5, 1, "v_y of particle 5 at step 100"),
                            (180, 10, 5, "omega_z of particle 10 at step 180"),
                            (199, 20, 0, "v_x of particle 20 at step 199")]:
        same = tags == tags[k]
        rp = rec.copy()
        rm = rec.copy()
        rp[t, same, 3 + q] += h
        rm[t, same, 3 + q] -= h
        d = (loss_of(rec_=rp) - loss_of(rec_=rm)) / (2 * h)
        fd.append({"parameter": name, "fd": d, "adjoint": float(o64["grad_vel"][t, k, q])})
    gp, gm = list(g), list(g)
    gp[0] += h
    gm[0] -= h
    fd.append({"parameter": "body force x", "fd": (loss_of(g_=tuple(gp)) - loss_of(g_=tuple(gm))) / (2 * h),
               "adjoint": float(o64["grad_body_force"][0])})
    fd.append({"parameter": "tau", "fd": (loss_of(tau_=tau + h) - loss_of(tau_=tau - h)) / (2 * h),
               "adjoint": float(o64["grad_tau"])})
    for e in fd:
        e["rel_err"] = abs(e["fd"] - e["adjoint"]) / max(abs(e["adjoint"]), 1e-300)

    def grads(o):
        return np.concatenate([o["grad_vel"].ravel(), o["grad_body_force"], [o["grad_tau"]]])

    return {
        "workload": f"periodic 128^3, tau {tau}, {nl} spheres r = 6 (+ images: {m}), body force {g[0]:g} in x, "
                    f"{steps} steps from rest, loss = sum of x-forces over the last 50 steps",
        "checkpoint_every": K, "loss": o64["loss"],
        "fp64": {"forward_ms": f64, "backward_ms": b64, "backward_over_forward": b64 / f64},
        "fp32": {"forward_ms": f32, "backward_ms": b32, "backward_over_forward": b32 / f32},
        "full_tape_fp64": {"forward_ms": ftape, "backward_ms": btape,
                           "max_rel_diff_vs_checkpointed": _rel(grads(o64), grads(otape))},
        "central_differences_fp64": {"h": h, "checks": fd, "max_rel_err": max(e["rel_err"] for e in fd)},
        "fp32_vs_fp64_grad_rel_err": {
            "velocities": _rel(o32["grad_vel"], o64["grad_vel"]),
            "body_force": _rel(o32["grad_body_force"], o64["grad_body_force"]),
            "tau": abs(o32["grad_tau"] - o64["grad_tau"]) / abs(o64["grad_tau"]),
            "loss": abs(o32["loss"] - o64["loss"]) / abs(o64["loss"]),
        },
    }


def precision(steps: int = 2000, seed: int = 2025, tau: float = 0.6, g=(1e-6, 0.0, 0.0), sample_every: int = 100,
              moving: bool = False) -> dict:
    """FP32 deviation form against the FP64 form on the same seeded inputs, both
    forms stepped in lockstep through the C ABI (a full coupling cycle per step).

    Default: a fixed bed -- the spheres at rest, the flow driven through them by
    the body force.  moving=True prescribes x += v, v ~ N(0, 0.01): at solid
    fraction 0.30 the reference's PSM collision then gains mass every step (its
    rest-population term, src/ibCompositeDynamics3D.hh:161,185, adds
    2 B (feq_0(j) - feq_0(rho uP)) per cell, which grows with |rho uP|^2 - |j|^2)
    until the run diverges, on the CPU restatement as on the GPU."""
    shape, p = W.polydisperse_512(seed)
    if not moving:
        p = W.Particles(p.x, np.zeros_like(p.v), np.zeros_like(p.w), p.r, p.tag)
    nl = p.n
    cap = 4 * nl
    L64 = lbdem.Lattice(*shape, 1.0 / tau, periodic=(1, 1, 1), precision=lbdem.PREC_FP64, body_force=g,
                        max_particles=cap, max_tag=nl + 1, max_radius=12.0)
    L32 = lbdem.Lattice(*shape, 1.0 / tau, periodic=(1, 1, 1), precision=lbdem.PREC_FP32_DEV, body_force=g,
                        max_particles=cap, max_tag=nl + 1, max_radius=12.0)
    q = p
    ferr, terr = [], []
    t0 = time.perf_counter()
    F32 = F64 = T32 = T64 = None
    for t in range(steps):
        gh = W.with_ghosts(q, shape)
        F64, T64 = L64.cycle(gh.x, gh.v, gh.w, gh.r, gh.tag)
        F32, T32 = L32.cycle(gh.x, gh.v, gh.w, gh.r, gh.tag)
        if (t + 1) % sample_every == 0:
            ferr.append(_rel(F32[:nl], F64[:nl]))
            terr.append(_rel(T32[:nl], T64[:nl]))
        if moving:
            q = W.advance(q, shape)
    secs = time.perf_counter() - t0
    u64 = L64.get_field(lbdem.FIELD_VELOCITY)
    u32 = L32.get_field(lbdem.FIELD_VELOCITY)
    du = u32 - u64
    per_particle = np.linalg.norm(F32[:nl] - F64[:nl], axis=1) / np.maximum(np.linalg.norm(F64[:nl], axis=1), 1e-300)
    out = {
        "workload": f"periodic 512x256x256, {nl} spheres r ~ U[4,10] (solid fraction 0.30), tau {tau}, "
                    f"body force {g[0]:g} in x, {steps} steps, "
                    + ("prescribed kinematics v ~ N(0, 0.01)" if moving else "fixed bed (spheres at rest)"),
        "velocity_field": {"rel_l2": float(np.linalg.norm(du) / np.linalg.norm(u64)),
                           "rel_linf": float(np.max(np.abs(du)) / np.max(np.abs(u64)))},
        "force": {"rel_err_final": ferr[-1] if ferr else None, "rel_err_max_over_samples": max(ferr) if ferr else None,
                  "per_particle_median": float(np.median(per_particle)),
                  "per_particle_p99": float(np.percentile(per_particle, 99))},
        "torque": {"rel_err_final": terr[-1] if terr else None, "rel_err_max_over_samples": max(terr) if terr else None},
        "mass_fp64": L64.mass(), "mass_fp32": L32.mass(),
        "wall_seconds_both_forms": secs,
    }
    L64.close()
    L32.close()
    return out


def window(steps: int = 6, K: int = 3, fp64: bool = False, seed: int = 2027) -> dict:
    """One adjoint window of the 128^3 case (x-force loss over every step), timed."""
    shape = (128, 128, 128)
    p = W.suspension(shape, n_max=64, radius=6.0, seed=seed)
    gh = W.with_ghosts(p, shape)
    rec = np.repeat(lbdem.pack_records(gh.x, gh.v, gh.w, gh.r, gh.tag)[None], steps, axis=0)
    w = np.zeros((steps, gh.n, 6))
    w[:, :p.n, 0] = 1.0
    prec = lbdem.PREC_FP64 if fp64 else lbdem.PREC_FP32_DEV
    with lbdem.Lattice(*shape, 1 / 0.6, precision=prec, body_force=(1e-6, 0, 0), max_particles=gh.n,
                       max_tag=p.n + 1, max_radius=8.0) as L:
        o = L.adjoint_window(rec, w, K)
        fwd, bwd = L.adjoint_timing()
    return {"steps": steps, "checkpoint_every": K, "form": "fp64" if fp64 else "fp32", "loss": o["loss"],
            "forward_ms": fwd, "backward_ms": bwd}


def channels(steps: int = 6, flow_axis: int = 2, domains: int = 512) -> dict:
    """The batched channels of workloads.channels stepped for a few coupling cycles
    (the first `domains` of the seeded sequence: profiling runs take fewer)."""
    ch = W.channels(n_domains=domains, flow_axis=flow_axis)
    doms = [d for d, _ in ch]
    g = [W.with_ghosts(p, d["shape"], d["periodic"]) for d, p in ch]
    counts = np.array([x.n for x in g], dtype=np.int32)
    rec = np.concatenate([lbdem.pack_records(x.x, x.v, x.w, x.r, x.tag) for x in g])
    with lbdem.Batch(doms, precision=lbdem.PREC_FP32_DEV, max_tag=64, max_radius=8.0, autotune=False) as B:
        t0 = time.perf_counter()
        for _ in range(steps):
            B.cycle(counts, rec)
        secs = time.perf_counter() - t0
        cells = B.cells()
    return {"domains": len(doms), "cells": cells, "steps": steps, "flow_axis": "xyz"[flow_axis],
            "mlups": cells * steps / secs / 1e6}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("which", choices=["adjoint", "precision", "window", "channels"])
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--checkpoint", type=int, default=3)
    ap.add_argument("--fp64", action="store_true")
    ap.add_argument("--flow-axis", type=int, default=2, choices=[0, 2])
    ap.add_argument("--domains", type=int, default=512)
    a = ap.parse_args()
    if a.which == "adjoint":
        r = adjoint(steps=a.steps or 200)
    elif a.which == "precision":
        r = precision(steps=a.steps or 2000)
    elif a.which == "window":
        r = window(steps=a.steps or 6, K=a.checkpoint, fp64=a.fp64)
    else:
        r = channels(steps=a.steps or 6, flow_axis=a.flow_axis, domains=a.domains)
    print(json.dumps(r))


if __name__ == "__main__":
    main()
