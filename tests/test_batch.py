"""Batched independent domains (lbdem_batch_*): every domain of a batch behaves as
a single lattice handle with the same configuration fed the same calls.

Domains of uneven size, periodicity and particle count (one without particles),
two of them pressure-driven channels (the Zhang rescale of
src/periodicPressureFunctionals3D.hh:121-159 as used in
examples/showcaseRectChannel/showcaseRectChannel.cpp:253-273).
"""
import numpy as np
import pytest

from helpers import rel_err, small_suspension

pytestmark = pytest.mark.gpu

TAU = 0.6


def channel_drop(shape, rho_in=1.0, rho_out=0.998):
    nx, ny, nz = shape
    return {"dimension": 0, "inlet": [0, 0, 1, ny - 2, 1, nz - 2], "outlet": [nx - 1, nx - 1, 1, ny - 2, 1, nz - 2],
            "rho_in": rho_in, "rho_out": rho_out}


def domains(force=False):
    d = [
        {"shape": (20, 14, 18), "periodic": (1, 1, 1), "omega": 1 / TAU, "max_particles": 16, "n": 4, "r": (2.0, 3.5)},
        {"shape": (33, 12, 16), "periodic": (1, 0, 0), "omega": 1 / 0.55, "max_particles": 16, "n": 3,
         "r": (2.0, 3.0), "drop": channel_drop((33, 12, 16))},
        {"shape": (9, 11, 7), "periodic": (0, 0, 0), "omega": 1 / TAU, "max_particles": 4, "n": 1, "r": (1.5, 2.0)},
        {"shape": (16, 16, 40), "periodic": (0, 0, 1), "omega": 1 / 0.7, "max_particles": 0, "n": 0, "r": (1, 1)},
        {"shape": (24, 10, 25), "periodic": (1, 0, 0), "omega": 1 / TAU, "max_particles": 8, "n": 2,
         "r": (2.0, 3.0), "drop": channel_drop((24, 10, 25), 1.001, 0.999)},
    ]
    if force:
        d[0]["body_force"] = (1e-5, 0.0, 2e-6)
    return d


def particles(doms, seed):
    out = []
    for k, d in enumerate(doms):
        if d["n"] == 0:
            out.append(None)
            continue
        out.append(small_suspension(d["shape"], d["n"], d["r"][0], d["r"][1], seed=seed + k, periodic=d["periodic"],
                                    overlap=True))
    return out


def advance(doms, parts):
    for d, p in zip(doms, parts):
        if p is None:
            continue
        p.x[:] = p.x + p.v
        for a in range(3):
            if d["periodic"][a]:
                p.x[:, a] %= d["shape"][a]


def packed(lb, parts):
    counts = np.array([0 if p is None else len(p.r) for p in parts], dtype=np.int32)
    recs = [lb.pack_records(p.x, p.v, p.w, p.r, p.tag) for p in parts if p is not None]
    rec = np.concatenate(recs) if recs else np.zeros((0, 12))
    return counts, rec


def init_state(target, d, k, batch):
    if "drop" in d:
        args = (1, 1.0, 0.998, 0.01, (d["shape"][0] - 1, d["shape"][1], d["shape"][2]), 0)
        if batch:
            target.init_profile(k, *args)
        else:
            target.init_profile(*args)


def singles(lb, doms, prec):
    out = []
    for k, d in enumerate(doms):
        L = lb.Lattice(*d["shape"], d["omega"], periodic=d["periodic"], precision=prec,
                       body_force=d.get("body_force", (0, 0, 0)), max_particles=max(d["max_particles"], 1),
                       max_tag=64, max_radius=8)
        init_state(L, d, k, False)
        if "drop" in d:
            dr = d["drop"]
            L.set_pressure_drop(dr["dimension"], dr["inlet"], dr["outlet"], dr["rho_in"], dr["rho_out"])
        out.append(L)
    return out


def make_batch(lb, doms, prec, use_graph=True, autotune=False):
    B = lb.Batch(doms, precision=prec, max_tag=64, max_radius=8, use_graph=use_graph, autotune=autotune)
    for k, d in enumerate(doms):
        init_state(B, d, k, True)
    return B


def run_pair(gpu, prec, steps, seed=5, force=False):
    doms = domains(force)
    parts = particles(doms, seed)
    B = make_batch(gpu, doms, prec)
    Ls = singles(gpu, doms, prec)
    FB = FS = None
    for it in range(steps):
        counts, rec = packed(gpu, parts)
        FB, TB = B.cycle(counts, rec, init_vel=(it == 0))
        FS, TS = [], []
        for L, p in zip(Ls, parts):
            if p is None:
                L.set_particles(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0),
                                np.zeros(0, dtype=np.int32))
                L.collide_and_stream()
                continue
            L.set_particles(p.x, p.v, p.w, p.r, p.tag, init_vel=(it == 0))
            L.collide_and_stream()
            F, T = L.get_forces()
            FS.append(F)
            TS.append(T)
        FS = np.concatenate(FS)
        advance(doms, parts)
    return B, Ls, FB, FS, doms


@pytest.mark.parametrize("prec", [0, 1])
def test_batch_equals_single_handles(gpu, prec):
    B, Ls, FB, FS, doms = run_pair(gpu, prec, 9)
    with B:
        assert B.step_count() == 9
        for k, L in enumerate(Ls):
            with L:
                assert np.array_equal(B.get_populations(k), L.get_populations()), f"domain {k}"
                for fld in (gpu.FIELD_SUBCELL_COUNT, gpu.FIELD_PARTICLE_ID):
                    assert np.array_equal(B.get_field(k, fld), L.get_field(fld)), f"domain {k}"
        assert rel_err(FB, FS) <= (1e-12 if prec == 0 else 1e-6)


def test_batch_with_body_force_matches_oracle(gpu, oracle):
    doms = domains(force=True)
    parts = particles(doms, 9)
    B = make_batch(gpu, doms, 0)
    ols = []
    for k, d in enumerate(doms):
        o = oracle.OracleLattice(*d["shape"], d["omega"], periodic=d["periodic"],
                                 body_force=d.get("body_force", (0, 0, 0)), threads=4)
        if "drop" in d:
            o.init_profile(1, 1.0, 0.998, 0.01, (d["shape"][0] - 1, d["shape"][1], d["shape"][2]), 0)
        ols.append(o)
    for it in range(6):
        counts, rec = packed(gpu, parts)
        FB, _ = B.cycle(counts, rec, init_vel=(it == 0))
        FO = []
        for d, o, p in zip(doms, ols, parts):
            if p is None:
                o.set_particles(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0),
                                np.zeros(0, dtype=np.int32))
            else:
                o.set_particles(p.x, p.v, p.w, p.r, p.tag, init_vel=(it == 0))
            if "drop" in d:
                dr = d["drop"]
                a_in, a_out = o.average_density(dr["inlet"]), o.average_density(dr["outlet"])
            o.collide_and_stream()
            if "drop" in d:
                o.zhang_rescale(dr["inlet"], 0, 1, dr["rho_in"], a_out)
                o.zhang_rescale(dr["outlet"], 0, -1, dr["rho_out"], a_in)
            if p is not None:
                FO.append(o.get_forces()[0])
        advance(doms, parts)
    with B:
        for k, o in enumerate(ols):
            assert rel_err(B.get_populations(k), o.get_populations()) <= 1e-12, f"domain {k}"
        assert rel_err(FB, np.concatenate(FO)) <= 1e-10


def test_graph_replay_equals_eager(gpu):
    doms = domains()
    outs = []
    for use_graph in (True, False):
        parts = particles(doms, 21)
        B = make_batch(gpu, doms, 1, use_graph=use_graph)
        for it in range(7):
            counts, rec = packed(gpu, parts)
            F, _ = B.cycle(counts, rec, init_vel=(it == 0))
            advance(doms, parts)
        outs.append((B, F))
    (Bg, Fg), (Be, Fe) = outs
    with Bg, Be:
        for k in range(len(doms)):
            assert np.array_equal(Bg.get_populations(k), Be.get_populations(k))
        assert rel_err(Fg, Fe) <= 1e-6


def test_launches_per_step_and_autotune(gpu):
    doms = domains()
    parts = particles(doms, 3)
    with make_batch(gpu, doms, 1, autotune=True) as B:
        counts, rec = packed(gpu, parts)
        B.cycle(counts, rec)
        B.cycle(counts, rec)                  # autotuned before this step
        bps, ms = B.tuning()
        assert 0 <= bps <= 3 and ms > 0
        n0 = B.launch_count()
        B.cycle(counts, rec)
        # prepare + bin, voxelize, collide-stream, one plane launch for both channels
        assert B.launch_count() - n0 == 4
        B.set_tuning(2)
        assert B.tuning()[0] == 2
        B.cycle(counts, rec)
        assert B.cells() == sum(int(np.prod(d["shape"])) for d in doms)


def test_channel_orientations_mirror_each_other(gpu):
    """The same pressure-driven channels stored with the flow along x and along z
    (x <-> z swapped: a reflection) give mirror-image results: F_z = P F_x,
    T_z = -P T_x, rho_z = rho_x transposed.  Checks the batch path's wall,
    periodic-wrap and plane-rescale handling along either axis."""
    import workloads as W
    out = []
    for axis in (0, 2):
        ch = W.channels(n_domains=4, seed=77, flow_axis=axis, rho_out=0.995)
        doms = [d for d, _ in ch]
        g = [W.with_ghosts(p, d["shape"], d["periodic"]) for d, p in ch]
        counts = np.array([x.n for x in g], dtype=np.int32)
        rec = np.concatenate([gpu.pack_records(x.x, x.v, x.w, x.r, x.tag) for x in g])
        with gpu.Batch(doms, precision=0, max_tag=64, max_radius=8) as B:
            for it in range(6):
                F, T = B.cycle(counts, rec, init_vel=(it == 0))
            rho = [B.get_field(k, gpu.FIELD_DENSITY) for k in range(len(doms))]
        out.append((F, T, rho))
    (Fx, Tx, rx), (Fz, Tz, rz) = out
    perm = [2, 1, 0]
    assert rel_err(Fz, Fx[:, perm]) <= 1e-10
    assert rel_err(Tz, -Tx[:, perm]) <= 1e-10
    for a, b in zip(rx, rz):
        assert rel_err(b, a.transpose(2, 1, 0)) <= 1e-13


def test_batch_rejects_bad_input(gpu):
    doms = domains()
    with make_batch(gpu, doms, 1) as B:
        counts = np.array([17, 0, 0, 0, 0], dtype=np.int32)         # above domain 0's capacity
        with pytest.raises(gpu.LbdemError) as e:
            B.set_particles(counts, np.zeros((17, 12)))
        assert e.value.status == 4
        buf = np.zeros(64)
        assert B.lib.lbdem_batch_get_field(B.h, 9, gpu.FIELD_DENSITY, buf.ctypes.data_as(gpu._P)) == 1
    bad = domains()
    bad[1]["drop"]["outlet"] = bad[1]["drop"]["inlet"]               # overlapping boxes
    with pytest.raises(gpu.LbdemError):
        gpu.Batch(bad, precision=1, max_tag=64)
