"""Adjoint of collide-stream + PSM momentum exchange (lbdem_adjoint_window).

The loss is sum_t sum_p weights[t][p] . (F_p(t), T_p(t)) over a window with the
particles' positions (hence solid fraction and owners) fixed and their linear
and angular velocities changing per step.  References:
* a float64 PyTorch model of the same forward map, differentiated by autograd
  over its full tape (tests/torch_psm.py), itself pinned to the oracle here;
* central finite differences (h = 1e-6) of the GPU's own FP64 forward;
* the GPU adjoint with a checkpoint every step (a full tape).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from helpers import rel_err, small_suspension  # noqa: E402
from torch_psm import TorchPSM  # noqa: E402

TAU = 0.6


def case(shape, periodic, n, seed, nsteps, g=(1e-5, -2e-6, 3e-6)):
    import workloads as W
    rng = np.random.default_rng(seed)
    sp = small_suspension(shape, n, 2.5, 3.5, seed=seed, periodic=periodic)
    gh = W.with_ghosts(sp, shape, periodic)
    m = len(gh.r)
    base = np.zeros((m, 12))
    base[:, 0:3] = gh.x
    base[:, 9] = gh.r
    base[:, 10] = gh.tag
    rec = np.repeat(base[None], nsteps, axis=0)
    # per-step velocities of every tag (ghost images copy their owner's)
    nl = len(sp.r)
    vloc = rng.normal(0, 0.01, (nsteps, nl, 3))
    wloc = rng.normal(0, 1e-3, (nsteps, nl, 3))
    owner = np.array([int(t) - 1 for t in gh.tag])
    rec[:, :, 3:6] = vloc[:, owner]
    rec[:, :, 6:9] = wloc[:, owner]
    weights = np.zeros((nsteps, m, 6))
    lo = nsteps // 3
    weights[lo:, :nl] = rng.normal(0, 1.0, (nsteps - lo, nl, 6))
    weights[lo:, :nl, 0] += 1.0                       # the x-force sum of the window
    return {"shape": shape, "periodic": periodic, "rec": rec, "weights": weights, "g": g, "nl": nl}


def initial_state(oracle, c, warm=4):
    """A non-trivial starting state: a few oracle steps from rest with the window's particles."""
    ol = oracle.OracleLattice(*c["shape"], 1 / TAU, periodic=c["periodic"], body_force=c["g"], threads=4)
    r0 = c["rec"][0]
    for _ in range(warm):
        ol.set_particles(r0[:, 0:3], r0[:, 3:6], r0[:, 6:9], r0[:, 9], r0[:, 10].astype(np.int32))
        ol.collide_and_stream()
    return ol


def torch_model(ol, c):
    st = ol.state()
    tags = c["rec"][0][:, 10].astype(np.int64)
    first = {}
    for k, t in enumerate(tags):
        first.setdefault(int(t), k)
    slot = np.where(st["id"] > 0, np.vectorize(lambda t: first.get(int(t), -1))(st["id"]), -1)
    return TorchPSM(c["shape"], c["periodic"], st["n"].astype(np.float64), slot, c["rec"][0][:, 0:3])


def torch_grads(model, f0, c):
    f = torch.tensor(f0.astype(np.float64), requires_grad=True)
    vel = torch.tensor(np.concatenate([c["rec"][:, :, 3:6], c["rec"][:, :, 6:9]], axis=2), requires_grad=True)
    tau = torch.tensor(TAU, dtype=torch.float64, requires_grad=True)
    g = torch.tensor(c["g"], dtype=torch.float64, requires_grad=True)
    loss, _ = model.window(f, vel, torch.tensor(c["weights"]), tau, g)
    loss.backward()
    return {"loss": float(loss.detach()), "grad_vel": vel.grad.numpy(), "grad_body_force": g.grad.numpy(),
            "grad_tau": float(tau.grad), "grad_f0": f.grad.numpy()}


# ---- CPU: the torch model reproduces the oracle's forward ---------------------------------------

@pytest.mark.parametrize("periodic", [(1, 1, 1), (1, 0, 0)])
def test_torch_model_matches_oracle(oracle, periodic):
    c = case((14, 12, 16), periodic, 3, 4, 6)
    ol = initial_state(oracle, c)
    model = torch_model(ol, c)
    f = torch.tensor(ol.get_populations().astype(np.float64)).reshape(19, -1)
    for t in range(6):
        r = c["rec"][t]
        ol.set_particles(r[:, 0:3], r[:, 3:6], r[:, 6:9], r[:, 9], r[:, 10].astype(np.int32))
        ol.collide_and_stream()
        Fo, To = ol.get_forces()
        vel = torch.tensor(np.concatenate([r[:, 3:6], r[:, 6:9]], axis=1))
        f, FT = model.step(f, vel, torch.tensor(TAU, dtype=torch.float64), torch.tensor(c["g"], dtype=torch.float64))
        assert rel_err(f.detach().numpy(), ol.get_populations().reshape(19, -1)) <= 1e-13
        assert rel_err(FT.detach().numpy()[:, :3], Fo) <= 1e-11
        assert rel_err(FT.detach().numpy()[:, 3:], To) <= 1e-11


# ---- GPU --------------------------------------------------------------------------------------

def gpu_window(lb, oracle, c, K, prec=0, want_f0=True, ol=None):
    ol = ol or initial_state(oracle, c)
    L = lb.Lattice(*c["shape"], 1 / TAU, periodic=c["periodic"], precision=prec, body_force=c["g"],
                   max_particles=64, max_tag=64, max_radius=8)
    L.set_populations(ol.get_populations())
    out = L.adjoint_window(c["rec"], c["weights"], K, want_f0=want_f0)
    return L, out, ol


@pytest.mark.gpu
@pytest.mark.parametrize("periodic", [(1, 1, 1), (1, 0, 0), (0, 0, 0)])
def test_adjoint_matches_torch_full_tape(gpu, oracle, periodic):
    c = case((16, 14, 18), periodic, 3, 11, 14)
    L, g_out, ol = gpu_window(gpu, oracle, c, K=4)
    ref = torch_grads(torch_model(ol, c), ol.get_populations(), c)
    with L:
        assert abs(g_out["loss"] - ref["loss"]) <= 1e-12 * abs(ref["loss"])
        assert rel_err(g_out["grad_vel"], ref["grad_vel"]) <= 1e-10
        assert rel_err(g_out["grad_body_force"], ref["grad_body_force"]) <= 1e-10
        assert abs(g_out["grad_tau"] - ref["grad_tau"]) <= 1e-10 * abs(ref["grad_tau"])
        assert rel_err(g_out["grad_f0"].reshape(19, -1), ref["grad_f0"].reshape(19, -1)) <= 1e-10


@pytest.mark.gpu
def test_checkpoint_interval_does_not_change_the_gradient(gpu, oracle):
    c = case((16, 14, 18), (1, 1, 1), 3, 12, 13)
    outs = []
    for K in (1, 3, 13):
        L, o, _ = gpu_window(gpu, oracle, c, K)
        L.close()
        outs.append(o)
    for o in outs[1:]:
        assert np.array_equal(o["grad_f0"], outs[0]["grad_f0"])      # deterministic tape and reverse sweep
        assert rel_err(o["grad_vel"], outs[0]["grad_vel"]) <= 1e-13
        assert rel_err(o["grad_body_force"], outs[0]["grad_body_force"]) <= 1e-13
        assert abs(o["grad_tau"] - outs[0]["grad_tau"]) <= 1e-13 * abs(outs[0]["grad_tau"])


@pytest.mark.gpu
def test_adjoint_against_central_differences(gpu, oracle):
    c = case((16, 14, 18), (1, 0, 1), 3, 13, 12)
    L, o, ol = gpu_window(gpu, oracle, c, K=5)
    L.close()
    f0 = ol.get_populations()
    h = 1e-6

    def loss_of(rec=None, g=None, tau=None):
        cc = dict(c)
        if rec is not None:
            cc["rec"] = rec
        if g is not None:
            cc["g"] = g
        t = TAU if tau is None else tau
        M = gpu.Lattice(*cc["shape"], 1 / t, periodic=cc["periodic"], body_force=cc["g"], max_particles=64,
                        max_tag=64, max_radius=8)
        M.set_populations(f0)
        val = M.adjoint_window(cc["rec"], cc["weights"], len(cc["rec"]))["loss"]
        M.close()
        return val

    checks = []
    tags = c["rec"][0][:, 10]
    for (t, p, q) in [(2, 0, 0), (7, 1, 2), (9, 2, 4), (5, 0, 3)]:
        same = tags == tags[p]
        rp = c["rec"].copy(); rm = c["rec"].copy()
        col = 3 + q
        rp[t, same, col] += h
        rm[t, same, col] -= h
        checks.append(((loss_of(rec=rp) - loss_of(rec=rm)) / (2 * h), o["grad_vel"][t, p, q]))
    for q in range(3):
        gp = list(c["g"]); gm = list(c["g"])
        gp[q] += h; gm[q] -= h
        checks.append(((loss_of(g=tuple(gp)) - loss_of(g=tuple(gm))) / (2 * h), o["grad_body_force"][q]))
    checks.append(((loss_of(tau=TAU + h) - loss_of(tau=TAU - h)) / (2 * h), o["grad_tau"]))
    for fd, ad in checks:
        assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-3 * abs(o["loss"])), (fd, ad)


@pytest.mark.gpu
def test_fp32_adjoint_close_to_fp64(gpu, oracle):
    c = case((16, 14, 18), (1, 1, 1), 3, 14, 12)
    L64, o64, ol = gpu_window(gpu, oracle, c, K=4)
    L32, o32, _ = gpu_window(gpu, oracle, c, K=4, prec=1, ol=ol)
    with L64, L32:
        assert rel_err(o32["grad_vel"], o64["grad_vel"]) <= 2e-3
        assert rel_err(o32["grad_body_force"], o64["grad_body_force"]) <= 2e-3
        assert abs(o32["grad_tau"] - o64["grad_tau"]) <= 2e-3 * abs(o64["grad_tau"])


@pytest.mark.gpu
def test_window_leaves_the_forward_state(gpu, oracle):
    c = case((16, 14, 18), (1, 1, 1), 3, 15, 9)
    L, o, ol = gpu_window(gpu, oracle, c, K=4, want_f0=False)
    M = gpu.Lattice(*c["shape"], 1 / TAU, periodic=c["periodic"], body_force=c["g"], max_particles=64, max_tag=64,
                    max_radius=8)
    M.set_populations(ol.get_populations())
    for t in range(9):
        r = c["rec"][t]
        M.set_particles(r[:, 0:3], r[:, 3:6], r[:, 6:9], r[:, 9], r[:, 10].astype(np.int32))
        M.collide_and_stream()
    with L, M:
        assert L.step_count() == M.step_count()
        assert np.array_equal(L.get_populations(), M.get_populations())
        FL, _ = L.get_forces()
        FM, _ = M.get_forces()
        assert rel_err(FL, FM) <= 1e-13
        fwd, bwd = L.adjoint_timing()
        assert fwd > 0 and bwd > 0


@pytest.mark.gpu
def test_adjoint_rejects_moving_particles_and_pressure_drop(gpu, oracle):
    c = case((16, 14, 18), (1, 1, 1), 2, 16, 4)
    with gpu.Lattice(*c["shape"], 1 / TAU, max_particles=64, max_tag=64, max_radius=8) as L:
        rec = c["rec"].copy()
        rec[2, 0, 0] += 0.5
        with pytest.raises(gpu.LbdemError) as e:
            L.adjoint_window(rec, c["weights"], 2)
        assert e.value.status == 1
    with gpu.Lattice(*c["shape"], 1 / TAU, periodic=(1, 0, 0), max_particles=64, max_tag=64, max_radius=8) as L:
        L.set_pressure_drop(0, [0, 0, 1, 12, 1, 16], [15, 15, 1, 12, 1, 16], 1.0, 0.999)
        with pytest.raises(gpu.LbdemError):
            L.adjoint_window(c["rec"], c["weights"], 2)


@pytest.mark.gpu
def test_fp32_checkpoint_interval_on_aligned_rows(gpu, oracle):
    """FP32 form on rows of a multiple of 4 cells (the staged, paired collide path):
    the backward pass recomputes each segment out of place into the tape, so the
    adjoint of the initial populations is bit-identical for any checkpoint
    interval only if that recomputation reproduces the forward states exactly
    (the per-particle sums are double atomics, whose order varies)."""
    c = case((16, 14, 20), (1, 1, 1), 3, 17, 10)
    outs = []
    for K in (1, 3, 10):
        L, o, _ = gpu_window(gpu, oracle, c, K, prec=1)
        L.close()
        outs.append(o)
    for o in outs[1:]:
        d0 = np.abs(o["grad_f0"] - outs[0]["grad_f0"]).max() / np.abs(outs[0]["grad_f0"]).max()
        assert np.array_equal(o["grad_f0"], outs[0]["grad_f0"]), f"grad_f0 differs by {d0:.3e}"
        assert rel_err(o["grad_vel"], outs[0]["grad_vel"]) <= 1e-12
        assert rel_err(o["grad_body_force"], outs[0]["grad_body_force"]) <= 1e-12
        assert abs(o["grad_tau"] - outs[0]["grad_tau"]) <= 1e-12 * abs(outs[0]["grad_tau"])


# ---- GPU adjoint as a torch.autograd.Function (check harness) ------------------------------------

class GpuPSMWindow(torch.autograd.Function):
    """The loss of a window of GPU PSM steps, L = sum_t sum_p w[t][p] . (F_p(t), T_p(t)),
    as a differentiable torch function of the initial populations f0, the per-step
    particle velocities and angular velocities vel [nsteps][n][6], the body force g
    and tau.  forward() runs lbdem_adjoint_window, which returns the loss together
    with every gradient (forward pass, checkpointed recomputation, hand-written
    reverse steps); backward() scales them by the incoming gradient.  Positions,
    radii and tags (rec_base) and the weights are constants."""

    @staticmethod
    def forward(ctx, f0, vel, g, tau, lb, shape, periodic, rec_base, weights, K, prec):
        rec = rec_base.copy()
        rec[:, :, 3:9] = vel.detach().cpu().numpy()
        with lb.Lattice(*shape, 1.0 / float(tau), periodic=periodic, precision=prec,
                        body_force=tuple(float(x) for x in g.detach().cpu()), max_particles=64, max_tag=64,
                        max_radius=8) as L:
            L.set_populations(f0.detach().cpu().numpy())
            out = L.adjoint_window(rec, weights, K, want_f0=True)
        ctx.grads = (torch.from_numpy(np.ascontiguousarray(out["grad_f0"], dtype=np.float64)).reshape(f0.shape),
                     torch.from_numpy(out["grad_vel"].copy()), torch.from_numpy(out["grad_body_force"].copy()),
                     torch.tensor(out["grad_tau"], dtype=torch.float64))
        return torch.tensor(out["loss"], dtype=torch.float64)

    @staticmethod
    def backward(ctx, gout):
        gf0, gvel, gg, gtau = ctx.grads
        return gout * gf0, gout * gvel, gout * gg, gout * gtau, None, None, None, None, None, None, None


@pytest.mark.gpu
def test_autograd_function_backward_matches_full_tape(gpu, oracle):
    """loss.backward() through GpuPSMWindow, inside a larger graph (the velocities
    are a scaled copy of a base table, tau and g derived tensors), against the
    float64 torch model's full tape on the same graph: loss 1e-12, every leaf
    gradient 1e-10."""
    c = case((16, 14, 18), (1, 0, 0), 3, 11, 12)
    ol = initial_state(oracle, c)
    f0_np = ol.get_populations().astype(np.float64)
    vel_np = np.concatenate([c["rec"][:, :, 3:6], c["rec"][:, :, 6:9]], axis=2)
    model = torch_model(ol, c)
    grads = []
    for use_gpu in (True, False):
        f0 = torch.tensor(f0_np, requires_grad=True)
        base = torch.tensor(vel_np, requires_grad=True)
        scale = torch.tensor(1.3, dtype=torch.float64, requires_grad=True)
        lt = torch.tensor(np.log(TAU), dtype=torch.float64, requires_grad=True)
        g = torch.tensor(c["g"], dtype=torch.float64, requires_grad=True)
        vel, tau = scale * base, torch.exp(lt)
        if use_gpu:
            loss = GpuPSMWindow.apply(f0, vel, g, tau, gpu, c["shape"], c["periodic"], c["rec"], c["weights"], 4, 0)
        else:
            loss, _ = model.window(f0.reshape(19, -1), vel, torch.tensor(c["weights"]), tau, g)
        (2.0 * loss).backward()
        grads.append({"loss": float(loss.detach()), "f0": f0.grad.numpy().reshape(19, -1), "base": base.grad.numpy(),
                      "scale": float(scale.grad), "lt": float(lt.grad), "g": g.grad.numpy()})
    got, ref = grads
    assert abs(got["loss"] - ref["loss"]) <= 1e-12 * abs(ref["loss"])
    for k in ("f0", "base", "g"):
        assert rel_err(got[k], ref[k]) <= 1e-10, k
    for k in ("scale", "lt"):
        assert abs(got[k] - ref[k]) <= 1e-10 * abs(ref[k]), k
    assert abs(ref["scale"]) > 0 and abs(ref["lt"]) > 0
