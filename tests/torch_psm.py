"""A float64 PyTorch model of the PSM lattice step, for the adjoint tests.

Test infrastructure: an independent vectorised restatement of the same forward
map as the oracle (src/ibCompositeDynamics3D.hh:130-203 written statement by
statement: BGK with Guo forcing, the B-weighted solid collision with the
bb / bbOpp pairs and the force loop, push streaming with half-way bounce-back),
over a fixed voxel state, differentiated by autograd.  Its full tape is the
reference adjoint the GPU's checkpointed adjoint is compared with.
"""
from __future__ import annotations

import numpy as np
import torch

CX = [0, -1, 0, 0, -1, -1, -1, -1, 0, 0, 1, 0, 0, 1, 1, 1, 1, 0, 0]
CY = [0, 0, -1, 0, -1, 1, 0, 0, -1, -1, 0, 1, 0, 1, -1, 0, 0, 1, 1]
CZ = [0, 0, 0, -1, 0, 0, -1, 1, -1, 1, 0, 0, 1, 0, 0, 1, -1, 1, -1]
WT = [1 / 3] + [1 / 18] * 3 + [1 / 36] * 6 + [1 / 18] * 3 + [1 / 36] * 6


def opp(i: int) -> int:
    return 0 if i == 0 else (i + 9 if i <= 9 else i - 9)


class TorchPSM:
    """Fixed geometry: shape, periodicity, per-cell sub-cell count and owner slot
    (-1: fluid), particle centres.  The arm d of a cell is the minimum image of
    cell - centre as in the force sum (src/ibProcessors3D.hh:230-243)."""

    def __init__(self, shape, periodic, nsub: np.ndarray, slot: np.ndarray, centres: np.ndarray):
        self.shape = tuple(int(v) for v in shape)
        nx, ny, nz = self.shape
        self.N = nx * ny * nz
        dt = torch.float64
        self.C = torch.tensor([CX, CY, CZ], dtype=dt).T            # [19, 3]
        self.W = torch.tensor(WT, dtype=dt)
        self.nsub = torch.tensor(nsub.reshape(-1).astype(np.float64))
        self.slot = torch.tensor(slot.reshape(-1).astype(np.int64))
        X, Y, Z = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
        pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()]).astype(np.float64)     # [3, N]
        d = np.zeros((3, self.N))
        s = slot.reshape(-1)
        ext = (nx, ny, nz)
        for q in range(3):
            dq = pos[q] - centres[np.maximum(s, 0), q]
            h = ext[q] // 2
            dq = np.where(dq > h, dq - ext[q], np.where(dq < -h, dq + ext[q], dq))
            d[q] = np.where(s >= 0, dq, 0.0)
        self.d = torch.tensor(d)
        # streaming: f_next[i][x] = out[i][x - c_i], or out[opp i][x] when x - c_i is beyond a wall
        idx = np.zeros((19, self.N), dtype=np.int64)
        for i in range(19):
            src = [pos[0] - CX[i], pos[1] - CY[i], pos[2] - CZ[i]]
            inside = np.ones(self.N, bool)
            for q in range(3):
                if periodic[q]:
                    src[q] = np.mod(src[q], ext[q])
                else:
                    inside &= (src[q] >= 0) & (src[q] < ext[q])
            cell_src = ((src[0] * ny + src[1]) * nz + src[2]).astype(np.int64)
            own = np.arange(self.N)
            idx[i] = np.where(inside, i * self.N + cell_src, opp(i) * self.N + own)
        self.idx = torch.tensor(idx)

    def feq(self, rb, r, J):
        cJ = self.C @ J                                              # [19, N]
        Jsq = (J * J).sum(0)
        return self.W[:, None] * (rb + 3 * cJ + r * (4.5 * cJ * cJ - 1.5 * Jsq))

    def step(self, f, vel, tau, g):
        """One collide-stream; vel: [nslot, 6] (v, omega) of this step.  Returns the
        streamed populations and the per-particle force and torque [nslot, 6]."""
        C, W = self.C, self.W
        omega = 1.0 / tau
        rb = f.sum(0)
        j = C.T @ f
        rho = 1 + rb
        r = 1 / rho
        J = j + 0.5 * rho * g[:, None]
        u = J * r
        pre = (1 - 0.5 * omega) * rho
        cu = C @ u
        cg = (C @ g)[:, None]
        ug = (u * g[:, None]).sum(0)
        src = W[:, None] * pre * (3 * (cg - ug) + 9 * cu * cg)
        fs = f * (1 - omega) + omega * self.feq(rb, r, J) + src
        full = (self.nsub == 125)[None, :]
        fs = torch.where(full, f, fs)
        # particle surface velocity of the owner: v + w x d
        s = torch.clamp(self.slot, min=0)
        v = vel[s, :3].T
        w = vel[s, 3:].T
        d = self.d
        uP = v + torch.stack([w[1] * d[2] - w[2] * d[1], -w[0] * d[2] + w[2] * d[0], w[0] * d[1] - w[1] * d[0]])
        uP = torch.where((self.slot >= 0)[None, :], uP, torch.zeros_like(uP))
        rbs = fs.sum(0)
        js = C.T @ fs
        rhos = 1 + rbs
        rs = 1 / rhos
        fEq = self.feq(rbs, rs, js)
        fEqS = self.feq(rbs, rs, uP * rhos)
        sf = self.nsub / 125.0
        ooo = tau - 0.5
        B = sf * ooo / ((1 - sf) + ooo)
        outs = [None] * 19
        outs[0] = f[0] + (1 - B) * (fs[0] - f[0]) + B * (fEq[0] - fEqS[0])
        F = torch.zeros((3, self.N), dtype=f.dtype)
        for i in range(1, 10):
            o = i + 9
            bb = B * ((f[o] - fEq[o]) - (f[i] - fEqS[i]))
            bbo = B * ((f[i] - fEq[i]) - (f[o] - fEqS[o]))
            outs[i] = f[i] + (1 - B) * (fs[i] - f[i]) + bb
            outs[o] = f[o] + (1 - B) * (fs[o] - f[o]) + bbo
            F = F - C[i][:, None] * (bb - bbo)
        out = torch.stack(outs)
        solid = (self.nsub > 0)[None, :]
        out = torch.where(solid, out, fs)
        F = torch.where(solid, F, torch.zeros_like(F))
        Tq = torch.stack([d[1] * F[2] - d[2] * F[1], d[2] * F[0] - d[0] * F[2], d[0] * F[1] - d[1] * F[0]])
        FT = torch.zeros((vel.shape[0], 6), dtype=f.dtype)
        m = self.slot >= 0
        FT = FT.index_add(0, self.slot[m], torch.cat([F, Tq])[:, m].T)
        nxt = out.reshape(-1)[self.idx]
        return nxt, FT

    def window(self, f0, vel, weights, tau, g):
        """Loss sum_t sum_p weights[t][p] . (F_p, T_p) over len(vel) steps."""
        f = f0.reshape(19, self.N)
        loss = torch.zeros((), dtype=f.dtype)
        for t in range(vel.shape[0]):
            f, FT = self.step(f, vel[t], tau, g)
            loss = loss + (weights[t] * FT).sum()
        return loss, f
