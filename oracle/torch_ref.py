"""Float64 PyTorch-autograd MLS-MPM (water and elastic) - TEST INFRASTRUCTURE.

A second, differentiable restatement of the substep of taichi-dev/taichi_elements
engine/mpm_solver.py (P2G :495-584, grid update :586-616 with the bounding
box, G2P :701-724), written with torch tensor operations so that autograd
gives the reference gradients the hand-written GPU adjoint is checked
against.  Only the two smooth materials are covered: water (F reset to
diag(J,1,1), :537-542) and elastic (fixed-corotated with h = 0.3, :519-521),
with per-particle Young's modulus E.  The polar rotation R = U V^T of the
corotated stress is computed by Newton's iteration R <- (R + R^{-T}) / 2,
which converges to U V^T for det F > 0 and differentiates stably where the
SVD's own gradient has 1/(s_i^2 - s_j^2) poles (F = I).

Used only by tests/ (checked against the C oracle's float64 forward and
against its central finite differences).
"""
from __future__ import annotations


import torch


def _weights(fx):
    return [0.5 * (1.5 - fx)**2, 0.75 - (fx - 1.0)**2, 0.5 * (fx - 0.5)**2]


def _polar(F, iters=20):
    R = F
    for _ in range(iters):
        R = 0.5 * (R + torch.linalg.inv(R).transpose(-1, -2))
    return R


class TorchMPM:
    """Constants follow engine/mpm_solver.py:82-87, 200-205 (3-D)."""

    def __init__(self, res, size=1.0, gravity=(0.0, -9.8, 0.0), padding=3, device="cpu"):
        self.res = tuple(int(r) for r in res)
        self.dx = size / self.res[0]
        self.inv_dx = 1.0 / self.dx
        self.p_vol = self.dx**3
        self.p_mass = self.p_vol * 1000
        self.nu = 0.2
        self.gravity = torch.tensor(gravity, dtype=torch.float64, device=device)
        self.padding = padding
        self.device = device
        self.margin = 8
        self.W = [r + 2 * self.margin for r in self.res]
        self.lo = -self.margin

    def substep(self, x, v, C, F, Jp, mat, E, dt):
        n = x.shape[0]
        dev = x.device
        I3 = torch.eye(3, dtype=x.dtype, device=dev)
        base = torch.floor(x.detach() * self.inv_dx - 0.5).long()
        fx = x * self.inv_dx - base.to(x.dtype)
        w = _weights(fx)
        water = (mat == 0)
        mu0 = E / (2 * (1 + self.nu))
        la0 = E * self.nu / ((1 + self.nu) * (1 - 2 * self.nu))
        Fw = torch.diag_embed(torch.stack([Jp, torch.ones_like(Jp), torch.ones_like(Jp)], 1))
        Fin = torch.where(water[:, None, None], Fw, F)
        Fn = (I3 + dt * C) @ Fin
        J = torch.linalg.det(Fn)
        h = torch.where(water, torch.ones_like(E), torch.full_like(E, 0.3))
        mu = torch.where(water, torch.zeros_like(E), mu0 * h)
        la = la0 * h
        R = _polar(torch.where(water[:, None, None], I3.expand(n, 3, 3), Fn))
        stress = 2 * mu[:, None, None] * (Fn - R) @ Fn.transpose(1, 2) + (la * J * (J - 1))[:, None, None] * I3
        Fd = torch.diag_embed(torch.stack([J, torch.ones_like(J), torch.ones_like(J)], 1))
        F_new = torch.where(water[:, None, None], Fd, Fn)
        Jp_new = torch.where(water, J, Jp)
        stress = (-dt * self.p_vol * 4 * self.inv_dx**2) * stress
        mass = torch.full_like(E, self.p_mass)
        A = stress + mass[:, None, None] * C
        W = self.W
        nn = W[0] * W[1] * W[2]
        gm = torch.zeros(nn, dtype=x.dtype, device=dev)
        gmv = torch.zeros(nn, 3, dtype=x.dtype, device=dev)
        idxs, wgts, offs = [], [], []
        for a in range(3):
            for b in range(3):
                for c in range(3):
                    off = torch.tensor([a, b, c], dtype=x.dtype, device=dev)
                    node = base + torch.tensor([a, b, c], device=dev) - self.lo
                    idx = (node[:, 0] * W[1] + node[:, 1]) * W[2] + node[:, 2]
                    wgt = w[a][:, 0] * w[b][:, 1] * w[c][:, 2]
                    dpos = (off - fx) * self.dx
                    gm = gm.index_add(0, idx, wgt * mass)
                    gmv = gmv.index_add(0, idx, wgt[:, None] * (mass[:, None] * v + (A @ dpos[:, :, None])[:, :, 0]))
                    idxs.append(idx)
                    wgts.append(wgt)
                    offs.append(off)
        has = gm > 0
        gv = torch.where(has[:, None], gmv / torch.where(has, gm, torch.ones_like(gm))[:, None] + dt * self.gravity,
                         gmv)
        # bounding box (:600-616), node index in the reference grid frame
        ar = torch.arange(nn, device=dev)
        ijk = torch.stack([ar // (W[1] * W[2]), (ar // W[2]) % W[1], ar % W[2]], 1) + self.lo
        for d in range(3):
            lo_hit = (ijk[:, d] < self.padding) & (gv[:, d] < 0)
            hi_hit = (ijk[:, d] >= self.res[d] - self.padding) & (gv[:, d] > 0)
            gv = torch.where((lo_hit | hi_hit)[:, None] & (torch.arange(3, device=dev) == d)[None],
                             torch.zeros_like(gv), gv)
        new_v = torch.zeros_like(v)
        new_C = torch.zeros_like(C)
        for idx, wgt, off in zip(idxs, wgts, offs):
            g = gv[idx]
            dpos = off - fx
            new_v = new_v + wgt[:, None] * g
            new_C = new_C + 4 * self.inv_dx * wgt[:, None, None] * g[:, :, None] * dpos[:, None, :]
        x_new = x + dt * new_v
        return x_new, new_v, new_C, F_new, Jp_new

    def rollout(self, x0, v0, mat, E, dt, nsub, checkpoint=True):
        n = x0.shape[0]
        C = torch.zeros(n, 3, 3, dtype=x0.dtype, device=x0.device)
        F = torch.eye(3, dtype=x0.dtype, device=x0.device).expand(n, 3, 3).clone()
        Jp = torch.ones(n, dtype=x0.dtype, device=x0.device)
        x, v = x0, v0
        for _ in range(nsub):
            if checkpoint and torch.is_grad_enabled():
                x, v, C, F, Jp = torch.utils.checkpoint.checkpoint(
                    lambda *a: self.substep(*a, mat, E, dt), x, v, C, F, Jp, use_reentrant=False)
            else:
                x, v, C, F, Jp = self.substep(x, v, C, F, Jp, mat, E, dt)
        return x


def com_loss(x, mat, target):
    """|centre of mass of the elastic particles - target|^2."""
    sel = mat == 1
    com = x[sel].mean(0)
    return ((com - target)**2).sum()
