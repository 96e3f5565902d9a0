"""Differentiable rollouts: gradients of a final-state loss with respect to
initial particle velocities and per-particle Young's modulus.

The reference (taichi-dev/taichi_elements) has no autodiff.  Here the forward
rollout is the engine's own substep; the backward pass runs the hand-written
adjoint kernels of csrc/mpm_adjoint.cu substep by substep in reverse.  Memory
is bounded by checkpointing: the full particle state is saved every
`checkpoint_every` substeps during the forward pass; the backward pass
recomputes one segment at a time from its checkpoint, keeping that segment's
states, and then walks it backwards.  Gradients are carried in buffers
indexed by original particle id.

Water and elastic particles are differentiated (snow and sand return maps are
non-smooth and stay forward-only); a rollout containing other materials is
rejected.  Surface colliders with friction are differentiated through their
projection and friction terms.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import NROWS, ROW_C, ROW_EP, ROW_F, ROW_ID, ROW_JP, ROW_MAT, ROW_V, ROW_X
from .mpm_solver import MPMSolver

GROWS = 25  # dL/dx 3, dL/dv 3, dL/dC 9, dL/dF 9, dL/dJp 1


class Rollout:
    """A fixed-length rollout of an MPMSolver's particles, differentiable in
    the initial velocities v0 (n,3) and per-particle E (n,), both indexed by
    original particle id."""

    def __init__(self, solver: MPMSolver, n_substeps: int, dt: float | None = None, checkpoint_every: int = 50):
        if not solver.per_particle_E:
            raise ValueError("the differentiable rollout needs MPMSolver(per_particle_E=True)")
        self.s = solver
        self.n_substeps = int(n_substeps)
        self.dt = float(dt if dt is not None else solver.default_dt)
        self.K = max(1, int(checkpoint_every))
        self.n = solver.n_particles
        mats = torch.unique(solver.full_state()['material'])
        if not bool(torch.all((mats == 0) | (mats == 1))):
            raise NotImplementedError("gradients are implemented for water and elastic particles only")
        solver._prepare(self.dt * self.n_substeps)
        self.dev = solver.device
        self.cap = solver._cap
        # initial state template (solver's current order)
        self.init = solver._state[solver._cur].clone()
        self.ids = self.init.view(torch.int32)[ROW_ID, :self.n].long()
        p = solver.params
        nbytes = ctypes.c_size_t(0)
        _lib.check(solver._lib.mpm_workspace_bytes(ctypes.byref(p), self.cap, ctypes.byref(nbytes)), "ws bytes")
        self.ws = torch.empty(int(nbytes.value), dtype=torch.uint8, device=self.dev)
        v = solver.views()
        nodes = v['grid_mom'].shape[0]
        self.keep = torch.zeros((nodes, 4), dtype=torch.float32, device=self.dev)
        self.ggrid = torch.zeros((nodes, 4), dtype=torch.float32, device=self.dev)
        self.bufs = [torch.zeros_like(self.init) for _ in range(2)]
        self.tmp = torch.zeros_like(self.init)
        self.checkpoints = []
        sp = ctypes.c_void_p(0)
        _lib.check(solver._lib.mpm_status_ptr(ctypes.byref(p), self.ws.data_ptr(), self.cap, ctypes.byref(sp)),
                   "status")
        off = sp.value - self.ws.data_ptr()
        self.status = self.ws[off:off + 4].view(torch.int32)

    # --------------------------------------------------------------- utils --

    @property
    def stream(self):
        return torch.cuda.current_stream(self.dev).cuda_stream

    def _call(self, name, *args):
        p = self.s.params
        _lib.check(getattr(self.s._lib, name)(ctypes.byref(p), *args), name)

    def _reset_ws(self):
        self._call("mpm_workspace_init", self.ws.data_ptr(), self.cap, self.stream)

    def _check(self):
        st = int(self.status.item())
        if st:
            self.status.zero_()
            raise RuntimeError(f"MPM device status {st} in the differentiable rollout")

    def _substep(self, cur, nxt):
        self._call("mpm_substep", self.ws.data_ptr(), self.cap, self.n, cur.data_ptr(), nxt.data_ptr(), self.dt, None,
                   self.stream)

    def _run(self, start_state, count, keep_every=None, keep_all=None):
        """Run `count` substeps from a copy of start_state (binning it fresh);
        returns the final buffer.  keep_every: append a checkpoint copy every
        K substeps (before the substep); keep_all: list receiving the state
        before every substep."""
        a, b = self.bufs
        a.copy_(start_state)
        self._reset_ws()
        self._call("mpm_bin_count", self.ws.data_ptr(), self.cap, a.data_ptr(), 0, self.n, self.stream)
        for t in range(count):
            if keep_every is not None and t % keep_every == 0:
                self.checkpoints.append(a.clone())
            if keep_all is not None:
                keep_all.append(a.clone())
            self._substep(a, b)
            a, b = b, a
        return a

    # ------------------------------------------------------------- forward --

    def initial_state(self, v0: torch.Tensor, E: torch.Tensor) -> torch.Tensor:
        st = self.init.clone()
        st[ROW_V:ROW_V + 3, :self.n] = v0.to(self.dev, torch.float32)[self.ids].t()
        st[ROW_EP, :self.n] = E.to(self.dev, torch.float32)[self.ids]
        st[ROW_C:ROW_C + 9, :self.n] = 0.0
        st[ROW_F:ROW_F + 9, :self.n] = 0.0
        for d in range(3):
            st[ROW_F + 4 * d, :self.n] = 1.0
        return st

    def by_id(self, st: torch.Tensor, row0: int, ncols: int) -> torch.Tensor:
        ids = st.view(torch.int32)[ROW_ID, :self.n].long()
        out = torch.empty((self.n, ncols), dtype=torch.float32, device=self.dev)
        out[ids] = st[row0:row0 + ncols, :self.n].t()
        return out

    def forward(self, v0: torch.Tensor, E: torch.Tensor) -> torch.Tensor:
        """Final positions (n,3) by particle id; saves checkpoints."""
        self.checkpoints = []
        final = self._run(self.initial_state(v0, E), self.n_substeps, keep_every=self.K)
        torch.cuda.synchronize()
        self._check()
        self.final = final.clone()
        return self.by_id(final, ROW_X, 3)

    # ------------------------------------------------------------ backward --

    def backward(self, gx_final: torch.Tensor):
        """dL/dv0 (n,3) and dL/dE (n,) by particle id, given dL/dx_final."""
        n, cap = self.n, self.cap
        gin = torch.zeros((GROWS, cap), dtype=torch.float32, device=self.dev)
        gout = torch.zeros_like(gin)
        gin[0:3, :n] = gx_final.to(self.dev, torch.float32).t()
        gE = torch.zeros(cap, dtype=torch.float32, device=self.dev)
        nseg = len(self.checkpoints)
        for seg in reversed(range(nseg)):
            t0 = seg * self.K
            count = min(self.K, self.n_substeps - t0)
            states = []
            self._run(self.checkpoints[seg], count, keep_all=states)
            self._reset_ws()
            for t in reversed(range(count)):
                cur = states[t]
                self._adjoint_substep(cur, gin, gout, gE)
                gin, gout = gout, gin
            del states
        torch.cuda.synchronize()
        self._check()
        gv0 = gin[3:6, :n].t().contiguous()
        return gv0, gE[:n].clone()

    def _adjoint_substep(self, cur, gin, gout, gE):
        ws, cap, n, s = self.ws.data_ptr(), self.cap, self.n, self.stream
        dt = self.dt
        self._call("mpm_bin_count", ws, cap, cur.data_ptr(), 0, n, s)
        self._call("mpm_bin_finalize", ws, cap, n, s)
        self._call("mpm_p2g", ws, cap, n, cur.data_ptr(), self.tmp.data_ptr(), dt, s)
        self._call("mpm_grid_snapshot", ws, cap, self.keep.data_ptr(), s)
        self._call("mpm_grid_update", ws, cap, dt, s)
        self.ggrid.zero_()
        self._call("mpm_g2p_adj", ws, cap, n, self.tmp.data_ptr(), dt, gin.data_ptr(), gout.data_ptr(),
                   self.ggrid.data_ptr(), s)
        self._call("mpm_grid_adj", ws, cap, self.keep.data_ptr(), self.ggrid.data_ptr(), dt, s)
        self._call("mpm_p2g_adj", ws, cap, n, cur.data_ptr(), self.tmp.data_ptr(), dt, gin.data_ptr(),
                   gout.data_ptr(), self.ggrid.data_ptr(), gE.data_ptr(), s)


class _RolloutFunction(torch.autograd.Function):

    @staticmethod
    def forward(ctx, v0, E, rollout):
        ctx.rollout = rollout
        return rollout.forward(v0.detach(), E.detach())

    @staticmethod
    def backward(ctx, gx):
        gv0, gE = ctx.rollout.backward(gx.contiguous())
        return gv0, gE, None


def rollout_positions(rollout: Rollout, v0: torch.Tensor, E: torch.Tensor) -> torch.Tensor:
    """Final positions of `rollout` as a differentiable function of the
    initial velocities v0 (n,3) and Young's moduli E (n,)."""
    return _RolloutFunction.apply(v0, E, rollout)
