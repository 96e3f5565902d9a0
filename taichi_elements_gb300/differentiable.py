"""Differentiable rollouts: gradients of a final-state loss with respect to
initial particle velocities and per-particle Young's modulus.

The reference (taichi-dev/taichi_elements) has no autodiff.  Here the forward
rollout is the engine's own substep; the backward pass runs the hand-written
adjoint kernels of csrc/mpm_adjoint.cu substep by substep in reverse.  Memory
is bounded by checkpointing: the full particle state is saved every
`checkpoint_every` substeps during the forward pass; the backward pass
recomputes one segment at a time from its checkpoint, keeping that segment's
states (and, when memory allows, each substep's workspace), and then walks it
backwards.  Inside a segment the gradient of each state is kept in that
state's own sorted column order, so the adjoint kernels read and write it
coalesced; between segments it is held by original particle id.

Water and elastic particles are differentiated (snow and sand return maps are
non-smooth and stay forward-only); a rollout containing other materials is
rejected.  Surface colliders with friction are differentiated through their
projection and friction terms.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import NROWS, ROW_C, ROW_EP, ROW_F, ROW_ID, ROW_V, ROW_X
from .mpm_solver import MPMSolver, capture_graph

GROWS = 26  # dL/dx 3, dL/dv 3, dL/dC 9, dL/dF 9, dL/dJp 1, dL/dE 1
GROW_V, GROW_E = 3, 25


class Rollout:
    """A fixed-length rollout of an MPMSolver's particles, differentiable in
    the initial velocities v0 (n,3) and per-particle E (n,), both indexed by
    original particle id.

    Buffers are allocated once (checkpoints, one segment of states, two
    gradient buffers and, when memory allows, one workspace and grid-momentum
    snapshot per substep of a segment), so each segment's forward,
    recomputation and adjoint run as CUDA graphs after their first use."""

    def __init__(self, solver: MPMSolver, n_substeps: int, dt: float | None = None, checkpoint_every: int = 50,
                 use_cuda_graph: bool = True, keep_workspaces: bool | None = None):
        if not solver.per_particle_E:
            raise ValueError("the differentiable rollout needs MPMSolver(per_particle_E=True)")
        if not solver.support_plasticity or solver.use_g2p2g or solver.quant:
            raise NotImplementedError("gradients follow the default substep (support_plasticity=True, "
                                      "use_g2p2g=False, quant=False)")
        self.s = solver
        self.n_substeps = int(n_substeps)
        self.dt = float(dt if dt is not None else solver.default_dt)
        self.K = max(1, min(int(checkpoint_every), self.n_substeps))
        self.n = solver.n_particles
        self.use_cuda_graph = use_cuda_graph
        mats = torch.unique(solver.full_state()['material'])
        if not bool(torch.all((mats == 0) | (mats == 1))):
            raise NotImplementedError("gradients are implemented for water and elastic particles only")
        solver._prepare(self.dt * self.n_substeps)
        self.dev = solver.device
        self.cap = solver._cap
        self.init = solver._state[solver._cur].clone()  # template in the solver's current order
        self.ids = self.init.view(torch.int32)[ROW_ID, :self.n].long()
        p = solver.params
        nbytes = ctypes.c_size_t(0)
        _lib.check(solver._lib.mpm_workspace_bytes(ctypes.byref(p), self.cap, ctypes.byref(nbytes)), "ws bytes")
        self.ws = torch.zeros(int(nbytes.value), dtype=torch.uint8, device=self.dev)
        nodes = solver.views()['grid_mom'].shape[0]
        self.keep = torch.zeros((nodes, 4), dtype=torch.float32, device=self.dev)
        self.ggrid = torch.zeros((nodes, 4), dtype=torch.float32, device=self.dev)
        self.nseg = (self.n_substeps + self.K - 1) // self.K
        self.a = torch.zeros_like(self.init)
        self.b = torch.zeros_like(self.init)
        self.ckpt = torch.zeros((self.nseg, NROWS, self.cap), dtype=torch.float32, device=self.dev)
        self.ring = torch.zeros((self.K, NROWS, self.cap), dtype=torch.float32, device=self.dev)
        self.tmp = torch.zeros_like(self.init)
        self.g = [torch.zeros((GROWS, self.cap), dtype=torch.float32, device=self.dev) for _ in range(2)]
        self.gid = torch.zeros((GROWS, self.cap), dtype=torch.float32, device=self.dev)  # by original id
        self.gmid = torch.zeros((3, self.cap), dtype=torch.float32, device=self.dev)
        sp = ctypes.c_void_p(0)
        _lib.check(solver._lib.mpm_status_ptr(ctypes.byref(p), self.ws.data_ptr(), self.cap, ctypes.byref(sp)),
                   "status")
        off = sp.value - self.ws.data_ptr()
        self.status = self.ws[off:off + 4].view(torch.int32)
        self.status_acc = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self._status_off = off
        # One workspace and one momentum snapshot per substep of a segment, so
        # the recompute keeps what the adjoint needs (binning, sorted order,
        # grid velocity, pre-update momentum) and the adjoint substep runs only
        # its three kernels.  Without room for them the adjoint substep re-runs
        # the forward binning, P2G and grid update into the single workspace.
        per_slot = int(nbytes.value) + self.keep.numel() * 4
        if keep_workspaces is None:
            free, _ = torch.cuda.mem_get_info(self.dev)
            keep_workspaces = self.K * per_slot <= free // 2
        self.keep_workspaces = bool(keep_workspaces)
        if self.keep_workspaces:
            self.ws_ring = torch.zeros((self.K, int(nbytes.value)), dtype=torch.uint8, device=self.dev)
            self.keep_ring = torch.zeros((self.K, nodes, 4), dtype=torch.float32, device=self.dev)
        self._graphs = {}
        self._seen = set()

    # --------------------------------------------------------------- utils --

    @property
    def stream(self):
        return torch.cuda.current_stream(self.dev).cuda_stream

    def _call(self, name, *args):
        p = self.s.params
        _lib.check(getattr(self.s._lib, name)(ctypes.byref(p), *args), name)

    def _reset_ws(self):
        self._call("mpm_workspace_init", self.ws.data_ptr(), self.cap, self.stream)

    def _bin(self, st):
        self._call("mpm_bin_count", self.ws.data_ptr(), self.cap, st.data_ptr(), 0, self.n, self.stream)

    def _collect_status(self):
        torch.bitwise_or(self.status_acc, self.status, out=self.status_acc)

    def _check(self, extra: int = 0):
        st = int(self.status_acc.item()) | extra
        if st:
            self.status_acc.zero_()
            raise RuntimeError(f"MPM device status {st} in the differentiable rollout")

    def _substep(self, cur, nxt):
        self._call("mpm_substep", self.ws.data_ptr(), self.cap, self.n, cur.data_ptr(), nxt.data_ptr(), self.dt, None,
                   self.stream)

    def _graphed(self, kind, count, fn):
        """Run fn(count); from its second use on, as a captured CUDA graph."""
        key = (kind, count)
        g = self._graphs.get(key)
        if g is None and self.use_cuda_graph and key in self._seen:
            g = capture_graph(self.dev, lambda: fn(count))
            self._graphs[key] = g
        if g is not None:
            g.replay()
        else:
            self._seen.add(key)
            fn(count)

    def _seg_len(self, seg):
        return min(self.K, self.n_substeps - seg * self.K)

    # ----------------------------------------------------- segment bodies --

    def _forward_ops(self, count):
        """count substeps from self.a (already binned); result in self.a."""
        a, b = self.a, self.b
        for _ in range(count):
            self._substep(a, b)
            a, b = b, a
        if count % 2:
            self.a.copy_(self.b)
        self._collect_status()

    def _recompute_ops(self, count):
        """From self.a: ring[t] = state before substep t, t < count."""
        if self.keep_workspaces:
            return self._recompute_kept(count)
        self._reset_ws()
        self._bin(self.a)
        a, b = self.a, self.b
        for t in range(count):
            self.ring[t].copy_(a)
            self._substep(a, b)
            a, b = b, a
        self._collect_status()
        self._reset_ws()

    def _recompute_kept(self, count):
        """From ring[0]: the forward of each substep t into its own workspace
        ws_ring[t] (snapshot keep_ring[t]); G2P writes ring[t+1] and bins it
        into ws_ring[t+1].  The last substep's G2P is not needed."""
        cap, n, s, dt = self.cap, self.n, self.stream, self.dt
        ws = [self.ws_ring[t].data_ptr() for t in range(count)]
        self._call("mpm_bin_count", ws[0], cap, self.ring[0].data_ptr(), 0, n, s)
        for t in range(count):
            cur = self.ring[t]
            nxt = self.ring[t + 1] if t + 1 < count else self.b
            self._call("mpm_bin_finalize", ws[t], cap, n, s)
            self._call("mpm_p2g", ws[t], cap, n, cur.data_ptr(), nxt.data_ptr(), dt, s)
            self._call("mpm_grid_snapshot", ws[t], cap, self.keep_ring[t].data_ptr(), s)
            self._call("mpm_grid_update", ws[t], cap, dt, s)
            if t + 1 < count:
                self._call("mpm_g2p_bin_into", ws[t], ws[t + 1], cap, n, nxt.data_ptr(), dt, None, s)

    def _adjoint_ops(self, count):
        """Walk ring[count-1 .. 0] backwards, from the gradient in self.gid
        (by id, with respect to the state after the segment) to the gradient
        with respect to the segment's first state, written back to self.gid."""
        gin, gout = self.g
        n, cap, s = self.n, self.cap, self.stream
        if self.keep_workspaces:  # columns in the order of the recomputed end state
            _lib.check(self.s._lib.mpm_grad_reorder(self.b.data_ptr(), cap, n, GROWS, self.gid.data_ptr(),
                                                    gin.data_ptr(), 1, s), "mpm_grad_reorder")
        else:
            gin.copy_(self.gid)
        for t in reversed(range(count)):
            if self.keep_workspaces:
                self._adjoint_kernels(self.ws_ring[t].data_ptr(), self.keep_ring[t], self.ring[t], gin, gout, 0)
            else:
                self._adjoint_substep(self.ring[t], gin, gout)
            gin, gout = gout, gin
        if self.keep_workspaces:
            _lib.check(self.s._lib.mpm_grad_reorder(self.ring[0].data_ptr(), cap, n, GROWS, gin.data_ptr(),
                                                    self.gid.data_ptr(), 0, s), "mpm_grad_reorder")
        else:
            self.gid.copy_(gin)
            self._collect_status()

    def _adjoint_kernels(self, ws, keep, cur, gin, gout, by_id):
        cap, n, s, dt = self.cap, self.n, self.stream, self.dt
        self.ggrid.zero_()
        self._call("mpm_g2p_adj", ws, cap, n, cur.data_ptr(), dt, gin.data_ptr(), self.gmid.data_ptr(),
                   self.ggrid.data_ptr(), by_id, s)
        self._call("mpm_grid_adj", ws, cap, keep.data_ptr(), self.ggrid.data_ptr(), dt, s)
        self._call("mpm_p2g_adj", ws, cap, n, cur.data_ptr(), dt, gin.data_ptr(), self.gmid.data_ptr(),
                   gout.data_ptr(), self.ggrid.data_ptr(), by_id, s)

    def _adjoint_substep(self, cur, gin, gout):
        """Re-run the forward of the substep from `cur` into the single
        workspace, then its adjoint (gradients by original id)."""
        ws, cap, n, s, dt = self.ws.data_ptr(), self.cap, self.n, self.stream, self.dt
        self._bin(cur)
        self._call("mpm_bin_finalize", ws, cap, n, s)
        self._call("mpm_p2g", ws, cap, n, cur.data_ptr(), self.tmp.data_ptr(), dt, s)
        self._call("mpm_grid_snapshot", ws, cap, self.keep.data_ptr(), s)
        self._call("mpm_grid_update", ws, cap, dt, s)
        self._adjoint_kernels(ws, self.keep, cur, gin, gout, 1)

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

    def _start(self, v0, E):
        self.a.copy_(self.initial_state(v0, E))
        self.status_acc.zero_()
        self._reset_ws()
        self._bin(self.a)

    def forward(self, v0: torch.Tensor, E: torch.Tensor, keep_checkpoints: bool = True) -> torch.Tensor:
        """Final positions (n,3) by particle id; saves the checkpoints."""
        self._start(v0, E)
        for seg in range(self.nseg):
            if keep_checkpoints:
                self.ckpt[seg].copy_(self.a)
            self._graphed("fwd", self._seg_len(seg), self._forward_ops)
        torch.cuda.current_stream(self.dev).synchronize()
        self._check()
        return self.by_id(self.a, ROW_X, 3)

    # ------------------------------------------------------------ backward --

    def backward(self, gx_final: torch.Tensor):
        """dL/dv0 (n,3) and dL/dE (n,) by particle id, given dL/dx_final."""
        n = self.n
        self.gid.zero_()
        self.gid[0:3, :n] = gx_final.to(self.dev, torch.float32).t()
        if self.keep_workspaces:
            # each workspace's cell counts and block flags return to zero when
            # its substep runs, so one clear per backward pass suffices
            self.ws_ring.zero_()
        for seg in reversed(range(self.nseg)):
            count = self._seg_len(seg)
            (self.ring[0] if self.keep_workspaces else self.a).copy_(self.ckpt[seg])
            self._graphed("rec", count, self._recompute_ops)
            self._graphed("adj", count, self._adjoint_ops)
        torch.cuda.current_stream(self.dev).synchronize()
        extra = 0
        if self.keep_workspaces:
            off = self._status_off
            for v in self.ws_ring[:, off:off + 4].view(torch.int32).reshape(-1).tolist():
                extra |= v
        self._check(extra)
        return self.gid[GROW_V:GROW_V + 3, :n].t().contiguous(), self.gid[GROW_E, :n].clone()


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


def com_loss(x: torch.Tensor, material: torch.Tensor, target: torch.Tensor) -> torch.Tensor:
    """The differentiable workload's loss: the squared distance of the
    elastic particles' centre of mass from a target point,
    |mean(x[material == 1]) - target|^2."""
    sel = material == MPMSolver.material_elastic
    com = x[sel].mean(0)
    return ((com - target)**2).sum()
