"""Many independent MLS-MPM scenes advanced by the same kernel launches.

The reference runs one ``MPMSolver`` per scene (engine/mpm_solver.py); a
caller with many small scenes loops over solvers, and each substep of each
scene is a handful of small launches.  ``BatchedMPM`` places every scene in
its own slot of one shared grid window: binning, block lists and grids are
shared, each particle carries its scene index in bits 8.. of its material
word, and the kernels read the scene's constants (dx, dt, Young's modulus,
gravity, bounding box, colliders) from a device table of per-scene
``MpmParams`` rows.  One substep of all scenes is one set of 10 launches;
frames of substeps are captured in a CUDA graph.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib, profiler
from .mpm_solver import capture_graph, frame_resort_interval
from ._lib import KIND_BOX, KIND_SURFACE, NROWS, ROW_C, ROW_F, ROW_ID, ROW_JP, ROW_MAT, ROW_V, ROW_X

MARGIN = 8  # grid nodes kept around each scene's domain


class BatchScene:
    """One scene of a batch: the constants a single MPMSolver would have
    (engine/mpm_solver.py:82-87, 200-210) plus its particles."""

    def __init__(self, res, x, material, v=None, size=1.0, E_scale=1.0, gravity=(0.0, -9.8, 0.0), postprocess=(),
                 dt=None, padding=3, water_density=1.0):
        self.res = tuple(int(r) for r in res)
        self.size = float(size)
        self.dx = self.size / self.res[0]
        self.inv_dx = 1.0 / self.dx
        self.default_dt = 2e-2 * self.dx / self.size
        self.dt = float(dt) if dt is not None else self.default_dt
        self.p_vol = self.dx**3
        self.p_mass = self.p_vol * 1000
        self.E, self.nu = 1e6 * self.size * E_scale, 0.2
        self.mu_0 = self.E / (2 * (1 + self.nu))
        self.lambda_0 = self.E * self.nu / ((1 + self.nu) * (1 - 2 * self.nu))
        sin_phi = math.sin(math.radians(45))
        self.alpha = math.sqrt(2 / 3) * 2 * sin_phi / (3 - sin_phi)
        self.gravity = tuple(float(g) for g in gravity)
        self.padding = padding
        self.water_density = water_density
        self.postprocess = [dict(kind=KIND_BOX, surface=0)] + [dict(c) for c in postprocess]
        self.x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 3)
        n = self.x.shape[0]
        self.v = np.zeros((n, 3), np.float32) if v is None else np.ascontiguousarray(v, dtype=np.float32).reshape(-1, 3)
        self.material = np.ascontiguousarray(np.broadcast_to(np.asarray(material, np.int32), (n,)))

    @classmethod
    def from_scene(cls, sc, **kw):
        """From a taichi_elements_gb300.scenes.Scene."""
        return cls(sc.res, sc.x, sc.material, sc.v, size=sc.size, E_scale=getattr(sc, "E_scale", 1.0),
                   postprocess=sc.postprocess, **kw)

    @property
    def n(self):
        return int(self.x.shape[0])

    def window(self):
        lo = [(-MARGIN // 4) * 4] * 3
        nb = [int(math.ceil((r + MARGIN - l) / 4.0)) for r, l in zip(self.res, lo)]
        return lo, nb


class BatchedMPM:
    """Advance many scenes together on one GPU."""

    def __init__(self, scenes, chunk=512, device=None, use_cuda_graph=True):
        if not scenes:
            raise ValueError("at least one scene is needed")
        self.device = torch.device(device if device is not None else "cuda")
        if self.device.type != "cuda" or not torch.cuda.is_available():
            raise RuntimeError("BatchedMPM needs a CUDA device; there is no CPU path")
        self._lib = _lib.load()
        self.scenes = list(scenes)
        self.chunk = int(chunk)
        self.use_cuda_graph = use_cuda_graph
        ns = len(self.scenes)
        # slot lattice
        wins = [s.window() for s in self.scenes]
        self.slot_nb = [max(w[1][d] for w in wins) for d in range(3)]
        sx = int(math.ceil(ns**(1.0 / 3.0)))
        sy = int(math.ceil(math.sqrt(ns / sx)))
        sz = int(math.ceil(ns / (sx * sy)))
        self.slots = [sx, sy, sz]
        self.win_nb = [self.slot_nb[d] * self.slots[d] for d in range(3)]
        # particles
        counts = [s.n for s in self.scenes]
        self.offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        self.n_particles = int(self.offsets[-1])
        self.cap = max(256, (self.n_particles + 255) // 256 * 256)
        self._header = self._make_header()
        rows = (_lib.MpmParams * ns)()
        for i, sc in enumerate(self.scenes):
            rows[i] = self._make_row(i, sc, wins[i][0])
        self._rows_host = rows
        self._rows = torch.frombuffer(bytearray(bytes(rows)), dtype=torch.uint8).to(self.device)
        self._state = [torch.zeros((NROWS, self.cap), dtype=torch.float32, device=self.device) for _ in range(2)]
        self._cur = 0
        self._seed()
        nbytes = ctypes.c_size_t(0)
        _lib.check(self._lib.mpm_workspace_bytes(ctypes.byref(self._header), self.cap, ctypes.byref(nbytes)),
                   "mpm_workspace_bytes")
        self._ws = torch.empty(int(nbytes.value), dtype=torch.uint8, device=self.device)
        _lib.check(self._lib.mpm_workspace_init(ctypes.byref(self._header), self._ws.data_ptr(), self.cap, self.stream),
                   "mpm_workspace_init")
        sp = ctypes.c_void_p(0)
        _lib.check(self._lib.mpm_status_ptr(ctypes.byref(self._header), self._ws.data_ptr(), self.cap,
                                            ctypes.byref(sp)), "mpm_status_ptr")
        off = sp.value - self._ws.data_ptr()
        self._status = self._ws[off:off + 4].view(torch.int32)
        _lib.check(self._lib.mpm_batch_bin_count(ctypes.byref(self._header), self._rows.data_ptr(),
                                                 self._ws.data_ptr(), self.cap, self._state[0].data_ptr(), 0,
                                                 self.n_particles, self.stream), "mpm_batch_bin_count")
        self._maxv = torch.zeros((1, ns), dtype=torch.float32, device=self.device)
        self._graphs = {}
        self._seen = set()
        self.total_substeps = 0
        # fuse_frames = True runs frames through mpm_batch_frame (the G2P of
        # one substep and the P2G of the next in one kernel, re-sorted about
        # every resort_every substeps).  Per-substep launches are the default:
        # on the 64-scene batch they are faster (0.90 against 1.00 ms per
        # substep for 4.1M particles), the scenes' small per-scene blocks
        # favouring the shared-memory staged G2P
        self.fuse_frames = False
        self.resort_every = 24

    @property
    def occupancy(self) -> int:
        """Register budget of the fused frames' particle kernel (0: 12 warps
        per SM, stencil loops unrolled; 1: 16 warps per SM, x loops rolled)."""
        return int(self._header.occupancy)

    @occupancy.setter
    def occupancy(self, value: int):
        self._header.occupancy = int(bool(value))
        self._graphs.clear()

    @property
    def stream(self) -> int:
        return torch.cuda.current_stream(self.device).cuda_stream

    def _make_header(self):
        p = _lib.MpmParams()
        p.version = _lib.ABI_VERSION
        for d in range(3):
            p.win_nb[d] = self.win_nb[d]
            p.win_lo[d] = 0
            p.slot_nb[d] = self.slot_nb[d]
            p.slots[d] = self.slots[d]
            p.res[d] = 1
        p.chunk = self.chunk
        p.plasticity = 1
        p.n_scenes = len(self.scenes)
        return p

    def _make_row(self, i, sc, lo):
        sx = i % self.slots[0]
        sy = (i // self.slots[0]) % self.slots[1]
        sz = i // (self.slots[0] * self.slots[1])
        origin = [4 * self.slot_nb[0] * sx, 4 * self.slot_nb[1] * sy, 4 * self.slot_nb[2] * sz]
        p = _lib.MpmParams.from_buffer_copy(self._header)
        for d in range(3):
            p.res[d] = sc.res[d]
            p.win_lo[d] = lo[d] - origin[d]
        p.padding = sc.padding
        p.unbounded = 0
        p.grid_size = 4096
        p.dx = sc.dx
        p.inv_dx = sc.inv_dx
        p.p_vol = sc.p_vol
        p.p_mass = sc.p_mass
        p.mu0 = sc.mu_0
        p.la0 = sc.lambda_0
        p.nu = sc.nu
        p.alpha = sc.alpha
        p.water_density = sc.water_density
        for d in range(3):
            p.gravity[d] = sc.gravity[d]
        p.stress_k = sc.p_vol * 4 * sc.inv_dx**2
        p.sand_k = (3 * sc.lambda_0 + 2 * sc.mu_0) / (2 * sc.mu_0)
        p.dt = sc.dt
        if len(sc.postprocess) > _lib.MAX_COLLIDERS:
            raise ValueError(f"at most {_lib.MAX_COLLIDERS} post-process entries per scene")
        p.n_colliders = len(sc.postprocess)
        for k, c in enumerate(sc.postprocess):
            r = p.colliders[k]
            r.kind = c["kind"]
            r.surface = c.get("surface", 0)
            nrm = list(c.get("normal", (0.0, 0.0, 0.0)))
            if c["kind"] == KIND_SURFACE:
                sc_n = 1.0 / math.sqrt(sum(t * t for t in nrm))
                nrm = [sc_n * t for t in nrm]
            for d in range(3):
                r.point[d] = c.get("point", (0, 0, 0))[d]
                r.normal[d] = nrm[d]
            r.radius = c.get("radius", 0.0)
            r.friction = c.get("friction", 0.0)
        return p

    def _seed(self):
        """seed_particle (engine/mpm_solver.py:823-838) for every scene."""
        s = self._state[0]
        si = s.view(torch.int32)
        for i, sc in enumerate(self.scenes):
            a, b = int(self.offsets[i]), int(self.offsets[i + 1])
            s[ROW_X:ROW_X + 3, a:b] = torch.from_numpy(sc.x).t().to(self.device)
            s[ROW_V:ROW_V + 3, a:b] = torch.from_numpy(sc.v).t().to(self.device)
            mat = torch.as_tensor(np.array(sc.material, dtype=np.int32)).to(self.device)
            si[ROW_MAT, a:b] = mat | (i << 8)
            s[ROW_JP, a:b] = torch.where(mat == 3, 0.0, 1.0)
        s[ROW_C:ROW_C + 9, :self.n_particles] = 0.0
        s[ROW_F:ROW_F + 9, :self.n_particles] = 0.0
        for d in range(3):
            s[ROW_F + 4 * d, :self.n_particles] = 1.0
        si[ROW_ID, :self.n_particles] = torch.arange(self.n_particles, dtype=torch.int32, device=self.device)

    def _launch(self, slot):
        cur = self._state[self._cur]
        nxt = self._state[1 - self._cur]
        mv = self._maxv[slot].data_ptr() if slot >= 0 else None
        if profiler.kernel_profiler:
            e0, e1 = profiler.substep_events()
            e0.record(torch.cuda.current_stream(self.device))
        _lib.check(self._lib.mpm_batch_substep(ctypes.byref(self._header), self._rows.data_ptr(), self._ws.data_ptr(),
                                               self.cap, self.n_particles, cur.data_ptr(), nxt.data_ptr(), mv,
                                               self.stream), "mpm_batch_substep")
        if profiler.kernel_profiler:
            e1.record(torch.cuda.current_stream(self.device))
            profiler.add_call("mpm_batch_substep", e0, e1)
        self._cur = 1 - self._cur

    def _launch_frame(self, count: int):
        """All `count` substeps as one fused frame (mpm_batch_frame)."""
        in_b = ctypes.c_int32(0)
        resort = frame_resort_interval(count, self.resort_every)
        evs, arr = profiler.frame_events(count, self.device) if profiler.kernel_profiler else (None, None)
        _lib.check(self._lib.mpm_batch_frame(ctypes.byref(self._header), self._rows.data_ptr(), self._ws.data_ptr(),
                                             self.cap, self.n_particles, self._state[self._cur].data_ptr(),
                                             self._state[1 - self._cur].data_ptr(), int(count),
                                             resort, self._maxv.data_ptr(), ctypes.byref(in_b), arr, self.stream),
                   "mpm_batch_frame")
        self._cur = (self._cur + int(in_b.value)) % 2
        if evs is not None:
            profiler.add_frame(count, evs, resort, prefix="batch ")

    def _launch_all(self, count: int):
        self._maxv[:count].zero_()
        if self.fuse_frames:
            self._launch_frame(count)
        else:
            for s in range(count):
                self._launch(s)

    def substeps(self, count: int):
        """Advance every scene by `count` substeps of its own dt (a frame);
        the frame is captured in a CUDA graph after its first run."""
        if count <= 0:
            return
        if self._maxv.shape[0] < count:
            self._maxv = torch.zeros((count, len(self.scenes)), dtype=torch.float32, device=self.device)
        key = (count, self._cur, self.fuse_frames, self.resort_every, self.occupancy)
        g = self._graphs.get(key)
        if profiler.kernel_profiler:  # events need the launches themselves
            g = None
        elif self.use_cuda_graph and g is None and key in self._seen:
            start = self._cur
            g = capture_graph(self.device, lambda: self._launch_all(count))
            self._cur = start
            self._graphs[key] = g
        if g is not None:
            g.replay()
            if self.fuse_frames:
                r = frame_resort_interval(count, self.resort_every)
                self._cur = (self._cur + (count + r - 1) // r) % 2
            else:
                self._cur = (self._cur + count) % 2
        else:
            self._seen.add(key)
            self._launch_all(count)
        self.total_substeps += count

    def check_status(self):
        st = int(self._status.item())
        if st:
            self._status.zero_()
            raise RuntimeError(f"MPM device status {st} in batched run")

    def max_velocity(self, count: int):
        """Per-substep, per-scene max |v| of the last frame: (count, n_scenes)."""
        return self._maxv[:count].cpu().numpy()

    def positions(self, i: int) -> np.ndarray:
        """Scene i's particle positions in its seeding order."""
        return self._gather(ROW_X, 3)[int(self.offsets[i]):int(self.offsets[i + 1])].cpu().numpy()

    def velocities(self, i: int) -> np.ndarray:
        return self._gather(ROW_V, 3)[int(self.offsets[i]):int(self.offsets[i + 1])].cpu().numpy()

    def _gather(self, row0, ncols):
        out = torch.empty((self.n_particles, ncols), dtype=torch.float32, device=self.device)
        _lib.check(self._lib.mpm_gather_rows(self._state[self._cur].data_ptr(), self.cap, self.n_particles, row0, ncols,
                                             out.data_ptr(), self.stream), "mpm_gather_rows")
        return out
