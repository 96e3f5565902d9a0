"""Drop-in replacement for taichi_elements' ``engine.mpm_solver.MPMSolver``.

The public surface follows engine/mpm_solver.py of taichi-dev/taichi_elements:
the constructor (:44-310), the material/surface constants (:16-42),
``add_cube`` (:861-884), ``add_ellipsoid`` (:980-1015), ``add_particles``
(:1097-1104), ``read_restart`` (:1128-1144), ``add_surface_collider``
(:647-687), ``add_sphere_collider`` (:618-642), ``add_bounding_box``
(:689-692), ``clear_grid_postprocess`` (:644-645), ``set_gravity``
(:316-319), ``set_source_velocity`` (:852-859), ``step`` (:748-821),
``particle_info`` (:1172-1191), ``clear_particles`` (:1193-1196) and the
frame writers ``write_particles`` / ``write_particles_ply`` (:1198-1209).

State lives in PyTorch CUDA tensors; every substep runs the hand-written
sm_103a kernels of libmpm_gb300.so through ctypes.  There is no CPU path: a
machine without a CUDA device, or without the built library, raises.

Extensions beyond the reference: ``substep(dt)``, per-particle Young's
modulus (``per_particle_E=True`` and the ``E`` argument of the seeding
calls), ``state_dict``/``load_state_dict`` (exact checkpoints of x, v, C, F,
Jp), ``tensors()`` (zero-copy device views), CUDA-graph capture of whole
frames, fused frames (the G2P of one substep and the P2G of the next in one
kernel, ``fuse_frames``) and a measured choice of the substep schedule
(``autotune=True``).

``quant=True`` keeps the particles in the packed layout of the reference's
quantized fields (engine/mpm_solver.py:106-127, :216-262): positions as
21-bit fixed point in [-2, 2), velocities as block floating point (a 7-bit
shared exponent and 19-bit mantissas), F as 16-bit fixed point of range
+-4.1 and the material in 16 bits; 84 bytes per particle instead of 112.
``support_plasticity=False`` drops the Jp updates (:62 and the
``ti.static(self.support_plasticity)`` branches).
"""
from __future__ import annotations

import ctypes
import math
import numbers
import sys
import threading
import time

import numpy as np
import torch

from . import _lib, profiler
from ._lib import (KIND_BOX, KIND_SPHERE, KIND_SURFACE, NROWS, QROWS, ROW_C, ROW_EP, ROW_F, ROW_ID, ROW_JP, ROW_MAT,
                   ROW_V, ROW_X)


class MPMError(RuntimeError):
    """A device-side fault reported through the engine's status word."""


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


class ParticleCount(int):
    """The particle count: an int that also reads like the reference's
    scalar field, ``solver.n_particles[None]`` (engine/mpm_solver.py:88,
    used by demo/demo_3d_bunnies_recursive.py:136)."""

    def __getitem__(self, key):
        if key is None or key == ():
            return int(self)
        raise TypeError("n_particles is a scalar: index it with [None]")


# Page-locked host buffers for device-to-host copies, shared by all
# solvers of the process: pairs of a pinned tensor and the numpy array that
# views it.  The numpy array is what callers receive; it (or any numpy view
# of it) is referenced while a caller holds it, and a pair is handed out
# again only when nothing but the pool references its array, so every
# returned array stays the caller's own, as the reference's fresh copies are.
# Unused pairs are dropped, oldest first, above _PINNED_POOL_BYTES.
_pinned_pool: list = []
_PINNED_POOL_BYTES = 8 << 30
_pinned_lock = threading.Lock()


def _pinned_buffer(shape, dtype):
    """A free (pinned tensor, numpy view) pair of this shape and dtype."""
    with _pinned_lock:
        return _pinned_buffer_locked(tuple(shape), dtype)


def _pinned_buffer_locked(shape, dtype):
    for pair in _pinned_pool:
        h, hn = pair
        # held by the pool alone: the pair, the local name, getrefcount's argument
        if h.dtype == dtype and tuple(h.shape) == shape and sys.getrefcount(hn) <= 3:
            return pair
    h = hn = pair = None  # the loop's names must not keep a pool array referenced
    h = torch.empty(shape, dtype=dtype, pin_memory=True)
    pair = (h, h.numpy())
    _pinned_pool.append(pair)
    total = sum(q[0].numel() * q[0].element_size() for q in _pinned_pool)
    i = 0
    while total > _PINNED_POOL_BYTES and i < len(_pinned_pool):
        q = _pinned_pool[i]
        if q is not pair and sys.getrefcount(q[1]) <= 2:  # the pair and the argument
            total -= q[0].numel() * q[0].element_size()
            del _pinned_pool[i]
        else:
            i += 1
        q = None
    return pair


def capture_graph(device, launch) -> torch.cuda.CUDAGraph:
    """A CUDA graph of the launches `launch()` makes, captured on a side
    stream ordered after the current one.  Unlike torch.cuda.graph this makes
    no device-wide synchronisation and frees no cached memory, and the
    capture restricts only the capturing thread, so solvers driven from other
    host threads keep launching, copying and capturing meanwhile."""
    g = torch.cuda.CUDAGraph()
    main = torch.cuda.current_stream(device)
    side = torch.cuda.Stream(device=device)
    side.wait_stream(main)
    with torch.cuda.stream(side):
        g.capture_begin(capture_error_mode="thread_local")
        try:
            launch()
        finally:
            g.capture_end()
    main.wait_stream(side)
    return g


def frame_resort_interval(count: int, target: int) -> int:
    """Re-sort interval for a fused frame of `count` substeps and a target
    interval: round(count / target) sorts (at least one) at equal spacing,
    so that no sort serves only the last substep or two of a frame."""
    sorts = max(1, int(count / max(1, target) + 0.5))
    return max(1, -(-count // sorts))


class MPMSolver:
    material_water = 0
    material_elastic = 1
    material_snow = 2
    material_sand = 3
    material_stationary = 4
    materials = {
        'WATER': material_water,
        'ELASTIC': material_elastic,
        'SNOW': material_snow,
        'SAND': material_sand,
        'STATIONARY': material_stationary,
    }

    surface_sticky = 0
    surface_slip = 1
    surface_separate = 2
    surfaces = {'STICKY': surface_sticky, 'SLIP': surface_slip, 'SEPARATE': surface_separate}

    # particles per P2G/G2P work item when the caller does not choose one
    DEFAULT_CHUNK = 512
    # grid nodes kept around the simulation box / particle bounding box
    WINDOW_MARGIN = 8

    def __init__(self,
                 res,
                 quant=False,
                 use_voxelizer=True,
                 size=1,
                 max_num_particles=2**30,
                 padding=3,
                 unbounded=False,
                 dt_scale=1,
                 E_scale=1,
                 voxelizer_super_sample=2,
                 use_g2p2g=False,
                 v_clamp_g2p2g=True,
                 use_bls=True,
                 g2p2g_allowed_cfl=0.9,
                 water_density=1.0,
                 support_plasticity=True,
                 use_adaptive_dt=False,
                 use_ggui=False,
                 use_emitter_id=False,
                 *,
                 device=None,
                 seed=0,
                 chunk=None,
                 use_cuda_graph=True,
                 per_particle_E=False,
                 autotune=False):
        self.dim = len(res)
        assert self.dim in (2, 3), "MPM solver supports only 2D and 3D simulations."
        if self.dim != 3:
            raise NotImplementedError("the GB300 engine implements the 3-D solver only")

        self.device = torch.device(device if device is not None else "cuda")
        if self.device.type != "cuda" or not torch.cuda.is_available():
            raise RuntimeError("MPMSolver (GB300 engine) needs a CUDA device; there is no CPU path")
        self._lib = _lib.load()

        self.quant = quant
        self.use_g2p2g = use_g2p2g
        self.v_clamp_g2p2g = v_clamp_g2p2g
        self.use_bls = use_bls
        self.g2p2g_allowed_cfl = g2p2g_allowed_cfl
        self.water_density = water_density
        self.grid_size = 4096
        self.t = 0.0
        self.res = tuple(int(r) for r in res)
        self.size = size
        # constants: engine/mpm_solver.py:82-87
        self.dx = size / res[0]
        self.inv_dx = 1.0 / self.dx
        self.default_dt = 2e-2 * self.dx / size * dt_scale
        self.p_vol = self.dx**self.dim
        self.p_rho = 1000
        self.p_mass = self.p_vol * self.p_rho
        self.max_num_particles = max_num_particles
        self.all_time_max_velocity = 0
        self.support_plasticity = support_plasticity
        self.use_adaptive_dt = use_adaptive_dt
        self.use_ggui = use_ggui
        self.F_bound = 4.0
        self.use_emitter_id = use_emitter_id
        self.unbounded = unbounded
        if unbounded:  # :143-149
            while self.grid_size <= 2 * max(self.res):
                self.grid_size *= 2
        self.offset = tuple(-self.grid_size // 2 for _ in range(self.dim))
        self.leaf_block_size = 4
        self.padding = padding
        # :200-210
        self.E, self.nu = 1e6 * size * E_scale, 0.2
        self.mu_0 = self.E / (2 * (1 + self.nu))
        self.lambda_0 = self.E * self.nu / ((1 + self.nu) * (1 - 2 * self.nu))
        friction_angle = math.radians(45)
        sin_phi = math.sin(friction_angle)
        self.alpha = math.sqrt(2 / 3) * 2 * sin_phi / (3 - sin_phi)
        self.total_substeps = 0
        self.voxelizer = None  # built on the first add_mesh (engine/mpm_solver.py:284-293)
        self.use_voxelizer = bool(use_voxelizer)
        self.voxelizer_super_sample = voxelizer_super_sample
        self.writers = []

        self.per_particle_E = bool(per_particle_E)
        # frames run fused (mpm_frame), re-sorting the particles by grid block
        # every `resort_every` substeps (the storage order drifts from the
        # positions in between); autotune.tune_schedule measures both choices
        self.fuse_frames = True
        self.resort_every = 24
        # MpmParams.occupancy: 0 = the fused and P2G kernels' stencil loops
        # fully unrolled at 12 warps per SM, 1 = rolled at 16 (the faster one
        # depends on the scene; autotune.tune_schedule measures both)
        self._occupancy = 0
        self.chunk = int(chunk) if chunk else self.DEFAULT_CHUNK
        self.use_cuda_graph = use_cuda_graph
        self.autotune = bool(autotune)
        self._tuned = False
        self.gravity = (0.0, -9.8, 0.0)
        self.source_velocity = (0.0, 0.0, 0.0)
        self.grid_postprocess = []  # records: dicts with kind/surface/...
        self.add_bounding_box(self.unbounded)

        self.n_particles = 0
        self._cap = 0
        self._state = [None, None]
        self._cur = 0
        self._color = None
        self._emitter = None
        self._ws = None
        self._binned = 0
        self._window = None  # (lo[3], nb[3])
        self._params = None
        self._params_version = 0
        self._graphs = {}
        self._graph_seen = set()
        # fused G2P2G mode (engine/mpm_solver.py:363-485): particles covered by
        # the finalized binning of the current state, the reference's
        # last_time_final_particles, and whether the grid velocities of the
        # previous substep are valid
        self._g2p2g_listed = 0
        self._last_final = 0
        self._g2p2g_grid_valid = False
        self._maxv = torch.zeros(1024, dtype=torch.float32, device=self.device)
        self._gen = torch.Generator(device=self.device)
        self._gen.manual_seed(int(seed))
        self._seed = int(seed)
        self._mesh_seed = 0
        self._seed_lo = None  # bounding box (in nodes) of all seeded regions
        self._seed_hi = None
        # bounding box (lo, hi) of the particle positions, known without a
        # device reduction after a frame's readback; None when unknown
        self._host_box = None
        self._readback = None  # page-locked buffers of the end-of-frame readback
        self._copy_stream = None  # side stream of particle_info's host copies
        self._set_window(*self._box_window())

    # ---------------------------------------------------------- params ---

    def _box_window(self):
        m = self.WINDOW_MARGIN
        lo = [(-m // 4) * 4] * 3
        hi = [r + m for r in self.res]
        return lo, hi

    def _set_window(self, lo, hi):
        lo = [int(math.floor(l / 4.0)) * 4 for l in lo]
        nb = [int(math.ceil((h - l) / 4.0)) for l, h in zip(lo, hi)]
        self._window = (lo, nb)
        self._params = None

    def _build_params(self) -> _lib.MpmParams:
        p = _lib.MpmParams()
        p.version = _lib.ABI_VERSION
        for d in range(3):
            p.res[d] = self.res[d]
            p.win_lo[d] = self._window[0][d]
            p.win_nb[d] = self._window[1][d]
        p.padding = self.padding
        p.unbounded = int(bool(self.unbounded))
        p.grid_size = self.grid_size
        p.has_Ep = int(self.per_particle_E)
        p.chunk = self.chunk
        p.plasticity = int(bool(self.support_plasticity))
        p.quant = int(bool(self.quant))
        p.occupancy = self._occupancy
        p.dx = self.dx
        p.inv_dx = self.inv_dx
        p.p_vol = self.p_vol
        p.p_mass = self.p_mass
        p.mu0 = self.mu_0
        p.la0 = self.lambda_0
        p.nu = self.nu
        p.alpha = self.alpha
        p.water_density = self.water_density
        for d in range(3):
            p.gravity[d] = self.gravity[d]
        p.stress_k = self.p_vol * 4 * self.inv_dx**2
        p.sand_k = (self.dim * self.lambda_0 + 2 * self.mu_0) / (2 * self.mu_0)
        if self.use_g2p2g and self.v_clamp_g2p2g and self.g2p2g_allowed_cfl > 0:
            p.v_clamp_k = self.dx * self.g2p2g_allowed_cfl  # :589, :594-598
        if len(self.grid_postprocess) > _lib.MAX_COLLIDERS:
            raise ValueError(f"at most {_lib.MAX_COLLIDERS} grid post-process entries are supported")
        p.n_colliders = len(self.grid_postprocess)
        for i, c in enumerate(self.grid_postprocess):
            r = p.colliders[i]
            r.kind = c["kind"]
            r.surface = c["surface"]
            for d in range(3):
                r.point[d] = c.get("point", (0, 0, 0))[d]
                r.normal[d] = c.get("normal", (0, 0, 0))[d]
            r.radius = c.get("radius", 0.0)
            r.friction = c.get("friction", 0.0)
        return p

    @property
    def params(self) -> _lib.MpmParams:
        if self._params is None:
            self._params = self._build_params()
            self._params_version += 1
            self._graphs.clear()
        return self._params

    @property
    def occupancy(self) -> int:
        """Register budget of the fused and P2G kernels (MpmParams.occupancy)."""
        return self._occupancy

    @occupancy.setter
    def occupancy(self, value):
        value = int(bool(value))
        if value != self._occupancy:
            self._occupancy = value
            self._invalidate_params()

    def _invalidate_params(self):
        self._params = None

    def set_gravity(self, g):
        assert isinstance(g, (tuple, list))
        assert len(g) == self.dim
        self.gravity = tuple(float(x) for x in g)
        self._invalidate_params()

    def set_source_velocity(self, velocity):
        """engine/mpm_solver.py:852-859: the velocity the seeding routines
        give new particles (None = zero).  Each add_* call sets it from its
        own `velocity` argument, as in the reference."""
        if velocity is not None:
            velocity = list(velocity)
            assert len(velocity) == self.dim
            self.source_velocity = tuple(float(v) for v in velocity)
        else:
            self.source_velocity = (0.0,) * self.dim

    # -------------------------------------------------------- colliders ---

    def add_sphere_collider(self, center, radius, surface=surface_sticky):
        center = list(center)
        self.grid_postprocess.append(
            dict(kind=KIND_SPHERE, surface=int(surface), point=tuple(center), radius=float(radius)))
        self._invalidate_params()

    def clear_grid_postprocess(self):
        self.grid_postprocess.clear()
        self._invalidate_params()

    def add_surface_collider(self, point, normal, surface=surface_sticky, friction=0.0):
        point = list(point)
        normal_scale = 1.0 / math.sqrt(sum(x**2 for x in normal))
        normal = list(normal_scale * x for x in normal)
        if surface == self.surface_sticky and friction != 0:
            raise ValueError('friction must be 0 on sticky surfaces.')
        self.grid_postprocess.append(
            dict(kind=KIND_SURFACE, surface=int(surface), point=tuple(point), normal=tuple(normal),
                 friction=float(friction)))
        self._invalidate_params()

    def add_bounding_box(self, unbounded):
        self.grid_postprocess.append(dict(kind=KIND_BOX, surface=int(bool(unbounded))))
        self._invalidate_params()

    @property
    def n_particles(self) -> ParticleCount:
        return ParticleCount(self._n)

    @n_particles.setter
    def n_particles(self, value):
        self._n = int(value)

    @property
    def particle(self):
        """Per-particle storage size in the form of the reference's particle
        SNode (demo/demo_3d_bunnies_recursive.py:151 prints
        ``particle._cell_size_bytes``): state rows plus colour and emitter id."""
        import types
        rows = QROWS if self.quant else NROWS
        return types.SimpleNamespace(_cell_size_bytes=4 * rows + 8)

    # ------------------------------------------------------ allocation ---

    @property
    def stream(self) -> int:
        return torch.cuda.current_stream(self.device).cuda_stream

    def _alloc(self, cap: int):
        """(Re)allocate particle buffers with capacity `cap`, keeping data."""
        cap = int((cap + 255) // 256 * 256)
        n = self.n_particles
        rows = QROWS if self.quant else NROWS
        new_state = [torch.zeros((rows, cap), dtype=torch.float32, device=self.device) for _ in range(2)]
        new_color = torch.zeros(cap, dtype=torch.int32, device=self.device)
        new_emit = torch.zeros(cap, dtype=torch.int32, device=self.device)
        if n > 0:
            new_state[0][:, :n] = self._state[self._cur][:, :n]
            new_color[:n] = self._color[:n]
            new_emit[:n] = self._emitter[:n]
        self._state = new_state
        self._cur = 0
        self._color = new_color
        self._emitter = new_emit
        self._cap = cap
        self._ws = None  # workspace depends on the capacity
        self._graphs.clear()

    def _ensure_workspace(self):
        if self._ws is not None:
            return
        p = self.params
        nbytes = ctypes.c_size_t(0)
        _lib.check(self._lib.mpm_workspace_bytes(ctypes.byref(p), self._cap, ctypes.byref(nbytes)),
                   "mpm_workspace_bytes")
        self._ws = torch.empty(int(nbytes.value), dtype=torch.uint8, device=self.device)
        _lib.check(self._lib.mpm_workspace_init(ctypes.byref(p), _ptr(self._ws), self._cap, self.stream),
                   "mpm_workspace_init")
        sp = ctypes.c_void_p(0)
        _lib.check(self._lib.mpm_status_ptr(ctypes.byref(p), _ptr(self._ws), self._cap, ctypes.byref(sp)),
                   "mpm_status_ptr")
        off = sp.value - _ptr(self._ws)
        self._status = self._ws[off:off + 4].view(torch.int32)
        self._binned = 0
        self._g2p2g_listed = 0
        self._g2p2g_grid_valid = False  # a new workspace has no grid of the previous substep
        self._graphs.clear()

    def _ensure_capacity(self, extra: int):
        need = self.n_particles + extra
        if need > self._cap:
            cap = max(need, 2 * self._cap, 1 << 16)
            cap = min(cap, max(self.max_num_particles, need))
            self._alloc(cap)

    def _cover(self, lo_pos, hi_pos):
        """Grow the grid window so positions in [lo_pos, hi_pos] keep their
        stencils inside it with the margin."""
        m = self.WINDOW_MARGIN
        wlo, wnb = self._window
        whi = [l + 4 * b for l, b in zip(wlo, wnb)]
        # non-finite coordinates do not move the window; the kernels flag them
        lo_n = [int(math.floor(l * self.inv_dx)) - m if math.isfinite(l) else wl for l, wl in zip(lo_pos, wlo)]
        hi_n = [int(math.ceil(h * self.inv_dx)) + m if math.isfinite(h) else wh for h, wh in zip(hi_pos, whi)]
        if all(a >= b for a, b in zip(lo_n, wlo)) and all(a <= b for a, b in zip(hi_n, whi)):
            return
        half = self.grid_size // 2
        new_lo = [max(-half, min(a, b)) for a, b in zip(lo_n, wlo)]
        new_hi = [min(half, max(a, b)) for a, b in zip(hi_n, whi)]
        self._set_window(new_lo, new_hi)
        self._ws = None

    def _rebin(self):
        """Bin particles that are not binned yet (all after a workspace reset)."""
        self._ensure_workspace()
        if self.use_g2p2g and self._g2p2g_listed:
            if self._g2p2g_listed == self.n_particles:
                return  # the finalized binning of the last substep covers every particle
            # particles were added since: the counts were consumed, count all again
            self._binned = 0
            self._g2p2g_listed = 0
        if self._binned < self.n_particles:
            p = self.params
            _lib.check(
                self._lib.mpm_bin_count(ctypes.byref(p), _ptr(self._ws), self._cap, _ptr(self._state[self._cur]),
                                        self._binned, self.n_particles, self.stream), "mpm_bin_count")
            self._binned = self.n_particles

    # ---------------------------------------------------------- seeding ---

    def _append(self, x: torch.Tensor, material, color, velocity, emitter_id=0, E=None, C=None, F=None, Jp=None):
        """Append particles with positions x (n,3) float32 on the device.
        engine/mpm_solver.py:823-838 (seed_particle): F = I, C = 0,
        Jp = 0 for sand and 1 otherwise, v = source velocity.  C, F (n,3,3)
        and Jp (n,) replace those defaults (exact checkpoints).  With
        quant=True the rows are packed on the device (x, v and F rounded to
        the stored formats)."""
        n = int(x.shape[0])
        if n == 0:
            return
        assert self.n_particles + n <= self.max_num_particles
        self._ensure_capacity(n)
        a, b = self.n_particles, self.n_particles + n
        st = self._state[self._cur]
        # float32 storage: the rows are written in place (slots a..b of the
        # state); packed storage builds them in float32 and packs them below
        s = torch.empty((NROWS, n), dtype=torch.float32, device=self.device) if self.quant else st[:, a:b]
        si = s.view(torch.int32)
        s[ROW_X:ROW_X + 3] = x.t()
        if isinstance(velocity, torch.Tensor):
            s[ROW_V:ROW_V + 3] = velocity.to(self.device, torch.float32).t()
        else:
            self.set_source_velocity(velocity)
            vel = list(self.source_velocity)
            for d in range(3):
                s[ROW_V + d] = float(np.float32(vel[d]))
        s[ROW_C:ROW_C + 9] = 0.0
        s[ROW_F:ROW_F + 9] = 0.0
        for d in range(3):
            s[ROW_F + 4 * d] = 1.0
        if isinstance(material, torch.Tensor):
            mat = material.to(self.device, torch.int32)
            si[ROW_MAT] = mat
            s[ROW_JP] = torch.where(mat == self.material_sand, 0.0, 1.0)
        else:
            si[ROW_MAT] = int(material)
            s[ROW_JP] = 0.0 if int(material) == self.material_sand else 1.0
        si[ROW_ID] = torch.arange(a, b, dtype=torch.int32, device=self.device)
        s[ROW_EP] = 0.0
        if self.per_particle_E:
            if E is None:
                s[ROW_EP] = float(self.E)
            elif isinstance(E, torch.Tensor):
                s[ROW_EP] = E.to(self.device, torch.float32)
            else:
                s[ROW_EP] = float(E)
        if C is not None:
            s[ROW_C:ROW_C + 9] = C.reshape(n, 9).t().to(self.device, torch.float32)
        if F is not None:
            s[ROW_F:ROW_F + 9] = F.reshape(n, 9).t().to(self.device, torch.float32)
        if Jp is not None:
            s[ROW_JP] = Jp.to(self.device, torch.float32)
        if self.quant:
            _lib.check(
                self._lib.mpm_quant_pack(_ptr(s), n, n, _ptr(st), self._cap, a, None, self.stream),
                "mpm_quant_pack")
        if isinstance(color, torch.Tensor):
            self._color[a:b] = color.to(self.device, torch.int32)
        else:
            self._color[a:b] = int(np.array(int(color), dtype=np.int64).astype(np.int32))
        self._emitter[a:b] = int(emitter_id)
        self.n_particles = b
        # bin the new particles (the window may have grown: that rebins all)
        self._rebin()

    def _note_region(self, lo, hi):
        if self.quant and any(not (-2.0 <= float(c) < 2.0) for c in list(lo) + list(hi)):
            raise ValueError("quant=True stores positions as fixed point in [-2, 2)")
        self._cover(lo, hi)
        if self._host_box is not None:  # new particles inside [lo, hi]: the union bounds all
            blo, bhi = self._host_box
            self._host_box = ([min(a, float(b)) for a, b in zip(blo, lo)], [max(a, float(b)) for a, b in zip(bhi, hi)])

    @staticmethod
    def _finite_bounds(x: torch.Tensor):
        """Per-axis min/max over the finite entries of an (n,3) tensor."""
        fin = torch.isfinite(x)
        lo = torch.where(fin, x, torch.full_like(x, float('inf'))).min(0).values
        hi = torch.where(fin, x, torch.full_like(x, float('-inf'))).max(0).values
        return lo.tolist(), hi.tolist()

    def add_cube(self, lower_corner, cube_size, material, color=0xFFFFFF, sample_density=None, velocity=None,
                 E=None):
        """engine/mpm_solver.py:861-884; positions lower + U[0,1) * size."""
        if sample_density is None:
            sample_density = 2**self.dim
        vol = 1
        for i in range(self.dim):
            vol = vol * cube_size[i]
        num_new_particles = int(sample_density * vol / self.dx**self.dim + 1)
        assert self.n_particles + num_new_particles <= self.max_num_particles
        lo = torch.tensor([float(v) for v in lower_corner], dtype=torch.float32, device=self.device)
        sz = torch.tensor([float(v) for v in cube_size], dtype=torch.float32, device=self.device)
        u = torch.rand((num_new_particles, 3), generator=self._gen, device=self.device, dtype=torch.float32)
        x = lo + u * sz
        self._note_region([float(a) for a in lower_corner],
                          [float(a) + float(b) for a, b in zip(lower_corner, cube_size)])
        self._append(x, material, color, velocity, E=E)

    def add_ellipsoid(self, center, radius, material, color=0xFFFFFF, sample_density=None, velocity=None, E=None):
        """engine/mpm_solver.py:980-1015 with rejection sampling in the unit
        sphere (:959-967)."""
        if sample_density is None:
            sample_density = 2**self.dim
        if isinstance(radius, numbers.Number):
            radius = [radius] * self.dim
        radius = list(radius)
        num_particles = 4 / 3 * math.pi
        for i in range(self.dim):
            num_particles *= radius[i] * self.inv_dx
        num_particles = int(math.ceil(num_particles * sample_density))
        assert self.n_particles + num_particles <= self.max_num_particles
        pts = []
        have = 0
        while have < num_particles:
            m = max(64, int((num_particles - have) * 2.1) + 64)
            u = torch.rand((m, 3), generator=self._gen, device=self.device, dtype=torch.float32) * 2 - 1
            u = u[(u * u).sum(1) <= 1]
            pts.append(u)
            have += int(u.shape[0])
        u = torch.cat(pts)[:num_particles]
        c = torch.tensor([float(v) for v in center], dtype=torch.float32, device=self.device)
        r = torch.tensor([float(v) for v in radius], dtype=torch.float32, device=self.device)
        x = c + u * r
        self._note_region([float(a) - float(b) for a, b in zip(center, radius)],
                          [float(a) + float(b) for a, b in zip(center, radius)])
        self._append(x, material, color, velocity, E=E)

    def add_particles(self, particles, material, color=0xFFFFFF, velocity=None, E=None):
        """engine/mpm_solver.py:1081-1104."""
        x = torch.as_tensor(np.asarray(particles, dtype=np.float32)).reshape(-1, 3)
        if x.shape[0] == 0:
            return
        self._note_region(*self._finite_bounds(x))
        self._append(x.to(self.device), material, color, velocity, E=E)

    def read_restart(self, num_particles, pos, vel, material, color):
        """engine/mpm_solver.py:1106-1144 (per-particle x, v, material,
        color; F = I, Jp reset, C = 0)."""
        num_particles = int(num_particles)
        if num_particles == 0:
            return

        def dev(a, dtype):
            # to the device first: conversions and the bounds run there
            a = np.asarray(a[:num_particles])
            t = torch.from_numpy(np.ascontiguousarray(a))
            return t.to(self.device).to(dtype)

        x = dev(pos, torch.float32).reshape(-1, 3)
        v = dev(vel, torch.float32).reshape(-1, 3)
        m = dev(material, torch.int32)
        # colours wrap to int32 like the reference's i32 field
        c = dev(color, torch.int64).to(torch.int32) if np.asarray(color).dtype != np.int32 else dev(color, torch.int32)
        self._note_region(*self._finite_bounds(x))
        self._append(x, m, c, v, E=None)

    def add_mesh(self, triangles, material, color=0xFFFFFF, sample_density=None, velocity=None, translation=None,
                 emmiter_id=0):
        """engine/mpm_solver.py:1049-1079: voxelize a triangle mesh (n, 9) on
        the GPU and seed particles in the voxels inside it
        (seed_from_voxels, :1017-1047)."""
        assert self.dim == 3
        if not self.use_voxelizer:
            raise RuntimeError("add_mesh needs MPMSolver(use_voxelizer=True)")
        if sample_density is None:
            sample_density = 2**self.dim
        self.set_source_velocity(velocity=velocity)
        t = [float(translation[i]) if translation else 0.0 for i in range(self.dim)]
        if self.voxelizer is None:
            from .voxelizer import Voxelizer
            self.voxelizer = Voxelizer(res=self.res, dx=self.dx, padding=self.padding,
                                       super_sample=self.voxelizer_super_sample, device=self.device)
        self.voxelizer.voxelize(triangles)
        self._mesh_seed += 1
        x = self.voxelizer.seed_particles(sample_density, self.grid_size, self.padding, t,
                                          self._seed * 1000003 + self._mesh_seed)
        if x.shape[0] == 0:
            return
        self._note_region(*self._finite_bounds(x))
        self._append(x, material, color, self.source_velocity, emitter_id=emmiter_id)

    def add_ngon(self, *args, **kwargs):
        raise ValueError("Add Ngon only works for 2D simulations")

    def add_texture_2d(self, *args, **kwargs):
        raise NotImplementedError("2-D texture seeding is not part of the 3-D GB300 engine")

    def clear_particles(self):
        """engine/mpm_solver.py:1193-1196."""
        self.n_particles = 0
        self._binned = 0
        self._ws = None
        self._host_box = None

    # ------------------------------------------------------------- step ---

    def _check_window_covers_particles(self, frame_dt: float):
        """Grow the grid window if particles got close to its edge.  The
        particles' bounding box comes from the last frame's readback when it
        is known (G2P reduces it on the device), else from a reduction here."""
        if self.n_particles == 0:
            return
        if self._host_box is not None:
            mn, mx = self._host_box
        else:
            mn, mx = self._finite_bounds(self._positions_f32())
        reach = (max(self.all_time_max_velocity, 1.0) * frame_dt * 2.0)
        self._cover([a - reach for a in mn], [b + reach for b in mx])
        if self._ws is None:
            self._rebin()

    def _frame_readback(self, count: int):
        """The one synchronisation of a frame: copies the per-substep max |v|
        and the workspace counters (status word, the particles' bounding box
        after the last substep) into page-locked buffers, raises on a device
        status, and returns the max |v| per substep."""
        if self._readback is None or self._readback[0].numel() < count:
            self._readback = (torch.empty(max(count, 64), dtype=torch.float32, pin_memory=True),
                              torch.empty(32, dtype=torch.int32, pin_memory=True))
        hv, hc = self._readback
        hv[:count].copy_(self._maxv[:count], non_blocking=True)
        hc.copy_(self._ws[:128].view(torch.int32), non_blocking=True)
        torch.cuda.current_stream(self.device).synchronize()
        maxv = hv[:count].numpy().copy()
        c = hc.numpy()
        self._raise_status(int(c[3]))
        keys = c[16:22].astype(np.int32)
        bits = np.where(keys >= 0, keys, keys ^ np.int32(0x7FFFFFFF)).astype(np.int32)
        box = bits.view(np.float32).astype(np.float64)
        if np.all(np.isfinite(box)) and np.all(box[:3] <= box[3:]):
            self._host_box = (box[:3].tolist(), box[3:].tolist())
        else:
            self._host_box = None
        return maxv

    def _check_status(self):
        self._raise_status(int(self._status.item()))

    def _raise_status(self, st: int):
        if st:
            self._status.zero_()
            msgs = []
            if st & _lib.STATUS_OUT_OF_GRID:
                msgs.append("particles left the grid window (their stencils were clamped)")
            if st & _lib.STATUS_NONFINITE:
                msgs.append("non-finite particle positions")
            if st & _lib.STATUS_TABLE_OVERFLOW:
                msgs.append("binning tables inconsistent (stale particle binning)")
            if st & _lib.STATUS_TIMEOUT:
                msgs.append("a kernel gave up waiting for staged particle data")
            raise MPMError("MPM device status: " + "; ".join(msgs))

    def _launch_substep(self, dt: float, maxv_slot: int):
        p = self.params
        cur = self._state[self._cur]
        nxt = self._state[1 - self._cur]
        mv = _ptr(self._maxv) + 4 * maxv_slot if maxv_slot >= 0 else None
        if profiler.kernel_profiler:
            e0, e1 = profiler.substep_events()
            e0.record(torch.cuda.current_stream(self.device))
            self._launch_substep_call(dt, p, cur, nxt, mv)
            e1.record(torch.cuda.current_stream(self.device))
            name = "mpm_g2p2g_substep" if self.use_g2p2g else ("mpm_substep (quant)" if self.quant else "mpm_substep")
            profiler.add_call(name, e0, e1)
        else:
            self._launch_substep_call(dt, p, cur, nxt, mv)

    def _launch_substep_call(self, dt, p, cur, nxt, mv):
        if self.use_g2p2g:
            first_new = self._last_final if self._g2p2g_grid_valid else 0
            _lib.check(
                self._lib.mpm_g2p2g_substep(ctypes.byref(p), _ptr(self._ws), self._cap, self.n_particles, _ptr(cur),
                                            _ptr(nxt), float(dt), first_new, 0 if self._g2p2g_listed else 1, mv,
                                            self.stream), "mpm_g2p2g_substep")
            self._cur = 1 - self._cur
            self._g2p2g_listed = self.n_particles
            self._binned = 0
            self._last_final = self.n_particles
            self._g2p2g_grid_valid = True
            return
        _lib.check(
            self._lib.mpm_substep(ctypes.byref(p), _ptr(self._ws), self._cap, self.n_particles, _ptr(cur), _ptr(nxt),
                                  float(dt), mv, self.stream), "mpm_substep")
        self._cur = 1 - self._cur

    def _prepare(self, frame_dt: float = 0.0):
        if self.n_particles == 0 and self._cap == 0:
            return  # nothing to step and no buffers yet (the reference steps empty solvers)
        self._ensure_workspace()
        self._rebin()
        self._check_window_covers_particles(frame_dt)
        self._ensure_workspace()
        self._rebin()

    def substep(self, dt: float):
        """One substep (engine/mpm_solver.py:789-797) with time step dt."""
        self._prepare(dt)
        self._host_box = None  # positions move without a readback
        if self.n_particles == 0:
            self.t += dt
            return
        self._maxv[:1].zero_()
        self._launch_substep(dt, 0)
        self.t += dt
        self.total_substeps += 1

    @staticmethod
    def count_substeps(frame_dt: float, default_dt: float):
        """Substep count and dt of engine/mpm_solver.py:752-771 (including the
        float64 loop that can run one more substep than `substeps`)."""
        substeps = int(frame_dt / default_dt) + 1
        dt = frame_dt / substeps
        frame_time_left = frame_dt
        count = 0
        while frame_time_left > 0:
            count += 1
            frame_time_left -= dt
        return count, dt

    @property
    def _fuses_frames(self) -> bool:
        """Frames run as fused substeps (mpm_frame for the reference's plain
        loop, mpm_g2p2g_frame for use_g2p2g): float32 storage only."""
        return self.fuse_frames and not self.quant

    def _launch_frame(self, count: int, dt: float):
        """All substeps of a frame, re-sorted every `resort_every` substeps:
        the plain loop fused (G2P of one substep with P2G of the next), or
        the G2P2G mode's substeps."""
        p = self.params
        in_b = ctypes.c_int32(0)
        evs, arr = profiler.frame_events(count, self.device) if profiler.kernel_profiler else (None, None)
        if self.use_g2p2g:
            if self._g2p2g_listed:  # per-substep calls left finalized lists: count afresh
                _lib.check(self._lib.mpm_bin_count(ctypes.byref(p), _ptr(self._ws), self._cap,
                                                   _ptr(self._state[self._cur]), 0, self.n_particles, self.stream),
                           "mpm_bin_count")
            first_new = self._last_final if self._g2p2g_grid_valid else 0
            _lib.check(
                self._lib.mpm_g2p2g_frame(ctypes.byref(p), _ptr(self._ws), self._cap, self.n_particles,
                                          _ptr(self._state[self._cur]), _ptr(self._state[1 - self._cur]), float(dt),
                                          int(count), int(self._frame_resort(count)), int(first_new),
                                          _ptr(self._maxv), ctypes.byref(in_b), arr, self.stream), "mpm_g2p2g_frame")
            # the state is binned (counts) for the next frame or substep
            self._g2p2g_listed = 0
            self._binned = self.n_particles
            self._last_final = self.n_particles
            self._g2p2g_grid_valid = True
        else:
            _lib.check(
                self._lib.mpm_frame(ctypes.byref(p), _ptr(self._ws), self._cap, self.n_particles,
                                    _ptr(self._state[self._cur]), _ptr(self._state[1 - self._cur]), float(dt),
                                    int(count), int(self._frame_resort(count)), _ptr(self._maxv), ctypes.byref(in_b), arr,
                                    self.stream), "mpm_frame")
        self._cur = (self._cur + int(in_b.value)) % 2
        if evs is not None:
            profiler.add_frame(count, evs, self._frame_resort(count), g2p2g=self.use_g2p2g)

    def _frame_resort(self, count: int) -> int:
        """The re-sort interval of a fused frame of `count` substeps: the
        number of sorts closest to count / resort_every (at least one),
        spread evenly over the frame."""
        return frame_resort_interval(count, self.resort_every)

    def _frame_swaps(self, count: int) -> int:
        """Buffer swaps of a fused frame: one per sort."""
        r = self._frame_resort(count)
        return (count + r - 1) // r

    def _launch_substeps(self, count: int, dt: float):
        self._maxv[:count].zero_()
        if self._fuses_frames:
            self._launch_frame(count, dt)
        else:
            for s in range(count):
                self._launch_substep(dt, s)

    def _run_frame(self, count: int, dt: float):
        """Run `count` substeps, through a CUDA graph when enabled."""
        if count > self._maxv.numel():
            self._maxv = torch.zeros(count, dtype=torch.float32, device=self.device)
        key = (count, float(dt), self._cur, self.n_particles, self._params_version, _ptr(self._ws),
               self._fuses_frames, self.resort_every)
        if self.use_g2p2g:  # the first substep's launch depends on the mode's state
            key += (bool(self._g2p2g_listed), self._last_final if self._g2p2g_grid_valid else 0)
        if not self.use_cuda_graph or profiler.kernel_profiler:  # events need the launches themselves
            self._launch_substeps(count, dt)
            return
        g = self._graphs.get(key)
        if g is None and key in self._graph_seen:
            start_cur = self._cur
            g = capture_graph(self.device, lambda: self._launch_substeps(count, dt))
            self._cur = start_cur  # capture does not execute
            self._graphs[key] = g
        if g is not None:
            g.replay()
            swaps = self._frame_swaps(count) if self._fuses_frames else count
            self._cur = (self._cur + swaps) % 2
            return
        self._graph_seen.add(key)
        self._launch_substeps(count, dt)

    def step(self, frame_dt, print_stat=False, smry_writer=None):
        """engine/mpm_solver.py:748-821."""
        begin_t = time.time()
        begin_substep = self.total_substeps
        count, dt = self.count_substeps(frame_dt, self.default_dt)
        if print_stat:
            print(f'needed substeps: {int(frame_dt / self.default_dt) + 1}')
        self._prepare(frame_dt)
        if self.autotune and not self._tuned and self.n_particles > 0:
            from .autotune import tune_schedule
            tune_schedule(self)
            self._tuned = True
        if self.use_adaptive_dt:
            self._host_box = None
            dts = self._adaptive_frame(frame_dt, dt)
            count = len(dts)
            maxv = self._maxv[:count].cpu().numpy() if self.n_particles > 0 else np.zeros(count, np.float32)
            if self.n_particles > 0:
                self._check_status()
        elif self.n_particles > 0:
            self._run_frame(count, dt)
            if self.use_g2p2g and not self._fuses_frames:  # k_g2p2g reduces no bounding box
                maxv = self._maxv[:count].cpu().numpy()
                self._check_status()
                self._host_box = None
            else:
                maxv = self._frame_readback(count)
            dts = [dt] * count
        else:
            maxv = np.zeros(count, dtype=np.float32)
            dts = [dt] * count
        if profiler.kernel_profiler:
            profiler.collect(sync=False)  # the frame's readback synchronised the stream
        for s in range(count):
            self.total_substeps += 1
            self.t += dts[s]
            if smry_writer is not None:
                smry_writer.add_scalar("substep_max_CFL", float(maxv[s]) * dts[s] / self.dx, self.total_substeps)
        dt = dts[-1] if dts else dt
        if count:
            self.all_time_max_velocity = max(self.all_time_max_velocity, float(maxv.max()))
        if print_stat:
            profiler.print_kernel_profiler_info()
            profiler.print_memory_profiler_info(self)
            cur_frame_velocity = float(maxv[-1]) if count else 0.0
            print(f'CFL: {cur_frame_velocity * dt / self.dx}')
            print(f'num particles={self.n_particles}')
            print(f'  frame time {time.time() - begin_t:.3f} s')
            print(f'  substep time {1000 * (time.time() - begin_t) / max(1, self.total_substeps - begin_substep):.3f} ms')

    def memory_report(self) -> list:
        """(name, bytes) of the device buffers this solver holds."""
        rows = []
        if self._state[0] is not None:
            r, cap = self._state[0].shape
            rows.append((f"particle state: 2 buffers x {r} rows x {cap} slots (float32"
                         f"{', packed' if self.quant else ''})", 2 * self._state[0].numel() * 4))
            rows.append(("particle colours and emitter ids", (self._color.numel() + self._emitter.numel()) * 4))
        if self._ws is not None:
            rows.append(("workspace: grid momentum / velocity window, block flags and lists, cell counters, "
                         "sort tables, status", self._ws.numel()))
        rows.append(("max |v| per substep", self._maxv.numel() * 4))
        return rows

    def compute_max_velocity(self) -> float:
        """engine/mpm_solver.py:726-735: the largest velocity component
        magnitude max_p max_d |v_pd| over the particles (0 without any)."""
        n = self.n_particles
        if n == 0:
            return 0.0
        return float(self._rows_f32()[ROW_V:ROW_V + 3, :n].abs().max().item())

    def compute_max_grid_velocity(self, grid_v=None) -> float:
        """engine/mpm_solver.py:737-746: the largest velocity component
        magnitude over the grid nodes of the last substep (0 before the
        first).  `grid_v` names the reference's grid field; the engine has
        one grid, so the argument is accepted and not used."""
        return self._max_grid_velocity()

    def _max_grid_velocity(self) -> float:
        """compute_max_grid_velocity (engine/mpm_solver.py:737-746) of the
        last substep's grid (0 before the first)."""
        if self._ws is None:
            return 0.0
        out = torch.zeros(1, dtype=torch.float32, device=self.device)
        p = self.params
        _lib.check(self._lib.mpm_max_grid_velocity(ctypes.byref(p), _ptr(self._ws), self._cap, _ptr(out),
                                                   self.stream), "mpm_max_grid_velocity")
        return float(out.item())

    def _adaptive_frame(self, frame_dt: float, dt: float):
        """The adaptive substep loop of engine/mpm_solver.py:756-766: before
        each substep dt = min(dt, allowed_cfl * dx / (max grid |v| + 1e-6),
        time left); one host round trip per substep, no CUDA graph."""
        dts = []
        frame_time_left = frame_dt
        if frame_dt / self.default_dt + 2 > self._maxv.numel():
            self._maxv = torch.zeros(int(frame_dt / self.default_dt) + 1024, dtype=torch.float32,
                                     device=self.device)
        self._maxv.zero_()
        while frame_time_left > 0:
            max_grid_v = self._max_grid_velocity()
            cfl_dt = self.g2p2g_allowed_cfl * self.dx / (max_grid_v + 1e-6)
            dt = min(dt, cfl_dt, frame_time_left)
            frame_time_left -= dt
            if len(dts) >= self._maxv.numel():  # a collapsing dt: grow the per-substep record
                self._maxv = torch.cat([self._maxv, torch.zeros_like(self._maxv)])
            if self.n_particles > 0:
                self._launch_substep(dt, len(dts))
            dts.append(dt)
        self.last_frame_dts = dts
        return dts

    # --------------------------------------------------------- readback ---

    def _rows_f32(self) -> torch.Tensor:
        """The current particle state in the float32 row layout (slot order):
        the state buffer itself, or with quant=True a decoded copy."""
        st = self._state[self._cur]
        if not self.quant:
            return st
        n = self.n_particles
        out = torch.empty((NROWS, max(n, 1)), dtype=torch.float32, device=self.device)
        _lib.check(self._lib.mpm_quant_unpack(_ptr(st), self._cap, 0, n, _ptr(out), out.shape[1], self.stream),
                   "mpm_quant_unpack")
        return out

    def _positions_f32(self) -> torch.Tensor:
        """Positions (3, n) as float32 in slot order; with quant=True decoded
        from the packed word pair (three 21-bit fields of scale 2^-19) by
        torch integer ops, without decoding the other rows."""
        n = self.n_particles
        st = self._state[self._cur]
        if not self.quant:
            return st[ROW_X:ROW_X + 3, :n].t()
        w = st[0:2, :n].view(torch.int32).to(torch.int64) & 0xFFFFFFFF
        w = w[0] | (w[1] << 32)
        out = torch.empty((n, 3), dtype=torch.float32, device=self.device)
        for d in range(3):
            q = (w >> (21 * d)) & 0x1FFFFF
            q = q - ((q >> 20) << 21)  # sign-extend 21 bits
            out[:, d] = q.to(torch.float32) * (1.0 / 524288.0)
        return out

    def _gather(self, row0: int, ncols: int, rows: torch.Tensor | None = None) -> torch.Tensor:
        n = self.n_particles
        out = torch.empty((n, ncols), dtype=torch.float32, device=self.device)
        if n:
            rows = self._rows_f32() if rows is None else rows
            _lib.check(
                self._lib.mpm_gather_rows(_ptr(rows), rows.shape[1], n, row0, ncols, _ptr(out),
                                          self.stream), "mpm_gather_rows")
        return out

    def particle_info(self):
        """engine/mpm_solver.py:1172-1191: copies in original particle order.

        The arrays are gathered on the device and copied into page-locked
        host buffers with one synchronisation for all of them.  The buffers
        come from a process-wide pool (_pinned_buffer) and are handed out
        again only once nothing references the returned arrays (or a view of
        them), so a caller can keep them as the reference's fresh copies."""
        n = self.n_particles
        if n == 0:
            data = {'position': np.zeros((0, 3), np.float32), 'velocity': np.zeros((0, 3), np.float32),
                    'material': np.zeros(0, np.int32), 'color': np.zeros(0, np.int32)}
            if self.use_emitter_id:
                data['emitter_ids'] = np.zeros(0, np.int32)
            return data
        # the copies run on a side stream, each behind its own gather, so the
        # copy engine works while the next field is gathered; the resident
        # fields go first
        main = torch.cuda.current_stream(self.device)
        if self._copy_stream is None:
            self._copy_stream = torch.cuda.Stream(device=self.device)
        side = self._copy_stream
        side.wait_stream(main)
        host = {}

        def copy(name, t):
            h, hn = _pinned_buffer(t.shape, t.dtype)
            t.record_stream(side)
            with torch.cuda.stream(side):
                h.copy_(t, non_blocking=True)
            host[name] = hn

        copy('color', self._color[:n])
        if self.use_emitter_id:
            copy('emitter_ids', self._emitter[:n])
        rows = self._rows_f32()
        for name, gather in (('position', lambda: self._gather(ROW_X, 3, rows)),
                             ('velocity', lambda: self._gather(ROW_V, 3, rows)),
                             ('material', lambda: self._gather(ROW_MAT, 1, rows).view(torch.int32).reshape(n) & 0xFF)):
            t = gather()
            side.wait_stream(main)
            copy(name, t)
        side.synchronize()
        keys = ['position', 'velocity', 'material', 'color'] + (['emitter_ids'] if self.use_emitter_id else [])
        return {k: host[k] for k in keys}

    def _to_host(self, *tensors):
        """numpy copies of device tensors through page-locked buffers, one
        synchronisation for all.  The buffers come from a process-wide pool
        (_pinned_buffer): pinning fresh host memory costs about 13 GB/s, a
        copy into pinned memory ~180 GB/s on GB300."""
        host = []
        for t in tensors:
            h, hn = _pinned_buffer(t.shape, t.dtype)
            h.copy_(t, non_blocking=True)
            host.append(hn)
        torch.cuda.current_stream(self.device).synchronize()
        return host

    def full_state(self):
        """All particle fields in original order as float32 device tensors:
        x (n,3), v (n,3), C (n,3,3), F (n,3,3), Jp (n,), material (n,) int32."""
        n = self.n_particles
        g = self._gather(0, ROW_ID)
        return {
            'x': g[:, ROW_X:ROW_X + 3],
            'v': g[:, ROW_V:ROW_V + 3],
            'C': g[:, ROW_C:ROW_C + 9].reshape(n, 3, 3),
            'F': g[:, ROW_F:ROW_F + 9].reshape(n, 3, 3),
            'Jp': g[:, ROW_JP],
            'material': g[:, ROW_MAT].contiguous().view(torch.int32) & 0xFF,
        }

    def state_dict(self):
        st = {k: v.clone() for k, v in self.full_state().items()}
        st['color'] = self._color[:self.n_particles].clone()
        st['t'] = self.t
        st['total_substeps'] = self.total_substeps
        return st

    def load_state_dict(self, st):
        """Replace all particles by an exact checkpoint from state_dict()."""
        self.clear_particles()
        x = st['x'].to(self.device, torch.float32)
        n = int(x.shape[0])
        lo = x.min(0).values.tolist() if n else [0, 0, 0]
        hi = x.max(0).values.tolist() if n else [0, 0, 0]
        if n:
            self._note_region(lo, hi)
            self._append(x, st['material'], st['color'], st['v'], C=st['C'], F=st['F'], Jp=st['Jp'])
        self.t = st.get('t', 0.0)
        self.total_substeps = st.get('total_substeps', 0)

    def tensors(self):
        """Zero-copy views of the current (sorted) particle state rows; with
        quant=True, views of a decoded float32 copy."""
        n = self.n_particles
        s = self._rows_f32()
        return {
            'x': s[ROW_X:ROW_X + 3, :n],
            'v': s[ROW_V:ROW_V + 3, :n],
            'C': s[ROW_C:ROW_C + 9, :n],
            'F': s[ROW_F:ROW_F + 9, :n],
            'Jp': s[ROW_JP, :n],
            'material': s.view(torch.int32)[ROW_MAT, :n],
            'id': s.view(torch.int32)[ROW_ID, :n],
        }

    def views(self):
        """Device views of the engine's binning and grid arrays (diagnostics
        and parity tests): counters, particle-block and grid-block lists (as
        window-linear block indices), per-particle-block counts and starts, the
        sorted order, cell keys, and the momentum / velocity grids as (nodes, 4)
        float32 in window block-major order."""
        self._ensure_workspace()
        p = self.params
        v = _lib.MpmViews()
        _lib.check(self._lib.mpm_views(ctypes.byref(p), _ptr(self._ws), self._cap, ctypes.byref(v)), "mpm_views")
        base = _ptr(self._ws)
        nb = self._window[1]
        nblk = nb[0] * nb[1] * nb[2]

        def sl(addr, count, dtype, width=1):
            off = addr - base
            t = self._ws[off:off + count * width * 4].view(dtype)
            return t.view(count, width) if width > 1 else t

        return {
            'counters': sl(v.counters, 32, torch.int32),
            'pblocks': sl(v.pblocks, nblk, torch.int32),
            'gblocks': sl(v.gblocks, nblk, torch.int32),
            'pblock_count': sl(v.pblock_count, nblk, torch.int32),
            'pblock_start': sl(v.pblock_start, nblk, torch.int32),
            'pid': sl(v.pid, self._cap, torch.int32),
            'cellkey': sl(v.cellkey, self._cap, torch.int32),
            'grid_mom': sl(v.grid_mom, nblk * 64, torch.float32, 4),
            'grid_vel': sl(v.grid_vel, nblk * 64, torch.float32, 4),
            'win_lo': list(self._window[0]),
            'win_nb': list(nb),
        }

    def write_particles(self, fn, slice_size=1000000):
        """engine/mpm_solver.py:1198-1200: the quantised .npz frame of
        engine/particle_io.py, quantised on the GPU."""
        from .particle_io import ParticleIO
        ParticleIO.write_particles(self, fn, slice_size)

    def write_particles_ply(self, fn):
        """engine/mpm_solver.py:1202-1209: positions and colours as a
        binary point-cloud .ply."""
        from .particle_io import write_particles_ply
        write_particles_ply(self, fn)
