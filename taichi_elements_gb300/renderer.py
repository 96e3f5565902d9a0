"""Particle path tracer on the GPU: taichi-dev/taichi_elements engine/renderer.py.

``Renderer`` keeps the reference's constructor arguments, camera controls
(``set_camera_pos``, ``look_at[None]``, ``set_up``, ``set_fov``,
``floor_height[None]``), ``initialize_particles_from_taichi_elements``
(reads a quantised frame), ``total_non_empty_voxels``,
``total_inserted_particles``, ``reset`` and ``render_frame(spp)`` returning
the (res[0], res[1], 3) float32 image; the work runs in the kernels of
csrc/mpm_render.cu.  ``initialize_particles_from_solver`` renders a running
MPMSolver's particles straight from device memory.  ``render_voxel=True``
draws the occupied cells as cubes (the reference's voxel view).
"""
from __future__ import annotations

import ctypes
import math
import struct
import zlib

import numpy as np
import torch

from . import _lib
from ._lib import ROW_V, ROW_X

RES = (1280, 720)  # engine/renderer.py:10
SHUTTER_BEGIN = -0.5  # :18
EXPOSURE = 1.5  # :20
LIGHT_DIRECTION = (1.2, 0.3, 0.7)  # :21
LIGHT_DIRECTION_NOISE = 0.03  # :22
LIGHT_COLOR = (1.0, 1.0, 1.0)  # :23


class RenderScene(ctypes.Structure):
    """Mirror of the C RenderScene (csrc/mpm_render.cu)."""
    _fields_ = [
        ("c0", ctypes.c_int32 * 3), ("nc", ctypes.c_int32 * 3),
        ("dx", ctypes.c_float), ("inv_dx", ctypes.c_float), ("radius", ctypes.c_float),
        ("bbox_min", ctypes.c_float * 3), ("bbox_max", ctypes.c_float * 3),
        ("shutter_begin", ctypes.c_float), ("shutter_time", ctypes.c_float), ("motion_blur", ctypes.c_int32),
        ("cam", ctypes.c_float * 3), ("look_at", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
        ("fov", ctypes.c_float), ("res", ctypes.c_int32 * 2), ("floor_height", ctypes.c_float),
        ("taichi_logo", ctypes.c_int32), ("light_dir", ctypes.c_float * 3), ("light_noise", ctypes.c_float),
        ("light_color", ctypes.c_float * 3), ("render_voxel", ctypes.c_int32), ("pad_", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
    ]


class _Field:
    """A Taichi 0-d field stand-in: ``f[None]`` reads and writes the value."""

    def __init__(self, value):
        self.value = value

    def __getitem__(self, key):
        return self.value

    def __setitem__(self, key, value):
        self.value = value


def _normalized(v):
    v = np.asarray(v, np.float32)
    return v / np.float32(np.sqrt(np.float32((v * v).sum())))


class Renderer:

    def __init__(self, dx=1 / 1024, sphere_radius=0.3 / 1024, render_voxel=False, shutter_time=1e-3, taichi_logo=True,
                 max_num_particles_million=128, res=RES, seed=0, device=None):
        assert sphere_radius * 2 < dx
        self.device = torch.device(device if device is not None else "cuda")
        self._lib = _lib.load()
        assert self._lib.mpm_render_scene_bytes() == ctypes.sizeof(RenderScene)
        self.res = (int(res[0]), int(res[1]))
        self.vignette_strength = 0.9
        self.vignette_radius = 0.0
        self.vignette_center = [0.5, 0.5]
        self.taichi_logo = taichi_logo
        self.render_voxel = bool(render_voxel)
        self.voxel_edges = 0.1
        self.shutter_time = shutter_time
        self.enable_motion_blur = self.shutter_time != 0.0
        self.dx = dx
        self.inv_dx = 1 / self.dx
        self.sphere_radius = sphere_radius
        self.max_num_particles = 1024 * 1024 * max_num_particles_million
        self.seed = int(seed)
        self.camera_pos = _Field((0.0, 0.0, 0.0))
        self.look_at = _Field((0.0, 0.0, 0.0))
        self.up = _Field((0.0, 1.0, 0.0))
        self.fov = _Field(0.23)
        self.floor_height = _Field(0.0)
        self.bbox = np.zeros((2, 3), np.float32)
        self.color_buffer = torch.zeros((self.res[0], self.res[1], 3), dtype=torch.float32, device=self.device)
        self.num_particles = 0
        self._samples = 0
        self._x = self._v = self._rgb = None
        self._start = self._count = self._list = self._occ = None
        self._cells = None
        self.set_up(0, 1, 0)
        self.set_fov(0.23)

    # --------------------------------------------------- camera controls --

    @property
    def stream(self) -> int:
        return torch.cuda.current_stream(self.device).cuda_stream

    def set_camera_pos(self, x, y, z):
        self.camera_pos[None] = (float(x), float(y), float(z))

    def set_up(self, x, y, z):
        self.up[None] = tuple(float(c) for c in _normalized((x, y, z)))

    def set_fov(self, fov):
        self.fov[None] = float(fov)

    # ---------------------------------------------------------- particles --

    def reset(self):
        self._x = self._v = self._rgb = None
        self._start = self._count = self._list = self._occ = None
        self.num_particles = 0
        self.color_buffer.zero_()
        self._samples = 0

    def _scene(self) -> RenderScene:
        s = RenderScene()
        c0, nc = self._cells
        for i in range(3):
            s.c0[i], s.nc[i] = c0[i], nc[i]
            s.bbox_min[i], s.bbox_max[i] = float(self.bbox[0, i]), float(self.bbox[1, i])
            s.cam[i] = self.camera_pos[None][i]
            s.look_at[i] = self.look_at[None][i]
            s.up[i] = self.up[None][i]
            s.light_dir[i] = LIGHT_DIRECTION[i]
            s.light_color[i] = LIGHT_COLOR[i]
        s.dx, s.inv_dx, s.radius = self.dx, self.inv_dx, self.sphere_radius
        s.shutter_begin, s.shutter_time = SHUTTER_BEGIN, self.shutter_time
        s.motion_blur = int(self.enable_motion_blur)
        s.fov = self.fov[None]
        s.res[0], s.res[1] = self.res
        s.floor_height = float(self.floor_height[None])
        s.taichi_logo = int(bool(self.taichi_logo))
        s.light_noise = LIGHT_DIRECTION_NOISE
        s.render_voxel = int(self.render_voxel)
        s.seed = self.seed
        return s

    def initialize_particles(self, x, v, color):
        """Particles x, v (n, 3) and colour (n, 3) uint8, as arrays or device
        tensors: bounding box (renderer.py:580-588) and cell lists
        (initialize_particle_grid, :482-517)."""
        self.reset()
        x = torch.as_tensor(x, dtype=torch.float32).to(self.device).contiguous()
        v = torch.as_tensor(v, dtype=torch.float32).to(self.device).contiguous()
        rgb = torch.as_tensor(color).to(self.device, torch.uint8).contiguous()
        n = int(x.shape[0])
        assert n <= self.max_num_particles
        mn = x.min(0).values.cpu().numpy()
        mx = x.max(0).values.cpu().numpy()
        c0, c1 = [], []
        for i in range(3):
            # bbox values are multiples of dx, 3 cells beyond the particles
            lo = math.floor(float(mn[i]) * self.inv_dx) - 3
            hi = math.floor(float(mx[i]) * self.inv_dx) + 3
            self.bbox[0, i] = lo * self.dx
            self.bbox[1, i] = hi * self.dx
            c0.append(lo)
            c1.append(hi + 1)
        self._cells = (c0, [b - a for a, b in zip(c0, c1)])
        ncell = int(np.prod(self._cells[1], dtype=np.int64))
        self._x, self._v, self._rgb = x, (v if self.enable_motion_blur else None), rgb
        self.num_particles = n
        scene = self._scene()
        count = torch.zeros(ncell, dtype=torch.int32, device=self.device)
        vp = self._v.data_ptr() if self._v is not None else None
        _lib.check(self._lib.mpm_render_cell_count(ctypes.byref(scene), x.data_ptr(), vp, n, count.data_ptr(),
                                                   self.stream), "mpm_render_cell_count")
        incl = torch.cumsum(count, 0, dtype=torch.int64)
        total = int(incl[-1].item())
        start = (incl - count).contiguous()
        fill = torch.zeros_like(count)
        lst = torch.empty(max(total, 1), dtype=torch.int32, device=self.device)
        _lib.check(self._lib.mpm_render_cell_fill(ctypes.byref(scene), x.data_ptr(), vp, n, start.data_ptr(),
                                                  fill.data_ptr(), total, lst.data_ptr(), self.stream),
                   "mpm_render_cell_fill")
        occ = torch.empty((ncell + 31) // 32, dtype=torch.int32, device=self.device)
        _lib.check(self._lib.mpm_render_occupancy(count.data_ptr(), ncell, occ.data_ptr(), self.stream),
                   "mpm_render_occupancy")
        self._start, self._count, self._list, self._occ = start, count, lst, occ

    def initialize_particles_from_taichi_elements(self, particle_fn):
        """renderer.py:574-601: a quantised frame written by write_particles."""
        from .particle_io import ParticleIO
        np_x, np_v, np_color = ParticleIO.read_particles_3d(particle_fn)
        self.initialize_particles(np_x, np_v, np_color)

    def initialize_particles_from_solver(self, solver):
        """The particles of a running MPMSolver, from device memory."""
        n = solver.n_particles
        rgb = torch.empty((n, 3), dtype=torch.uint8, device=solver.device)
        _lib.check(self._lib.mpm_unpack_colors(solver._color.data_ptr(), n, rgb.data_ptr(), solver.stream),
                   "mpm_unpack_colors")
        self.initialize_particles(solver._gather(ROW_X, 3), solver._gather(ROW_V, 3), rgb)

    def total_non_empty_voxels(self) -> int:
        return int((self._count > 0).sum().item()) if self._count is not None else 0

    def total_inserted_particles(self) -> int:
        return int(self._count.sum().item()) if self._count is not None else 0

    # ---------------------------------------------------------- rendering --

    def render(self, spp: int = 1):
        """Add `spp` samples of every pixel to the colour buffer
        (renderer.py:396-480)."""
        if self._count is None:
            raise RuntimeError("no particles: call initialize_particles* first")
        scene = self._scene()
        vp = self._v.data_ptr() if self._v is not None else None
        _lib.check(self._lib.mpm_render_samples(ctypes.byref(scene), self._occ.data_ptr(), self._start.data_ptr(),
                                                self._count.data_ptr(),
                                                self._list.data_ptr(), self._x.data_ptr(), vp, self._rgb.data_ptr(),
                                                self._samples, int(spp), self.color_buffer.data_ptr(), self.stream),
                   "mpm_render_samples")
        self._samples += int(spp)

    def copy(self, samples: int) -> np.ndarray:
        """renderer.py:519-531: the displayed image for `samples` samples."""
        img = torch.empty_like(self.color_buffer)
        _lib.check(self._lib.mpm_render_tonemap(self.res[0], self.res[1], self.color_buffer.data_ptr(),
                                                self.vignette_strength, self.vignette_radius,
                                                self.vignette_center[0], self.vignette_center[1], EXPOSURE,
                                                int(samples), img.data_ptr(), self.stream), "mpm_render_tonemap")
        return img.cpu().numpy()

    def render_frame(self, spp, batch: int = 8):
        """renderer.py:603-619: `spp` samples, then the tone-mapped image
        (res[0], res[1], 3) float32."""
        done = 0
        while done < spp:
            k = min(batch, spp - done)
            self.render(k)
            done += k
        return self.copy(spp)

    def first_hits(self, orig, dirs, t=0.0) -> np.ndarray:
        """Nearest hits (distance, normal xyz, colour rgb) of given rays, no
        randomness (renderer.py:368-386)."""
        o = torch.as_tensor(np.asarray(orig, np.float32)).to(self.device).contiguous()
        d = torch.as_tensor(np.asarray(dirs, np.float32)).to(self.device).contiguous()
        out = torch.empty((o.shape[0], 7), dtype=torch.float32, device=self.device)
        scene = self._scene()
        vp = self._v.data_ptr() if self._v is not None else None
        _lib.check(self._lib.mpm_render_first_hits(ctypes.byref(scene), self._occ.data_ptr(), self._start.data_ptr(),
                                                   self._count.data_ptr(),
                                                   self._list.data_ptr(), self._x.data_ptr(), vp, self._rgb.data_ptr(),
                                                   o.data_ptr(), d.data_ptr(), o.shape[0], float(t), out.data_ptr(),
                                                   self.stream), "mpm_render_first_hits")
        return out.cpu().numpy()


def write_png(img: np.ndarray, fn: str):
    """A (res[0], res[1], 3) image in the reference's layout (x right, y up,
    values in [0, 1]) as an 8-bit RGB PNG."""
    a = (np.clip(np.asarray(img, np.float32), 0.0, 1.0) * 255.0 + 0.5).astype(np.uint8)
    rows = a.transpose(1, 0, 2)[::-1]
    h, w = rows.shape[0], rows.shape[1]
    raw = b"".join(b"\x00" + rows[r].tobytes() for r in range(h))

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)

    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
    with open(fn, "wb") as f:
        f.write(png)
