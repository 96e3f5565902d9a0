"""Mesh voxelizer on the GPU: taichi-dev/taichi_elements engine/voxelizer.py.

``Voxelizer(res, dx, super_sample=2, precision="f64", padding=3)`` keeps the
reference's grid rule (each resolution rounded up to a power of two, times
``super_sample``; voxel size dx / super_sample, :16-35) and its signed
crossing count per voxel (``voxelize``, :128-144), computed by the kernels
of csrc/mpm_voxelize.cu into a dense int32 tensor ``voxels`` (rx, ry, rz).
``seed_particles`` is the emitter loop of MPMSolver.seed_from_voxels
(engine/mpm_solver.py:1017-1047) and returns the new positions on the
device.  Only the reference's default float64 precision is provided.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib


def _pow2(r: int) -> int:
    p = 1
    while p < r:
        p *= 2
    return p


class Voxelizer:

    def __init__(self, res, dx, super_sample=2, precision="f64", padding=3, device=None):
        assert len(res) == 3
        if precision not in ("f64", np.float64, "float64"):
            raise NotImplementedError("the GB300 voxelizer computes in float64 (the reference's default)")
        self.device = torch.device(device if device is not None else "cuda")
        self._lib = _lib.load()
        r = [_pow2(int(x)) for x in res]
        self.super_sample = int(super_sample)
        self.res = (r[0] * self.super_sample, r[1] * self.super_sample, r[2] * self.super_sample)
        self.dx = dx / super_sample
        self.inv_dx = 1 / self.dx
        self.padding = int(padding)
        self.voxels = None

    @property
    def stream(self) -> int:
        return torch.cuda.current_stream(self.device).cuda_stream

    def voxelize(self, triangles):
        """engine/voxelizer.py:128-144: triangles (n, 9) array-like, xyz of
        the three vertices; replaces the voxel grid."""
        tri = np.asarray(triangles)
        assert tri.ndim == 2 and tri.shape[1] == 9
        t = torch.as_tensor(np.ascontiguousarray(tri, dtype=np.float64)).to(self.device)
        if self.voxels is None:
            self.voxels = torch.empty(self.res, dtype=torch.int32, device=self.device)
        rx, ry, rz = self.res
        _lib.check(self._lib.mpm_voxelize(t.data_ptr() if t.numel() else None, t.shape[0], rx, ry, rz, self.dx,
                                          self.padding, self.voxels.data_ptr(), self.stream), "mpm_voxelize")
        return self.voxels

    def seed_particles(self, sample_density, grid_size, padding, translation, seed):
        """Positions (m, 3) float32 on the device of the particles that
        seed_from_voxels (engine/mpm_solver.py:1017-1047) emits."""
        rx, ry, rz = self.res
        cols = rx * ry
        counts = torch.empty(cols, dtype=torch.int32, device=self.device)
        _lib.check(self._lib.mpm_voxel_seed_count(self.voxels.data_ptr(), rx, ry, rz, int(sample_density),
                                                  self.super_sample, int(grid_size), int(padding), int(seed),
                                                  counts.data_ptr(), self.stream), "mpm_voxel_seed_count")
        incl = torch.cumsum(counts.to(torch.int64), 0)
        total = int(incl[-1].item()) if cols else 0
        offsets = (incl - counts.to(torch.int64)).contiguous()
        x = torch.empty((max(total, 1), 3), dtype=torch.float32, device=self.device)
        tr = [float(np.float32(v)) for v in translation]
        _lib.check(self._lib.mpm_voxel_seed_emit(self.voxels.data_ptr(), rx, ry, rz, int(sample_density),
                                                 self.super_sample, int(grid_size), int(padding), int(seed),
                                                 float(np.float32(self.dx)), tr[0], tr[1], tr[2],
                                                 offsets.data_ptr(), total, x.data_ptr(), self.stream),
                   "mpm_voxel_seed_emit")
        return x[:total]
