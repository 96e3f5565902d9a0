"""Particle frame output in the reference's formats, computed on the GPU.

``ParticleIO`` mirrors taichi-dev/taichi_elements engine/particle_io.py: the
quantised ``.npz`` frame (``write_particles``, :12-76) with keys ``ranges``
(2, 3, 2) float32, ``x_and_v`` (n, 3) uint32 = (24-bit x << 8) + 8-bit v and
``color`` (n, 3) uint8; its reader (:78-106); and the conversion to a
binary point-cloud ``.ply`` (:108-120, engine/mesh_io.py:26-44).

The ranges, the quantisation and the colour bytes are computed by the
kernels of csrc/mpm_io.cu on the solver's device state; only the packed
result (15 bytes per particle) crosses to the host.  Reading a frame back is
host numpy work, as in the reference.
"""
from __future__ import annotations

import gc
import time

import numpy as np
import torch

from . import _lib
from ._lib import ROW_X


class ParticleIO:
    v_bits = 8
    x_bits = 32 - v_bits

    @staticmethod
    def quantize(solver):
        """(ranges, x_and_v, color) of the solver's particles as numpy
        arrays, original particle order (the arrays write_particles saves)."""
        n = solver.n_particles
        if n == 0:
            raise ValueError("no particles to write")
        lib, dev, s = solver._lib, solver.device, solver.stream
        st = solver._rows_f32()
        keys = torch.empty(12, dtype=torch.int32, device=dev)
        ranges = torch.empty(12, dtype=torch.float32, device=dev)
        xv = torch.empty((n, 3), dtype=torch.int32, device=dev)
        rgb = torch.empty((n, 3), dtype=torch.uint8, device=dev)
        _lib.check(lib.mpm_particle_ranges(st.data_ptr(), st.shape[1], n, keys.data_ptr(), ranges.data_ptr(), s),
                   "mpm_particle_ranges")
        _lib.check(lib.mpm_quantize_particles(st.data_ptr(), st.shape[1], n, ranges.data_ptr(), xv.data_ptr(), s),
                   "mpm_quantize_particles")
        _lib.check(lib.mpm_unpack_colors(solver._color.data_ptr(), n, rgb.data_ptr(), s), "mpm_unpack_colors")
        ranges_h, xv_h, rgb_h = solver._to_host(ranges, xv, rgb)
        return ranges_h.reshape(2, 3, 2), xv_h.view(np.uint32), rgb_h

    @staticmethod
    def write_particles(solver, fn, slice_size=1000000):
        """engine/particle_io.py:12-76.  `slice_size` is accepted for the
        reference's signature; the device computes the frame in one pass."""
        t = time.time()
        ranges, x_and_v, color = ParticleIO.quantize(solver)
        np.savez(fn, ranges=ranges, x_and_v=x_and_v, color=color)
        print(f'Writing to disk: {time.time() - t:.3f} s')

    @staticmethod
    def read_particles_3d(fn):
        return ParticleIO.read_particles(fn, 3)

    @staticmethod
    def read_particles_2d(fn):
        return ParticleIO.read_particles(fn, 2)

    @staticmethod
    def read_particles(fn, dim):
        """engine/particle_io.py:86-106."""
        data = np.load(fn)
        ranges = data['ranges']
        color = data['color']
        x_and_v = data['x_and_v']
        del data
        gc.collect()
        x = (x_and_v >> ParticleIO.v_bits).astype(np.float32) / ((2**ParticleIO.x_bits - 1))
        for c in range(dim):
            x[:, c] = x[:, c] * (ranges[0, c, 1] - ranges[0, c, 0]) + ranges[0, c, 0]
        v = (x_and_v & (2**ParticleIO.v_bits - 1)).astype(np.float32) / (2**ParticleIO.v_bits - 1)
        for c in range(dim):
            v[:, c] = v[:, c] * (ranges[1, c, 1] - ranges[1, c, 0]) + ranges[1, c, 0]
        return x, v, color

    @staticmethod
    def convert_particle_to_ply(fns):
        """engine/particle_io.py:108-120."""
        for fn in fns:
            print(f'Converting {fn}...')
            x, _, color = ParticleIO.read_particles_3d(fn)
            x = x.astype(np.float32)
            color = (color[:, 2].astype(np.uint32) << 16) + (color[:, 1].astype(np.uint32) << 8) + color[:, 0]
            color = color[:, None]
            pos_color = np.hstack([x, color.view(np.float32)])
            del x, color
            gc.collect()
            write_point_cloud(fn + ".ply", pos_color)


def write_point_cloud(fn, pos_and_color):
    """engine/mesh_io.py:26-44: binary little-endian PLY of (n, 4) float32
    rows (x, y, z, colour bits)."""
    num_particles = len(pos_and_color)
    with open(fn, 'wb') as f:
        header = f"""ply
format binary_little_endian 1.0
comment Created by taichi
element vertex {num_particles}
property float x
property float y
property float z
property uchar red
property uchar green
property uchar blue
property uchar placeholder
end_header
"""
        f.write(str.encode(header))
        f.write(pos_and_color.tobytes())


def write_particles_ply(solver, fn):
    """engine/mpm_solver.py:1202-1210: positions and raw colour bits of all
    particles as a point cloud (positions gathered to original order on the
    device)."""
    n = solver.n_particles
    np_x = solver._gather(ROW_X, 3).cpu().numpy()
    np_color = solver._color[:n].cpu().numpy().view(np.uint32)
    data = np.hstack([np_x, (np_color[:, None]).view(np.float32)])
    write_point_cloud(fn, data)
