"""CPU restatement of the quantised particle frame format - TEST INFRASTRUCTURE.

Follows taichi-dev/taichi_elements engine/particle_io.py:
* ``write_arrays`` = ParticleIO.write_particles (:12-76) on in-memory arrays
  (x, v float32 (n, 3), colour int32 (n,), original particle order):
  per-dimension [min, max] ranges (:44-45), the narrow-range rule
  hi = max(lo + 1e-5, hi) (:48-50), 24-bit / 8-bit quantisation (:51-56) and
  the packing (qx << 8) + qv (:57), colour bytes (:62-74);
* ``read_arrays`` = ParticleIO.read_particles (:86-106).
The arithmetic is the reference's numpy expression, evaluated in float32
under numpy >= 2 promotion (python scalars are weak).

Pinned: tests check it against tests/golden/particle_io.npz, which
tests/golden/make_particle_io_golden.py produced by running the reference's
own functions.  Used only by tests/ and the CPU leg of bench.py.
"""
from __future__ import annotations

import numpy as np

V_BITS = 8
X_BITS = 32 - V_BITS


def ranges_of(x: np.ndarray, v: np.ndarray) -> np.ndarray:
    ranges = np.ndarray((2, 3, 2), dtype=np.float32)
    for d in range(3):
        ranges[0, d] = [np.min(x[:, d]), np.max(x[:, d])]
        ranges[1, d] = [np.min(v[:, d]), np.max(v[:, d])]
        for c in range(2):
            ranges[c, d, 1] = max(ranges[c, d, 0] + 1e-5, ranges[c, d, 1])
    return ranges


def write_arrays(x: np.ndarray, v: np.ndarray, color: np.ndarray):
    """(ranges (2,3,2) f32, x_and_v (n,3) u32, rgb (n,3) u8)."""
    x = np.asarray(x, np.float32)
    v = np.asarray(v, np.float32)
    n = x.shape[0]
    ranges = ranges_of(x, v)
    x_and_v = np.ndarray((n, 3), dtype=np.uint32)
    for d in range(3):
        qx = ((x[:, d] - ranges[0, d, 0]) * (1 / (ranges[0, d, 1] - ranges[0, d, 0])) * (2**X_BITS - 1) +
              0.499).astype(np.uint32)
        qv = ((v[:, d] - ranges[1, d, 0]) * (1 / (ranges[1, d, 1] - ranges[1, d, 0])) * (2**V_BITS - 1) +
              0.499).astype(np.uint32)
        x_and_v[:, d] = (qx << V_BITS) + qv
    c32 = np.asarray(color).astype(np.float32).astype(np.uint32)  # the reference stages colours in float32
    rgb = np.ndarray((n, 3), dtype=np.uint8)
    for c in range(3):
        rgb[:, c] = (c32 >> (8 * (2 - c))) & 255
    return ranges, x_and_v, rgb


def read_arrays(ranges: np.ndarray, x_and_v: np.ndarray):
    x = (x_and_v >> V_BITS).astype(np.float32) / (2**X_BITS - 1)
    for c in range(3):
        x[:, c] = x[:, c] * (ranges[0, c, 1] - ranges[0, c, 0]) + ranges[0, c, 0]
    v = (x_and_v & (2**V_BITS - 1)).astype(np.float32) / (2**V_BITS - 1)
    for c in range(3):
        v[:, c] = v[:, c] * (ranges[1, c, 1] - ranges[1, c, 0]) + ranges[1, c, 0]
    return x, v
