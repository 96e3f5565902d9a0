"""CPU checks of the path tracer's restatement (engine/renderer_utils.py
known answers) and the PNG writer; no GPU needed."""
import struct
import zlib

import numpy as np

from oracle import renderer_ref as R
from taichi_elements_gb300.renderer import write_png

F = np.float32


def test_intersect_sphere_head_on_and_miss():
    o = np.array([0, 0, 0], F)
    d = np.array([0, 0, 1], F)
    assert abs(R.intersect_sphere(o, d, np.array([0, 0, 5], F), 1.0) - 4.0) < 1e-5
    assert R.intersect_sphere(o, d, np.array([0, 3, 5], F), 1.0) == R.INF


def test_ray_aabb():
    inter, near, far = R.ray_aabb(np.zeros(3, F), np.ones(3, F), np.array([-1, 0.5, 0.5], F),
                                  np.array([1, 0, 0], F))
    assert inter and abs(near - 1) < 1e-6 and abs(far - 2) < 1e-6
    assert not R.ray_aabb(np.zeros(3, F), np.ones(3, F), np.array([-1, 2, 0.5], F), np.array([1, 0, 0], F))[0]


def test_inside_taichi_known_points():
    assert R.inside_taichi(0.0, 0.0) == 0      # outside the disc
    assert R.inside_taichi(0.5, 1.01) == 1     # the ring
    assert R.inside_taichi(0.5, 0.25) == 1     # small dot in the lower half
    assert R.inside_taichi(0.5, 0.75) == 0     # small dot in the upper half
    assert R.inside_taichi(0.5, 0.4) == 0      # lower lobe
    assert R.inside_taichi(0.5, 0.6) == 1      # upper lobe
    assert R.inside_taichi(0.3, 0.5) == 1 and R.inside_taichi(0.7, 0.5) == 0


def test_floor_ray_march_converges_to_the_plane():
    d = R.normalized(np.array([0.3, -0.8, 0.2], F))
    dist = R.ray_march(np.array([0, 1, 0], F), d, F(0.0))
    assert abs(dist - 1 / abs(d[1])) < 1e-4


def test_tonemap_formula():
    buf = np.full((4, 2, 3), 2.0)
    img = R.tonemap(buf, 2)
    assert np.isclose(img[2, 1, 0], np.sqrt(1.0 * 1.5))


def test_png_writer(tmp_path):
    img = np.zeros((5, 3, 3), F)
    img[4, 2] = (1.0, 0.5, 0.0)  # top-right pixel
    fn = tmp_path / "a.png"
    write_png(img, str(fn))
    b = fn.read_bytes()
    assert b[:8] == b"\x89PNG\r\n\x1a\n"
    w, h = struct.unpack(">II", b[16:24])
    assert (w, h) == (5, 3)
    idat = b[b.index(b"IDAT") + 4:b.index(b"IEND") - 8]
    raw = zlib.decompress(idat)
    row0 = np.frombuffer(raw[1:1 + 15], np.uint8).reshape(5, 3)
    assert tuple(row0[4]) == (255, 128, 0)
