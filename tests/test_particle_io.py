"""The quantised particle frame format (engine/particle_io.py): the CPU
restatement against golden vectors that the reference's own functions
produced (tests/golden/make_particle_io_golden.py), the host-side reader and
the PLY writer.  All bit-exact; no GPU needed."""
import os

import numpy as np
import pytest

from oracle import particle_io_ref as R
from taichi_elements_gb300.particle_io import ParticleIO, write_point_cloud

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "particle_io.npz")
CASES = ("random", "narrow", "wide")


@pytest.fixture(scope="module")
def golden():
    with np.load(GOLDEN) as d:
        return {k: d[k] for k in d.files}


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference_golden(golden, case):
    ranges, x_and_v, rgb = R.write_arrays(golden[f"{case}_x"], golden[f"{case}_v"], golden[f"{case}_color"])
    assert ranges.dtype == np.float32 and x_and_v.dtype == np.uint32 and rgb.dtype == np.uint8
    np.testing.assert_array_equal(ranges.view(np.uint32), golden[f"{case}_ranges"].view(np.uint32))
    np.testing.assert_array_equal(x_and_v, golden[f"{case}_x_and_v"])
    np.testing.assert_array_equal(rgb, golden[f"{case}_rgb"])
    x, v = R.read_arrays(ranges, x_and_v)
    np.testing.assert_array_equal(x.view(np.uint32), golden[f"{case}_xdec"].view(np.uint32))
    np.testing.assert_array_equal(v.view(np.uint32), golden[f"{case}_vdec"].view(np.uint32))


@pytest.mark.parametrize("case", CASES)
def test_reader_decodes_reference_frames(golden, case, tmp_path):
    fn = tmp_path / f"{case}.npz"
    np.savez(fn, ranges=golden[f"{case}_ranges"], x_and_v=golden[f"{case}_x_and_v"], color=golden[f"{case}_rgb"])
    x, v, color = ParticleIO.read_particles_3d(str(fn))
    np.testing.assert_array_equal(x.view(np.uint32), golden[f"{case}_xdec"].view(np.uint32))
    np.testing.assert_array_equal(v.view(np.uint32), golden[f"{case}_vdec"].view(np.uint32))
    np.testing.assert_array_equal(color, golden[f"{case}_rgb"])


def test_quantisation_edges():
    # the top of the range rounds to 2^24 - 1 (or wraps past it), v to 255
    x = np.array([[0.0, 1.0, 2.0], [1.0, 2.0, 3.0]], np.float32)
    v = np.array([[-1.0, 0.0, 0.0], [1.0, 0.0, 0.0]], np.float32)
    ranges, x_and_v, _ = R.write_arrays(x, v, np.zeros(2, np.int32))
    assert x_and_v[0, 0] == 0 and (x_and_v[1, 0] >> 8) in ((1 << 24) - 1, 0)
    assert ranges[1, 1, 1] == np.float32(np.float32(0.0) + np.float32(1e-5))


def test_ply_writer_layout(tmp_path):
    pos = np.arange(12, dtype=np.float32).reshape(4, 3)
    col = np.array([0x010203, 0xFFFFFF, 0, 0x123456], np.uint32)
    fn = tmp_path / "p.ply"
    write_point_cloud(str(fn), np.hstack([pos, col[:, None].view(np.float32)]))
    raw = fn.read_bytes()
    head, body = raw.split(b"end_header\n", 1)
    assert b"element vertex 4" in head and b"format binary_little_endian 1.0" in head
    rows = np.frombuffer(body, np.float32).reshape(4, 4)
    np.testing.assert_array_equal(rows[:, :3], pos)
    np.testing.assert_array_equal(rows[:, 3].view(np.uint32), col)
