"""GPU particle output (csrc/mpm_io.cu through MPMSolver.write_particles)
against the reference's golden frames and the CPU restatement: bit-exact."""
import os

import numpy as np
import pytest

from oracle import particle_io_ref as R
from taichi_elements_gb300 import scenes
from taichi_elements_gb300.mpm_solver import MPMSolver
from taichi_elements_gb300.particle_io import ParticleIO

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "particle_io.npz")


def frame(fn):
    with np.load(fn) as d:
        return d["ranges"], d["x_and_v"], d["color"]


@pytest.mark.parametrize("case", ("random", "narrow", "wide"))
def test_write_particles_matches_reference_golden(case, tmp_path):
    with np.load(GOLDEN) as d:
        x, v, color = d[f"{case}_x"], d[f"{case}_v"], d[f"{case}_color"]
        want = d[f"{case}_ranges"], d[f"{case}_x_and_v"], d[f"{case}_rgb"]
    s = MPMSolver((16, 16, 16), size=8.0)
    s.read_restart(len(x), x, v, np.zeros(len(x), np.int32), color)
    fn = str(tmp_path / f"{case}.npz")
    s.write_particles(fn)
    got = frame(fn)
    np.testing.assert_array_equal(got[0].view(np.uint32), want[0].view(np.uint32))
    np.testing.assert_array_equal(got[1], want[1])
    np.testing.assert_array_equal(got[2], want[2])


def test_write_particles_after_substeps_matches_oracle(tmp_path):
    """Sorted device state (the solver has stepped) against the CPU
    restatement of the same particles in original order."""
    sc = scenes.smoke_scene()
    sc.color = np.random.default_rng(1).integers(0, 1 << 24, sc.n).astype(np.int32)
    s = sc.make_solver()
    s.step(4e-3)
    info = s.particle_info()
    fn = str(tmp_path / "f.npz")
    s.write_particles(fn)
    got = frame(fn)
    want = R.write_arrays(info["position"], info["velocity"], info["color"])
    np.testing.assert_array_equal(got[0].view(np.uint32), want[0].view(np.uint32))
    np.testing.assert_array_equal(got[1], want[1])
    np.testing.assert_array_equal(got[2], want[2])
    x, v, _ = ParticleIO.read_particles_3d(fn)
    ext = (want[0][0, :, 1] - want[0][0, :, 0]).max()
    assert np.abs(x - info["position"]).max() <= 2 * ext / (2**24 - 1) + 1e-6


def test_write_particles_ply_original_order(tmp_path):
    sc = scenes.smoke_scene()
    sc.color = np.random.default_rng(2).integers(0, 1 << 24, sc.n).astype(np.int32)
    s = sc.make_solver()
    s.step(2e-3)
    fn = tmp_path / "p.ply"
    s.write_particles_ply(str(fn))
    body = fn.read_bytes().split(b"end_header\n", 1)[1]
    rows = np.frombuffer(body, np.float32).reshape(-1, 4)
    info = s.particle_info()
    np.testing.assert_array_equal(rows[:, :3], info["position"])
    np.testing.assert_array_equal(rows[:, 3].view(np.int32), info["color"])
