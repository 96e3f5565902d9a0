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


def test_blender_cache_frame_round_trip(tmp_path):
    """blender/operators.py:228-247 for a GB300 solver: the five attribute
    files hold particle_info's arrays in original order, and the header is
    the reference's format (checked against its own bytes on the CPU)."""
    from taichi_elements_gb300 import blender_cache as B
    from taichi_elements_gb300.mpm_solver import MPMSolver
    s = MPMSolver((32, 32, 32), use_emitter_id=True)
    s.add_cube((0.3, 0.3, 0.3), (0.2, 0.2, 0.2), MPMSolver.material_snow, color=0x123456)
    s.add_ellipsoid((0.6, 0.6, 0.6), 0.1, MPMSolver.material_water, color=0xABCDEF, velocity=(1, 0, 0))
    for _ in range(3):
        s.step(4e-3)
    path = B.save_particles(s, str(tmp_path), 17)
    assert os.path.basename(path) == 'particles_000017.bin'
    out = B.read_pars(path)
    info = s.particle_info()
    n = info['position'].shape[0]
    np.testing.assert_array_equal(out[B.POS].reshape(n, 3), info['position'])
    np.testing.assert_array_equal(out[B.VEL].reshape(n, 3), info['velocity'])
    np.testing.assert_array_equal(out[B.COL], info['color'])
    np.testing.assert_array_equal(out[B.MAT], info['material'])
    np.testing.assert_array_equal(out[B.EMT], info['emitter_ids'])
