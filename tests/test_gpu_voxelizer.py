"""GPU mesh voxelizer and add_mesh emitter (csrc/mpm_voxelize.cu) against
the CPU restatement: voxel counts bit-exact; seeded particles one per
inside voxel at the default density, each inside its voxel."""
import numpy as np
import pytest

from oracle import voxelizer_ref as V
from taichi_elements_gb300 import scenes
from taichi_elements_gb300.mpm_solver import MPMSolver
from taichi_elements_gb300.voxelizer import Voxelizer

pytestmark = pytest.mark.gpu


def soup(seed, n=400):
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.15, 0.85, (n, 1, 3))
    return (c + rng.normal(0, 0.08, (n, 3, 3))).reshape(n, 9).astype(np.float32)


def in_positive_voxel(vox, rel):
    """Each particle sits in a voxel with a positive count (a position that
    float32 rounding put on a voxel face may belong to either side)."""
    ok = np.zeros(len(rel), bool)
    sides = [np.clip(np.floor(rel + e).astype(np.int64), 0, np.array(vox.shape) - 1) for e in (-1e-3, 1e-3)]
    for a in sides:
        for b in sides:
            for c in sides:
                ok |= vox[a[:, 0], b[:, 1], c[:, 2]] > 0
    return ok.all()


MESHES = {
    "box": lambda: scenes.box_mesh((0.2, 0.3, 0.25), (0.6, 0.7, 0.55)),
    "sphere": lambda: scenes.icosphere((0.5, 0.5, 0.5), 0.3, 3),
    "torus": lambda: scenes.torus_mesh((0.5, 0.45, 0.5), 0.25, 0.08),
    "soup": lambda: soup(3),
}


@pytest.mark.parametrize("name", sorted(MESHES))
@pytest.mark.parametrize("res", [(32, 32, 32), (24, 40, 16)])
def test_voxel_counts_bit_exact(name, res):
    tri = MESHES[name]()
    vz = Voxelizer(res, 1.0 / res[0], padding=3)
    got = vz.voxelize(tri).cpu().numpy()
    want = V.voxelize(tri, vz.res, vz.dx, padding=3)
    assert got.shape == want.shape == V.grid_res(res)
    np.testing.assert_array_equal(got, want)


def test_add_mesh_seeds_one_particle_per_inside_voxel():
    s = MPMSolver((32, 32, 32), use_emitter_id=True)
    tri = scenes.icosphere((0.5, 0.5, 0.5), 0.25, 3)
    s.add_mesh(tri, MPMSolver.material_elastic, color=0x00FF00, velocity=(0.5, -1.0, 0.0), emmiter_id=7)
    vox = s.voxelizer.voxels.cpu().numpy()
    info = s.particle_info()
    assert s.n_particles == int((vox > 0).sum()) > 1000
    assert in_positive_voxel(vox, info["position"] / np.float32(s.voxelizer.dx))
    np.testing.assert_array_equal(info["velocity"], np.tile(np.float32([0.5, -1.0, 0.0]), (s.n_particles, 1)))
    assert (info["material"] == MPMSolver.material_elastic).all() and (info["color"] == 0x00FF00).all()
    assert (info["emitter_ids"] == 7).all()
    s.step(2e-3)
    assert np.isfinite(s.particle_info()["position"]).all()


def test_add_mesh_density_translation_and_determinism():
    def run():
        s = MPMSolver((32, 32, 32), seed=5)
        s.add_mesh(scenes.box_mesh((0.1, 0.1, 0.1), (0.3, 0.3, 0.3)), MPMSolver.material_water, sample_density=12,
                   translation=(0.2, 0.25, 0.3))
        return s
    a, b = run(), run()
    vox = a.voxelizer.voxels.cpu().numpy()
    npos = int((vox > 0).sum())
    assert npos < a.n_particles <= 2 * npos  # s = 12 / 8 = 1.5 particles per voxel
    xa, xb = a.particle_info()["position"], b.particle_info()["position"]
    np.testing.assert_array_equal(xa, xb)
    assert in_positive_voxel(vox, (xa - np.float32([0.2, 0.25, 0.3])) / np.float32(a.voxelizer.dx))
