"""GPU path tracer (csrc/mpm_render.cu) against the CPU restatement
(oracle/renderer_ref.py): cell lists, nearest hits of camera rays, and the
light transport in distribution (the random streams differ)."""
import numpy as np
import pytest

from oracle import renderer_ref as R
from taichi_elements_gb300 import scenes
from taichi_elements_gb300.renderer import Renderer

pytestmark = pytest.mark.gpu
F = np.float32


def particle_scene(n, seed=0, blur=True):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.3, 0.6, (n, 3)).astype(F)
    x[:, 1] = rng.uniform(0.02, 0.3, n).astype(F)
    v = (rng.normal(0, 1.0, (n, 3)) if blur else np.zeros((n, 3))).astype(F)
    rgb = rng.integers(0, 256, (n, 3)).astype(np.uint8)
    return x, v, rgb


def make(x, v, rgb, dx=1 / 64, shutter=1e-3, res=(32, 18), logo=True, voxel=False):
    r = Renderer(dx=dx, sphere_radius=0.3 * dx, shutter_time=shutter, taichi_logo=logo, res=res, seed=1,
                 render_voxel=voxel)
    r.set_camera_pos(0.45, 0.45, 1.6)
    r.look_at[None] = (0.45, 0.12, 0.45)
    r.floor_height[None] = 0.0
    r.initialize_particles(x, v, rgb)
    return r


def test_cell_lists_match_restatement():
    x, v, rgb = particle_scene(300, seed=1)
    r = make(x, v, rgb, shutter=2e-2)  # long shutter: particles span several cells
    g = R.Grid(x, r.dx)
    assert np.array_equal(g.c0, r._cells[0]) and np.array_equal(g.nc, r._cells[1])
    lists = R.cell_lists(g, x, v, r.sphere_radius, r.shutter_time)
    want = np.zeros(int(np.prod(g.nc)), np.int64)
    for (i, j, k), ps in lists.items():
        want[((i - g.c0[0]) * g.nc[1] + (j - g.c0[1])) * g.nc[2] + (k - g.c0[2])] = len(ps)
    got = r._count.cpu().numpy()
    assert got.sum() == want.sum() > 300
    assert (got != want).mean() < 1e-3
    # the lists hold the right particles
    cnt, start, lst = r._count.cpu().numpy(), r._start.cpu().numpy(), r._list.cpu().numpy()
    for (i, j, k), ps in list(lists.items())[:200]:
        c = ((i - g.c0[0]) * g.nc[1] + (j - g.c0[1])) * g.nc[2] + (k - g.c0[2])
        if cnt[c] == len(ps):
            assert sorted(lst[start[c]:start[c] + cnt[c]]) == sorted(ps)


@pytest.mark.parametrize("voxel", [False, True])
def test_first_hits_match_restatement(voxel):
    x, v, rgb = particle_scene(3000, seed=2)
    r = make(x, v, rgb, voxel=voxel)
    g = R.Grid(x, r.dx)
    lists = R.cell_lists(g, x, v, r.sphere_radius, r.shutter_time)
    pos, d = R.camera_rays(r.res, r.camera_pos[None], r.look_at[None], r.up[None], r.fov[None],
                           np.full(r.res + (2,), 0.5, F))
    pos, d = pos.reshape(-1, 3), d.reshape(-1, 3)
    t = 2e-4
    got = r.first_hits(pos, d, t)
    agree, close = 0, 0
    for q in range(len(pos)):
        dist, nrm, col = R.next_hit(g, lists, x, v, rgb, F(r.sphere_radius), pos[q], d[q], F(t), F(0.0), True,
                                    voxel=voxel)
        same = np.allclose(got[q, 1:4], nrm, atol=1e-3) and np.allclose(got[q, 4:7], col, atol=1e-5)
        agree += same
        close += same and abs(got[q, 0] - dist) <= 1e-4 * max(1.0, abs(dist))
    assert agree >= 0.995 * len(pos), agree / len(pos)
    assert close >= 0.995 * len(pos), close / len(pos)
    hits = got[:, 0] < 1e9
    assert hits.mean() > 0.3  # the view sees particles and floor


def test_light_transport_matches_restatement_in_distribution():
    """Floor and back plane only (the particles sit far outside every
    path): per-region means of the linear colour buffer."""
    x = np.array([[100.0, -100.0, 100.0], [100.02, -100.0, 100.0]], F)
    r = make(x, np.zeros_like(x), np.full((2, 3), 200, np.uint8), shutter=0.0, res=(32, 18), logo=False)
    r.set_camera_pos(0.5, 0.6, 2.0)
    r.look_at[None] = (0.5, 0.0, 0.0)
    gpu_spp = 2048
    r.render(gpu_spp)
    gmean = r.color_buffer.cpu().numpy() / gpu_spp
    rng = np.random.default_rng(0)
    n_spp = 64
    s1 = np.zeros(r.res + (3,))
    s2 = np.zeros(r.res + (3,))
    for _ in range(n_spp):
        b = R.render_no_particles(r.res, r.camera_pos[None], r.look_at[None], r.up[None], r.fov[None], 1, 0.0,
                                  False, rng)
        s1 += b
        s2 += b * b
    cmean = s1 / n_spp
    var = np.maximum(s2 / n_spp - cmean**2, 1e-12)
    # 4 x 3 pixel regions
    def reg(a):
        return a.reshape(8, 4, 6, 3, 3).mean((1, 3))
    se = np.sqrt(reg(var) / 12 * (1 / n_spp + 1 / gpu_spp))
    z = np.abs(reg(gmean) - reg(cmean)) / np.maximum(se, 1e-6)
    assert z.max() < 6.0, z.max()
    assert reg(gmean).mean() > 0.05  # the floor is lit


def test_render_frame_from_a_solver_and_from_a_frame_file(tmp_path):
    sc = scenes.smoke_scene()
    s = sc.make_solver()
    s.step(4e-3)
    fn = str(tmp_path / "f.npz")
    s.write_particles(fn)
    a = Renderer(dx=1 / 128, sphere_radius=0.3 / 128, res=(64, 36), seed=3)
    a.set_camera_pos(0.5, 0.6, 2.0)
    a.look_at[None] = (0.5, 0.3, 0.4)
    a.initialize_particles_from_taichi_elements(fn)
    img = a.render_frame(spp=8)
    assert img.shape == (64, 36, 3) and np.isfinite(img).all() and img.max() > 0
    assert a.total_inserted_particles() >= s.n_particles and a.total_non_empty_voxels() > 0
    b = Renderer(dx=1 / 128, sphere_radius=0.3 / 128, res=(64, 36), seed=3)
    b.set_camera_pos(0.5, 0.6, 2.0)
    b.look_at[None] = (0.5, 0.3, 0.4)
    b.initialize_particles_from_solver(s)
    assert b.num_particles == a.num_particles
    assert np.isfinite(b.render_frame(spp=4)).all()
