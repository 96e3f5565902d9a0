"""Batched multi-scene mode: every scene of a batch must evolve exactly as an
independent MPMSolver with the same constants would (up to float32
summation order), and the slot layout must keep scenes apart."""
import numpy as np
import pytest

from taichi_elements_gb300 import scenes
from taichi_elements_gb300.batched import BatchScene, MARGIN


def small_scenes():
    rng = np.random.default_rng(21)
    out = []
    for i, (r, mat, E_scale) in enumerate([(32, 0, 1.0), (48, 1, 0.05), (24, 2, 0.3), (40, 3, 1.0), (32, 4, 1.0)]):
        n = int(rng.integers(1500, 4000))
        lo = rng.uniform(0.2, 0.45, 3)
        x = (lo + 0.25 * rng.random((n, 3))).astype(np.float32)
        v = np.broadcast_to(rng.uniform(-1, 1, 3).astype(np.float32), (n, 3))
        pp = [dict(kind=0, surface=1, point=(0.5, 0.25, 0.5), normal=(0.1, 1.0, 0.0), friction=0.0)] if i % 2 else \
             [dict(kind=1, surface=2, point=(0.5, 0.5, 0.5), radius=0.1)]
        out.append(BatchScene((r, r, r), x, mat, v, E_scale=E_scale, gravity=(0.0, -9.8 - i, 0.0), postprocess=pp))
    return out


def test_slot_layout_host_logic():
    sc = small_scenes()
    wins = [s.window() for s in sc]
    for (lo, nb), s in zip(wins, sc):
        assert all(l % 4 == 0 for l in lo)
        assert all(l + 4 * b >= r + MARGIN for l, b, r in zip(lo, nb, s.res))


@pytest.mark.gpu
def test_batched_matches_independent_solvers():
    from taichi_elements_gb300.batched import BatchedMPM
    from taichi_elements_gb300.mpm_solver import MPMSolver
    sc = small_scenes()
    B = BatchedMPM(sc)
    nsub = 25
    B.substeps(nsub)
    B.check_status()
    for i, s in enumerate(sc):
        m = MPMSolver(s.res, E_scale=s.E / 1e6)
        m.set_gravity(s.gravity)
        for c in s.postprocess[1:]:
            if c["kind"] == 0:
                m.add_surface_collider(c["point"], c["normal"], c.get("surface", 0), c.get("friction", 0.0))
            else:
                m.add_sphere_collider(c["point"], c["radius"], c.get("surface", 0))
        m.read_restart(s.n, s.x, s.v, s.material, np.zeros(s.n, np.int32))
        for _ in range(nsub):
            m.substep(s.dt)
        ref = m.particle_info()
        got = B.positions(i)
        assert np.abs(got - ref['position']).max() < 2e-6, i
        assert np.abs(B.velocities(i) - ref['velocity']).max() < 1e-4 * max(1.0, np.abs(ref['velocity']).max()), i
    mv = B.max_velocity(nsub)
    assert mv.shape == (nsub, len(sc)) and np.all(mv > 0)


@pytest.mark.gpu
def test_batched_graph_replay_matches_eager():
    from taichi_elements_gb300.batched import BatchedMPM
    sc = small_scenes()
    a = BatchedMPM(sc, use_cuda_graph=True)
    b = BatchedMPM(sc, use_cuda_graph=False)
    for _ in range(3):
        a.substeps(10)
        b.substeps(10)
    for i in range(len(sc)):
        assert np.abs(a.positions(i) - b.positions(i)).max() < 1e-5
