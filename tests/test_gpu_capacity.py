"""Particle capacity: the reference grows its particle field in chunks
(engine/mpm_solver.py:213-214) and asserts against max_num_particles when
seeding (:874, :913, :1012).  Here the state buffers grow by doubling: every
growth keeps the particles already there, in both storage layouts, and a
request beyond max_num_particles fails the same assertion."""
import numpy as np
import pytest

from taichi_elements_gb300.mpm_solver import MPMSolver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("quant", [False, True])
def test_growth_keeps_particles(quant):
    s = MPMSolver((64, 64, 64), quant=quant, seed=3)
    caps = []
    before = None
    # 16,778 + 56,624 + 89,916 + 56,624 particles: capacity 65,536 -> 131,072 -> 262,144
    for k, (lo, side, mat) in enumerate([((0.1, 0.1, 0.1), 0.2, 1), ((0.5, 0.1, 0.5), 0.3, 0), ((0.1, 0.5, 0.1), 0.35, 2),
                                         ((0.55, 0.55, 0.55), 0.3, 3)]):
        if before is not None:
            n0 = before['position'].shape[0]
            s.add_cube(lo, (side, side, side), mat)
            after = s.particle_info()
            for key in ('position', 'velocity', 'material', 'color'):
                np.testing.assert_array_equal(after[key][:n0], before[key], err_msg=key)
        else:
            s.add_cube(lo, (side, side, side), mat)
        caps.append(s._cap)
        s.step(2e-3)
        before = s.particle_info()
        assert np.isfinite(before['position']).all()
    assert len(set(caps)) >= 3, caps  # the buffers grew at least twice
    s._check_status()


def test_max_num_particles_assertion():
    s = MPMSolver((32, 32, 32), max_num_particles=1000)
    s.add_cube((0.4, 0.4, 0.4), (0.05, 0.05, 0.05), 0)  # int(8 * 1.25e-4 * 32^3 + 1) = 33 particles
    with pytest.raises(AssertionError):
        s.add_cube((0.2, 0.2, 0.2), (0.3, 0.3, 0.3), 0)
    assert s.n_particles == 33
