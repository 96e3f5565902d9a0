"""MPMSolver(support_plasticity=False) (engine/mpm_solver.py:62 and the
``ti.static(self.support_plasticity)`` branches of p2g :508-566 and of the
fused g2p2g :419-476) against the oracle run with the same flag: water
restarts from F = I, h = 1, Jp is never updated and sand carries no stress.
The four cubes get a linear velocity field (strain rate up to 8/s) on top of
their drift, so snow clamps, sand yields and water compresses within the
first substeps; both flag values are checked on the same scene.

Tolerances as for the default substep: grid and particle fields after one
substep within rel L-inf 1e-5 / 1e-6 of float64 (or never worse than 4x the
float32 oracle's own error), 100-substep trajectories within rel L2 1e-3."""
import numpy as np
import pytest
import torch

from helpers import assert_bounds, oracle_config
from oracle import oracle as O
from taichi_elements_gb300 import scenes
from test_gpu_g2p2g import errors as fused_errors
from test_gpu_parity import _one_substep_errors

pytestmark = pytest.mark.gpu


def _scene(per_cube=20000):
    sc = scenes.four_materials_128(per_cube=per_cube)
    rng = np.random.default_rng(7)
    v = sc.v.astype(np.float64).copy()
    for m in range(4):
        sel = sc.material == m
        c = sc.x[sel].mean(0)
        v[sel] += (sc.x[sel] - c) @ rng.uniform(-8, 8, (3, 3)).T
    sc.v = v.astype(np.float32)
    return sc


@pytest.mark.parametrize("plasticity", [False, True])
def test_one_substep_parity_sheared(plasticity):
    sc = _scene()
    s = sc.make_solver(support_plasticity=plasticity)
    for _ in range(30):
        s.substep(sc.default_dt)
    torch.cuda.synchronize()
    jp0 = s.full_state()['Jp'].cpu().numpy()
    errs = _one_substep_errors(s, sc.default_dt)
    assert_bounds(f"sheared four materials, plasticity {plasticity}", errs, f32_calibrated=True)
    if not plasticity:
        np.testing.assert_array_equal(s.full_state()['Jp'].cpu().numpy(), jp0)


def test_trajectory_100_substeps_without_plasticity():
    sc = _scene()
    s = sc.make_solver(support_plasticity=False)
    cfg = oracle_config(s)
    assert cfg.support_plasticity is False
    R = O.Runner(cfg, O.Particles.seeded(sc.x, sc.material, v=sc.v))
    dt = sc.default_dt
    R.run(dt, 100)
    for _ in range(100):
        s.substep(dt)
    g = s.full_state()['x'].cpu().numpy().astype(np.float64)
    err = np.linalg.norm(g - R.P.x) / np.linalg.norm(R.P.x)
    assert err < 1e-3, err
    # the default solver moves differently on the same scene
    d = sc.make_solver()
    for _ in range(100):
        d.substep(dt)
    gd = d.full_state()['x'].cpu().numpy().astype(np.float64)
    assert np.linalg.norm(gd - R.P.x) / np.linalg.norm(R.P.x) > 10 * err


def test_g2p2g_without_plasticity_matches_oracle():
    sc = _scene(per_cube=8000)
    s = sc.make_solver(use_g2p2g=True, support_plasticity=False)
    cfg = oracle_config(s)
    P64 = O.Particles.seeded(sc.x, sc.material, v=sc.v)
    win = O.Window.covering(P64.x, cfg.inv_dx, margin=16)
    R64 = O.G2P2GRunner(cfg, P64, win)
    R32 = O.G2P2GRunner(cfg, P64.astype(np.float32), win)
    dt = sc.default_dt
    for _ in range(8):
        s.substep(dt)
        R64.step(dt)
        R32.step(dt)
    assert_bounds("sheared four materials, fused, no plasticity, 8 substeps", fused_errors(s, R64, R32, win),
                  f32_calibrated=True)
