"""The fused G2P2G mode (MPMSolver(use_g2p2g=True); engine/mpm_solver.py
:363-485 and the step loop :773-787) against the C oracle's restatement of
it (oracle_g2p2g, float64 and float32).

Tolerances as for the plain substep: after k substeps, grid velocities on the
grid-active nodes within rel L-inf 1e-5 and particle x / F / Jp within 1e-6
(v 1e-5) of float64, or never worse than 4x the float32 oracle's own error;
100-substep trajectories within rel L2 1e-3 of float64 positions."""
import numpy as np
import pytest

from helpers import assert_bounds, gpu_grid, oracle_config, rel_inf, window_lookup
from oracle import oracle as O
from taichi_elements_gb300 import scenes

pytestmark = pytest.mark.gpu



def gpu_particles(s):
    st = s.full_state()
    return {k: st[k].cpu().numpy().astype(np.float64) for k in ('x', 'v', 'F', 'Jp')}


def errors(s, R64, R32, win):
    g = gpu_particles(s)
    coords, vel = gpu_grid(s.views(), 'grid_vel')
    gv64 = R64.gv.reshape(tuple(win.W) + (3,))
    gv32 = R32.gv.reshape(tuple(win.W) + (3,))
    ref_v = window_lookup(win, coords, gv64)
    vscale = max(np.abs(R64.P.v).max(), 1e-3)
    fs = max(1.0, np.abs(R64.P.F).max())
    js = max(1.0, np.abs(R64.P.Jp).max())
    return {
        'grid_v': (rel_inf(vel[:, :3], ref_v), rel_inf(window_lookup(win, coords, gv32), ref_v)),
        'x': (rel_inf(g['x'], R64.P.x, 1.0), rel_inf(R32.P.x, R64.P.x, 1.0)),
        'v': (rel_inf(g['v'], R64.P.v, vscale), rel_inf(R32.P.v, R64.P.v, vscale)),
        'F': (rel_inf(g['F'], R64.P.F, fs), rel_inf(R32.P.F, R64.P.F, fs)),
        'Jp': (rel_inf(g['Jp'], R64.P.Jp, js), rel_inf(R32.P.Jp, R64.P.Jp, js)),
    }


def start(sc):
    s = sc.make_solver(use_g2p2g=True)
    cfg = oracle_config(sc)
    P64 = O.Particles.seeded(sc.x, sc.material, v=sc.v)
    win = O.Window.covering(P64.x, cfg.inv_dx, margin=16)
    return s, O.G2P2GRunner(cfg, P64, win), O.G2P2GRunner(cfg, P64.astype(np.float32), win), win


@pytest.mark.parametrize("scene_fn,nsub", [(scenes.smoke_scene, 1), (scenes.smoke_scene, 12),
                                           (lambda: scenes.four_materials_128(per_cube=8000), 8)])
def test_g2p2g_substeps_match_oracle(scene_fn, nsub):
    sc = scene_fn()
    s, R64, R32, win = start(sc)
    dt = sc.default_dt
    for _ in range(nsub):
        s.substep(dt)
        R64.step(dt)
        R32.step(dt)
    assert_bounds(f"{sc.name} fused, {nsub} substeps", errors(s, R64, R32, win), f32_calibrated=nsub > 1)


def test_g2p2g_trajectory_100_substeps():
    sc = scenes.smoke_scene()
    s, R64, _, _ = start(sc)
    dt = sc.default_dt
    for _ in range(100):
        s.substep(dt)
        R64.step(dt)
    x = gpu_particles(s)['x']
    err = np.linalg.norm(x - R64.P.x) / np.linalg.norm(R64.P.x)
    assert err < 1e-3, err


def test_g2p2g_frames_and_particles_added_between_frames():
    """step() frames (CUDA graphs from the second frame) and a cube added
    after them: the new particles skip the gather in their first substep."""
    sc = scenes.smoke_scene()
    s = sc.make_solver(use_g2p2g=True)
    for _ in range(3):
        s.step(1e-3)
    s.add_cube((0.4, 0.6, 0.4), (0.1, 0.1, 0.1), s.material_water, velocity=(0.0, -1.0, 0.0))
    # oracle from the engine's state: particles (old ones first) and its grid
    cfg = oracle_config(s)
    st = s.full_state()
    P = O.Particles(*(st[k].cpu().numpy().astype(np.float64) for k in ('x', 'v', 'C', 'F', 'Jp')),
                    st['material'].cpu().numpy().astype(np.int32))
    win = O.Window.covering(P.x, cfg.inv_dx, margin=16)
    R = O.G2P2GRunner(cfg, P, win)
    coords, vel = gpu_grid(s.views(), 'grid_vel')
    gv = np.zeros(tuple(win.W) + (3,))
    inside = np.all((coords >= win.lo) & (coords < win.lo + win.W), 1)
    gv[tuple((coords[inside] - win.lo).T)] = vel[inside, :3]
    R.gv = gv.reshape(-1)
    R.last_final = s._last_final
    assert R.last_final < P.n
    dt = s.default_dt
    s.substep(dt)
    R.step(dt)
    g = gpu_particles(s)
    assert rel_inf(g['x'], R.P.x, 1.0) < 1e-5
    assert rel_inf(g['v'], R.P.v, max(np.abs(R.P.v).max(), 1e-3)) < 1e-4
    new = np.arange(R.last_final, P.n)
    assert np.allclose(g['v'][new], R.P.v[new], atol=1e-5)


@pytest.mark.parametrize("v_clamp", [True, False])
def test_g2p2g_grid_velocity_clamp(v_clamp):
    """A cube launched faster than the CFL bound: with v_clamp_g2p2g=True
    (the default) the grid velocities are clamped to +-0.9 dx / dt per
    component after gravity (engine/mpm_solver.py:589-598), so the gathered
    particle velocities stay inside it; with v_clamp_g2p2g=False they do not.
    Both match the oracle run with the same setting."""
    rng = np.random.default_rng(11)
    res = (64, 64, 64)
    dt = 2e-2 / 64
    va = 0.9 * (1 / 64) / dt
    n = 8000
    x = (0.4 + 0.15 * rng.random((n, 3))).astype(np.float32)
    v = np.broadcast_to(np.array([1.4 * va, -1.2 * va, 0.5 * va], np.float32), (n, 3)).copy()
    sc = scenes.Scene("fast_cube_64", res, x, v, np.full(n, scenes.WATER, np.int32), 4)
    s = sc.make_solver(use_g2p2g=True, v_clamp_g2p2g=v_clamp)
    cfg = oracle_config(sc)
    P64 = O.Particles.seeded(sc.x, sc.material, v=sc.v)
    win = O.Window.covering(P64.x, cfg.inv_dx, margin=24)
    cfl = 0.9 if v_clamp else 0.0
    R64 = O.G2P2GRunner(cfg, P64, win, v_clamp_cfl=cfl)
    R32 = O.G2P2GRunner(cfg, P64.astype(np.float32), win, v_clamp_cfl=cfl)
    for _ in range(4):
        s.substep(dt)
        R64.step(dt)
        R32.step(dt)
    assert_bounds(f"{sc.name} fused, 4 substeps, clamp {v_clamp}", errors(s, R64, R32, win), f32_calibrated=True)
    vmax = np.abs(gpu_particles(s)['v']).max(0)
    if v_clamp:
        assert np.all(vmax <= va * (1 + 1e-6)), vmax
    else:
        assert vmax[0] > 1.3 * va, vmax


@pytest.mark.parametrize("resort", [1, 3, 16])
def test_g2p2g_frames_match_oracle(resort):
    """step() frames of the mode through mpm_g2p2g_frame: re-sorted every
    `resort` substeps (1: every substep writes the sorted order), in place in
    between."""
    sc = scenes.four_materials_128(per_cube=8000)
    s, R64, R32, win = start(sc)
    s.resort_every = resort
    count, dt = s.count_substeps(20 * sc.default_dt * 0.999, sc.default_dt)
    s.step(20 * sc.default_dt * 0.999)
    assert s.total_substeps == count
    for _ in range(count):
        R64.step(dt)
        R32.step(dt)
    assert_bounds(f"{sc.name} G2P2G frame of {count} substeps, re-sort every {resort}", errors(s, R64, R32, win),
                  f32_calibrated=True)


def test_g2p2g_frames_alternate_with_single_substeps():
    """A frame, single substeps (the per-substep kernel, as the adaptive-dt
    loop runs it), then another frame: each hands the binning and the grid to
    the next."""
    sc = scenes.smoke_scene()
    s, R64, R32, win = start(sc)
    s.resort_every = 4
    dt = sc.default_dt
    for kind in ("frame", "substep", "substep", "frame"):
        if kind == "frame":
            count, fdt = s.count_substeps(6 * dt * 0.999, dt)
            s.step(6 * dt * 0.999)
        else:
            count, fdt = 1, dt
            s.substep(dt)
        for _ in range(count):
            R64.step(fdt)
            R32.step(fdt)
    assert_bounds("smoke G2P2G frames and substeps", errors(s, R64, R32, win), f32_calibrated=True)


def test_g2p2g_frame_after_particles_were_added():
    """Particles added between frames: the next frame's first substep lets
    them skip the gather (id >= first_new), in the sorted pass."""
    sc = scenes.smoke_scene()
    s = sc.make_solver(use_g2p2g=True)
    s.resort_every = 3
    for _ in range(2):
        s.step(1e-3)
    s.add_cube((0.4, 0.6, 0.4), (0.1, 0.1, 0.1), s.material_water, velocity=(0.0, -1.0, 0.0))
    cfg = oracle_config(s)
    st = s.full_state()
    P = O.Particles(*(st[k].cpu().numpy().astype(np.float64) for k in ('x', 'v', 'C', 'F', 'Jp')),
                    st['material'].cpu().numpy().astype(np.int32))
    win = O.Window.covering(P.x, cfg.inv_dx, margin=16)
    R = O.G2P2GRunner(cfg, P, win)
    coords, vel = gpu_grid(s.views(), 'grid_vel')
    gv = np.zeros(tuple(win.W) + (3,))
    inside = np.all((coords >= win.lo) & (coords < win.lo + win.W), 1)
    gv[tuple((coords[inside] - win.lo).T)] = vel[inside, :3]
    R.gv = gv.reshape(-1)
    R.last_final = s._last_final
    assert R.last_final < P.n
    count, dt = s.count_substeps(4 * s.default_dt * 0.999, s.default_dt)
    s.step(4 * s.default_dt * 0.999)
    for _ in range(count):
        R.step(dt)
    g = gpu_particles(s)
    assert rel_inf(g['x'], R.P.x, 1.0) < 1e-5
    assert rel_inf(g['v'], R.P.v, max(np.abs(R.P.v).max(), 1e-3)) < 1e-4


def test_g2p2g_frames_rolled_match_oracle():
    """The G2P2G frames with MpmParams.occupancy = 1 (rolled stencil loops)."""
    sc = scenes.four_materials_128(per_cube=8000)
    s, R64, R32, win = start(sc)
    s.occupancy = 1
    s.resort_every = 3
    count, dt = s.count_substeps(20 * sc.default_dt * 0.999, sc.default_dt)
    s.step(20 * sc.default_dt * 0.999)
    for _ in range(count):
        R64.step(dt)
        R32.step(dt)
    assert_bounds(f"{sc.name} G2P2G frame of {count} substeps, rolled kernels", errors(s, R64, R32, win),
                  f32_calibrated=True)
