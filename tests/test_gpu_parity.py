"""GPU parity of the engine against the CPU oracle (float64 and float32).

Tolerances (GPU float32 vs oracle float64, one substep from one state):
  binning, active-block lists, per-block counts:     bit-exact
  grid mass / momentum after P2G:                    rel L-inf <= 1e-5
  grid velocity after the update:                    rel L-inf <= 1e-5
  particle x, F (scale 1), v:                        rel L-inf <= 1e-6 / 1e-6 / 1e-5
and never worse than 4x the float32 oracle's own error against float64.
Trajectories: positions after 100 substeps within rel L2 1e-3 of float64.
"""

import numpy as np
import pytest
import torch

from helpers import (assert_bounds, block_coords, gpu_grid, lib_call, oracle_config, particles_from_solver,
                     rel_inf, run_phases, window_lookup)
from oracle import oracle as O
from taichi_elements_gb300 import scenes
from taichi_elements_gb300.mpm_solver import MPMSolver, MPMError

pytestmark = pytest.mark.gpu


def test_binning_bit_exact_water_cube():
    sc = scenes.water_cube_64()
    s = sc.make_solver()
    s._prepare(sc.default_dt)
    lib_call(s, "mpm_bin_finalize", s._ws.data_ptr(), s._cap, s.n_particles, torch.cuda.current_stream().cuda_stream)
    v = s.views()
    torch.cuda.synchronize()
    npb, ngb = int(v['counters'][0]), int(v['counters'][1])
    assert int(v['counters'][4]) == sc.n
    pb = block_coords(v['pblocks'][:npb].cpu().numpy(), v['win_lo'], v['win_nb'])
    gb = block_coords(v['gblocks'][:ngb].cpu().numpy(), v['win_lo'], v['win_nb'])
    counts = v['pblock_count'][:npb].cpu().numpy()
    ref_pb, ref_counts, ref_gb = O.active_sets(sc.x, s.inv_dx)
    np.testing.assert_array_equal(pb, ref_pb)
    np.testing.assert_array_equal(counts, ref_counts)
    np.testing.assert_array_equal(gb, ref_gb)
    # the sorted order is a permutation grouping particles by block
    pid = v['pid'][:sc.n].cpu().numpy()
    assert np.array_equal(np.sort(pid), np.arange(sc.n))
    starts = v['pblock_start'][:npb].cpu().numpy()
    assert np.array_equal(starts, np.concatenate([[0], np.cumsum(counts)[:-1]]))
    key = v['cellkey'][:sc.n].cpu().numpy()
    blk_of_sorted = key[pid] >> 6
    expect = np.repeat(v['pblocks'][:npb].cpu().numpy(), counts)
    np.testing.assert_array_equal(blk_of_sorted, expect)
    # rank-major order inside each block: consecutive entries of one level
    # are distinct cells in increasing order
    cell = key[pid] & 63
    for k in range(0, npb, max(1, npb // 50)):
        seg = cell[starts[k]:starts[k] + counts[k]]
        lv_breaks = np.nonzero(np.diff(seg) <= 0)[0]
        assert len(lv_breaks) < counts[k]


def _evolve(sc, n_sub, **kw):
    s = sc.make_solver(**kw)
    for _ in range(n_sub):
        s.substep(sc.default_dt)
    torch.cuda.synchronize()
    return s


def _one_substep_errors(s, dt, nthreads=1):
    cfg = oracle_config(s)
    P64 = particles_from_solver(s, np.float64)
    P32 = particles_from_solver(s, np.float32)
    win = O.Window.covering(P64.x, cfg.inv_dx)
    _, gm64, gmv64, gv64 = O.substep(cfg, P64, dt, win, nthreads)
    _, gm32, gmv32, gv32 = O.substep(cfg, P32, dt, win, nthreads)
    views, out = run_phases(s, dt)
    Pg = particles_from_solver(s, np.float64)
    coords, mom = out['mom']
    _, vel = out['vel']
    # every oracle node with mass is a GPU grid-active node
    assert np.isclose(window_lookup(win, coords, gm64).sum(), gm64.sum(), rtol=1e-12)
    ref_m = window_lookup(win, coords, gm64)
    ref_mv = window_lookup(win, coords, gmv64)
    ref_v = window_lookup(win, coords, gv64)
    f32_m = window_lookup(win, coords, gm32)
    f32_mv = window_lookup(win, coords, gmv32)
    f32_v = window_lookup(win, coords, gv32)
    vscale = max(np.abs(P64.v).max(), 1e-3)
    errs = {
        'grid_m': (rel_inf(mom[:, 0], ref_m), rel_inf(f32_m, ref_m)),
        'grid_mv': (rel_inf(mom[:, 1:], ref_mv), rel_inf(f32_mv, ref_mv)),
        'grid_v': (rel_inf(vel[:, :3], ref_v), rel_inf(f32_v, ref_v)),
        'x': (rel_inf(Pg.x, P64.x, 1.0), rel_inf(P32.x, P64.x, 1.0)),
        'v': (rel_inf(Pg.v, P64.v, vscale), rel_inf(P32.v, P64.v, vscale)),
        'F': (rel_inf(Pg.F, P64.F, max(1.0, np.abs(P64.F).max())), rel_inf(P32.F, P64.F, max(1.0, np.abs(P64.F).max()))),
        'Jp': (rel_inf(Pg.Jp, P64.Jp, max(1.0, np.abs(P64.Jp).max())),
               rel_inf(P32.Jp, P64.Jp, max(1.0, np.abs(P64.Jp).max()))),
        'C': (rel_inf(Pg.C, P64.C, 4 * cfg.inv_dx * vscale), rel_inf(P32.C, P64.C, 4 * cfg.inv_dx * vscale)),
    }
    return errs


@pytest.mark.parametrize("scene_fn,n_pre", [(scenes.smoke_scene, 40), (lambda: scenes.four_materials_128(per_cube=20000), 30)])
def test_one_substep_parity(scene_fn, n_pre):
    sc = scene_fn()
    s = _evolve(sc, n_pre)
    errs = _one_substep_errors(s, sc.default_dt)
    assert_bounds(sc.name, errs, f32_calibrated=True)


def _dense_swirl_scene():
    """30,000 particles in a cube of ~3.8 cells per side (about 500 per cell)
    turning at 20 rad/s: cells hold far more than 64 particles, so ranks of
    64 and above take the arrival path of the binning while particles keep
    crossing cells."""
    rng = np.random.default_rng(21)
    n = 30000
    c = np.array([0.5, 0.5, 0.5], np.float32)
    x = (c - 0.06 + 0.12 * rng.random((n, 3))).astype(np.float32)
    w = np.array([0.0, 20.0, 5.0])
    v = np.cross(w, x - c).astype(np.float32)
    mat = np.where(np.arange(n) % 2 == 0, scenes.WATER, scenes.ELASTIC).astype(np.int32)
    return scenes.Scene("dense_swirl_32", (32, 32, 32), x, v, mat, 20)


def test_one_substep_parity_dense_cells():
    sc = _dense_swirl_scene()
    keys = np.floor(sc.x.astype(np.float32) * np.float32(32) - np.float32(0.5)).astype(np.int64)
    _, counts = np.unique(keys, axis=0, return_counts=True)
    assert counts.max() > 64
    s = _evolve(sc, 10)
    s._check_status()
    errs = _one_substep_errors(s, sc.default_dt)
    assert_bounds(sc.name, errs, f32_calibrated=True)
    s.substep(sc.default_dt)
    s._check_status()


def test_trajectory_100_substeps_four_materials():
    sc = scenes.four_materials_128(per_cube=20000)
    s = sc.make_solver()
    cfg = oracle_config(sc)
    P = O.Particles.seeded(sc.x, sc.material, v=sc.v)
    R = O.Runner(cfg, P)
    dt = sc.default_dt
    R.run(dt, 100)
    for _ in range(100):
        s.substep(dt)
    g = s.full_state()['x'].cpu().numpy().astype(np.float64)
    err = np.linalg.norm(g - R.P.x) / np.linalg.norm(R.P.x)
    assert err < 1e-3, err


def test_trajectory_colliders_smoke_scene():
    sc = scenes.smoke_scene()
    s = sc.make_solver()
    cfg = oracle_config(sc)
    R = O.Runner(cfg, O.Particles.seeded(sc.x, sc.material, v=sc.v))
    dt = sc.default_dt
    R.run(dt, 100)
    for _ in range(100):
        s.substep(dt)
    g = s.full_state()['x'].cpu().numpy().astype(np.float64)
    err = np.linalg.norm(g - R.P.x) / np.linalg.norm(R.P.x)
    assert err < 1e-3, err


def test_step_substep_count_and_graph_matches_eager():
    sc = scenes.smoke_scene()
    a = sc.make_solver(use_cuda_graph=True)
    b = sc.make_solver(use_cuda_graph=False)
    for _ in range(3):
        a.step(4e-3)
        b.step(4e-3)
    n, _ = MPMSolver.count_substeps(4e-3, a.default_dt)
    assert a.total_substeps == 3 * n == b.total_substeps
    xa = a.particle_info()['position']
    xb = b.particle_info()['position']
    assert np.abs(xa - xb).max() < 1e-5


def test_particle_info_original_order_and_fields():
    sc = scenes.smoke_scene()
    color = np.arange(sc.n, dtype=np.int32) * 7
    sc.color = color
    s = sc.make_solver(use_emitter_id=True)
    info = s.particle_info()
    np.testing.assert_array_equal(info['position'], sc.x)
    np.testing.assert_array_equal(info['velocity'], sc.v)
    np.testing.assert_array_equal(info['material'], sc.material)
    np.testing.assert_array_equal(info['color'], color)
    assert info['emitter_ids'].shape == (sc.n,)
    s.step(2e-3)
    info2 = s.particle_info()
    np.testing.assert_array_equal(info2['material'], sc.material)
    np.testing.assert_array_equal(info2['color'], color)
    # particles stay near where they were: the readback is in original order
    assert np.abs(info2['position'] - sc.x).max() < 0.05
    # the reference's scalar-field reads and per-particle size keep working
    assert s.n_particles[None] == sc.n and s.n_particles == sc.n
    assert s.particle._cell_size_bytes == 4 * 28 + 8


def test_seeding_counts_match_reference_rules():
    s = MPMSolver((32, 32, 32))
    s.add_cube((0.2, 0.2, 0.2), (0.3, 0.2, 0.1), s.material_elastic)
    assert s.n_particles == int(8 * 0.3 * 0.2 * 0.1 / (1 / 32)**3 + 1)
    n0 = s.n_particles
    s.add_ellipsoid((0.5, 0.5, 0.5), 0.1, s.material_snow, velocity=(0, -1, 0))
    import math
    assert s.n_particles - n0 == int(math.ceil(4 / 3 * math.pi * (0.1 * 32)**3 * 8))
    x = s.particle_info()['position']
    assert np.all(np.linalg.norm(x[n0:] - 0.5, axis=1) <= 0.1 + 1e-6)
    assert np.all((x[:n0] >= 0.2 - 1e-7) & (x[:n0] <= np.array([0.5, 0.4, 0.3]) + 1e-7))
    st = s.full_state()
    assert torch.all(st['Jp'] == 1)
    assert torch.allclose(st['F'], torch.eye(3, device=st['F'].device).expand_as(st['F']))
    s2 = MPMSolver((16, 16, 16))
    s2.add_cube((0.3, 0.3, 0.3), (0.2, 0.2, 0.2), s2.material_sand)
    assert torch.all(s2.full_state()['Jp'] == 0)
    with pytest.raises(ValueError):
        s2.add_surface_collider((0, 0, 0), (0, 1, 0), surface=s2.surface_sticky, friction=0.5)


def test_nonfinite_positions_raise():
    s = MPMSolver((16, 16, 16))
    x = np.full((100, 3), 0.5, np.float32)
    x[7, 1] = np.nan
    s.add_particles(x, s.material_elastic)
    with pytest.raises(MPMError):
        s.step(1e-3)


def test_window_grows_for_far_particles():
    s = MPMSolver((16, 16, 16), unbounded=True)
    s.add_cube((1.5, 0.5, 0.5), (0.1, 0.1, 0.1), s.material_water, velocity=(5, 0, 0))
    s.step(5e-3)
    x = s.particle_info()['position']
    assert np.all(x[:, 0] > 1.5)


def test_per_particle_E_matches_oracle():
    sc = scenes.smoke_scene()
    n = sc.n
    E = np.exp(np.random.default_rng(0).uniform(np.log(1e4), np.log(1e6), n)).astype(np.float32)
    s = MPMSolver(sc.res, per_particle_E=True)
    for m in range(4):
        sel = sc.material == m
        s.add_particles(sc.x[sel], m, velocity=None, E=torch.as_tensor(E[sel]))
    cfg = oracle_config(s)
    P = O.Particles.seeded(np.concatenate([sc.x[sc.material == m] for m in range(4)]),
                           np.concatenate([sc.material[sc.material == m] for m in range(4)]),
                           E=np.concatenate([E[sc.material == m] for m in range(4)]).astype(np.float64))
    dt = s.default_dt
    R = O.Runner(cfg, P)
    R.run(dt, 20)
    for _ in range(20):
        s.substep(dt)
    g = s.full_state()['x'].cpu().numpy()
    assert np.linalg.norm(g - R.P.x) / np.linalg.norm(R.P.x) < 1e-4


@pytest.mark.parametrize("name", ["mixed_32", "walls_24"])
def test_golden_fixture_one_substep(name):
    """One substep from the committed fixture state (all five materials,
    colliders, walls) against the fixture's float64 outputs; the bound is
    calibrated by the float32 oracle's own error on the same state."""
    import json
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"{name}.npz"))
    pp = json.loads(str(g["postprocess"]))
    s = MPMSolver(tuple(int(r) for r in g["res"]))
    for c in pp[1:]:
        if c["kind"] == 0:
            s.add_surface_collider(c["point"], c["normal"], c.get("surface", 0), c.get("friction", 0.0))
        else:
            s.add_sphere_collider(c["point"], c["radius"], c.get("surface", 0))
    n = g["x"].shape[0]
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float32)
    s.load_state_dict(dict(x=t(g["x"]), v=t(g["v"]), C=t(g["C"]), F=t(g["F"]), Jp=t(g["Jp"]),
                           material=torch.as_tensor(g["material"]), color=torch.zeros(n, dtype=torch.int32)))
    dt = float(g["dt"])
    s.substep(dt)
    st = {k: v.cpu().numpy().astype(np.float64) for k, v in s.full_state().items() if k != 'material'}
    cfg = O.Config(res=tuple(g["res"]), postprocess=pp)
    P32 = O.Particles(*(g[k].astype(np.float32) for k in ("x", "v", "C", "F", "Jp")), g["material"].copy())
    O.substep(cfg, P32, dt)
    vs = np.abs(g["out_v"]).max()
    for f, scale in (("x", 1.0), ("v", vs), ("F", 1.0), ("Jp", 1.0), ("C", 4 * cfg.inv_dx * vs)):
        eg = np.abs(st[f] - g["out_" + f]).max() / scale
        e32 = np.abs(getattr(P32, f) - g["out_" + f]).max() / scale
        assert eg <= max(1e-6, 4 * e32), f"{f}: gpu {eg:.3g} f32 oracle {e32:.3g}"


def test_autotune_picks_a_candidate_and_leaves_state_untouched():
    from taichi_elements_gb300.autotune import CANDIDATES, tune_chunk
    sc = scenes.smoke_scene()
    s = sc.make_solver()
    before = s.full_state()['x'].clone()
    c = tune_chunk(s)
    assert c in CANDIDATES and s.chunk == c
    assert torch.equal(s.full_state()['x'], before)
    s.step(2e-3)
    ref = sc.make_solver(chunk=512)
    ref.step(2e-3)
    assert np.abs(s.particle_info()['position'] - ref.particle_info()['position']).max() < 1e-5


def test_schedule_autotune_applies_a_measured_choice_and_leaves_state_untouched():
    from taichi_elements_gb300.autotune import CANDIDATES, RESORT_CANDIDATES, tune_schedule
    sc = scenes.smoke_scene()
    s = sc.make_solver()
    before = s.full_state()['x'].clone()
    choice = tune_schedule(s)
    assert choice["mode"] in ("frame", "substep") and choice["chunk"] in CANDIDATES
    assert set(map(int, choice["frame_ms"])) == set(RESORT_CANDIDATES)
    assert set(map(int, choice["frame_ms_rolled"])) == set(RESORT_CANDIDATES)
    assert s.fuse_frames == (choice["mode"] == "frame") and s.chunk == choice["chunk"]
    assert s.occupancy == choice["occupancy"]
    if s.fuse_frames:
        assert s.resort_every == choice["resort"]
    assert torch.equal(s.full_state()['x'], before)
    s.step(2e-3)
    ref = sc.make_solver(chunk=512)
    ref.fuse_frames = False
    ref.step(2e-3)
    assert np.abs(s.particle_info()['position'] - ref.particle_info()['position']).max() < 1e-5


def test_adaptive_dt_frames_match_oracle_with_the_same_steps():
    """use_adaptive_dt=True (engine/mpm_solver.py:756-766): each substep's dt
    is min(dt, 0.9 dx / (max grid |v| + 1e-6), time left), the frame's dts
    add up to frame_dt, and the oracle run with the same dts lands on the
    same positions."""
    sc = scenes.smoke_scene()
    sc.v[:] = np.float32([0.0, -6.0, 0.0])  # fast enough for the CFL bound to act
    s = sc.make_solver(use_adaptive_dt=True)
    frame_dt = 4e-3
    s.step(frame_dt)
    first = list(s.last_frame_dts)
    s.step(frame_dt)
    dts = s.last_frame_dts
    assert abs(sum(dts) - frame_dt) < 1e-12
    default = frame_dt / (int(frame_dt / s.default_dt) + 1)
    assert min(dts) < default  # the CFL bound shortened some substeps
    assert all(b <= a + 1e-15 for a, b in zip(dts, dts[1:-1]))  # dt never grows inside a frame
    # oracle: the same two frames substep by substep
    cfg = oracle_config(sc)
    R = O.Runner(cfg, O.Particles.seeded(sc.x, sc.material, v=sc.v))
    for dt in first + dts:
        R.run(dt, 1)
    g = s.full_state()['x'].cpu().numpy().astype(np.float64)
    err = np.linalg.norm(g - R.P.x) / np.linalg.norm(R.P.x)
    assert err < 1e-4, err


def test_empty_cleared_and_refilled_solver():
    s = MPMSolver((16, 16, 16))
    s.step(1e-3)  # no particles: time advances, nothing launches
    assert s.t > 0 and s.n_particles == 0
    s.add_cube((0.3, 0.3, 0.3), (0.2, 0.2, 0.2), s.material_water)
    n1 = s.n_particles
    s.step(1e-3)
    s.clear_particles()
    assert s.n_particles == 0
    s.step(1e-3)
    s.add_cube((0.4, 0.4, 0.4), (0.1, 0.1, 0.1), s.material_elastic)
    s.step(1e-3)
    info = s.particle_info()
    assert 0 < s.n_particles < n1 and np.isfinite(info['position']).all()
    assert (info['material'] == s.material_elastic).all()


def test_unbounded_trajectory_leaving_the_box_matches_oracle():
    s = MPMSolver((16, 16, 16), unbounded=True)
    s.add_cube((0.8, 0.4, 0.4), (0.1, 0.1, 0.1), s.material_elastic, velocity=(4.0, 0.0, 0.0))
    x0 = s.particle_info()['position']
    cfg = oracle_config(s)
    lo = np.array([-16, -64, -16], np.int32)  # nodes; the particles travel +x and fall
    win = O.Window(lo, np.array([96, 96, 64], np.int32))
    R = O.Runner(cfg, O.Particles.seeded(x0, s.material_elastic, v=np.float32([4.0, 0.0, 0.0])), win=win)
    dt = s.default_dt
    for _ in range(60):
        s.substep(dt)
    R.run(dt, 60)
    g = s.full_state()['x'].cpu().numpy().astype(np.float64)
    assert g[:, 0].min() > 1.0  # left the nominal box
    assert np.linalg.norm(g - R.P.x) / np.linalg.norm(R.P.x) < 1e-4


def test_sticky_sphere_and_slip_plane_trajectory():
    sc = scenes.smoke_scene()
    sc.postprocess = [dict(kind=1, surface=0, point=(0.45, 0.3, 0.45), radius=0.1),
                      dict(kind=0, surface=1, point=(0.5, 0.1, 0.5), normal=(0.0, 1.0, 0.2), friction=0.0)]
    s = sc.make_solver()
    cfg = oracle_config(sc)
    R = O.Runner(cfg, O.Particles.seeded(sc.x, sc.material, v=sc.v))
    dt = sc.default_dt
    R.run(dt, 80)
    for _ in range(80):
        s.substep(dt)
    g = s.full_state()['x'].cpu().numpy().astype(np.float64)
    assert np.linalg.norm(g - R.P.x) / np.linalg.norm(R.P.x) < 1e-3


def test_max_velocity_queries():
    """compute_max_velocity (engine/mpm_solver.py:726-735) on the particles'
    velocities and compute_max_grid_velocity (:737-746) on the last
    substep's grid, against numpy on the same data."""
    sc = scenes.smoke_scene()
    s = sc.make_solver()
    assert s.compute_max_velocity() == pytest.approx(float(np.abs(sc.v).max()), rel=1e-7)
    assert s.compute_max_grid_velocity() == 0.0
    s.step(6 * sc.default_dt)
    v = s.particle_info()["velocity"]
    assert s.compute_max_velocity() == float(np.abs(v).max())
    _, vel = gpu_grid(s.views(), "grid_vel")
    assert s.compute_max_grid_velocity(None) == pytest.approx(float(np.abs(vel[:, :3]).max()), rel=1e-7)
