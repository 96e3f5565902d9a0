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


@pytest.mark.gpu
def test_batched_64_scenes_match_oracle():
    """The 64-scene batch of the batched benchmark (grids 32-96^3, 8K-300K
    particles in 1-3 cubes, four materials, per-scene E from 1e4 to 1e6),
    with a collider per scene and initial velocities added, 8 substeps in
    one batched frame, launched per substep and as fused frames; every scene
    against the float64 oracle run with that
    scene's own constants, dt and colliders.  Positions on unit scale and
    velocities on the scene's largest speed, relative L-inf, with the bound
    table of tests/helpers.py raised to 4x the float32 oracle's own error
    where that is larger (eight substeps of float32 rounding)."""
    import os
    from helpers import assert_bounds, rel_inf
    from oracle import oracle as O
    from taichi_elements_gb300.batched import BatchedMPM
    raw = scenes.batched_scenes()
    rng = np.random.default_rng(44)
    bs = []
    for i, sc in enumerate(raw):
        v = np.broadcast_to(rng.uniform(-1, 1, 3).astype(np.float32), (sc.n, 3))
        if i % 3 == 0:
            pp = [dict(kind=0, surface=2, point=(0.5, 0.35, 0.5), normal=(0.2, 1.0, 0.1), friction=0.3)]
        elif i % 3 == 1:
            pp = [dict(kind=1, surface=1, point=(0.5, 0.5, 0.5), radius=0.15)]
        else:
            pp = [dict(kind=0, surface=1, point=(0.5, 0.2, 0.5), normal=(0.0, 1.0, 0.0), friction=0.0)]
        bs.append(BatchScene(sc.res, sc.x, sc.material, v, E_scale=sc.E_scale, postprocess=pp))
    nsub = 8
    from taichi_elements_gb300._lib import ROW_V, ROW_X
    # per-substep launches (the default), and fused frames (mpm_batch_frame,
    # re-sorted every 3 substeps, the 16-warp fused kernel)
    runs_gpu = {}
    for label, fuse in (("per-substep", False), ("fused frames", True)):
        B = BatchedMPM(bs, use_cuda_graph=False)
        if fuse:
            B.fuse_frames, B.resort_every, B.occupancy = True, 3, 1
        B.substeps(nsub)
        B.check_status()
        runs_gpu[label] = (B._gather(ROW_X, 3).cpu().numpy(), B._gather(ROW_V, 3).cpu().numpy(),
                           [int(o) for o in B.offsets])
        del B
    worst = {label: {"x": (0.0, 0.0), "v": (0.0, 0.0)} for label in runs_gpu}
    threads = os.cpu_count() or 1
    for i, s in enumerate(bs):
        cfg = O.Config(res=s.res, E_scale=s.E / 1e6, gravity=s.gravity, postprocess=s.postprocess)
        runs = {}
        for dtype in (np.float64, np.float32):
            R = O.Runner(cfg, O.Particles.seeded(s.x, s.material, v=s.v, dtype=dtype), nthreads=threads)
            R.run(s.dt, nsub)
            runs[dtype] = R.P
        P64, P32 = runs[np.float64], runs[np.float32]
        vs = max(np.abs(P64.v).max(), 1e-3)
        for label, (X, V, off) in runs_gpu.items():
            errs = {"x": (rel_inf(X[off[i]:off[i + 1]], P64.x, 1.0), rel_inf(P32.x, P64.x, 1.0)),
                    "v": (rel_inf(V[off[i]:off[i + 1]], P64.v, vs), rel_inf(P32.v, P64.v, vs))}
            assert_bounds(f"{label}, scene {i} ({s.n} particles, {s.res[0]}^3, E {s.E:.3g})", errs,
                          f32_calibrated=True)
            for k in worst[label]:
                if errs[k][0] > worst[label][k][0]:
                    worst[label][k] = errs[k]
    for label, w in worst.items():
        print(f"\n{label}: worst over {len(bs)} scenes: x {w['x'][0]:.2e} (f32 {w['x'][1]:.1e}), "
              f"v {w['v'][0]:.2e} (f32 {w['v'][1]:.1e})")


@pytest.mark.gpu
@pytest.mark.parametrize("resort,occupancy", [(1, 0), (3, 0), (24, 0), (3, 1), (24, 1)])
def test_batched_frames_match_per_substep_launches(resort, occupancy):
    """mpm_batch_frame (fused frames, re-sorted about every `resort`
    substeps; both register budgets of the fused kernel) against the batch's
    per-substep launches: the same arithmetic in another order, so positions
    agree to float32 rounding and every scene's max |v| per substep
    matches."""
    from taichi_elements_gb300._lib import ROW_X
    from taichi_elements_gb300.batched import BatchedMPM
    bs = small_scenes()
    a = BatchedMPM(bs, use_cuda_graph=False)
    b = BatchedMPM(bs, use_cuda_graph=False)
    a.fuse_frames = True
    a.resort_every = resort
    a.occupancy = occupancy
    b.fuse_frames = False
    nsub = 10
    a.substeps(nsub)
    b.substeps(nsub)
    a.check_status()
    b.check_status()
    xa, xb = a._gather(ROW_X, 3).cpu().numpy(), b._gather(ROW_X, 3).cpu().numpy()
    assert np.abs(xa - xb).max() < 1e-5
    ma, mb = a.max_velocity(nsub), b.max_velocity(nsub)
    assert ma.shape == (nsub, len(bs))
    assert np.allclose(ma, mb, rtol=1e-4, atol=1e-6)
