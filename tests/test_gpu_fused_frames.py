"""Frames of the plain substep loop run fused (mpm_frame): the particles
after step(frame_dt) against the float64 oracle running the same plain
substeps, for several re-sort intervals (1: every substep sorts, so every
substep is a sort + streaming G2P; 1000: one sort, then fused substeps to
the end of the frame), with CUDA-graph replay against eager launches.

Bounds: the bound table of tests/helpers.py with the float32 calibration of
multi-substep comparisons (a field's bound is 4x the float32 oracle's own
error where that is larger); C on its natural scale 4 inv_dx max |v|.
"""
import numpy as np
import pytest
import torch

from helpers import assert_bounds, oracle_config, rel_inf
from oracle import oracle as O
from taichi_elements_gb300 import scenes

pytestmark = pytest.mark.gpu


def _oracle_frame(sc, count, dt):
    out = {}
    for dtype in (np.float64, np.float32):
        R = O.Runner(oracle_config(sc), O.Particles.seeded(sc.x, sc.material, v=sc.v, dtype=dtype))
        R.run(dt, count)
        out[dtype] = R.P
    return out[np.float64], out[np.float32]


def _errors(s, P64, P32):
    st = {k: v.cpu().numpy().astype(np.float64) for k, v in s.full_state().items() if k != "material"}
    vs = max(np.abs(P64.v).max(), 1e-3)
    cs = 4 * s.inv_dx * vs
    js = max(1.0, np.abs(P64.Jp).max())
    fs = max(1.0, np.abs(P64.F).max())
    return {"x": (rel_inf(st["x"], P64.x, 1.0), rel_inf(P32.x, P64.x, 1.0)),
            "v": (rel_inf(st["v"], P64.v, vs), rel_inf(P32.v, P64.v, vs)),
            "C": (rel_inf(st["C"], P64.C, cs), rel_inf(P32.C, P64.C, cs)),
            "F": (rel_inf(st["F"], P64.F, fs), rel_inf(P32.F, P64.F, fs)),
            "Jp": (rel_inf(st["Jp"], P64.Jp, js), rel_inf(P32.Jp, P64.Jp, js))}


@pytest.mark.parametrize("resort", [1, 3, 8, 1000])
@pytest.mark.parametrize("scene_fn", [scenes.smoke_scene, lambda: scenes.four_materials_128(per_cube=20000)])
def test_fused_frame_matches_oracle(scene_fn, resort):
    sc = scene_fn()
    s = sc.make_solver()
    s.resort_every = resort
    frame_dt = 20 * sc.default_dt * 0.999
    count, dt = s.count_substeps(frame_dt, sc.default_dt)
    s.step(frame_dt)
    assert s.total_substeps == count
    P64, P32 = _oracle_frame(sc, count, dt)
    assert_bounds(f"{sc.name}, fused frame of {count} substeps, re-sort every {resort}", _errors(s, P64, P32),
                  f32_calibrated=True)


def test_fused_frames_graph_replay_matches_eager():
    sc = scenes.smoke_scene()
    a = sc.make_solver(use_cuda_graph=True)
    b = sc.make_solver(use_cuda_graph=False)
    for s in (a, b):
        s.resort_every = 5
    for _ in range(4):  # the third and fourth frames replay a graph
        a.step(4e-3)
        b.step(4e-3)
    torch.cuda.synchronize()
    xa, xb = a.particle_info()["position"], b.particle_info()["position"]
    assert np.abs(xa - xb).max() < 1e-5


@pytest.mark.parametrize("fuse", [True, False])
def test_rolled_kernels_match_oracle(fuse):
    """MpmParams.occupancy = 1 (the fused and P2G kernels' stencil x loops
    rolled, 16 warps per SM): a fused frame, and the per-substep launches,
    against the float64 oracle as above."""
    sc = scenes.four_materials_128(per_cube=20000)
    s = sc.make_solver()
    s.occupancy = 1
    s.fuse_frames = fuse
    s.resort_every = 3
    frame_dt = 20 * sc.default_dt * 0.999
    count, dt = s.count_substeps(frame_dt, sc.default_dt)
    s.step(frame_dt)
    P64, P32 = _oracle_frame(sc, count, dt)
    assert_bounds(f"{sc.name}, rolled kernels, {'fused frame' if fuse else 'per-substep'} of {count} substeps",
                  _errors(s, P64, P32), f32_calibrated=True)
