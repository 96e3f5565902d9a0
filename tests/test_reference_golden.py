"""The oracle against outputs of the reference's own solver code.

tests/golden/ref_*.npz hold what taichi-dev/taichi_elements
engine/mpm_solver.py computes when its kernels run (under the stand-in
``taichi`` module of tests/golden/taichi_standin.py, see
tests/golden/make_reference_golden.py): one substep phase by phase in
float64 and float32, a trajectory through ``MPMSolver.step`` and three
substeps of the fused ``use_g2p2g=True`` mode.  The C oracle in float64 must
reproduce the float64 run to rounding (the two are independent executions of
the same arithmetic), and its float32 build must stay within the float32
run's own distance from float64.  The binning of the oracle (active blocks
and per-block counts) must equal the reference's ``build_pid`` lists.
"""
import numpy as np
import pytest

from helpers import REF_CASES, ref_config, ref_fixture, ref_particles, rel_inf
from oracle import oracle as O


def _lookup(win, nodes, arr):
    return arr[tuple((nodes - win.lo[None]).T)]


@pytest.mark.parametrize("name", REF_CASES)
def test_oracle_float64_reproduces_reference_substep(name):
    g = ref_fixture(name)
    cfg = ref_config(g)
    P = ref_particles(g)
    dt = float(g["dt"])
    win, gm, gmv, gv = O.substep(cfg, P, dt)
    nodes = g["f64_grid_nodes"]
    # every node with mass is a node of the reference's active blocks
    assert np.isclose(_lookup(win, nodes, gm).sum(), gm.sum(), rtol=1e-13)
    # 1e-10: the two float64 SVDs agree to ~1e-11 in U V^T where singular
    # values repeat (degenerate_24); elsewhere the fields agree to ~1e-14
    assert rel_inf(_lookup(win, nodes, gm), g["f64_grid_m"]) < 1e-13
    assert rel_inf(_lookup(win, nodes, gmv), g["f64_grid_mv"]) < 1e-10
    assert rel_inf(_lookup(win, nodes, gv), g["f64_grid_v"]) < 1e-10
    for f in ("x", "v", "C", "F", "Jp"):
        if "f64_out_" + f in g:
            assert rel_inf(getattr(P, f), g["f64_out_" + f]) < 1e-10, f
    # compute_max_velocity (:726-735) is the largest |v_i| after G2P
    assert abs(np.abs(P.v).max() - float(g["f64_maxv"])) <= 1e-10 * float(g["f64_maxv"])


@pytest.mark.parametrize("name", REF_CASES)
def test_oracle_binning_equals_reference_build_pid(name):
    g = ref_fixture(name)
    cfg = ref_config(g)
    pb, counts, gb = O.active_sets(g["in_x"], cfg.inv_dx)
    np.testing.assert_array_equal(pb, g["f64_pblocks"])
    np.testing.assert_array_equal(counts, g["f64_pcounts"])
    # the reference's grid-active blocks: those its P2G writes activate
    np.testing.assert_array_equal(gb, g["f64_gblocks"])
    # float32 positions bin identically in both precisions of the reference
    np.testing.assert_array_equal(g["f32_pblocks"], g["f64_pblocks"])


# The float32 oracle against the reference's float32 run: both round every
# operation to float32 but sum in different orders (and the reference's
# SVD is a different algorithm), so they agree to float32 noise; the bound is
# 8x the reference float32 run's own distance from float64 on each field,
# and no tighter than 2e-6: the stand-in's float32 SVD is a float64 SVD
# rounded to float32, more accurate than a float32 SVD (Taichi's or the
# oracle's Jacobi sweeps), whose error reaches F through snow's
# F = U clamp(sigma) V^T at about 1e-6.
@pytest.mark.parametrize("name", REF_CASES)
def test_oracle_float32_within_reference_float32_noise(name):
    g = ref_fixture(name)
    cfg = ref_config(g)
    P = ref_particles(g, np.float32)
    win, gm, gmv, gv = O.substep(cfg, P, float(g["dt"]))
    nodes = g["f32_grid_nodes"]
    vs = max(np.abs(g["f64_out_v"]).max(), 1e-3)
    pairs = [("grid_m", _lookup(win, nodes, gm), None), ("grid_mv", _lookup(win, nodes, gmv), None),
             ("grid_v", _lookup(win, nodes, gv), None), ("out_x", P.x, 1.0), ("out_v", P.v, vs),
             ("out_F", P.F, 1.0), ("out_C", P.C, None)]
    for key, ours, scale in pairs:
        ref_noise = rel_inf(g["f32_" + key], g["f64_" + key], scale)
        err = rel_inf(ours, g["f64_" + key], scale)
        assert err <= max(8 * ref_noise, 2e-6), f"{key}: {err:.3g} vs reference float32 {ref_noise:.3g}"


@pytest.mark.parametrize("name", REF_CASES)
def test_oracle_trajectory_reproduces_reference_step(name):
    """MPMSolver.step(frame_dt) itself: the substep count of its float64 loop
    and the particles after the frame."""
    g = ref_fixture(name)
    if "traj_x" not in g:
        pytest.skip("no trajectory for this state")
    cfg = ref_config(g)
    count, dt = O.substep_count(float(g["traj_frame_dt"]), cfg.default_dt)
    assert count == int(g["traj_substeps"])
    P = ref_particles(g)
    R = O.Runner(cfg, P, nthreads=1)
    R.run(dt, count)
    for f in ("x", "v", "C", "F", "Jp"):
        if "traj_" + f in g:
            assert rel_inf(getattr(R.P, f), g["traj_" + f]) < 1e-11, f


def test_oracle_fused_mode_reproduces_reference_g2p2g():
    """use_g2p2g=True (g2p2g :363-485 and its loop :773-787): grid velocities
    carried between substeps, the first substep skipping the gather, the
    velocity clamp of v_clamp_g2p2g."""
    g = ref_fixture("g2p2g_24")
    cfg = ref_config(g)
    P = ref_particles(g)
    win = O.Window.covering(P.x, cfg.inv_dx)
    R = O.G2P2GRunner(cfg, P, win, v_clamp_cfl=0.9)
    dt = float(g["substep_dt"])
    for k in range(3):
        gm, gv = R.step(dt)
        nodes = g[f"sub{k}_grid_nodes"]
        assert rel_inf(_lookup(win, nodes, gm), g[f"sub{k}_grid_m"]) < 1e-12
        assert rel_inf(_lookup(win, nodes, gv), g[f"sub{k}_grid_v"]) < 1e-11
        for f in ("x", "v", "F", "Jp"):
            assert rel_inf(getattr(P, f), g[f"sub{k}_{f}"]) < 1e-11, (k, f)
