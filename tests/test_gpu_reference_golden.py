"""The GPU engine against outputs of the reference's own solver code.

tests/golden/ref_*.npz hold what taichi-dev/taichi_elements
engine/mpm_solver.py computes when its kernels run (see
tests/golden/make_reference_golden.py).  Here the engine starts from the same
state through the drop-in API and runs one substep phase by phase through the
C ABI; every field is compared with the reference's float64 run.  The raw
errors are printed (pytest -s shows them).

Bounds (relative L-inf against the reference float64 run; grid fields over
the nodes of the reference's active blocks, scaled by the field's largest
magnitude; x and F on unit scale; v on the largest particle speed):

  field    bound   source
  binning  exact   active blocks, per-block counts, grid-active blocks
  grid_m   1e-5    target (grid mass)
  grid_mv  1e-5    target (grid momentum)
  x        1e-6    target
  F        1e-6    target
  Jp       1e-6    same scale as F
  v        1e-5    calibrated: the reference's own float32 run is 0.5-2.8e-6
                   from its float64 run on these states (reordered float32
                   sums of 27 nodes), above the target 1e-6
  grid_v   1e-5    calibrated: v = mv / m divides two 1e-6-accurate sums;
                   the reference's float32 run reaches 5.7e-6
  C        2e-5    calibrated: C sums 27 terms of |w v dpos| * 4 inv_dx; the
                   reference's float32 run reaches 3.1e-6

Trajectories through step(frame_dt) (6 substeps): positions within rel L2
1e-5 of the reference's float64 trajectory (the target 1e-3 is for 100
substeps).  The fused mode is compared after each of three substeps with the
plain bounds, except F and Jp at 2e-6 or 4x the float32 oracle's own error
after that substep where larger: each substep multiplies them by a
float32-rounded update, so their error grows by about 1e-6 per substep (the
float32 oracle: 1.4e-6 for F and 2.2e-6 for Jp after the third).
"""
import numpy as np
import pytest
import torch

from helpers import REF_CASES, block_coords, ref_config, ref_fixture, ref_kw, ref_particles, rel_inf, run_phases
from oracle import oracle as O
from taichi_elements_gb300.mpm_solver import MPMSolver

pytestmark = pytest.mark.gpu

BOUND = {"grid_m": 1e-5, "grid_mv": 1e-5, "grid_v": 1e-5, "x": 1e-6, "F": 1e-6, "Jp": 1e-6, "v": 1e-5, "C": 2e-5}


def make_solver(g, **extra):
    import ast
    kw = dict(ref_kw(g))
    kw.update(extra)
    s = MPMSolver(tuple(int(r) for r in g["res"]), **kw)
    for c in ast.literal_eval(str(g["postprocess"])):
        if c["kind"] == "surface":
            s.add_surface_collider(c["point"], c["normal"], surface=c["surface"], friction=c["friction"])
        else:
            s.add_sphere_collider(c["center"], c["radius"], surface=c["surface"])
    n = int(g["n"])
    st = {"x": torch.as_tensor(g["in_x"]), "v": torch.as_tensor(g["in_v"]),
          "C": torch.as_tensor(g["in_C"] if "in_C" in g else np.zeros((n, 3, 3), np.float32)),
          "F": torch.as_tensor(g["in_F"]),
          "Jp": torch.as_tensor(g["in_Jp"] if "in_Jp" in g else np.ones(n, np.float32)),
          "material": torch.as_tensor(g["in_material"]), "color": torch.full((n,), 0xFFFFFF, dtype=torch.int32)}
    s.load_state_dict(st)
    return s


# States whose float32 evaluation is ill-conditioned even in the reference:
# degenerate_24 (inverted, rank-deficient, repeated-singular-value F for every
# material) exists to pin the SVD sign convention, where a wrong convention
# would make errors of order 1.  The reference's own float32 run is up to
# 6e-4 from its float64 run there, so the bound is 8x that distance.
NOISY = {"degenerate_24"}


def _reference_f32_noise(g):
    vs = max(np.abs(g["f64_out_v"]).max(), 1e-3)
    out = {"grid_m": rel_inf(g["f32_grid_m"], g["f64_grid_m"]), "grid_mv": rel_inf(g["f32_grid_mv"], g["f64_grid_mv"]),
           "grid_v": rel_inf(g["f32_grid_v"], g["f64_grid_v"]),
           "x": rel_inf(g["f32_out_x"], g["f64_out_x"], 1.0), "v": rel_inf(g["f32_out_v"], g["f64_out_v"], vs),
           "F": rel_inf(g["f32_out_F"], g["f64_out_F"], max(1.0, np.abs(g["f64_out_F"]).max())),
           "C": rel_inf(g["f32_out_C"], g["f64_out_C"])}
    out["Jp"] = rel_inf(g["f32_out_Jp"], g["f64_out_Jp"], max(1.0, np.abs(g["f64_out_Jp"]).max())) \
        if "f32_out_Jp" in g else 0.0
    return out


def _lookup(coords, ref_nodes, ref_vals):
    """Reference values at the engine's node coordinates (0 where the
    reference has no active block)."""
    index = {tuple(c): k for k, c in enumerate(ref_nodes)}
    out = np.zeros((len(coords),) + ref_vals.shape[1:])
    hit = np.zeros(len(coords), bool)
    for k, c in enumerate(coords):
        j = index.get(tuple(c))
        if j is not None:
            out[k] = ref_vals[j]
            hit[k] = True
    return out, hit


@pytest.mark.parametrize("name", REF_CASES)
def test_gpu_substep_matches_reference_run(name):
    g = ref_fixture(name)
    s = make_solver(g)
    dt = float(g["dt"])
    views, out = run_phases(s, dt)
    npb, ngb = int(views["counters"][0]), int(views["counters"][1])
    pb = block_coords(views["pblocks"][:npb].cpu().numpy(), views["win_lo"], views["win_nb"])
    gb = block_coords(views["gblocks"][:ngb].cpu().numpy(), views["win_lo"], views["win_nb"])
    np.testing.assert_array_equal(pb, g["f64_pblocks"])
    np.testing.assert_array_equal(views["pblock_count"][:npb].cpu().numpy(), g["f64_pcounts"])
    np.testing.assert_array_equal(gb, g["f64_gblocks"])
    coords, mom = out["mom"]
    _, vel = out["vel"]
    ref_m, hit = _lookup(coords, g["f64_grid_nodes"], g["f64_grid_m"])
    assert hit.all()  # the engine's grid-active nodes are the reference's
    ref_mv, _ = _lookup(coords, g["f64_grid_nodes"], g["f64_grid_mv"])
    ref_v, _ = _lookup(coords, g["f64_grid_nodes"], g["f64_grid_v"])
    st = s.full_state()
    vs = max(np.abs(g["f64_out_v"]).max(), 1e-3)
    err = {"grid_m": rel_inf(mom[:, 0], ref_m), "grid_mv": rel_inf(mom[:, 1:], ref_mv),
           "grid_v": rel_inf(vel[:, :3], ref_v),
           "x": rel_inf(st["x"].cpu().numpy(), g["f64_out_x"], 1.0),
           "v": rel_inf(st["v"].cpu().numpy(), g["f64_out_v"], vs),
           "F": rel_inf(st["F"].cpu().numpy(), g["f64_out_F"], max(1.0, np.abs(g["f64_out_F"]).max())),
           "C": rel_inf(st["C"].cpu().numpy(), g["f64_out_C"])}
    if "f64_out_Jp" in g:
        err["Jp"] = rel_inf(st["Jp"].cpu().numpy(), g["f64_out_Jp"], max(1.0, np.abs(g["f64_out_Jp"]).max()))
    bound = dict(BOUND)
    if name in NOISY:  # ill-conditioned states: 8x the reference float32 run's own error
        noise = _reference_f32_noise(g)
        bound = {k: max(BOUND[k], 8 * noise[k]) for k in BOUND}
    print(f"\n{name}: " + " ".join(f"{k}={v:.2e}/{bound[k]:.1e}" for k, v in err.items()))
    for k, e in err.items():
        assert e <= bound[k], f"{k}: {e:.3g} > {bound[k]:.1e}"
    assert int(s._status.item()) == 0


@pytest.mark.parametrize("name", REF_CASES)
def test_gpu_step_trajectory_matches_reference_step(name):
    g = ref_fixture(name)
    if "traj_x" not in g:
        pytest.skip("no trajectory for this state")
    s = make_solver(g)
    s.step(float(g["traj_frame_dt"]))
    assert s.total_substeps == int(g["traj_substeps"])
    x = s.particle_info()["position"].astype(np.float64)
    ref = g["traj_x"]
    l2 = float(np.linalg.norm(x - ref) / np.linalg.norm(ref))
    print(f"\n{name}: {s.total_substeps} substeps, positions rel L2 {l2:.2e}, "
          f"L-inf {np.abs(x - ref).max():.2e}")
    assert l2 <= 1e-5


def test_gpu_fused_mode_matches_reference_g2p2g():
    g = ref_fixture("g2p2g_24")
    s = make_solver(g, use_g2p2g=True)
    dt = float(g["substep_dt"])
    # the float32 oracle's own F and Jp error after each substep calibrates
    # their bound: 2e-6, or 4x that error where larger (it grows about 1e-6
    # per substep; the oracle reaches 1.4e-6 and 2.2e-6 after the third)
    cfg = ref_config(g)
    P32 = ref_particles(g, np.float32)
    R32 = O.G2P2GRunner(cfg, P32, O.Window.covering(np.asarray(g["in_x"], np.float64), cfg.inv_dx, margin=16))
    for k in range(3):
        s.step(dt)
        R32.step(dt)
        st = s.full_state()
        vs = max(np.abs(g[f"sub{k}_v"]).max(), 1e-3)
        ex = rel_inf(st["x"].cpu().numpy(), g[f"sub{k}_x"], 1.0)
        ev = rel_inf(st["v"].cpu().numpy(), g[f"sub{k}_v"], vs)
        eF = rel_inf(st["F"].cpu().numpy(), g[f"sub{k}_F"], 1.0)
        eJ = rel_inf(st["Jp"].cpu().numpy(), g[f"sub{k}_Jp"], 1.0)
        bF = max(2e-6, 4 * rel_inf(R32.P.F, g[f"sub{k}_F"], 1.0))
        bJ = max(2e-6, 4 * rel_inf(R32.P.Jp, g[f"sub{k}_Jp"], 1.0))
        print(f"\ng2p2g substep {k}: x={ex:.2e} v={ev:.2e} F={eF:.2e} (bound {bF:.1e}) Jp={eJ:.2e} (bound {bJ:.1e})")
        assert ex <= BOUND["x"] and ev <= BOUND["v"] and eF <= bF and eJ <= bJ


@pytest.mark.parametrize("name", REF_CASES)
def test_gpu_max_velocity_matches_reference(name):
    """compute_max_velocity (engine/mpm_solver.py:726-735): the largest
    |v_i| over the particles after G2P, as the substep records it."""
    g = ref_fixture(name)
    s = make_solver(g)
    s.substep(float(g["dt"]))
    got = float(s._maxv[0].item())
    ref = float(g["f64_maxv"])
    print(f"\n{name}: max |v| {got:.7g} (reference {ref:.7g})")
    assert abs(got - ref) <= (8 * max(_reference_f32_noise(g)["v"], 1e-6)) * ref
