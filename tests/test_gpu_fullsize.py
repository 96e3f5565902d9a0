"""Full-size checks of the two large configurations — 16M particles on a
256^3 grid (64 ellipsoids) and 2M particles on a 128^3 grid (four
materials) — through size-independent properties: the binning (particle
blocks, per-block counts, grid-active blocks) bit-exact against a
vectorised numpy restatement of build_pid and the P2G activation rule, and
P2G conserving mass and momentum (the quadratic weights satisfy
sum_i w_i = 1 and sum_i w_i (x_i - x_p) = 0, so the stress terms add no net
momentum), after a few substeps so that v and the stresses are nonzero."""
import numpy as np
import pytest
import torch

from helpers import block_coords, lib_call
from oracle import oracle as O
from taichi_elements_gb300 import scenes

pytestmark = pytest.mark.gpu


def active_sets_vectorised(x, inv_dx):
    base = O.base_cells(x, inv_dx)
    pb, counts = np.unique(np.floor_divide(base, 4), axis=0, return_counts=True)
    lo, hi = np.floor_divide(base, 4), np.floor_divide(base + 2, 4)
    off = lo.min(0) - 1
    span = hi.max(0) - off + 2
    keys = []
    for d in np.array([[a, b, c] for a in (0, 1) for b in (0, 1) for c in (0, 1)]):
        cand = lo + d
        ok = np.all(cand <= hi, axis=1)
        c = cand[ok] - off
        keys.append((c[:, 0] * span[1] + c[:, 1]) * span[2] + c[:, 2])
    k = np.unique(np.concatenate(keys))
    gb = np.stack([k // (span[1] * span[2]), (k // span[2]) % span[1], k % span[2]], 1) + off
    return pb, counts, gb


@pytest.mark.parametrize("scene_fn", [scenes.ellipsoids_256, scenes.four_materials_128])
def test_fullsize_binning_and_p2g_conservation(scene_fn):
    sc = scene_fn()
    s = sc.make_solver()
    dt = sc.default_dt
    for _ in range(3):
        s.substep(dt)
    s._prepare(dt)
    st = torch.cuda.current_stream().cuda_stream
    ws, cap, n = s._ws.data_ptr(), s._cap, s.n_particles
    lib_call(s, "mpm_bin_finalize", ws, cap, n, st)
    v = s.views()
    torch.cuda.synchronize()
    npb, ngb = int(v['counters'][0]), int(v['counters'][1])
    x = s.full_state()['x'].cpu().numpy()
    ref_pb, ref_counts, ref_gb = active_sets_vectorised(x, s.inv_dx)
    np.testing.assert_array_equal(block_coords(v['pblocks'][:npb].cpu().numpy(), v['win_lo'], v['win_nb']), ref_pb)
    np.testing.assert_array_equal(v['pblock_count'][:npb].cpu().numpy(), ref_counts)
    np.testing.assert_array_equal(block_coords(v['gblocks'][:ngb].cpu().numpy(), v['win_lo'], v['win_nb']), ref_gb)
    # P2G alone (a cleared momentum grid), then the grid sums
    cur, nxt = s._state[s._cur], s._state[1 - s._cur]
    lib_call(s, "mpm_p2g", ws, cap, n, cur.data_ptr(), nxt.data_ptr(), dt, st)
    gb = v['gblocks'][:ngb].to(torch.int64)
    addr = (gb[:, None] * 64 + torch.arange(64, device=gb.device)[None]).reshape(-1)
    g = v['grid_mom'][addr].double()
    stt = s.full_state()
    mat = stt['material']
    pm = torch.full((n,), s.p_mass, dtype=torch.float64, device=g.device)
    pm[mat == 0] *= s.water_density
    mass = pm.sum()
    mom = (pm[:, None] * stt['v'].double()).sum(0)
    assert abs(float(g[:, 0].sum() / mass) - 1.0) < 1e-5
    scale = float((pm[:, None] * stt['v'].double().abs()).sum())
    assert float((g[:, 1:].sum(0) - mom).abs().max()) < 1e-4 * scale
    lib_call(s, "mpm_grid_update", ws, cap, dt, st)
    lib_call(s, "mpm_g2p", ws, cap, n, nxt.data_ptr(), dt, None, st)
    s._cur = 1 - s._cur
    torch.cuda.synchronize()
    assert int(s._status.item()) == 0
    assert torch.isfinite(s.full_state()['x']).all()
