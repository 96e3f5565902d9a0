"""MPMSolver(quant=True): packed particle storage on the GPU
(engine/mpm_solver.py:106-127, :216-262, :415-416).

* mpm_quant_pack / mpm_quant_unpack against the numpy statement of the
  formats (oracle/quant_ref.py): bit-exact words and values.
* Seeding stores the packed values of x, v and F = I.
* Substeps (plain and the fused G2P2G mode) against the float32 oracle run
  with the same quantization from the same decoded state.  The grid after
  P2G comes from identical inputs (rel L-inf 1e-5, as unquantized); stored
  fields can differ where float32 rounding noise crosses a rounding
  boundary of the packed format: at most one unit of the format (x: 2^-19,
  F: 4.1 / 2^15, v: one mantissa unit, 2^-17 of the largest component,
  plus the plain substep's 1e-5 of the largest velocity),
  on under 1% of the particles for x and 5% for F (v's unit sits close to
  float32 noise, so only the bound applies to it).
"""
import numpy as np
import pytest
import torch

from helpers import gpu_grid, oracle_config, rel_inf, window_lookup
from oracle import oracle as O
from oracle import quant_ref as Q
from taichi_elements_gb300 import _lib, scenes
from taichi_elements_gb300.mpm_solver import MPMError
from test_gpu_parity import run_phases

pytestmark = pytest.mark.gpu

X_UNIT = 2.0**-19
F_UNIT = float(Q.F_SCALE)


def test_pack_unpack_bit_exact_against_numpy():
    L = _lib.load()
    rng = np.random.default_rng(1)
    n = 100_003
    rows = rng.standard_normal((28, n)).astype(np.float32)
    rows[0:3] = rng.uniform(-1.99, 1.99, (3, n))
    rows[3:6] = rng.standard_normal((3, n)) * 10.0**rng.uniform(-9, 4, (1, n))
    rows[15:24] = rng.uniform(-4.6, 4.6, (9, n))
    rows[25] = rng.integers(0, 5, n).astype(np.int32).view(np.float32)
    rows[26] = np.arange(n, dtype=np.int32).view(np.float32)
    words = Q.pack(rows)
    dev = torch.device("cuda")
    r = torch.from_numpy(rows).to(dev)
    cap = n + 1000
    pk = torch.zeros((Q.QROWS, cap), dtype=torch.float32, device=dev)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    s = torch.cuda.current_stream().cuda_stream
    # pack into slots [500, 500 + n)
    _lib.check(L.mpm_quant_pack(r.data_ptr(), n, n, pk.data_ptr(), cap, 500, st.data_ptr(), s), "pack")
    got = pk[:, 500:500 + n].cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(got, words)
    assert int(st.item()) == 0
    back = torch.zeros((28, n), dtype=torch.float32, device=dev)
    _lib.check(L.mpm_quant_unpack(pk.data_ptr(), cap, 500, n, back.data_ptr(), n, s), "unpack")
    np.testing.assert_array_equal(back.cpu().numpy().view(np.uint32), Q.unpack(words).view(np.uint32))
    # a position outside [-2, 2) is clamped and flagged
    r[0, 7] = 2.5
    _lib.check(L.mpm_quant_pack(r.data_ptr(), n, n, pk.data_ptr(), cap, 0, st.data_ptr(), s), "pack")
    assert int(st.item()) & _lib.STATUS_OUT_OF_GRID


def test_seeding_stores_packed_values():
    sc = scenes.four_materials_128(per_cube=5000)
    s = sc.make_solver(quant=True)
    st = s.full_state()
    n = sc.n
    xq, vq, Fq = Q.values(sc.x, sc.v, np.broadcast_to(np.eye(3, dtype=np.float32).reshape(1, 9), (n, 9)))
    np.testing.assert_array_equal(st['x'].cpu().numpy(), xq)
    np.testing.assert_array_equal(st['v'].cpu().numpy(), vq)
    np.testing.assert_array_equal(st['F'].cpu().numpy().reshape(n, 9), Fq)
    np.testing.assert_array_equal(st['material'].cpu().numpy(), sc.material)
    info = s.particle_info()
    np.testing.assert_array_equal(info['position'], xq)
    assert s._state[0].shape[0] == _lib.QROWS
    # the position-only decode of the window checks equals the full decode
    torch.testing.assert_close(s._positions_f32(), s._rows_f32()[0:3, :n].t(), rtol=0, atol=0)
    with pytest.raises(ValueError):
        s.add_cube((1.9, 0.5, 0.5), (0.2, 0.1, 0.1), 0)


def _sheared(per_cube):
    sc = scenes.four_materials_128(per_cube=per_cube)
    rng = np.random.default_rng(7)
    v = sc.v.astype(np.float64).copy()
    for m in range(4):
        sel = sc.material == m
        v[sel] += (sc.x[sel] - sc.x[sel].mean(0)) @ rng.uniform(-8, 8, (3, 3)).T
    sc.v = v.astype(np.float32)
    return sc


def _oracle_particles(s):
    st = s.full_state()
    P = O.Particles(*(st[k].cpu().numpy().astype(np.float32) for k in ('x', 'v', 'C', 'F', 'Jp')),
                    st['material'].cpu().numpy().astype(np.int32))
    return P


def _field_errors(g, o, unit):
    d = np.abs(g - o).reshape(g.shape[0], -1).max(1)
    return d.max() / unit, float((d > 0).mean())


def _check_fields(s, P, v_tol_rel=2.0**-17):
    st = s.full_state()
    x = st['x'].cpu().numpy()
    F = st['F'].cpu().numpy()
    v = st['v'].cpu().numpy()
    ex, fx = _field_errors(x, P.x, X_UNIT)
    eF, fF = _field_errors(F, P.F, F_UNIT)
    # v: one mantissa unit of the particle's largest component on top of the
    # plain substep's bound for v (1e-5 of the largest velocity: float32
    # atomics reorder the grid sums)
    dv = np.abs(v - P.v).max(1) - v_tol_rel * np.abs(P.v).max(1)
    ev = dv.max() / np.abs(P.v).max()
    assert ex <= 1.0001 and fx < 0.01, (ex, fx)
    assert eF <= 1.01 and fF < 0.05, (eF, fF)  # one unit up to float32 rounding of q * scale
    assert ev <= 1e-5, ev


@pytest.mark.parametrize("plasticity", [True, False])
def test_quant_substep_matches_quantized_oracle(plasticity):
    sc = _sheared(20000)
    s = sc.make_solver(quant=True, support_plasticity=plasticity)
    dt = sc.default_dt
    for _ in range(20):
        s.substep(dt)
    torch.cuda.synchronize()
    cfg = oracle_config(s)
    cfg.quant = True
    P = _oracle_particles(s)
    P64 = P.astype(np.float64)
    win = O.Window.covering(P.x, cfg.inv_dx)
    _, gm, gmv, _ = O.substep(cfg, P64.copy(), dt, win)
    O.substep(cfg, P, dt, win)
    _, out = run_phases(s, dt)  # grid snapshots between the phases
    coords, mom = out['mom']
    assert rel_inf(mom[:, 0], window_lookup(win, coords, gm)) < 1e-5
    assert rel_inf(mom[:, 1:], window_lookup(win, coords, gmv)) < 1e-5
    _check_fields(s, P)


def test_quant_g2p2g_without_plasticity_matches_quantized_oracle():
    """The configuration of the reference's quantized demos: quant=True,
    use_g2p2g=True, support_plasticity=False."""
    sc = _sheared(8000)
    s = sc.make_solver(quant=True, use_g2p2g=True, support_plasticity=False)
    dt = np.float32(sc.default_dt)
    for _ in range(10):
        s.substep(float(dt))
    torch.cuda.synchronize()
    cfg = oracle_config(s)
    cfg.quant = True
    P = _oracle_particles(s)
    win = O.Window.covering(P.x, cfg.inv_dx, margin=16)
    # the fused substep gathers from the grid velocities of the previous one
    coords, vel = gpu_grid(s.views(), 'grid_vel')
    gv = np.zeros(tuple(win.W) + (3,), np.float32)
    gv[tuple((coords - win.lo[None]).T)] = vel[:, :3]
    R = O.G2P2GRunner(cfg, P, win)
    R.gv = gv.reshape(-1)
    R.last_final = P.n
    s.substep(float(dt))
    R.step(dt)
    torch.cuda.synchronize()
    coords, vel = gpu_grid(s.views(), 'grid_vel')
    ref = window_lookup(win, coords, R.gv.reshape(tuple(win.W) + (3,)))
    # the fused stress reads the rounded F (:417, :441-452): where float32
    # noise moved an entry of F by one unit (4.1 / 2^15) the stress moves
    # with it, about 1e-4 of a node velocity per affected particle
    assert rel_inf(vel[:, :3], ref) < 2e-3
    _check_fields(s, P)


def test_quant_trajectory_and_frames():
    """100 substeps through step() frames (CUDA graphs) stay within rel L2
    1e-3 of the quantized float32 oracle; the stored fields remain values
    of the packed formats; the status word stays clear."""
    sc = _sheared(20000)
    s = sc.make_solver(quant=True)
    cfg = oracle_config(s)
    cfg.quant = True
    P = _oracle_particles(s)
    R = O.Runner(cfg, P)
    dt = sc.default_dt
    R.run(dt, 100)
    for _ in range(100):
        s.substep(dt)
    st = s.full_state()
    x = st['x'].cpu().numpy().astype(np.float64)
    err = np.linalg.norm(x - R.P.x) / np.linalg.norm(R.P.x)
    assert err < 1e-3, err
    xq, vq, Fq = O.quant_values(st['x'].cpu().numpy(), st['v'].cpu().numpy(), st['F'].cpu().numpy())
    np.testing.assert_array_equal(xq, st['x'].cpu().numpy())
    np.testing.assert_array_equal(vq, st['v'].cpu().numpy())
    np.testing.assert_array_equal(Fq, st['F'].cpu().numpy())
    s.step(4e-3)
    s.step(4e-3)
    try:
        s._check_status()
    except MPMError as e:  # pragma: no cover - reported with the message
        pytest.fail(str(e))
