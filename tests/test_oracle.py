"""CPU tests of the oracle: pins against golden fixtures, the independent
numpy restatement, numpy's SVD, and known-answer physics of
engine/mpm_solver.py (taichi-dev/taichi_elements)."""
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


# ------------------------------------------------------------------- SVD --

def test_svd_matches_numpy_and_convention():
    rng = np.random.default_rng(0)
    for t in range(300):
        A = rng.standard_normal((3, 3))
        if t % 3 == 0:
            A = np.eye(3) + 0.05 * rng.standard_normal((3, 3))
        U, s, V = O.svd3(A)
        assert np.abs(U @ np.diag(s) @ V.T - A).max() < 1e-12
        assert abs(np.linalg.det(U) - 1) < 1e-12 and abs(np.linalg.det(V) - 1) < 1e-12
        assert s[0] >= s[1] >= abs(s[2]) - 1e-15
        assert np.sign(s[2]) == np.sign(np.linalg.det(A)) or abs(s[2]) < 1e-14
        ref = np.linalg.svd(A, compute_uv=False)
        np.testing.assert_allclose(np.abs(s), ref, rtol=1e-12, atol=1e-14)


def test_svd_degenerate_and_inverted():
    for A in (np.eye(3), np.diag([2.0, 2.0, 2.0]), np.diag([1.0, 1.0, -1.0]), np.diag([3.0, 0.0, 1.0]),
              np.zeros((3, 3)), np.diag([-1.0, -2.0, 0.5])):
        U, s, V = O.svd3(A)
        assert np.abs(U @ np.diag(s) @ V.T - A).max() < 1e-12
        assert abs(np.linalg.det(U) - 1) < 1e-12 and abs(np.linalg.det(V) - 1) < 1e-12
        if np.linalg.det(A) < 0:
            assert s[2] < 0


def test_svd_float32_accuracy():
    rng = np.random.default_rng(1)
    worst = 0.0
    for _ in range(2000):
        A = (np.eye(3) + 0.02 * rng.standard_normal((3, 3))).astype(np.float32)
        U, s, V = O.svd3(A, np.float32)
        worst = max(worst, np.abs(U.astype(np.float64) @ np.diag(s) @ V.T - A).max())
        assert np.abs(U.T.astype(np.float64) @ U - np.eye(3)).max() < 2e-6
    assert worst < 3e-6


# -------------------------------------------------------- golden fixtures --

@pytest.mark.parametrize("name", ["mixed_32", "walls_24"])
def test_c_oracle_matches_golden(name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    cfg = O.Config(res=tuple(g["res"]), postprocess=json.loads(str(g["postprocess"])))
    P = O.Particles(g["x"].copy(), g["v"].copy(), g["C"].copy(), g["F"].copy(), g["Jp"].copy(),
                    g["material"].copy())
    win, gm, gmv, gv = O.substep(cfg, P, float(g["dt"]))
    nodes = g["grid_nodes"]
    idx = tuple((nodes - win.lo[None]).T)
    assert rel(gm[idx], g["grid_m"]) < 1e-12
    assert rel(gmv[idx], g["grid_mv"]) < 1e-10
    assert rel(gv[idx], g["grid_v"]) < 1e-10
    assert np.isclose(gm.sum(), g["grid_m"].sum(), rtol=1e-12)
    for f in ("x", "v", "C", "F", "Jp"):
        assert rel(getattr(P, f), g["out_" + f]) < 1e-10, f
    # the float32 oracle stays close to the float64 fixture; the fixture's
    # random per-particle strains make the stress divergence a cancellation,
    # so float32 loses a few more digits here than on a smooth state
    P32 = O.Particles(*(g[k].astype(np.float32) for k in ("x", "v", "C", "F", "Jp")), g["material"].copy())
    O.substep(cfg, P32, float(g["dt"]))
    assert np.abs(P32.x - g["out_x"]).max() < 5e-5
    assert np.abs(P32.F - g["out_F"]).max() < 5e-5


def test_c_oracle_matches_numpy_restatement_per_particle_E():
    rng = np.random.default_rng(3)
    cfg = O.Config(res=(32, 32, 32))
    n = 500
    x = 0.3 + 0.4 * rng.random((n, 3))
    mat = rng.integers(0, 4, n)
    E = np.exp(rng.uniform(np.log(1e4), np.log(1e6), n))
    P = O.Particles.seeded(x, mat, v=rng.uniform(-1, 1, (n, 3)), E=E)
    P.F = P.F + 0.01 * rng.standard_normal((n, 3, 3))
    Pn = P.copy()
    out, _ = O.np_substep(cfg, Pn, 1e-4)
    O.substep(cfg, P, 1e-4)
    for f in ("x", "v", "F", "Jp"):
        assert rel(getattr(P, f), getattr(out, f)) < 1e-10, f


def test_c_oracle_matches_numpy_restatement_without_plasticity():
    """support_plasticity=False (engine/mpm_solver.py:62): both restatements
    agree, Jp never changes, sand keeps (I + dt C) F and water restarts from
    F = I (its F[0,0] is det(I + dt C))."""
    rng = np.random.default_rng(5)
    cfg = O.Config(res=(32, 32, 32), support_plasticity=False)
    n = 600
    x = 0.3 + 0.4 * rng.random((n, 3))
    mat = rng.integers(0, 5, n)
    P = O.Particles.seeded(x, mat, v=rng.uniform(-1, 1, (n, 3)))
    P.F = P.F + 0.02 * rng.standard_normal((n, 3, 3))
    P.C = 5.0 * rng.standard_normal((n, 3, 3))
    P.Jp = P.Jp * rng.uniform(0.9, 1.1, n)
    P0 = P.copy()
    Pn = P.copy()
    dt = 1e-4
    out, _ = O.np_substep(cfg, Pn, dt)
    O.substep(cfg, P, dt)
    for f in ("x", "v", "F", "Jp"):
        assert rel(getattr(P, f), getattr(out, f)) < 1e-10, f
    np.testing.assert_array_equal(P.Jp, P0.Jp)
    G = np.eye(3) + dt * P0.C
    sand = mat == O.MAT_SAND
    np.testing.assert_allclose(P.F[sand], (G @ P0.F)[sand], rtol=0, atol=1e-14)
    water = mat == O.MAT_WATER
    np.testing.assert_allclose(P.F[water, 0, 0], np.linalg.det(G[water]), rtol=1e-12)
    # with plasticity the same state takes different Jp and sand F
    Pp = P0.copy()
    O.substep(O.Config(res=(32, 32, 32)), Pp, dt)
    assert not np.array_equal(Pp.Jp, P0.Jp)


def test_g2p2g_oracle_clamps_grid_velocity():
    """The fused mode clamps grid velocities to +-cfl * dx / dt per component
    after gravity (engine/mpm_solver.py:589-598); the gathered particle
    velocities then stay inside the bound."""
    rng = np.random.default_rng(6)
    cfg = O.Config(res=(32, 32, 32))
    n = 2000
    x = 0.4 + 0.2 * rng.random((n, 3))
    dt = cfg.default_dt
    va = 0.9 * cfg.dx / dt
    v0 = np.array([1.4 * va, -1.2 * va, 0.5 * va])
    out = {}
    for cfl in (0.9, 0.0):
        P = O.Particles.seeded(x, O.MAT_WATER, v=v0)
        win = O.Window.covering(P.x, cfg.inv_dx, margin=24)
        R = O.G2P2GRunner(cfg, P, win, v_clamp_cfl=cfl)
        for _ in range(3):
            R.step(dt)
        out[cfl] = np.abs(R.P.v).max(0)
    assert np.all(out[0.9] <= va * (1 + 1e-12))
    assert out[0.0][0] > 1.3 * va


# --------------------------------------------------------- known answers --

def test_single_particle_partition_of_unity():
    """Mass distributed by the quadratic B-spline sums to p_mass; the APIC
    offsets sum to zero (engine/mpm_solver.py:577-584)."""
    cfg = O.Config(res=(16, 16, 16), gravity=(0, 0, 0))
    rng = np.random.default_rng(4)
    for _ in range(20):
        x = 0.3 + 0.4 * rng.random((1, 3))
        P = O.Particles.seeded(x, O.MAT_ELASTIC, v=np.array([[0.3, -0.2, 0.1]]))
        win = O.Window.covering(P.x, cfg.inv_dx)
        gm, gmv = O.p2g(cfg, P, 1e-4, win)
        assert np.isclose(gm.sum(), cfg.p_mass, rtol=1e-14)
        np.testing.assert_allclose(gmv.reshape(-1, 3).sum(0), cfg.p_mass * np.array([0.3, -0.2, 0.1]), rtol=1e-13)


def test_identity_F_gives_zero_elastic_stress():
    """F = I and C = 0: no stress, so P2G momentum is m v only."""
    cfg = O.Config(res=(16, 16, 16))
    x = np.array([[0.51, 0.47, 0.53]])
    for mat in (O.MAT_ELASTIC, O.MAT_SNOW, O.MAT_WATER):
        P = O.Particles.seeded(x, mat, v=np.zeros((1, 3)))
        win = O.Window.covering(P.x, cfg.inv_dx)
        gm, gmv = O.p2g(cfg, P, 1e-4, win)
        assert np.abs(gmv).max() < 1e-18


def test_p2g_conserves_mass_and_momentum():
    rng = np.random.default_rng(5)
    cfg = O.Config(res=(32, 32, 32))
    n = 400
    P = O.Particles.seeded(0.3 + 0.4 * rng.random((n, 3)), rng.integers(0, 5, n), v=rng.uniform(-1, 1, (n, 3)))
    P.F = P.F + 0.02 * rng.standard_normal((n, 3, 3))
    mass = np.where(P.material == O.MAT_WATER, cfg.p_mass * cfg.water_density, cfg.p_mass)
    win = O.Window.covering(P.x, cfg.inv_dx)
    gm, gmv = O.p2g(cfg, P.copy(), 1e-4, win)
    assert np.isclose(gm.sum(), mass.sum(), rtol=1e-13)
    # stress and C terms integrate to zero momentum: sum_i w_ip (x_i - x_p) = 0
    np.testing.assert_allclose(gmv.reshape(-1, 3).sum(0), (mass[:, None] * P.v).sum(0), rtol=1e-10, atol=1e-14)


def test_free_fall_interior_nodes():
    """No stress, uniform v: interior node velocity is v + g dt exactly, and
    G2P returns it with C = 0 (engine/mpm_solver.py:591-593, :714-724)."""
    cfg = O.Config(res=(32, 32, 32))
    rng = np.random.default_rng(6)
    n = 2000
    v0 = np.array([0.2, 0.1, -0.3])
    P = O.Particles.seeded(0.4 + 0.2 * rng.random((n, 3)), O.MAT_ELASTIC, v=np.broadcast_to(v0, (n, 3)))
    dt = 1e-4
    win, gm, gmv, gv = O.substep(cfg, P, dt)
    m = gm > 0
    np.testing.assert_allclose(gv[m], np.broadcast_to(v0 + dt * np.array(cfg.gravity), gv[m].shape), rtol=1e-12)
    np.testing.assert_allclose(P.v, np.broadcast_to(v0 + dt * np.array(cfg.gravity), (n, 3)), rtol=1e-12)
    assert np.abs(P.C).max() < 1e-9


def test_sand_projection_expansion_resets_sigma():
    """tr >= 0 in sand_projection: sigma -> 1 and Jp = tr, F -> rotation
    (engine/mpm_solver.py:331-332)."""
    cfg = O.Config(res=(16, 16, 16))
    x = np.array([[0.5, 0.5, 0.5]])
    P = O.Particles.seeded(x, O.MAT_SAND)
    P.F[0] = np.diag([1.05, 1.02, 1.01])
    win = O.Window.covering(P.x, cfg.inv_dx)
    O.p2g(cfg, P, 1e-4, win)
    np.testing.assert_allclose(P.F[0], np.eye(3), atol=1e-12)
    assert np.isclose(P.Jp[0], np.log(1.05) + np.log(1.02) + np.log(1.01))


def test_snow_clamp_and_hardening():
    cfg = O.Config(res=(16, 16, 16))
    P = O.Particles.seeded(np.array([[0.5, 0.5, 0.5]]), O.MAT_SNOW)
    P.F[0] = np.diag([1.1, 0.9, 1.0])
    win = O.Window.covering(P.x, cfg.inv_dx)
    O.p2g(cfg, P, 1e-4, win)
    s = np.linalg.svd(P.F[0], compute_uv=False)
    assert s.max() <= 1 + 4.5e-3 + 1e-12 and s.min() >= 1 - 2.5e-2 - 1e-12
    assert np.isclose(P.Jp[0], (1.1 / (1 + 4.5e-3)) * (0.9 / (1 - 2.5e-2)))


def test_surface_collider_modes():
    """Sticky zeroes, slip removes the normal component, separate removes
    only the inward part; friction shrinks the tangential speed."""
    base = dict(point=(0.5, 0.5, 0.5), normal=(0, 1, 0))
    cfg0 = O.Config(res=(16, 16, 16), gravity=(0, 0, 0),
                    postprocess=[dict(kind=O.KIND_SURFACE, surface=0, **base)])
    cfg1 = O.Config(res=(16, 16, 16), gravity=(0, 0, 0),
                    postprocess=[dict(kind=O.KIND_SURFACE, surface=1, **base)])
    cfg2 = O.Config(res=(16, 16, 16), gravity=(0, 0, 0),
                    postprocess=[dict(kind=O.KIND_SURFACE, surface=2, friction=0.5, **base)])
    win = O.Window(np.array([0, 0, 0], np.int32), np.array([16, 16, 16], np.int32))
    gm = np.zeros((16, 16, 16))
    gm[4, 4, 4] = 1.0  # node y = 4/16 < 0.5: inside the collider half-space
    gmv = np.zeros((16, 16, 16, 3))
    gmv[4, 4, 4] = (1.0, -2.0, 0.0)
    v0 = O.grid_update(cfg0, gm, gmv, 1e-4, win)[4, 4, 4]
    v1 = O.grid_update(cfg1, gm, gmv, 1e-4, win)[4, 4, 4]
    v2 = O.grid_update(cfg2, gm, gmv, 1e-4, win)[4, 4, 4]
    np.testing.assert_allclose(v0, 0)
    np.testing.assert_allclose(v1, (1.0, 0.0, 0.0))
    np.testing.assert_allclose(v2, (max(0.0, 1.0 - 2.0 * 0.5), 0.0, 0.0))


def test_bounding_box_blocks_outward_motion():
    cfg = O.Config(res=(16, 16, 16), gravity=(0, 0, 0))
    win = O.Window(np.array([0, 0, 0], np.int32), np.array([16, 16, 16], np.int32))
    gm = np.ones((16, 16, 16))
    gmv = np.zeros((16, 16, 16, 3))
    gmv[1, 8, 8] = (-1.0, 0.5, 0.0)
    gmv[14, 8, 8] = (1.0, 0.5, 0.0)
    gv = O.grid_update(cfg, gm, gmv, 1e-4, win)
    np.testing.assert_allclose(gv[1, 8, 8], (0.0, 0.5, 0.0))
    np.testing.assert_allclose(gv[14, 8, 8], (0.0, 0.5, 0.0))


# ---------------------------------------------------------- host logic ---

def test_substep_count_quirk():
    """engine/mpm_solver.py:752-771 can run one more substep than
    int(frame_dt/default_dt)+1 because of float64 accumulation."""
    assert O.substep_count(8e-3, 2e-2 / 64)[0] == 27
    assert O.substep_count(4e-3, 2e-2 / 24)[0] == 6
    n, dt = O.substep_count(1e-3, 1e-3)
    assert n in (2, 3) and math.isclose(dt, 5e-4)


def test_active_sets_bruteforce():
    rng = np.random.default_rng(8)
    x = (0.2 + 0.6 * rng.random((3000, 3))).astype(np.float32)
    inv_dx = 64.0
    pb, counts, gb = O.active_sets(x, inv_dx)
    base = O.base_cells(x, inv_dx)
    assert counts.sum() == len(x)
    touched = set()
    for b in base:
        for a in range(3):
            for c in range(3):
                for d in range(3):
                    touched.add(tuple((b + (a, c, d)) // 4))
    assert set(map(tuple, gb)) == touched


def test_base_cell_float32_rounding():
    """x*inv_dx - 0.5 is two float32 roundings (engine/mpm_solver.py:357)."""
    x = np.array([[0.5078125 - 2**-25, 0.1, 0.9]], dtype=np.float32)
    b = O.base_cells(x, 64.0)
    s = np.float32(x[0, 0]) * np.float32(64.0)
    assert b[0, 0] == int(np.floor(np.float32(s) - np.float32(0.5)))
