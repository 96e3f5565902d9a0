"""Packed particle storage of quant=True on the CPU: the numpy statement of
the formats (oracle/quant_ref.py) against the C oracle's quantizer, known
answers for the bit layout and rounding, and the quantized oracle substep
(engine/mpm_solver.py:106-127, :216-262, :415-416)."""
import numpy as np

from oracle import oracle as O
from oracle import quant_ref as Q


def _random_state(rng, n):
    x = rng.uniform(-2.2, 2.2, (n, 3)).astype(np.float32)
    v = (rng.standard_normal((n, 3)) * 10.0**rng.uniform(-9, 4, (n, 1))).astype(np.float32)
    F = rng.uniform(-4.6, 4.6, (n, 3, 3)).astype(np.float32)
    # edge cases: ties, range ends, zeros, a subnormal, a huge velocity
    x[:6] = [[0.5 / 524288, -0.5 / 524288, 1.5 / 524288], [2.0 - 1 / 524288, -2.0, 0.0],
             [1.999999, -1.999999, 3.0], [1.0, -1.0, 1 / 524288], [0, 0, 0], [-0.0, 1e-30, -1e-30]]
    v[:5] = [[0, 0, 0], [1e-40, 0, 0], [1.0, 0.5, -0.25], [-0.0, 0, 1e30], [262143.5 / 1024, 1, 0]]
    F[0] = np.eye(3)
    F[1] = 4.1
    return x, v, F


def test_numpy_formats_match_c_oracle_quantizer():
    rng = np.random.default_rng(1)
    x, v, F = _random_state(rng, 50000)
    xq, vq, Fq = Q.values(x, v, F.reshape(-1, 9))
    xo, vo, Fo = O.quant_values(x, v, F)
    np.testing.assert_array_equal(xq, xo)
    np.testing.assert_array_equal(vq, vo)
    np.testing.assert_array_equal(Fq.reshape(-1, 3, 3), Fo)


def test_known_answers():
    # x: 21-bit fixed point of scale 2^-19, ties away from zero, clamped to [-2, 2)
    xq, _, _ = Q.values(np.array([[0.5 / 524288, -0.5 / 524288, 2.5]], np.float32), np.zeros((1, 3), np.float32),
                        np.zeros((1, 9), np.float32))
    np.testing.assert_array_equal(xq, [[1 / 524288, -1 / 524288, 2.0 - 1 / 524288]])
    # v = (1, 0.5, -0.25): max in [2^0, 2^1) -> unit 2^-17, e = 83
    e, m = Q.v_codes(np.array([[1.0, 0.5, -0.25]], np.float32))
    assert e[0] == 83 and list(m[0]) == [1 << 17, 1 << 16, -(1 << 15)]
    # F = I is stored as round(2^15 / 4.1) = 7992 units of 4.1 / 2^15
    _, _, Fq = Q.values(np.zeros((1, 3), np.float32), np.zeros((1, 3), np.float32),
                        np.eye(3, dtype=np.float32).reshape(1, 9))
    assert Q.F_codes(np.float32(1.0)) == 7992
    np.testing.assert_array_equal(Fq[0, [0, 4, 8]], np.float32(7992) * Q.F_SCALE)
    # word layout
    rows = np.zeros((28, 1), np.float32)
    rows[0:3, 0] = [1.0, -1.0, 1 / 524288]
    rows[3:6, 0] = [1.0, 0.5, -0.25]
    rows[15:24, 0] = np.eye(3).reshape(9)
    rows[25, 0] = np.array([3], np.int32).view(np.float32)[0]
    w = Q.pack(rows)[:, 0]
    wx = int(w[0]) | (int(w[1]) << 32)
    assert wx == (1 << 19) | (((1 << 21) - (1 << 19)) << 21) | (1 << 42)
    wv = int(w[2]) | (int(w[3]) << 32)
    assert wv == 83 | ((1 << 17) << 7) | ((1 << 16) << 26) | (((1 << 19) - (1 << 15)) << 45)
    assert w[4] == 7992 and w[6] == 7992 and w[8] == 7992 | (3 << 16)


def test_pack_unpack_round_trip():
    rng = np.random.default_rng(2)
    n = 20000
    x, v, F = _random_state(rng, n)
    rows = rng.standard_normal((28, n)).astype(np.float32)
    rows[0:3], rows[3:6], rows[15:24] = x.T, v.T, F.reshape(n, 9).T
    rows[25] = rng.integers(0, 5, n).astype(np.int32).view(np.float32)
    rows[26] = np.arange(n, dtype=np.int32).view(np.float32)
    w = Q.pack(rows)
    r = Q.unpack(w)
    xq, vq, Fq = Q.values(x, v, F.reshape(n, 9))
    np.testing.assert_array_equal(r[0:3], xq.T)
    np.testing.assert_array_equal(r[3:6], vq.T)
    np.testing.assert_array_equal(r[15:24], Fq.T)
    for k in (6, 14, 24, 25, 26, 27):
        np.testing.assert_array_equal(r[k].view(np.int32), rows[k].view(np.int32))
    np.testing.assert_array_equal(Q.pack(r), w)  # stored values re-encode to the same words


def test_quantized_oracle_substep_stores_representable_values():
    """After a quantized substep (plain and fused), x, v and F are values of
    the packed formats; the fused mode keeps |F| <= F_bound."""
    rng = np.random.default_rng(3)
    n = 3000
    x = 0.3 + 0.4 * rng.random((n, 3))
    mat = rng.integers(0, 5, n)
    for fused in (False, True):
        cfg = O.Config(res=(32, 32, 32), quant=True)
        P = O.Particles.seeded(x, mat, v=rng.uniform(-1, 1, (n, 3)), dtype=np.float32)
        P.F = P.F + np.float32(0.02) * rng.standard_normal((n, 3, 3)).astype(np.float32)
        big = np.nonzero(mat == O.MAT_ELASTIC)[0][:20]
        P.F[big] = np.diag([4.09, 1.0, 1.0]).astype(np.float32)  # beyond F_bound: the fused update clamps
        P.x, P.v, P.F = O.quant_values(P.x, P.v, P.F)
        P.C = (5.0 * rng.standard_normal((n, 3, 3))).astype(np.float32)
        win = O.Window.covering(P.x, cfg.inv_dx, margin=16)
        if fused:
            R = O.G2P2GRunner(cfg, P, win)
            R.step(np.float32(cfg.default_dt))
            R.step(np.float32(cfg.default_dt))
            f_bound = O.quant_values(np.zeros((1, 3), np.float32), np.zeros((1, 3), np.float32),
                                     np.full((1, 3, 3), 4.0, np.float32))[2][0, 0, 0]
            assert np.abs(P.F).max() <= f_bound
        else:
            O.substep(cfg, P, cfg.default_dt, win)
        xq, vq, Fq = O.quant_values(P.x, P.v, P.F)
        np.testing.assert_array_equal(xq, P.x)
        np.testing.assert_array_equal(vq, P.v)
        np.testing.assert_array_equal(Fq, P.F)
