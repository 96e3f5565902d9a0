"""numpy restatement of the packed particle storage of quant=True - TEST
INFRASTRUCTURE (used only by tests/).

The reference declares its particle fields with Taichi's quantized types
(taichi-dev/taichi_elements engine/mpm_solver.py:106-127, bit-packed at
:216-262): x as ``quant.fixed(21, max_value=2.0)``, v as
``quant.float(exp=7, frac=19)`` with a shared exponent, F as
``quant.fixed(16, max_value=F_bound + 0.1)`` and the material as a 16-bit
unsigned integer.  This module states the formats the GB300 engine uses for
them, bit for bit:

* x: q = round(x * 2^19) in [-2^20, 2^20 - 1]; word pair
  q0 | q1 << 21 | q2 << 42 (21-bit two's complement fields);
* v: block floating point; with M = max |v_d| in [2^(k-1), 2^k), the unit is
  2^u, u = clamp(k - 18, -100, 27), m_d = round(v_d / 2^u) (a carry of the
  largest to 2^18 moves to u + 1), |m_d| <= 2^18 - 1; word pair
  (u + 100) | m0 << 7 | m1 << 26 | m2 << 45 (19-bit two's complement);
* F: q = round(F * float32(2^15 / 4.1)) in [-32768, 32767], value
  q * float32(4.1 / 2^15); words (F00,F01) (F02,F10) (F11,F12) (F20,F21)
  (F22, material), low half first;
* rows 9 Jp, 10 id, 11 Young's modulus, 12-20 C as float32 bits.

round() is round to nearest with ties away from zero, evaluated in float32
as the device does (product rounded, then + 0.5 with the sign, truncated).

Parity with the reference's quantized storage is unpinned: Taichi (which
owns the bit-level rounding of its quantized types) is not importable here.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32
QROWS = 21
X_INV, X_SCALE = F32(524288.0), F32(1.0 / 524288.0)
F_INV, F_SCALE = F32(32768.0 / 4.1), F32(4.1 / 32768.0)
V_BIAS = 100


def q_round(s: np.ndarray) -> np.ndarray:
    s = np.asarray(s, F32)
    t = (s + np.copysign(F32(0.5), s).astype(F32)).astype(F32)
    # the device's float -> int32 conversion saturates
    return np.clip(np.trunc(t.astype(np.float64)), -2.0**31, 2.0**31 - 1).astype(np.int64)


def _codes(a, inv, lo, hi):
    a = np.asarray(a, F32)
    fin = np.isfinite(a)
    q = q_round(np.where(fin, a, F32(0)) * inv)
    return np.where(fin, np.clip(q, lo, hi), 0)


def x_codes(x: np.ndarray) -> np.ndarray:
    """Non-finite positions store 0."""
    return _codes(x, X_INV, -(1 << 20), (1 << 20) - 1)


def F_codes(F: np.ndarray) -> np.ndarray:
    """Out-of-range entries saturate, non-finite ones store 0."""
    return _codes(F, F_INV, -32768, 32767)


def v_codes(v: np.ndarray):
    """(e, m) of velocities (n,3) float32: exponent codes (n,) and mantissas (n,3)."""
    v = np.asarray(v, F32)
    fin = np.isfinite(v).all(1)
    v = np.where(fin[:, None], v, F32(0))  # a non-finite velocity stores 0
    M = np.abs(v).max(1)
    k = ((M.view(np.uint32) >> 23) & 0xFF).astype(np.int64) - 126
    u = np.clip(k - 18, -V_BIAS, 127 - V_BIAS)
    m = q_round(v * np.ldexp(F32(1), -u).astype(F32)[:, None])
    carry = (np.abs(m).max(1) >= (1 << 18)) & (u < 127 - V_BIAS)
    if carry.any():
        u = u + carry
        m = q_round(v * np.ldexp(F32(1), -u).astype(F32)[:, None])
    m = np.clip(m, -((1 << 18) - 1), (1 << 18) - 1)
    return u + V_BIAS, m


def values(x, v, F):
    """The stored values (float32) of x (n,3), v (n,3), F (n,3,3)."""
    e, m = v_codes(v)
    vq = (m.astype(F32) * np.ldexp(F32(1), e - V_BIAS).astype(F32)[:, None]).astype(F32)
    return x_codes(x).astype(F32) * X_SCALE, vq, (F_codes(F).astype(F32) * F_SCALE).astype(F32)


def _split64(w: np.ndarray):
    w = w.astype(np.uint64)
    return (w & np.uint64(0xFFFFFFFF)).astype(np.uint32), (w >> np.uint64(32)).astype(np.uint32)


def pack(rows: np.ndarray) -> np.ndarray:
    """float32 row layout (28, n) -> packed words (21, n) uint32."""
    rows = np.ascontiguousarray(rows, F32)
    n = rows.shape[1]
    out = np.zeros((QROWS, n), np.uint32)
    qx = x_codes(rows[0:3].T)
    wx = np.zeros(n, np.uint64)
    for d in range(3):
        wx |= (qx[:, d].astype(np.uint64) & np.uint64(0x1FFFFF)) << np.uint64(21 * d)
    out[0], out[1] = _split64(wx)
    e, m = v_codes(rows[3:6].T)
    wv = e.astype(np.uint64)
    for d in range(3):
        wv |= (m[:, d].astype(np.uint64) & np.uint64(0x7FFFF)) << np.uint64(7 + 19 * d)
    out[2], out[3] = _split64(wv)
    qf = F_codes(rows[15:24].T).astype(np.int64) & 0xFFFF
    mat = rows[25].view(np.int32).astype(np.int64) & 0xFFFF
    halves = np.concatenate([qf, mat[:, None]], 1).astype(np.uint32)
    for r in range(5):
        out[4 + r] = halves[:, 2 * r] | (halves[:, 2 * r + 1] << np.uint32(16))
    out[9] = rows[24].view(np.uint32)
    out[10] = rows[26].view(np.uint32)
    out[11] = rows[27].view(np.uint32)
    out[12:21] = rows[6:15].view(np.uint32)
    return out


def _sext(v: np.ndarray, bits: int) -> np.ndarray:
    v = v.astype(np.int64) & ((1 << bits) - 1)
    return np.where(v >= (1 << (bits - 1)), v - (1 << bits), v)


def unpack(words: np.ndarray) -> np.ndarray:
    """packed words (21, n) -> float32 row layout (28, n)."""
    words = np.ascontiguousarray(words, np.uint32)
    n = words.shape[1]
    rows = np.zeros((28, n), F32)
    wx = words[0].astype(np.uint64) | (words[1].astype(np.uint64) << np.uint64(32))
    for d in range(3):
        q = _sext((wx >> np.uint64(21 * d)).astype(np.int64), 21)
        rows[d] = q.astype(F32) * X_SCALE
    wv = words[2].astype(np.uint64) | (words[3].astype(np.uint64) << np.uint64(32))
    e = (wv & np.uint64(127)).astype(np.int64)
    sc = np.ldexp(F32(1), e - V_BIAS).astype(F32)
    for d in range(3):
        m = _sext((wv >> np.uint64(7 + 19 * d)).astype(np.int64), 19)
        rows[3 + d] = m.astype(F32) * sc
    for a in range(9):
        wd = words[4 + a // 2]
        h = (wd >> np.uint32(16)) if a & 1 else (wd & np.uint32(0xFFFF))
        rows[15 + a] = _sext(h.astype(np.int64), 16).astype(F32) * F_SCALE
    rows[25] = (words[8] >> np.uint32(16)).astype(np.int32).view(F32)
    rows[24] = words[9].view(F32)
    rows[26] = words[10].view(F32)
    rows[27] = words[11].view(F32)
    rows[6:15] = words[12:21].view(F32)
    return rows
