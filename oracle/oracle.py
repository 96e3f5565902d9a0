"""Python front-end of the MLS-MPM oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/, by ``__graft_entry__.smoke()`` and by the CPU-baseline leg of
``bench.py``; never by the product package.  It wraps two independent CPU
restatements of taichi-dev/taichi_elements engine/mpm_solver.py:

* ``liboracle`` (mpm_oracle.c / mpm_oracle_impl.h): C, float64 and float32
  builds, OpenMP; also the timed CPU baseline.
* ``np_substep``: a vectorised numpy float64 restatement using
  ``numpy.linalg.svd`` (with the rotation sign convention fixed up), used to
  cross-check the C restatement.

Parity is unpinned against the reference's own outputs: the reference ships
no golden vectors and its Taichi runtime (taichi==1.1.0, not vendored) cannot
be imported on these machines.  The restatement is pinned by known-answer
physics tests (partition of unity, conservation, free fall, zero stress at
F = I) and by agreement of the two restatements.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
import os
import subprocess
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libmpm_oracle.so"

MAT_WATER, MAT_ELASTIC, MAT_SNOW, MAT_SAND, MAT_STATIONARY = 0, 1, 2, 3, 4
KIND_SURFACE, KIND_SPHERE, KIND_BOX = 0, 1, 2


def build(force: bool = False) -> Path:
    srcs = [HERE / "mpm_oracle.c", HERE / "mpm_oracle_impl.h"]
    if force or not LIB_PATH.exists() or any(s.stat().st_mtime > LIB_PATH.stat().st_mtime for s in srcs):
        subprocess.run(["make", "-C", str(HERE)] + (["-B"] if force else []), check=True, capture_output=True)
    return LIB_PATH


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        vp, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
        for sfx, real in (("_d", ctypes.c_double), ("_f", ctypes.c_float)):
            getattr(L, "oracle_svd3" + sfx).argtypes = [vp, vp, vp, vp]
            getattr(L, "oracle_p2g" + sfx).argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, vp, real, vp, vp, vp, vp, i32]
            getattr(L, "oracle_p2g" + sfx).restype = i32
            getattr(L, "oracle_grid_update" + sfx).argtypes = [vp, vp, i32, i32, i32, i32, vp, real, vp, vp, vp, vp,
                                                               vp, i32]
            getattr(L, "oracle_g2p" + sfx).argtypes = [vp, i64, vp, vp, vp, vp, real, vp, vp, vp, i32]
            getattr(L, "oracle_g2p" + sfx).restype = i32
            getattr(L, "oracle_substeps" + sfx).argtypes = [vp, vp, i32, i32, i32, i32, vp, i64, vp, vp, vp, vp, vp,
                                                            vp, vp, real, i32, vp, vp, vp, vp, vp, vp, vp, vp, i32,
                                                            vp]
            getattr(L, "oracle_substeps" + sfx).restype = i32
            getattr(L, "oracle_g2p2g" + sfx).argtypes = [vp, vp, i32, i32, i32, i32, vp, i64, i64, vp, vp, vp, vp,
                                                         vp, vp, real, vp, vp, vp, vp, vp]
            getattr(L, "oracle_g2p2g" + sfx).restype = i32
            getattr(L, "oracle_quant_values" + sfx).argtypes = [i64, vp, vp, vp]
            getattr(L, "oracle_quant_values" + sfx).restype = None
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


@dataclass
class Config:
    """Solver constants of engine/mpm_solver.py:44-310 (3-D)."""
    res: tuple
    size: float = 1.0
    dt_scale: float = 1.0
    E_scale: float = 1.0
    padding: int = 3
    unbounded: bool = False
    water_density: float = 1.0
    gravity: tuple = (0.0, -9.8, 0.0)
    support_plasticity: bool = True
    # fused G2P2G mode: grid velocities clamped to +-cfl * dx / dt (0 = off)
    v_clamp_cfl: float = 0.0
    # quant=True: stored x, v, F rounded to the packed formats
    quant: bool = False
    # grid_postprocess list; the bounding box first, as the constructor adds it
    postprocess: list = field(default_factory=lambda: [dict(kind=KIND_BOX, surface=0)])

    def __post_init__(self):
        self.res = tuple(int(r) for r in self.res)
        self.grid_size = 4096
        if self.unbounded:
            while self.grid_size <= 2 * max(self.res):
                self.grid_size *= 2
            self.postprocess = [dict(kind=KIND_BOX, surface=1) if c["kind"] == KIND_BOX else c
                                for c in self.postprocess]
        self.dx = self.size / self.res[0]  # :82
        self.inv_dx = 1.0 / self.dx
        self.default_dt = 2e-2 * self.dx / self.size * self.dt_scale  # :84
        self.p_vol = self.dx**3
        self.p_mass = self.p_vol * 1000
        self.E, self.nu = 1e6 * self.size * self.E_scale, 0.2  # :201
        self.mu_0 = self.E / (2 * (1 + self.nu))
        self.lambda_0 = self.E * self.nu / ((1 + self.nu) * (1 - 2 * self.nu))
        sin_phi = math.sin(math.radians(45))
        self.alpha = math.sqrt(2 / 3) * 2 * sin_phi / (3 - sin_phi)  # :207-210

    def pd(self) -> np.ndarray:
        return np.array([
            self.dx, self.inv_dx, self.p_vol, self.p_mass, self.mu_0, self.lambda_0, self.alpha, self.water_density,
            self.gravity[0], self.gravity[1], self.gravity[2], self.p_vol * 4 * self.inv_dx**2,
            (3 * self.lambda_0 + 2 * self.mu_0) / (2 * self.mu_0), self.nu, float(bool(self.support_plasticity)),
            self.dx * self.v_clamp_cfl, float(bool(self.quant))
        ], dtype=np.float64)

    def coll(self) -> np.ndarray:
        a = np.zeros((max(1, len(self.postprocess)), 12), dtype=np.float64)
        for i, c in enumerate(self.postprocess):
            a[i, 0] = c["kind"]
            a[i, 1] = c.get("surface", 0)
            a[i, 2:5] = c.get("point", (0, 0, 0))
            n = np.asarray(c.get("normal", (0, 0, 0)), dtype=np.float64)
            if c["kind"] == KIND_SURFACE:
                n = n / math.sqrt(float((n**2).sum()))  # :653-655
            a[i, 5:8] = n
            a[i, 8] = c.get("radius", 0.0)
            a[i, 9] = c.get("friction", 0.0)
        return a


def substep_count(frame_dt: float, default_dt: float):
    """engine/mpm_solver.py:752-771: (number of substeps actually run, dt)."""
    substeps = int(frame_dt / default_dt) + 1
    dt = frame_dt / substeps
    left = frame_dt
    n = 0
    while left > 0:
        n += 1
        left -= dt
    return n, dt


# ------------------------------------------------------------- binning --

def base_cells(x: np.ndarray, inv_dx: float) -> np.ndarray:
    """floor(x * inv_dx - 0.5) in float32, engine/mpm_solver.py:357."""
    x32 = np.asarray(x, dtype=np.float32)
    s = x32 * np.float32(inv_dx)
    t = s - np.float32(0.5)
    return np.floor(t).astype(np.int64)


def active_sets(x: np.ndarray, inv_dx: float, block: int = 4):
    """Leaf blocks of the base cells (build_pid, :344-361) with their particle
    counts, and the blocks that P2G's 3^3 stencils touch (the blocks Taichi
    activates during P2G, :582-584).  Block coordinates in the reference's
    global grid index frame, as sorted (k,3) arrays."""
    base = base_cells(x, inv_dx)
    pb = np.floor_divide(base, block)
    pblocks, counts = np.unique(pb, axis=0, return_counts=True)
    lo = np.floor_divide(base, block)
    hi = np.floor_divide(base + 2, block)
    touched = set()
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                d = np.array([dx, dy, dz])
                cand = lo + d
                ok = np.all(cand <= hi, axis=1)
                for b in map(tuple, cand[ok]):
                    touched.add(b)
    gblocks = np.array(sorted(touched), dtype=np.int64).reshape(-1, 3)
    return pblocks, counts, gblocks


# ------------------------------------------------------------- C oracle --

def svd3(A: np.ndarray, dtype=np.float64):
    """Oracle SVD of one 3x3 matrix: U, s, V with A = U diag(s) V^T."""
    sfx = "_d" if dtype == np.float64 else "_f"
    A = np.ascontiguousarray(A, dtype=dtype)
    U = np.zeros((3, 3), dtype)
    V = np.zeros((3, 3), dtype)
    s = np.zeros(3, dtype)
    getattr(lib(), "oracle_svd3" + sfx)(_p(A), _p(U), _p(s), _p(V))
    return U, s, V


class Window:
    """Dense grid window [lo, lo+W) in the reference's grid index frame."""

    def __init__(self, lo, W):
        self.lo = np.ascontiguousarray(lo, dtype=np.int32)
        self.W = np.ascontiguousarray(W, dtype=np.int32)

    @classmethod
    def covering(cls, x: np.ndarray, inv_dx: float, margin: int = 8):
        b = base_cells(x, inv_dx)
        lo = (np.floor_divide(b.min(0) - margin, 4) * 4).astype(np.int32)
        hi = b.max(0) + 3 + margin
        W = (np.ceil((hi - lo) / 4.0) * 4).astype(np.int32)
        return cls(lo, W)

    @property
    def nnodes(self) -> int:
        return int(np.prod(self.W.astype(np.int64)))


@dataclass
class Particles:
    """Particle state in the reference's layout (AoS per particle)."""
    x: np.ndarray
    v: np.ndarray
    C: np.ndarray
    F: np.ndarray
    Jp: np.ndarray
    material: np.ndarray
    E: np.ndarray | None = None

    @classmethod
    def seeded(cls, x, material, v=None, dtype=np.float64, E=None):
        """seed_particle, engine/mpm_solver.py:823-838."""
        x = np.ascontiguousarray(x, dtype=dtype).reshape(-1, 3)
        n = x.shape[0]
        mat = np.ascontiguousarray(np.broadcast_to(np.asarray(material, dtype=np.int32), (n,)))
        vv = np.zeros((n, 3), dtype) if v is None else np.ascontiguousarray(np.broadcast_to(v, (n, 3)), dtype=dtype)
        F = np.ascontiguousarray(np.broadcast_to(np.eye(3, dtype=dtype), (n, 3, 3)))
        C = np.zeros((n, 3, 3), dtype)
        Jp = np.where(mat == MAT_SAND, 0.0, 1.0).astype(dtype)
        Ep = None if E is None else np.ascontiguousarray(np.broadcast_to(E, (n,)), dtype=dtype)
        return cls(x.copy(), vv.copy(), C, F.copy(), Jp, mat, Ep)

    def astype(self, dtype):
        return Particles(*(a.astype(dtype) if a is not None and a.dtype.kind == "f" else
                           (None if a is None else a.copy()) for a in
                           (self.x, self.v, self.C, self.F, self.Jp, self.material, self.E)))

    def copy(self):
        return self.astype(self.x.dtype)

    @property
    def n(self):
        return self.x.shape[0]


def p2g(cfg: Config, P: Particles, dt: float, win: Window, nthreads: int = 1):
    """P2G (engine/mpm_solver.py:487-584) into a zeroed dense window grid.
    Updates P.F and P.Jp in place; returns (m, mv) arrays shaped W and W+(3,)."""
    dt_ = P.x.dtype
    sfx = "_d" if dt_ == np.float64 else "_f"
    gm = np.zeros(win.nnodes, dt_)
    gmv = np.zeros(win.nnodes * 3, dt_)
    bad = getattr(lib(), "oracle_p2g" + sfx)(_p(cfg.pd()), P.n, _p(P.x), _p(P.v), _p(P.C), _p(P.F), _p(P.Jp),
                                               _p(P.material), _p(P.E), dt_.type(dt), _p(win.lo), _p(win.W),
                                               _p(gm), _p(gmv), nthreads)
    if bad:
        raise ValueError(f"{bad} particles outside the oracle window")
    return gm.reshape(tuple(win.W)), gmv.reshape(tuple(win.W) + (3,))


def grid_update(cfg: Config, gm: np.ndarray, gmv: np.ndarray, dt: float, win: Window, nthreads: int = 1):
    """Grid update (:586-616) and post-processing (:618-692); returns v."""
    dt_ = gm.dtype
    sfx = "_d" if dt_ == np.float64 else "_f"
    gm = np.ascontiguousarray(gm).reshape(-1)
    gv = np.ascontiguousarray(gmv).reshape(-1).copy()
    res = np.asarray(cfg.res, dtype=np.int32)
    coll = cfg.coll()
    getattr(lib(), "oracle_grid_update" + sfx)(_p(cfg.pd()), _p(res), cfg.padding, int(cfg.unbounded),
                                               cfg.grid_size, len(cfg.postprocess), _p(coll), dt_.type(dt),
                                               _p(win.lo), _p(win.W), _p(gm), _p(gv), None, nthreads)
    return gv.reshape(tuple(win.W) + (3,))


def g2p(cfg: Config, P: Particles, gv: np.ndarray, dt: float, win: Window, nthreads: int = 1):
    """G2P (:694-724) in place on P."""
    dt_ = P.x.dtype
    sfx = "_d" if dt_ == np.float64 else "_f"
    gv = np.ascontiguousarray(gv, dtype=dt_).reshape(-1)
    bad = getattr(lib(), "oracle_g2p" + sfx)(_p(cfg.pd()), P.n, _p(P.x), _p(P.v), _p(P.C), _p(P.material),
                                               dt_.type(dt), _p(win.lo), _p(win.W), _p(gv), nthreads)
    if bad:
        raise ValueError(f"{bad} particles outside the oracle window")


def substep(cfg: Config, P: Particles, dt: float, win: Window | None = None, nthreads: int = 1):
    """One full substep; returns the grid after P2G and after the update."""
    if win is None:
        win = Window.covering(P.x, cfg.inv_dx)
    gm, gmv = p2g(cfg, P, dt, win, nthreads)
    gv = grid_update(cfg, gm, gmv, dt, win, nthreads)
    g2p(cfg, P, gv, dt, win, nthreads)
    return win, gm, gmv, gv


def quant_values(x, v, F):
    """The values quant=True stores for positions (n,3), velocities (n,3)
    and deformation gradients (n,3,3): copies of the same dtype
    (float64 or float32)."""
    x, v, F = (np.ascontiguousarray(a).copy() for a in (x, v, F))
    sfx = "_d" if x.dtype == np.float64 else "_f"
    getattr(lib(), "oracle_quant_values" + sfx)(x.shape[0], _p(x), _p(v), _p(F))
    return x, v, F


class Runner:
    """Many substeps with the block-sparse C loop (the timed CPU baseline)."""

    def __init__(self, cfg: Config, P: Particles, win: Window | None = None, nthreads: int | None = None):
        self.cfg = cfg
        self.P = P
        self.win = win or Window.covering(P.x, cfg.inv_dx, margin=16)
        self.nthreads = nthreads or os.cpu_count() or 1
        dt_ = P.x.dtype
        nn = self.win.nnodes
        self.gm = np.zeros(nn, dt_)
        self.gmv = np.zeros(nn * 3, dt_)
        nblk = nn // 64
        self.blkflag = np.zeros(nblk, np.uint8)
        self.pkey = np.zeros(P.n, np.int32)
        self.order = np.zeros(P.n, np.int64)
        self.bcount = np.zeros(nblk + 1, np.int64)
        self.res = np.asarray(cfg.res, dtype=np.int32)
        self.coll = cfg.coll()

    def run(self, dt: float, nsub: int):
        P = self.P
        dt_ = P.x.dtype
        sfx = "_d" if dt_ == np.float64 else "_f"
        maxv = np.zeros(max(1, nsub), dt_)
        bad = getattr(lib(), "oracle_substeps" + sfx)(
            _p(self.cfg.pd()), _p(self.res), self.cfg.padding, int(self.cfg.unbounded), self.cfg.grid_size,
            len(self.cfg.postprocess), _p(self.coll), P.n, _p(P.x), _p(P.v), _p(P.C), _p(P.F), _p(P.Jp),
            _p(P.material), _p(P.E), dt_.type(dt), nsub, _p(self.win.lo), _p(self.win.W), _p(self.gm), _p(self.gmv),
            _p(self.blkflag), _p(self.pkey), _p(self.order), _p(self.bcount), self.nthreads, _p(maxv))
        if bad:
            raise ValueError(f"{bad} particles left the oracle window")
        return maxv


class G2P2GRunner:
    """The fused G2P2G mode (engine/mpm_solver.py:363-485, :773-787): the
    grid velocities persist between substeps; particles added since the last
    substep (index >= last_final) skip the gather.  C is not carried.
    The grid update clamps velocities to +-v_clamp_cfl * dx / dt per
    component (v_clamp_g2p2g=True and g2p2g_allowed_cfl=0.9 by default,
    :589-598); v_clamp_cfl=0 turns the clamp off."""

    def __init__(self, cfg: Config, P: Particles, win: Window, v_clamp_cfl: float = 0.9):
        cfg = dataclasses.replace(cfg, v_clamp_cfl=v_clamp_cfl)
        self.cfg, self.P, self.win = cfg, P, win
        self.gv = np.zeros(win.nnodes * 3, P.x.dtype)
        self.last_final = 0
        self.res = np.asarray(cfg.res, dtype=np.int32)
        self.coll = cfg.coll()

    def step(self, dt: float):
        P = self.P
        dt_ = P.x.dtype
        sfx = "_d" if dt_ == np.float64 else "_f"
        gm = np.zeros(self.win.nnodes, dt_)
        gmv = np.zeros(self.win.nnodes * 3, dt_)
        bad = getattr(lib(), "oracle_g2p2g" + sfx)(
            _p(self.cfg.pd()), _p(self.res), self.cfg.padding, int(self.cfg.unbounded), self.cfg.grid_size,
            len(self.cfg.postprocess), _p(self.coll), P.n, self.last_final, _p(P.x), _p(P.v), _p(P.F), _p(P.Jp),
            _p(P.material), _p(P.E), dt_.type(dt), _p(self.win.lo), _p(self.win.W), _p(self.gv), _p(gm), _p(gmv))
        if bad:
            raise ValueError(f"{bad} particles left the oracle window")
        self.gv = gmv
        self.last_final = P.n
        return gm.reshape(tuple(self.win.W)), gmv.reshape(tuple(self.win.W) + (3,))


# ------------------------------------------------- numpy restatement ---

def _svd_rot(F):
    """numpy SVD with U, V rotations and the sign of det on the last value."""
    U, s, Vt = np.linalg.svd(F)
    V = np.swapaxes(Vt, -1, -2).copy()
    dU = np.linalg.det(U)
    dV = np.linalg.det(V)
    fixU = dU < 0
    U[fixU, :, 2] *= -1
    s = s.copy()
    s[fixU, 2] *= -1
    fixV = dV < 0
    V[fixV, :, 2] *= -1
    s[fixV, 2] *= -1
    return U, s, V


def np_substep(cfg: Config, P: Particles, dt: float):
    """Independent float64 numpy restatement of one substep
    (engine/mpm_solver.py:495-584, 586-692, 701-724).  Returns (gm, gv) as
    dicts keyed by global node index."""
    x, v, C, F, Jp, mat = (P.x.astype(np.float64), P.v.astype(np.float64), P.C.astype(np.float64),
                           P.F.astype(np.float64), P.Jp.astype(np.float64), P.material)
    n = x.shape[0]
    base = base_cells(P.x, cfg.inv_dx)
    fx = x * cfg.inv_dx - base
    w = [0.5 * (1.5 - fx)**2, 0.75 - (fx - 1)**2, 0.5 * (fx - 0.5)**2]
    I3 = np.eye(3)
    Fw = F.copy()
    water = mat == MAT_WATER
    plast = bool(cfg.support_plasticity)
    Fw[water] = I3
    Fw[water, 0, 0] = Jp[water] if plast else 1.0  # :508-511
    Fn = (I3 + dt * C) @ Fw
    mu0 = np.full(n, cfg.mu_0) if P.E is None else P.E / (2 * (1 + cfg.nu))
    la0 = np.full(n, cfg.lambda_0) if P.E is None else P.E * cfg.nu / ((1 + cfg.nu) * (1 - 2 * cfg.nu))
    if P.E is not None:
        mu0 = np.where(P.E > 0, mu0, cfg.mu_0)
        la0 = np.where(P.E > 0, la0, cfg.lambda_0)
    h = np.where((mat != MAT_WATER) & plast, np.exp(10 * (1 - Jp)), 1.0)
    h = np.where(mat == MAT_ELASTIC, 0.3, h)
    mu = np.where(water, 0.0, mu0 * h)
    la = la0 * h
    U, sig, V = _svd_rot(Fn)
    J = np.ones(n)
    Jp_new = Jp.copy()
    sand = mat == MAT_SAND
    snow = mat == MAT_SNOW
    ns = np.where(snow[:, None], np.clip(sig, 1 - 2.5e-2, 1 + 4.5e-3), sig)
    ns_use = np.where(sand[:, None], sig, ns)
    Jp_new = np.where(sand, Jp, Jp * np.prod(sig / ns_use, axis=1))
    J = np.where(sand, 1.0, np.prod(ns_use, axis=1))
    Fnew = Fn.copy()
    Fnew[water] = I3
    Fnew[water, 0, 0] = J[water]
    Jp_new[water] = J[water]
    Fnew[snow] = (U[snow] * ns[snow][:, None, :]) @ np.swapaxes(V[snow], -1, -2)
    R = U @ np.swapaxes(V, -1, -2)
    stress = 2 * mu[:, None, None] * (Fnew - R) @ np.swapaxes(Fnew, -1, -2) + \
        (la * J * (J - 1))[:, None, None] * I3
    if not plast:  # no Jp field; sand carries no stress (:553-566 skipped)
        Jp_new = Jp.copy()
        stress[sand] = 0.0
    elif sand.any():
        s_ = sig[sand]
        eps = np.log(np.maximum(np.abs(s_), 1e-4))
        tr = eps.sum(1) + Jp[sand]
        eh = eps - tr[:, None] / 3
        ehn = np.linalg.norm(eh, axis=1) + 1e-20
        sk = (3 * la0[sand] + 2 * mu0[sand]) / (2 * mu0[sand])
        dg = ehn + sk * tr * cfg.alpha
        out = np.exp(eps - (np.maximum(0, dg) / ehn)[:, None] * eh)
        out = np.where((tr >= 0)[:, None], 1.0, out)
        Jp_new[sand] = np.where(tr >= 0, tr, 0.0)
        Us, Vs = U[sand], V[sand]
        Fs = (Us * out[:, None, :]) @ np.swapaxes(Vs, -1, -2)
        lsig = np.log(out)
        cen = 2 * mu0[sand][:, None] * lsig / out + la0[sand][:, None] * lsig.sum(1, keepdims=True) / out
        stress[sand] = (Us * cen[:, None, :]) @ np.swapaxes(Vs, -1, -2) @ np.swapaxes(Fs, -1, -2)
        Fnew[sand] = Fs
    stress = (-dt * cfg.p_vol * 4 * cfg.inv_dx**2) * stress
    mass = np.where(water, cfg.p_mass * cfg.water_density, cfg.p_mass)
    affine = stress + mass[:, None, None] * C
    gm = {}
    gmv = {}
    keys_all = []
    vals_m = []
    vals_mv = []
    for a in range(3):
        for b in range(3):
            for c in range(3):
                off = np.array([a, b, c])
                dpos = (off - fx) * cfg.dx
                wt = w[a][:, 0] * w[b][:, 1] * w[c][:, 2]
                mv = wt[:, None] * (mass[:, None] * v + np.einsum("nij,nj->ni", affine, dpos))
                keys_all.append(base + off)
                vals_m.append(wt * mass)
                vals_mv.append(mv)
    keys = np.concatenate(keys_all)
    vm = np.concatenate(vals_m)
    vmv = np.concatenate(vals_mv)
    uk, inv = np.unique(keys, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    m_acc = np.zeros(len(uk))
    mv_acc = np.zeros((len(uk), 3))
    np.add.at(m_acc, inv, vm)
    np.add.at(mv_acc, inv, vmv)
    gv_acc = mv_acc.copy()
    pos = m_acc > 0
    gv_acc[pos] = mv_acc[pos] / m_acc[pos][:, None] + dt * np.asarray(cfg.gravity)
    for ci in cfg.postprocess:
        I = uk
        if ci["kind"] == KIND_BOX:
            for d in range(3):
                if ci.get("surface", 0):
                    lo, hi = -cfg.grid_size // 2 + cfg.padding, cfg.grid_size // 2 - cfg.padding
                else:
                    lo, hi = cfg.padding, cfg.res[d] - cfg.padding
                gv_acc[(I[:, d] < lo) & (gv_acc[:, d] < 0), d] = 0
                gv_acc[(I[:, d] >= hi) & (gv_acc[:, d] > 0), d] = 0
        elif ci["kind"] == KIND_SURFACE:
            nrm = np.asarray(ci["normal"], dtype=np.float64)
            nrm = nrm / np.linalg.norm(nrm)
            off = I * cfg.dx - np.asarray(ci["point"])
            inside = off @ nrm < 0
            vv = gv_acc[inside]
            if ci.get("surface", 0) == 0:
                vv[:] = 0
            else:
                nc = vv @ nrm
                s = nc if ci["surface"] == 1 else np.minimum(nc, 0)
                vv = vv - nrm[None] * s[:, None]
                vn = np.linalg.norm(vv, axis=1)
                fr = (nc < 0) & (vn > 1e-30)
                mag = np.maximum(0, vn + nc * ci.get("friction", 0.0))
                vv[fr] = vv[fr] / vn[fr][:, None] * mag[fr][:, None]
            gv_acc[inside] = vv
        else:
            off = I * cfg.dx - np.asarray(ci["point"])
            r2 = (off**2).sum(1)
            inside = r2 < ci["radius"]**2
            vv = gv_acc[inside]
            if ci.get("surface", 0) == 0:
                vv[:] = 0
            else:
                nrm = off[inside] / (np.sqrt(r2[inside]) + 1e-5)[:, None]
                nc = (nrm * vv).sum(1)
                s = nc if ci["surface"] == 1 else np.minimum(nc, 0)
                vv = vv - nrm * s[:, None]
            gv_acc[inside] = vv
    # G2P
    lut = {tuple(k): i for i, k in enumerate(uk)}
    new_v = np.zeros((n, 3))
    new_C = np.zeros((n, 3, 3))
    for a in range(3):
        for b in range(3):
            for c in range(3):
                off = np.array([a, b, c])
                idx = np.array([lut[tuple(k)] for k in base + off])
                g = gv_acc[idx]
                wt = w[a][:, 0] * w[b][:, 1] * w[c][:, 2]
                dpos = off - fx
                new_v += wt[:, None] * g
                new_C += 4 * cfg.inv_dx * wt[:, None, None] * g[:, :, None] * dpos[:, None, :]
    moving = mat != MAT_STATIONARY
    out = Particles(x.copy(), v.copy(), C.copy(), Fnew, Jp_new, mat.copy(), P.E)
    out.v[moving] = new_v[moving]
    out.C[moving] = new_C[moving]
    out.x[moving] = x[moving] + dt * new_v[moving]
    grid = {tuple(k): (m_acc[i], mv_acc[i], gv_acc[i]) for i, k in enumerate(uk)}
    return out, grid
