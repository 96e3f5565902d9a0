"""Seeded synthetic scenes of the benchmark and parity workloads.

Each generator returns a ``Scene`` with float32 positions, velocities,
int32 materials, the grid resolution, the grid post-process records and the
substep count of the workload it names.  Positions come from
``numpy.random.default_rng(seed)`` so the GPU engine and the CPU oracle see
identical inputs.  The shapes restate the workloads of the MLS-MPM solver
benchmark (particle counts, grids, material mixes); no external dataset is
used.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

WATER, ELASTIC, SNOW, SAND, STATIONARY = 0, 1, 2, 3, 4


@dataclass
class Scene:
    name: str
    res: tuple
    x: np.ndarray  # (n,3) float32
    v: np.ndarray  # (n,3) float32
    material: np.ndarray  # (n,) int32
    substeps: int
    postprocess: list = field(default_factory=list)  # extra colliders (box implied)
    size: float = 1.0
    E_p: np.ndarray | None = None
    color: np.ndarray | None = None
    E_scale: float = 1.0
    target: np.ndarray | None = None

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    @property
    def dx(self) -> float:
        return self.size / self.res[0]

    @property
    def default_dt(self) -> float:
        return 2e-2 * self.dx / self.size

    def make_solver(self, **kw):
        """An MPMSolver loaded with this scene through read_restart."""
        from .mpm_solver import MPMSolver
        kw.setdefault("E_scale", self.E_scale)
        s = MPMSolver(self.res, size=self.size, **kw)
        for c in self.postprocess:
            if c["kind"] == 0:
                s.add_surface_collider(c["point"], c["normal"], c.get("surface", 0), c.get("friction", 0.0))
            elif c["kind"] == 1:
                s.add_sphere_collider(c["point"], c["radius"], c.get("surface", 0))
        color = self.color if self.color is not None else np.full(self.n, 0xFFFFFF, np.int32)
        s.read_restart(self.n, self.x, self.v, self.material, color)
        return s


def _cube(rng, lo, side, n):
    return (np.asarray(lo, np.float32) + rng.random((n, 3), dtype=np.float32) * np.float32(side)).astype(np.float32)


def _ellipsoid(rng, c, a, n):
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = rng.random(n)**(1.0 / 3.0)
    return (np.asarray(c) + d * r[:, None] * np.asarray(a)).astype(np.float32)


def water_cube_64(seed: int = 1) -> Scene:
    """Plain 3-D MLS-MPM, dense 64^3 grid on [0,1]^3: one water cube with
    lower corner (0.3,0.3,0.3), side 0.4, 8 particles per cell (the add_cube
    count rule, int(8*0.4^3*64^3+1) = 134,218 particles), v = 0, 100
    substeps."""
    rng = np.random.default_rng(seed)
    res = (64, 64, 64)
    n = int(8 * 0.4**3 * 64**3 + 1)
    x = _cube(rng, (0.3, 0.3, 0.3), 0.4, n)
    return Scene("water_cube_64", res, x, np.zeros((n, 3), np.float32), np.zeros(n, np.int32), 100)


def four_materials_128(seed: int = 2, per_cube: int = 500_000) -> Scene:
    """3-D multi-material on a 128^3 grid: four non-overlapping cubes of
    `per_cube` particles (water, elastic, snow, sand) at 8 particles per cell,
    each with one velocity drawn from U[-1,1]^3; 500 substeps."""
    rng = np.random.default_rng(seed)
    res = (128, 128, 128)
    dx = 1.0 / 128
    side = (per_cube / 8.0)**(1.0 / 3.0) * dx
    pad = 3 * dx + 0.02
    gap = (1.0 - 2 * pad - 2 * side) / 3.0
    xs, vs, ms = [], [], []
    corners = [(pad + gap, 0.25, pad + gap), (pad + 2 * gap + side, 0.25, pad + gap),
               (pad + gap, 0.25, pad + 2 * gap + side), (pad + 2 * gap + side, 0.25, pad + 2 * gap + side)]
    for mat, lo in zip((WATER, ELASTIC, SNOW, SAND), corners):
        xs.append(_cube(rng, lo, side, per_cube))
        vel = rng.uniform(-1.0, 1.0, 3).astype(np.float32)
        vs.append(np.broadcast_to(vel, (per_cube, 3)))
        ms.append(np.full(per_cube, mat, np.int32))
    return Scene("four_materials_128", res, np.concatenate(xs), np.ascontiguousarray(np.concatenate(vs)),
                 np.concatenate(ms), 500)


def ellipsoids_256(seed: int = 3, n_total: int = 16_000_000, n_ellipsoids: int = 64) -> Scene:
    """3-D large sparse scene on a 256^3 grid: `n_total` particles in 64
    ellipsoids (semi-axes U[0.02,0.08]^3, centres with x,z uniform inside the
    box and y in the upper half), split in proportion to volume (about 28
    particles per cell at 16M), materials elastic/snow 50/50 per ellipsoid,
    v = 0, a sticky ground-plane surface collider at y = 0.05; 200 substeps."""
    rng = np.random.default_rng(seed)
    res = (256, 256, 256)
    pad = 3.0 / 256
    axes = rng.uniform(0.02, 0.08, (n_ellipsoids, 3))
    cen = np.empty((n_ellipsoids, 3))
    for i in range(n_ellipsoids):
        a = axes[i]
        cen[i, 0] = rng.uniform(a[0] + pad, 1 - a[0] - pad)
        cen[i, 2] = rng.uniform(a[2] + pad, 1 - a[2] - pad)
        cen[i, 1] = rng.uniform(0.5, 1 - a[1] - pad)
    vol = np.prod(axes, axis=1)
    counts = np.floor(vol / vol.sum() * n_total).astype(np.int64)
    counts[: n_total - counts.sum()] += 1
    mats = np.where(rng.random(n_ellipsoids) < 0.5, ELASTIC, SNOW).astype(np.int32)
    xs, ms = [], []
    for i in range(n_ellipsoids):
        xs.append(_ellipsoid(rng, cen[i], axes[i], int(counts[i])))
        ms.append(np.full(int(counts[i]), mats[i], np.int32))
    x = np.concatenate(xs)
    pp = [dict(kind=0, surface=0, point=(0.0, 0.05, 0.0), normal=(0.0, 1.0, 0.0), friction=0.0)]
    return Scene("ellipsoids_256", res, x, np.zeros_like(x), np.concatenate(ms), 200, postprocess=pp)


def batched_scenes(seed: int = 4, n_scenes: int = 64):
    """64 independent scenes: grid res from {32,48,64,96}^3, particle counts
    log-uniform in [8K, 300K] over 1-3 random cubes at 8 particles per cell,
    material per cube uniform over water/elastic/snow/sand, per-scene E
    log-uniform in [1e4, 1e6]; 50-substep frames.  A cube that would not fit
    inside the box at 8 particles per cell (large counts on coarse grids) is
    shrunk to fit, which raises its particle density."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(n_scenes):
        r = int(rng.choice([32, 48, 64, 96]))
        dx = 1.0 / r
        n = int(np.exp(rng.uniform(np.log(8e3), np.log(3e5))))
        k = int(rng.integers(1, 4))
        split = np.diff(np.concatenate([[0], np.sort(rng.choice(np.arange(1, n), k - 1, replace=False)), [n]]))
        E = float(np.exp(rng.uniform(np.log(1e4), np.log(1e6))))
        xs, ms = [], []
        for j in range(k):
            m = int(split[j])
            margin = 3 * dx + 0.01
            side = (m / 8.0)**(1.0 / 3.0) * dx
            side = min(side, 1 - 2 * margin - 0.02)
            lo = rng.uniform(margin, 1 - margin - side, 3)
            xs.append(_cube(rng, lo, side, m))
            ms.append(np.full(m, int(rng.integers(0, 4)), np.int32))
        x = np.concatenate(xs)
        sc = Scene(f"batched_{s}", (r, r, r), x, np.zeros_like(x), np.concatenate(ms), 50)
        sc.E_scale = E / 1e6
        out.append(sc)
    return out


def elastic_on_water(seed: int = 5, res: int = 64, n_each: int = 100_000) -> Scene:
    """Differentiable workload: an elastic cube of `n_each` particles resting
    on a water slab of `n_each` particles spanning the box floor; 2000
    substeps.  ``target`` (a seeded point in [0.3,0.7]^3) is attached."""
    rng = np.random.default_rng(seed)
    dx = 1.0 / res
    pad = 3 * dx
    span = 1 - 2 * pad - 2 * dx
    thick = n_each / 8.0 * dx**3 / (span * span)
    slab = np.empty((n_each, 3), np.float32)
    u = rng.random((n_each, 3), dtype=np.float32)
    slab[:, 0] = pad + dx + u[:, 0] * span
    slab[:, 2] = pad + dx + u[:, 2] * span
    slab[:, 1] = pad + dx + u[:, 1] * thick
    side = (n_each / 8.0)**(1.0 / 3.0) * dx
    cube = _cube(rng, (0.5 - side / 2, pad + dx + thick + dx, 0.5 - side / 2), side, n_each)
    x = np.concatenate([slab, cube])
    mat = np.concatenate([np.full(n_each, WATER, np.int32), np.full(n_each, ELASTIC, np.int32)])
    sc = Scene("elastic_on_water", (res, res, res), x, np.zeros_like(x), mat, 2000)
    sc.target = rng.uniform(0.3, 0.7, 3)
    return sc


def smoke_scene(seed: int = 7) -> Scene:
    """Tiny mixed scene after the reference's tests/test_3d.py shapes: a 24^3
    grid with a snow ball, an elastic bar, a sand block and water."""
    rng = np.random.default_rng(seed)
    res = (24, 24, 24)
    parts = [(_ellipsoid(rng, (0.3, 0.5, 0.4), (0.1, 0.1, 0.1), 1500), SNOW, (0, -1, 0)),
             (_cube(rng, (0.5, 0.5, 0.3), 0.15, 1500), ELASTIC, (0.3, 0, 0)),
             (_cube(rng, (0.25, 0.2, 0.55), 0.2, 1500), SAND, (0, 0, 0)),
             (_cube(rng, (0.55, 0.15, 0.55), 0.2, 1500), WATER, (0, 0, -0.5))]
    x = np.concatenate([p[0] for p in parts])
    v = np.concatenate([np.broadcast_to(np.asarray(p[2], np.float32), (len(p[0]), 3)) for p in parts])
    m = np.concatenate([np.full(len(p[0]), p[1], np.int32) for p in parts])
    pp = [dict(kind=1, surface=1, point=(0.5, 0.35, 0.5), radius=0.08),
          dict(kind=0, surface=2, point=(0.5, 0.12, 0.5), normal=(0.1, 1.0, 0.0), friction=0.2)]
    return Scene("smoke_24", res, x, np.ascontiguousarray(v), m, 10, postprocess=pp)


# ------------------------------------------------------------- meshes ----
# Closed triangle meshes (n, 9) float32 for the add_mesh emitter; the
# reference's own mesh tests download theirs, these stand in for them.

def box_mesh(lo, hi) -> np.ndarray:
    """Axis-aligned box, outward-facing triangles."""
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    c = np.array([[lo[0] if i & 1 == 0 else hi[0], lo[1] if i & 2 == 0 else hi[1], lo[2] if i & 4 == 0 else hi[2]]
                  for i in range(8)])
    quads = [(0, 2, 6, 4), (1, 5, 7, 3), (0, 4, 5, 1), (2, 3, 7, 6), (0, 1, 3, 2), (4, 6, 7, 5)]
    tris = []
    for a, b, cc, d in quads:
        tris += [(a, cc, b), (a, d, cc)]
    return np.array([np.concatenate([c[i], c[j], c[k]]) for i, j, k in tris], np.float32)


def icosphere(center, radius, subdiv=3) -> np.ndarray:
    """Sphere from a subdivided icosahedron."""
    t = (1.0 + 5**0.5) / 2
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t), (t, 0, -1),
         (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    v = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}

        def mid(i, j):
            key = (min(i, j), max(i, j))
            if key not in cache:
                m = v[i] + v[j]
                v.append(m / np.linalg.norm(m))
                cache[key] = len(v) - 1
            return cache[key]

        nf = []
        for a, b, c in f:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    cen = np.asarray(center, np.float64)
    return np.array([np.concatenate([cen + radius * v[a], cen + radius * v[b], cen + radius * v[c]]) for a, b, c in f],
                    np.float32)


def torus_mesh(center, R, r, nu=48, nv=24) -> np.ndarray:
    """Torus around the y axis."""
    cen = np.asarray(center, np.float64)

    def p(i, j):
        u, w = 2 * np.pi * i / nu, 2 * np.pi * j / nv
        return cen + np.array([(R + r * np.cos(w)) * np.cos(u), r * np.sin(w), (R + r * np.cos(w)) * np.sin(u)])

    tris = []
    for i in range(nu):
        for j in range(nv):
            a, b, c, d = p(i, j), p(i + 1, j), p(i + 1, j + 1), p(i, j + 1)
            tris += [np.concatenate([a, c, b]), np.concatenate([a, d, c])]
    return np.array(tris, np.float32)
