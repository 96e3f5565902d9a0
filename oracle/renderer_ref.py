"""CPU restatement of the particle path tracer - TEST INFRASTRUCTURE.

Follows taichi-dev/taichi_elements engine/renderer.py and
engine/renderer_utils.py in float32:
* ``cell_lists``: initialize_particle_grid (:482-517) with
  sphere_aabb_intersect_motion (renderer_utils.py:133-147);
* ``next_hit``: dda_particle (:297-366) or, for the voxel view, dda_voxel
  (:217-281) with voxel_color (:146-160), the z = -5.5 plane (:375-380), the
  floor reached by sphere tracing (ray_march :180-191, sdf_normal :193-203,
  sdf_color :205-214 with inside_taichi, renderer_utils.py:164-195);
* ``render_no_particles``: the path tracer of render (:396-480) vectorised
  over paths, for scenes whose particles no ray reaches (floor, plane, light,
  bounces, Russian roulette), used for statistical agreement;
* ``tonemap``: copy (:519-531).
Random numbers are numpy's; the reference's ti.random stream cannot be
reproduced, so rendered images agree in distribution.  Parity of the
deterministic parts (cell lists, first hits) is against this restatement;
the reference itself needs Taichi (unpinned).  Used only by tests/.
"""
from __future__ import annotations

import numpy as np

F = np.float32
INF = F(1e10)
EPS = F(1e-4)
DIST_LIMIT = F(100.0)
LIGHT_DIRECTION = np.array([1.2, 0.3, 0.7], F)
LIGHT_NOISE = F(0.03)
SHUTTER_BEGIN = F(-0.5)


def normalized(a):
    a = np.asarray(a, F)
    return a * (F(1.0) / np.sqrt(np.sum(a * a, axis=-1, keepdims=True, dtype=F)).astype(F))


def point_aabb_distance2(bmin, bmax, o):
    p = np.maximum(np.minimum(o, bmax), bmin)
    d = p - o
    return F(np.sum(d * d, dtype=F))


def sphere_aabb_intersect_motion(bmin, bmax, o1, o2, r):
    lo, hi = F(0.0), F(1.0)
    for _ in range(64):
        if not lo + F(1e-5) < hi:
            break
        m1 = F(2.0) * lo / F(3.0) + hi / F(3.0)
        m2 = lo / F(3.0) + F(2.0) * hi / F(3.0)
        d1 = point_aabb_distance2(bmin, bmax, (F(1.0) - m1) * o1 + m1 * o2)
        d2 = point_aabb_distance2(bmin, bmax, (F(1.0) - m2) * o1 + m2 * o2)
        if d2 > d1:
            hi = m2
        else:
            lo = m1
    return point_aabb_distance2(bmin, bmax, (F(1.0) - lo) * o1 + lo * o2) < r * r


class Grid:
    """Cell grid of the renderer: cells [c0, c0 + nc), bounding box."""

    def __init__(self, x, dx):
        self.dx = F(dx)
        self.inv_dx = F(1.0 / dx)
        mn, mx = x.min(0), x.max(0)
        lo = [int(np.floor(float(mn[i]) * (1.0 / dx))) - 3 for i in range(3)]
        hi = [int(np.floor(float(mx[i]) * (1.0 / dx))) + 3 for i in range(3)]
        self.c0 = np.array(lo)
        self.nc = np.array([h - l + 1 for l, h in zip(lo, hi)])
        self.bmin = np.array([l * dx for l in lo], F)
        self.bmax = np.array([h * dx for h in hi], F)

    def inside(self, i, j, k):
        p = np.array([i, j, k], F) * self.dx
        return bool(np.all(self.bmin <= p) and np.all(p < self.bmax))


def cell_lists(grid: Grid, x, v, radius, shutter_time, motion_blur=True):
    """{cell (i, j, k): [particle, ...]} (renderer.py:482-517)."""
    radius = F(radius)
    lists = {}
    sb = SHUTTER_BEGIN * F(shutter_time) if motion_blur else F(0.0)
    se = (SHUTTER_BEGIN + F(1.0)) * F(shutter_time) if motion_blur else F(0.0)
    for p in range(len(x)):
        xp = x[p].astype(F)
        vp = v[p].astype(F) if motion_blur else np.zeros(3, F)
        ipos = np.floor(xp * grid.inv_dx).astype(np.int64)
        ob, oe = sb * vp, se * vp
        a, b = np.minimum(ob, oe), np.maximum(ob, oe)
        lo = np.floor(a * grid.inv_dx).astype(np.int64) - 1
        hi = np.ceil(b * grid.inv_dx).astype(np.int64) + 2
        for i in range(lo[0], hi[0]):
            for j in range(lo[1], hi[1]):
                for k in range(lo[2], hi[2]):
                    c = (ipos[0] + i, ipos[1] + j, ipos[2] + k)
                    if not grid.inside(*c):
                        continue
                    bmin = np.array(c, F) * grid.dx
                    bmax = (np.array(c, F) + F(1.0)) * grid.dx
                    if sphere_aabb_intersect_motion(bmin, bmax, xp + ob, xp + oe, radius):
                        lists.setdefault(c, []).append(p)
    return lists


def ray_aabb(bmin, bmax, o, d):
    inter, near, far = True, -INF, INF
    for i in range(3):
        if d[i] == 0:
            if o[i] < bmin[i] or o[i] > bmax[i]:
                inter = False
        else:
            i1 = (bmin[i] - o[i]) / d[i]
            i2 = (bmax[i] - o[i]) / d[i]
            far = min(max(i1, i2), far)
            near = max(min(i1, i2), near)
    if near > far:
        inter = False
    return inter, F(near), F(far)


def intersect_sphere(pos, d, center, radius):
    T = pos - center
    B = F(2.0) * F(np.dot(T, d))
    old = F(0.5) * (-B)
    dist = old
    T = (pos + d * old) - center
    B = F(2.0) * F(np.dot(T, d))
    C = F(np.dot(T, T)) - F(radius) * F(radius)
    delta = B * B - F(4.0) * C
    if delta > 0:
        r1 = F(0.5) * (-B - np.sqrt(delta)) + old
        if r1 > 0:
            dist = r1
    else:
        dist = INF
    return F(dist)


def inside_taichi(px, py):
    def disc(cx, cy, r):
        return (px - cx)**2 + (py - cy)**2 <= r * r
    ret = -1
    for cond, val in ((not disc(0.5, 0.5, 0.52), 0), (not disc(0.5, 0.5, 0.495), 1), (disc(0.5, 0.25, 0.08), 1),
                      (disc(0.5, 0.75, 0.08), 0), (disc(0.5, 0.25, 0.25), 0), (disc(0.5, 0.75, 0.25), 1)):
        if cond and ret == -1:
            ret = val
    if ret == -1:
        ret = 1 if px < 0.5 else 0
    return ret


def dda_particle(grid, lists, x, v, rgb, radius, eye, d, t, motion_blur):
    d = d.copy()
    for i in range(3):
        if abs(d[i]) < F(1e-6):
            d[i] = F(1e-6)
    closest, normal, color = INF, np.zeros(3, F), np.zeros(3, F)
    inter, near, _ = ray_aabb(grid.bmin, grid.bmax, eye, d)
    near = max(F(0.0), near)
    if not inter:
        return closest, normal, color
    pos = eye + d * (near + EPS)
    rinv = F(1.0) / d
    rs = np.where(d > 0, 1, -1)
    o = grid.inv_dx * pos
    ip = np.floor(o).astype(np.int64)
    dis = (ip.astype(F) - o + F(0.5) + rs.astype(F) * F(0.5)) * rinv
    for _ in range(int(grid.nc.sum()) + 8):
        if not grid.inside(*ip):
            normal = np.zeros(3, F)
            break
        for p in lists.get(tuple(int(c) for c in ip), ()):
            xp = x[p].astype(F) + (F(t) * v[p].astype(F) if motion_blur else F(0.0))
            dist = intersect_sphere(eye, d, xp, radius)
            if dist < closest and dist > 0:
                closest = dist
                normal = normalized((eye + dist * d) - xp)
                color = rgb[p].astype(F) * F(1.0 / 255.0)
        if closest < INF:
            break
        if dis[0] <= dis[1] and dis[0] <= dis[2]:
            m = 0
        elif dis[1] <= dis[0] and dis[1] <= dis[2]:
            m = 1
        else:
            m = 2
        dis[m] += F(rs[m]) * rinv[m]
        ip[m] += rs[m]
    return closest, normal, color


def voxel_color(pos, inv_dx):
    p = pos * inv_dx
    p = p - np.floor(p)
    count = int(np.sum((p < F(0.1)) | (p > F(1.0) - F(0.1))))
    f = F(1.0) if count >= 2 else F(0.0)
    return np.array([0.9, 0.8, 1.0], F) * (F(1.3) - F(1.2) * f)


def dda_voxel(grid, lists, eye, d):
    """renderer.py:217-281: the first cell holding a particle."""
    d = d.copy()
    for i in range(3):
        if abs(d[i]) < F(1e-6):
            d[i] = F(1e-6)
    rinv = F(1.0) / d
    rs = np.where(d > 0, 1, -1)
    hit, normal, color = INF, np.zeros(3, F), np.zeros(3, F)
    inter, near, _ = ray_aabb(grid.bmin, grid.bmax, eye, d)
    if not inter:
        return hit, normal, color
    near = max(F(0.0), near)
    pos = eye + d * (near + F(5.0) * EPS)
    o = grid.inv_dx * pos
    ip = np.floor(o).astype(np.int64)
    dis = (ip.astype(F) - o + F(0.5) + rs.astype(F) * F(0.5)) * rinv
    for _ in range(int(grid.nc.sum()) + 8):
        occupied = tuple(int(c) for c in ip) in lists
        inside = grid.inside(*ip)
        if occupied:
            mini = ((ip.astype(F) - o + F(0.5) - rs.astype(F) * F(0.5)) * rinv).max()
            hit = F(mini * grid.dx + near)
            color = voxel_color(eye + hit * d, grid.inv_dx)
            break
        if dis[0] <= dis[1] and dis[0] < dis[2]:
            m = 0
        elif dis[1] <= dis[0] and dis[1] <= dis[2]:
            m = 1
        else:
            m = 2
        dis[m] += F(rs[m]) * rinv[m]
        ip[m] += rs[m]
        normal = np.zeros(3, F)
        normal[m] = -rs[m]
        if not inside:
            break
    return hit, normal, color


def ray_march(p, d, floor_height):
    dist, j = F(0.0), 0
    while j < 200 and (p[1] + dist * d[1]) - floor_height > F(1e-8) and dist < DIST_LIMIT:
        dist += (p[1] + dist * d[1]) - floor_height
        j += 1
    return INF if dist > DIST_LIMIT else F(dist)


def floor_color(p, taichi_logo):
    scale = F(1.0)
    if taichi_logo:
        scale = F(1.0) if inside_taichi(float(p[0]), float(p[2])) else F(0.4)
    return scale * np.array([0.3, 0.5, 0.7], F)


def next_hit(grid, lists, x, v, rgb, radius, pos, d, t, floor_height, taichi_logo, motion_blur=True, voxel=False):
    if voxel:
        closest, normal, color = dda_voxel(grid, lists, pos, d)
    else:
        closest, normal, color = dda_particle(grid, lists, x, v, rgb, radius, pos, d, t, motion_blur)
    if d[2] != 0:
        rc = -(pos[2] + F(5.5)) / d[2]
        if 0 < rc < closest:
            closest, normal, color = F(rc), np.array([0, 0, 1], F), np.array([0.6, 0.7, 0.7], F)
    rm = ray_march(pos, d, F(floor_height))
    if rm < DIST_LIMIT and rm < closest:
        closest = rm
        normal = np.array([0, 1, 0], F)  # sdf_normal of the floor plane
        color = floor_color(pos + d * rm, taichi_logo)
    return closest, normal, color


def camera_rays(res, cam, look_at, up, fov, jitter):
    """Primary rays of every pixel (renderer.py:402-410); jitter (res0, res1,
    2) in [0, 1), pixel (u, v)."""
    u, v = np.meshgrid(np.arange(res[0], dtype=F), np.arange(res[1], dtype=F), indexing="ij")
    aspect = F(res[0] / res[1])
    fov = F(fov)
    d0 = normalized(np.asarray(look_at, F) - np.asarray(cam, F))
    fu = F(2.0) * fov * (u + jitter[..., 0]) / F(res[1]) - fov * aspect - F(1e-5)
    fv = F(2.0) * fov * (v + jitter[..., 1]) / F(res[1]) - fov - F(1e-5)
    du = normalized(np.cross(d0, np.asarray(up, F)))
    dv = normalized(np.cross(du, d0))
    d = normalized(d0[None, None] + fu[..., None] * du[None, None] + fv[..., None] * dv[None, None])
    return np.broadcast_to(np.asarray(cam, F), d.shape).copy(), d.astype(F)


def _floor_and_plane(pos, d, floor_height, taichi_logo):
    """Vectorised next_hit for rays that meet no particle."""
    n = pos.shape[0]
    closest = np.full(n, INF, F)
    normal = np.zeros((n, 3), F)
    color = np.zeros((n, 3), F)
    with np.errstate(divide="ignore", invalid="ignore"):
        rc = np.where(d[:, 2] != 0, -(pos[:, 2] + F(5.5)) / d[:, 2], F(-1.0)).astype(F)
    m = (rc > 0) & (rc < closest)
    closest[m], normal[m], color[m] = rc[m], (0, 0, 1), (0.6, 0.7, 0.7)
    dist = np.zeros(n, F)
    run = np.ones(n, bool)
    for _ in range(200):
        s = (pos[:, 1] + dist * d[:, 1]) - F(floor_height)
        run &= (s > F(1e-8)) & (dist < DIST_LIMIT)
        if not run.any():
            break
        dist = np.where(run, dist + s, dist).astype(F)
    rm = np.where(dist > DIST_LIMIT, INF, dist).astype(F)
    m = (rm < DIST_LIMIT) & (rm < closest)
    hp = pos + d * rm[:, None]
    closest[m], normal[m] = rm[m], (0, 1, 0)
    if m.any():
        color[m] = np.stack([floor_color(p, taichi_logo) for p in hp[m]])
    return closest, normal, color


def _out_dir(n, r1, r2):
    u = np.tile(np.array([1, 0, 0], F), (n.shape[0], 1))
    m = np.abs(n[:, 1]) < F(1 - 1e-3)
    if m.any():
        u[m] = normalized(np.cross(n[m], np.array([0, 1, 0], F)))
    v = np.cross(n, u)
    phi = F(2 * np.pi) * r1
    ay, ax = np.sqrt(r2), np.sqrt(F(1.0) - r2)
    return (ax[:, None] * (np.cos(phi)[:, None] * u + np.sin(phi)[:, None] * v) + ay[:, None] * n).astype(F)


def render_no_particles(res, cam, look_at, up, fov, spp, floor_height, taichi_logo, rng):
    """Colour buffer (res0, res1, 3) summed over spp samples, for a scene whose
    particles no ray reaches (renderer.py:396-480, vectorised over paths)."""
    buf = np.zeros((res[0] * res[1], 3), np.float64)
    for _ in range(spp):
        pos, d = camera_rays(res, cam, look_at, up, fov, rng.random((res[0], res[1], 2), dtype=F))
        pos, d = pos.reshape(-1, 3), d.reshape(-1, 3)
        n = pos.shape[0]
        contrib = np.zeros((n, 3), F)
        thr = np.ones((n, 3), F)
        alive = np.ones(n, bool)
        for _depth in range(4):
            idx = np.nonzero(alive)[0]
            if idx.size == 0:
                break
            closest, nrm, col = _floor_and_plane(pos[idx], d[idx], floor_height, taichi_logo)
            hit = np.sum(nrm * nrm, 1) != 0
            hp = pos[idx] + d[idx] * closest[:, None]
            sky = idx[~hit]
            alive[sky] = False
            h = idx[hit]
            if h.size:
                nd = _out_dir(nrm[hit], rng.random(h.size, dtype=F), rng.random(h.size, dtype=F))
                d[h] = nd
                pos[h] = hp[hit] + F(1e-4) * nd
                thr[h] *= col[hit]
                noise = (rng.random((h.size, 3), dtype=F) - F(0.5)) * LIGHT_NOISE
                direct = normalized(LIGHT_DIRECTION[None] + noise)
                dt = np.sum(direct * nrm[hit], 1, dtype=F)
                lit = dt > 0
                if lit.any():
                    sd, _, _ = _floor_and_plane(pos[h][lit], direct[lit], floor_height, taichi_logo)
                    ok = sd > DIST_LIMIT
                    hl = h[lit][ok]
                    contrib[hl] += thr[hl] * dt[lit][ok][:, None]
            # Russian roulette for every path of this bounce (sky paths end anyway)
            maxc = thr[idx].max(1)
            rr = rng.random(idx.size, dtype=F) > maxc
            thr[idx[rr]] = 0
            alive[idx[rr]] = False
            keep = idx[~rr]
            thr[keep] = thr[keep] / thr[keep].max(1, keepdims=True)
        buf += contrib
    return buf.reshape(res[0], res[1], 3)


def tonemap(buf, samples, vignette_strength=0.9, vignette_radius=0.0, center=(0.5, 0.5), exposure=1.5):
    rx, ry = buf.shape[:2]
    u, v = np.meshgrid(np.arange(rx) / rx, np.arange(ry) / ry, indexing="ij")
    darken = 1.0 - vignette_strength * np.maximum(np.sqrt((u - center[0])**2 + (v - center[1])**2) - vignette_radius,
                                                  0)
    return np.sqrt(buf * darken[..., None] * exposure / samples)
