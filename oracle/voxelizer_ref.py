"""CPU restatement of the mesh voxelizer - TEST INFRASTRUCTURE.

Follows taichi-dev/taichi_elements engine/voxelizer.py:46-126
(Voxelizer.voxelize_triangles) in float64, the reference's default
precision: vertex jitter (:53-64), bounding rectangle of voxel columns
clamped to the padding (:66-79), normal = normalized((b - a) x (c - a))
with the |n.z| < 1e-10 skip (:81-84), the inside_ccw test of column centres
in either winding (:10-13, :90-96), the crossing height
int(-n.(base - a) / n.z * inv_dx + 0.5) clamped to res[1] - padding
(:97-101) and the signed fill of [padding, height) (:41-44, :102-108).
Operations are evaluated one at a time in the reference's order (numpy does
not contract them).

Parity unpinned: the reference's kernel needs the Taichi compiler, which is
not importable here, and its tests download their mesh.  Taichi's typing of
Python float literals inside the kernel (the jitter vector, 0.5) is taken as
float64 here.  Used only by tests/.
"""
from __future__ import annotations

import numpy as np

JITTER = np.array([-0.057616723909439505, -0.25608986292614977, 0.06716309129743714])


def grid_res(res, super_sample=2):
    out = []
    for r in res:
        p = 1
        while p < r:
            p *= 2
        out.append(p * super_sample)
    return tuple(out)


def _cross2d(ax, ay, bx, by):
    return ax * by - ay * bx


def _inside_ccw(px, py, a, b, c):
    apx, apy = a[0] - px, a[1] - py
    bpx, bpy = b[0] - px, b[1] - py
    cpx, cpy = c[0] - px, c[1] - py
    return (_cross2d(apx, apy, bpx, bpy) >= 0) & (_cross2d(bpx, bpy, cpx, cpy) >= 0) & (_cross2d(cpx, cpy, apx, apy)
                                                                                         >= 0)


def voxelize(triangles, res, dx, padding=3):
    """Voxel counts (rx, ry, rz) int32 for voxel grid `res` and voxel size dx."""
    rx, ry, rz = res
    inv_dx = 1 / dx
    vox = np.zeros(res, np.int32)
    tri = np.asarray(triangles, np.float64).reshape(-1, 3, 3)
    jit = JITTER * 1e-8
    for t in tri:
        a, b, c = t[0] + jit, t[1] + jit, t[2] + jit
        bmin = np.minimum(np.minimum(a, b), c)
        bmax = np.maximum(np.maximum(a, b), c)
        p_min = max(padding, int(np.floor(bmin[0] * inv_dx)))
        p_max = min(rx - padding, int(np.floor(bmax[0] * inv_dx)) + 1)
        q_min = max(padding, int(np.floor(bmin[1] * inv_dx)))
        q_max = min(ry - padding, int(np.floor(bmax[1] * inv_dx)) + 1)
        e1, e2 = b - a, c - a
        n = np.array([e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]])
        length = np.sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2])
        n = n * (1.0 / length)
        if not abs(n[2]) >= 1e-10 or p_max <= p_min or q_max <= q_min:
            continue
        inc = 1 if n[2] > 0 else -1
        p, q = np.meshgrid(np.arange(p_min, p_max), np.arange(q_min, q_max), indexing="ij")
        px = (p.astype(np.float64) + 0.5) * dx
        py = (q.astype(np.float64) + 0.5) * dx
        hit = _inside_ccw(px, py, a, b, c) | _inside_ccw(px, py, a, c, b)
        dot = (n[0] * (px - a[0]) + n[1] * (py - a[1])) + n[2] * (0.0 - a[2])
        hf = (-dot / n[2]) * inv_dx + 0.5
        height = np.trunc(np.clip(hf, -2147483000.0, 2147483000.0)).astype(np.int64)
        height = np.minimum(np.minimum(height, ry - padding), rz)
        for pi, qi, h in zip(p[hit], q[hit], height[hit]):
            if h > padding:
                vox[pi, qi, padding:h] += inc
    return vox
