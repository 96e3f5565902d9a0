"""The constitutive update of P2G on chosen deformation gradients, through the
diagnostic entry point mpm_constitutive_eval (the device code the P2G
kernels run), against the reference's corotated stress
(engine/mpm_solver.py:527-551) evaluated in float64 with numpy's SVD:
stress = 2 mu (F - U V^T) F^T + la J (J - 1) I, F = (I + dt C) F_old,
affine = -dt p_vol 4 inv_dx^2 stress + p_mass C (:569-574).

Flattened particles: the vertical row of F about 1e-9 times a combination of
the other two rows, the state an elastic body reaches when it lies flattened
against a wall (det F at float32 rounding level, around 1e-17).  Newton's
polar iteration can overflow on them (whether it does depends on the
rounding of the kernel it is inlined in), and the update must then take the
SVD: every output must be finite.  The stress stays well conditioned
there (the undetermined part of U V^T multiplies the vanishing singular
value), so elastic and stationary particles are compared with the float64
evaluation at 1e-5 of the largest affine entry; well-conditioned
deformation gradients (rotation times a stretch of a few percent) at the
same bound.  Snow is checked for finiteness (its clamp rebuilds F).
"""
import ctypes

import numpy as np
import pytest
import torch

from taichi_elements_gb300.mpm_solver import MPMSolver

pytestmark = pytest.mark.gpu


def _rotations(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
                     np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
                     np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)


def flattened(rng, n):
    r0 = np.stack([0.96 + 0.03 * rng.random(n), 0.01 * rng.standard_normal(n), 0.003 * rng.standard_normal(n)], -1)
    r2 = np.stack([0.003 * rng.standard_normal(n), 0.003 * rng.standard_normal(n), 0.95 + 0.03 * rng.random(n)], -1)
    r1 = 1e-9 * rng.standard_normal((n, 1)) * r0 + 1e-9 * rng.standard_normal((n, 1)) * r2
    F = np.stack([r0, r1, r2], 1)
    C = 0.15 * rng.standard_normal((n, 3, 3))
    C[:, 1, 0] = 1e-5 * rng.standard_normal(n)
    C[:, 1, 1] = -89.0 + rng.standard_normal(n)
    C[:, 1, 2] = 1e-5 * rng.standard_normal(n)
    return F.astype(np.float32), C.astype(np.float32)


def regular(rng, n):
    F = _rotations(rng, n) @ (np.eye(3) + 0.04 * rng.standard_normal((n, 3, 3)))
    return F.astype(np.float32), (3.0 * rng.standard_normal((n, 3, 3))).astype(np.float32)


def evaluate(s, mat, F, C, Jp, dt):
    dev = s.device
    m = torch.as_tensor(mat, dtype=torch.int32, device=dev)
    f = torch.as_tensor(F.reshape(-1, 9), device=dev).contiguous()
    c = torch.as_tensor(C.reshape(-1, 9), device=dev).contiguous()
    j = torch.as_tensor(Jp, device=dev).contiguous()
    a = torch.empty_like(f)
    p = s.params
    rc = s._lib.mpm_constitutive_eval(ctypes.byref(p), len(mat), m.data_ptr(), f.data_ptr(), c.data_ptr(),
                                      j.data_ptr(), a.data_ptr(), float(dt), torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    return f.cpu().numpy().reshape(-1, 3, 3), j.cpu().numpy(), a.cpu().numpy().reshape(-1, 3, 3)


def reference_affine(p, mat, F, C, Jp, dt):
    """float64 corotated affine matrix of elastic (h = 0.3) and stationary
    (h = exp(10 (1 - Jp))) particles."""
    F64, C64 = F.astype(np.float64), C.astype(np.float64)
    Fn = (np.eye(3) + dt * C64) @ F64
    U, sig, Vt = np.linalg.svd(Fn)
    R = U @ Vt  # U V^T: unchanged by the sign convention of the SVD
    J = np.linalg.det(Fn)
    h = np.where(mat == 1, 0.3, np.exp(10.0 * (1.0 - Jp.astype(np.float64))))
    mu, la = p.mu0 * h, p.la0 * h
    stress = 2 * mu[:, None, None] * ((Fn - R) @ np.swapaxes(Fn, 1, 2)) + \
        (la * J * (J - 1))[:, None, None] * np.eye(3)
    return -dt * p.stress_k * stress + p.p_mass * C64


@pytest.mark.parametrize("kind", ["flattened", "regular"])
def test_constitutive_update_matches_float64_corotated_stress(kind):
    s = MPMSolver((32, 32, 32), size=1)
    s.add_cube((0.4, 0.4, 0.4), (0.1, 0.1, 0.1), MPMSolver.material_elastic)  # parameters and workspace
    s._prepare(s.default_dt)
    rng = np.random.default_rng(61 if kind == "flattened" else 62)
    n = 20000
    F, C = (flattened if kind == "flattened" else regular)(rng, 3 * n)
    mat = np.repeat(np.array([1, 4, 2], np.int32), n)
    Jp = np.ones(3 * n, np.float32)
    dt = s.default_dt
    Fo, Jo, A = evaluate(s, mat, F, C, Jp, dt)
    for name, arr in (("F", Fo), ("Jp", Jo), ("affine", A)):
        bad = ~np.isfinite(arr.reshape(3 * n, -1)).all(1)
        assert not bad.any(), f"{kind}: {int(bad.sum())} non-finite {name} (materials {np.unique(mat[bad])})"
    sel = mat != 2
    ref = reference_affine(s.params, mat[sel], F[sel], C[sel], Jp[sel], dt)
    err = np.abs(A[sel] - ref).max() / np.abs(ref).max()
    # elastic and stationary F is (I + dt C) F itself
    Fref = (np.eye(3) + dt * C[sel].astype(np.float64)) @ F[sel].astype(np.float64)
    errF = np.abs(Fo[sel] - Fref).max()
    print(f"\n{kind}: affine rel L-inf {err:.2e}, F abs L-inf {errF:.2e}")
    assert err <= 1e-5
    assert errF <= 1e-6


def test_flattened_elastic_cube_stays_finite():
    """The scene of the 64-scene batch (scenes.batched_scenes()[46]: a soft
    elastic cube, E 1.8e4, 112,617 particles, 32^3) that lands and lies
    flattened on the floor: without the polar iteration's overflow check its
    particles turned non-finite about 1236 substeps in (fused frames and
    per-substep launches alike; the float32 and float64 oracles stay
    finite).  1400 substeps in fused frames of 50."""
    from taichi_elements_gb300 import scenes
    sc = scenes.batched_scenes()[46]
    s = sc.make_solver()
    frame_dt = 50 * s.default_dt * 0.999
    for _ in range(28):
        s.step(frame_dt)  # raises on a device status (non-finite positions)
    assert s.total_substeps >= 1400
    st = s.full_state()
    for k in ("x", "v", "C", "F", "Jp"):
        assert bool(torch.isfinite(st[k]).all()), k
