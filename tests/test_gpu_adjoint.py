"""Gradients of a final-state loss through a GPU rollout (float32 forward,
hand-written adjoint, checkpointed segments) against two float64
references: PyTorch autograd through oracle/torch_ref.py, and central
finite differences of the C oracle along 10 random directions each for the
initial velocities and for E.  Case: the differentiable scene's small copy,
a 32^3 grid with 2,000 water + 2,000 elastic particles, 200 substeps,
checkpoints every 50.

Tolerance: relative L2 error of dL/dv0 and dL/dE against the float64
autograd gradient <= 1e-3, and each directional derivative within 2e-3 of
the finite difference (relative to the larger of |FD| and the gradient's
norm times the direction's RMS); float32 round-off over the rollout sets
this bound (measured on a GB300: 4e-7 and 9e-6 against autograd, <= 2e-4
against FD).
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from oracle.torch_ref import TorchMPM
from oracle.torch_ref import com_loss as com_loss_ref
from taichi_elements_gb300 import scenes

pytestmark = pytest.mark.gpu

NSUB = 200
K = 50
NDIR = 10


def make_case(seed=3, n_each=2000):
    sc = scenes.elastic_on_water(res=32, n_each=n_each)
    rng = np.random.default_rng(seed)
    n = sc.n
    v0 = (sc.v + rng.normal(0.0, 0.3, (n, 3))).astype(np.float32)
    E = np.exp(rng.uniform(np.log(2e4), np.log(2e5), n)).astype(np.float32)
    return sc, v0, E


def gpu_grads(sc, v0, E, nsub=NSUB, k=K, keep_workspaces=None, colliders=()):
    from taichi_elements_gb300.differentiable import Rollout, com_loss, rollout_positions
    from taichi_elements_gb300.mpm_solver import MPMSolver
    s = MPMSolver(sc.res, per_particle_E=True)
    for c in colliders:
        if c["kind"] == O.KIND_SURFACE:
            s.add_surface_collider(c["point"], c["normal"], c["surface"], c.get("friction", 0.0))
        else:
            s.add_sphere_collider(c["point"], c["radius"], c["surface"])
    for m in (0, 1):
        sel = sc.material == m
        s.add_particles(sc.x[sel], m, E=torch.as_tensor(E[sel]))
    # particle ids follow the add order: water first, then elastic
    order = np.concatenate([np.nonzero(sc.material == m)[0] for m in (0, 1)])
    R = Rollout(s, nsub, checkpoint_every=k, keep_workspaces=keep_workspaces)
    v = torch.tensor(v0[order], device="cuda", requires_grad=True)
    e = torch.tensor(E[order], device="cuda", requires_grad=True)
    x = rollout_positions(R, v, e)
    mat = torch.as_tensor(sc.material[order], device="cuda")
    L = com_loss(x, mat, torch.tensor(sc.target, dtype=torch.float32, device="cuda"))
    L.backward()
    inv = np.argsort(order)
    return (float(L), x.detach().cpu().numpy()[inv], v.grad.cpu().numpy()[inv], e.grad.cpu().numpy()[inv])


def torch_grads(sc, v0, E):
    T = TorchMPM(sc.res)
    x0 = torch.tensor(sc.x, dtype=torch.float64)
    v = torch.tensor(v0, dtype=torch.float64, requires_grad=True)
    e = torch.tensor(E, dtype=torch.float64, requires_grad=True)
    mat = torch.tensor(sc.material)
    xT = T.rollout(x0, v, mat, e, sc.default_dt, NSUB)
    L = com_loss_ref(xT, mat, torch.tensor(sc.target))
    L.backward()
    return float(L), xT.detach().numpy(), v.grad.numpy(), e.grad.numpy()


def test_adjoint_matches_float64_autograd():
    sc, v0, E = make_case()
    Lg, xg, gv, gE = gpu_grads(sc, v0, E)
    Lr, xr, gv_r, gE_r = torch_grads(sc, v0, E)
    assert np.abs(xg - xr).max() < 1e-4
    assert abs(Lg - Lr) <= 1e-3 * abs(Lr) + 1e-9
    ev = np.linalg.norm(gv - gv_r) / np.linalg.norm(gv_r)
    eE = np.linalg.norm(gE - gE_r) / np.linalg.norm(gE_r)
    print(f"adjoint vs float64 autograd: x {np.abs(xg - xr).max():.2e}, L {abs(Lg - Lr) / abs(Lr):.2e}, "
          f"dL/dv0 {ev:.2e}, dL/dE {eE:.2e}")
    assert ev < 1e-3, ev
    assert eE < 1e-3, eE


def test_adjoint_directional_derivatives_match_finite_differences():
    sc, v0, E = make_case(seed=4)
    _, _, gv, gE = gpu_grads(sc, v0, E)
    cfg = O.Config(res=sc.res)
    sel = sc.material == 1

    def loss(v, e):
        P = O.Particles.seeded(sc.x, sc.material, v=v.astype(np.float64), E=e.astype(np.float64))
        R = O.Runner(cfg, P)
        R.run(sc.default_dt, NSUB)
        return float(((R.P.x[sel].mean(0) - sc.target)**2).sum())

    rng = np.random.default_rng(7)
    v0d, Ed = v0.astype(np.float64), E.astype(np.float64)

    def close(gd, fd, g, d):
        scale = np.linalg.norm(g) * np.linalg.norm(d) / np.sqrt(d.size)  # typical |<g, d>|
        return abs(gd - fd) <= 2e-3 * max(abs(fd), scale)

    for _ in range(NDIR):
        d = rng.standard_normal(v0.shape)
        h = 1e-4
        fd = (loss(v0d + h * d, Ed) - loss(v0d - h * d, Ed)) / (2 * h)
        print(f"FD v0 direction: adjoint {(gv * d).sum():.6e} fd {fd:.6e}")
        assert close((gv * d).sum(), fd, gv, d), ((gv * d).sum(), fd)
        dE = rng.standard_normal(E.shape) * Ed
        hE = 1e-4
        fdE = (loss(v0d, Ed + hE * dE) - loss(v0d, Ed - hE * dE)) / (2 * hE)
        print(f"FD E direction: adjoint {(gE * dE).sum():.6e} fd {fdE:.6e}")
        assert close((gE * dE).sum(), fdE, gE * Ed, dE / Ed), ((gE * dE).sum(), fdE)


def test_adjoint_with_and_without_kept_workspaces_agree():
    """The recompute that keeps one workspace per substep and the one that
    re-runs each substep's forward before its adjoint give the same
    gradients (up to the order of float atomics); 40 substeps in segments of
    16, 16 and 8."""
    sc, v0, E = make_case(seed=5, n_each=1200)
    a = gpu_grads(sc, v0, E, nsub=40, k=16, keep_workspaces=True)
    b = gpu_grads(sc, v0, E, nsub=40, k=16, keep_workspaces=False)
    assert np.abs(a[1] - b[1]).max() < 1e-5
    for ga, gb in ((a[2], b[2]), (a[3], b[3])):
        assert np.linalg.norm(ga - gb) <= 1e-3 * np.linalg.norm(gb)


def test_adjoint_through_colliders_matches_finite_differences():
    """The transposed collider projections of the adjoint grid update: a
    separate plane with friction 0.3 tilted through the water slab and a
    slip sphere in the elastic cube (engine/mpm_solver.py:618-687), against
    float64 central differences of the C oracle run with the same colliders
    (the PyTorch reference models only the bounding box)."""
    sc, v0, E = make_case(seed=6)
    # the plane passes no grid node (a node on it would make the inside test
    # a matter of rounding, and the float32 and float64 runs would differ)
    colliders = [dict(kind=O.KIND_SURFACE, surface=2, point=(0.5, 0.1513, 0.5), normal=(0.23, 1.0, 0.11),
                      friction=0.3),
                 dict(kind=O.KIND_SPHERE, surface=1, point=(0.5, 0.27, 0.35), radius=0.08)]
    _, _, gv, gE = gpu_grads(sc, v0, E, colliders=colliders)
    cfg = O.Config(res=sc.res, postprocess=[dict(kind=O.KIND_BOX, surface=0)] + colliders)
    sel = sc.material == 1

    def loss(v, e):
        P = O.Particles.seeded(sc.x, sc.material, v=v.astype(np.float64), E=e.astype(np.float64))
        R = O.Runner(cfg, P)
        R.run(sc.default_dt, NSUB)
        return float(((R.P.x[sel].mean(0) - sc.target)**2).sum())

    # the colliders change the motion: the loss differs from the free run's
    free = O.Runner(O.Config(res=sc.res), O.Particles.seeded(sc.x, sc.material, v=v0.astype(np.float64),
                                                             E=E.astype(np.float64)))
    free.run(sc.default_dt, NSUB)
    L_free = float(((free.P.x[sel].mean(0) - sc.target)**2).sum())
    L_coll = loss(v0.astype(np.float64), E.astype(np.float64))
    assert abs(L_coll - L_free) > 1e-3 * abs(L_free)
    rng = np.random.default_rng(8)
    v0d, Ed = v0.astype(np.float64), E.astype(np.float64)

    def close(gd, fd, g, d):
        scale = np.linalg.norm(g) * np.linalg.norm(d) / np.sqrt(d.size)
        return abs(gd - fd) <= 2e-3 * max(abs(fd), scale)

    for _ in range(NDIR):
        d = rng.standard_normal(v0.shape)
        h = 1e-4
        fd = (loss(v0d + h * d, Ed) - loss(v0d - h * d, Ed)) / (2 * h)
        print(f"colliders, FD v0 direction: adjoint {(gv * d).sum():.6e} fd {fd:.6e}")
        assert close((gv * d).sum(), fd, gv, d), ((gv * d).sum(), fd)
        dE = rng.standard_normal(E.shape) * Ed
        fdE = (loss(v0d, Ed + h * dE) - loss(v0d, Ed - h * dE)) / (2 * h)
        print(f"colliders, FD E direction: adjoint {(gE * dE).sum():.6e} fd {fdE:.6e}")
        assert close((gE * dE).sum(), fdE, gE * Ed, dE / Ed), ((gE * dE).sum(), fdE)

