"""Generates the golden fixtures of tests/golden/ (run from the repo root).

The reference (taichi-dev/taichi_elements) ships no golden vectors and its
Taichi runtime is not importable here, so the fixtures are produced by the
independent float64 numpy restatement ``oracle.oracle.np_substep`` of
engine/mpm_solver.py (one substep each).  They pin the C oracle and the GPU
engine to the same numbers across machines; they do not replace a run of the
reference itself.

    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def mixed_state(seed, n, res):
    rng = np.random.default_rng(seed)
    x = 0.25 + 0.5 * rng.random((n, 3))
    mat = rng.integers(0, 5, n).astype(np.int32)
    P = O.Particles.seeded(x, mat, v=rng.uniform(-1, 1, (n, 3)))
    # smooth-ish deformation: F = I + small random strain, C random
    P.F = P.F + 0.02 * rng.standard_normal((n, 3, 3))
    P.C = 2.0 * rng.standard_normal((n, 3, 3))
    P.Jp = np.where(mat == O.MAT_SAND, -0.02 * rng.random(n), 1 + 0.01 * rng.standard_normal(n))
    P.Jp = np.where(mat == O.MAT_WATER, 1 + 0.005 * rng.standard_normal(n), P.Jp)
    # water F is diag(J,1,1) in the reference
    w = mat == O.MAT_WATER
    P.F[w] = np.eye(3)
    P.F[w, 0, 0] = P.Jp[w]
    return P


CASES = {
    "mixed_32": dict(seed=11, n=600, res=(32, 32, 32), dt=1e-4,
                     pp=[dict(kind=O.KIND_BOX, surface=0),
                         dict(kind=O.KIND_SURFACE, surface=2, point=(0.5, 0.3, 0.5), normal=(0.2, 1, 0.1),
                              friction=0.3),
                         dict(kind=O.KIND_SPHERE, surface=1, point=(0.5, 0.5, 0.5), radius=0.1)]),
    "walls_24": dict(seed=12, n=400, res=(24, 24, 24), dt=2e-4,
                     pp=[dict(kind=O.KIND_BOX, surface=0),
                         dict(kind=O.KIND_SPHERE, surface=0, point=(0.5, 0.5, 0.5), radius=0.15),
                         dict(kind=O.KIND_SURFACE, surface=1, point=(0.5, 0.5, 0.5), normal=(1, 1, 0))]),
}


def make(name, c):
    cfg = O.Config(res=c["res"], postprocess=c["pp"])
    P = mixed_state(c["seed"], c["n"], c["res"])
    if name == "walls_24":
        # push particles against the walls so the box condition acts
        P.x[:, 0] = np.where(P.x[:, 0] < 0.5, 0.1 + 0.02 * P.x[:, 0], 0.88 + 0.02 * P.x[:, 0])
    P0 = P.copy()
    out, grid = O.np_substep(cfg, P, c["dt"])
    keys = np.array(sorted(grid.keys()), dtype=np.int64)
    gm = np.array([grid[tuple(k)][0] for k in keys])
    gmv = np.array([grid[tuple(k)][1] for k in keys])
    gv = np.array([grid[tuple(k)][2] for k in keys])
    np.savez_compressed(
        os.path.join(OUT, f"{name}.npz"), res=np.asarray(c["res"]), dt=c["dt"], seed=c["seed"],
        x=P0.x, v=P0.v, C=P0.C, F=P0.F, Jp=P0.Jp, material=P0.material,
        out_x=out.x, out_v=out.v, out_C=out.C, out_F=out.F, out_Jp=out.Jp,
        grid_nodes=keys, grid_m=gm, grid_mv=gmv, grid_v=gv, postprocess=json.dumps(c["pp"]))


if __name__ == "__main__":
    for k, c in CASES.items():
        make(k, c)
        print("wrote", k)
