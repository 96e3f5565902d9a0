"""Golden vectors of the substep made by the reference's own solver code.

Loads taichi-dev/taichi_elements engine/mpm_solver.py from the reference
checkout under the stand-in ``taichi`` module of tests/golden/taichi_standin.py
(the real Taichi 1.1.0 runtime cannot be installed here) and runs its
kernels on small seeded scenes:

* one substep phase by phase, in the order of ``MPMSolver.step``
  (engine/mpm_solver.py:789-797): ``grid.deactivate_all``, ``build_pid``
  (:344-361), ``p2g`` (:487-584, with ``sand_projection`` :321-342),
  ``grid_normalization_and_gravity`` (:586-598), the post-process list
  (bounding box :600-616, ``add_sphere_collider`` :618-642,
  ``add_surface_collider`` :647-687), ``g2p`` (:694-724) and
  ``compute_max_velocity`` (:726-735), recording the active blocks, the grid
  after P2G, the grid after the update and the particles;
* a short trajectory through ``MPMSolver.step(frame_dt)`` itself (:748-821);
* the fused mode (``use_g2p2g=True``, ``g2p2g`` :363-485, loop :773-787)
  over three substeps.

Every case runs in float64 (fields and arithmetic; the reference run with
default_fp=f64) and, for the one-substep cases, in float32.  Initial states
are set through ``read_restart`` (:1106-1144) plus direct writes of C, F and
Jp into the particle fields (the reference has no API for an evolved state).

Run in the build container, where the reference checkout is readable:

    python tests/golden/make_reference_golden.py

It writes tests/golden/ref_<case>.npz.
"""
import contextlib
import importlib.util
import io
import os
import sys
import time
import types

import numpy as np

REF = "/root/reference"
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import taichi_standin as ti  # noqa: E402

MAT_WATER, MAT_ELASTIC, MAT_SNOW, MAT_SAND, MAT_STATIONARY = 0, 1, 2, 3, 4


def load_reference_solver():
    sys.modules["taichi"] = ti
    pkg = types.ModuleType("engine")
    pkg.__path__ = []
    sys.modules["engine"] = pkg
    spec = importlib.util.spec_from_file_location("engine.mpm_solver", os.path.join(REF, "engine", "mpm_solver.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["engine.mpm_solver"] = mod
    spec.loader.exec_module(mod)
    return mod.MPMSolver


# ------------------------------------------------------------- scenes ----

def _rot(rng):
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def evolved_state(rng, centers, half, n_each, mats, v_amp=1.0):
    """Clusters of particles per material with a deformed state: F a rotation
    times a strain of a few percent (snow beyond its clamp range, sand in
    tension and compression), random affine C, hardening Jp."""
    xs, ms = [], []
    for c, m in zip(centers, mats):
        xs.append(np.asarray(c) + half * (2 * rng.random((n_each, 3)) - 1))
        ms.append(np.full(n_each, m, np.int32))
    x = np.concatenate(xs).astype(np.float32)
    mat = np.concatenate(ms)
    n = len(x)
    v = (v_amp * rng.uniform(-1, 1, (n, 3))).astype(np.float32)
    F = np.empty((n, 3, 3))
    for p in range(n):
        F[p] = _rot(rng) @ (np.eye(3) + 0.04 * rng.standard_normal((3, 3)))
    C = 3.0 * rng.standard_normal((n, 3, 3))
    Jp = 1.0 + 0.02 * rng.standard_normal(n)
    sand = mat == MAT_SAND
    Jp[sand] = rng.uniform(-0.03, 0.01, sand.sum())  # both branches of the return map
    water = mat == MAT_WATER
    F[water] = np.eye(3)
    F[water, 0, 0] = 1.0 + 0.01 * rng.standard_normal(water.sum())
    Jp[water] = F[water, 0, 0]
    st = mat == MAT_STATIONARY
    Jp[st] = 1.0
    return dict(x=x, v=v, C=C.astype(np.float32), F=F.astype(np.float32), Jp=Jp.astype(np.float32), material=mat)


def case_mixed(rng):
    s = evolved_state(rng, [(0.3, 0.45, 0.3), (0.55, 0.5, 0.35), (0.4, 0.3, 0.6), (0.65, 0.3, 0.65),
                            (0.5, 0.7, 0.5)], 0.06, 300, [MAT_WATER, MAT_ELASTIC, MAT_SNOW, MAT_SAND, MAT_STATIONARY])
    pp = [dict(kind="surface", point=(0.5, 0.2513, 0.5), normal=(0.21, 1.0, 0.13), surface=2, friction=0.3),
          dict(kind="sphere", center=(0.5, 0.55, 0.5), radius=0.1, surface=1)]
    return dict(res=(24, 24, 24), state=s, postprocess=pp, kw={})


def case_walls(rng):
    """Particles pressed against the domain walls (the box condition acts),
    a sticky sphere, a sticky plane and a slip plane with friction; some
    elastic particles inverted (det F < 0) and one nearly degenerate;
    water_density 1.5."""
    s = evolved_state(rng, [(0.17, 0.5, 0.5), (0.83, 0.5, 0.5), (0.5, 0.17, 0.5), (0.5, 0.5, 0.83)],
                      0.05, 250, [MAT_ELASTIC, MAT_SNOW, MAT_WATER, MAT_SAND], v_amp=0.5)
    n = len(s["x"])
    out = np.sign(s["x"] - 0.5) * (np.abs(s["x"] - 0.5) > 0.25)
    s["v"] = (s["v"] + 2.0 * out).astype(np.float32)  # moving into the walls
    el = np.nonzero(s["material"] == MAT_ELASTIC)[0]
    inv = el[:20]
    s["F"][inv, :, 2] *= -1.0  # det F < 0
    s["F"][el[20]] = np.diag([1.0, 1.0, 1e-3]).astype(np.float32)  # nearly rank-deficient
    s["F"][el[21]] = np.eye(3, dtype=np.float32)  # repeated singular values
    assert n == 1000
    pp = [dict(kind="sphere", center=(0.5, 0.5, 0.5), radius=0.12, surface=0),
          dict(kind="surface", point=(0.5, 0.13, 0.5), normal=(0.0, 1.0, 0.0), surface=0, friction=0.0),
          dict(kind="surface", point=(0.8013, 0.5, 0.5), normal=(-1.0, 0.31, 0.07), surface=1, friction=0.2)]
    return dict(res=(24, 24, 24), state=s, postprocess=pp, kw=dict(water_density=1.5))


def case_unbounded(rng):
    """unbounded=True: the box condition sits at +-grid_size/2 -+ padding, so
    particles leave the nominal [0, 1]^3 box freely."""
    s = evolved_state(rng, [(0.04, 0.5, 0.5), (0.96, 0.04, 0.5)], 0.05, 200, [MAT_ELASTIC, MAT_WATER], v_amp=0.3)
    s["v"][:, 0] -= 2.0 * (s["x"][:, 0] < 0.5) - 2.0 * (s["x"][:, 0] >= 0.5)
    s["v"][:, 1] -= 1.5 * (s["x"][:, 1] < 0.2)
    return dict(res=(24, 24, 24), state=s, postprocess=[], kw=dict(unbounded=True))


def case_no_plasticity(rng):
    """support_plasticity=False: no Jp field, water restarts from F = I,
    sand carries no stress."""
    s = evolved_state(rng, [(0.3, 0.4, 0.3), (0.6, 0.4, 0.35), (0.35, 0.4, 0.65), (0.65, 0.4, 0.65)], 0.06, 250,
                      [MAT_WATER, MAT_ELASTIC, MAT_SNOW, MAT_SAND])
    pp = [dict(kind="surface", point=(0.5, 0.3, 0.5), normal=(0.0, 1.0, 0.0), surface=2, friction=0.3)]
    return dict(res=(24, 24, 24), state=s, postprocess=pp, kw=dict(support_plasticity=False))


def case_degenerate(rng):
    """Deformation gradients that stress the SVD convention, for every
    material that takes the SVD: inverted (det F < 0), rank-deficient,
    repeated and nearly repeated singular values, strong stretch and strong
    compression, each rotated at random."""
    s = evolved_state(rng, [(0.3, 0.5, 0.3), (0.6, 0.5, 0.35), (0.35, 0.5, 0.65), (0.65, 0.5, 0.65)], 0.06, 240,
                      [MAT_ELASTIC, MAT_SNOW, MAT_SAND, MAT_STATIONARY], v_amp=0.3)
    kinds = [np.diag([1.0, 1.0, -1.0]), np.diag([1.0, 0.8, 0.0]), np.eye(3) * 1.001, np.diag([1.02, 1.02, 0.99]),
             np.diag([1.0, 1.0, 1.0 + 1e-6]), np.diag([2.5, 0.4, 1.0]), np.diag([0.5, 0.6, 0.7]),
             np.diag([1.03, -0.97, 1.0])]
    n = len(s["x"])
    F = np.empty((n, 3, 3))
    for p in range(n):
        R1, R2 = _rot(rng), _rot(rng)
        F[p] = R1 @ kinds[p % len(kinds)] @ R2.T
    s["F"] = F.astype(np.float32)
    s["C"] = (0.3 * s["C"]).astype(np.float32)
    # one substep only: a rank-deficient snow particle ends with Jp = 0 (its
    # hardening becomes e^10), which makes a longer trajectory meaningless
    return dict(res=(24, 24, 24), state=s, postprocess=[], kw={}, no_trajectory=True)


def case_flattened(rng):
    """Particles flattened against the floor, the state a soft elastic cube
    reaches some hundred substeps after it lands: the vertical row of F is
    about 1e-9 times a combination of the other two rows (the small
    off-diagonal rates of C make it so), so det F is at the level of float32
    rounding, around 1e-17; C has a large negative vertical rate.  A layer
    two cells above the floor of elastic, snow and stationary particles: the
    materials whose rotation factor can come from Newton's polar iteration
    instead of the SVD."""
    n_each = 250
    xs, ms = [], []
    for k, m in enumerate([MAT_ELASTIC, MAT_SNOW, MAT_STATIONARY]):
        cx = 0.3 + 0.2 * k
        xs.append(np.column_stack([cx + 0.08 * (2 * rng.random(n_each) - 1),
                                   (2.0 + 0.9 * rng.random(n_each)) / 24.0,
                                   0.5 + 0.08 * (2 * rng.random(n_each) - 1)]))
        ms.append(np.full(n_each, m, np.int32))
    x = np.concatenate(xs).astype(np.float32)
    mat = np.concatenate(ms)
    n = len(x)
    F = np.empty((n, 3, 3))
    C = np.empty((n, 3, 3))
    for p in range(n):
        r0 = np.array([0.96 + 0.03 * rng.random(), 0.01 * rng.standard_normal(), 0.003 * rng.standard_normal()])
        r2 = np.array([0.003 * rng.standard_normal(), 0.003 * rng.standard_normal(), 0.95 + 0.03 * rng.random()])
        F[p] = [r0, 1e-9 * rng.standard_normal() * r0 + 1e-9 * rng.standard_normal() * r2, r2]
        C[p] = 0.15 * rng.standard_normal((3, 3))
        C[p, 1] = [1e-5 * rng.standard_normal(), -89.0 + rng.standard_normal(), 1e-5 * rng.standard_normal()]
    v = (0.05 * rng.uniform(-1, 1, (n, 3))).astype(np.float32)
    v[:, 1] = 0.0
    s = dict(x=x, v=v, C=C.astype(np.float32), F=F.astype(np.float32), Jp=np.ones(n, np.float32), material=mat)
    return dict(res=(24, 24, 24), state=s, postprocess=[], kw={}, no_trajectory=True)


CASES = {"mixed_24": case_mixed, "walls_24": case_walls, "unbounded_24": case_unbounded,
         "no_plasticity_24": case_no_plasticity, "degenerate_24": case_degenerate,
         "flattened_24": case_flattened}


# ------------------------------------------------------------ running ----

def make_solver(MPMSolver, case):
    s = MPMSolver(case["res"], use_voxelizer=False, max_num_particles=1 << 14, **case["kw"])
    for c in case["postprocess"]:
        if c["kind"] == "surface":
            s.add_surface_collider(c["point"], c["normal"], surface=c["surface"], friction=c["friction"])
        else:
            s.add_sphere_collider(c["center"], c["radius"], surface=c["surface"])
    st = case["state"]
    n = len(st["x"])
    s.read_restart(n, st["x"], st["v"], st["material"], np.full(n, 0xFFFFFF, np.int32))
    if not s.use_g2p2g:
        s.C.from_numpy(st["C"])
    s.F.from_numpy(st["F"])
    if s.support_plasticity:
        s.Jp.from_numpy(st["Jp"])
    return s


def particles(s):
    out = dict(x=s.x.to_numpy(), v=s.v.to_numpy(), F=s.F.to_numpy())
    if not s.use_g2p2g:
        out["C"] = s.C.to_numpy()
    if s.support_plasticity:
        out["Jp"] = s.Jp.to_numpy()
    return out


def one_substep(s, dt):
    """The body of MPMSolver.step for one substep (:789-799), phase by phase."""
    tree = s.grid_m.snode.tree
    s.grid.deactivate_all()
    s.build_pid(s.pid, s.grid_m, 0.5)
    pblocks = np.array([k for k in sorted(tree.lists)], dtype=np.int64).reshape(-1, 3)
    pcounts = np.array([len(tree.lists[k]) for k in sorted(tree.lists)], dtype=np.int64)
    s.p2g(dt)
    nodes, m = tree.node_values(s.grid_m)
    _, mv = tree.node_values(s.grid_v)
    s.grid_normalization_and_gravity(dt, s.grid_v, s.grid_m)
    for p in s.grid_postprocess:
        p(s.t, dt, s.grid_v)
    s.t += dt
    nodes2, v = tree.node_values(s.grid_v)
    assert np.array_equal(nodes, nodes2)
    s.g2p(dt)
    maxv = s.compute_max_velocity()
    out = dict(pblocks=pblocks, pcounts=pcounts, grid_nodes=nodes, grid_m=m, grid_mv=mv, grid_v=v,
               gblocks=np.array(tree.active_blocks(), dtype=np.int64).reshape(-1, 3), maxv=np.float64(maxv))
    out.update({"out_" + k: val for k, val in particles(s).items()})
    return out


# Collider planes and spheres are placed so that no grid node lies on their
# surface: a node exactly on a plane makes the collider's branch a matter of
# rounding, and float32 and float64 runs would then differ by a whole
# projection at that node.


def run_case(MPMSolver, name, fn, traj_substeps=6):
    rng = np.random.default_rng(sum(map(ord, name)))
    case = fn(rng)
    st = case["state"]
    res = dict(res=np.array(case["res"]), n=len(st["x"]), **{"in_" + k: v for k, v in st.items()})
    res["postprocess"] = np.array(repr(case["postprocess"]))
    res["kw"] = np.array(repr(case["kw"]))
    for prec in ("f64", "f32"):
        ti.set_precision(prec)
        s = make_solver(MPMSolver, case)
        dt = float(np.float32(s.default_dt))
        res["dt"] = dt
        t0 = time.time()
        with contextlib.redirect_stdout(io.StringIO()):
            out = one_substep(s, dt)
        print(f"  {name} {prec}: one substep {time.time() - t0:.1f} s, {len(out['grid_nodes'])} nodes")
        res.update({f"{prec}_{k}": v for k, v in out.items()})
    if case.get("no_trajectory"):
        return res
    # trajectory through MPMSolver.step itself, float64
    ti.set_precision("f64")
    s = make_solver(MPMSolver, case)
    frame_dt = traj_substeps * s.default_dt * 0.999
    t0 = time.time()
    with contextlib.redirect_stdout(io.StringIO()):
        s.step(frame_dt)
    print(f"  {name} f64: step() of {s.total_substeps} substeps {time.time() - t0:.1f} s")
    res["traj_frame_dt"] = frame_dt
    res["traj_substeps"] = s.total_substeps
    res.update({"traj_" + k: v for k, v in particles(s).items()})
    return res


def run_g2p2g(MPMSolver, nsub=3):
    """use_g2p2g=True: three fused substeps through MPMSolver.step (one
    substep per frame), particles and the output grid after each."""
    rng = np.random.default_rng(77)
    st = evolved_state(rng, [(0.35, 0.45, 0.4), (0.6, 0.5, 0.45), (0.45, 0.3, 0.6)], 0.06, 250,
                       [MAT_WATER, MAT_ELASTIC, MAT_SNOW], v_amp=0.5)
    case = dict(res=(24, 24, 24), state=st, kw=dict(use_g2p2g=True),
                postprocess=[dict(kind="surface", point=(0.5, 0.2513, 0.5), normal=(0.0, 1.0, 0.0), surface=2,
                                  friction=0.3)])
    res = dict(res=np.array(case["res"]), n=len(st["x"]), **{"in_" + k: v for k, v in st.items()})
    res["postprocess"] = np.array(repr(case["postprocess"]))
    ti.set_precision("f64")
    s = make_solver(MPMSolver, case)
    dt = float(np.float32(s.default_dt))
    res["dt"] = dt
    for k in range(nsub):
        with contextlib.redirect_stdout(io.StringIO()):
            s.step(dt * 0.999)  # one substep of dt * 0.999
        tree = s.grid_m[s.input_grid].snode.tree
        nodes, v = tree.node_values(s.grid_v[s.input_grid])
        _, m = tree.node_values(s.grid_m[s.input_grid])
        res[f"sub{k}_grid_nodes"] = nodes
        res[f"sub{k}_grid_v"] = v
        res[f"sub{k}_grid_m"] = m
        res.update({f"sub{k}_" + key: val for key, val in particles(s).items()})
    res["substep_dt"] = dt * 0.999
    print(f"  g2p2g_24: {nsub} fused substeps")
    return res


def main():
    MPMSolver = load_reference_solver()
    only = sys.argv[1:]
    for name, fn in CASES.items():
        if only and name not in only:
            continue
        res = run_case(MPMSolver, name, fn)
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **res)
    if not only or "g2p2g_24" in only:
        np.savez_compressed(os.path.join(HERE, "ref_g2p2g_24.npz"), **run_g2p2g(MPMSolver))


if __name__ == "__main__":
    main()
