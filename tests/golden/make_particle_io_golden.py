"""Golden vectors of the quantised particle frame format, made by running
the reference's own ``ParticleIO.write_particles`` and ``read_particles_3d``
(taichi-dev/taichi_elements engine/particle_io.py:12-106) on seeded inputs.

The reference module imports ``taichi`` (and, through engine/mesh_io.py,
``plyfile``) at the top but the two functions use only numpy plus the
solver's ``n_particles`` / field accessors / ``copy_ranged``
(engine/mpm_solver.py:1158-1162).  Neither package is installed here, so
empty stand-in modules satisfy the imports and a small fake solver serves
the arrays.  Run in the build container, where the reference checkout is
readable:

    python tests/golden/make_particle_io_golden.py

It writes tests/golden/particle_io.npz (inputs and the reference's outputs
per case).  Arithmetic follows the installed numpy's promotion rules
(numpy >= 2: python scalars are weak, so the whole expression stays in
float32).
"""
import importlib.util
import os
import sys
import tempfile
import types

import numpy as np

REF = "/root/reference"
HERE = os.path.dirname(os.path.abspath(__file__))


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def load_reference_particle_io():
    """engine/particle_io.py and engine/mesh_io.py loaded from their files
    (the package's __init__ would import the Taichi solver)."""
    sys.modules.setdefault("taichi", types.ModuleType("taichi"))
    ply = types.ModuleType("plyfile")
    ply.PlyData = None
    sys.modules.setdefault("plyfile", ply)
    pkg = types.ModuleType("engine")
    pkg.__path__ = []
    sys.modules["engine"] = pkg
    _load("engine.mesh_io", os.path.join(REF, "engine", "mesh_io.py"))
    return _load("engine.particle_io", os.path.join(REF, "engine", "particle_io.py")).ParticleIO


class _Scalar:
    def __init__(self, a):
        self.a = a


class _Vector:
    def __init__(self, a):
        self.a = a

    def get_scalar_field(self, d):
        return _Scalar(self.a[:, d])


class FakeSolver:
    """The attributes ParticleIO.write_particles reads from an MPMSolver."""
    dim = 3

    def __init__(self, x, v, color):
        self.n_particles = {None: len(x)}
        self.x = _Vector(x)
        self.v = _Vector(v)
        self.color = _Scalar(color)

    def copy_ranged(self, np_x, field, begin, end):
        np_x[:end - begin] = field.a[begin:end]


def cases():
    rng = np.random.default_rng(11)
    out = {}
    n = 3000
    out["random"] = (rng.uniform(0.1, 0.9, (n, 3)).astype(np.float32),
                     rng.normal(0.0, 2.0, (n, 3)).astype(np.float32),
                     rng.integers(0, 1 << 24, n).astype(np.int32), 1000)
    n = 500
    x = rng.uniform(0.2, 0.3, (n, 3)).astype(np.float32)
    x[:, 0] = np.float32(0.25)  # a zero-width range
    x[:7, 2] = np.float32(0.3) + np.float32(3e-6) * np.arange(7, dtype=np.float32)  # a range narrower than 1e-5
    x[7:, 2] = np.float32(0.3)
    out["narrow"] = (x, np.zeros((n, 3), np.float32), np.full(n, 0xFFFFFF, np.int32), 1 << 20)
    n = 2048
    x = rng.uniform(-3.0, 5.0, (n, 3)).astype(np.float32)
    v = rng.uniform(-40.0, 40.0, (n, 3)).astype(np.float32)
    # exact extremes and values one float32 step inside them
    x[0], x[1] = -3.0, 5.0
    x[2] = np.nextafter(np.float32(5.0), np.float32(0.0))
    v[0], v[1] = -40.0, 40.0
    out["wide"] = (x, v, rng.integers(0, 1 << 24, n).astype(np.int32), 777)
    return out


def main():
    P = load_reference_particle_io()
    store = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, (x, v, color, slice_size) in cases().items():
            fn = os.path.join(tmp, name + ".npz")
            P.write_particles(FakeSolver(x, v, color), fn, slice_size=slice_size)
            with np.load(fn) as d:
                ranges, x_and_v, rgb = d["ranges"], d["x_and_v"], d["color"]
            xd, vd, _ = P.read_particles_3d(fn)
            store.update({f"{name}_x": x, f"{name}_v": v, f"{name}_color": color,
                          f"{name}_slice": np.int64(slice_size), f"{name}_ranges": ranges,
                          f"{name}_x_and_v": x_and_v, f"{name}_rgb": rgb, f"{name}_xdec": xd,
                          f"{name}_vdec": vd})
    np.savez_compressed(os.path.join(HERE, "particle_io.npz"), **store)
    print("wrote", os.path.join(HERE, "particle_io.npz"), sorted(cases()))


if __name__ == "__main__":
    main()
