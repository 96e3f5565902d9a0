"""Golden bytes of the Blender add-on's particle cache, made by running the
reference's own ``write_pars`` and ``read_pars`` (taichi-dev/taichi_elements
blender/particles_io.py:40-98) on seeded inputs.

The module imports ``bpy`` at the top and ``read_pars`` resolves file names
with ``bpy.path.abspath``; Blender is not installed here, so a stand-in
module with an identity ``abspath`` satisfies it.  Run in the build
container, where the reference checkout is readable:

    python tests/golden/make_blender_cache_golden.py

It writes tests/golden/blender_cache.npz: per case the input arrays, the
header bytes and the five attribute files' bytes the reference wrote, and
the arrays its reader returned.
"""
import importlib.util
import os
import sys
import tempfile
import types

import numpy as np

REF = "/root/reference"
HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ('pos', 'vel', 'col', 'mat', 'emt')


def load_reference():
    bpy = types.ModuleType("bpy")
    bpy.path = types.SimpleNamespace(abspath=lambda p: p)
    sys.modules["bpy"] = bpy
    spec = importlib.util.spec_from_file_location("ref_particles_io", os.path.join(REF, "blender", "particles_io.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def cases():
    rng = np.random.default_rng(11)
    out = []
    for n, frame in ((300, 7), (1, 123456), (0, 0)):
        out.append(dict(frame=frame,
                        pos=rng.uniform(-1, 2, (n, 3)).astype(np.float32),
                        vel=rng.standard_normal((n, 3)).astype(np.float32),
                        col=rng.integers(0, 2**24, n).astype(np.int32),
                        mat=rng.integers(0, 5, n).astype(np.int32),
                        emt=rng.integers(-1, 4, n).astype(np.int32)))
    return out


def main():
    ref = load_reference()
    store = {}
    with tempfile.TemporaryDirectory() as d:
        for k, c in enumerate(cases()):
            fname = 'particles_{0:0>6}'.format(c['frame'])
            fpath = os.path.join(d, fname)
            par = {ref.POS: c['pos'], ref.VEL: c['vel'], ref.COL: c['col'], ref.MAT: c['mat'], ref.EMT: c['emt']}
            header = bytes(ref.write_pars(par, fpath, fname))
            with open(fpath + '.bin', 'wb') as f:
                f.write(header)
            caches = {}
            ref.read_pars(fpath + '.bin', caches, d)
            store[f'{k}_frame'] = np.array(c['frame'])
            store[f'{k}_header'] = np.frombuffer(header, np.uint8)
            for a, name in enumerate(NAMES):
                store[f'{k}_in_{name}'] = c[name]
                with open(f'{fpath}_{name}.bin', 'rb') as f:
                    store[f'{k}_file_{name}'] = np.frombuffer(f.read(), np.uint8)
                store[f'{k}_read_{name}'] = caches[d][a]
    store['ncases'] = np.array(len(cases()))
    np.savez_compressed(os.path.join(HERE, 'blender_cache.npz'), **store)
    print('wrote', os.path.join(HERE, 'blender_cache.npz'))


if __name__ == '__main__':
    main()
