"""The Blender add-on's particle cache (blender/particles_io.py:40-98,
blender/operators.py:228-247) against golden bytes written and read by the
reference's own functions (tests/golden/make_blender_cache_golden.py)."""
import os

import numpy as np
import pytest

from taichi_elements_gb300 import blender_cache as B

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ('pos', 'vel', 'col', 'mat', 'emt')


def _golden():
    return np.load(os.path.join(HERE, 'golden', 'blender_cache.npz'))


def test_writer_bytes_match_reference(tmp_path):
    g = _golden()
    for k in range(int(g['ncases'])):
        fname = 'particles_{0:0>6}'.format(int(g[f'{k}_frame']))
        fpath = os.path.join(tmp_path, fname)
        par = {B.POS: g[f'{k}_in_pos'], B.VEL: g[f'{k}_in_vel'], B.COL: g[f'{k}_in_col'], B.MAT: g[f'{k}_in_mat'],
               B.EMT: g[f'{k}_in_emt']}
        header = bytes(B.write_pars(par, fpath, fname))
        assert header == g[f'{k}_header'].tobytes()
        for name in NAMES:
            with open(f'{fpath}_{name}.bin', 'rb') as f:
                assert f.read() == g[f'{k}_file_{name}'].tobytes(), name


def test_reader_matches_reference(tmp_path):
    g = _golden()
    for k in range(int(g['ncases'])):
        fname = 'particles_{0:0>6}'.format(int(g[f'{k}_frame']))
        with open(os.path.join(tmp_path, fname + '.bin'), 'wb') as f:
            f.write(g[f'{k}_header'].tobytes())
        for name in NAMES:
            with open(os.path.join(tmp_path, f'{fname}_{name}.bin'), 'wb') as f:
                f.write(g[f'{k}_file_{name}'].tobytes())
        caches = {}
        out = B.read_pars(os.path.join(tmp_path, fname + '.bin'), caches, str(tmp_path))
        assert caches[str(tmp_path)] is out
        for a, name in enumerate(NAMES):
            np.testing.assert_array_equal(out[a], g[f'{k}_read_{name}'])
            assert out[a].dtype == g[f'{k}_read_{name}'].dtype


def test_reader_rejects_other_versions(tmp_path):
    p = os.path.join(tmp_path, 'x.bin')
    with open(p, 'wb') as f:
        f.write(np.array([2, 0], np.uint32).tobytes())
    with pytest.raises(ValueError):
        B.read_pars(p)
