"""The allocation-free substep (mpm_substep_noalloc) against the regular one.

Callers that cannot allocate device memory when they step the simulation
(for instance code that runs inside another library's stream capture or
memory pool) use mpm_substep_noalloc, whose scratch is a static array inside
the library.  This test drives both entry points through the C ABI on copies
of the same particle state, two substeps in a row, and checks that they agree
within the tolerance of the float32 atomic-summation order: positions and F
to 1e-6 absolute (domain and F are of unit scale), velocities to 1e-5 of the
largest speed.  It also checks the size limits are rejected without device
work.  It runs alone in a fresh process or after the other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

from taichi_elements_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu

E_CAPACITY = -4


def _gather(solver, buf, row0, ncols):
    n = solver.n_particles
    out = torch.empty((n, ncols), dtype=torch.float32, device=solver.device)
    _lib.check(solver._lib.mpm_gather_rows(buf.data_ptr(), solver._cap, n, row0, ncols, out.data_ptr(),
                                           torch.cuda.current_stream().cuda_stream), "mpm_gather_rows")
    return out.cpu().numpy()


def _solver(per_particle_E):
    sc = scenes.smoke_scene()
    if not per_particle_E:
        return sc, sc.make_solver()
    # per-particle Young's modulus, spread over a factor of e around the
    # solver's E, so the has_Ep branch of P2G is the one that runs
    s = sc.make_solver(per_particle_E=True)
    rng = np.random.default_rng(11)
    E = (s.E * np.exp(rng.uniform(-0.5, 0.5, s.n_particles))).astype(np.float32)
    st = s._state[s._cur]
    ids = st[_lib.ROW_ID, :s.n_particles].view(torch.int32).long()
    st[_lib.ROW_EP, :s.n_particles] = torch.as_tensor(E, device=s.device)[ids]
    return sc, s


@pytest.mark.parametrize("per_particle_E", [False, True])
def test_noalloc_substep_matches_regular_substep(per_particle_E):
    sc, s = _solver(per_particle_E)
    dt = sc.default_dt
    s._prepare(dt)  # regular path: workspace allocated, particles binned
    lib = s._lib
    p = s.params
    stream = torch.cuda.current_stream().cuda_stream
    n, cap = s.n_particles, s._cap
    # regular path ping-pongs between the solver's two buffers; the
    # allocation-free path gets its own copies of the same initial state
    a_cur, a_nxt = s._state[s._cur], s._state[1 - s._cur]
    b_cur, b_nxt = a_cur.clone(), torch.zeros_like(a_cur)
    for _ in range(2):
        _lib.check(lib.mpm_substep(ctypes.byref(p), s._ws.data_ptr(), cap, n, a_cur.data_ptr(), a_nxt.data_ptr(),
                                   dt, None, stream), "mpm_substep")
        _lib.check(lib.mpm_substep_noalloc(ctypes.byref(p), cap, n, b_cur.data_ptr(), b_nxt.data_ptr(), dt, None,
                                           stream), "mpm_substep_noalloc")
        torch.cuda.synchronize()
        xa, xb = _gather(s, a_nxt, _lib.ROW_X, 3), _gather(s, b_nxt, _lib.ROW_X, 3)
        va, vb = _gather(s, a_nxt, _lib.ROW_V, 3), _gather(s, b_nxt, _lib.ROW_V, 3)
        Fa, Fb = _gather(s, a_nxt, _lib.ROW_F, 9), _gather(s, b_nxt, _lib.ROW_F, 9)
        ja, jb = _gather(s, a_nxt, _lib.ROW_JP, 1), _gather(s, b_nxt, _lib.ROW_JP, 1)
        assert np.all(np.isfinite(xb))
        assert np.abs(xa - xb).max() <= 1e-6
        assert np.abs(va - vb).max() <= 1e-5 * max(1.0, np.abs(va).max())
        assert np.abs(Fa - Fb).max() <= 1e-6
        assert np.abs(ja - jb).max() <= 1e-6
        a_cur, a_nxt = a_nxt, a_cur
        b_cur, b_nxt = b_nxt, b_cur


def test_noalloc_rejects_sizes_beyond_its_scratch():
    sc = scenes.smoke_scene()
    s = sc.make_solver()
    p = s.params
    dummy = torch.zeros((_lib.NROWS, 70000), dtype=torch.float32, device=s.device)
    stream = torch.cuda.current_stream().cuda_stream
    rc = s._lib.mpm_substep_noalloc(ctypes.byref(p), 70000, 70000, dummy.data_ptr(), dummy.data_ptr(), 1e-4, None,
                                    stream)
    assert rc == E_CAPACITY
    # a 256^3 grid window needs far more than the static scratch
    big = _lib.MpmParams.from_buffer_copy(p)
    for d in range(3):
        big.win_nb[d] = 68
    rc = s._lib.mpm_substep_noalloc(ctypes.byref(big), 70000, 100, dummy.data_ptr(), dummy.data_ptr(), 1e-4, None,
                                    stream)
    assert rc == E_CAPACITY
