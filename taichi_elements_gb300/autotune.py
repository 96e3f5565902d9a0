"""Measured choice of the P2G/G2P work-item size (particles per CTA item).

The engine splits each active 4^3 grid block's particles into work items of
`chunk` particles; one CTA processes one item with its shared-memory tiles.
Large items amortise the tile flush, small items give a small scene enough
CTAs to fill 152 SMs.  ``tune_chunk`` times a few substeps for each candidate
on a scratch copy of the solver's particles (the simulation itself is not
advanced) and keeps the fastest.  Results are cached in memory per
(device, particle-count bucket, grid resolution, per-particle E), and in the
JSON file named by the MPM_GB300_TUNE_CACHE environment variable when it is
set.
"""
from __future__ import annotations

import ctypes
import json
import math
import os
import threading

import torch

from . import _lib

CANDIDATES = (128, 256, 512, 1024)
_cache: dict = {}
_lock = threading.Lock()


def _key(solver) -> str:
    dev = torch.cuda.get_device_name(solver.device)
    bucket = int(math.log2(max(solver.n_particles, 1)))
    return f"{dev}|{bucket}|{'x'.join(map(str, solver.res))}|{int(solver.per_particle_E)}"


def _load_file():
    path = os.environ.get("MPM_GB300_TUNE_CACHE")
    if path and os.path.exists(path):
        try:
            with open(path) as f:
                _cache.update(json.load(f))
        except (OSError, ValueError):
            pass


def _save_file():
    path = os.environ.get("MPM_GB300_TUNE_CACHE")
    if path:
        try:
            with open(path, "w") as f:
                json.dump(_cache, f, indent=1)
        except OSError:
            pass


def time_chunks(solver, candidates=CANDIDATES, substeps=8, dt=None):
    """Milliseconds per substep for each candidate chunk, measured on a copy."""
    solver._prepare(dt or solver.default_dt)
    dt = float(dt or solver.default_dt)
    lib = solver._lib
    n, cap = solver.n_particles, solver._cap
    bufs = [solver._state[solver._cur].clone(), torch.empty_like(solver._state[0])]
    ws = torch.empty_like(solver._ws)
    stream = torch.cuda.current_stream(solver.device)
    out = {}
    for c in candidates:
        p = _lib.MpmParams.from_buffer_copy(solver.params)
        p.chunk = int(c)
        pp = ctypes.byref(p)
        bufs[0].copy_(solver._state[solver._cur])
        _lib.check(lib.mpm_workspace_init(pp, ws.data_ptr(), cap, stream.cuda_stream), "mpm_workspace_init")
        _lib.check(lib.mpm_bin_count(pp, ws.data_ptr(), cap, bufs[0].data_ptr(), 0, n, stream.cuda_stream),
                   "mpm_bin_count")
        cur = 0

        def run(k):
            nonlocal cur
            for _ in range(k):
                _lib.check(lib.mpm_substep(pp, ws.data_ptr(), cap, n, bufs[cur].data_ptr(), bufs[1 - cur].data_ptr(),
                                           dt, None, stream.cuda_stream), "mpm_substep")
                cur = 1 - cur

        run(2)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run(substeps)
        e1.record(stream)
        torch.cuda.synchronize()
        out[int(c)] = e0.elapsed_time(e1) / substeps
    return out


def tune_chunk(solver, candidates=CANDIDATES, substeps=8) -> int:
    """Set solver.chunk to the fastest candidate (cached per shape)."""
    with _lock:
        if not _cache:
            _load_file()
        key = _key(solver)
        best = _cache.get(key)
    if best is None:
        times = time_chunks(solver, candidates, substeps)
        best = min(times, key=times.get)
        with _lock:
            _cache[key] = best
            _save_file()
    if solver.chunk != best:
        solver.chunk = int(best)
        solver._invalidate_params()
    return int(best)
