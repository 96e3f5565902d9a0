"""Measured choice of the substep schedule.

Two schedules run the reference's plain substep loop with the same
arithmetic:

* per-substep launches (mpm_substep): every substep sorts the particles by
  grid block, and G2P stages each block's 6^3 velocity halo in shared memory.
  The engine splits each active 4^3 grid block's particles into work items of
  `chunk` particles; large items amortise the halo staging, small items give
  a small scene enough CTAs to fill 152 SMs.
* fused frames (mpm_frame): the particles are re-sorted about every
  `resort` substeps (evenly over the frame); in between, the G2P of one
  substep (velocity gathers through L1, no halo staging) and the P2G of the
  next run as one kernel.  Frequent sorts keep the scatter tiles dense; rare
  sorts save the sort's data movement.

``tune_chunk`` times the chunk candidates; ``tune_schedule`` times fused
frames for each re-sort candidate, with the fused kernels' stencil loops
unrolled (12 warps per SM) and rolled (16 warps per SM, MpmParams.occupancy),
against the per-substep schedule at its best chunk and applies the fastest.  Both run on a scratch copy of the
solver's particles (the simulation itself is not advanced).  Results are
cached in memory per (device, particle-count bucket, grid resolution,
per-particle E, material mix), and in the JSON file named by the
MPM_GB300_TUNE_CACHE environment variable when it is set.
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
RESORT_CANDIDATES = (8, 12, 16, 24, 48)
_cache: dict = {}
_lock = threading.Lock()


def material_mix(solver) -> str:
    """The materials present, as a string of material ids ("013")."""
    n = solver.n_particles
    if n == 0 or solver.quant:
        return "-"
    m = solver._state[solver._cur][_lib.ROW_MAT, :n].view(torch.int32) & 0xFF
    present = torch.bincount(m.long(), minlength=8)[:8].cpu().numpy()
    return "".join(str(k) for k in range(8) if present[k] > 0)


def _key(solver, what="chunk") -> str:
    dev = torch.cuda.get_device_name(solver.device)
    bucket = int(math.log2(max(solver.n_particles, 1)))
    key = f"{dev}|{bucket}|{'x'.join(map(str, solver.res))}|{int(solver.per_particle_E)}"
    key += f"|{'g2p2g' if solver.use_g2p2g else 'plain'}{'|q' if solver.quant else ''}"
    return key if what == "chunk" else f"{what}|{key}|{material_mix(solver)}"


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
        calls = 0

        def run(k):
            nonlocal cur, calls
            for _ in range(k):
                a, b = bufs[cur].data_ptr(), bufs[1 - cur].data_ptr()
                if solver.use_g2p2g:  # the first call finalizes the counts and gathers nothing
                    _lib.check(lib.mpm_g2p2g_substep(pp, ws.data_ptr(), cap, n, a, b, dt, n if calls else 0,
                                                     0 if calls else 1, None, stream.cuda_stream),
                               "mpm_g2p2g_substep")
                else:
                    _lib.check(lib.mpm_substep(pp, ws.data_ptr(), cap, n, a, b, dt, None, stream.cuda_stream),
                               "mpm_substep")
                cur = 1 - cur
                calls += 1

        run(2)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run(substeps)
        e1.record(stream)
        e1.synchronize()
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


def time_frames(solver, candidates=RESORT_CANDIDATES, substeps=48, dt=None, occupancy=0):
    """Milliseconds per substep of a fused frame of `substeps` substeps for
    each target re-sort interval (spread over the frame as step() spreads
    it), with the kernels' register budget `occupancy` (MpmParams.occupancy),
    measured on a copy."""
    from .mpm_solver import frame_resort_interval
    solver._prepare(dt or solver.default_dt)
    dt = float(dt or solver.default_dt)
    lib = solver._lib
    n, cap = solver.n_particles, solver._cap
    bufs = [torch.empty_like(solver._state[0]), torch.empty_like(solver._state[0])]
    ws = torch.empty_like(solver._ws)
    maxv = torch.zeros(substeps, dtype=torch.float32, device=solver.device)
    stream = torch.cuda.current_stream(solver.device)
    p = _lib.MpmParams.from_buffer_copy(solver.params)
    p.occupancy = int(occupancy)
    pp = ctypes.byref(p)
    out = {}
    for r in candidates:
        bufs[0].copy_(solver._state[solver._cur])
        _lib.check(lib.mpm_workspace_init(pp, ws.data_ptr(), cap, stream.cuda_stream), "mpm_workspace_init")
        _lib.check(lib.mpm_bin_count(pp, ws.data_ptr(), cap, bufs[0].data_ptr(), 0, n, stream.cuda_stream),
                   "mpm_bin_count")
        cur = 0
        frames = 0

        eff = frame_resort_interval(substeps, r)

        def frame():
            nonlocal cur, frames
            in_b = ctypes.c_int32(0)
            a, b = bufs[cur].data_ptr(), bufs[1 - cur].data_ptr()
            if solver.use_g2p2g:  # the first frame's first substep gathers nothing
                _lib.check(lib.mpm_g2p2g_frame(pp, ws.data_ptr(), cap, n, a, b, dt, substeps, eff,
                                               n if frames else 0, maxv.data_ptr(), ctypes.byref(in_b), None,
                                               stream.cuda_stream), "mpm_g2p2g_frame")
            else:
                _lib.check(lib.mpm_frame(pp, ws.data_ptr(), cap, n, a, b, dt, substeps, eff, maxv.data_ptr(),
                                         ctypes.byref(in_b), None, stream.cuda_stream), "mpm_frame")
            cur = (cur + in_b.value) % 2
            frames += 1

        frame()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        frame()
        e1.record(stream)
        e1.synchronize()
        out[int(r)] = e0.elapsed_time(e1) / substeps
    return out


def tune_schedule(solver, resort_candidates=RESORT_CANDIDATES, chunk_candidates=CANDIDATES, substeps=48) -> dict:
    """Measure fused frames for each re-sort interval and per-substep
    launches for each chunk, apply the fastest (solver.fuse_frames,
    solver.resort_every, solver.chunk) and return the choice with the
    measured milliseconds per substep."""
    with _lock:
        if not _cache:
            _load_file()
        key = _key(solver, "schedule")
        best = _cache.get(key)
    if best is None:
        chunks = time_chunks(solver, chunk_candidates, substeps=8)
        chunk = min(chunks, key=chunks.get)
        frames = {} if solver.quant else time_frames(solver, resort_candidates, substeps)
        rolled = {} if solver.quant else time_frames(solver, resort_candidates, substeps, occupancy=1)
        best = {"chunk": int(chunk), "substep_ms": {str(c): t for c, t in chunks.items()},
                "frame_ms": {str(r): t for r, t in frames.items()},
                "frame_ms_rolled": {str(r): t for r, t in rolled.items()}}
        options = [(t, r, 0) for r, t in frames.items()] + [(t, r, 1) for r, t in rolled.items()]
        if options and min(options)[0] < chunks[chunk]:
            _, r, occ = min(options)
            best.update(mode="frame", resort=int(r), occupancy=int(occ))
        else:
            best.update(mode="substep", resort=int(solver.resort_every), occupancy=0)
        with _lock:
            _cache[key] = best
            _save_file()
    solver.fuse_frames = best["mode"] == "frame"
    solver.resort_every = int(best["resort"])
    solver.occupancy = int(best.get("occupancy", 0))
    if solver.chunk != best["chunk"]:
        solver.chunk = int(best["chunk"])
        solver._invalidate_params()
    return dict(best, key=key)
