"""Kernel and memory profiler of the solvers.

The reference prints Taichi's profiler tables from `step(print_stat=True)`
(engine/mpm_solver.py:809-814: `ti.profiler.print_kernel_profiler_info()` and
`ti.profiler.print_memory_profiler_info()`), with the kernel profiler switched
on by `ti.init(kernel_profiler=True)`.  Here the switch is
`profiler.kernel_profiler = True` (or `enable()`).  While it is on, the solvers
launch their frames without CUDA graphs and record CUDA events on the
launching stream around every launch group of a frame (the events that
`mpm_frame`, `mpm_g2p2g_frame` and `mpm_batch_frame` take) and around each
per-substep call.  The durations accumulate per launch group until
`clear_kernel_profiler_info()`; they are read after the frame's own
synchronisation, so profiling adds no host round trip to a frame.
"""
from __future__ import annotations

import ctypes
import threading

import torch

kernel_profiler = False

# launch group -> durations (ms)
_records: dict[str, list[float]] = {}
# (decode, name prefix, last event) of the calls whose events have not been read yet
_pending: list = []
# solvers in several host threads share the records
_lock = threading.Lock()


def enable(on: bool = True) -> None:
    global kernel_profiler
    kernel_profiler = bool(on)


def clear_kernel_profiler_info() -> None:
    with _lock:
        _records.clear()
        _pending.clear()


def frame_events(count: int, device=None):
    """Timing events for one frame of `count` substeps and the ctypes array
    of their handles, in the order the frame records them: events[5k + j]
    for substep k (its start; after the binning of the state, i.e. the
    previous plain run's closing G2P or the G2P2G mode's binning pass; after
    the sort's finalize; after the particle kernel; after the grid update),
    events[5 count] and [5 count + 1] around the frame's closing pass.
    The events belong to `device` (the current one by default) and are
    created on its current stream, the one the frame launches on."""
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(5 * count + 2)]
    with torch.cuda.device(device):
        stream = torch.cuda.current_stream()
        for e in evs:
            e.record(stream)  # creates the event before its handle is taken
    return evs, (ctypes.c_void_p * len(evs))(*[e.cuda_event for e in evs])


def frame_kernel_times(count: int, evs, resort: int, g2p2g: bool = False) -> dict:
    """Per launch group durations (ms) of one frame from its completed
    events.  Plain frames: the sort's P2G (k_p2g), the fused substeps
    (k_fused), the closing G2P that also bins (k_g2p_stream); G2P2G frames:
    the sorting pass (k_fused_sorted), the in-place substeps (k_fused) and
    the binning passes (k_bin_box).  "binning" is the sorts' finalize (seven
    small kernels), "grid" the grid update with the block-flag passes."""
    sort_k, bin_k = ("k_fused_sorted", "k_bin_box") if g2p2g else ("k_p2g", "k_g2p_stream")
    out = {sort_k: [], "k_fused": [], bin_k: [], "binning": [], "grid": []}

    def t(i, j):
        return evs[i].elapsed_time(evs[j])

    for k in range(count):
        b = 5 * k
        if k % resort == 0:
            if k > 0:
                out[bin_k].append(t(b, b + 1))
            out["binning"].append(t(b + 1, b + 2))
            out[sort_k].append(t(b + 2, b + 3))
        else:
            out["k_fused"].append(t(b + 2, b + 3))
        out["grid"].append(t(b + 3, b + 4))
    out[bin_k].append(t(5 * count, 5 * count + 1))
    return out


def add_frame(count: int, evs, resort: int, g2p2g: bool = False, prefix: str = "") -> None:
    """Queue a frame's events for the records."""
    with _lock:
        _pending.append((lambda: frame_kernel_times(count, evs, resort, g2p2g), prefix, evs[-1]))


def substep_events():
    """A (start, end) event pair for one per-substep call."""
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def add_call(name: str, e0, e1) -> None:
    """Queue one timed call (both events recorded)."""
    with _lock:
        _pending.append((lambda: {name: [e0.elapsed_time(e1)]}, "", e1))


def collect(sync: bool = True) -> None:
    """Move the queued event durations into the records: every queued call,
    waiting for its last event (sync), or only the calls whose last event has
    completed (a solver's own frame after its readback; calls of solvers in
    other threads may still be running and stay queued)."""
    with _lock:
        pending = list(_pending)
        _pending.clear()
    done, keep = [], []
    for item in pending:
        if sync:
            item[2].synchronize()
        elif not item[2].query():
            keep.append(item)
            continue
        done.append(item)
    results = [(prefix, decode()) for decode, prefix, _ in done]
    with _lock:
        _pending.extend(keep)
        for prefix, r in results:
            for name, ms in r.items():
                if ms:
                    _records.setdefault(prefix + name, []).extend(ms)


def query_kernel_profiler_info(name: str) -> dict:
    """count, total, min, avg and max (ms) of one launch group."""
    collect()
    with _lock:
        ms = list(_records.get(name, []))
    if not ms:
        return {"count": 0, "total_ms": 0.0, "min_ms": 0.0, "avg_ms": 0.0, "max_ms": 0.0}
    return {"count": len(ms), "total_ms": sum(ms), "min_ms": min(ms), "avg_ms": sum(ms) / len(ms),
            "max_ms": max(ms)}


def kernel_profiler_table() -> list:
    """(name, count, total ms, min, avg, max) per launch group, largest total first."""
    collect()
    rows = []
    with _lock:
        items = [(name, list(ms)) for name, ms in _records.items()]
    for name, ms in items:
        rows.append((name, len(ms), sum(ms), min(ms), sum(ms) / len(ms), max(ms)))
    rows.sort(key=lambda r: -r[2])
    return rows


def print_kernel_profiler_info() -> None:
    if not kernel_profiler:
        print("kernel profiler is off: set taichi_elements_gb300.profiler.kernel_profiler = True")
        return
    rows = kernel_profiler_table()
    total = sum(r[2] for r in rows)
    dev = torch.cuda.get_device_name() if torch.cuda.is_available() else "no device"
    rule = "=" * 78
    print(rule)
    print(f"kernel profiler (CUDA events per launch group) on {dev}")
    print(rule)
    print(f"[ {'%':>6}  {'total':>9}  {'count':>7} | {'min':>8} {'avg':>8} {'max':>8} ms] launch group")
    print("-" * 78)
    for name, cnt, tot, lo, avg, hi in rows:
        pct = 100.0 * tot / total if total > 0 else 0.0
        print(f"[{pct:6.2f}%  {tot / 1e3:8.3f}s  {cnt:6d}x | {lo:8.3f} {avg:8.3f} {hi:8.3f}   ] {name}")
    print("-" * 78)
    print(f"[100.00%] total {total / 1e3:.3f} s over {len(rows)} launch groups")
    print(rule)


def print_memory_profiler_info(solver=None) -> None:
    rule = "=" * 78
    print(rule)
    print("device memory")
    print(rule)
    if solver is not None:
        rows = solver.memory_report()
        for name, nbytes in rows:
            print(f"  {nbytes / 2**20:12.2f} MiB  {name}")
        print(f"  {sum(b for _, b in rows) / 2**20:12.2f} MiB  held by this solver")
    if torch.cuda.is_available():
        print(f"  {torch.cuda.memory_allocated() / 2**20:12.2f} MiB  allocated by the process "
              f"({torch.cuda.memory_reserved() / 2**20:.2f} MiB reserved)")
    print(rule)
