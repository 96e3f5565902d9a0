"""The kernel profiler behind step(print_stat=True) (engine/mpm_solver.py:809-814
prints Taichi's kernel and memory profiler tables there).

CPU: the decoding of a frame's events into launch groups, for plain and
G2P2G frames, and the table.  GPU: step(print_stat=True) with the profiler on
prints every launch group of the frame with the counts its schedule implies,
the memory table, and leaves the simulation's result unchanged; batched
frames are recorded too.
"""
import contextlib
import io

import numpy as np
import pytest

from taichi_elements_gb300 import profiler


class _Ev:
    """A stand-in for a completed CUDA event: elapsed_time is the difference
    of the recorded timestamps (ms)."""

    def __init__(self, t):
        self.t = t

    def elapsed_time(self, other):
        return other.t - self.t

    def query(self):
        return True

    def synchronize(self):
        pass


def _events(count):
    # event i recorded at time i^2 / 8: every interval distinct
    return [_Ev(i * i / 8.0) for i in range(5 * count + 2)]


@pytest.fixture(autouse=True)
def _clean():
    was = profiler.kernel_profiler
    profiler.clear_kernel_profiler_info()
    yield
    profiler.clear_kernel_profiler_info()
    profiler.kernel_profiler = was


@pytest.mark.parametrize("g2p2g", [False, True])
@pytest.mark.parametrize("count,resort", [(1, 1), (5, 2), (7, 3), (6, 6), (4, 1)])
def test_frame_decoding(count, resort, g2p2g):
    evs = _events(count)
    kt = profiler.frame_kernel_times(count, evs, resort, g2p2g)
    sort_k, bin_k = ("k_fused_sorted", "k_bin_box") if g2p2g else ("k_p2g", "k_g2p_stream")
    sorts = (count + resort - 1) // resort
    assert len(kt[sort_k]) == sorts
    assert len(kt["binning"]) == sorts
    assert len(kt["k_fused"]) == count - sorts
    assert len(kt["grid"]) == count
    # a binning pass before every sort but the first, and the frame's closing one
    assert len(kt[bin_k]) == sorts
    t = lambda i, j: evs[j].t - evs[i].t  # noqa: E731
    for k in range(count):
        b = 5 * k
        if k % resort == 0:
            assert t(b + 2, b + 3) in kt[sort_k]
            assert t(b + 1, b + 2) in kt["binning"]
        else:
            assert t(b + 2, b + 3) in kt["k_fused"]
        assert t(b + 3, b + 4) in kt["grid"]
    assert kt[bin_k][-1] == t(5 * count, 5 * count + 1)


def test_records_table_and_print():
    profiler.enable()
    evs = _events(4)
    profiler.add_frame(4, evs, 2)
    profiler.add_call("mpm_substep", _Ev(1.0), _Ev(3.5))
    profiler.add_call("mpm_substep", _Ev(0.0), _Ev(0.5))
    profiler.collect(sync=False)
    q = profiler.query_kernel_profiler_info("mpm_substep")
    assert q["count"] == 2 and q["total_ms"] == 3.0 and q["min_ms"] == 0.5 and q["max_ms"] == 2.5
    rows = profiler.kernel_profiler_table()
    names = [r[0] for r in rows]
    assert set(names) == {"k_p2g", "k_fused", "k_g2p_stream", "binning", "grid", "mpm_substep"}
    assert [r[2] for r in rows] == sorted((r[2] for r in rows), reverse=True)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        profiler.print_kernel_profiler_info()
    text = buf.getvalue()
    for n in names:
        assert n in text
    assert "100.00%" in text
    profiler.clear_kernel_profiler_info()
    assert profiler.kernel_profiler_table() == []


def test_collect_keeps_unfinished_calls():
    """Without a wait, calls whose last event has not completed (a solver in
    another thread still running) stay queued until they have."""
    profiler.enable()

    class Pending(_Ev):
        done = False

        def query(self):
            return self.done

    late = Pending(2.0)
    profiler.add_call("a", _Ev(0.0), _Ev(1.0))
    profiler.add_call("b", _Ev(0.0), late)
    profiler.collect(sync=False)
    assert len(profiler._pending) == 1 and list(profiler._records) == ["a"]
    profiler.collect(sync=False)
    assert len(profiler._pending) == 1
    late.done = True
    profiler.collect(sync=False)
    assert not profiler._pending
    assert profiler.query_kernel_profiler_info("b")["total_ms"] == 2.0


def test_off_prints_a_hint():
    profiler.enable(False)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        profiler.print_kernel_profiler_info()
    assert "kernel profiler is off" in buf.getvalue()


@pytest.mark.gpu
@pytest.mark.parametrize("use_g2p2g", [False, True])
def test_print_stat_prints_launch_groups(use_g2p2g):
    import torch

    from taichi_elements_gb300 import scenes
    sc = scenes.smoke_scene()
    frame_dt = 7.5 * sc.default_dt

    def run(prof):
        profiler.enable(prof)
        profiler.clear_kernel_profiler_info()
        s = sc.make_solver(use_g2p2g=use_g2p2g)
        s.resort_every = 3
        buf = io.StringIO()
        with contextlib.redirect_stdout(buf):
            s.step(frame_dt, print_stat=True)
            s.step(frame_dt, print_stat=True)
        torch.cuda.synchronize()
        return s, buf.getvalue()

    s0, _ = run(False)
    s1, text = run(True)
    count, _ = s1.count_substeps(frame_dt, s1.default_dt)
    r = s1._frame_resort(count)
    sorts = (count + r - 1) // r
    sort_k, bin_k = ("k_fused_sorted", "k_bin_box") if use_g2p2g else ("k_p2g", "k_g2p_stream")
    rows = {name: cnt for name, cnt, *_ in profiler.kernel_profiler_table()}
    assert rows[sort_k] == 2 * sorts
    assert rows["k_fused"] == 2 * (count - sorts)
    assert rows["grid"] == 2 * count
    assert rows["binning"] == 2 * sorts
    assert rows[bin_k] == 2 * sorts
    for name in rows:
        assert name in text
    assert "held by this solver" in text and "particle state" in text
    for q in profiler.kernel_profiler_table():
        assert q[3] > 0.0  # every launch group took time
    # the same kernels: profiling leaves the result as it was (float
    # atomics make the sums' order, and so the last bits, vary between runs)
    a = s0.particle_info()["position"].astype(np.float64)
    b = s1.particle_info()["position"].astype(np.float64)
    assert np.abs(a - b).max() <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("fuse", [False, True])
def test_batched_frames_are_profiled(fuse):
    import torch

    from test_batched import small_scenes
    from taichi_elements_gb300.batched import BatchedMPM
    profiler.enable()
    profiler.clear_kernel_profiler_info()
    B = BatchedMPM(small_scenes())
    B.fuse_frames, B.resort_every = fuse, 4
    for _ in range(2):  # the second frame would replay a graph without the profiler
        B.substeps(10)
    B.check_status()
    torch.cuda.synchronize()
    rows = {name: cnt for name, cnt, *_ in profiler.kernel_profiler_table()}
    if fuse:
        from taichi_elements_gb300.mpm_solver import frame_resort_interval
        r = frame_resort_interval(10, 4)
        sorts = 2 * ((10 + r - 1) // r)
        assert rows["batch k_p2g"] == sorts and rows["batch k_fused"] == 20 - sorts
        assert rows["batch grid"] == 20 and rows["batch k_g2p_stream"] == sorts
    else:
        assert rows == {"mpm_batch_substep": 20}
