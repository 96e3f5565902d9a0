#!/usr/bin/env python
"""Benchmark of the GB300 MLS-MPM engine: particle-substeps/s.

A "step" is one MLS-MPM substep (P2G, grid update, G2P, and the binning of
the substeps that re-sort) over the whole particle set of the workload.
Default workload: the large sparse scene, 16M particles in 64 ellipsoids on
a 256^3 grid (elastic/snow, ground collider), seeded synthetic inputs.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload ellipsoids_256|four_materials_128|water_cube_64|batched_64|elastic_on_water]

Prints one JSON line.  `value` times K substeps with state resident in HBM,
run as frames through mpm_frame (the kernels MPMSolver.step runs: fused
G2P+P2G substeps, re-sorted every `resort_every`), with the schedule the
autotuner measured (CUDA events on the launching stream, barrier +
synchronize on both sides, max over ranks; events around every launch group
give the per-kernel times).  `e2e` runs the drop-in API end to end:
read_restart from pinned host arrays, step(frame_dt) frames and
particle_info() readback, after two untimed runs of the same sequence; it
reports the median of three timed runs.
`--impl reference` times the CPU restatement of the reference's substep
(C/OpenMP float32 oracle, all host threads) on a bounded sample.
Under torchrun each rank runs an independent replica (replicas only: the
single-scene substep has no data-parallel split without a halo exchange).
"""
from __future__ import annotations

import argparse
import ctypes
import gc
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ALGO_BYTES_PER_PARTICLE = 204  # read x,v,C,F,Jp,mat once (104) + write x,v,C,F,Jp (100)
ALGO_BYTES_PER_NODE = 64  # P2G flush 16 + grid read 16 + grid write 16 + G2P read 16
P2G_BYTES_PER_PARTICLE = 144  # read 104 + write F, Jp 40
P2G_BYTES_PER_NODE = 16
G2P_BYTES_PER_PARTICLE = 60  # write x, v, C
G2P_BYTES_PER_NODE = 16
GRID_BYTES_PER_NODE = 32
# packed storage (quant=True): x 8, v 8, F with the material 20, C 36, Jp 4
Q_ALGO_BYTES_PER_PARTICLE = 152  # read 76 + write x, v, C, F, Jp 76
Q_P2G_BYTES_PER_PARTICLE = 100  # read 76 + write F, Jp 24
KERNELS_PER_SUBSTEP = 10  # 7 binning kernels + p2g + grid + g2p
FINALIZE_LAUNCHES = 7  # mpm_bin_finalize
# k_fused does the particle side of one whole substep (the G2P of one substep
# and the P2G of the next): the per-substep particle figure above, and per
# node the G2P read and the P2G flush
FUSED_BYTES_PER_PARTICLE = ALGO_BYTES_PER_PARTICLE
FUSED_BYTES_PER_NODE = 32


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_scene(name):
    from taichi_elements_gb300 import scenes
    return {
        "ellipsoids_256": scenes.ellipsoids_256,
        "four_materials_128": scenes.four_materials_128,
        "water_cube_64": scenes.water_cube_64,
    }[name]()


def describe(sc):
    return {
        "ellipsoids_256": "3-D large sparse: 16M particles in 64 ellipsoids (semi-axes U[0.02, 0.08], centres in "
                          "the upper half), 256^3 grid, elastic/snow 50/50, ground collider, f32; the ellipsoids "
                          "of that distribution occupy ~8.5% of the 8^3 blocks (active_8cubed_block_fraction), "
                          "not the ~15% the configuration is quoted with",
        "four_materials_128": "3-D multi-material: 4 cubes x 500K (water/elastic/snow/sand), 128^3 grid, f32",
        "water_cube_64": "plain 3-D: water cube 134,218 particles, 64^3 grid, f32",
    }[sc.name]


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.out = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is None:
            return
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            self.out = ""

    def summary(self):
        if not self.out:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init():
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, ws):
    """Maximum of a per-rank float over all ranks (the slowest replica's
    time); a CPU tensor when the process group runs on gloo."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank, steps, ws, total_ms):
    """Whole-job throughput of N independent replicas: the units all ranks
    processed divided by the slowest rank's time (max over ranks)."""
    return units_per_rank * steps * ws / (total_ms / 1e3)


def kernel_traffic(kernel, n_particles):
    """DRAM bytes per launch of `kernel`: the per-particle figure of the
    committed ncu capture (profiles/dram_four_materials_128.txt) times the
    particle count, or None when the summary has no figure for it."""
    path = os.path.join(ROOT, "profiles", "dram_four_materials_128.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) == 2 and parts[0] == f"{kernel}_dram_bytes_per_particle":
                return float(parts[1]) * n_particles
    return None


def block8_fraction(solver):
    """Fraction of the domain's 8^3-cell blocks that hold particles (the
    sparsity the large-scene configuration is quoted with)."""
    import torch
    x = solver.full_state()["x"]
    cells = torch.floor(x * solver.inv_dx).to(torch.int64)
    b = torch.div(cells, 8, rounding_mode="floor")
    nb = [max(1, r // 8) for r in solver.res]
    key = (b[:, 0] * nb[1] + b[:, 1]) * nb[2] + b[:, 2]
    return int(torch.unique(key).numel()) / float(nb[0] * nb[1] * nb[2])


def count_nodes(solver):
    """Distinct grid nodes touched by particle stencils (mass > 0)."""
    import torch
    v = solver.views()
    ng = int(v["counters"][1].item())
    gb = v["gblocks"][:ng].long()
    addr = (gb[:, None] * 64 + torch.arange(64, device=gb.device)[None]).reshape(-1)
    return int((v["grid_vel"][addr, 3] > 0).sum().item())


def frame_plan(steps, frame):
    """Substep counts of the frames that run `steps` substeps."""
    out = []
    while steps > 0:
        out.append(min(frame, steps))
        steps -= out[-1]
    return out


def frame_launches(count, resort):
    """Kernel launches of one mpm_frame call: per sort the finalize, P2G and
    grid update (and the closing G2P of the previous run), per fused substep
    the fused kernel, two flag passes and the grid update, and the frame's
    closing G2P."""
    sorts = (count + resort - 1) // resort
    return sorts * (FINALIZE_LAUNCHES + 2) + (sorts - 1) + (count - sorts) * 4 + 1


def time_frames(solver, dt, plan, stream):
    """Runs the frames of `plan` through mpm_frame (the kernels of step()),
    recording CUDA events around every launch group on the launching stream.
    Returns the events per frame (synchronised)."""
    import torch

    from taichi_elements_gb300 import _lib, profiler
    with torch.cuda.stream(stream):
        made = [profiler.frame_events(c) for c in plan]
    evs, arrays = [m[0] for m in made], [m[1] for m in made]
    torch.cuda.synchronize()
    if max(plan) > solver._maxv.numel():
        solver._maxv = torch.zeros(max(plan), dtype=torch.float32, device=solver.device)
    p = solver.params

    def run():
        for c, arr in zip(plan, arrays):
            in_b = ctypes.c_int32(0)
            a = solver._state[solver._cur].data_ptr()
            b = solver._state[1 - solver._cur].data_ptr()
            if solver.use_g2p2g:  # every particle took part in the previous substep
                _lib.check(solver._lib.mpm_g2p2g_frame(ctypes.byref(p), solver._ws.data_ptr(), solver._cap,
                                                       solver.n_particles, a, b, float(dt), int(c),
                                                       solver._frame_resort(c), solver.n_particles,
                                                       solver._maxv.data_ptr(), ctypes.byref(in_b), arr,
                                                       stream.cuda_stream), "mpm_g2p2g_frame")
            else:
                _lib.check(solver._lib.mpm_frame(ctypes.byref(p), solver._ws.data_ptr(), solver._cap,
                                                 solver.n_particles, a, b, float(dt), int(c),
                                                 solver._frame_resort(c), solver._maxv.data_ptr(),
                                                 ctypes.byref(in_b), arr, stream.cuda_stream), "mpm_frame")
            solver._cur = (solver._cur + in_b.value) % 2
    return evs, run


def frame_kernel_times(plan, evs, resorts, g2p2g=False):
    """Per launch group durations (ms) over the frames of time_frames (the
    decoding of taichi_elements_gb300.profiler.frame_kernel_times, frame by
    frame).  `resorts`: each frame's re-sort interval."""
    from taichi_elements_gb300.profiler import frame_kernel_times as one_frame
    out = {}
    for c, ev, resort in zip(plan, evs, resorts):
        for k, v in one_frame(c, ev, resort, g2p2g).items():
            out.setdefault(k, []).extend(v)
    return out


def run_gb300(args):
    import torch

    from taichi_elements_gb300 import _lib

    ws, rank, local = dist_init()
    sc = make_scene(args.workload)
    skw = dict(quant=True) if args.quant else {}
    solver = sc.make_solver(chunk=args.chunk, **skw) if args.chunk else sc.make_solver(**skw)
    solver.use_cuda_graph = False  # events between launches; the graph replays the same kernels
    dt = sc.default_dt
    tuned = None
    if args.chunk is None and args.resort is None and args.schedule is None and args.occupancy is None:
        from taichi_elements_gb300.autotune import tune_schedule
        tuned = tune_schedule(solver)
    if args.resort is not None:
        solver.resort_every = args.resort
    if args.schedule is not None:
        solver.fuse_frames = args.schedule == "frame"
    if args.occupancy is not None:
        solver.occupancy = args.occupancy
    fused = solver._fuses_frames
    lib = solver._lib
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    def substep_phases(ev=None):
        p = solver.params
        pp = ctypes.byref(p)
        wsp, cap, n = solver._ws.data_ptr(), solver._cap, solver.n_particles
        cur = solver._state[solver._cur].data_ptr()
        nxt = solver._state[1 - solver._cur].data_ptr()
        if ev is not None:
            ev[0].record(stream)
        _lib.check(lib.mpm_bin_finalize(pp, wsp, cap, n, sptr), "bin")
        if ev is not None:
            ev[1].record(stream)
        _lib.check(lib.mpm_p2g(pp, wsp, cap, n, cur, nxt, dt, sptr), "p2g")
        if ev is not None:
            ev[2].record(stream)
        _lib.check(lib.mpm_grid_update(pp, wsp, cap, dt, sptr), "grid")
        if ev is not None:
            ev[3].record(stream)
        _lib.check(lib.mpm_g2p(pp, wsp, cap, n, nxt, dt, None, sptr), "g2p")
        if ev is not None:
            ev[4].record(stream)
        solver._cur = 1 - solver._cur

    solver._prepare(dt * (args.steps + args.warmup))
    plan = frame_plan(args.steps, args.frame)
    if fused:
        _, warm = time_frames(solver, dt, [args.warmup], stream)
        warm()
        evs, run = time_frames(solver, dt, plan, stream)
    else:
        for _ in range(args.warmup):
            substep_phases()
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(args.steps)]

        def run():
            for k in range(args.steps):
                substep_phases(evs[k])
    torch.cuda.synchronize()
    n_nodes = count_nodes(solver)
    occupancy = block8_fraction(solver)

    # timed region: K substeps, CUDA events on the launching stream
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        start.record(stream)
        run()
        stop.record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    total_ms = allmax(start.elapsed_time(stop), ws)
    st = int(solver._status.item())
    if st:
        raise RuntimeError(f"device status {st} during the benchmark")
    n = solver.n_particles
    value = replica_value(n, args.steps, ws, total_ms)
    peak, peak_kind = load_peaks()
    sub_bytes = (Q_ALGO_BYTES_PER_PARTICLE if args.quant else ALGO_BYTES_PER_PARTICLE) * n + \
        ALGO_BYTES_PER_NODE * n_nodes
    if fused:
        resorts = [solver._frame_resort(c) for c in plan]
        kt = frame_kernel_times(plan, evs, resorts)
        launches = sum(frame_launches(c, r) for c, r in zip(plan, resorts))
        totals = {k: float(sum(v)) for k, v in kt.items()}
        phases = {k: totals[k] / args.steps for k in totals}
        per_launch = {k: (totals[k] / len(v) if v else 0.0) for k, v in kt.items()}
        kernel_bytes = {"k_fused": FUSED_BYTES_PER_PARTICLE * n + FUSED_BYTES_PER_NODE * n_nodes,
                        "k_p2g": P2G_BYTES_PER_PARTICLE * n + P2G_BYTES_PER_NODE * n_nodes,
                        "k_g2p_stream": G2P_BYTES_PER_PARTICLE * n + G2P_BYTES_PER_NODE * n_nodes}
        top = max(kernel_bytes, key=lambda k: totals[k])
        schedule = {"mode": "fused frames (mpm_frame)", "resort_every": solver.resort_every,
                    "occupancy": solver.occupancy,
                    "resort_per_frame": resorts,
                    "frames": plan, "launches_per_kernel": {k: len(v) for k, v in kt.items()},
                    "ms_per_launch": per_launch}
    else:
        ph = np.array([[e[i].elapsed_time(e[i + 1]) for i in range(4)] for e in evs])
        launches = KERNELS_PER_SUBSTEP * args.steps
        phases = dict(zip(("binning", "k_p2g", "grid", "k_g2p"), ph.mean(0)))
        per_launch = dict(phases)
        totals = {k: v * args.steps for k, v in phases.items()}
        per_p2g = Q_P2G_BYTES_PER_PARTICLE if args.quant else P2G_BYTES_PER_PARTICLE
        kernel_bytes = {"k_p2g": per_p2g * n + P2G_BYTES_PER_NODE * n_nodes}
        top = "k_p2g"
        schedule = {"mode": "per-substep launches (mpm_substep phases)", "chunk": solver.chunk}
    top_ach = kernel_bytes[top] / (per_launch[top] / 1e3) / 1e9
    no_bin_ms = (total_ms - totals["binning"]) / args.steps
    sub_ach = sub_bytes / (no_bin_ms / 1e3) / 1e9
    full_ach = sub_bytes / (total_ms / args.steps / 1e3) / 1e9
    traffic = None if args.quant else kernel_traffic(top, n)
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(sc, args, ws, (solver.fuse_frames, solver.resort_every, solver.chunk))
    batched = None
    if not args.no_batched:
        batched = run_batched_measure()
    adjoint = None
    if not args.no_adjoint:
        adjoint = run_adjoint_measure()
    render = None
    if not args.no_render:
        render = run_render_measure(solver, rank == 0 and not args.no_cpu)
    g2p2g = None
    if not args.no_g2p2g:
        g2p2g = run_g2p2g_measure(sc, solver.resort_every)
    quant = None
    if not args.no_quant:
        quant = run_quant_measure(sc)
    pio = mesh = None
    if not args.no_io:
        pio = run_particle_output_measure(solver, peak, peak_kind, rank == 0 and not args.no_cpu)
        mesh = run_mesh_emitter_measure(peak, peak_kind, rank == 0 and not args.no_cpu)
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(sc, args)
    line = {
        "metric": "particle-substeps/s",
        "value": value,
        "unit": "particle-substeps/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded numpy scene generator; no dataset)",
        "config": {
            "workload": f"{sc.name}: {describe(sc)}" + (", packed particle storage (quant=True)" if args.quant else ""),
            "particles": n,
            "grid": list(sc.res),
            "grid_nodes_touched": n_nodes,
            "active_8cubed_block_fraction": round(occupancy, 4),
            "dt": dt,
            "l2": f"inputs larger than L2: particle state {n * 212 / 1e9:.2f} GB per buffer pair",
            "parallelism": f"replicas x{ws}",
            "chunk": solver.chunk,
            "autotune": tuned,
        },
        "schedule": schedule,
        "phases_ms_per_substep": phases,
        "roofline": {"bound": "hbm", "kernel": top, "achieved": top_ach, "peak": peak, "unit": "GB/s",
                     "frac": top_ach / peak, "traffic": traffic,
                     "algorithmic_bytes_per_launch": kernel_bytes[top], "ms_per_launch": per_launch[top],
                     "peak_source": peak_kind},
        "roofline_substep": {"bound": "hbm", "kernels": "all but binning", "achieved": sub_ach, "peak": peak,
                             "unit": "GB/s", "frac": sub_ach / peak,
                             "with_binning": {"achieved": full_ach, "frac": full_ach / peak},
                             "algorithmic_bytes_per_substep": sub_bytes, "peak_source": peak_kind},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "e2e": e2e,
        "cpu_baseline": cpu,
        "g2p2g": g2p2g,
        "quant": quant,
        "render": render,
        "particle_output": pio,
        "mesh_emitter": mesh,
        # last, so that a truncated tail of the line still shows them
        "batched": batched,
        "fwd_adjoint": adjoint,
    }
    if rank == 0:
        print(json.dumps(line))


def run_e2e(sc, args, ws, schedule):
    """End to end through the drop-in API: pinned host arrays -> read_restart
    -> step(frame_dt) frames -> particle_info(), with the schedule of the
    timed substeps (fuse_frames, resort_every, chunk)."""
    import torch

    from taichi_elements_gb300.mpm_solver import MPMSolver
    x = torch.from_numpy(sc.x).pin_memory()
    v = torch.from_numpy(sc.v).pin_memory()
    m = torch.from_numpy(sc.material).pin_memory()
    c = torch.from_numpy(np.full(sc.n, 0xFFFFFF, np.int32)).pin_memory()
    frames = args.e2e_frames
    frame_dt = args.e2e_substeps * sc.default_dt * 0.999
    count, _ = MPMSolver.count_substeps(frame_dt, sc.default_dt)

    def once(timed):
        s = MPMSolver(sc.res, size=sc.size, chunk=schedule[2])
        s.fuse_frames, s.resort_every = schedule[0], schedule[1]
        for cc in sc.postprocess:
            s.add_surface_collider(cc["point"], cc["normal"], cc.get("surface", 0), cc.get("friction", 0.0))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.read_restart(sc.n, x.numpy(), v.numpy(), m.numpy(), c.numpy())
        t1 = time.perf_counter()
        outs, parts = [], []
        for _ in range(frames):
            a = time.perf_counter()
            s.step(frame_dt)
            b = time.perf_counter()
            outs.append(s.particle_info())
            parts.append((b - a, time.perf_counter() - b))
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        del s, outs
        gc.collect()
        return t, t1 - t0, parts

    # warm-up: library, allocations, CUDA-graph capture, page-locked host
    # buffers (the caching host allocator keeps them for the timed run)
    once(False)
    once(False)
    barrier(ws)
    runs = [once(True) for _ in range(3)]  # the median run: one-time host costs vary between runs
    t, t_read, parts = sorted(runs, key=lambda r: r[0])[1]
    t = allmax(t, ws)
    h2d = sc.n * (12 + 12 + 4 + 4)
    d2h = sc.n * (12 + 12 + 4 + 4)
    return {"value": sc.n * count * frames * ws / t, "unit": "particle-substeps/s",
            "h2d_bytes_per_step": h2d / frames, "d2h_bytes_per_step": d2h,
            "step": f"one step(frame_dt) frame of {count} substeps + particle_info(); read_restart of the scene "
                    f"from pinned host memory inside the timed region (amortised over {frames} frames)",
            "ms": {"read_restart": 1e3 * t_read, "step": [1e3 * a for a, _ in parts],
                   "particle_info": [1e3 * b for _, b in parts]},
            "frames": frames, "seconds": t, "seconds_of_runs": [r[0] for r in runs]}


# algorithmic bytes per particle of one quantised frame: the range pass reads
# x, v (24); quantisation reads x, v, id (28) and writes x_and_v (12); the
# colour pass reads 4 and writes 3
IO_BYTES_PER_PARTICLE = 24 + 28 + 12 + 7


def run_particle_output_measure(solver, peak, peak_kind, with_cpu, reps=20):
    """The reference's quantised frame (engine/particle_io.py:12-76) of the
    bench scene: the three device kernels timed with CUDA events, the frame
    to host numpy arrays end to end, and the CPU restatement on a sample."""
    import torch

    from taichi_elements_gb300._lib import ROW_V, ROW_X
    from taichi_elements_gb300.particle_io import ParticleIO
    n, lib, s = solver.n_particles, solver._lib, solver.stream
    st = solver._state[solver._cur]
    keys = torch.empty(12, dtype=torch.int32, device="cuda")
    ranges = torch.empty(12, dtype=torch.float32, device="cuda")
    xv = torch.empty((n, 3), dtype=torch.int32, device="cuda")
    rgb = torch.empty((n, 3), dtype=torch.uint8, device="cuda")

    def kernels():
        lib.mpm_particle_ranges(st.data_ptr(), solver._cap, n, keys.data_ptr(), ranges.data_ptr(), s)
        lib.mpm_quantize_particles(st.data_ptr(), solver._cap, n, ranges.data_ptr(), xv.data_ptr(), s)
        lib.mpm_unpack_colors(solver._color.data_ptr(), n, rgb.data_ptr(), s)

    for _ in range(3):
        kernels()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        kernels()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    ach = IO_BYTES_PER_PARTICLE * n / (ms / 1e3) / 1e9
    ParticleIO.quantize(solver)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ParticleIO.quantize(solver)
    t_e2e = time.perf_counter() - t0
    out = {"value": n / (ms / 1e3), "unit": "particles/s (quantised frame, device kernels)",
           "ms_per_frame": ms, "particles": n,
           "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                        "algorithmic_bytes_per_particle": IO_BYTES_PER_PARTICLE, "peak_source": peak_kind},
           "e2e": {"value": n / t_e2e, "unit": "particles/s (device state to host numpy frame arrays)",
                   "d2h_bytes": 15 * n + 48},
           "gpu_launches_per_frame": 5}
    if with_cpu:
        from oracle import particle_io_ref as R
        m = min(n, 2_000_000)
        x = solver._gather(ROW_X, 3)[:m].cpu().numpy()
        v = solver._gather(ROW_V, 3)[:m].cpu().numpy()
        col = solver._color[:m].cpu().numpy()
        t0 = time.perf_counter()
        R.write_arrays(x, v, col)
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": m / tc, "unit": "particles/s", "cores": 1, "kind": "port",
                               "sample": f"{m} particles of the scene through the numpy restatement of "
                                         "ParticleIO.write_particles (the reference's own code is numpy)"}
    return out


# algorithmic bytes per voxel of one add_mesh: clearing the grid (4), the
# column scan (read 4 + write 4), the seed count and emit passes (4 + 4)
VOX_BYTES_PER_VOXEL = 20


def run_mesh_emitter_measure(peak, peak_kind, with_cpu, reps=5):
    """add_mesh on a 256^3 solver (a 512^3 voxel grid): a 20,480-triangle
    sphere, voxelized and seeded by the device kernels, timed with CUDA
    events; the CPU restatement of the voxelizer on a sample of triangles."""
    import torch

    from taichi_elements_gb300 import scenes
    from taichi_elements_gb300.voxelizer import Voxelizer
    tri = scenes.icosphere((0.5, 0.5, 0.5), 0.35, 5)
    vz = Voxelizer((256, 256, 256), 1.0 / 256, padding=3)
    stream = torch.cuda.current_stream()

    def once():
        vz.voxelize(tri)
        return vz.seed_particles(8, 4096, 3, (0.0, 0.0, 0.0), 1)

    x = once()
    torch.cuda.synchronize()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    tv = ts = 0.0
    for _ in range(reps):
        e0.record(stream)
        vz.voxelize(tri)
        e1.record(stream)
        x = vz.seed_particles(8, 4096, 3, (0.0, 0.0, 0.0), 1)
        e2.record(stream)
        torch.cuda.synchronize()
        tv += e0.elapsed_time(e1) / reps
        ts += e1.elapsed_time(e2) / reps
    nvox = vz.res[0] * vz.res[1] * vz.res[2]
    ach = VOX_BYTES_PER_VOXEL * nvox / ((tv + ts) / 1e3) / 1e9
    out = {"value": len(tri) / (tv / 1e3), "unit": "triangles/s (voxelize, device kernels)",
           "triangles": len(tri), "voxel_grid": list(vz.res), "particles_emitted": int(x.shape[0]),
           "ms_voxelize": tv, "ms_seed": ts,
           "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                        "algorithmic_bytes_per_voxel": VOX_BYTES_PER_VOXEL, "peak_source": peak_kind},
           "gpu_launches": 5}
    if with_cpu:
        from oracle import voxelizer_ref as V
        sample = tri[::40]
        t0 = time.perf_counter()
        V.voxelize(sample, vz.res, vz.dx, padding=3)
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": len(sample) / tc, "unit": "triangles/s", "cores": 1, "kind": "port",
                               "sample": f"{len(sample)} of the triangles through the numpy restatement of "
                                         "Voxelizer.voxelize_triangles on the same 512^3 voxel grid"}
    return out


def run_mode_measure(sc, substeps=50, warmup=5, **solver_kw):
    """The same scene with other solver modes (use_g2p2g, quant,
    support_plasticity): K substeps timed with CUDA events; returns
    (ms per substep, particles)."""
    import torch
    s = sc.make_solver(chunk=512, **solver_kw)
    dt = sc.default_dt
    s._prepare(dt)
    for _ in range(warmup):
        s._launch_substep(dt, -1)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(substeps):
        s._launch_substep(dt, -1)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / substeps
    if int(s._status.item()):
        raise RuntimeError(f"device status set during the {solver_kw} measurement")
    n = s.n_particles
    rows = int(s._state[0].shape[0])
    del s
    torch.cuda.empty_cache()
    return ms, n, rows


def run_quant_measure(sc, substeps=50):
    """quant=True (engine/mpm_solver.py:106-127, :216-262): the packed
    particle layout in the plain substep and in the fused G2P2G mode with
    support_plasticity=False (the reference's quantized demos)."""
    out = {"unit": "particle-substeps/s", "substeps": substeps}
    for key, kw in (("plain", dict(quant=True)),
                    ("g2p2g_no_plasticity", dict(quant=True, use_g2p2g=True, support_plasticity=False))):
        ms, n, rows = run_mode_measure(sc, substeps, **kw)
        out[key] = {"value": n / (ms / 1e3), "ms_per_substep": ms}
        out["state_bytes_per_particle"] = 4 * rows
    out["float32_state_bytes_per_particle"] = 4 * 28
    return out


def run_g2p2g_measure(sc, resort, substeps=50, warmup=5, tune=True):
    """The same scene in the fused G2P2G mode (MPMSolver(use_g2p2g=True),
    engine/mpm_solver.py:363-485): K substeps as one frame through
    mpm_g2p2g_frame (what step() runs, with the mode's own tuned re-sort
    interval and register budget, or re-sorted every `resort` substeps
    without the tuner), then K substeps of per-substep launches (substep()
    and the adaptive-dt loop), each timed with CUDA events."""
    import torch
    s = sc.make_solver(use_g2p2g=True, chunk=512)
    s.use_cuda_graph = False
    s.resort_every = resort
    tuned = None
    if tune:
        from taichi_elements_gb300.autotune import tune_schedule
        tuned = tune_schedule(s)
    dt = sc.default_dt
    s._prepare(dt)
    s._maxv = torch.zeros(max(substeps, warmup), dtype=torch.float32, device=s.device)
    stream = torch.cuda.current_stream()

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / substeps

    s.fuse_frames = True  # the frames are measured whichever launch mode the tuner preferred
    s._launch_substeps(warmup, dt)  # the first frame: fresh particles, the mode's state
    evs, run = time_frames(s, dt, [substeps], stream)
    ms_frame = timed(run)
    kt = frame_kernel_times([substeps], evs, [s._frame_resort(substeps)], g2p2g=True)
    s.fuse_frames = False
    s._g2p2g_listed = 0  # time_frames left the state binned (counts), as a frame does
    for _ in range(warmup):
        s._launch_substep(dt, -1)
    ms_sub = timed(lambda: [s._launch_substep(dt, -1) for _ in range(substeps)])
    if int(s._status.item()):
        raise RuntimeError("device status set during the G2P2G measurement")
    n = s.n_particles
    eff = s._frame_resort(substeps)
    sorts = (substeps + eff - 1) // eff
    out = {"value": n / (ms_frame / 1e3), "unit": "particle-substeps/s (fused G2P2G mode)",
           "ms_per_substep": ms_frame, "substeps": substeps, "resort_every": s.resort_every,
           "occupancy": s.occupancy,
           "autotune": None if tuned is None else {k: tuned[k] for k in ("frame_ms", "frame_ms_rolled", "mode")},
           "gpu_launches": sorts * (FINALIZE_LAUNCHES + 4) + (sorts - 1) + (substeps - sorts) * 4 + 1,
           "ms_per_launch": {k: (sum(v) / len(v) if v else 0.0) for k, v in kt.items()},
           "per_substep_launches": {"value": n / (ms_sub / 1e3), "ms_per_substep": ms_sub},
           "note": "use_g2p2g=True semantics (reference :363-485): C not stored, p_mass for every material"}
    del s
    torch.cuda.empty_cache()
    return out


def run_render_measure(solver, with_cpu, spp=8):
    """The path tracer on the bench scene's particles (renderer.py with the
    render_particles.py settings at res 512: dx = 1/512, sphere radius
    0.3/512, shutter 2e-3, 1280 x 720): cell-list build and `spp` samples
    per pixel timed with CUDA events."""
    import torch

    from taichi_elements_gb300.renderer import Renderer
    r = Renderer(dx=1 / 512, sphere_radius=0.3 / 512, shutter_time=2e-3, taichi_logo=False)
    r.set_camera_pos(3.24, 1.86, -4.57)
    r.look_at[None] = (0.5, 0.3, 0.5)
    r.floor_height[None] = -5e-3
    stream = torch.cuda.current_stream()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    torch.cuda.synchronize()
    e0.record(stream)
    r.initialize_particles_from_solver(solver)
    e1.record(stream)
    r.render(spp)
    e2.record(stream)
    torch.cuda.synchronize()
    t_build, t_render = e0.elapsed_time(e1), e1.elapsed_time(e2)
    npix = r.res[0] * r.res[1]
    out = {"value": npix * spp / (t_render / 1e3), "unit": "pixel-samples/s (path tracing, device kernel)",
           "resolution": list(r.res), "spp": spp, "ms_per_spp": t_render / spp, "ms_cell_lists": t_build,
           "particles": r.num_particles, "listed_particle_cells": r.total_inserted_particles(),
           "gpu_launches": 2 + spp // 8 + (1 if spp % 8 else 0)}
    if with_cpu:
        import numpy as np

        from oracle import renderer_ref as R
        sel = np.random.default_rng(0).choice(r.num_particles, size=min(r.num_particles, 1000), replace=False)
        x = r._x[torch.as_tensor(sel, device=r._x.device)].cpu().numpy()
        v = np.zeros_like(x)
        rgb = r._rgb[torch.as_tensor(sel, device=r._rgb.device)].cpu().numpy()
        g = R.Grid(x, r.dx)
        lists = R.cell_lists(g, x, v, r.sphere_radius, 0.0, motion_blur=False)
        pos, d = R.camera_rays(r.res, r.camera_pos[None], r.look_at[None], r.up[None], r.fov[None],
                               np.full(r.res + (2,), 0.5, np.float32))
        pos, d = pos.reshape(-1, 3)[::4000], d.reshape(-1, 3)[::4000]
        t0 = time.perf_counter()
        for q in range(len(pos)):
            R.next_hit(g, lists, x, v, rgb, np.float32(r.sphere_radius), pos[q], d[q], np.float32(0.0),
                       np.float32(-5e-3), False, motion_blur=False)
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": len(pos) / tc, "unit": "ray hits/s (nearest-hit query only)", "cores": 1,
                               "kind": "port", "sample": f"{len(pos)} camera rays against 1,000 of the particles "
                                                         "through the python restatement of next_hit"}
    del r
    torch.cuda.empty_cache()
    return out


def run_batched_measure(frames=3, substeps=50):
    """64 independent scenes (grids 32-96^3, 8K-300K particles each) advanced
    by the batched engine in CUDA-graph frames of `substeps` substeps (its
    default per-substep launches, then the same frames fused at both register
    budgets, each from the initial state), and the same scenes advanced by
    the plain solver looped scene by scene."""
    import torch

    from taichi_elements_gb300 import scenes
    from taichi_elements_gb300.batched import BatchedMPM, BatchScene
    raw = scenes.batched_scenes()
    total = sum(s.n for s in raw)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fuse_frames, occupancy=0):
        """Frames from the scenes' initial state: per-substep launches, or
        fused frames (mpm_batch_frame) with the fused kernel's budget."""
        B = BatchedMPM([BatchScene.from_scene(s) for s in raw])
        B.fuse_frames, B.occupancy = fuse_frames, occupancy
        for _ in range(2):
            B.substeps(substeps)  # first run, then graph capture
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(frames):
            B.substeps(substeps)
        e1.record(stream)
        torch.cuda.synchronize()
        B.check_status()
        return e0.elapsed_time(e1) / 1e3

    t_b = timed(False)
    t_bs = timed(True)
    t_bs16 = timed(True, 1)
    solvers = [s.make_solver() for s in raw]
    for sv, s in zip(solvers, raw):
        sv._prepare(s.default_dt)
        for _ in range(2):
            sv._run_frame(substeps, s.default_dt)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(frames):
        for sv, s in zip(solvers, raw):
            sv._run_frame(substeps, s.default_dt)
    e1.record(stream)
    torch.cuda.synchronize()
    t_l = e0.elapsed_time(e1) / 1e3
    v_b = total * substeps * frames / t_b
    v_l = total * substeps * frames / t_l
    return {"value": v_b, "unit": "particle-substeps/s", "looped_plain_value": v_l, "speedup_vs_looped": v_b / v_l,
            "fused_frames_value": total * substeps * frames / t_bs,
            "fused_frames_16warps_value": total * substeps * frames / t_bs16,
            "scenes": len(raw), "particles": total, "substeps_per_frame": substeps, "frames": frames,
            "workload": "64 scenes, grids {32,48,64,96}^3, 8K-300K particles in 1-3 cubes, 4 materials, "
                        "per-scene E log-uniform 1e4-1e6, CUDA-graph 50-substep frames"}


def run_adjoint_measure(n_substeps=2000, checkpoint_every=50):
    """Differentiable workload: a 64^3 grid with an elastic cube of 100K
    particles on a 100K-particle water slab, per-particle E, 2000 substeps,
    checkpoints every 50.  Times the plain forward rollout and the forward
    (with checkpoints) plus the hand-written adjoint of a centre-of-mass loss
    with respect to initial velocities and E."""
    import torch

    from taichi_elements_gb300 import scenes
    from taichi_elements_gb300.differentiable import Rollout, com_loss, rollout_positions
    from taichi_elements_gb300.mpm_solver import MPMSolver
    sc = scenes.elastic_on_water()
    rng = np.random.default_rng(5)
    E = np.full(sc.n, 1e6, np.float32) * np.exp(rng.uniform(-0.5, 0.5, sc.n)).astype(np.float32)
    s = MPMSolver(sc.res, per_particle_E=True)
    for m in (0, 1):
        sel = sc.material == m
        s.add_particles(sc.x[sel], m, E=torch.as_tensor(E[sel]))
    from taichi_elements_gb300.autotune import tune_chunk
    tune_chunk(s)
    R = Rollout(s, n_substeps, checkpoint_every=checkpoint_every)
    v0 = torch.zeros((sc.n, 3), device="cuda")
    e = torch.tensor(np.concatenate([E[sc.material == m] for m in (0, 1)]), device="cuda")
    mat = torch.tensor(np.concatenate([sc.material[sc.material == m] for m in (0, 1)]), device="cuda")
    target = torch.tensor(sc.target, dtype=torch.float32, device="cuda")
    for _ in range(2):  # warm-up: first runs, then CUDA-graph capture
        R.forward(v0, e, keep_checkpoints=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    R.forward(v0, e, keep_checkpoints=False)  # plain forward rollout
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    for _ in range(2):
        v = v0.clone().requires_grad_(True)
        ee = e.clone().requires_grad_(True)
        com_loss(rollout_positions(R, v, ee), mat, target).backward()
    v = v0.clone().requires_grad_(True)
    ee = e.clone().requires_grad_(True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x = rollout_positions(R, v, ee)
    L = com_loss(x, mat, target)
    L.backward()
    torch.cuda.synchronize()
    t_all = time.perf_counter() - t0
    return {"value": sc.n * n_substeps / t_all, "unit": "particle-substeps/s (forward+adjoint)",
            "plain_forward_value": sc.n * n_substeps / t_fwd, "fwd_adjoint_over_forward": t_all / t_fwd,
            "particles": sc.n, "substeps": n_substeps, "checkpoint_every": checkpoint_every, "chunk": s.chunk,
            "seconds_forward": t_fwd, "seconds_forward_adjoint": t_all,
            "grad_norms": {"v0": float(v.grad.norm()), "E": float(ee.grad.norm())},
            "workload": "64^3 grid, elastic cube 100K on water slab 100K, per-particle E, f32, "
                        "loss |com_elastic(T) - target|^2"}


def cpu_baseline(sc, args, budget_s=None):
    """The oracle port (C/OpenMP float32, every host thread) on a bounded
    sample: whole-scene substeps until the time budget is used."""
    from oracle import oracle as O
    budget_s = budget_s or args.cpu_budget
    cfg = O.Config(res=sc.res, size=sc.size, postprocess=[dict(kind=O.KIND_BOX, surface=0)] + list(sc.postprocess))
    P = O.Particles.seeded(sc.x, sc.material, v=sc.v, dtype=np.float32)
    threads = os.cpu_count() or 1
    R = O.Runner(cfg, P, nthreads=threads)
    dt = sc.default_dt
    R.run(dt, 1)  # warm-up (page-in)
    done = 0
    t0 = time.perf_counter()
    while True:
        R.run(dt, 1)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return {"value": sc.n * done / el, "unit": "particle-substeps/s", "cores": threads, "kind": "port",
            "sample": f"{done} substeps of the full {sc.n}-particle scene ({el:.1f} s)"}


def run_reference(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    sc = make_scene(args.workload)
    cfg = O.Config(res=sc.res, size=sc.size, postprocess=[dict(kind=O.KIND_BOX, surface=0)] + list(sc.postprocess))
    P = O.Particles.seeded(sc.x, sc.material, v=sc.v, dtype=np.float32)
    threads = os.cpu_count() or 1
    R = O.Runner(cfg, P, nthreads=threads)
    dt = sc.default_dt
    for _ in range(args.warmup):
        R.run(dt, 1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        R.run(dt, 1)
    el = time.perf_counter() - t0
    value = sc.n * args.steps / el
    line = {
        "impl": "reference",
        "metric": "particle-substeps/s",
        "value": value,
        "unit": "particle-substeps/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded numpy scene generator; no dataset)",
        "config": {"workload": f"{sc.name}: {describe(sc)}", "particles": sc.n, "grid": list(sc.res),
                   "parallelism": "host CPU"},
        "cpu_baseline": {"value": value, "unit": "particle-substeps/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} whole-scene substeps after {args.warmup} warm-up substeps; "
                                   "the reference's Taichi runtime is not installable here, so its substep "
                                   "runs as the C/OpenMP restatement"},
        "e2e": {"value": value, "unit": "particle-substeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=None)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="ellipsoids_256",
                    choices=["ellipsoids_256", "four_materials_128", "water_cube_64", "elastic_on_water",
                             "batched_64"])
    ap.add_argument("--chunk", type=int, default=None)
    ap.add_argument("--resort", type=int, default=None, help="fused frames re-sorted every this many substeps")
    ap.add_argument("--frame", type=int, default=50, help="substeps per mpm_frame call in the timed region")
    ap.add_argument("--schedule", choices=["frame", "substep"], default=None,
                    help="fused frames or per-substep launches (default: the autotuner's choice)")
    ap.add_argument("--occupancy", type=int, choices=[0, 1], default=None,
                    help="fused/P2G kernels unrolled at 12 warps per SM (0) or rolled at 16 (1)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-io", action="store_true", help="skip the particle-output and mesh-emitter measurements")
    ap.add_argument("--no-g2p2g", action="store_true", help="skip the fused G2P2G-mode measurement")
    ap.add_argument("--no-quant", action="store_true", help="skip the packed-storage (quant=True) measurement")
    ap.add_argument("--quant", action="store_true",
                    help="run the timed substeps with packed particle storage (quant=True)")
    ap.add_argument("--no-render", action="store_true", help="skip the path-tracer measurement")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--e2e-frames", type=int, default=3)
    ap.add_argument("--e2e-substeps", type=int, default=50)
    args = ap.parse_args()
    if args.workload == "elastic_on_water":  # the differentiable workload alone
        print(json.dumps(run_adjoint_measure(n_substeps=args.steps or 2000)))
        return
    if args.workload == "batched_64":  # the 64-scene batched workload alone
        print(json.dumps(run_batched_measure()))
        return
    if args.impl == "reference":
        args.steps = 3 if args.steps is None else args.steps
        args.warmup = 1 if args.warmup is None else args.warmup
        run_reference(args)
    else:
        args.steps = 200 if args.steps is None else args.steps
        args.warmup = 5 if args.warmup is None else args.warmup
        if args.warmup < 3:
            args.warmup = 3
        run_gb300(args)


if __name__ == "__main__":
    main()
