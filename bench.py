#!/usr/bin/env python
"""PBF particle-updates/s on one GB300 (one JSON line on stdout).

Workload (default): the 1,048,576-particle colliding-blocks scene (two 64x128x64
lattices, h = 0.0125, 4 Jacobi iterations, FP32), synthetic and seeded. A step is one
full PBF time step of every particle (Particles::timeStep, particles.cpp:250-297).

* ``value``: particle-updates/s with the state resident in HBM, device time of exactly
  K steps, each replayed as one CUDA graph, from CUDA events on the simulator's stream.
  Every timed step advances the configured initial state (cell-sorted once, then
  restored from a device snapshot between steps), so each step does the full work of
  one PBF step over the configured input: with the configured tensile k = 0.1 the
  reference's formulas blow the blocks apart within one step (FP64 restatement: median
  displacement several particle spacings), so a rollout would not keep that work.
  Snapshot restore and an L2 flush (256 MiB write) run between steps, outside the events.
* ``phases_ms_per_step``: the same K steps timed again, launched stream-ordered with
  CUDA events between phases (``phases_pass``).
* ``e2e``: the same metric through the C ABI with host buffers: per step
  pbf_set_state (H2D of positions and velocities from pinned memory), pbf_step, and
  pbf_get_state (D2H of positions and velocities), wall-clocked.
* ``roofline``: the dominant kernel's algorithmic bytes per launch over its average
  event-timed launch duration in the phase pass, against the measured HBM copy
  bandwidth.
* ``cpu_baseline``: the reference's own step (built from its sources) on a bounded
  sample of the workload on the host cores, else the FP64 restatement.
* ``--impl reference``: the reference CPU step alone, on the same config and metric.

Multi-GPU: replicas only (every rank runs the same scene; weak scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "PBF particle-updates/s at 1M (4 iters); batched & adjoint vs plain, 1 GB300"
UNIT = "particle-updates/s"

# Algorithmic HBM bytes per particle for each phase (FP32 SoA; each phase reads and
# writes its unique per-particle data once): B(I) = 340 + 56 I + 8 C/N.
ALGO_BYTES = {"predict": 64 + 24, "sort": 104, "gather": 0, "lambda": 20, "deltap": 36,
              "xsph": 84, "vorticity": 64, "neighbors": 16, "scan": 0, "stats": 0}
# DRAM bytes per particle per launch measured by ncu (dram__bytes_read.sum +
# dram__bytes_write.sum) on the 1M colliding-blocks scene: profiles/k_deltap_colliding_blocks_1m.md,
# profiles/k_lambda_colliding_blocks_1m.md and profiles/k_nbr_build_colliding_blocks_1m.md.
PER_ITERATION = ("lambda", "deltap")  # phases launched once per Jacobi iteration
NCU_TRAFFIC_PER_PARTICLE: dict[str, float] = {"deltap": 141.8, "lambda": 99.8, "neighbors": 86.0}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(gpu_index)], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def sample_block(scene, side=16):
    """A side^3 sub-lattice of the first block (bottom corner): the CPU baseline's sample."""
    nx, ny = 64, 128
    idx = [(k * ny + j) * nx + i for k in range(side) for j in range(side) for i in range(side)]
    idx = np.asarray(idx)
    return scene.pos[idx], scene.vel[idx]


def run_reference_sample(scene, steps, procs, side=16):
    """The reference step (oracle/_ref) on `procs` disjoint side^3 samples in parallel
    (side^3 sub-lattices of the first block, moved along z, so side <= 64)."""
    from oracle import ref_runner

    if not ref_runner.available():
        return None
    pos, vel = sample_block(scene, side)
    # disjoint samples: shift each copy's lattice window along z inside block A
    samples = []
    for p in range(procs):
        k0 = (p * side) % 64
        nx, ny = 64, 128
        idx = np.asarray([((k0 + k) % 64 * ny + j) * nx + i for k in range(side) for j in range(side)
                          for i in range(side)])
        samples.append((scene.pos[idx], scene.vel[idx]))
    from concurrent.futures import ThreadPoolExecutor

    with ThreadPoolExecutor(max_workers=procs) as ex:
        outs = list(ex.map(lambda s: ref_runner.run(s[0], s[1], scene.params, steps=steps, mode="literal",
                                                    restart=True), samples))
    secs = max(o["seconds"] for o in outs)
    n = samples[0][0].shape[0]
    return {"value": procs * n * steps / secs, "seconds": secs, "n": n, "steps": steps, "procs": procs}


def reference_fit_1m(scene, sides=(12, 16, 24, 32)) -> dict | None:
    """The reference step's cost at the workload's full size, extrapolated: one process
    steps side^3 sub-lattices of the workload (3 steps below 10,000 particles, 1 above);
    the reference's all-pairs neighbour search makes its time per step grow with N^2, and
    the least-squares fit t(N) = a N^2 + b N over the measured sizes (each point weighted by
    1/t, so each counts by its relative error) gives t at the full N. Labelled
    "extrapolated": the full step is not run. Its per-pair cost grows from 13,824 to 32,768
    particles as the particles outgrow the host's caches, so the fit is a floor."""
    from oracle import ref_runner

    if not ref_runner.available():
        return None
    pts = []
    for side in sides:
        steps = 3 if side ** 3 < 10000 else 1
        r = run_reference_sample(scene, steps, 1, side)
        pts.append((r["n"], r["seconds"] / steps))
    n = np.array([p[0] for p in pts], dtype=np.float64)
    t = np.array([p[1] for p in pts], dtype=np.float64)
    A = np.stack([n * n, n], 1) / t[:, None]
    (a, b), *_ = np.linalg.lstsq(A, np.ones_like(t), rcond=None)
    big = float(scene.n)
    t_big = a * big * big + b * big
    return {"value": big / t_big, "unit": UNIT, "kind": "extrapolated", "cores": 1,
            "seconds_per_step": t_big, "fit": "t(N) = a N^2 + b N, least squares in relative error",
            "a": float(a), "b": float(b),
            "measured": [{"particles": int(p[0]), "seconds_per_step": p[1]} for p in pts],
            "sample": f"reference step on {', '.join(f'{s}^3' for s in sides)} sub-lattices of {scene.name}, "
                      f"1 process; extrapolated to {scene.n} particles"}


def port_steps(pos, vel, params, steps, threads):
    """The FP64 restatement, `steps` single steps each from (pos, vel); returns seconds."""
    from oracle import oracle

    secs = 0.0
    for _ in range(steps):
        t = time.perf_counter()
        oracle.step(pos, vel, params, steps=1, threads=threads)
        secs += time.perf_counter() - t
    return secs


def cpu_baseline(scene, budget_s: float):
    """Reference step on one core, sized to roughly budget_s of CPU work."""
    from oracle import ref_runner

    if ref_runner.available():
        probe = run_reference_sample(scene, 2, 1)
        per_step = probe["seconds"] / 2
        steps = max(2, min(400, int(budget_s / max(per_step, 1e-4))))
        r = run_reference_sample(scene, steps, 1)
        out = {"value": r["value"], "unit": UNIT, "cores": 1, "kind": "reference",
               "sample": f"reference particles.cpp step (FP64, O(N^2) all-pairs) on a {r['n']}-particle "
                         f"16^3 sub-lattice of the workload, {steps} steps each from the sample's configured "
                         f"initial state, 1 thread; the reference's cost "
                         f"per particle grows with N, so this sample overstates its speed on the full scene",
               "sample_particles": r["n"]}
        fit = reference_fit_1m(scene)
        if fit:
            out["extrapolated_1m"] = fit
        return out
    pos, vel = sample_block(scene, 32)
    dt = port_steps(pos, vel, scene.params, 2, 1) / 2
    steps = max(1, min(200, int(budget_s / max(dt, 1e-4))))
    secs = port_steps(pos, vel, scene.params, steps, 1)
    return {"value": pos.shape[0] * steps / secs, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"FP64 restatement (uniform grid) on a {pos.shape[0]}-particle sub-lattice, {steps} steps, "
                      f"1 thread (reference build unavailable)"}


def cpu_port_all_cores(scene, budget_s: float):
    """The FP64 restatement (fp64-grid: uniform grid, OpenMP) on the full workload, every
    step from the configured state, on all host threads: the same-size CPU figure."""
    from oracle import oracle

    pos, vel = scene.pos, scene.vel
    threads = oracle.max_threads()
    dt = port_steps(pos, vel, scene.params, 1, threads)
    steps = max(1, min(20, int(budget_s / max(dt, 1e-4))))
    secs = port_steps(pos, vel, scene.params, steps, threads)
    return {"value": pos.shape[0] * steps / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"FP64 restatement (uniform grid, OpenMP) on the full {pos.shape[0]}-particle workload, "
                      f"{steps} steps each from the configured state"}


def workload_config(scene, extra=None):
    cfg = {"workload": scene.name, "particles": int(scene.n), "iters": scene.params.iters, "h": scene.params.h,
           "dt": scene.params.dt, "seed": scene.seed, "l2": "flushed between timed steps (256 MiB write, untimed)",
           "protocol": "each timed step advances the configured initial state (device snapshot restored between "
                       "steps, untimed)",
           "parallelism": "replicas", "notes": scene.notes}
    if extra:
        cfg.update(extra)
    return cfg


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(x: float, world: int) -> float:
    from fluid_gb300.shard import max_over_ranks

    return max_over_ranks(x, world)


def barrier(world):
    from fluid_gb300.shard import barrier as _barrier

    _barrier(world)


def bench_batched(args, world, rank, local, steps: int = 10, warmup: int = 3) -> dict:
    """256 independent scenes of 2k-32k particles: one batched handle (one launch per
    phase over every scene, the step replayed as a CUDA graph, launch shapes from the
    autotuner) against the same scenes stepped one at a time, each with its own graph.
    Both time device work with CUDA events per step; every step starts from the scenes'
    configured state (snapshot restored between steps, untimed). With several ranks the
    scenes are partitioned by scene (fluid_gb300.shard, balanced by particle count) and
    each rank steps its share; the job's time is the slowest rank's."""
    import torch

    from fluid_gb300 import pbf, scenes
    from fluid_gb300.params import PBF_FLAG_GRAPH
    from fluid_gb300.shard import max_over_ranks, shard_scenes

    b = scenes.batched_256()
    mine = shard_scenes(b.counts, world)[rank]
    first = np.concatenate([[0], np.cumsum(b.counts)])
    pos = np.concatenate([b.pos[first[k]:first[k + 1]] for k in mine])
    vel = np.concatenate([b.vel[first[k]:first[k + 1]] for k in mine])
    counts = [b.counts[k] for k in mine]
    boxes = [b.boxes[k] for k in mine]
    prm = b.params.with_(flags=PBF_FLAG_GRAPH)
    dt = prm.dt
    sim = pbf.Simulator(pos, vel, prm, device=local, counts=counts, boxes=boxes)
    sim.sort()
    sim.snapshot()
    tuning = sim.autotune(dt, reps=2)
    stream = torch.cuda.ExternalStream(sim.stream)
    for _ in range(warmup):
        sim.restore()
        sim.step_async(dt, 1)
    sim.sync()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for k in range(steps):
        sim.restore()
        ev[k][0].record(stream)
        sim.step_async(dt, 1)
        ev[k][1].record(stream)
    sim.sync()
    batched_s = max_over_ranks(sum(a.elapsed_time(z) for a, z in ev) / 1e3, world)
    sim.close()

    singles = []
    for k in mine:
        s1 = pbf.Simulator(b.pos[first[k]:first[k + 1]], b.vel[first[k]:first[k + 1]], prm, device=local)
        s1.set_tuning(**tuning)
        s1.sort()
        s1.snapshot()
        singles.append(s1)
    for s1 in singles:  # warm each graph
        for _ in range(2):
            s1.restore()
            s1.step_async(dt, 1)
        s1.sync()
    single_s = 0.0
    for _ in range(steps):
        for s1 in singles:
            st = torch.cuda.ExternalStream(s1.stream)
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s1.restore()
            a.record(st)
            s1.step_async(dt, 1)
            z.record(st)
            s1.sync()
            single_s += a.elapsed_time(z) / 1e3
    for s1 in singles:
        s1.close()
    single_s = max_over_ranks(single_s, world)
    n_total = int(sum(b.counts))
    v_b = n_total * steps / batched_s
    v_1 = n_total * steps / single_s
    return {"workload": "batched_256", "scenes": len(b.counts), "particles": n_total,
            "counts_min_max": [min(b.counts), max(b.counts)], "steps": steps,
            "value": v_b, "one_at_a_time": v_1, "speedup": v_b / v_1, "unit": UNIT,
            "ms_per_step": batched_s / steps * 1e3, "one_at_a_time_ms_per_step": single_s / steps * 1e3,
            "graph": True, "tuning": tuning, "ranks": world,
            "sharding": "scenes partitioned over ranks by particle count" if world > 1 else "one rank"}


def bench_reference(args, scene, world, rank):
    if rank != 0:
        return 0
    procs = max(1, min(os.cpu_count() or 1, 64))
    from oracle import ref_runner

    if not ref_runner.available():
        # fall back to the FP64 restatement (the oracle port) on all host threads
        from oracle import oracle

        pos, vel = sample_block(scene, 48)
        threads = oracle.max_threads()
        port_steps(pos, vel, scene.params, max(args.warmup, 1), threads)
        secs = port_steps(pos, vel, scene.params, args.steps, threads)
        value = pos.shape[0] * args.steps / secs
        kind, cores = "port", threads
        sample = f"FP64 restatement (OpenMP) on a {pos.shape[0]}-particle sub-lattice, {args.steps} steps"
        ms = secs / args.steps * 1e3
        run_n = pos.shape[0]
        fit = None
    else:
        run_reference_sample(scene, max(args.warmup, 1), procs)  # warm-up
        r = run_reference_sample(scene, args.steps, procs)
        value, kind, cores = r["value"], "reference", procs
        sample = (f"reference particles.cpp step (unmodified but for the parameter block), {procs} processes x "
                  f"{r['n']}-particle disjoint 16^3 sub-lattices of the workload, {args.steps} steps each; "
                  f"its all-pairs search makes the full {scene.n}-particle step far slower than this sample")
        ms = r["seconds"] / args.steps * 1e3
        run_n = procs * r["n"]
        fit = reference_fit_1m(scene)
    cfg = workload_config(scene, {"particles": int(run_n), "source_workload": scene.name,
                                  "source_particles": int(scene.n),
                                  "sample": "disjoint sub-lattices of the source workload, stepped independently"})
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if fit:
        line["extrapolated_1m"] = fit
    print(json.dumps(line))
    return 0


def bench_adjoint(args, local, steps: int = 30, big_steps: int = 5) -> dict:
    """Adjoint against plain forward. Workload: the 32^3 block of scenes.adjoint_32k over
    its 30-step rollout: the forward steps run from the initial state keeping a
    checkpoint (x, v) before every step, then pbf_adjoint_step_device runs once per step
    in reverse from those checkpoints (recording recompute of the step + its reverse).
    Every timed step is bracketed by CUDA events on the handle's stream, with an L2
    flush before it in both arms. The same pair is also timed at 1M particles
    (colliding_blocks_1m, every step from the configured state) and the whole
    torch.autograd rollout (forward with checkpoints + backward) end to end."""
    import torch

    from fluid_gb300 import pbf, scenes
    from fluid_gb300.autograd import rollout

    dev = f"cuda:{local}"
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def pair(sc, nsteps, rollout_mode):
        prm = sc.params.with_(flags=0)
        sim = pbf.Simulator(sc.pos, sc.vel, prm, device=local)
        n = sim.n
        dt = prm.dt
        st = torch.cuda.ExternalStream(sim.stream)
        x0 = torch.tensor(sc.pos.astype(np.float32), device=dev)
        v0 = torch.tensor(sc.vel.astype(np.float32), device=dev)
        ckx = torch.empty((nsteps if rollout_mode else 0, n, 3), dtype=torch.float32, device=dev)
        ckv = torch.empty_like(ckx)
        g = [torch.zeros((n, 3), dtype=torch.float32, device=dev) for _ in range(4)]
        g[0].normal_()
        r0 = torch.zeros(nsteps, dtype=torch.float64, device=dev)
        ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
        fwd, adj = [], []
        if not rollout_mode:  # every step from the configured state, sorted once (as the main leg)
            sim.sort()
            sim.snapshot()
        for rep in range(2):  # the first pass warms both paths
            fwd.clear()
            adj.clear()
            if rollout_mode:
                sim.set_state_device(x0.data_ptr(), v0.data_ptr(), torch.cuda.current_stream().cuda_stream)
            torch.cuda.synchronize()
            with torch.cuda.stream(st):
                for t in range(nsteps):
                    if rollout_mode:
                        sim.get_state_device(ckx[t].data_ptr(), ckv[t].data_ptr(), None, st.cuda_stream)
                    else:
                        sim.restore()
                    flush.zero_()
                    a, z = ev(), ev()
                    a.record(st)
                    sim.step_async(dt, 1)
                    z.record(st)
                    fwd.append((a, z))
                for t in range(nsteps - 1, -1, -1):
                    if rollout_mode:
                        xp, vp = ckx[t].data_ptr(), ckv[t].data_ptr()
                    else:
                        sim.restore()
                        xp = vp = None  # the restored state
                    flush.zero_()
                    a, z = ev(), ev()
                    a.record(st)
                    sim.adjoint_step_device(dt, xp, vp, g[0].data_ptr(), g[1].data_ptr(), g[2].data_ptr(),
                                            g[3].data_ptr(), r0[t].data_ptr(), stream=st.cuda_stream)
                    z.record(st)
                    adj.append((a, z))
            sim.sync()
            torch.cuda.synchronize()
        f_ms = sum(a.elapsed_time(z) for a, z in fwd) / nsteps
        a_ms = sum(a.elapsed_time(z) for a, z in adj) / nsteps
        out = {"particles": n, "steps": nsteps, "forward_ms_per_step": f_ms, "adjoint_ms_per_step": a_ms,
               "ratio": a_ms / f_ms, "forward_updates_per_s": n / (f_ms / 1e3),
               "adjoint_updates_per_s": n / (a_ms / 1e3)}
        if rollout_mode:  # the torch.autograd rollout, forward + backward, end to end on the device
            rho0 = torch.tensor(prm.rest_density, dtype=torch.float64, requires_grad=True)
            tgt = x0 + 0.01
            times = []
            for rep in range(2):
                v = v0.clone().requires_grad_(True)
                torch.cuda.synchronize()
                a, m, z = ev(), ev(), ev()
                a.record()
                xT, vT = rollout(sim, x0, v, rho0, nsteps)
                loss = ((xT - tgt) ** 2).mean()
                m.record()
                loss.backward()
                z.record()
                torch.cuda.synchronize()
                times.append((a.elapsed_time(m), m.elapsed_time(z)))
            out["autograd_forward_ms"], out["autograd_backward_ms"] = times[-1]
            out["autograd_ratio"] = (times[-1][0] + times[-1][1]) / (f_ms * nsteps)
        sim.close()
        return out

    small = pair(scenes.adjoint_32k(), steps, True)
    big = pair(scenes.colliding_blocks_1m(), big_steps, False)
    return {"workload": "adjoint_32k", "unit": UNIT, "l2": "flushed (256 MiB) before every timed step",
            **small, "at_1m": {"workload": "colliding_blocks_1m", **big},
            "target_ratio": 3.0}


def bench_surface(sim, prm) -> dict:
    """The marching-cubes surface (pbf_surface) of the workload's configured state over the
    collider box at updateSurface's settings (iso 0.95 rest density, step 0.5 h): one call,
    wall-clocked after a warm-up call (cell sort of the state, corner field, classify,
    scan, emit with normals, D2H of the triangles)."""
    import ctypes

    from fluid_gb300 import pbf

    L = pbf.lib()
    iso, step = 0.95 * prm.rest_density, 0.5 * prm.h
    lo = np.ascontiguousarray(prm.box_lo, dtype=np.float64)
    hi = np.ascontiguousarray(prm.box_hi, dtype=np.float64)
    count = ctypes.c_size_t(0)
    sim.restore()
    rc = L.pbf_surface(sim._h, iso, step, lo.ctypes.data_as(pbf.P), hi.ctypes.data_as(pbf.P), None, None, 0,
                       ctypes.byref(count))
    if rc:
        raise RuntimeError(L.pbf_last_error(sim._h).decode())
    t = count.value
    xyz = np.zeros((max(t, 1), 9), dtype=np.float32)
    nrm = np.zeros((max(t, 1), 9), dtype=np.float32)
    times = []
    for _ in range(3):
        sim.restore()
        sim.sync()
        t0 = time.perf_counter()
        rc = L.pbf_surface(sim._h, iso, step, lo.ctypes.data_as(pbf.P), hi.ctypes.data_as(pbf.P),
                           xyz.ctypes.data_as(pbf.P), nrm.ctypes.data_as(pbf.P), t, ctypes.byref(count))
        times.append(time.perf_counter() - t0)
        if rc:
            raise RuntimeError(L.pbf_last_error(sim._h).decode())
    cubes = 1
    for a in range(3):
        cubes *= int((prm.box_hi[a] - prm.box_lo[a]) / step) + 1
    ms = min(times[1:]) * 1e3
    return {"workload": "surface of the configured state over the collider box", "iso": iso, "step": step,
            "cubes": cubes, "triangles": t, "ms": ms, "cubes_per_s": cubes / (ms / 1e3),
            "timing": "wall clock of one pbf_surface call with host output, best of 2 after a warm-up"}


RENDER_SETTINGS = (1280, 720, 16, 3, 4)  # width, height, camera rays per pixel, depth, area-light samples


def render_reference_sample(settings=(4, 3, 4)) -> dict | None:
    """The reference's own PathTracer::render_to_file (oracle/_ref, one thread) on the
    committed Cornell-box fixture (the reference's default 720 particles): two frames,
    64 x 48 and 128 x 96; the per-path cost is the difference of their times over the
    difference of their paths, so the reference's surface and BVH build (the same in both)
    drop out."""
    from oracle import ref_runner

    if not ref_runner.render_available():
        return None
    from tests.golden.make_golden import params_from_json
    from tests.golden.make_render_golden import camera_from_json, scene_from_arrays

    g = np.load(ROOT / "tests" / "golden" / "render_p_default.npz")
    scene, cam, prm = scene_from_arrays(g), camera_from_json(str(g["camera"])), params_from_json(str(g["params"]))
    aa, depth, area = settings
    t = {}
    for (W, H) in ((64, 48), (128, 96)):
        t[(W, H)] = min(ref_runner.render(scene, cam, g["pos"], prm, W, H, ns_aa=aa, max_depth=depth,
                                          ns_area_light=area, seed=1)["seconds"] for _ in range(2))
    paths = (128 * 96 - 64 * 48) * aa
    dt = t[(128, 96)] - t[(64, 48)]
    return {"paths_per_s": paths / dt if dt > 0 else None, "cores": 1, "kind": "reference",
            "sample": f"reference render_to_file, Cornell box with the reference's 720 default particles "
                      f"({len(g['surf_xyz'])} surface triangles), ns_aa {aa}, depth {depth}, area samples {area}: "
                      f"(t(128x96) - t(64x48)) over the difference in paths",
            "seconds": {f"{w}x{h}": v for (w, h), v in t.items()}}


def bench_render(sim, prm, settings=RENDER_SETTINGS, reference: bool = True) -> dict:
    """Path tracing (pbf_render) of the workload's configured state in a Cornell box on the
    collider box, RENDER_SETTINGS, the surface over the collider box at updateSurface's
    settings. Device time of each phase from the call's own CUDA events (surface: cell
    sort, field, count, host read of the count, emit; hierarchy build; trace + tone map),
    best of 2 frames after a warm-up; the wall time adds the 8-bit frame's copy to the host."""
    from fluid_gb300 import render as R

    W, H, aa, depth, area = settings
    scene, cam = R.cornell_box(prm.box_lo, prm.box_hi)
    sim.restore()
    sim.set_render_scene(scene)
    best = None
    for i in range(3):
        sim.restore()
        sim.sync()
        t0 = time.perf_counter()
        out = sim.render(cam, W, H, aa, depth, area, seed=1 + i, lo=prm.box_lo, hi=prm.box_hi, hdr=False)
        wall = time.perf_counter() - t0
        if i and (best is None or out["stats"]["ms_total"] < best[0]["ms_total"]):
            best = (out["stats"], wall)
    st, wall = best
    paths = W * H * aa
    line = {"workload": "configured state in a Cornell box on the collider box", "width": W, "height": H,
            "ns_aa": aa, "max_ray_depth": depth, "ns_area_light": area, "triangles": st["triangles"],
            "surface_triangles": st["surface_triangles"], "ms_surface": st["ms_surface"], "ms_bvh": st["ms_bvh"],
            "ms_trace": st["ms_trace"], "ms_frame_wall": wall * 1e3, "paths_per_s": paths / (st["ms_trace"] / 1e3),
            "timing": "CUDA events per phase inside pbf_render; best of 2 after a warm-up"}
    try:
        ref = render_reference_sample((aa, depth, area)) if reference else None
    except Exception as exc:  # the reference's renderer is a reported baseline only
        ref = {"unavailable": str(exc)[:200]}
    if ref:
        line["cpu_reference"] = ref
    return line


def bench_ours(args, scene, world, rank, local):
    import torch

    from fluid_gb300 import pbf
    from fluid_gb300.params import PBF_FLAG_GRAPH, PBF_FLAG_STATS

    torch.cuda.set_device(local)
    # the timed region replays each step as one CUDA graph (events only around steps)
    prm = scene.params.with_(flags=PBF_FLAG_STATS | PBF_FLAG_GRAPH)
    sim = pbf.Simulator(scene.pos, scene.vel, prm, device=local)
    n = sim.n
    dt = prm.dt
    stream = torch.cuda.ExternalStream(sim.stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    sim.sort()
    sim.snapshot()
    tuning = sim.autotune(dt, reps=3) if not args.no_autotune else sim.tuning()
    for _ in range(args.warmup):
        sim.restore()
        sim.step_async(dt, 1)
    sim.sync()

    gpu_index = local
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        try:
            gpu_index = int(vis.split(",")[local])
        except ValueError:
            pass

    def timed_steps(s, st, steps):
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        barrier(world)
        torch.cuda.synchronize()
        with torch.cuda.stream(st):
            for k in range(steps):
                s.restore()
                flush.zero_()
                starts[k].record(st)
                s.step_async(dt, 1)
                ends[k].record(st)
        s.sync()
        torch.cuda.synchronize()
        barrier(world)
        return [a.elapsed_time(z) for a, z in zip(starts, ends)]

    clocks = ClockSampler(gpu_index)
    time.sleep(0.3)
    step_ms = timed_steps(sim, stream, args.steps)
    clk = clocks.stop()
    total_ms = reduce_max(sum(step_ms), world)
    value = world * n * args.steps / (total_ms / 1e3)

    # The same step from the caller's particle order: the state is uploaded in its original
    # (unsorted) order before every step (pbf_set_state_device, untimed), so the step's cell
    # sort starts from an unsorted array, as it does after pbf_set_state.
    x0d = torch.tensor(scene.pos.astype(np.float32), device=f"cuda:{local}")
    v0d = torch.tensor(scene.vel.astype(np.float32), device=f"cuda:{local}")
    uns = []
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for k in range(args.steps + 1):
            sim.set_state_device(x0d.data_ptr(), v0d.data_ptr(), stream.cuda_stream)
            flush.zero_()
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            sim.step_async(dt, 1)
            z.record(stream)
            if k:  # the first step warms the unsorted-start graph
                uns.append((a, z))
    sim.sync()
    torch.cuda.synchronize()
    uns_ms = reduce_max(sum(a.elapsed_time(z) for a, z in uns), world) / len(uns)
    del x0d, v0d
    stats = sim.stats()
    surface = bench_surface(sim, prm) if not args.no_surface else None
    render = bench_render(sim, prm) if not args.no_render else None

    # phase breakdown: the same K steps again, launched stream-ordered (no graph) with
    # CUDA events between phases on the simulator's stream
    psim = pbf.Simulator(scene.pos, scene.vel, scene.params.with_(flags=PBF_FLAG_STATS), device=local)
    psim.set_tuning(**tuning)
    psim.sort()
    psim.snapshot()
    pstream = torch.cuda.ExternalStream(psim.stream)
    psim.set_profiling(True)
    for _ in range(args.warmup):
        psim.restore()
        psim.step_async(dt, 1)
    psim.sync()
    psim.reset_phase_times()
    prof_ms = timed_steps(psim, pstream, args.steps)
    phases = psim.phase_times()
    psim.set_profiling(False)
    psim.close()

    # dominant kernel (by device time in the phase pass) and its roofline
    peak, peak_kind = peaks()
    dom = max((k for k in phases if ALGO_BYTES.get(k, 0) > 0), key=lambda k: phases[k][0])
    dom_ms, dom_launches = phases[dom]
    per_launch_s = dom_ms / max(dom_launches if dom in PER_ITERATION else args.steps, 1) / 1e3
    algo = ALGO_BYTES[dom] * n
    achieved = algo / per_launch_s / 1e9
    traffic = NCU_TRAFFIC_PER_PARTICLE.get(dom)
    step_bytes = (340 + 56 * prm.iters) * n
    # the same figures for every phase with algorithmic bytes: per launch for the passes that
    # run once per iteration (their bytes are per launch), per step for the others (whose
    # bytes cover all of the phase's launches: the sort's scatter, rank and large-cell sort)
    per_kernel = {}
    for k, (ms, cnt) in phases.items():
        if ALGO_BYTES.get(k, 0) > 0 and cnt > 0:
            units = cnt if k in PER_ITERATION else args.steps
            sec = ms / units / 1e3
            per_kernel[k] = {"launches_per_step": cnt / args.steps,
                             "per": "launch" if k in PER_ITERATION else "step", "ms": sec * 1e3,
                             "algo_bytes": ALGO_BYTES[k] * n,
                             "achieved": ALGO_BYTES[k] * n / sec / 1e9,
                             "frac": ALGO_BYTES[k] * n / sec / 1e9 / peak,
                             "share_of_phase_pass": ms / sum(prof_ms)}
    launches = int(sum(v[1] for v in phases.values()))

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        xh = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
        vh = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
        x0 = scene.pos.astype(np.float32)
        v0 = scene.vel.astype(np.float32)
        L = pbf.lib()
        xp, vp = xh.ctypes.data_as(pbf.P), vh.ctypes.data_as(pbf.P)
        tot = 0.0
        e2e_steps = max(1, args.steps)
        for k in range(e2e_steps + 1):
            xh[:] = x0  # the configured input, as a host caller would hand it over
            vh[:] = v0
            with torch.cuda.stream(stream):
                flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rc = L.pbf_set_state(sim._h, xp, vp)
            rc |= L.pbf_step(sim._h, dt, 1)
            rc |= L.pbf_get_state(sim._h, xp, vp, None)
            t1 = time.perf_counter()
            if rc:
                raise RuntimeError(L.pbf_last_error(sim._h).decode())
            if k > 0:  # the first iteration warms the unsorted-input path
                tot += t1 - t0
        tot = reduce_max(tot, world)
        e2e = {"value": world * n * e2e_steps / tot, "unit": UNIT, "h2d_bytes_per_step": 2 * n * 12,
               "d2h_bytes_per_step": 2 * n * 12, "ms_per_step": tot / e2e_steps * 1e3,
               "path": "pbf_set_state + pbf_step + pbf_get_state (positions and velocities), pinned host buffers"}
    sim.close()

    batched = bench_batched(args, world, rank, local) if not args.no_batched else None
    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(scene, {"launch": "CUDA graph replay of each step"}),
        "start_order": {"presorted": {"ms_per_step": total_ms / args.steps, "value": value},
                        "unsorted": {"ms_per_step": uns_ms, "value": world * n / (uns_ms / 1e3)},
                        "note": "value is timed from the cell-sorted configured state; 'unsorted' times the "
                                "same step from the caller's particle order (state uploaded before each step)"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": None if traffic is None else traffic * n,
                     "algo_bytes_per_launch": algo, "avg_launch_ms": per_launch_s * 1e3,
                     "step_frac": step_bytes / (total_ms / args.steps / 1e3) / 1e9 / peak,
                     "kernels": per_kernel},
        "phases_ms_per_step": {k: v[0] / args.steps for k, v in phases.items()},
        "phases_pass": {"launch": "stream-ordered with events between phases (no graph)",
                        "ms_per_step": sum(prof_ms) / args.steps},
        "tuning": tuning,
        "gpu_launches": launches,
        "clocks": clk,
        "pair_rate": {"neighbour_pairs_per_step": stats["mean_neighbors"] * n * (2 * prm.iters + 2),
                      "pairs_per_s": stats["mean_neighbors"] * n * (2 * prm.iters + 2) / (total_ms / args.steps / 1e3),
                      "passes": 2 * prm.iters + 2,
                      "note": "every pass over the fixed neighbour sets (lambda and delta-p per iteration, XSPH, "
                              "vorticity) evaluates each (i, j) from i's side; the build's candidate tests are "
                              "not counted"},
        "stats": {"mean_density_over_rho0": stats["mean_density"] / prm.rest_density,
                  "mean_neighbors": stats["mean_neighbors"], "max_neighbors": stats["max_neighbors"]},
    }
    if e2e:
        line["e2e"] = e2e
    if surface:
        line["surface"] = surface
    if render:
        line["render"] = render
    if batched:
        line["batched"] = batched
    if not args.no_adjoint:
        line["adjoint"] = bench_adjoint(args, local)
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(scene, args.cpu_seconds)
        line["cpu_port_all_cores"] = cpu_port_all_cores(scene, min(args.cpu_seconds, 10.0))
    print(json.dumps(line))
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="colliding_blocks_1m")
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-surface", action="store_true")
    ap.add_argument("--no-render", action="store_true")
    ap.add_argument("--render-only", action="store_true",
                    help="only the path-tracing leg (one JSON object), e.g. for an ncu capture")
    ap.add_argument("--render-settings", type=int, nargs=5, default=list(RENDER_SETTINGS),
                    metavar=("W", "H", "AA", "DEPTH", "LIGHT_SAMPLES"))
    ap.add_argument("--adjoint-only", action="store_true",
                    help="run only the adjoint leg and print its object (a profiling aid, not a bench line)")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    from fluid_gb300 import scenes

    world, rank, local = dist_setup()
    if world > 1 and args.impl == "ours":
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    if args.render_only:
        import torch

        from fluid_gb300 import pbf

        torch.cuda.set_device(local)
        build = scenes.SCENES[args.workload]
        scene = build() if args.seed is None else build(args.seed)
        with pbf.Simulator(scene.pos, scene.vel, scene.params, device=local) as sim:
            sim.snapshot()
            line = bench_render(sim, scene.params, tuple(args.render_settings), reference=not args.no_cpu_baseline)
        print(json.dumps({"render": line}))
        return 0
    if args.adjoint_only:
        import torch

        torch.cuda.set_device(local)
        print(json.dumps({"adjoint": bench_adjoint(args, local)}))
        return 0
    build = scenes.SCENES[args.workload]
    scene = build() if args.seed is None else build(args.seed)
    try:
        if args.impl == "reference":
            return bench_reference(args, scene, world, rank)
        return bench_ours(args, scene, world, rank, local)
    finally:
        if world > 1 and args.impl == "ours":
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
