"""Benchmark of the explicit snow-MPM step on GB300.

Default workload (the plain large single scene): two snowballs colliding
head-on at +-5 m/s, 1,048,576 particles (8 per cell), 256^3 grid, h = 1/256,
dt = 2e-5, FAST mode (FP32, error <= 1e-5 vs the FP64 oracle per step).

A step is one ExplicitTimeUpdate::update(dt) over the whole scene. The L2
cache (129 MB) is flushed by writing a 256 MB buffer before each timed step;
each step is timed with CUDA events on the library's stream.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0). --impl reference times the reference's own
compute shaders compiled as C++ (oracle/_ref) on the host cores, or the
oracle restatement when those are not built.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s batched vs per-scene at ≤1e-5 rel err; p50/p99 job latency"
UNIT = "particle-steps/s"
L2_FLUSH_BYTES = 256 << 20

# Algorithmic bytes (FP32 SoA state), per particle-step and per active grid
# node: P2G reads 72 B per particle (x, m, v, V0, F_E, J_p) and writes 16 B
# per node; G2P + advance reads 64 B and writes 64 B per particle and reads
# 24 B per node; the grid update moves 40 B per node. The fused kernel
# (G2P + advance of this step, P2G of the next) carries both figures.
BYTES_G2P2G = (72 + 128, 16 + 24)
BYTES_GRID = (0, 40)

# From a one-launch ncu capture of the fused kernel on this workload at the
# work split named in TRAFFIC_SOURCE, keyed by (particles, grid edge); other
# workloads report null: DRAM bytes (read + write) per launch, and warp
# instructions per launch for the issue roofline.
TRAFFIC_MEASURED = {(1 << 20, 256): 144.3e6}
INSTRUCTIONS_MEASURED = {(1 << 20, 256): 173.2e6}
TRAFFIC_SOURCE = ("not counted in this run: separate ncu --set full captures of one k_g2p2g launch of this "
                  "workload (256 particles per item, 2 CTAs per SM; sort interval 8 and 32 alike)")
# warp-instruction issue peak: 152 SMs x 4 schedulers x 2.07 GHz
ISSUE_PEAK = 152 * 4 * 2.07e9
# FP32 peak: 152 SMs x 128 lanes x 2 flops per FMA x 2.07 GHz; the algorithmic
# flops of one particle-step (axis weights and gradients ~150, P2G ~64 x 30,
# G2P ~64 x 30, one 3x3 SVD ~1000, F_E algebra ~200) are an estimate
FP32_PEAK = 152 * 128 * 2 * 2.07e9
FLOPS_PER_PARTICLE_STEP = 4200


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def kernels_per_step(n_colliders, sort_step, key_bits):
    plain = 4  # begin (counters, colliders), compact (+ prefixes), grid, g2p2g
    if not sort_step:
        return plain
    passes = (key_bits + 7) // 8
    # keys, (hist + 3 scan + scatter) per pass, permute, heads, items, prefix
    return plain + 1 + passes * 5 + 4


def reduce_max_ms(total_ms, dist_mod, device):
    """Slowest rank's timed total (all ranks get it)."""
    import torch
    t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
    dist_mod.all_reduce(t, op=dist_mod.ReduceOp.MAX)
    return float(t.item())


def replica_value(world, particles, steps, total_ms):
    """Whole-job particle-steps/s of `world` replicas that each advance
    `particles` particles by `steps` steps, timed by the slowest rank."""
    return world * particles * steps / (total_ms * 1e-3)


def bench_ours(args, local_rank, barrier=lambda: None):
    import torch

    from snow_gb300 import api, native as N, scenes

    torch.cuda.set_device(local_rank)
    t0 = time.time()
    s = scenes.cfg2_two_snowballs(n=args.particles, grid_edge=args.grid)
    gen_s = time.time() - t0
    ctx = api.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    sim = api.SimScene(ctx, s, mode=N.MODE_FAST)
    sim.upload().init()
    n = s.n
    dt = s.dt
    # work split chosen by the autotuner (on real steps of a copy of this
    # scene), or given with --tuning
    if args.tuning:
        si, im, cp = (int(v) for v in args.tuning.split(","))
        sim.set_tuning(si, im, cp)
        tuning = dict(sort_interval=si, items_max=im, ctas_per_sm=cp, steps_taken=0)
    else:
        # tuned on a scratch copy, so the timed run starts from the scene's
        # initial state
        scratch = api.SimScene(ctx, s, mode=N.MODE_FAST).upload().init()
        tb = api.Batch(ctx, [scratch])
        tuning = tb.autotune([dt])
        tb.close()
        scratch.close()
        sim.set_tuning(tuning["sort_interval"], tuning["items_max"], tuning["ctas_per_sm"])
    # the warm-up starts with a binning step (set_tuning re-bins at the next
    # step), so the step graphs with and without binning both exist before
    # the clock starts
    sim.set_tuning(tuning["sort_interval"], tuning["items_max"], tuning["ctas_per_sm"])
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local_rank}")
    for _ in range(args.warmup):
        sim.step(dt, 1)
    ctx.synchronize()
    # the timed window starts at a binning point: its first step re-bins, and
    # so does every sort_interval-th step after it (or every step while
    # particles leave their tiles), so the window carries at least its share
    # of the binning cost
    sim.set_tuning(tuning["sort_interval"], tuning["items_max"], tuning["ctas_per_sm"])
    pt0 = sim.phase_times()
    binnings0, wide0 = pt0["binnings"], pt0["wide"]
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local_rank) as clocks:
        barrier()
        torch.cuda.synchronize()
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                starts[i].record(stream)
            sim.step(dt, 1)
            with torch.cuda.stream(stream):
                ends[i].record(stream)
        torch.cuda.synchronize()
        barrier()
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = sum(step_ms)
    pt1 = sim.phase_times()
    binnings, wide = pt1["binnings"] - binnings0, pt1["wide"] - wide0
    st = sim.stats()
    if st["nonfinite"]:
        raise RuntimeError("non-finite particle state in the timed run")

    # per-kernel device time (eager launches with events around each phase)
    ctx.set_profiling(True)
    sim.phase_times(reset=True)
    prof_steps = max(8, min(args.steps, 32))
    sim.step(dt, prof_steps)
    ph = sim.phase_times(reset=True)
    ctx.set_profiling(False)

    # active nodes: count from a dense download right after a P2G dispatch
    sim.dispatch(N.K_RIGID_ADVANCE, dt)
    sim.dispatch(N.K_P2G, dt)
    g = sim.grid()
    A = int(np.count_nonzero(g["mass"] > 0))
    sim.dispatch(N.K_G_FORCE, dt)
    sim.dispatch(N.K_G2P, dt)
    del g
    # the scene's state after the timed steps and after one more step from
    # it, for the oracle's check of that step at full size (outside every
    # timed region)
    check_states = None
    if not args.no_cpu_baseline:
        y0 = sim.download()
        sim.step(dt, 1)
        check_states = (y0, sim.download())

    # FAST phases: sort (rigid advance + binning), grid (compaction + grid
    # update), g2p2g (the fused particle kernel)
    per = {"sort": ph["sort_ms"], "grid": ph["grid_ms"], "g2p2g": ph["g2p_ms"]}
    per = {k: v / max(ph["steps"], 1) for k, v in per.items()}
    peak, peak_kind = measured_peak_hbm()
    dominant = max(("g2p2g", "grid"), key=lambda k: per[k])
    b = {"g2p2g": BYTES_G2P2G, "grid": BYTES_GRID}[dominant]
    alg_bytes = b[0] * n + b[1] * A
    achieved = alg_bytes / (per[dominant] * 1e-3) / 1e9

    # end to end through the C ABI: upload from host arrays, init, per step
    # one step + a device->host read of the step's bulk statistics, download.
    # inputs and outputs in pinned host memory, filled before the clock starts
    e2e_steps = args.steps

    def pinned(*shape):
        return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()

    hx, hv, hm = pinned(n, 3), pinned(n, 3), pinned(n)
    hx[:], hv[:], hm[:] = s.x, s.v, s.m
    hout = dict(x=pinned(n, 3), v=pinned(n, 3), FE=pinned(n, 3, 3), Jp=pinned(n), volume=pinned(n))
    split = {}
    t1 = time.perf_counter()
    sim2 = api.SimScene(ctx, s, mode=N.MODE_FAST)
    sim2.set_tuning(tuning["sort_interval"], tuning["items_max"], tuning["ctas_per_sm"])
    t = time.perf_counter()
    split["create_ms"] = 1e3 * (t - t1)
    sim2.upload(hx, hv, hm).init()
    ctx.synchronize()
    t2 = time.perf_counter()
    split["upload_init_ms"] = 1e3 * (t2 - t)
    # every step's statistics are read, one step behind, so the GPU does not
    # wait for the host round trip
    for i in range(e2e_steps):
        sim2.step(dt, 1)
        sim2.stats_enqueue(i % 2)
        if i > 0:
            ctx.stats_read((i - 1) % 2)
    ctx.stats_read((e2e_steps - 1) % 2)
    t3 = time.perf_counter()
    split["steps_ms"] = 1e3 * (t3 - t2)
    out = sim2.download(out=hout)
    e2e_s = time.perf_counter() - t1
    split["download_ms"] = 1e3 * (time.perf_counter() - t3)
    h2d = n * (12 + 12 + 4)
    d2h_stats = 8 * 20
    d2h_final = n * (12 + 12 + 36 + 4 + 4)
    sim2.close()
    del out

    key_bits = math.ceil(math.log2(((args.grid + 3) // 4) ** 3 * 64))
    plain_k = kernels_per_step(len(s.colliders), False, key_bits)
    bin_k = kernels_per_step(len(s.colliders), True, key_bits)
    launches = args.steps * plain_k + binnings * (bin_k - plain_k)
    res = dict(total_ms=total_ms, step_ms=step_ms, n=n, A=A, per=per, dominant=dominant, alg_bytes=alg_bytes,
               achieved=achieved, peak=peak, peak_kind=peak_kind, clocks=clocks.summary(), e2e_s=e2e_s,
               e2e_steps=e2e_steps, e2e_split=split, h2d=h2d, d2h=d2h_stats + d2h_final / e2e_steps, launches=launches,
               gen_s=gen_s, stats=st, scene=s, tuning=tuning, check_states=check_states, binnings=binnings,
               wide=wide)
    ctx.close()
    return res


def _events(stream, n):
    import torch
    return [torch.cuda.Event(enable_timing=True) for _ in range(n)]


def bench_batched(args, local_rank, at_scale=False, n_scenes=None, steps=None, tuning=None):
    """Many independent scenes of uneven size: the plain per-scene loop (each
    scene's own step, scenes one after another) against the batched step (one
    launch per phase for all scenes, CUDA graph, autotuned work split). Both
    advance the same scenes by the same steps; the inputs are far larger than
    L2, so no flush is needed.
      default:   64 scenes, 10k-500k particles log-uniform, 64^3-192^3 grids,
                 per-scene E0 and xi (~10M particles, ~1.7 GB of state);
      at_scale:  16 snow blocks of 2M-8M particles dropped onto a sphere
                 collider, 384^3-512^3 grids (~80M particles).
    `tuning` (sort interval, particles per item, CTAs per SM) replaces the
    autotuner, whose ~3,200 steps take minutes on the 80M-particle batch."""
    import torch

    from snow_gb300 import api, scenes

    torch.cuda.set_device(local_rank)
    t0 = time.time()
    n_scenes = n_scenes or args.batch_scenes
    scs = scenes.cfg4_batch(n_scenes=n_scenes) if at_scale else scenes.cfg3_batch(n_scenes=n_scenes)
    gen_s = time.time() - t0
    ntot = sum(s.n for s in scs)
    dts = [s.dt for s in scs]
    ctx = api.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    K, W = steps or args.batch_steps, args.warmup

    def timed(fn):
        ev = _events(stream, 2)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            ev[0].record(stream)
        fn()
        with torch.cuda.stream(stream):
            ev[1].record(stream)
        torch.cuda.synchronize()
        return ev[0].elapsed_time(ev[1])

    plain = [api.SimScene(ctx, s).upload().init() for s in scs]
    for _ in range(W):
        for sim, dt in zip(plain, dts):
            sim.step(dt, 1)

    def plain_loop():
        for _ in range(K):
            for sim, dt in zip(plain, dts):
                sim.step(dt, 1)

    plain_ms = timed(plain_loop)
    # the same loop launching each step's kernels one by one (no CUDA graph)
    ctx.set_graphs(False)
    eager_ms = timed(plain_loop)
    ctx.set_graphs(True)
    check = sorted(range(len(scs)), key=lambda i: scs[i].n)[:4]
    for sim in plain:
        sim.close()
    del plain

    # the work split is tuned on scratch copies (autotuning takes real steps),
    # so the timed batch covers the same steps as the per-scene loop
    if tuning is None:
        scratch = [api.SimScene(ctx, s).upload().init() for s in scs]
        tb = api.Batch(ctx, scratch)
        tuning = tb.autotune(dts)
        tb.close()
        for sim in scratch:
            sim.close()
        del scratch
    else:
        si, im, cp = tuning
        tuning = dict(sort_interval=si, items_max=im, ctas_per_sm=cp, ms_per_step=None, steps_taken=0)
    sims = [api.SimScene(ctx, s).upload().init() for s in scs]
    batch = api.Batch(ctx, sims).set_tuning(tuning["sort_interval"], tuning["items_max"], tuning["ctas_per_sm"])
    for _ in range(W):
        batch.step(1, dts)
    batch_ms = timed(lambda: batch.step(K, dts))
    batch_per_step = []
    for _ in range(3):
        batch_per_step.append(timed(lambda: batch.step(1, dts)))
    diff = 0.0
    # the batched scenes took 3 more steps: compare after re-running plain
    # copies of the check scenes to the same step count
    for i in check:
        p = api.SimScene(ctx, scs[i]).upload().init()
        p.step(dts[i], W + K + 3)
        a, b = p.download(), sims[i].download()
        diff = max(diff, float(np.abs(a["x"] - b["x"]).max()))
        p.close()
    batch.close()
    for sim in sims:
        sim.close()
    ctx.close()
    v_plain = ntot * K / (plain_ms * 1e-3)
    v_eager = ntot * K / (eager_ms * 1e-3)
    v_batch = ntot * K / (batch_ms * 1e-3)
    grids = f"grids {min(s.grid_dim[0] for s in scs)}^3-{max(s.grid_dim[0] for s in scs)}^3"
    if at_scale:
        wl = (f"{len(scs)} snow blocks dropped onto a sphere collider, {ntot} particles in total (2M-8M each), "
              f"{grids}, dt=2e-5")
    else:
        wl = (f"{len(scs)} independent scenes, {ntot} particles in total (10k-500k log-uniform), {grids}, "
              f"E0 ~ U[4.8e4, 1.4e5], xi ~ U[5, 10], dt=1e-4")
    return {"workload": wl,
            "steps": K, "warmup": W, "particles": ntot,
            "plain_per_scene": {"value": v_plain, "unit": UNIT, "ms_per_step": plain_ms / K,
                                "launch": "each scene's step replayed as its own CUDA graph"},
            "plain_per_scene_eager": {"value": v_eager, "unit": UNIT, "ms_per_step": eager_ms / K,
                                      "launch": "each scene's kernels launched one by one"},
            "speedup_vs_eager": v_batch / v_eager,
            "batched": {"value": v_batch, "unit": UNIT, "ms_per_step": batch_ms / K},
            "speedup": v_batch / v_plain,
            "tuning": {k: tuning[k] for k in ("sort_interval", "items_max", "ctas_per_sm", "ms_per_step",
                                              "steps_taken")},
            "max_abs_dx_plain_vs_batched": diff,
            "l2": "inputs larger than L2 (no flush)", "scene_generation_s": gen_s}


def bench_serving(args, local_rank):
    """Continuous batching under Poisson arrivals: jobs of 20k-2M particles
    (log-uniform) and 50-2000 steps (uniform) arrive at `rate` per second for
    `seconds`, are admitted by an HBM budget and batched by the native
    server; the run ends when every job has finished. Job scenes come from a
    pre-generated pool (sampling 2M-particle shapes takes longer than the
    arrival gap) with each arrival's own step count."""
    from snow_gb300 import api, scenes

    rng = np.random.default_rng(0x5EED0005)
    pool = [scenes.serving_job(rng, index=i) for i in range(args.serve_pool)]
    arrivals = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / args.serve_rate)
        if t > args.serve_seconds:
            break
        arrivals.append((t, int(rng.integers(len(pool))), int(rng.integers(50, 2001))))
    srv = api.Server(local_rank, hbm_budget=int(args.serve_budget_gb * (1 << 30)), chunk_steps=16,
                     max_active_particles=args.serve_cap, policy=args.serve_policy)
    t0 = time.perf_counter()
    ids = {}
    for at, j, steps in arrivals:
        now = time.perf_counter() - t0
        if at > now:
            time.sleep(at - now)
        ids[srv.submit(pool[j], steps=steps)] = (j, steps)
    drained = True
    try:
        srv.drain(timeout_s=args.serve_drain_s)
    except Exception:
        drained = False  # report what finished; closing waits for the admitted jobs
    wall = time.perf_counter() - t0
    res = srv.poll(len(ids) + 16)
    stats = srv.stats()
    srv.close()
    ok = [r for r in res if r["status"] == 0]
    lat = sorted(r["latency_s"] for r in ok)
    q = sorted(r["queue_s"] for r in ok)
    svc = sorted(r["service_s"] for r in ok)

    def pct(v, p):
        return float(np.percentile(v, p)) if v else None

    psteps = sum(r["n"] * r["steps"] for r in ok)
    offered = sum(pool[j].n * st for j, st in ids.values()) / args.serve_seconds
    return {"workload": f"Poisson arrivals at {args.serve_rate}/s for {args.serve_seconds} s, jobs of 20k-2M "
                        f"particles (log-uniform, pool of {len(pool)} scenes) x 50-2000 steps, HBM budget "
                        f"{args.serve_budget_gb} GB, chunks of 16 steps, {args.serve_policy} under a cap of "
                        f"{args.serve_cap} particles stepped together",
            "jobs": len(ids), "completed": len(ok), "failed": len(res) - len(ok), "drained": drained,
            "value": psteps / wall, "unit": UNIT, "wall_s": wall, "busy_s": stats["busy_s"],
            "offered_particle_steps_per_s": offered,
            "latency_s": {"p50": pct(lat, 50), "p99": pct(lat, 99), "max": lat[-1] if lat else None},
            "queue_s": {"p50": pct(q, 50), "p99": pct(q, 99)},
            "service_s": {"p50": pct(svc, 50), "p99": pct(svc, 99)}}


def cpu_baseline_port(scene, steps=2):
    """The oracle restatement in the shaders' FP32 arithmetic (FAITHFUL32) on
    all host cores, on the same scene: `steps` full steps after init."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    o = O.OracleSim(scene, mode=O.FAITHFUL32, threads=threads).upload_std140(*scene.std140()).init()
    t = time.perf_counter()
    o.step(n=steps)
    el = time.perf_counter() - t
    return dict(value=scene.n * steps / el, unit=UNIT, cores=threads, kind="port",
                sample=f"{steps} full steps of the same {scene.n}-particle scene, FP32 int32-fixed-point "
                       f"restatement of the shaders, OpenMP over {threads} threads")


def _oracle_from_state(scene, y, threads):
    """The FP64 oracle (EXACT64: no fixed point, no V rounding; OpenMP)
    restarted from a FAST scene's downloaded state y. Only det F_P enters a
    step, so F_P = diag(J_p, 1, 1); densities come from the particles'
    initial volumes. The colliders must be static (their advanced positions
    are not downloaded)."""
    from oracle import oracle as O
    from snow_gb300 import scenes

    n = len(y["x"])
    fp = np.zeros((n, 3, 3))
    fp[:, 0, 0] = y["Jp"]
    fp[:, 1, 1] = fp[:, 2, 2] = 1.0
    s3 = scenes.Scene(**{k: getattr(scene, k) for k in ("grid_pos", "grid_dim", "grid_spacing", "young", "poisson",
                                                        "hardening", "crit_compression", "crit_stretch", "alpha",
                                                        "gravity", "dt")})
    s3.colliders = list(scene.colliders)
    s3.x, s3.v, s3.m = y["x"], y["v"], scene.m.copy()
    rho = np.where(y["volume"] > 0, s3.m.astype(np.float64) / np.maximum(y["volume"], 1e-30), 0.0)
    o = O.OracleSim(s3, mode=O.EXACT64, vround=False, threads=threads)
    return o.upload(FE=y["FE"].astype(np.float64), FP=fp).set_density(rho)


def _inside_colliders(scene, x):
    """Particles at least two cells inside a sphere collider or behind a
    half-plane collider of the scene (where a collider fixes the grid
    velocity at every node of their stencils)."""
    x = np.asarray(x, np.float64)
    h = scene.grid_spacing
    inside = np.zeros(len(x), bool)
    for c in scene.colliders:
        if c.type == 1:
            inside |= np.linalg.norm(x - np.asarray(c.pos), axis=1) < c.radius - 2 * h
        else:
            inside |= (x - np.asarray(c.pos)) @ np.asarray(c.normal) < -2 * h
    return inside


def _check_report(scene, y0, y1, tol, start):
    """One FP64 oracle step from y0 against the GPU's next state y1, with the
    errors of oracle.parity_errors (strict velocity floor 1e-3 m/s, and the
    FLIP-scale bound for particles stopped within the step), the latter's
    maximum also split between particles deep inside a collider and the
    rest."""
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    t = time.perf_counter()
    o = _oracle_from_state(scene, y0, threads)
    flip = o.step_with_flip_scale()
    ref = o.state()
    oracle_s = time.perf_counter() - t
    e = O.parity_errors(y1, ref, flip)
    bound = max(e["max"][k] for k in ("x", "v_flip", "FE", "Jp"))
    dv = np.linalg.norm(np.asarray(y1["v"], np.float64) - ref["v"], axis=1)
    speed = np.linalg.norm(ref["v"], axis=1)
    stopped = int(np.count_nonzero(dv > tol * np.maximum(speed, 1e-3)))
    vf = dv / np.maximum(np.maximum(speed, 1e-3), flip)
    inside = _inside_colliders(scene, y0["x"])
    return {"oracle": "EXACT64 (FP64, OpenMP)", "particles": len(y0["x"]), "steps": 1, "tolerance": tol,
            "start": start, "max": e["max"], "p99": e["p99"], "median": e["median"],
            "within_tolerance": bool(bound <= tol), "strict_v_within_tolerance": bool(e["max"]["v"] <= tol),
            "particles_above_strict_v": stopped, "v_worst": e["v_worst"], "v_flip_worst": e["v_flip_worst"],
            "particles_above_v_flip": int(np.count_nonzero(vf > tol)),
            "v_flip_max_inside_colliders": float(vf[inside].max()) if inside.any() else None,
            "v_flip_max_elsewhere": float(vf[~inside].max()) if (~inside).any() else None,
            "particles_inside_colliders": int(inside.sum()),
            "oracle_s": oracle_s,
            "threads": threads}


def oracle_check(scene, states, tol=1e-5):
    """The FAST path on the full timed workload: one FP64 oracle step,
    restarted from the GPU's state after the timed steps, against the GPU's
    own next step (per-field relative errors; the GPU's advance starts from
    warm SVD frames)."""
    if any(tuple(c.vel) != (0.0, 0.0, 0.0) for c in scene.colliders):
        return None  # moving colliders: their positions after the run are not carried over
    y0, y1 = states
    return _check_report(scene, y0, y1, tol,
                         "the workload's state after the timed steps (GPU state, warm SVD frames)")


def oracle_check_batched_at_scale(local_rank, n=2_097_152, edge=384, warm=3, tol=1e-5, gap=-0.01):
    """The batched path at the size of the 16-scene batch's scenes: a snow
    block of n particles on a 384^3 grid moving down at 2 m/s onto a static
    sphere collider, stepped by snow_batch_step together with a small scene,
    `warm` batched steps and then one more, which the FP64 oracle repeats
    from the GPU's state. gap < 0 sinks the sphere's top that far into the
    block (its bottom layer starts inside the collider, where the grid stops
    it); gap = 0 starts the block touching the sphere."""
    import torch

    from snow_gb300 import api, scenes

    torch.cuda.set_device(local_rank)
    t0 = time.perf_counter()
    big = scenes.snow_block_on_sphere(0x5EED0014, n, edge, gap=gap, v0=(0.0, -2.0, 0.0))
    small = scenes.small_scene(n=20000, grid_edge=64, seed=0x5EED0015, v0=(1.0, -2.0, 0.5))
    gen_s = time.perf_counter() - t0
    ctx = api.Context(local_rank)
    sims = [api.SimScene(ctx, s).upload().init() for s in (big, small)]
    batch = api.Batch(ctx, sims)
    dts = [big.dt, small.dt]
    batch.step(warm, dts)
    y0 = sims[0].download()
    batch.step(1, dts)
    y1 = sims[0].download()
    batch.close()
    for g in sims:
        g.close()
    ctx.close()
    r = _check_report(big, y0, y1, tol, f"after {warm} batched steps (GPU state, warm SVD frames)")
    where = (f"bottom layer inside a static sphere collider (its top {-gap:g} m into the block)" if gap < 0 else
             "touching a static sphere collider")
    r.update(workload=f"snow block of {big.n} particles on a {edge}^3 grid, {where} (radius "
                      f"{big.colliders[-1].radius:.4f}), moving at 2 m/s, stepped by snow_batch_step beside a "
                      f"20,000-particle scene", scene_generation_s=gen_s)
    return r


def bench_reference(args):
    """The reference's compute shaders compiled as C++ (oracle/_ref), or the
    oracle's FP32 restatement where they are not built, on all host cores:
    every warm-up and timed step advances the workload's whole scene (all
    particles, the dense grid), as ExplicitTimeUpdate::update does."""
    from oracle import oracle as O
    from snow_gb300 import scenes

    threads = os.cpu_count() or 1
    s = scenes.cfg2_two_snowballs(n=args.particles, grid_edge=args.grid)
    kind = "reference" if O.ref_lib() is not None else "port"
    if kind == "reference":
        sim = O.RefSim(s, threads=threads).upload_std140(*s.std140()).init()
        stepper = lambda: sim.update()
    else:
        sim = O.OracleSim(s, mode=O.FAITHFUL32, threads=threads).upload_std140(*s.std140()).init()
        stepper = lambda: sim.step()
    for _ in range(args.warmup):
        stepper()
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        stepper()
        times.append(time.perf_counter() - t)
    total = sum(times)
    value = s.n * args.steps / total
    what = ("the reference's compute shaders compiled as C++" if kind == "reference"
            else "the oracle's FP32 restatement of the shaders")
    sample_desc = (f"the whole {s.n}-particle scene ({args.grid}^3 grid) every step: {args.warmup} warm-up + "
                   f"{args.steps} timed steps of {what}, OpenMP over {threads} threads; "
                   f"median {statistics.median(times):.3f} s per step")
    return dict(value=value, unit=UNIT, cores=threads, kind=kind, sample=sample_desc, total_s=total,
                ms_per_step=1e3 * total / args.steps)


def bench_implicit(args, local_rank):
    """The semi-implicit update (absent from the reference, whose
    SemiImplicitTimeUpdate is empty) on the headline's geometry with a stiff
    material, a long step and a rough velocity field (seeded 1 m/s jitter on
    top of the +-5 m/s collision), where the CR solve iterates. The same scene
    stepped explicitly is timed beside it. L2 flushed before every timed step."""
    import torch

    from snow_gb300 import api, scenes

    torch.cuda.set_device(local_rank)
    young, dt, jitter = 1.4e7, 5e-4, 1.0

    def scene(beta):
        s = scenes.cfg2_two_snowballs(n=args.particles, grid_edge=args.grid)
        s.young, s.dt = young, dt
        rng = np.random.default_rng(0x5EED0006)
        s.v = (s.v + rng.normal(scale=jitter, size=s.v.shape)).astype(np.float32)
        s.implicit_beta, s.implicit_tolerance, s.implicit_max_iters = beta, 1e-5, 50
        return s

    ctx = api.Context(local_rank)
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local_rank}")
    out = {}
    for beta in (1.0, 0.0):
        s = scene(beta)
        sim = api.SimScene(ctx, s).upload().init().set_tuning(2, 256, 2)
        for _ in range(args.warmup):
            sim.step(dt, 1)
        ctx.synchronize()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        with ClockSampler(local_rank) as clocks:
            torch.cuda.synchronize()
            for i in range(args.steps):
                with torch.cuda.stream(stream):
                    flush.zero_()
                    starts[i].record(stream)
                sim.step(dt, 1)
                with torch.cuda.stream(stream):
                    ends[i].record(stream)
            torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / args.steps
        r = dict(ms_per_step=ms, value=s.n / (ms * 1e-3), clocks=clocks.summary())
        if beta > 0:
            # CR iterations of the steps that follow
            its = []
            for _ in range(4):
                sim.step(dt, 1)
                rep = sim.solver_report()
                its.append(rep["iterations"])
            r.update(iterations=its, residual=rep["residual"], initial_residual=rep["initial_residual"])
            # the same steps launched kernel by kernel (no graph): the host
            # launches every CR iteration up to the cap, the finished ones
            # return at once; this is also the pass in which a profiler sees
            # the solve's kernels (a graph runs them inside a conditional node)
            ctx.set_profiling(True)
            sim.phase_times(reset=True)
            sim.step(dt, 4)
            ph = sim.phase_times(reset=True)
            ctx.set_profiling(False)
            r.update(eager_ms=ph["total_ms"] / ph["steps"])
        st = sim.stats()
        if st["nonfinite"]:
            raise RuntimeError("non-finite particle state in the semi-implicit run")
        out[beta] = r
        sim.close()
    ctx.close()
    imp, exp = out[1.0], out[0.0]
    return {"metric": METRIC, "value": imp["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": imp["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattice)",
            "config": {"workload": f"semi-implicit update (beta 1, CR tolerance 1e-5, cap 50): two snowballs "
                                   f"at +-5 m/s plus seeded {jitter} m/s velocity jitter, {args.particles} "
                                   f"particles, {args.grid}^3 grid, E={young:g}, dt={dt:g}, FAST mode",
                       "particles": args.particles, "grid": f"{args.grid}^3", "dt": dt,
                       "l2": "flushed (256 MB write) before every timed step", "tuning": "2,256,2"},
            "cr_iterations_per_step": imp["iterations"], "cr_residual": imp["residual"],
            "cr_initial_residual": imp["initial_residual"], "eager_ms_per_step": imp["eager_ms"],
            "explicit_same_scene": {"value": exp["value"], "ms_per_step": exp["ms_per_step"]},
            "clocks": imp["clocks"]}


def workload_config(args):
    return {"workload": f"two snowballs colliding head-on at +-5 m/s, {args.particles} particles (8 per cell), "
                        f"{args.grid}^3 grid, h=1/{args.grid}, dt=2e-5, FAST mode",
            "particles": args.particles, "grid": f"{args.grid}^3", "dt": 2e-5, "mode": "fast (FP32)",
            "l2": "flushed (256 MB write) before every timed step", "parallelism": "replicas"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=64)
    ap.add_argument("--warmup", type=int, default=8)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--particles", type=int, default=1 << 20)
    ap.add_argument("--grid", type=int, default=256)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-scale-check", action="store_true",
                    help="skip the oracle check of a batched step of a 2M-particle, 384^3 scene")
    ap.add_argument("--tuning", default="", help="SORT_INTERVAL,ITEMS_MAX,CTAS_PER_SM instead of autotuning")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=16)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--no-batched-at-scale", action="store_true",
                    help="skip the 16-scene batch of 2M-8M particles (384^3-512^3) in the default run")
    ap.add_argument("--serve-rate", type=float, default=20.0)
    ap.add_argument("--serve-pool", type=int, default=24)
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-drain-s", type=float, default=300.0)
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--serve-policy", default="srpt", choices=["fifo", "srpt"])
    ap.add_argument("--serve-cap", type=int, default=4 << 20, help="particles stepped together (0 = all)")
    ap.add_argument("--workload", default="default", choices=["default", "batch16", "implicit"],
                    help="batch16: only the 16-scene batch at scale (2M-8M particles each); implicit: the "
                         "semi-implicit update on the headline geometry; one JSON line each")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local_rank = rank_info()

    if args.impl == "reference":
        if rank != 0:
            return 0
        r = bench_reference(args)
        line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+i32", "data": "synthetic",
                "config": dict(workload_config(args), mode="the reference compute shaders compiled as C++ (FP32 + int32 fixed point)", l2="n/a (host)"), "impl": "reference",
                "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": r["kind"],
                                 "sample": r["sample"]},
                "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    if args.workload == "implicit":
        if rank != 0:
            return 0
        if "--steps" not in sys.argv:
            args.steps = 16
        print(json.dumps(bench_implicit(args, local_rank)))
        return 0

    if args.workload == "batch16":
        if rank != 0:
            return 0
        if "--batch-scenes" not in sys.argv:
            args.batch_scenes = 16
        if "--batch-steps" not in sys.argv:
            args.batch_steps = 8
        r = bench_batched(args, local_rank, at_scale=True)
        b = r["batched"]
        line = {"metric": METRIC, "value": b["value"], "unit": UNIT, "n_gpus": 1, "steps": r["steps"],
                "warmup": r["warmup"], "ms_per_step": b["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattice)",
                "config": {"workload": r["workload"], "particles": r["particles"], "mode": "fast (FP32)",
                           "l2": r["l2"], "parallelism": "replicas", "tuning": r["tuning"]},
                "plain_per_scene": r["plain_per_scene"], "speedup": r["speedup"],
                "plain_per_scene_eager": r["plain_per_scene_eager"], "speedup_vs_eager": r["speedup_vs_eager"],
                "max_abs_dx_plain_vs_batched": r["max_abs_dx_plain_vs_batched"],
                "scene_generation_s": r["scene_generation_s"]}
        print(json.dumps(line))
        return 0

    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    res = bench_ours(args, local_rank, barrier=dist.barrier if dist is not None else (lambda: None))
    total_ms = res["total_ms"]
    if dist is not None:
        total_ms = reduce_max_ms(total_ms, dist, f"cuda:{local_rank}")
        dist.barrier()
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    n = res["n"]
    value = replica_value(world, n, args.steps, total_ms)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattice)",
        "config": dict(workload_config(args), tuning={k: res["tuning"][k] for k in
                                                       ("sort_interval", "items_max", "ctas_per_sm")}),
        "roofline": {"bound": "hbm", "kernel": res["dominant"], "achieved": res["achieved"],
                     "peak": res["peak"], "unit": "GB/s", "frac": res["achieved"] / res["peak"],
                     "peak_source": res["peak_kind"],
                     "traffic": (TRAFFIC_MEASURED.get((args.particles, args.grid))
                                 if res["dominant"] == "g2p2g" else None),
                     "traffic_source": TRAFFIC_SOURCE,
                     "algorithmic_bytes_per_launch": res["alg_bytes"], "active_nodes": res["A"]},
        "issue_roofline": ({"achieved": INSTRUCTIONS_MEASURED[(args.particles, args.grid)] /
                                        (res["per"]["g2p2g"] * 1e-3),
                            "peak": ISSUE_PEAK, "unit": "warp-instructions/s",
                            "frac": INSTRUCTIONS_MEASURED[(args.particles, args.grid)] /
                                    (res["per"]["g2p2g"] * 1e-3) / ISSUE_PEAK,
                            "kernel": "g2p2g", "instructions_per_launch": INSTRUCTIONS_MEASURED[
                                (args.particles, args.grid)]}
                           if (args.particles, args.grid) in INSTRUCTIONS_MEASURED else None),
        "flop_roofline": {"achieved": FLOPS_PER_PARTICLE_STEP * n / (res["per"]["g2p2g"] * 1e-3) / 1e12,
                          "peak": FP32_PEAK / 1e12, "unit": "TFLOP/s (FP32)", "kernel": "g2p2g",
                          "frac": FLOPS_PER_PARTICLE_STEP * n / (res["per"]["g2p2g"] * 1e-3) / FP32_PEAK,
                          "flops_per_particle_step": FLOPS_PER_PARTICLE_STEP,
                          "note": "algorithmic estimate of the flops, not counted ones"},
        "phase_ms": res["per"],
        "clocks": res["clocks"],
        "e2e": {"value": n * res["e2e_steps"] / res["e2e_s"], "unit": UNIT,
                "h2d_bytes_per_step": res["h2d"] / res["e2e_steps"], "d2h_bytes_per_step": res["d2h"],
                "note": "scene create + upload from pinned host memory + init + per step (step + a read of its "
                        "statistics, one step behind) + download into pinned host memory, through the C ABI",
                "split_ms": res["e2e_split"]},
        "gpu_launches": res["launches"],
        "wide_particles": {"value": res["wide"], "steps": args.steps,
                           "note": "particles whose P2G contributions outgrew the fixed-point scales' fast range "
                                   "in the timed steps (scattered with int64 contributions)"},
        "step_ms_p50": statistics.median(res["step_ms"]), "step_ms_max": max(res["step_ms"]),
    }
    side = world == 1  # the side legs run on a single GPU only (a replica run times the headline alone)
    if side and not args.no_batched:
        line["batched"] = bench_batched(args, local_rank)
    if side and not args.no_batched_at_scale:
        line["batched_at_scale"] = bench_batched(args, local_rank, at_scale=True, n_scenes=16, steps=8,
                                                 tuning=(8, 256, 2))
    if side and not args.no_serving:
        line["serving"] = bench_serving(args, local_rank)
    if side and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_port(res["scene"], steps=2)
        # the same leg checks the timed workload's next step against the
        # oracle, and one batched step at the size of the 16-scene batch's
        # scenes
        if res["check_states"] is not None:
            line["oracle_check"] = oracle_check(res["scene"], res["check_states"])
        if not args.no_scale_check:
            line["oracle_check_batched_at_scale"] = oracle_check_batched_at_scale(local_rank)
            line["oracle_check_batched_at_scale_contact"] = oracle_check_batched_at_scale(local_rank, gap=0.0)
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
