"""Python host API over the C ABI, shaped like the reference's simulation
layer:

  reference (src/snow/simulation/)              here
  ---------------------------------------------------------------------------
  TimeUpdate(PhysicalScene&&)                   ExplicitTimeUpdate(scene, ...)
  ExplicitTimeUpdate::init()  (explicittimeupdate.cpp:4-34)   .init()
  ExplicitTimeUpdate::update(double dt) (:36-63)              .update(dt)
  SemiImplicitTimeUpdate (empty in the reference:  SemiImplicitTimeUpdate(scene, beta=...)
    semiimplicittimeupdate.cpp:3-5)
  MPMPhysicEngine(unique_ptr<TimeUpdate>)       MPMPhysicEngine(time_update)
  MPMPhysicEngine::init() / update(dt)          .init() / .update(dt)

``scene`` is a snow_gb300.scenes.Scene (the PhysicalScene: particles, grid,
colliders, material). Errors raise SnowError with the library's status.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import List, Optional, Sequence

import numpy as np

from . import native as N
from .scenes import Scene


class Context:
    """One GPU, one CUDA stream, an optional HBM budget in bytes."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self.L = N.load()
        h = C.c_void_p()
        st = self.L.snow_ctx_create(int(device), int(hbm_budget), C.byref(h))
        if st != N.SNOW_OK:
            raise N.SnowError(st, "snow_ctx_create failed")
        self.h = h

    def check(self, st):
        if st != N.SNOW_OK:
            raise N.SnowError(st, self.L.snow_last_error(self.h).decode())

    def synchronize(self):
        self.check(self.L.snow_ctx_synchronize(self.h))

    def set_profiling(self, on: bool):
        self.check(self.L.snow_ctx_set_profiling(self.h, int(bool(on))))

    def stats_read(self, slot: int = 0) -> dict:
        s = N.SnowStats()
        self.check(self.L.snow_ctx_stats_read(self.h, int(slot), C.byref(s)))
        return _stats_dict(s)

    def set_graphs(self, on: bool):
        """False: single-scene steps launch kernels one by one (no CUDA graph)."""
        self.check(self.L.snow_ctx_set_graphs(self.h, int(bool(on))))

    @property
    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        return int(self.L.snow_ctx_stream(self.h) or 0)

    @property
    def bytes_in_use(self) -> int:
        return int(self.L.snow_ctx_bytes_in_use(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.L.snow_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def params_for(scene: Scene, mode: int, sort_interval: int = 0) -> N.SnowParams:
    p = N.SnowParams()
    for k in range(3):
        p.grid_pos[k] = scene.grid_pos[k]
        p.grid_dim[k] = int(scene.grid_dim[k])
        p.gravity[k] = scene.gravity[k]
    p.grid_spacing = scene.grid_spacing
    p.young, p.poisson, p.hardening = scene.young, scene.poisson, scene.hardening
    p.crit_compression, p.crit_stretch = scene.crit_compression, scene.crit_stretch
    p.alpha = scene.alpha
    p.mode = int(mode)
    p.sort_interval = int(sort_interval)
    p.implicit_beta = float(getattr(scene, "implicit_beta", 0.0))
    p.implicit_tolerance = float(getattr(scene, "implicit_tolerance", 0.0))
    p.implicit_max_iters = int(getattr(scene, "implicit_max_iters", 0))
    return p


def colliders_for(scene: Scene):
    n = len(scene.colliders)
    arr = (N.SnowCollider * max(1, n))()
    for i, c in enumerate(scene.colliders):
        for k in range(3):
            arr[i].pos[k] = c.pos[k]
            arr[i].vel[k] = c.vel[k]
            arr[i].normal[k] = c.normal[k]
        arr[i].type = int(c.type)
        arr[i].radius = c.radius
        arr[i].friction = c.friction
    return arr, n


class SimScene:
    """A scene resident on the GPU."""

    def __init__(self, ctx: Context, scene: Scene, mode: int = N.MODE_FAST, capacity: int = 0,
                 sort_interval: int = 0):
        self.ctx, self.L, self.scene, self.mode = ctx, ctx.L, scene, mode
        self.params = params_for(scene, mode, sort_interval)
        arr, n = colliders_for(scene)
        self._coll = arr
        h = C.c_void_p()
        ctx.check(self.L.snow_scene_create(ctx.h, C.byref(self.params), arr, n, int(capacity), C.byref(h)))
        self.h = h
        self.n = 0

    def close(self):
        # A destroyed context has already released its scenes.
        if getattr(self, "h", None) and getattr(self.ctx, "h", None):
            self.L.snow_scene_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- data in ---------------------------------------------------------
    def upload(self, x=None, v=None, m=None, FE=None, FP=None):
        s = self.scene
        x = np.ascontiguousarray(s.x if x is None else x, np.float32)
        v = np.ascontiguousarray(s.v if v is None else v, np.float32)
        m = np.ascontiguousarray(s.m if m is None else m, np.float32)
        fe = None if FE is None else np.ascontiguousarray(FE, np.float32)
        fp = None if FP is None else np.ascontiguousarray(FP, np.float32)
        self.n = len(x)
        self.ctx.check(self.L.snow_scene_upload(self.h, N.ptr(x), N.ptr(v), N.ptr(m), N.ptr(fe), N.ptr(fp), self.n))
        return self

    def upload_std140(self, pxm, pv, pfe, pfp):
        a = [np.ascontiguousarray(pxm, np.float32), np.ascontiguousarray(pv, np.int32),
             np.ascontiguousarray(pfe, np.float32), np.ascontiguousarray(pfp, np.float32)]
        self.n = len(a[0])
        self.ctx.check(self.L.snow_scene_upload_std140(self.h, N.ptr(a[0]), N.ptr(a[1], C.c_int32), N.ptr(a[2]),
                                                       N.ptr(a[3]), self.n))
        return self

    def set_volume(self, volume):
        vol = np.ascontiguousarray(volume, np.float32)
        self.ctx.check(self.L.snow_scene_set_volume(self.h, N.ptr(vol), len(vol)))
        return self

    # -- the step ----------------------------------------------------------
    def init(self):
        self.ctx.check(self.L.snow_scene_init(self.h))
        return self

    def step(self, dt: Optional[float] = None, n: int = 1):
        self.ctx.check(self.L.snow_scene_step(self.h, float(self.scene.dt if dt is None else dt), int(n)))
        return self

    def dispatch(self, kernel: int, dt: Optional[float] = None):
        self.ctx.check(self.L.snow_dispatch(self.h, int(kernel), float(self.scene.dt if dt is None else dt)))
        return self

    # -- data out ----------------------------------------------------------
    def download(self, fp: bool = False, out: Optional[dict] = None):
        """Particle state in upload order. `out` may hold preallocated
        float32 arrays x, v (N x 3), FE (N x 3 x 3), Jp, volume (N) -- e.g.
        views of pinned host memory -- which are filled and returned."""
        n = self.n
        if out is not None:
            x, v, fe, jp, vol = out["x"], out["v"], out["FE"], out["Jp"], out["volume"]
            for a in (x, v, fe, jp, vol):
                if a.dtype != np.float32 or not a.flags.c_contiguous or a.size * 4 != a.nbytes or len(a) != n:
                    raise ValueError("download: out arrays must be C-contiguous float32 with N rows")
        else:
            x, v = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
            fe, jp, vol = np.zeros((n, 3, 3), np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32)
        fpa = np.zeros((n, 3, 3), np.float32) if fp else None
        self.ctx.check(self.L.snow_scene_download(self.h, N.ptr(x), N.ptr(v), N.ptr(fe), N.ptr(fpa), N.ptr(jp),
                                                  N.ptr(vol)))
        out = dict(x=x, v=v, FE=fe, Jp=jp, volume=vol)
        if fp:
            out["FP"] = fpa
        return out

    def download_std140(self):
        n = self.n
        pxm, pv = np.zeros((n, 4), np.float32), np.zeros((n, 4), np.int32)
        fe, fp = np.zeros((n, 16), np.float32), np.zeros((n, 16), np.float32)
        self.ctx.check(self.L.snow_scene_download_std140(self.h, N.ptr(pxm), N.ptr(pv, C.c_int32), N.ptr(fe),
                                                         N.ptr(fp)))
        return pxm, pv, fe, fp

    def grid(self):
        G = int(np.prod(self.scene.grid_dim))
        mass, mom = np.zeros(G, np.float32), np.zeros((G, 3), np.float32)
        force, vstar = np.zeros((G, 3), np.float32), np.zeros((G, 3), np.float32)
        self.ctx.check(self.L.snow_scene_download_grid(self.h, N.ptr(mass), N.ptr(mom), N.ptr(force), N.ptr(vstar)))
        return dict(mass=mass, mom=mom, force=force, vstar=vstar)

    def colliders(self):
        n = max(1, len(self.scene.colliders))
        arr = (N.SnowCollider * n)()
        self.ctx.check(self.L.snow_scene_download_colliders(self.h, arr))
        return np.array([[arr[i].pos[k] for k in range(3)] for i in range(len(self.scene.colliders))], np.float32)

    def stats(self) -> dict:
        s = N.SnowStats()
        self.ctx.check(self.L.snow_scene_stats(self.h, C.byref(s)))
        return _stats_dict(s)

    def set_tuning(self, sort_interval: int, items_max: int = 256, ctas_per_sm: int = 2):
        t = N.SnowTuning(int(sort_interval), int(items_max), int(ctas_per_sm), 0, 0.0)
        self.ctx.check(self.L.snow_scene_set_tuning(self.h, C.byref(t)))
        return self

    def stats_enqueue(self, slot: int = 0):
        """Queues this scene's statistics into a context slot; read them with
        Context.stats_read(slot) (a loop can read step i while i + 1 runs)."""
        self.ctx.check(self.L.snow_scene_stats_enqueue(self.h, int(slot)))
        return self

    def cell_keys(self):
        n = self.n
        keys, perm = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        self.ctx.check(self.L.snow_scene_cell_keys(self.h, N.ptr(keys, C.c_uint32), N.ptr(perm, C.c_uint32)))
        return keys, perm

    def phase_times(self, reset: bool = False) -> dict:
        t = N.SnowPhaseTimes()
        self.ctx.check(self.L.snow_scene_phase_times(self.h, C.byref(t), int(bool(reset))))
        return dict(sort_ms=t.sort_ms, p2g_ms=t.p2g_ms, grid_ms=t.grid_ms, g2p_ms=t.g2p_ms,
                    solve_ms=t.other_ms, total_ms=t.total_ms, steps=int(t.steps), binnings=int(t.binnings),
                    wide=int(t.wide))

    def check(self):
        """Waits for the queued work; raises SnowError for a condition the
        device counted (timeout, pool overflow, non-finite state)."""
        self.ctx.check(self.L.snow_scene_check(self.h))
        return self

    def set_wait_limit(self, wait_ns: int = 0, unsent_bytes: int = 0):
        """Bounded copy waits of the FAST kernels (snow_scene_set_wait_limit)."""
        self.ctx.check(self.L.snow_scene_set_wait_limit(self.h, int(wait_ns), int(unsent_bytes)))
        return self

    def solver_report(self) -> dict:
        """The last step's semi-implicit solve (iterations, relative residuals)."""
        r = N.SnowSolverReport()
        self.ctx.check(self.L.snow_scene_solver_report(self.h, C.byref(r)))
        return dict(iterations=r.iterations, max_iters=r.max_iters, residual=r.residual,
                    initial_residual=r.initial_residual)


class Batch:
    """Many FAST scenes advanced together: one launch per phase for all of
    them, the step captured as a CUDA graph."""

    def __init__(self, ctx: Context, sims: Sequence[SimScene]):
        self.ctx, self.L, self.sims = ctx, ctx.L, list(sims)
        hs = (C.c_void_p * len(self.sims))(*[s.h.value for s in self.sims])
        h = C.c_void_p()
        ctx.check(self.L.snow_batch_create(ctx.h, hs, len(self.sims), C.byref(h)))
        self.h = h

    def step(self, n: int = 1, dt: Optional[Sequence[float]] = None):
        dts = None
        if dt is not None:
            dts = (C.c_double * len(self.sims))(*[float(d) for d in dt])
        self.ctx.check(self.L.snow_batch_step(self.h, dts, int(n)))
        return self

    def set_tuning(self, sort_interval: int, items_max: int, ctas_per_sm: int):
        t = N.SnowTuning(int(sort_interval), int(items_max), int(ctas_per_sm), 0, 0.0)
        self.ctx.check(self.L.snow_batch_set_tuning(self.h, C.byref(t)))
        return self

    def signature(self) -> str:
        """Key of the tuning cache: scene count, particle total (2 significant
        digits) and the set of grid sizes."""
        n = sum(s.n for s in self.sims)
        grids = sorted({tuple(int(g) for g in s.scene.grid_dim) for s in self.sims})
        return f"{len(self.sims)}|{float(f'{n:.2g}'):.0f}|" + ",".join("x".join(map(str, g)) for g in grids)

    def autotune(self, dt: Optional[Sequence[float]] = None, cache: Optional[str] = None) -> dict:
        """Chooses sort interval, particles per work item and CTAs per SM by
        timing real steps of the batch (they advance the scenes), or applies
        the choice kept in the JSON file `cache` for this batch's signature."""
        import json
        import os
        key = self.signature()
        table = {}
        if cache and os.path.exists(cache):
            with open(cache) as f:
                table = json.load(f)
            if key in table:
                c = table[key]
                self.set_tuning(c["sort_interval"], c["items_max"], c["ctas_per_sm"])
                return dict(c, steps_taken=0, cached=True)
        dts = None
        if dt is not None:
            dts = (C.c_double * len(self.sims))(*[float(d) for d in dt])
        t = N.SnowTuning()
        self.ctx.check(self.L.snow_batch_autotune(self.h, dts, C.byref(t)))
        out = dict(sort_interval=t.sort_interval, items_max=t.items_max, ctas_per_sm=t.ctas_per_sm,
                   ms_per_step=t.ms_per_step)
        if cache:
            table[key] = out
            tmp = cache + ".tmp"
            with open(tmp, "w") as f:
                json.dump(table, f, indent=1, sort_keys=True)
            os.replace(tmp, cache)
        return dict(out, steps_taken=t.steps_taken, cached=False)

    def close(self):
        # Destroying the context or any member scene releases the batch too.
        alive = getattr(self.ctx, "h", None) and all(getattr(s, "h", None) for s in self.sims)
        if getattr(self, "h", None) and alive:
            self.L.snow_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _stats_dict(s: N.SnowStats) -> dict:
    return dict(mass=s.mass, momentum=np.array(s.momentum[:]), kinetic_energy=s.kinetic_energy,
                center_of_mass=np.array(s.center_of_mass[:]), bbox_min=np.array(s.bbox_min[:]),
                bbox_max=np.array(s.bbox_max[:]), mean_jp=s.mean_jp, nonfinite=int(s.nonfinite), n=int(s.n))


class Server:
    """Continuous-batching simulation server (snow_server_* in the C ABI): a
    native worker thread admits submitted jobs while their device footprint
    fits the HBM budget and advances admitted jobs together, chunk by chunk;
    jobs join and leave at chunk boundaries. With `max_active_particles`,
    only that many particles step per chunk, chosen in arrival order
    ("fifo") or least remaining work first ("srpt")."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, max_active: int = 0, chunk_steps: int = 0,
                 max_active_particles: int = 0, policy: str = "fifo"):
        self.L = N.load()
        pol = {"fifo": N.SERVE_FIFO, "srpt": N.SERVE_SRPT}[policy]
        cfg = N.SnowServerConfig(int(device), int(hbm_budget), int(max_active), int(chunk_steps),
                                 int(max_active_particles), pol)
        h = C.c_void_p()
        st = self.L.snow_server_create(C.byref(cfg), C.byref(h))
        if st != N.SNOW_OK:
            raise N.SnowError(st, "snow_server_create failed")
        self.h = h

    def submit(self, scene: Scene, steps: Optional[int] = None, dt: Optional[float] = None,
               keep_state: bool = False, sort_interval: int = 0) -> int:
        """Queues a job (FAST mode); returns its id. The arrays are copied."""
        p = params_for(scene, N.MODE_FAST, sort_interval)
        coll, nc = colliders_for(scene)
        x = np.ascontiguousarray(scene.x, dtype=np.float32)
        v = np.ascontiguousarray(scene.v, dtype=np.float32)
        m = np.ascontiguousarray(scene.m, dtype=np.float32)
        d = N.SnowJobDesc(C.pointer(p), C.cast(coll, C.POINTER(N.SnowCollider)), nc, N.ptr(x), N.ptr(v), N.ptr(m), len(m),
                          int(steps if steps is not None else scene.steps),
                          float(dt if dt is not None else scene.dt), int(bool(keep_state)))
        jid = C.c_uint64()
        st = self.L.snow_server_submit(self.h, C.byref(d), C.byref(jid))
        if st != N.SNOW_OK:
            raise N.SnowError(st, "snow_server_submit failed")
        return int(jid.value)

    def poll(self, max_results: int = 256) -> List[dict]:
        out = (N.SnowJobResult * max_results)()
        n = C.c_int()
        st = self.L.snow_server_poll(self.h, out, max_results, C.byref(n))
        if st != N.SNOW_OK:
            raise N.SnowError(st, "snow_server_poll failed")
        return [dict(id=int(r.id), status=int(r.status), n=int(r.n), steps=int(r.steps), queue_s=r.queue_s,
                     service_s=r.service_s, latency_s=r.latency_s, stats=_stats_dict(r.stats))
                for r in out[:n.value]]

    def fetch(self, job_id: int, n: int) -> dict:
        """Final state of a finished job submitted with keep_state."""
        x = np.empty((n, 3), np.float32)
        v = np.empty((n, 3), np.float32)
        fe = np.empty((n, 3, 3), np.float32)
        jp = np.empty(n, np.float32)
        st = self.L.snow_server_fetch(self.h, int(job_id), N.ptr(x), N.ptr(v), N.ptr(fe), N.ptr(jp))
        if st != N.SNOW_OK:
            raise N.SnowError(st, "snow_server_fetch failed")
        return dict(x=x, v=v, FE=fe, Jp=jp)

    def stats(self) -> dict:
        r = N.SnowServerStats()
        st = self.L.snow_server_stats(self.h, C.byref(r))
        if st != N.SNOW_OK:
            raise N.SnowError(st, "snow_server_stats failed")
        return {k: getattr(r, k) for k, _ in N.SnowServerStats._fields_}

    def drain(self, timeout_s: float = 600.0):
        st = self.L.snow_server_drain(self.h, float(timeout_s))
        if st != N.SNOW_OK:
            raise N.SnowError(st, "snow_server_drain: jobs still running")

    def close(self):
        if getattr(self, "h", None):
            self.L.snow_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ExplicitTimeUpdate:
    """Drop-in for the reference's ExplicitTimeUpdate : TimeUpdate."""

    def __init__(self, physical_scene: Scene, ctx: Optional[Context] = None, mode: int = N.MODE_FAST):
        self.scene = physical_scene
        self.ctx = ctx or Context()
        self.sim = SimScene(self.ctx, physical_scene, mode=mode)

    def init(self):
        self.sim.upload().init()

    def update(self, dt: float):
        self.sim.step(dt, 1)


class SemiImplicitTimeUpdate(ExplicitTimeUpdate):
    """The reference's SemiImplicitTimeUpdate : TimeUpdate
    (src/snow/simulation/timeUpdate/semiimplicittimeupdate.hpp:6-12), whose
    init/update are empty there (semiimplicittimeupdate.cpp:3-5), carried out:
    each update solves (M + beta dt^2 K) v = M v* on the grid before G2P
    (Stomakhin et al. 2013, eq. 9). FAST mode."""

    def __init__(self, physical_scene: Scene, ctx: Optional[Context] = None, beta: float = 1.0,
                 tolerance: float = 0.0, max_iters: int = 0):
        scene = dataclasses.replace(physical_scene, implicit_beta=float(beta),
                                    implicit_tolerance=float(tolerance), implicit_max_iters=int(max_iters))
        super().__init__(scene, ctx=ctx, mode=N.MODE_FAST)


class MPMPhysicEngine:
    """Drop-in for the reference's MPMPhysicEngine (MPMPhysicEngine.cpp:3-7)."""

    def __init__(self, time_update: ExplicitTimeUpdate):
        self.integration = time_update

    def init(self) -> bool:
        self.integration.init()
        return True

    def update(self, dt: float):
        self.integration.update(dt)
