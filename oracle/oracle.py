"""ORACLE / TEST INFRASTRUCTURE ONLY -- ctypes front end to the CPU checkers.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module. It never stands in for the product.

  OracleSim  : this project's restatement (snow_oracle.cpp), modes
               FAITHFUL32 / EXACT64 / EXACT32 / FAITHFUL64.
  RefSim     : the reference's own compute shaders compiled as C++
               (oracle/_ref, see ref_translate.py); available where the
               reference tree or its translated sources are present.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

FAITHFUL32, EXACT64, EXACT32, FAITHFUL64 = 0, 1, 2, 3
PH_RIGID, PH_RESET, PH_P2G, PH_GRID, PH_G2P, PH_ADVANCE, PH_GMASS, PH_PVOLUME, PH_IMPLICIT = range(9)

_lib = None
_ref = None


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


def lib():
    global _lib
    if _lib is None:
        so = _build.build_oracle()
        _lib = C.CDLL(so)
        dp, fp, ip, up = C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int), C.POINTER(C.c_uint32)
        _lib.oracle_create.restype = C.c_void_p
        _lib.oracle_create.argtypes = [C.c_void_p, C.c_int]
        _lib.oracle_destroy.argtypes = [C.c_void_p]
        _lib.oracle_upload.argtypes = [C.c_void_p, dp, dp, dp, dp, dp, C.c_size_t]
        _lib.oracle_upload_std140.argtypes = [C.c_void_p, fp, ip, fp, fp, C.c_size_t]
        _lib.oracle_phase.argtypes = [C.c_void_p, C.c_int, C.c_double]
        _lib.oracle_init.argtypes = [C.c_void_p]
        _lib.oracle_step.argtypes = [C.c_void_p, C.c_double, C.c_int]
        _lib.oracle_download.argtypes = [C.c_void_p, dp, dp, dp, dp, dp, dp]
        _lib.oracle_download_std140.argtypes = [C.c_void_p, fp, ip, fp, fp]
        _lib.oracle_download_grid.argtypes = [C.c_void_p, dp, dp, dp, dp]
        _lib.oracle_download_grid_fixed.argtypes = [C.c_void_p, ip, ip]
        _lib.oracle_download_accumulators.argtypes = [C.c_void_p, dp, dp]
        _lib.oracle_download_colliders.argtypes = [C.c_void_p, dp]
        _lib.oracle_set_density.argtypes = [C.c_void_p, dp]
        _lib.oracle_svd.argtypes = [dp, dp, dp, dp, C.c_int, C.c_int, C.c_int]
        _lib.oracle_lame.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, fp, fp]
        _lib.oracle_cell_keys.argtypes = [fp, C.c_size_t, fp, ip, C.c_float, up, up, up]
        _lib.oracle_set_implicit.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int]
        _lib.oracle_hessian.argtypes = [C.c_void_p, dp, dp]
        _lib.oracle_force_at.argtypes = [C.c_void_p, dp, C.c_double, dp]
        _lib.oracle_solver_report.argtypes = [C.c_void_p, dp]
        _lib.oracle_flip_scale.argtypes = [C.c_void_p, dp]
    return _lib


def ref_lib():
    """The compiled reference shaders, or None when unavailable."""
    global _ref
    if _ref is None:
        so = _build.build_ref()
        if so is None or not os.path.exists(so):
            return None
        _ref = C.CDLL(so)
        fp, ip = C.POINTER(C.c_float), C.POINTER(C.c_int)
        _ref.snowref_create.restype = C.c_void_p
        _ref.snowref_create.argtypes = [C.c_void_p]
        _ref.snowref_destroy.argtypes = [C.c_void_p]
        _ref.snowref_upload.argtypes = [C.c_void_p, fp, ip, fp, fp, C.c_uint]
        _ref.snowref_dispatch.argtypes = [C.c_void_p, C.c_int, C.c_double]
        _ref.snowref_init.argtypes = [C.c_void_p]
        _ref.snowref_update.argtypes = [C.c_void_p, C.c_double]
        _ref.snowref_download.argtypes = [C.c_void_p, fp, ip, fp, fp]
        _ref.snowref_download_accumulators.argtypes = [C.c_void_p, ip, ip, ip, ip]
        _ref.snowref_download_grid.argtypes = [C.c_void_p, ip, ip, fp, fp]
        _ref.snowref_download_colliders.argtypes = [C.c_void_p, fp]
    return _ref


class _OracleDesc(C.Structure):
    _fields_ = [
        ("grid_pos", C.c_double * 3), ("grid_dim", C.c_int * 3), ("grid_spacing", C.c_double),
        ("young", C.c_double), ("poisson", C.c_double), ("hardening", C.c_double),
        ("crit_compression", C.c_double), ("crit_stretch", C.c_double), ("alpha", C.c_double),
        ("gravity", C.c_double * 3), ("n_colliders", C.c_int),
        ("collider_pos", C.POINTER(C.c_double)), ("collider_type", C.POINTER(C.c_int)),
        ("collider_vel", C.POINTER(C.c_double)), ("collider_radius", C.POINTER(C.c_double)),
        ("collider_normal", C.POINTER(C.c_double)), ("collider_friction", C.POINTER(C.c_double)),
        ("vround", C.c_int), ("qround", C.c_int), ("threads", C.c_int),
    ]


class _RefDesc(C.Structure):
    _fields_ = [
        ("grid_pos", C.c_float * 3), ("grid_dim", C.c_int * 3), ("grid_spacing", C.c_float),
        ("young", C.c_float), ("poisson", C.c_float), ("hardening", C.c_float),
        ("crit_compression", C.c_float), ("crit_stretch", C.c_float), ("n_colliders", C.c_int),
        ("collider_pos", C.POINTER(C.c_float)), ("collider_type", C.POINTER(C.c_int)),
        ("collider_vel", C.POINTER(C.c_float)), ("collider_radius", C.POINTER(C.c_float)),
        ("collider_normal", C.POINTER(C.c_float)), ("collider_friction", C.POINTER(C.c_float)),
        ("threads", C.c_int),
    ]


def _collider_arrays(scene, dtype):
    cs = scene.colliders
    n = len(cs)
    pos = np.array([c.pos for c in cs], dtype).reshape(n, 3) if n else np.zeros((1, 3), dtype)
    typ = np.array([c.type for c in cs], np.int32) if n else np.zeros(1, np.int32)
    vel = np.array([c.vel for c in cs], dtype).reshape(n, 3) if n else np.zeros((1, 3), dtype)
    rad = np.array([c.radius for c in cs], dtype) if n else np.zeros(1, dtype)
    nor = np.array([c.normal for c in cs], dtype).reshape(n, 3) if n else np.zeros((1, 3), dtype)
    fri = np.array([c.friction for c in cs], dtype) if n else np.zeros(1, dtype)
    return n, [np.ascontiguousarray(a) for a in (pos, typ, vel, rad, nor, fri)]


class OracleSim:
    """The restatement on one scene. mode: FAITHFUL32 / EXACT64 / ..."""

    def __init__(self, scene, mode=EXACT64, vround=None, qround=True, threads=1):
        self.L = lib()
        self.scene = scene
        self.mode = mode
        if vround is None:
            vround = mode in (FAITHFUL32, FAITHFUL64)
        n, arrs = _collider_arrays(scene, np.float64)
        self._keep = arrs
        d = _OracleDesc()
        for k in range(3):
            d.grid_pos[k] = float(np.float32(scene.grid_pos[k]))
            d.grid_dim[k] = int(scene.grid_dim[k])
            d.gravity[k] = float(np.float32(scene.gravity[k]))
        f32 = lambda v: float(np.float32(v))  # the shaders receive float uniforms
        d.grid_spacing = f32(scene.grid_spacing)
        d.young, d.poisson, d.hardening = f32(scene.young), f32(scene.poisson), f32(scene.hardening)
        d.crit_compression, d.crit_stretch = f32(scene.crit_compression), f32(scene.crit_stretch)
        d.alpha = f32(scene.alpha)
        d.n_colliders = n
        pos, typ, vel, rad, nor, fri = arrs
        d.collider_pos, d.collider_type = _p(pos, C.c_double), _p(typ, C.c_int)
        d.collider_vel, d.collider_radius = _p(vel, C.c_double), _p(rad, C.c_double)
        d.collider_normal, d.collider_friction = _p(nor, C.c_double), _p(fri, C.c_double)
        d.vround, d.qround, d.threads = int(bool(vround)), int(bool(qround)), int(threads)
        self.h = self.L.oracle_create(C.byref(d), mode)
        self.n = scene.n
        self.G = int(np.prod(scene.grid_dim))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.oracle_destroy(self.h)
            self.h = None

    def upload(self, FE=None, FP=None):
        s = self.scene
        x = np.ascontiguousarray(s.x, np.float64)
        v = np.ascontiguousarray(s.v, np.float64)
        m = np.ascontiguousarray(s.m, np.float64)
        fe = None if FE is None else np.ascontiguousarray(FE, np.float64).reshape(-1, 9)
        fp = None if FP is None else np.ascontiguousarray(FP, np.float64).reshape(-1, 9)
        self.L.oracle_upload(self.h, _p(x, C.c_double), _p(v, C.c_double), _p(m, C.c_double),
                             _p(fe, C.c_double), _p(fp, C.c_double), self.n)
        return self

    def upload_std140(self, pxm, pv, pfe, pfp):
        a = [np.ascontiguousarray(pxm, np.float32), np.ascontiguousarray(pv, np.int32),
             np.ascontiguousarray(pfe, np.float32), np.ascontiguousarray(pfp, np.float32)]
        self.L.oracle_upload_std140(self.h, _p(a[0], C.c_float), _p(a[1], C.c_int), _p(a[2], C.c_float),
                                    _p(a[3], C.c_float), len(a[0]))
        return self

    def init(self):
        self.L.oracle_init(self.h)
        return self

    def set_density(self, rho):
        r = np.ascontiguousarray(rho, np.float64)
        self.L.oracle_set_density(self.h, _p(r, C.c_double))
        return self

    def step(self, dt=None, n=1):
        self.L.oracle_step(self.h, float(self.scene.dt if dt is None else dt), int(n))
        return self

    def phase(self, which, dt=None):
        self.L.oracle_phase(self.h, int(which), float(self.scene.dt if dt is None else dt))

    def step_with_flip_scale(self, dt=None):
        """One step (the phases of step()), returning per particle the
        magnitude scale of its FLIP velocity update taken between the grid
        update and G2P: alpha |v_p| + sum_i w_ip (|v*_i| + alpha |p_i/m_i|)."""
        for ph in (PH_RIGID, PH_RESET, PH_P2G, PH_GRID, PH_IMPLICIT):
            self.phase(ph, dt)
        out = np.zeros(self.n)
        self.L.oracle_flip_scale(self.h, _p(out, C.c_double))
        for ph in (PH_G2P, PH_ADVANCE):
            self.phase(ph, dt)
        return out

    def state(self):
        n = self.n
        x, v = np.zeros((n, 3)), np.zeros((n, 3))
        m, rho = np.zeros(n), np.zeros(n)
        fe, fp = np.zeros((n, 3, 3)), np.zeros((n, 3, 3))
        self.L.oracle_download(self.h, _p(x, C.c_double), _p(v, C.c_double), _p(m, C.c_double),
                               _p(fe, C.c_double), _p(fp, C.c_double), _p(rho, C.c_double))
        return dict(x=x, v=v, m=m, FE=fe, FP=fp, rho=rho, Jp=np.linalg.det(fp))

    def state_std140(self):
        n = self.n
        pxm, pv = np.zeros((n, 4), np.float32), np.zeros((n, 4), np.int32)
        fe, fp = np.zeros((n, 16), np.float32), np.zeros((n, 16), np.float32)
        self.L.oracle_download_std140(self.h, _p(pxm, C.c_float), _p(pv, C.c_int), _p(fe, C.c_float),
                                      _p(fp, C.c_float))
        return pxm, pv, fe, fp

    def grid(self):
        G = self.G
        mass, mom, force, vstar = np.zeros(G), np.zeros((G, 3)), np.zeros((G, 3)), np.zeros((G, 3))
        self.L.oracle_download_grid(self.h, _p(mass, C.c_double), _p(mom, C.c_double), _p(force, C.c_double),
                                    _p(vstar, C.c_double))
        return dict(mass=mass, mom=mom, force=force, vstar=vstar)

    def grid_fixed(self):
        G = self.G
        gv, gf = np.zeros((G, 4), np.int32), np.zeros((G, 4), np.int32)
        self.L.oracle_download_grid_fixed(self.h, _p(gv, C.c_int), _p(gf, C.c_int))
        return gv, gf

    def accumulators(self):
        n = self.n
        vp, dv = np.zeros((n, 3)), np.zeros((n, 3, 3))
        self.L.oracle_download_accumulators(self.h, _p(vp, C.c_double), _p(dv, C.c_double))
        return vp, dv

    def colliders(self):
        out = np.zeros((max(1, len(self.scene.colliders)), 3))
        self.L.oracle_download_colliders(self.h, _p(out, C.c_double))
        return out[:len(self.scene.colliders)]

    # ---- semi-implicit velocity update (EXACT modes) ----
    def set_implicit(self, beta, tol=1e-6, max_iters=50):
        self.L.oracle_set_implicit(self.h, float(beta), float(tol), int(max_iters))
        return self

    def hessian(self, u):
        """K u for a grid field u (G x 3) at the current particle state."""
        u = np.ascontiguousarray(u, np.float64).reshape(self.G, 3)
        out = np.zeros((self.G, 3))
        self.L.oracle_hessian(self.h, _p(u, C.c_double), _p(out, C.c_double))
        return out

    def force_at(self, u, eps):
        """Grid force with every particle's F_E deformed by the grid field eps u."""
        u = np.ascontiguousarray(u, np.float64).reshape(self.G, 3)
        out = np.zeros((self.G, 3))
        self.L.oracle_force_at(self.h, _p(u, C.c_double), float(eps), _p(out, C.c_double))
        return out

    def solver_report(self):
        out = np.zeros(3)
        self.L.oracle_solver_report(self.h, _p(out, C.c_double))
        return dict(iterations=int(out[0]), residual=float(out[1]), initial_residual=float(out[2]))


class RefSim:
    """The reference's compute shaders (compiled as C++) on one scene, fed
    with the reference's std140 buffers."""

    def __init__(self, scene, threads=1):
        self.L = ref_lib()
        if self.L is None:
            raise RuntimeError("compiled reference shaders unavailable")
        self.scene = scene
        n, arrs = _collider_arrays(scene, np.float32)
        self._keep = arrs
        d = _RefDesc()
        for k in range(3):
            d.grid_pos[k] = scene.grid_pos[k]
            d.grid_dim[k] = int(scene.grid_dim[k])
        d.grid_spacing = scene.grid_spacing
        d.young, d.poisson, d.hardening = scene.young, scene.poisson, scene.hardening
        d.crit_compression, d.crit_stretch = scene.crit_compression, scene.crit_stretch
        d.n_colliders = n
        pos, typ, vel, rad, nor, fri = arrs
        d.collider_pos, d.collider_type = _p(pos, C.c_float), _p(typ, C.c_int)
        d.collider_vel, d.collider_radius = _p(vel, C.c_float), _p(rad, C.c_float)
        d.collider_normal, d.collider_friction = _p(nor, C.c_float), _p(fri, C.c_float)
        d.threads = int(threads)
        self.h = self.L.snowref_create(C.byref(d))
        self.G = int(np.prod(scene.grid_dim))
        self.n = 0

    def __del__(self):
        if getattr(self, "h", None):
            self.L.snowref_destroy(self.h)
            self.h = None

    def upload_std140(self, pxm, pv, pfe, pfp):
        self._bufs = [np.ascontiguousarray(pxm, np.float32), np.ascontiguousarray(pv, np.int32),
                      np.ascontiguousarray(pfe, np.float32), np.ascontiguousarray(pfp, np.float32)]
        a = self._bufs
        self.n = len(a[0])
        self.L.snowref_upload(self.h, _p(a[0], C.c_float), _p(a[1], C.c_int), _p(a[2], C.c_float),
                              _p(a[3], C.c_float), self.n)
        return self

    def init(self):
        self.L.snowref_init(self.h)
        return self

    def update(self, dt=None):
        self.L.snowref_update(self.h, float(self.scene.dt if dt is None else dt))
        return self

    def dispatch(self, which, dt=None):
        self.L.snowref_dispatch(self.h, int(which), float(self.scene.dt if dt is None else dt))

    def state_std140(self):
        n = self.n
        pxm, pv = np.zeros((n, 4), np.float32), np.zeros((n, 4), np.int32)
        fe, fp = np.zeros((n, 16), np.float32), np.zeros((n, 16), np.float32)
        self.L.snowref_download(self.h, _p(pxm, C.c_float), _p(pv, C.c_int), _p(fe, C.c_float), _p(fp, C.c_float))
        return pxm, pv, fe, fp

    def grid(self):
        G = self.G
        gv, gf = np.zeros((G, 4), np.int32), np.zeros((G, 4), np.int32)
        gvn, gxm = np.zeros((G, 4), np.float32), np.zeros((G, 4), np.float32)
        self.L.snowref_download_grid(self.h, _p(gv, C.c_int), _p(gf, C.c_int), _p(gvn, C.c_float),
                                     _p(gxm, C.c_float))
        return gv, gf, gvn, gxm

    def accumulators(self):
        n = self.n
        a = [np.zeros((n, 4), np.int32) for _ in range(4)]
        self.L.snowref_download_accumulators(self.h, *[_p(x, C.c_int) for x in a])
        return a

    def colliders(self):
        out = np.zeros((max(1, len(self.scene.colliders)), 4), np.float32)
        self.L.snowref_download_colliders(self.h, _p(out, C.c_float))
        return out[:len(self.scene.colliders)]


def svd(a, fp64=True, vround=False):
    a = np.ascontiguousarray(a, np.float64).reshape(-1, 9)
    n = len(a)
    w, s, v = np.zeros((n, 9)), np.zeros((n, 9)), np.zeros((n, 9))
    lib().oracle_svd(_p(a, C.c_double), _p(w, C.c_double), _p(s, C.c_double), _p(v, C.c_double), n,
                     int(fp64), int(vround))
    return w.reshape(n, 3, 3), s.reshape(n, 3, 3), v.reshape(n, 3, 3)


def lame(young, poisson, hardening, jp):
    mu, lam = C.c_float(), C.c_float()
    lib().oracle_lame(young, poisson, hardening, jp, C.byref(mu), C.byref(lam))
    return mu.value, lam.value


def cell_keys(x, grid_pos, grid_dim, h):
    x = np.ascontiguousarray(x, np.float32).reshape(-1, 3)
    n = len(x)
    gp = np.ascontiguousarray(grid_pos, np.float32)
    gd = np.ascontiguousarray(grid_dim, np.int32)
    lin, blk, perm = np.zeros(n, np.uint32), np.zeros(n, np.uint32), np.zeros(n, np.uint32)
    lib().oracle_cell_keys(_p(x, C.c_float), n, _p(gp, C.c_float), _p(gd, C.c_int), float(np.float32(h)),
                           _p(lin, C.c_uint32), _p(blk, C.c_uint32), _p(perm, C.c_uint32))
    return lin, blk, perm


def parity_errors(got, ref, flip_scale=None):
    """Per-particle relative errors of a single-precision state `got` against
    an oracle state `ref` (dicts with x, v, FE, Jp), as the parity tests and
    the benchmark's full-size check report them:

      x       |dx| / max(|x|, 1e-3 m)
      v       |dv| / max(|v|, 1e-3 m/s)                  (the strict floor)
      v_flip  |dv| / max(|v|, 1e-3 m/s, S_p)             (needs flip_scale)
      FE      max|dF_E| / max|F_E| per particle
      Jp      |dJ_p| / |J_p|

    S_p = alpha |v_p| + sum_i w_ip (|v*_i| + alpha |p_i/m_i|) is the size of
    the terms the FLIP update v' = alpha v_p + sum_i w_ip (v*_i - alpha
    p_i/m_i) adds up (OracleSim.step_with_flip_scale). A particle that a
    collider or the snow around it stops within the step has |v'| << S_p;
    any single-precision evaluation of the update resolves v' only to a few
    ulps of S_p there, so for such particles the strict floor cannot be met
    and v_flip is the bound that FP32 arithmetic allows.
    Returns the max, p99 and median of each and the data of the particles
    with the largest v and v_flip errors."""
    x, v = np.asarray(got["x"], np.float64), np.asarray(got["v"], np.float64)
    speed = np.linalg.norm(ref["v"], axis=1)
    dv = np.linalg.norm(v - ref["v"], axis=1)
    err = {
        "x": (np.abs(x - ref["x"]) / np.maximum(np.abs(ref["x"]), 1e-3)).max(1),
        "v": dv / np.maximum(speed, 1e-3),
        "FE": np.abs(np.asarray(got["FE"], np.float64) - ref["FE"]).max((1, 2)) / np.abs(ref["FE"]).max((1, 2)),
        "Jp": np.abs(np.asarray(got["Jp"], np.float64) - ref["Jp"]) / np.abs(ref["Jp"]),
    }
    if flip_scale is not None:
        err["v_flip"] = dv / np.maximum(np.maximum(speed, 1e-3), flip_scale)
    out = {"max": {k: float(e.max()) for k, e in err.items()},
           "p99": {k: float(np.percentile(e, 99)) for k, e in err.items()},
           "median": {k: float(np.median(e)) for k, e in err.items()}}
    w = int(np.argmax(err["v"]))
    out["v_worst"] = {"ref": ref["v"][w].tolist(), "got": v[w].tolist(), "x": ref["x"][w].tolist(),
                      "flip_scale": None if flip_scale is None else float(flip_scale[w])}
    if flip_scale is not None:
        w = int(np.argmax(err["v_flip"]))
        out["v_flip_worst"] = {"ref": ref["v"][w].tolist(), "got": v[w].tolist(), "x": ref["x"][w].tolist(),
                               "flip_scale": float(flip_scale[w])}
    return out
