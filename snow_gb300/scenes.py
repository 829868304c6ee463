"""Seeded scene generators and the scene description shared by the host API,
the bench and the tests.

A scene mirrors what the reference's launcher builds before it calls
``ExplicitTimeUpdate::init`` (src/snow/utils/launchHelper/explicit.cpp:2-91):
a dense grid (origin, dimensions, spacing), the six wall half-planes placed
GRID_COLLISION_PLANE_OFFSET nodes inside each face (explicit.cpp:9-67) and a
particle list (position, velocity, mass; F_E = F_P = I). Material constants
default to src/snow/utils/defines.hpp:50-54.

Particle sampling for the synthetic workloads: a jittered lattice with 8
particles per grid cell (2x2x2 sub-lattice, uniform jitter of +-h/8 about
each sub-lattice point), mass rho*h^3/8 with rho = 400 kg/m^3. The particle
count N is binding: a shape keeps its stated centre and is scaled so that
exactly N lattice points fall inside it (the N closest to the centre under the
shape's own norm).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

# src/snow/utils/defines.hpp:14-54 and the shader constants
GRID_POS = (0.5125, 0.5125, 1.5125)
GRID_DIM = (201, 201, 201)
GRID_SPACING = 0.05
GRID_COLLISION_PLANE_OFFSET = 4
PHYSIC_DT = 1e-3
YOUNG_MODULUS = 6e6
POISSON = 0.2
HARDENING = 30.0
CRIT_COMPRESSION = 1.0e-2
CRIT_STRETCH = 1e-3
ALPHA = 0.95          # g2pTransfer.glsl:2, particleAdvance.glsl:2
GRAVITY = (0.0, -9.81, 0.0)  # gForceCompute.glsl:39
FRICTION = 0.2        # collider.hpp:16
SNOW_DENSITY = 400.0

COLLIDER_HALF_PLANE = 0
COLLIDER_SPHERE = 1


@dataclasses.dataclass
class Collider:
    pos: tuple
    type: int = COLLIDER_HALF_PLANE
    vel: tuple = (0.0, 0.0, 0.0)
    radius: float = 0.0
    normal: tuple = (0.0, 0.0, 0.0)
    friction: float = FRICTION


@dataclasses.dataclass
class Scene:
    grid_pos: tuple = GRID_POS
    grid_dim: tuple = GRID_DIM
    grid_spacing: float = GRID_SPACING
    young: float = YOUNG_MODULUS
    poisson: float = POISSON
    hardening: float = HARDENING
    crit_compression: float = CRIT_COMPRESSION
    crit_stretch: float = CRIT_STRETCH
    alpha: float = ALPHA
    gravity: tuple = GRAVITY
    dt: float = PHYSIC_DT
    steps: int = 1
    colliders: List[Collider] = dataclasses.field(default_factory=list)
    # semi-implicit velocity update: beta > 0 solves (M + beta dt^2 K) v = M v*
    # each step (0 = the explicit step; tolerance / iterations 0 = defaults)
    implicit_beta: float = 0.0
    implicit_tolerance: float = 0.0
    implicit_max_iters: int = 0
    x: Optional[np.ndarray] = None   # N x 3 float32
    v: Optional[np.ndarray] = None   # N x 3 float32
    m: Optional[np.ndarray] = None   # N float32
    name: str = "scene"

    @property
    def n(self) -> int:
        return 0 if self.x is None else int(self.x.shape[0])

    def std140(self):
        """The reference's particle buffers exactly as ParticleSystem::initSSBO
        writes them (particlesystem.cpp:101-228): pxm N x vec4 (x, m), pv N x
        ivec4 (v * 1e8 as int, 0), pFE and pFP N x mat4 (column-major, upper
        3x3 = I, [3][3] = 0 as in particle.hpp:8-11)."""
        n = self.n
        pxm = np.zeros((n, 4), np.float32)
        pxm[:, :3] = self.x
        pxm[:, 3] = self.m
        pv = np.zeros((n, 4), np.int32)
        pv[:, :3] = np.trunc(self.v.astype(np.float64) * 1e8).astype(np.int32)
        fe = np.zeros((n, 16), np.float32)
        fe[:, [0, 5, 10]] = 1.0
        return pxm, pv, fe, fe.copy()


def walls(grid_pos, grid_dim, h, offset=GRID_COLLISION_PLANE_OFFSET, friction=FRICTION):
    """The six half-planes of explicit.cpp:9-67: three through
    grid_pos + offset*h with normals +x, +y, +z and three through
    grid_pos + (dim - offset)*h with normals -x, -y, -z. Positions are formed
    in double and stored as float, as Mesh::setPosition(float, ...) does."""
    lo = tuple(float(np.float32(grid_pos[k] + offset * h)) for k in range(3))
    hi = tuple(float(np.float32(grid_pos[k] + (grid_dim[k] - offset) * h)) for k in range(3))
    out = []
    for k in range(3):
        nrm = [0.0, 0.0, 0.0]
        nrm[k] = 1.0
        out.append(Collider(pos=lo, normal=tuple(nrm), friction=friction))
    for k in range(3):
        nrm = [0.0, 0.0, 0.0]
        nrm[k] = -1.0
        out.append(Collider(pos=hi, normal=tuple(nrm), friction=friction))
    return out


def _lattice_points(center, half_extent_cells, h, rng, origin=(0.0, 0.0, 0.0)):
    """Jittered 2x2x2-per-cell lattice covering the box centre +- half_extent."""
    c = np.asarray(center, np.float64)
    ext = np.asarray(half_extent_cells, np.float64) * h
    lo = np.floor((c - ext - np.asarray(origin)) / h).astype(np.int64)
    hi = np.ceil((c + ext - np.asarray(origin)) / h).astype(np.int64)
    axes = [np.arange(2 * lo[k], 2 * hi[k]) for k in range(3)]
    g = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3).astype(np.float64)
    pts = (g + 0.5) * (h / 2.0) + np.asarray(origin)
    pts += rng.uniform(-h / 8.0, h / 8.0, size=pts.shape)
    return pts


def sample_shape(kind, center, n, h, rng, aspect=(1.0, 1.0, 1.0)):
    """Exactly n lattice particles filling a sphere or box about `center`,
    scaled to hold n particles at 8 per cell. Returns float32 N x 3."""
    aspect = np.asarray(aspect, np.float64)
    cells = n / 8.0
    if kind == "sphere":
        r_cells = (3.0 * cells / (4.0 * math.pi)) ** (1.0 / 3.0)
        half = np.full(3, r_cells * 1.15 + 2)
    else:
        s = (cells / np.prod(aspect)) ** (1.0 / 3.0)
        half = aspect * s / 2.0 * 1.15 + 2
    pts = _lattice_points(center, half, h, rng)
    d = (pts - np.asarray(center)) / (np.asarray(aspect) * h)
    if kind == "sphere":
        key = np.sqrt((d ** 2).sum(1))
    else:
        key = np.abs(d).max(1)
    # the n smallest keys, ties broken by a random secondary key so the
    # selection stays isotropic (the same set a full lexsort would give)
    tie = rng.random(len(key))
    if len(key) < n:
        raise ValueError("sampling box too small")
    kv = np.partition(key, n - 1)[n - 1]
    less = np.flatnonzero(key < kv)
    eq = np.flatnonzero(key == kv)
    picked = eq[np.argsort(tie[eq], kind="stable")[:n - len(less)]]
    sel = pts[np.sort(np.concatenate([less, picked]))]
    return sel.astype(np.float32)


def unit_box_scene(grid_edge, **kw) -> Scene:
    """Domain [0, 1]^3 with grid_edge^3 nodes, h = 1/grid_edge, walls at 4h."""
    h = 1.0 / grid_edge
    dim = (grid_edge, grid_edge, grid_edge)
    pos = (0.0, 0.0, 0.0)
    s = Scene(grid_pos=pos, grid_dim=dim, grid_spacing=h, colliders=walls(pos, dim, h), **kw)
    return s


def cfg1_snowball(seed: int = 0x5EED0001, n: int = 32768) -> Scene:
    """Plain single scene: one snowball, ~32k particles, 64^3 grid, h = 1/64,
    E0 = 1.4e5, nu = 0.2, theta_c = 2.5e-2, theta_s = 7.5e-3, xi = 10,
    v0 = (0, -2, 0), dt = 1e-4, 100 steps."""
    rng = np.random.default_rng(seed)
    s = unit_box_scene(64, young=1.4e5, poisson=0.2, hardening=10.0, crit_compression=2.5e-2,
                       crit_stretch=7.5e-3, dt=1e-4, steps=100, name="cfg1_snowball")
    h = s.grid_spacing
    s.x = sample_shape("sphere", (0.5, 0.4, 0.5), n, h, rng)
    s.v = np.tile(np.array([0.0, -2.0, 0.0], np.float32), (n, 1))
    s.m = np.full(n, SNOW_DENSITY * h ** 3 / 8.0, np.float32)
    return s


def cfg2_two_snowballs(seed: int = 0x5EED0002, n: int = 1 << 20, grid_edge: int = 256) -> Scene:
    """Plain large scene: two snowballs colliding head-on at +-5 m/s, n
    particles in total, 256^3 grid, dt = 2e-5, 500 steps."""
    rng = np.random.default_rng(seed)
    s = unit_box_scene(grid_edge, young=1.4e5, poisson=0.2, hardening=10.0, crit_compression=2.5e-2,
                       crit_stretch=7.5e-3, dt=2e-5, steps=500, name="cfg2_two_snowballs")
    h = s.grid_spacing
    a = sample_shape("sphere", (0.25, 0.5, 0.5), n // 2, h, rng)
    b = sample_shape("sphere", (0.75, 0.5, 0.5), n - n // 2, h, rng)
    s.x = np.concatenate([a, b])
    s.v = np.concatenate([np.tile(np.array([5.0, 0, 0], np.float32), (len(a), 1)),
                          np.tile(np.array([-5.0, 0, 0], np.float32), (len(b), 1))])
    s.m = np.full(n, SNOW_DENSITY * h ** 3 / 8.0, np.float32)
    return s


def _round_up(x, m):
    return int(math.ceil(x / m) * m)


def cfg3_batch(seed: int = 0x5EED0003, n_scenes: int = 64, n_min: int = 10_000, n_max: int = 500_000,
               steps: int = 100) -> List[Scene]:
    """Batched: independent scenes with log-uniform particle counts, grid
    edge matched to the shape's extent (64..192), E0 ~ U[4.8e4, 1.4e5],
    xi ~ U[5, 10], sphere or box, random initial velocity |v| <= 4 m/s."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        kind = "sphere" if rng.random() < 0.5 else "box"
        r_cells = (3.0 * n / 8.0 / (4.0 * math.pi)) ** (1.0 / 3.0)
        edge = min(192, max(64, _round_up(5.0 * r_cells, 32)))
        s = unit_box_scene(edge, young=float(rng.uniform(4.8e4, 1.4e5)), poisson=0.2,
                           hardening=float(rng.uniform(5.0, 10.0)), crit_compression=2.5e-2,
                           crit_stretch=7.5e-3, dt=1e-4, steps=steps, name=f"cfg3_{i:02d}")
        h = s.grid_spacing
        center = (0.5 + rng.uniform(-0.05, 0.05), 0.5 + rng.uniform(-0.05, 0.05),
                  0.5 + rng.uniform(-0.05, 0.05))
        srng = np.random.default_rng(seed * 1000 + i)
        s.x = sample_shape(kind, center, n, h, srng)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        speed = float(rng.uniform(0.0, 4.0))
        s.v = np.tile((d * speed).astype(np.float32), (n, 1))
        s.m = np.full(n, SNOW_DENSITY * h ** 3 / 8.0, np.float32)
        out.append(s)
    return out


def snow_block_on_sphere(seed: int, n: int, edge: int, gap: float = 0.02, v0=(0.0, 0.0, 0.0)) -> Scene:
    """A snow block (0.6 x 0.3 x 0.6 aspect, n particles at 8 per cell,
    centred at (0.5, 0.6, 0.5)) above a static sphere collider (type 1,
    radius 0.15 scaled with the block) whose top lies `gap` below the
    block's bottom face (a negative gap sinks the sphere into the block), in
    a unit box of edge^3 nodes, dt = 2e-5, moving at v0."""
    s = unit_box_scene(edge, young=1.4e5, poisson=0.2, hardening=10.0, crit_compression=2.5e-2,
                       crit_stretch=7.5e-3, dt=2e-5, steps=200, name=f"block_{n}_{edge}")
    h = s.grid_spacing
    aspect = (0.6, 0.3, 0.6)
    srng = np.random.default_rng(seed)
    s.x = sample_shape("box", (0.5, 0.6, 0.5), n, h, srng, aspect=aspect)
    ext = (s.x.max(0) - s.x.min(0)).astype(np.float64)
    scale = ext[0] / 0.6
    s.colliders.append(Collider(pos=(0.5, 0.6 - 0.15 * scale - 0.5 * ext[1] - gap, 0.5),
                                type=COLLIDER_SPHERE, radius=float(0.15 * scale)))
    s.v = np.tile(np.asarray(v0, np.float32), (n, 1))
    s.m = np.full(n, SNOW_DENSITY * h ** 3 / 8.0, np.float32)
    return s


def cfg4_batch(seed: int = 0x5EED0004, n_scenes: int = 16, n_min: int = 2_000_000, n_max: int = 8_000_000,
               steps: int = 200) -> List[Scene]:
    """Batched at scale: snow blocks (0.6 x 0.3 x 0.6 aspect) dropped onto a
    sphere collider (type 1, radius 0.15 scaled with the block), grids of
    384^3..512^3."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_scenes):
        n = int(rng.integers(n_min, n_max + 1))
        edge = int(rng.choice([384, 448, 512]))
        s = snow_block_on_sphere(seed * 1000 + i, n, edge)
        s.steps = steps
        s.name = f"cfg4_{i:02d}"
        out.append(s)
    return out


def serving_job(rng, n_min=20_000, n_max=2_000_000, steps_min=50, steps_max=2000, index=0) -> Scene:
    """One serving request: particle count log-uniform, step count uniform,
    shape and material drawn as for the batched scenes."""
    n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
    steps = int(rng.integers(steps_min, steps_max + 1))
    kind = "sphere" if rng.random() < 0.5 else "box"
    r_cells = (3.0 * n / 8.0 / (4.0 * math.pi)) ** (1.0 / 3.0)
    edge = min(256, max(64, _round_up(5.0 * r_cells, 32)))
    s = unit_box_scene(edge, young=float(rng.uniform(4.8e4, 1.4e5)), poisson=0.2,
                       hardening=float(rng.uniform(5.0, 10.0)), crit_compression=2.5e-2,
                       crit_stretch=7.5e-3, dt=1e-4, steps=steps, name=f"job_{index}")
    h = s.grid_spacing
    srng = np.random.default_rng(int(rng.integers(1 << 62)))
    s.x = sample_shape(kind, (0.5, 0.5, 0.5), n, h, srng)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    s.v = np.tile((d * float(rng.uniform(0.0, 4.0))).astype(np.float32), (n, 1))
    s.m = np.full(n, SNOW_DENSITY * h ** 3 / 8.0, np.float32)
    return s


def small_scene(n: int = 2000, grid_edge: int = 32, seed: int = 7, v0=(0.0, -2.0, 0.0), kind="sphere",
                center=(0.5, 0.45, 0.5), **kw) -> Scene:
    """A small snowball for parity tests (the oracle finishes in seconds)."""
    rng = np.random.default_rng(seed)
    params = dict(young=1.4e5, poisson=0.2, hardening=10.0, crit_compression=2.5e-2, crit_stretch=7.5e-3,
                  dt=1e-4, name=f"small_{n}_{grid_edge}")
    params.update(kw)
    s = unit_box_scene(grid_edge, **params)
    h = s.grid_spacing
    s.x = sample_shape(kind, center, n, h, rng)
    s.v = np.tile(np.asarray(v0, np.float32), (n, 1))
    s.m = np.full(n, SNOW_DENSITY * h ** 3 / 8.0, np.float32)
    return s


def reference_scene(x, v=None, m=None) -> Scene:
    """A particle list placed in the reference's default world
    (defines.hpp: 201^3 grid at GRID_POS, h = 0.05, six walls)."""
    x = np.asarray(x, np.float32).reshape(-1, 3)
    n = len(x)
    s = Scene(colliders=walls(GRID_POS, GRID_DIM, GRID_SPACING), name="reference_default")
    s.x = x
    s.v = np.zeros((n, 3), np.float32) if v is None else np.asarray(v, np.float32).reshape(-1, 3)
    s.m = np.full(n, 1.25e-3, np.float32) if m is None else np.asarray(m, np.float32).reshape(-1)
    return s


# ---- particles from files ---------------------------------------------------
_FLOAT_PREFIX = None


def _stof(text: str) -> float:
    """std::stof: skip leading white space, convert the longest prefix that
    reads as a float, raise ValueError when nothing converts."""
    import re
    global _FLOAT_PREFIX
    if _FLOAT_PREFIX is None:
        _FLOAT_PREFIX = re.compile(r"[+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan)",
                                   re.IGNORECASE)
    t = text.lstrip(" \t\n\v\f\r")
    mt = _FLOAT_PREFIX.match(t)
    if not mt:
        raise ValueError(f"stof: no conversion of {text!r}")
    return float(np.float32(float(mt.group(0))))


def particles_from_xyz(path: str, pos=(0.0, 0.0, 0.0), scale=(1.0, 1.0, 1.0), mass: float = 6.25e-3):
    """Particles from a text file with one `x,y,z` line per particle, as
    ParticleSystem::initParticlesFromFile reads it (particlesystem.cpp:14-38):
    position = scale * (x, y, z) + pos, velocity 0, mass 6.25e-3 each. Each
    field converts like std::stof (a malformed line raises ValueError, where
    the reference's stof throws); a line without a comma yields its one
    number for x, y and z, as the reference's substr/erase arithmetic does.
    A missing file is reported and yields no particles, like the reference.
    Returns (x N x 3, v N x 3, m N) as float32."""
    import os
    import sys
    if not os.path.exists(path):
        print(f"Error: File {path} not found.", file=sys.stderr)
        return np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), np.zeros(0, np.float32)
    pts = []
    with open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            c = line.find(",")
            x = _stof(line if c < 0 else line[:c])
            line = line if c < 0 else line[c + 1:]
            c = line.find(",")
            y = _stof(line if c < 0 else line[:c])
            line = line if c < 0 else line[c + 1:]
            z = _stof(line)
            pts.append((x, y, z))
    xyz = np.asarray(pts, np.float32).reshape(-1, 3)
    sc = np.asarray(scale, np.float32)
    off = np.asarray(pos, np.float32)
    x = (sc * xyz + off).astype(np.float32)
    n = len(x)
    return x, np.zeros((n, 3), np.float32), np.full(n, mass, np.float32)


def add_particles(scene: Scene, x, v, m) -> Scene:
    """Appends particles to a scene (the reference's ParticleSystem holds the
    particles of every init call in one list)."""
    def cat(a, b, shape):
        b = np.asarray(b, np.float32).reshape(shape)
        return b if a is None else np.concatenate([a, b])
    scene.x = cat(scene.x, x, (-1, 3))
    scene.v = cat(scene.v, v, (-1, 3))
    scene.m = cat(scene.m, m, (-1,))
    return scene
