"""Generates the golden vectors in tests/golden/*.npz from the snow
reference's own compute shaders, compiled as C++ by oracle/ref_translate.py
and driven in the reference's dispatch order (oracle/ref_driver.cpp).

Each fixture holds a scene description, the reference's std140 particle
buffers as uploaded (ParticleSystem::initSSBO), the buffers after
ExplicitTimeUpdate::init, and the particle buffers plus the non-zero grid
nodes after each of a few ExplicitTimeUpdate::update(dt) calls.

Run where the reference tree exists:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from snow_gb300 import scenes  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def scene_to_json(s: scenes.Scene) -> str:
    d = {k: getattr(s, k) for k in ("grid_pos", "grid_dim", "grid_spacing", "young", "poisson", "hardening",
                                    "crit_compression", "crit_stretch", "alpha", "gravity", "dt", "name")}
    d["colliders"] = [dict(pos=list(c.pos), type=c.type, vel=list(c.vel), radius=c.radius, normal=list(c.normal),
                           friction=c.friction) for c in s.colliders]
    d["grid_pos"], d["grid_dim"], d["gravity"] = list(d["grid_pos"]), list(d["grid_dim"]), list(d["gravity"])
    return json.dumps(d)


def particles3x3(buf16):
    """Upper-left 3x3 of std140 mat4s, column-major, N x 9."""
    b = buf16.reshape(-1, 4, 4)
    return np.ascontiguousarray(b[:, :3, :3].reshape(-1, 9))


def fixture(name, s: scenes.Scene, steps: int):
    bufs = s.std140()
    ref = O.RefSim(s, threads=os.cpu_count()).upload_std140(*bufs).init()
    out = dict(scene=np.array(scene_to_json(s)), pxm0=bufs[0], pv0=bufs[1])
    pxm, pv, fe, fp = ref.state_std140()
    out["pv_init"] = pv
    for k in range(1, steps + 1):
        ref.update()
        pxm, pv, fe, fp = ref.state_std140()
        out[f"pxm_{k}"], out[f"pv_{k}"] = pxm, pv
        out[f"fe_{k}"], out[f"fp_{k}"] = particles3x3(fe), particles3x3(fp)
    gv, gf, gvn, _ = ref.grid()
    nz = np.nonzero((gv != 0).any(1) | (gf != 0).any(1))[0].astype(np.int32)
    out["grid_nodes"], out["grid_gv"], out["grid_gf"], out["grid_gvn"] = nz, gv[nz], gf[nz], gvn[nz]
    out["colliders_cx"] = ref.colliders()
    out["steps"] = np.array(steps)
    path = os.path.join(OUT, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{path}: N={s.n} steps={steps} grid_nodes={len(nz)} {os.path.getsize(path) // 1024} KB")


def main():
    # 1. One particle in the reference's default world (snowSingleParticle.cpp).
    rng = np.random.default_rng(1)
    x = np.array([[5.0, 1.7125, 5.0]]) + rng.uniform(0, 1, (1, 3))
    fixture("single_particle", scenes.reference_scene(x), steps=3)

    # 2. A 6^3 lattice at 0.025 spacing placed as snowSquare.cpp places its
    #    lattice: z = 0.9625 lies below the default grid origin (z = 1.5125),
    #    so no particle reaches a grid node. The same lattice moved to
    #    z = 1.9625 sits on the floor wall inside the grid.
    g = np.stack(np.meshgrid(*[np.arange(6)] * 3, indexing="ij"), -1).reshape(-1, 3)
    x = np.array([0.9625, 0.72, 0.9625]) + 0.025 * g[:, [0, 2, 1]]
    fixture("lattice_6_outside", scenes.reference_scene(x), steps=2)
    x = np.array([0.9625, 0.72, 1.9625]) + 0.025 * g[:, [0, 2, 1]]
    fixture("lattice_6", scenes.reference_scene(x), steps=3)

    # 3. A small snowball with the snowball material falling on the floor.
    fixture("snowball_1500", scenes.small_scene(n=1500, grid_edge=32, seed=11), steps=3)

    # 4. Fast impact onto the floor: exercises the plasticity clamp and the
    #    friction branch of the wall collider.
    s = scenes.small_scene(n=800, grid_edge=32, seed=12, v0=(1.5, -8.0, 0.5), center=(0.5, 0.2, 0.5))
    fixture("impact_800", s, steps=4)

    # 5. Two balls colliding head-on around a moving sphere collider.
    rng = np.random.default_rng(13)
    s = scenes.unit_box_scene(32, young=1.4e5, poisson=0.2, hardening=10.0, crit_compression=2.5e-2,
                              crit_stretch=7.5e-3, dt=1e-4, name="two_balls_sphere")
    h = s.grid_spacing
    a = scenes.sample_shape("sphere", (0.35, 0.5, 0.5), 400, h, rng)
    b = scenes.sample_shape("sphere", (0.65, 0.52, 0.5), 400, h, rng)
    s.x = np.concatenate([a, b])
    s.v = np.concatenate([np.tile([5.0, 0, 0], (400, 1)), np.tile([-5.0, 0, 0], (400, 1))]).astype(np.float32)
    s.m = np.full(800, scenes.SNOW_DENSITY * h ** 3 / 8, np.float32)
    s.colliders.append(scenes.Collider(pos=(0.5, 0.38, 0.5), type=scenes.COLLIDER_SPHERE, radius=0.08,
                                       vel=(0.0, 1.0, 0.0), friction=0.3))
    fixture("two_balls_sphere", s, steps=3)


if __name__ == "__main__":
    main()
