"""Shared helpers for the tests: fixture loading and error metrics."""
import json
import os

import numpy as np

from snow_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = json.loads(str(z["scene"]))
    cols = [scenes.Collider(pos=tuple(c["pos"]), type=c["type"], vel=tuple(c["vel"]), radius=c["radius"],
                            normal=tuple(c["normal"]), friction=c["friction"]) for c in d.pop("colliders")]
    s = scenes.Scene(colliders=cols, **{k: (tuple(v) if isinstance(v, list) else v) for k, v in d.items()})
    pxm0, pv0 = z["pxm0"], z["pv0"]
    s.x = pxm0[:, :3].copy()
    s.m = pxm0[:, 3].copy()
    s.v = (pv0[:, :3].astype(np.float64) * 1e-8).astype(np.float32)
    return s, z


def mat3x3_from_std140(buf16):
    """N x 16 column-major mat4 -> N x 3 x 3 (row, col)."""
    b = np.asarray(buf16).reshape(-1, 4, 4)   # [p, c, r]
    return np.ascontiguousarray(b[:, :3, :3].transpose(0, 2, 1))


def rel_err(a, b, floor):
    """max_i |a_i - b_i| / max(|b_i|, floor), per row-free flattening."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)
