"""Headless export of particle positions, in place of the reference's
ParticleSystem::render (particlesystem.cpp:4-13), which draws the position
buffer as GL points each frame: positions are written to files every
`every` steps, as `.npy` (N x 3 float32) or as `.xyz` text with one `x,y,z`
line per particle (the format particles_from_xyz reads back)."""
from __future__ import annotations

import os
from typing import List

import numpy as np


def write_positions(path: str, x: np.ndarray) -> str:
    x = np.asarray(x, np.float32).reshape(-1, 3)
    if path.endswith(".npy"):
        np.save(path, x)
    elif path.endswith(".xyz"):
        # 9 significant digits read back to the same float32
        np.savetxt(path, x, fmt="%.9g", delimiter=",")
    else:
        raise ValueError(f"unknown export format: {path}")
    return path


class PositionExporter:
    """Steps a SimScene and writes its positions every `every` steps to
    out_dir/<prefix>_<step>.<fmt> (step 0 = the state before stepping)."""

    def __init__(self, sim, out_dir: str, every: int = 10, fmt: str = "npy", prefix: str = "frame"):
        if every < 1 or fmt not in ("npy", "xyz"):
            raise ValueError("every >= 1 and fmt in ('npy', 'xyz')")
        self.sim, self.out_dir, self.every, self.fmt, self.prefix = sim, out_dir, every, fmt, prefix
        self.step_count = 0
        self.files: List[str] = []
        os.makedirs(out_dir, exist_ok=True)

    def _write(self):
        x = self.sim.download()["x"]
        path = os.path.join(self.out_dir, f"{self.prefix}_{self.step_count:06d}.{self.fmt}")
        self.files.append(write_positions(path, x))

    def run(self, n_steps: int, dt=None) -> List[str]:
        if self.step_count == 0 and not self.files:
            self._write()
        done = 0
        while done < n_steps:
            k = min(self.every - self.step_count % self.every, n_steps - done)
            self.sim.step(dt, k)
            done += k
            self.step_count += k
            if self.step_count % self.every == 0:
                self._write()
        return self.files
