"""Training pairs for the far-field surrogate, generated by the batched engine.

A structure is a binary permittivity map {1.0, 2.43} on 256 x 256 cells of
5 nm: 2 to 12 lamellae stacked along y with random thicknesses, gaps and
widths, their centres offset along x in a zigzag (alternating side, random
amplitude).  Each map is simulated with MPI_TM_UPML (CW source at 0 deg,
10-cell UPML around the 256^2 map, 12 optical periods) at the 31 wavelengths
400, 410, ..., 700 nm by the batched FP32 engine (FP64 far-field sums), and
the target is the far-field intensity |E(phi)|^2 of ntffTM_Frequency at the
360 angles: a 31 x 360 float32 array per map.
"""
from __future__ import annotations

import math
import time

import numpy as np

from ..engine import Batch, FieldInfo

GRID = 256
H_U = 5
PML = 10
EPS_HI = 2.43
LAMBDAS = np.arange(400, 701, 10)
C_S = 0.7071


def lamella_map(rng: np.random.Generator) -> np.ndarray:
    """One structure: (256, 256) array of {0, 1} (1 = eps 2.43), [x][y]."""
    m = np.zeros((GRID, GRID), np.uint8)
    n = int(rng.integers(2, 13))
    thick = rng.uniform(4, 16, n)
    gap = rng.uniform(4, 16, n)
    total = thick.sum() + gap[:-1].sum()
    if total > 220:
        thick *= 220 / total
        gap *= 220 / total
        total = 220
    width = rng.uniform(24, 200, n)
    amp = rng.uniform(0, 24)
    y = (GRID - total) / 2
    for q in range(n):
        off = (amp if q % 2 == 0 else -amp) + rng.uniform(-4, 4)
        x0 = int(round(GRID / 2 + off - width[q] / 2))
        x1 = int(round(GRID / 2 + off + width[q] / 2))
        y0, y1 = int(round(y)), int(round(y + thick[q]))
        m[max(0, x0):min(GRID, x1), max(0, y0):min(GRID, max(y1, y0 + 1))] = 1
        y += thick[q] + gap[q]
    return m


def make_maps(n: int, seed: int = 20261203 + 4) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.stack([lamella_map(rng) for _ in range(n)])


def field_info(lam_nm: int) -> FieldInfo:
    side = (GRID + 2 * PML) * H_U
    steps = int(math.ceil(12 * (lam_nm / H_U) / C_S))
    return FieldInfo(side, side, H_U, PML, int(lam_nm), 0, steps)


def eps_of(m: np.ndarray) -> np.ndarray:
    """EPS_EZ of the whole (256 + 2 PML)^2 grid for a map."""
    e = np.ones((GRID + 2 * PML, GRID + 2 * PML))
    e[PML:PML + GRID, PML:PML + GRID] = np.where(m > 0, EPS_HI, 1.0)
    return e


class Generator:
    """Simulates maps in groups of `group` structures x 31 wavelengths, one
    batched engine reused for every group."""

    def __init__(self, group: int = 64, lambdas=LAMBDAS, tblock: int = 4):
        from ..engine import OPT_TBLOCK
        self.lambdas = list(lambdas)
        self.group = group
        fis = [field_info(lam) for _ in range(group) for lam in self.lambdas]
        self.batch = Batch("MPI_TM_UPML", fis, "f32")
        self.batch.set_option(OPT_TBLOCK, tblock)
        self.cell_steps = sum((f.width_nm // H_U) ** 2 * f.step_num for f in fis)
        self.seconds = 0.0

    def far_field(self, maps: np.ndarray) -> np.ndarray:
        """|E|^2 at 360 angles: (len(maps), n_lambda, 360) float32."""
        nl = len(self.lambdas)
        out = np.zeros((len(maps), nl, 360), np.float32)
        for g0 in range(0, len(maps), self.group):
            part = maps[g0:g0 + self.group]
            self.batch.reset()
            for q in range(self.group):
                e = eps_of(part[q] if q < len(part) else part[-1])
                for k in range(nl):
                    self.batch.instances[q * nl + k].set_eps(e)
            for s in self.batch.instances:
                s.synchronize()
            t = time.perf_counter()
            self.batch.run()
            self.seconds += time.perf_counter() - t
            for q in range(len(part)):
                for k in range(nl):
                    f = self.batch.instances[q * nl + k].frequency()
                    out[g0 + q, k] = (np.abs(f) ** 2).astype(np.float32)
        return out

    def close(self):
        self.batch.close()
