"""Training pairs for the far-field surrogate, generated by the batched engine.

A structure is a binary permittivity map {1.0, 2.43} on 256 x 256 cells of
5 nm: 2 to 12 lamellae stacked along y with random thicknesses, gaps and
widths, their centres offset along x in a zigzag (alternating side, random
amplitude).  The target is its far-field intensity at the 31 wavelengths
400, 410, ..., 700 nm and 360 angles (31 x 360 float32), MPI_TM_UPML at
0 degrees with a 10-cell UPML around the 256^2 map, FP32 fields and FP64
far-field sums, from one of two generators of the batched engine:

* broadband (default): one run per map, driven by the reference's Gaussian
  pulse (field.c:224-256, carrier 550 nm), the NTFF path samples of every step
  transformed at the 31 wavelengths (fdtd_batch_broadband); the intensity is
  per unit incident wave, angle a is the direction a;
* cw: 31 runs per map, one per wavelength, 12 optical periods of the CW wave,
  far field from ntffTM_Frequency of the final fields (angle a is the
  direction a + 180).

The two agree up to one scale per wavelength and the CW runs' distance from
steady state; the broadband runs cost about 25x fewer cell-updates.
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


BROADBAND_STEPS = 2500      # the pulse and the structures' ringing have left the 276^2 grid
BROADBAND_CARRIER = 550


class Generator:
    """Simulates maps in groups of `group` structures, one batched engine
    reused for every group: broadband (one pulse run per map) or cw (31 runs
    per map)."""

    def __init__(self, group: int = 64, lambdas=LAMBDAS, tblock: int = 4, mode: str = "broadband",
                 steps: int = BROADBAND_STEPS):
        from ..engine import OPT_TBLOCK
        self.lambdas = list(lambdas)
        self.group = group
        self.mode = mode
        if mode == "broadband":
            side = (GRID + 2 * PML) * H_U
            fis = [FieldInfo(side, side, H_U, PML, BROADBAND_CARRIER, 0, steps) for _ in range(group)]
            self.batch = Batch("MPI_TM_UPML", fis, "f32", no_time_ntff=False)
            self.batch.broadband(self.lambdas)
        elif mode == "cw":
            fis = [field_info(lam) for _ in range(group) for lam in self.lambdas]
            self.batch = Batch("MPI_TM_UPML", fis, "f32")
        else:
            raise ValueError(f"unknown generator mode {mode!r}")
        self.batch.set_option(OPT_TBLOCK, tblock)
        self.cell_steps = sum((f.width_nm // H_U) ** 2 * f.step_num for f in fis)
        self.seconds = 0.0

    def far_field(self, maps: np.ndarray) -> np.ndarray:
        """Far-field intensity at 360 angles: (len(maps), n_lambda, 360) float32."""
        if self.mode == "broadband":
            return self._broadband(maps)
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

    def _broadband(self, maps: np.ndarray) -> np.ndarray:
        out = np.zeros((len(maps), len(self.lambdas), 360), np.float32)
        for g0 in range(0, len(maps), self.group):
            part = maps[g0:g0 + self.group]
            self.batch.reset()
            for q, s in enumerate(self.batch.instances):
                s.set_eps(eps_of(part[q] if q < len(part) else part[-1]))
            for s in self.batch.instances:
                s.synchronize()
            t = time.perf_counter()
            self.batch.run()
            self.seconds += time.perf_counter() - t
            out[g0:g0 + len(part)] = self.batch.broadband_spectra()[:len(part)].astype(np.float32)
        return out

    def close(self):
        self.batch.close()
