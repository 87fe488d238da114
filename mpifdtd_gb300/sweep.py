"""Structure sweeps: many Mie-cylinder instances through the batched engine.

The sweep workload: seeded cylinders with radius r ~ U(100, 800) nm,
permittivity eps ~ U(1.5, 4.0) and wavelength lambda ~ U(380, 780) nm, 5 nm
cells, a square domain of 2r + 2 lambda plus 20 cells (10-cell UPML on each
side), and 12 optical periods of steps (period = lambda_s / 0.7071 steps,
lambda_s = lambda / h_u, field.c:100-106), MPI_TM_UPML with the CW source.
The far field of each instance is ntffTM_Frequency (360 angles, FP64) of its
final fields.

run_batch() advances every instance in one batched engine (fdtd_batch_*);
run_sequential() runs the same instances one at a time through the
single-simulation engine, the per-structure loop of the reference's driver
(main.c:114-138) on one GPU.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np

from .engine import (MODEL_CIRCLE, OPT_NTFF_MODE, OPT_TBLOCK, OPT_TBLOCK_COLS, OPT_TBLOCK_ROWS, Batch, FieldInfo,
                     Simulation)

H_U = 5
PML = 10
C_S = 0.7071  # field.h:70


@dataclass
class MieCase:
    fi: FieldInfo
    radius_nm: float
    eps: float
    lambda_nm: int

    @property
    def cells(self) -> int:
        n = self.fi.width_nm // self.fi.h_u_nm
        return n * n


def mie_sweep(n: int = 256, seed: int = 20261203 + 2, periods: float = 12.0):
    """The seeded sweep of n cylinders (cases in draw order)."""
    rng = np.random.default_rng(seed)
    r = rng.uniform(100.0, 800.0, n)
    eps = rng.uniform(1.5, 4.0, n)
    lam = np.rint(rng.uniform(380.0, 780.0, n)).astype(int)
    cases = []
    for q in range(n):
        cells = int(math.ceil((2 * r[q] + 2 * lam[q]) / H_U)) + 2 * PML
        steps = int(math.ceil(periods * (lam[q] / H_U) / C_S))
        fi = FieldInfo(cells * H_U, cells * H_U, H_U, PML, int(lam[q]), 0, steps)
        cases.append(MieCase(fi, float(r[q]), float(eps[q]), int(lam[q])))
    return cases


def run_batch(cases, precision="f32", tblock=4, cols=1, rows=0):
    """All cases in one batched engine (rows: tile height, 0 = the engine's
    choice per instance); returns (far fields [n, 360] complex, stepping
    seconds, end-to-end seconds, kernel launches)."""
    t0 = time.perf_counter()
    b = Batch("MPI_TM_UPML", [c.fi for c in cases], precision)
    b.set_option(OPT_TBLOCK, tblock)
    if cols != 1:
        b.set_option(OPT_TBLOCK_COLS, cols)
    if rows:
        b.set_option(OPT_TBLOCK_ROWS, rows)
    for s, c in zip(b.instances, cases):
        s.fill_model(MODEL_CIRCLE, [c.radius_nm, c.eps])
    for s in b.instances:
        s.synchronize()
    t1 = time.perf_counter()
    b.run()
    t2 = time.perf_counter()
    ff = np.stack([s.frequency() for s in b.instances])
    t3 = time.perf_counter()
    launches = b.launches
    b.close()
    return ff, t2 - t1, t3 - t0, launches


def run_sequential(cases, precision="f64", ntff_mode=3):
    """The cases one at a time through the single-simulation engine (one-step
    kernels; ntff_mode 3: no time-domain NTFF, the far field comes from the
    frequency NTFF at the end as in the batch); returns (far fields, stepping
    seconds, end-to-end seconds)."""
    ff = []
    t_step = 0.0
    t0 = time.perf_counter()
    for c in cases:
        s = Simulation("MPI_TM_UPML", c.fi, precision)
        s.set_option(OPT_NTFF_MODE, ntff_mode)
        s.fill_model(MODEL_CIRCLE, [c.radius_nm, c.eps])
        s.synchronize()
        a = time.perf_counter()
        s.run(c.fi.step_num)
        s.synchronize()
        t_step += time.perf_counter() - a
        ff.append(s.frequency())
        s.close()
    return np.stack(ff), t_step, time.perf_counter() - t0


def farfield_rel_err(ff, ref):
    """Per-instance relative L2 error of the complex 360-angle far field."""
    ff = np.asarray(ff)
    ref = np.asarray(ref)
    return np.linalg.norm(ff - ref, axis=1) / np.linalg.norm(ref, axis=1)
