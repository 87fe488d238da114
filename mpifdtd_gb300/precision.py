"""Error of the FP32-field engine against the FP64 engine.

FP32 mode keeps the stencil state in float2 while the NTFF accumulation, the
far-field transform and the spectrum stay FP64.  Every FP32 result is meant to
come with its error against FP64 on the same input; this module measures it:

* field relative L2 of each field component after `steps` steps,
* relative L2 of the NTFF accumulators (the time-domain far field),
* far-field error in dB: 10 log10 of the ratio of the FP32 and FP64 far-field
  intensity per angle, from the frequency-domain NTFF of the final fields
  (ntffTM_Frequency / ntffTE_Frequency; MPI solvers) or the time-domain
  far-field energy per angle, and where the run fits the reference's
  8192-point spectrum from the spectrum at the source wavelength; reported as
  the maximum over angles with non-negligible power, with the relative L2 of
  the complex frequency-domain far field beside it.
"""
from __future__ import annotations

import numpy as np

from .engine import F32, F64, Simulation


def _rel(a, b):
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / d) if d else float(np.linalg.norm(a - b))


def _db_max(p32, p64, floor=1e-3):
    p32 = np.asarray(p32, dtype=np.float64)
    p64 = np.asarray(p64, dtype=np.float64)
    keep = p64 > floor * p64.max()
    if not keep.any():
        return 0.0
    return float(np.max(np.abs(10 * np.log10(p32[keep] / p64[keep]))))


def compare_precisions(solver, fi, model, steps, eps=None):
    """Run the same case in FP64 and FP32; return the error report (dict).

    model: (model id, params) for Simulation.fill_model, or None with eps
    given as the arguments of Simulation.set_eps."""
    sims = {}
    for name, prec in (("f64", F64), ("f32", F32)):
        s = Simulation(solver, fi, prec)
        if model is not None:
            s.fill_model(*model)
        else:
            s.set_eps(*eps)
        s.run(steps)
        sims[name] = s
    a, b = sims["f32"], sims["f64"]
    names = ("Ez", "Hx", "Hy") if a.tm else ("Ex", "Ey", "Hz")
    rep = {"steps": steps, "field_rel_l2": {}, "solver": solver}
    for w, n in enumerate(names):
        rep["field_rel_l2"][n] = _rel(a.field(w), b.field(w))
    rep["ntff_rel_l2"] = max(_rel(a.ntff(w), b.ntff(w)) for w in range(3))
    if a.mpi:  # frequency-domain far field at the source wavelength (ntffTM_Frequency / ntffTE_Frequency)
        f32, f64 = a.frequency(), b.frequency()
        rep["farfield_db_max"] = _db_max(np.abs(f32) ** 2, np.abs(f64) ** 2)
        rep["farfield_rel_l2"] = _rel(f32, f64)
    else:      # time-domain far-field energy per angle
        e32 = sum(np.sum(np.abs(a.ntff(w).reshape(360, -1)) ** 2, axis=1) for w in range(3))
        e64 = sum(np.sum(np.abs(b.ntff(w).reshape(360, -1)) ** 2, axis=1) for w in range(3))
        rep["farfield_db_max"] = _db_max(e32, e64)
    if fi.step_num <= 8192:
        s32, s64 = a.spectrum(), b.spectrum()
        lam = min(max(fi.lambda_nm, 380), 700) - 380
        rep["spectrum_db_max_at_lambda"] = _db_max(s32[lam], s64[lam])
        rep["spectrum_rel_l2"] = _rel(s32, s64)
    for s in sims.values():
        s.close()
    return rep
