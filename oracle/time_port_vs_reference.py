"""Times the oracle's C restatement against the reference's own sources
compiled unmodified (oracle/_ref), one core each, on the CPU-baseline sample
(1040^2 cells of 2 nm, MPI_TM_UPML FP64 with the 360-angle NTFF), and writes
oracle/port_speed.json.  Test infrastructure: it needs the reference sources
($MPIFDTD_REFERENCE, else the REF of oracle/ref.mk), so it runs on the build
host only; bench.py reports the recorded ratio beside its CPU baseline.

    python oracle/time_port_vs_reference.py
"""
from __future__ import annotations

import json
import platform
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

from oracle.pyoracle import FieldInfo, Model, OracleSim, RefSim  # noqa: E402

SAMPLE = FieldInfo(2080, 2080, 2, 16, 500, 0, 20000)
STEPS = 30


def rate(cls, model):
    s = cls("MPI_TM_UPML", SAMPLE, model)
    s.step(3)
    t = time.perf_counter()
    s.step(STEPS)
    dt = time.perf_counter() - t
    n = (SAMPLE.width_nm // SAMPLE.h_u_nm) * (SAMPLE.height_nm // SAMPLE.h_u_nm)
    return n * STEPS / dt / 1e6


def main():
    rows = []
    models = {"circle r 400 nm": Model.circle(400),
              "morpho ridge 8 lamellae": Model.morpho(450, 80, 90, 8, 50, 0.0, 2.43)}
    for name, model in models.items():
        for rep in range(3):
            port, ref = rate(OracleSim, model), rate(RefSim, model)
            rows.append({"model": name, "port_mcell_s": port, "reference_mcell_s": ref, "ratio": port / ref})
    ratios = sorted(r["ratio"] for r in rows)
    out = {"what": "one core, 1040^2 MPI_TM_UPML FP64 with NTFF, 30 steps: oracle restatement vs the "
                   "reference's sources compiled unmodified (oracle/ref.mk)",
           "host": f"{platform.machine()} {platform.processor() or ''}".strip(),
           "ratio_port_over_reference_median": ratios[len(ratios) // 2],
           "ratio_range": [ratios[0], ratios[-1]], "runs": rows}
    (HERE / "port_speed.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps({k: out[k] for k in ("ratio_port_over_reference_median", "ratio_range")}))


if __name__ == "__main__":
    main()
