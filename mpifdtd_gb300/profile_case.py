"""Fixed cases for kernel profiling and timing (the commands under profiles/).

    python -m mpifdtd_gb300.profile_case tblock --grid 4096 --k 4 --rows 128 --steps 16 [--precision f32]
    python -m mpifdtd_gb300.profile_case gemm --m 8192 --n 8192 --kdim 8192
    python -m mpifdtd_gb300.profile_case sweep --structures 64 [--k 4 --cols 1 --batch-rows 0]
    python -m mpifdtd_gb300.profile_case onestep --solver MPI_TE_UPML --grid 4096 --precision f64 --steps 8
    python -m mpifdtd_gb300.profile_case farfield --grid 1024 [--solver MPI_TM_UPML]
    python -m mpifdtd_gb300.profile_case broadband --structures 64 --steps 2500
    python -m mpifdtd_gb300.profile_case serial --solver TM_UPML --grid 16384 --precision f32 --k 4 [--cols 1] --steps 32
    python -m mpifdtd_gb300.profile_case all ...    (tblock and gemm, the blocked case first)

tblock: the morpho ridge on a (grid + 32)^2 MPI_TM_UPML grid with temporal
blocking depth k and tile rows fixed (no autotuning), steps timed with CUDA
events on the engine's stream.  onestep: the same ridge with the one-step
kernels of any UPML solver (tm_e/tm_h, te_e/te_h).  farfield: a Mie cylinder
run with the running DFT enabled, then the frequency-domain NTFF
(frequency_kernel) and the DFT far field.  broadband: the surrogate's data
generator, one batched pulse run over `structures` lamella maps.  serial: the
ridge with a serial UPML solver (H half-step first, pulse source) blocked k
steps per launch (0: one step), the whole step timed.  gemm: C = A B^T in BF16 with FP32 output on
the surrogate's tcgen05 kernel, timed with CUDA events.  One JSON line each.
"""
from __future__ import annotations

import argparse
import json


def tblock(a):
    import torch

    import mpifdtd_gb300 as m
    side = (a.grid + 32) * 2
    sim = m.Simulation("MPI_TM_UPML", m.FieldInfo(side, side, 2, 16, 500, 0, 20000), a.precision)
    sim.fill_model(m.MODEL_MORPHO, [600.0, 80.0, 90.0, 8.0, 50.0, 0.0, 2.43, 0.0])
    sim.set_option(m.OPT_TBLOCK, a.k)
    sim.set_option(m.OPT_TBLOCK_ROWS, a.rows)
    sim.run(max(a.k, 4))
    sim.synchronize()
    st = torch.cuda.ExternalStream(sim.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sim.profile(True)
    e0.record(st)
    sim.run(a.steps)
    e1.record(st)
    e1.synchronize()
    p = sim.profile_read()
    ms = e0.elapsed_time(e1) / a.steps
    cells = sim.n_px * sim.n_py
    stencil = (p["e_half"] + p["h_half"]) / p["steps"]
    b_alg = 100 if a.precision == "f32" else 200
    print(json.dumps({"case": "tblock", "grid": [sim.n_px, sim.n_py], "precision": a.precision, "k": a.k,
                      "rows": a.rows, "steps": a.steps, "ms_per_step": ms, "gcell_per_s": cells / ms / 1e6,
                      "stencil_ms_per_step": stencil, "stencil_alg_gbs": cells * b_alg / stencil / 1e6,
                      "ntff_deposit_ms_per_step": p["ntff_deposit"] / p["steps"]}), flush=True)
    sim.close()


def onestep(a):
    import torch

    import mpifdtd_gb300 as m
    side = (a.grid + 32) * 2
    sim = m.Simulation(a.solver, m.FieldInfo(side, side, 2, 16, 500, 0, 20000), a.precision)
    sim.fill_model(m.MODEL_MORPHO, [600.0, 80.0, 90.0, 8.0, 50.0, 0.0, 2.43, 0.0])
    sim.run(4)
    sim.synchronize()
    st = torch.cuda.ExternalStream(sim.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sim.profile(True)
    e0.record(st)
    sim.run(a.steps)
    sim.flush()
    e1.record(st)
    e1.synchronize()
    p = sim.profile_read()
    ms = e0.elapsed_time(e1) / a.steps
    cells = sim.n_px * sim.n_py
    print(json.dumps({"case": "onestep", "solver": a.solver, "grid": [sim.n_px, sim.n_py], "precision": a.precision,
                      "steps": a.steps, "ms_per_step": ms, "gcell_per_s": cells / ms / 1e6,
                      "ms_per_launch": {k: v / p["steps"] for k, v in p.items() if k != "steps"}}), flush=True)
    sim.close()


def serial(a):
    import torch

    import mpifdtd_gb300 as m
    side = (a.grid + 32) * 2
    sim = m.Simulation(a.solver, m.FieldInfo(side, side, 2, 16, 500, 0, 20000), a.precision)
    sim.fill_model(m.MODEL_MORPHO, [600.0, 80.0, 90.0, 8.0, 50.0, 0.0, 2.43, 0.0])
    sim.set_option(m.OPT_TBLOCK, a.k)
    if a.cols != 1:
        sim.set_option(m.OPT_TBLOCK_COLS, a.cols)
    sim.run(8)
    sim.synchronize()
    st = torch.cuda.ExternalStream(sim.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    sim.run(a.steps)
    sim.flush()
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / a.steps
    print(json.dumps({"case": "serial", "solver": a.solver, "grid": [sim.n_px, sim.n_py], "precision": a.precision,
                      "k": a.k, "cols": a.cols, "steps": a.steps, "ms_per_step": ms,
                      "gcell_per_s": sim.n_px * sim.n_py / ms / 1e6, "status": sim.status}), flush=True)
    sim.close()


def farfield(a):
    import time

    import torch

    import mpifdtd_gb300 as m
    side = (a.grid + 20) * 5
    sim = m.Simulation(a.solver, m.FieldInfo(side, side, 5, 10, 500, 0, 4000), "f64")
    sim.fill_model(m.MODEL_CIRCLE, [0.25 * a.grid * 5, 2.25])
    sim.dft_enable(list(range(400, 701, 10)))
    sim.run(a.steps)
    sim.synchronize()
    t = time.perf_counter()
    for _ in range(3):
        sim.frequency()
    t_freq = (time.perf_counter() - t) / 3
    t = time.perf_counter()
    sim.dft_far_field()
    t_dft = time.perf_counter() - t
    torch.cuda.synchronize()
    print(json.dumps({"case": "farfield", "solver": a.solver, "grid": [sim.n_px, sim.n_py], "steps": a.steps,
                      "frequency_s": t_freq, "dft_far_field_s": t_dft}), flush=True)
    sim.close()


def broadband(a):
    import time

    from mpifdtd_gb300.surrogate.data import Generator, make_maps
    gen = Generator(group=a.structures, steps=a.steps)
    maps = make_maps(a.structures, 1)
    gen.far_field(maps)                 # first run: plan, graph
    t = time.perf_counter()
    s0 = gen.seconds
    gen.far_field(maps)
    wall = time.perf_counter() - t
    run = gen.seconds - s0
    print(json.dumps({"case": "broadband", "structures": a.structures, "steps": a.steps, "run_s": run,
                      "wall_s": wall, "structures_per_s_run": a.structures / run,
                      "structures_per_s_wall": a.structures / wall}), flush=True)
    gen.close()


def gemm(a):
    import torch

    from mpifdtd_gb300.surrogate import kernels as K
    g = torch.Generator(device="cuda").manual_seed(1)
    A = torch.randn(a.m, a.kdim, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(a.n, a.kdim, device="cuda", generator=g).to(torch.bfloat16)
    C = torch.empty(a.m, a.n, device="cuda")
    for _ in range(3):
        K.gemm(A, B, C)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record()
    for _ in range(reps):
        K.gemm(A, B, C)
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    flops = 2.0 * a.m * a.n * a.kdim
    print(json.dumps({"case": "gemm", "m": a.m, "n": a.n, "k": a.kdim, "ms": ms, "tflops": flops / ms / 1e9,
                      "err_word": int(K.err_word().item())}), flush=True)


def sweep(a):
    from mpifdtd_gb300.sweep import mie_sweep, run_batch
    cases = mie_sweep(a.structures)
    cell_steps = sum(c.cells * c.fi.step_num for c in cases)
    _, t, _, launches = run_batch(cases, "f32", tblock=a.k, cols=a.cols, rows=a.batch_rows)
    print(json.dumps({"case": "sweep", "structures": a.structures, "k": a.k, "cols": a.cols, "rows": a.batch_rows,
                      "seconds": t,
                      "structures_per_s": a.structures / t, "gcell_per_s": cell_steps / t / 1e9, "launches": launches}),
          flush=True)


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m mpifdtd_gb300.profile_case")
    ap.add_argument("case", choices=["tblock", "gemm", "sweep", "onestep", "farfield", "broadband", "serial", "all"])
    ap.add_argument("--solver", default="MPI_TM_UPML")
    ap.add_argument("--structures", type=int, default=64)
    ap.add_argument("--cols", type=int, default=1)
    ap.add_argument("--batch-rows", type=int, default=0, help="sweep: tile rows (0: the engine's choice)")
    ap.add_argument("--grid", type=int, default=4096)
    ap.add_argument("--k", type=int, default=4)
    ap.add_argument("--rows", type=int, default=128)
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--precision", default="f32", choices=["f32", "f64"])
    ap.add_argument("--m", type=int, default=8192)
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--kdim", type=int, default=8192)
    a = ap.parse_args(argv)
    if a.case in ("tblock", "all"):
        tblock(a)
    if a.case in ("gemm", "all"):
        gemm(a)
    if a.case == "sweep":
        sweep(a)
    if a.case == "onestep":
        onestep(a)
    if a.case == "farfield":
        farfield(a)
    if a.case == "broadband":
        broadband(a)
    if a.case == "serial":
        serial(a)


if __name__ == "__main__":
    main()
