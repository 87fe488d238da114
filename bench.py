#!/usr/bin/env python3
"""Benchmark of the UPML time-stepping path (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Workload (the configuration the HBM-fraction target is quoted on): the
morpho-scale ridge on a 16416 x 16416 grid (16384^2 + 16-cell UPML per side),
2 nm cells, lambda 500 nm, 0 deg, step_num 20000, MPI_TM_UPML in FP64, with the
360-angle time-domain NTFF every step.  Ridge: 8 lamellae, 80 nm eps 2.43 /
90 nm air, lamella widths uniform in [300, 600] nm (seeded), 50 nm trunk.
One bench step is one update() + field_nextStep() over the whole grid.

value : Gcell-updates/s with the state resident in HBM (device-timed with CUDA
        events on the engine's stream; 32 GB of state, larger than L2, so no
        flush is needed between steps).
e2e   : the same metric through the C ABI with host buffers: the permittivity
        goes host->device (fdtd_set_eps), K per-step fdtd_update() calls driven
        by a host clock as simulator_calc() does, then Ez and the three NTFF
        accumulators come back device->host, all inside the timed region.
roofline : the stencil half-step pair (E + H kernels) against the measured
        HBM copy bandwidth, with the algorithmic 200 B per FP64 TM cell-update.
variants : the same workload with FP32 fields and FP64 NTFF, temporally
        blocked (depth and tile rows from fdtd_autotune), the FP32-vs-FP64
        error (field relative L2, far-field dB) on the 1044^2 Mie cylinder, and
        the batched sweep of 256 Mie cylinders (structures/s, FP32 batched
        engine against the FP64 engine structure by structure), and the
        learned far-field surrogate (trained here on FDTD data from the
        batched engine; held-out error, structures/s with and without the
        1 % FDTD audit, against the batched FDTD engine).
cpu_baseline / --impl reference : the oracle's C restatement of the reference
        (oracle/fdtd_oracle.c, the reference's own loops) on every host core,
        one independent down-scaled instance per core (the reference's own
        task parallelism, main.c:114-138).
With --gpus N > 1 every rank runs its own replica (the path is not sharded
across GPUs here), value = all ranks' cell-updates / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Gcell-updates/s & %HBM peak"
UNIT = "Gcell-updates/s"
# FieldInfo: width_nm, height_nm, h_u_nm, pml, lambda_nm, angle_deg, step_num
FIELD = (32832, 32832, 2, 16, 500, 0, 20000)
SAMPLE_FIELD = (2080, 2080, 2, 16, 500, 0, 20000)     # CPU sample: 1040^2, same ridge and cell size
B_ALG = {("tm", "f64"): 200, ("te", "f64"): 208, ("tm", "f32"): 100, ("te", "f32"): 104}


def morpho_params(seed=20261203 + 3):
    """morphoScaleModel parameters of the workload (per-lamella widths)."""
    rng = np.random.default_rng(seed)
    widths = rng.uniform(300.0, 600.0, size=8)
    # width, thick0, thick1, layers, branch, edge_rate, eps, per_lamella, widths...
    return [float(widths.max()), 80.0, 90.0, 8.0, 50.0, 0.0, 2.43, 1.0] + [float(w) for w in widths]


def workload_config():
    n = FIELD[0] // FIELD[2]
    return {
        "workload": f"morpho-scale ridge, MPI_TM_UPML FP64, {n}x{n} ({n - 32}^2 + 16-cell UPML), "
                    "2 nm cells, lambda 500 nm, 360-angle time-domain NTFF every step",
        "grid": [n, n], "cells_per_step": n * n, "h_u_nm": 2, "pml": 16,
        "lambda_nm": 500, "angle_deg": 0, "step_num": 20000, "solver": "MPI_TM_UPML", "precision": "f64",
        "model": {"kind": "morpho", "layers": 8, "thick_nm": [80, 90], "eps": 2.43,
                  "widths_nm": "uniform[300,600] seeded", "branch_nm": 50},
        "l2": "no flush: 32 GB of state per step, far larger than the 129 MB L2",
        "step": "one update() + field_nextStep() over the whole grid",
    }


# ---------------------------------------------------------------- helpers

def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""

    def summary(self):
        rows = []
        for line in (self.out or "").splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[4:8]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for _, _, flags in rows for q, f in enumerate(flags) if f.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, STREAM-style copy)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s (MEASURED_PEAKS.json absent)"


def ncu_traffic_per_cell():
    """DRAM bytes per cell-update of the E and H kernels from the committed ncu summary."""
    p = ROOT / "profiles" / "ncu_traffic.json"
    try:
        d = json.loads(p.read_text())
        return float(d["stencil_dram_bytes_per_cell"]), d.get("source", "")
    except Exception:
        return None, ""


# ---------------------------------------------------------------- CPU arms

def cpu_sample_run(steps, threads, ntff=True):
    """Oracle restatement on `threads` cores, one independent instance each
    (ntff=False: without the time-domain NTFF, to split a step's time)."""
    from oracle.pyoracle import FieldInfo, Model, oracle_bench
    p = morpho_params()
    model = Model(2, p)  # MODEL_MORPHO with the same parameter vector layout
    fi = FieldInfo(*SAMPLE_FIELD)
    dt = oracle_bench("MPI_TM_UPML", fi, model, steps, threads, ntff=ntff)
    if dt <= 0:
        raise RuntimeError("oracle sample failed")
    n = (SAMPLE_FIELD[0] // SAMPLE_FIELD[2]) * (SAMPLE_FIELD[1] // SAMPLE_FIELD[2])
    return n * steps * threads / dt / 1e9, dt, n


def grid_cells_and_path(field):
    """Cells per step and NTFF path cells (field.c:132-142: 5 cells inside the PML) of a FieldInfo."""
    n_px, n_py, pml = field[0] // field[2], field[1] // field[2], field[3]
    return n_px * n_py, 2 * ((n_px - pml - 5) - (pml + 5)) + 2 * ((n_py - pml - 5) - (pml + 5))


def cpu_baseline(steps, threads):
    """The oracle port on the down-scaled sample (the measured value), plus the
    corrections a reader needs to compare it with the 16416^2 workload: the
    sample timed again without the NTFF gives a per-cell stencil cost and a
    per-path-cell NTFF cost, which project the same cores' rate to the full
    grid, where the 360-angle NTFF is a far smaller share of a step; and the
    port's speed against the reference's own compiled sources."""
    value, dt, n = cpu_sample_run(steps, threads)
    _, dt0, _ = cpu_sample_run(steps, threads, ntff=False)
    cells_s, path_s = grid_cells_and_path(SAMPLE_FIELD)
    cells_f, path_f = grid_cells_and_path(FIELD)
    t_cell = dt0 / steps / cells_s                          # s per cell-update, per instance
    t_path = max(dt - dt0, 0.0) / steps / path_s            # s per NTFF path cell and step, per instance
    t_full = cells_f * t_cell + path_f * t_path
    out = {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{threads} independent {SAMPLE_FIELD[0] // 2}x{SAMPLE_FIELD[1] // 2} instances of the same "
                     f"ridge (2 nm cells, MPI_TM_UPML FP64 with NTFF), {steps} steps each, {dt:.1f} s",
           "ntff_share_of_step": {"sample_1040": max(dt - dt0, 0.0) / dt,
                                  "projected_16416": path_f * t_path / t_full},
           "projected_value_16416": cells_f * threads / t_full / 1e9,
           "projection": "per-cell stencil and per-path-cell NTFF costs of the sample (timed with and "
                         "without the NTFF), applied to the 16416^2 grid's cells and path; cache effects of "
                         "the larger grid are not modelled"}
    try:
        ps = json.loads((ROOT / "oracle" / "port_speed.json").read_text())
        out["port_vs_compiled_reference"] = {
            "ratio": ps["ratio_port_over_reference_median"], "range": ps["ratio_range"], "where": ps["what"],
            "host": ps["host"], "note": "measured on the build host by oracle/time_port_vs_reference.py "
                                        "(the reference sources are not on the GPU host)"}
    except (OSError, KeyError, ValueError):
        pass
    return out


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = host_threads()
    # warm-up: W steps per instance, untimed (also builds the oracle)
    if args.warmup > 0:
        cpu_sample_run(max(1, min(args.warmup, 3)), threads)
    cpu = cpu_baseline(args.steps, threads)
    value = cpu["value"]
    dt = value and (SAMPLE_FIELD[0] // 2) * (SAMPLE_FIELD[1] // 2) * args.steps * threads / (value * 1e9)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(),
        "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's loops restated in C (oracle/fdtd_oracle.c, bit-identical to the reference "
                "on its golden vectors); the reference sources are not present on this host",
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- replicas

def max_over_ranks(ms, ws, device):
    """The slowest rank's time (ms); every rank gets it."""
    if ws <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_rank, ws, t_max_ms):
    """Whole-job throughput in G units/s: every rank's units over the slowest rank's time."""
    return units_per_rank * ws / (t_max_ms * 1e-3) / 1e9


# ---------------------------------------------------------------- GPU arm

def run_gpu_arm(args):
    import torch

    import mpifdtd_gb300 as m

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    fi = m.FieldInfo(*FIELD)
    sim = m.Simulation("MPI_TM_UPML", fi, "f64")
    sim.fill_model(m.MODEL_MORPHO, morpho_params())
    cells = sim.n_px * sim.n_py
    stream = torch.cuda.ExternalStream(sim.stream)

    # warm-up
    sim.run(args.warmup)
    sim.synchronize()

    # timed region: K steps, device-timed on the engine stream
    launches0 = sim.launches
    sim.profile(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        e0.record(stream)
        sim.run(args.steps)
        sim.flush()                     # the NTFF deposit of every timed step lands before e1
        e1.record(stream)
        e1.synchronize()
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    prof = sim.profile_read()
    sim.profile(False)
    launches = sim.launches - launches0
    if sim.status != 0:
        raise RuntimeError(f"engine status {sim.status:#x}")
    t_max = max_over_ranks(ms, ws, "cuda")
    value = job_value(cells * args.steps, ws, t_max)

    # roofline of the stencil pair (E + H half-step kernels)
    peak, peak_src = measured_peak_hbm()
    stencil_ms = (prof["e_half"] + prof["h_half"]) / max(1, prof["steps"])
    b_alg = B_ALG[("tm", "f64")]
    achieved = cells * b_alg / (stencil_ms * 1e-3) / 1e9
    tr_cell, tr_src = ncu_traffic_per_cell()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": (tr_cell * cells if tr_cell else None),
                "kernel": "stencil half-step pair (tm_e_kernel + tm_h_kernel), per step",
                "bytes_per_cell_alg": b_alg, "peak_source": peak_src,
                "traffic_source": tr_src or "no committed ncu summary",
                "ms_per_launch": {"e_half": prof["e_half"] / prof["steps"], "h_half": prof["h_half"] / prof["steps"],
                                  "ntff_gather": prof["ntff_gather"] / prof["steps"],
                                  "ntff_deposit": prof["ntff_deposit"] / prof["steps"]}}

    # e2e through the C ABI with host buffers
    e2e = None if args.no_e2e else run_e2e(m, sim, args, torch)
    sim.close()
    variants = None if args.no_variants else run_variants(m, args, torch, cells, t_max / args.steps)

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            cpu = cpu_baseline(150, host_threads())
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(), "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "clocks": clk.summary(), "gpu_launches": launches,
            "hbm_frac": roofline["frac"], "variants": variants,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def time_workload(m, args, torch, solver, precision, tune):
    """The bench workload (16416^2 morpho ridge, NTFF every step) with another
    solver / precision: args.steps steps device-timed on the engine stream
    after the warm-up, the buffered NTFF deposit flushed inside the timing;
    tune: temporal blocking picked by fdtd_autotune first."""
    sim = m.Simulation(solver, m.FieldInfo(*FIELD), precision)
    sim.fill_model(m.MODEL_MORPHO, morpho_params())
    cells = sim.n_px * sim.n_py
    stream = torch.cuda.ExternalStream(sim.stream)
    sim.run(args.warmup)
    t = sim.autotune() if tune else None
    if t:
        sim.run(max(args.warmup, 2 * max(1, t["tblock"])))
    sim.synchronize()
    sim.profile(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    sim.run(args.steps)
    sim.flush()
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    prof = sim.profile_read()
    sim.profile(False)
    if sim.status != 0:
        raise RuntimeError(f"engine status {sim.status:#x}")
    sim.close()
    stencil = (prof["e_half"] + prof["h_half"]) / max(1, prof["steps"])
    b_alg = B_ALG[("tm" if "TM" in solver else "te", precision)]
    out = {"solver": solver, "precision": precision, "value": cells / (ms * 1e-3) / 1e9, "unit": UNIT,
           "ms_per_step": ms, "stencil_ms_per_step": stencil,
           "stencil_alg_gbs": cells * b_alg / (stencil * 1e-3) / 1e9, "bytes_per_cell_alg": b_alg,
           "ntff_deposit_ms_per_step": prof["ntff_deposit"] / max(1, prof["steps"])}
    if t:
        out.update(tblock=t["tblock"], tblock_rows=t["tblock_rows"], tblock_cols=t["tblock_cols"],
                   stencil_ms_per_step_one_step_kernels=[c[-1] for c in t["candidates"] if c[0] == 0][0],
                   autotune=[list(c) for c in t["candidates"]])
    else:
        out["stencil_frac_of_hbm_peak"] = out["stencil_alg_gbs"] / measured_peak_hbm()[0]
    return out


def run_variants(m, args, torch, cells, ms_f64):
    """The same workload with FP32 fields (FP64 NTFF) and temporal blocking
    picked by the engine's autotuner, the TE solver in FP64 and FP32, and the
    FP32-vs-FP64 error on config 2 (the 1044^2 Mie cylinder, TM and TE, all
    4000 steps, NTFF 20 cells inside the PML)."""
    from mpifdtd_gb300.precision import compare_precisions
    out = {}
    r = time_workload(m, args, torch, "MPI_TM_UPML", "f32", tune=True)
    r["speedup_vs_fp64"] = ms_f64 / r["ms_per_step"]
    r["note"] = "algorithmic GB/s above the HBM peak is the temporal blocking: K steps per HBM pass"
    out["fp32_tm"] = r
    if not args.no_te:
        te64 = time_workload(m, args, torch, "MPI_TE_UPML", "f64", tune=False)
        te32 = time_workload(m, args, torch, "MPI_TE_UPML", "f32", tune=True)
        te32["speedup_vs_fp64"] = te64["ms_per_step"] / te32["ms_per_step"]
        out["te_f64"], out["fp32_te"] = te64, te32
    fi = m.FieldInfo(5220, 5220, 5, 10, 500, 0, 4000, ntff_inset=20)
    out["fp32_error_vs_fp64"] = {}
    for solver in ("MPI_TM_UPML", "MPI_TE_UPML"):
        rep = compare_precisions(solver, fi, (m.MODEL_CIRCLE, [500.0, 2.25]), steps=4000)
        out["fp32_error_vs_fp64"][solver] = {
            "case": "config 2: 1044^2 Mie cylinder r 500 nm eps 2.25, lambda 500 nm, 4000 steps, "
                    "NTFF 20 cells inside the PML",
            "field_rel_l2": rep["field_rel_l2"], "ntff_rel_l2": rep["ntff_rel_l2"],
            "farfield_db_max": rep["farfield_db_max"], "farfield_rel_l2": rep.get("farfield_rel_l2")}
    if not args.no_sweep:
        out["sweep"] = run_sweep()
    if not args.no_surrogate:
        out["surrogate"] = run_surrogate()
    return out


def run_surrogate(n_train=16384, n_val=256, steps=30000, lr=6e-4, views=4, audit_frac=0.01):
    """The learned far-field surrogate against the batched FDTD engine.

    Data: seeded random lamella maps (256^2, eps {1, 2.43}), each simulated
    once by the batched FP32 engine with the Gaussian pulse and a running DFT
    (fdtd_batch_broadband) to the 360-angle far-field intensity at 31
    wavelengths (400..700 nm).  The network (Fourier neural operator,
    tcgen05 BF16 kernels) trains on n_train maps plus their mirror images,
    each minibatch structure randomly translated within its map (same far-field
    intensity), and is evaluated on n_val held-out maps (relative L2 error of
    the 31 x 360 intensity per structure), its prediction averaged over
    `views` symmetric views (the map, its mirror image, translations).
    Screening: the network predicts, 1 % of each screening batch is audited
    by FDTD, a batch whose audit exceeds the tolerance is re-simulated by FDTD
    (measured, fallback included).  The audit alone costs 1 % of the FDTD
    work, so the screening rate is at most 1 / audit_frac = 100x the FDTD
    rate, whatever the network's speed."""
    import numpy as np
    from mpifdtd_gb300.surrogate import screen as S
    from mpifdtd_gb300.surrogate.data import Generator, make_maps
    from mpifdtd_gb300.surrogate.model import FNO
    import time as _time
    gen = Generator(group=256)
    t_wall = _time.perf_counter()
    maps, inten, sec = S.generate(n_train + n_val, 20261203 + 4, gen)
    t_wall = _time.perf_counter() - t_wall
    fdtd_rate = (n_train + n_val) / sec
    net = FNO(seed=1)
    t_train = S.train(net, maps[:n_train], inten[:n_train], steps=steps, batch=128, lr=lr, shift=True)
    ev = S.evaluate(net, maps[n_train:], inten[n_train:], inten[:n_train], views=views)
    ev1 = S.evaluate(net, maps[n_train:], inten[n_train:])
    rate = S.inference_rate(net)
    out = {
        "unit": "structures/s (31 wavelengths x 360 angles each)",
        "fdtd_batched_fp32": {"structures_per_s": fdtd_rate, "seconds": sec, "structures": n_train + n_val,
                              "generator": "broadband: one Gaussian-pulse run of 2500 steps per map, running DFT "
                                           "at the 31 wavelengths (fdtd_batch_broadband), 256 maps per batch",
                              "timing": "the batch runs (fdtd_batch_run); the ratios below use this rate",
                              "structures_per_s_wall": (n_train + n_val) / t_wall,
                              "wall": "map generation, permittivity upload, runs and the far-field read-out"},
        "audit_fraction": audit_frac,
        "audit_ceiling_vs_fdtd": 1.0 / audit_frac,
        "training": {"maps": n_train, "with_mirror_images": 2 * n_train, "random_translations": True,
                     "steps": steps, "batch": 128, "lr": lr, "seconds": t_train},
        "heldout_rel_l2": ev, "views": views, "heldout_rel_l2_one_view": ev1,
        "network_structures_per_s": rate, "network_vs_fdtd": rate / fdtd_rate,
        "network_structures_per_s_with_views": rate / views,
    }
    # the screening path at the 2 % tolerance (fallback measured), and the cost
    # of the 1 % audit alone (a tolerance no audit exceeds: the throughput the
    # pipeline keeps when its audits pass)
    # (the audit-only line screens 16384 maps in one batch: its 164 audits run as one FDTD batch near the
    # generator's own efficiency, which a 41-map audit of a 4096-map batch does not reach)
    for key, tol, n in (("screen_tol_0.02", 0.02, 256), ("screen_audit_only", float("inf"), 16384)):
        screen_maps = make_maps(n, 20261203 + 40)
        k = max(1, int(np.ceil(audit_frac * n)))
        audit_gen = Generator(group=k)
        _, st = S.screen(net, screen_maps, gen, audit_frac=audit_frac, tol=tol, batch=n, audit_gen=audit_gen,
                         views=views)
        audit_gen.close()
        out[key] = {"structures": n, "tolerance": tol if tol != float("inf") else None,
                    "structures_per_s": st["structures_per_s"], "vs_fdtd": st["structures_per_s"] / fdtd_rate,
                    "fallback_batches": st["fallback_batches"], "batches": st["batches"],
                    "audit_rel_l2": st["audit_errors"]}
    # The gate: a screening batch keeps the network's answers only if all k of its audits are within the
    # tolerance; with a fraction p of structures within it, that happens with probability about p^k.
    p = ev["within_2pct"]
    out["gate_at_0.02"] = {
        "within_tolerance_fraction": p,
        "pass_probability": {"3_audits_(256_maps)": p ** 3, "41_audits_(4096_maps)": p ** 41},
        "target_met": bool(out["screen_tol_0.02"]["vs_fdtd"] >= 100 and out["screen_tol_0.02"]["fallback_batches"] == 0),
        "why": f"the held-out error straddles the 2 % tolerance (median {100 * ev['median']:.2f} %, p90 "
               f"{100 * ev['p90']:.2f} %), so a batch whose audits all pass is a matter of chance and a 4096-map "
               "batch almost always falls back; with 1 % audited, the screening rate cannot exceed 100x the FDTD "
               "rate even with a free network",
    }
    gen.close()
    return out


def run_sweep():
    """The batched Mie sweep: 256 seeded cylinders (r 100-800 nm, eps 1.5-4.0,
    lambda 380-780 nm, 5 nm cells, 236^2..643^2 grids, 12 periods), FP32 fields
    in one batched engine against the FP64 engine run structure by structure,
    far field from the FP64 frequency NTFF (360 angles) of each."""
    from mpifdtd_gb300.sweep import farfield_rel_err, mie_sweep, run_batch, run_sequential
    cases = mie_sweep(256)
    cell_steps = sum(c.cells * c.fi.step_num for c in cases)
    ff32, t32, e2e32, launches = run_batch(cases, "f32", tblock=4)
    ff64, t64, e2e64 = run_sequential(cases, "f64")
    err = farfield_rel_err(ff32, ff64)
    return {
        "workload": "256 Mie cylinders, MPI_TM_UPML, 12 optical periods each, FP64 frequency NTFF at 360 angles",
        "unit": "structures/s", "cell_updates": cell_steps,
        "batched_fp32": {"structures_per_s": len(cases) / t32, "gcell_per_s": cell_steps / t32 / 1e9,
                         "seconds": t32, "e2e_seconds": e2e32, "gpu_launches": launches,
                         "tblock": 4, "timing": "wall clock around fdtd_batch_run (synchronous)"},
        "sequential_fp64": {"structures_per_s": len(cases) / t64, "gcell_per_s": cell_steps / t64 / 1e9,
                            "seconds": t64, "e2e_seconds": e2e64,
                            "timing": "wall clock around each fdtd_run + synchronize, summed"},
        "speedup_fp32_batched_vs_fp64": t64 / t32,
        "farfield_rel_l2_fp32_vs_fp64": {"max": float(err.max()), "median": float(np.median(err))},
    }


def run_e2e(m, sim, args, torch):
    """K steps through the C ABI with host buffers, copies inside the timed region."""
    n_px, n_py = sim.n_px, sim.n_py
    n = n_px * n_py
    # the workload's EPS_EZ as a host program holds it: written by the CPU into pinned memory
    staging = torch.empty(n, dtype=torch.float64, pin_memory=True)
    sim.eps_into(0, staging.data_ptr())
    eps_h = torch.empty(n, dtype=torch.float64, pin_memory=True)
    eps_h.copy_(staging)                                   # CPU copy
    del staging
    ez_h = torch.empty(2 * n, dtype=torch.float64, pin_memory=True)
    nt_len = 360 * sim.array_size
    nt_h = [torch.empty(2 * nt_len, dtype=torch.float64, pin_memory=True) for _ in range(3)]
    for b in [ez_h] + nt_h:                                # first touch of the host pages, outside the timing
        b.zero_()

    def one_pass():
        sim.reset()
        sim.synchronize()
        t = time.perf_counter()
        sim.set_eps_ptr(eps_h.data_ptr())                  # H2D
        sim.synchronize()
        t_in = time.perf_counter()
        clock, ray = 0.0, 0.0
        for _ in range(args.steps):                        # simulator_calc(): update() then field_nextStep()
            sim.update(clock, ray)
            clock += 1.0
            ray = 1.0 - float(np.exp(-(0.01 * clock) ** 2))
        sim.synchronize()
        t_steps = time.perf_counter()
        sim.field_into(0, ez_h.data_ptr())                 # D2H
        for w in range(3):
            sim.ntff_into(w, nt_h[w].data_ptr())
        return t_in - t, t_steps - t_in, time.perf_counter() - t_steps

    # one untimed pass of the same sequence first (the GPU leaves its idle clocks; one cold pass measured
    # 0.27-0.34 s with 0.1 s moving between its copy and step phases from run to run)
    first = one_pass()
    s_in, s_steps, s_out = one_pass()
    dt = s_in + s_steps + s_out
    h2d = n * 8
    d2h = n * 16 + 3 * nt_len * 16
    return {"value": n * args.steps / dt / 1e9, "unit": UNIT, "h2d_bytes_per_step": h2d / args.steps,
            "d2h_bytes_per_step": d2h / args.steps, "seconds": dt, "untimed_first_pass_s": sum(first),
            "split_s": {"h2d": s_in, "steps": s_steps, "d2h": s_out},
            "copy_gbs": {"h2d": h2d / max(s_in, 1e-9) / 1e9, "d2h": d2h / max(s_out, 1e-9) / 1e9},
            "path": "fdtd_set_eps (pinned host) + fdtd_update x K + fdtd_get_field/fdtd_get_ntff (pinned host)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-variants", action="store_true", help="skip the FP32 / temporal-blocking line items")
    ap.add_argument("--no-sweep", action="store_true", help="skip the batched 256-structure sweep")
    ap.add_argument("--no-te", action="store_true", help="skip the TE lines of the 16416^2 workload")
    ap.add_argument("--no-surrogate", action="store_true", help="skip the learned-surrogate line item")
    ap.add_argument("--grid", type=int, default=0,
                    help="interior cells per side for a smaller case of the same workload (profiling)")
    args = ap.parse_args()
    if args.grid:
        global FIELD
        side = (args.grid + 2 * FIELD[3]) * FIELD[2]
        FIELD = (side, side) + FIELD[2:]
    if args.warmup < 3:
        args.warmup = 3
    if args.warmup + args.steps > FIELD[6]:
        raise SystemExit("steps + warmup must not exceed step_num (20000)")
    if args.impl == "reference":
        return run_reference_arm(args)
    return run_gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
