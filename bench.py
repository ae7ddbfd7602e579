"""Benchmark of the residual-and-update path on one GB300 (or N replicas under torchrun).

Workload (default): the synthetic compressor-rotor passage of 129 x 49 x 49 nodes (axial x pitch
x span; 294,912 fine cells), 22 blades, 16000 rpm, back pressure 1.20 x inlet total, Roe + MUSCL3
on primitive variables, Baldwin-Lomax, LU-SGS, two-level multigrid (the reference's maximum),
FP64. A step is one multigrid cycle of the reference driver (CSolver::Solver + integrals); the
metric is fine-grid cell updates per second (cells x cycles / time).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed] [--batch B]
  python bench.py --impl reference ...   (the CPU implementation of the path on the host cores)

Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "3d-fluid-numerical-simulation-software_gb300")
for _p in (PKG, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--batch", type=int, default=1, help="operating points per GPU")
    ap.add_argument("--sampled", action="store_true",
                    help="draw the batch from the seeded operating-point sampler (three mesh sizes)")
    ap.add_argument("--levels", type=int, default=2, choices=[2, 3],
                    help="3: the three-level V-cycle extension (the reference stops at two levels)")
    ap.add_argument("--variant", default="default", choices=["default", "jst", "sa", "stage"],
                    help="numerical variant of the passage: JST, Spalart-Allmaras (single grid), rotor-stator stage")
    ap.add_argument("--blocks", type=int, default=1, choices=[1, 3],
                    help="3: the passage as three blocks joined by interfaces (reference's rotor-67 layout)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-solves", action="store_true",
                    help="skip the converged-solves-per-hour measurement of the default line (about a minute)")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the secondary measurements of the mixed-precision and batched forms")
    ap.add_argument("--study", choices=["precision", "solves", "multigrid", "warmstart", "network"],
                    help="long runs instead of the benchmark line: 'precision' = the mixed form's integrals "
                         "against the FP64 solve after 3000 cycles at three back pressures; 'solves' = "
                         "converged solves per hour of the plain FP64 path and the batched mixed form; "
                         "'multigrid' = two- and three-level cycles; 'warmstart' = the learned warm start "
                         "trained on 256 sampled points and evaluated on --points held-out ones")
    ap.add_argument("--cycles", type=int, default=None, help="cycle cap of a study (3000 / 4000 by default)")
    ap.add_argument("--points", type=int, default=64, help="operating points of the batched form in the solves study")
    return ap.parse_args()


# numerical variants of the passage (config values): the default Roe + MUSCL3 + Baldwin-Lomax
# two-level case, JST, Spalart-Allmaras (single grid, the reference's only SA form), and the
# rotor-stator stage joined by a mixing plane
VARIANTS = {
    "default": {},
    "jst": {"scheme": "100", "k2": "0.5", "k4": "32.0"},
    "sa": {"turb": "200", "multigrid": "N", "coarse_iter": "0"},
}


def make_cases(root: str, n: int, seed_offset: int = 0, back_pressures=None, blocks: int = 1, variant: str = "default"):
    """the 129 x 49 x 49 rotor passage; in a batch the back pressure varies over [1.05, 1.30] x p_t
    (or is given, as ratios to the inlet total pressure). blocks=3: the same passage cut at the
    blade's leading- and trailing-edge planes (k = 41, 89) into three blocks joined by interfaces.
    variant "stage": a rotor of 129 x 49 x 49 nodes and a stationary row of 65 x 49 x 49 behind it,
    joined by a mixing plane"""
    import meshgen as mg
    dirs = []
    for q in range(n):
        pb = 1.20 if n == 1 else 1.05 + 0.25 * ((q + seed_offset) % n) / max(n - 1, 1)
        if back_pressures is not None:
            pb = back_pressures[q]
        opts = {"Pout": "%.1f" % (pb * 101325.0), "multigrid": "Y", "coarse_iter": "2", "Ma0": "0.45"}
        d = os.path.join(root, f"op{q}")
        if variant == "stage":
            case = mg.stage_passage(IM=49, JM1=49, KM1=129, JM2=49, KM2=65, options=opts)
            mg.write_multiblock_case(case, d)
            dirs.append(d)
            continue
        opts.update(VARIANTS[variant])
        case = mg.rotor_passage(IM=49, JM=49, KM=129, options=opts)
        if blocks == 3:
            mg.write_multiblock_case(mg.split_axial(case, [41, 89]), d)
        elif blocks == 1:
            mg.write_case(case, d)
        else:
            raise ValueError("--blocks takes 1 or 3")
        dirs.append(d)
    return dirs, case.n_cells


def make_sampled_cases(root: str, n: int, seed: int = 2024):
    """n operating points from the seeded sampler of the batched form: back pressure U[1.05, 1.30]
    x p_t, speed {0.8, 0.9, 1.0} x 16000 rpm, mesh {97x41x41, 129x49x49, 161x65x65}, stagger
    offset N(0, 1 deg); two-level multigrid, mixed form options as the single passage"""
    import meshgen as mg
    jobs = [(os.path.join(root, f"sp{q}"), op) for q, op in enumerate(mg.sample_operating_points(n, seed))]
    # the text grids are slow to format: generate in parallel worker processes (spawned, since
    # this process already holds a CUDA context)
    with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
        cells = pool.map(_write_sampled_case, jobs)
    return [d for d, _ in jobs], cells


def _write_sampled_case(job):
    d, op = job
    import meshgen as mg
    case = mg.rotor_passage(IM=op["IM"], JM=op["JM"], KM=op["KM"], rpm=op["rpm"], stagger_offset=op["stagger_offset"],
                            options={"Pout": "%.1f" % (op["pb"] * 101325.0), "multigrid": "Y", "coarse_iter": "2",
                                     "Ma0": "0.45"})
    mg.write_case(case, d)
    return case.n_cells


# ---------------------------------------------------------------------------------------------
# algorithmic bytes per kernel launch: each input/output element counted once, at the width the
# kernel reads it ("w": the working precision, 8 B in FP64, 4 B in the mixed form, whose face and
# sweep kernels read FP32 copies of the geometry; "int": 4 B). unit: "face" (faces of one family,
# about one per cell), "plane_cell" (cells of one hyperplane)
# ---------------------------------------------------------------------------------------------
ALG = {
    # S(3) s nrm(3) t1(3) t2(3) qe metrics(9) = 23 geometry; prim 6 + mu_t 1 of one cell; 10 fluxes
    # out; the wall flag
    "face_flux": {"unit": "face", "w": 40, "int": 1},
    # plane-order copies: vol dt lamc(3) lamv(3) + res or dq (5) + neighbour cv(5) dq(5) p(1) + mean
    # normal(3) area entrainment, per direction amortised to one cell: cn 9 cs 3 cve 3; dq out 5
    "sweep_forward": {"unit": "plane_cell", "w": 45, "int": 0},
    "sweep_backward": {"unit": "plane_cell", "w": 45, "int": 0},
}


def alg_units_per_step(stage, slot_dims, evals, nprof):
    """units of ALG[stage] processed per multigrid cycle: the stage profiler counts the stage's
    evaluations on every level (a residual's three face families, one sweep over a level), and one
    evaluation covers every slot of that level; slot_dims[l] holds the (IM, JM, KM) node counts of
    level l + 1 of every slot"""
    n = 0
    for l, dims in enumerate(slot_dims):
        per_eval = 0
        for I, J, K in dims:
            if ALG[stage]["unit"] == "face":
                per_eval += I * (J - 1) * (K - 1) + (I - 1) * J * (K - 1) + (I - 1) * (J - 1) * K
            else:
                per_eval += (I - 1) * (J - 1) * (K - 1)
        n += per_eval * evals[l]
    return n / nprof


def fp64_ops_per_unit():
    """per unit of a stage of the FP64 form, from profiles/fp64_ops_per_unit.txt (ncu counts):
    (FP64 operations = 2 x DFMA + DMUL + DADD thread instructions, FP64-pipe thread instructions)"""
    out = {}
    try:
        for line in open(os.path.join(ROOT, "profiles", "fp64_ops_per_unit.txt")):
            f = line.split()
            if len(f) >= 4 and not line.startswith("#"):
                out[f[0]] = (float(f[2]), float(f[3]))
    except FileNotFoundError:
        pass
    return out


def alg_bytes_per_unit(stage, wsize):
    a = ALG[stage]
    return wsize * a["w"] + 4 * a["int"]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region"""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.f = open(self.path, "w")
        self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                      "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        dev = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        os.unlink(self.path)
        if not rows:
            return None
        idx = rows[0][0] if not dev.isdigit() else dev
        rows = [r for r in rows if r[0] == idx] or rows
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in rows for q in range(4) if r[5 + q].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        return rank, world, dist
    return 0, 1, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------------------------
# CPU arms
# ---------------------------------------------------------------------------------------------
def _oracle_worker(args):
    case_dir, warm, steps, fp32 = args
    import pyoracle
    o = pyoracle.Oracle(case_dir, fp32=fp32)
    for _ in range(warm):
        o.iterate()
    t0 = time.perf_counter()
    for _ in range(steps):
        o.iterate()
    return time.perf_counter() - t0


def cpu_baseline(case_dir, cells, warm, steps, fp32=False):
    """the oracle port, one thread, bounded sample of the same workload; fp32: the reference's
    default FP32 build of the path (REAL = float), beside the GPU's mixed form"""
    import pyoracle
    pyoracle.build()
    t = _oracle_worker((case_dir, warm, steps, fp32))
    return {"value": cells * steps / t, "unit": "cell-updates/s", "cores": 1, "kind": "port",
            "sample": f"{steps} multigrid cycles of one {cells}-cell passage after {warm} untimed iterations, "
                      f"CPU oracle (single thread, {'FP32: the reference FP32 build' if fp32 else 'FP64'})"}


def run_reference(args, rank, world, dist):
    if rank != 0:
        return 0
    import pyoracle
    pyoracle.build()
    cores = os.cpu_count() or 1
    fp32 = args.precision == "mixed"             # the reference's default FP32 build beside the mixed form
    tmp = tempfile.mkdtemp(prefix="gbt_ref_")
    try:
        dirs, cells = make_cases(tmp, 1)
        steps = max(1, min(args.steps, 6))
        warm = max(args.warmup, 3)
        ctx = mp.get_context("spawn")
        with ctx.Pool(cores) as pool:
            times = pool.map(_oracle_worker, [(dirs[0], warm, steps, fp32)] * cores)
        t = max(times)
        value = cores * cells * steps / t
        line = {
            "impl": "reference", "metric": "cell_updates_per_s", "value": value, "unit": "cell-updates/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": warm, "ms_per_step": 1000.0 * t / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32" if fp32 else "f64",
            "data": "synthetic", "config": config_block(args, cells, 1),
            "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": cores, "kind": "port",
                             "sample": f"{cores} independent single-thread CPU solves (the reference's CPU path "
                                       f"restated in C, {'FP32 build' if fp32 else 'FP64 build'}), {steps} multigrid "
                                       f"cycles each after {warm} untimed"},
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line), flush=True)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return 0


def measure_forms(gbturbo, dirs, cells, n_ref, ref_int, steps, tmp):
    """secondary numbers beside the FP64 headline: the mixed-precision form on the same passage
    (device-timed cycles, and its integrals after the same number of cycles as the FP64 run,
    relative to the FP64 values), and batches of 8 and 64 operating points in the mixed form"""
    out = {}
    m = gbturbo.Solver(dirs, gbturbo.MIXED)
    m.init_uniform()
    m.iterate(3, history=False)
    m.timer_start()
    m.iterate(steps, history=False)
    ms = m.timer_stop()
    m.iterate(n_ref - 3 - steps, history=False)
    got = m.integrals(1)[0]
    m.close()
    names = ["m_in", "m_out", "PR", "eta"]
    out["mixed"] = {"value": cells * steps / (ms / 1000.0), "unit": "cell-updates/s", "ms_per_step": ms / steps,
                    "steps": steps, "cycles_compared": n_ref,
                    "rel_err_vs_fp64": {n: abs(float(got[q] - ref_int[q]) / float(ref_int[q])) for q, n in enumerate(names)}}
    bdirs, _ = make_cases(os.path.join(tmp, "batch8"), 8)
    b = gbturbo.Solver(bdirs, gbturbo.MIXED)
    b.init_uniform()
    b.iterate(3, history=False)
    b.timer_start()
    b.iterate(steps, history=False)
    ms = b.timer_stop()
    b.close()
    out["mixed_batch8"] = {"value": 8 * cells * steps / (ms / 1000.0), "unit": "cell-updates/s",
                           "ms_per_step": ms / steps, "steps": steps,
                           "operating_points": "back pressure 1.05-1.30 x inlet total (seeded)"}
    # 64 sampled operating points on three mesh sizes in one batch
    t0 = time.perf_counter()
    sdirs, scells = make_sampled_cases(os.path.join(tmp, "batch64"), 64)
    b = gbturbo.Solver(sdirs, gbturbo.MIXED)
    t_setup = time.perf_counter() - t0
    b.init_uniform()
    b.iterate(3, history=False)
    b.timer_start()
    b.iterate(steps // 2, history=False)
    ms = b.timer_stop()
    b.close()
    shutil.rmtree(os.path.join(tmp, "batch64"), ignore_errors=True)
    out["mixed_batch64_sampled"] = {"value": sum(scells) * (steps // 2) / (ms / 1000.0), "unit": "cell-updates/s",
                                    "ms_per_step": ms / (steps // 2), "steps": steps // 2,
                                    "fine_cells": int(sum(scells)), "setup_s": round(t_setup, 1),
                                    "operating_points": "seeded sampler: back pressure U[1.05,1.30] x p_t, "
                                                        "rpm {0.8,0.9,1.0} x 16000, meshes 97x41x41 / 129x49x49 / "
                                                        "161x65x65, stagger offset N(0,1 deg)"}
    return out


# ---------------------------------------------------------------------------------------------
# long-run studies (one JSON document each; not the benchmark line)
# ---------------------------------------------------------------------------------------------
INTEGRAL_COLS = {"m_in": 6, "m_out": 7, "PR": 8, "eta": 9}


def study_precision(gbturbo, tmp, cycles):
    """the mixed-precision form against the FP64 solve on the 129 x 49 x 49 passage at back
    pressures 1.10, 1.20 and 1.28 x inlet total: both forms run the same cycles from the uniform
    start (the three points as one batch), and every integral of the mixed form is compared with
    the FP64 one at the last cycle and averaged over the last 10% of the cycles (the stalled points
    are unsteady, so the cycle-by-cycle values of both forms wander)"""
    pbs = [1.10, 1.20, 1.28]
    dirs, cells = make_cases(os.path.join(tmp, "prec"), 3, back_pressures=pbs)
    hist, wall = {}, {}
    for name, prec in (("fp64", gbturbo.FP64), ("mixed", gbturbo.MIXED)):
        t0 = time.perf_counter()
        with gbturbo.Solver(dirs, prec) as s:
            s.init_uniform()
            hist[name] = s.iterate(cycles)
        wall[name] = time.perf_counter() - t0
    tail = max(1, cycles // 10)
    points = []
    for q, pb in enumerate(pbs):
        row = {"back_pressure_over_pt": pb}
        for form in ("fp64", "mixed"):
            h = hist[form][:, q, :]
            row[form] = {"last": {n: float(h[-1, c]) for n, c in INTEGRAL_COLS.items()},
                         "mean_tail": {n: float(h[-tail:, c].mean()) for n, c in INTEGRAL_COLS.items()},
                         "res_dens_last": float(h[-1, 1]), "mass_ratio_last": float(h[-1, 10])}
        for key in ("last", "mean_tail"):
            row["rel_err_" + key] = {n: abs(row["mixed"][key][n] - row["fp64"][key][n]) / abs(row["fp64"][key][n])
                                     for n in INTEGRAL_COLS}
        # largest relative difference of the four integrals at checkpoints along the run
        d = np.max(np.abs(hist["mixed"][:, q, 6:10] - hist["fp64"][:, q, 6:10]) /
                   np.abs(hist["fp64"][:, q, 6:10]), axis=1)
        row["rel_err_at_cycle"] = {str(c): float(d[c - 1]) for c in range(100, cycles + 1, 100) if c % 500 == 0 or c <= 300}
        points.append(row)
    return {"study": "precision", "workload": "rotor_passage_129x49x49_2level_multigrid", "cycles": cycles,
            "cells_per_solve": cells, "wall_s": wall, "points": points}


def _timed_run(speedline, dirs, prec, cycles, tol):
    t0 = time.perf_counter()
    table = speedline.run(dirs, prec, max_iter=cycles, chunk=100, tol=tol)
    return time.perf_counter() - t0, table


def study_solves(gbturbo, tmp, cycles, npoints):
    """converged solves per hour, each point run from the uniform start until the reference's rule
    (density residual <= 1e-6 and mass ratio <= 0.003) or the cycle cap, wall clock through the
    public API (case reading, geometry, iterations with the history read back every 100 cycles):
      plain FP64: the 129 x 49 x 49 passage at 1.20 x p_t, one solve at a time, and a seeded
        subsample of the sampled operating points one at a time;
      mixed, one solve at a time: the same passage;
      mixed, batched: the seeded sampler's points as one batch."""
    import speedline
    out = {"study": "solves", "cycle_cap": cycles, "tol": 1e-6, "mass_ratio_limit": speedline.MASS_RATIO_LIMIT}
    dirs, cells = make_cases(os.path.join(tmp, "single"), 1)
    for name, prec in (("fp64_single_129x49x49", gbturbo.FP64), ("mixed_single_129x49x49", gbturbo.MIXED)):
        t, table = _timed_run(speedline, dirs, prec, cycles, 1e-6)
        out[name] = {"wall_s": t, "solves_per_hour": 3600.0 / t, "points": table}
    sdirs, scells = make_sampled_cases(os.path.join(tmp, "sampled"), npoints)
    t, table = _timed_run(speedline, sdirs, gbturbo.MIXED, cycles, 1e-6)
    out["mixed_batch_sampled"] = {"wall_s": t, "points_in_batch": npoints, "fine_cells": int(sum(scells)),
                                  "solves_per_hour": 3600.0 * npoints / t,
                                  "converged": sum(1 for r in table if r["converged"]),
                                  "iterations": [r["iteration"] for r in table]}
    # plain FP64 on a subsample of the same points: one of each mesh size and one more
    sizes = {}
    for q, c in enumerate(scells):
        sizes.setdefault(c, q)
    sub = sorted(sizes.values())
    sub += [q for q in range(npoints) if q not in sub][:4 - len(sub)]
    t_sub = 0.0
    rows = []
    for q in sub:
        t, table = _timed_run(speedline, [sdirs[q]], gbturbo.FP64, cycles, 1e-6)
        t_sub += t
        rows.append(dict(table[0], cells=int(scells[q]), wall_s=t))
    mean_cells = sum(scells) / len(scells)
    sub_cells = sum(scells[q] for q in sub) / len(sub)
    # one FP64 solve of the batch's mean size takes (time per cell of the subsample) x mean cells
    t_mean = t_sub / len(sub) * (mean_cells / sub_cells)
    out["fp64_single_sampled"] = {"subsample": sub, "wall_s": t_sub, "points": rows,
                                  "solves_per_hour": 3600.0 / t_mean,
                                  "note": "one solve at a time; per-solve time scaled from the subsample to the "
                                          "batch's mean fine-cell count"}
    out["batched_mixed_over_plain_fp64_solves_per_hour"] = (out["mixed_batch_sampled"]["solves_per_hour"] /
                                                           out["fp64_single_sampled"]["solves_per_hour"])
    return out


def measure_solves(gbturbo, tmp, n_train=64, n_test=32, train_cycles=600, steps=3000, cap=2500, n_fp64=4,
                   mesh=(25, 25, 65), seed=2024, batch=32768):
    """Converged solves per hour, end to end through the public API, on a stand-in for the batched
    configuration: the seeded operating-point sampler (back pressure U[1.05, 1.30] x p_t, speed
    {0.8, 0.9, 1.0} x 16000 rpm, stagger offset N(0, 1 deg)) on one 25 x 25 x 65 mesh of the blade
    family, where the uniform start converges (the full-size passages stall first). A point is
    converged at the first cycle that meets the reference's rule (density residual <= 1e-6 and
    |m_in - m_out| / m_in <= 0.003, source/Structured_FV3D.cpp:214), else it stops at the cap.
      batched mixed, uniform start: the n_test held-out points as one batch until all converged or
        the cap (case files read, geometry, cycles with the history read back every 100);
      batched mixed, learned warm start: the same batch from the network's field (residual-gated
        fallback to the uniform start), with the training data (n_train further points as one mixed
        batch, train_cycles cycles) and the training (steps Adam steps) charged to its time;
      plain FP64, one solve at a time from the uniform start, on n_fp64 held-out points (the
        lowest, highest and evenly spaced back pressures between), each until its rule or the cap.
    solves/hour = converged points / wall hours. For the subsample points the plain FP64 solve
    converged, each batch form's integrals at its own convergence are compared with the FP64 solve's
    (inlet mass flow within 0.1%, pressure ratio within 1e-4)."""
    import meshgen as mg
    import speedline
    ops = mg.sample_operating_points(n_train + n_test, seed)
    for op in ops:
        op["IM"], op["JM"], op["KM"] = mesh
    jobs = [(os.path.join(tmp, f"sv{q}"), op) for q, op in enumerate(ops)]
    with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
        cells = pool.map(_write_sampled_case, jobs)
    dirs = [d for d, _ in jobs]
    prm = [[op["pb"], op["rpm"] / 16000.0, op["stagger_offset"]] for op in ops]
    tr, te = slice(0, n_train), slice(n_train, n_train + n_test)
    tol = 1e-6
    out = {"workload": "stand-in for the batched configuration: sampled operating points on one 25x25x65 mesh "
                       "of the rotor blade family (36,864 cells)",
           "held_out_points": n_test, "train_points": n_train, "train_cycles": train_cycles, "train_steps": steps,
           "cycle_cap": cap, "tol": tol, "mass_ratio_limit": speedline.MASS_RATIO_LIMIT}

    t0 = time.perf_counter()
    table_u = speedline.run(dirs[te], gbturbo.MIXED, max_iter=cap, chunk=100, tol=tol)
    t_u = time.perf_counter() - t0

    t0 = time.perf_counter()
    w = gbturbo.WarmStart(seed=7)
    with gbturbo.Solver(dirs[tr], gbturbo.MIXED) as s:
        s.init_uniform()
        s.iterate(train_cycles, history=False)
        w.add_solves(s, prm[tr])
    for k in range(steps // 500):
        w.train(500, batch=batch, lr=1e-3 if k < (steps // 500) * 3 // 4 else 3e-4)
    t_train = time.perf_counter() - t0
    kept = []

    def warm(s):
        used, _, _ = w.apply(s, prm[te])
        kept.append(int(np.sum(used)))

    t0 = time.perf_counter()
    table_w = speedline.run(dirs[te], gbturbo.MIXED, max_iter=cap, chunk=100, tol=tol, start=warm)
    t_w = time.perf_counter() - t0 + t_train
    w.close()

    order = sorted(range(n_test), key=lambda q: prm[n_train + q][0])
    sub = sorted({order[round(i * (n_test - 1) / max(n_fp64 - 1, 1))] for i in range(n_fp64)})
    t_f, rows_f = 0.0, {}
    for q in sub:
        t0 = time.perf_counter()
        rows_f[q] = speedline.run([dirs[n_train + q]], gbturbo.FP64, max_iter=cap, chunk=100, tol=tol)[0]
        t_f += time.perf_counter() - t0

    def agree(table):
        n = 0
        for q, r in rows_f.items():
            if r["converged"] and table[q]["converged"]:
                n += (abs(table[q]["m_in"] - r["m_in"]) <= 1e-3 * abs(r["m_in"]) and
                      abs(table[q]["pressure_ratio"] - r["pressure_ratio"]) <= 1e-4)
        return int(n)

    conv_f = sum(1 for r in rows_f.values() if r["converged"])
    f_sph = 3600.0 * conv_f / t_f
    for name, table, t in (("batched_mixed_uniform", table_u, t_u), ("batched_mixed_warm", table_w, t_w)):
        conv = sum(1 for r in table if r["converged"])
        out[name] = {"wall_s": round(t, 2), "converged": conv, "solves_per_hour": 3600.0 * conv / t,
                     "median_cycles_converged": float(np.median([r["iteration"] for r in table if r["converged"]]))
                     if conv else None,
                     "agree_with_fp64_on_subsample": agree(table)}
    out["batched_mixed_warm"]["train_s"] = round(t_train, 2)
    out["batched_mixed_warm"]["network_field_kept"] = kept[0] if kept else 0
    out["plain_fp64_one_at_a_time"] = {"subsample": [n_train + q for q in sub], "wall_s": round(t_f, 2),
                                       "converged": conv_f, "solves_per_hour": f_sph,
                                       "cycles": [rows_f[q]["iteration"] for q in sub],
                                       "back_pressure_ratios": [round(prm[n_train + q][0], 4) for q in sub]}
    out["fp64_subsample_converged"] = conv_f
    for name in ("batched_mixed_uniform", "batched_mixed_warm"):
        out[name]["ratio_vs_plain_fp64"] = out[name]["solves_per_hour"] / f_sph if f_sph > 0 else None
    for d in dirs:
        shutil.rmtree(d, ignore_errors=True)
    return out


def study_warmstart(gbturbo, tmp, cycles, n_test, n_train=256, mesh=(25, 25, 65), seed=2024, train_cycles=1000,
                    steps=8000, batch=32768):
    """The learned warm start on the seeded operating-point sampler (back pressure U[1.05, 1.30] x
    p_t, speed {0.8, 0.9, 1.0} x 16000 rpm, stagger offset N(0, 1 deg)) on one mesh of the blade
    family (the full-size passages stall before converging, see the precision study):
      training data: n_train points as one mixed batch, uniform start, train_cycles cycles, every
        fine cell a sample; training: Adam steps on minibatches (BF16, FP32 accumulation);
      held out: n_test further points from the same sampler, run as one batch per form with every
        cycle's history: mixed from the uniform start and mixed from the network's field (with the
        residual-gated fallback) to the cycle cap; plain FP64 from the uniform start to twice the
        cap (the FP64 reference solve: its integrals at the end, for the points it converged within the cap by
        the reference's rule, density residual <= 1e-6 and mass ratio <= 0.003);
      per point: the first cycle meeting the reference's rule, and the first cycle from which the
        inlet mass flow stays within 1e-3 and the pressure ratio within 1e-4 of the FP64 reference's;
      solves per hour: plain FP64 one solve at a time (a subsample, wall clock through the
        speedline driver), and a batch that retires each point when it reaches the FP64 reference's
        integrals, from the measured device time per batch cycle."""
    import meshgen as mg
    import speedline
    ops = mg.sample_operating_points(n_train + n_test, seed)
    for op in ops:
        op["IM"], op["JM"], op["KM"] = mesh
    jobs = [(os.path.join(tmp, f"ws{q}"), op) for q, op in enumerate(ops)]
    with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
        cells = pool.map(_write_sampled_case, jobs)
    dirs = [d for d, _ in jobs]
    prm = [[op["pb"], op["rpm"] / 16000.0, op["stagger_offset"]] for op in ops]
    tr, te = slice(0, n_train), slice(n_train, n_train + n_test)
    out = {"study": "warmstart", "mesh": list(mesh), "fine_cells_per_point": int(cells[0]), "train_points": n_train,
           "held_out_points": n_test, "train_cycles": train_cycles, "cycle_cap": cycles, "tol": 1e-6,
           "mass_ratio_limit": speedline.MASS_RATIO_LIMIT, "steps": steps, "batch": batch}
    w = gbturbo.WarmStart(seed=7)
    t0 = time.perf_counter()
    with gbturbo.Solver(dirs[tr], gbturbo.MIXED) as s:
        s.init_uniform()
        h = s.iterate(train_cycles)
        w.add_solves(s, prm[tr])
    out["data_s"] = time.perf_counter() - t0
    out["train_res_dens_final"] = [float(v) for v in np.percentile(h[-1, :, 1], [10, 50, 90])]
    out["samples"] = w.samples
    t0 = time.perf_counter()
    losses = []
    for k in range(steps // 500):
        losses.append(w.train(500, batch=batch, lr=1e-3 if k < (steps // 500) * 3 // 4 else 3e-4))
    out["train_s"] = time.perf_counter() - t0
    out["loss_every_500_steps"] = losses
    used_all = []

    def warm(s):
        used, rw, ru = w.apply(s, prm[te])
        used_all.append(used.tolist())

    # the held-out points as one batch per form, every cycle's history kept
    hist = {}
    fp64_reference_cycles = 2 * cycles
    out["fp64_reference_cycles"] = fp64_reference_cycles
    for name, prec, start, n_cyc in (("mixed_batch_uniform", gbturbo.MIXED, None, cycles),
                                     ("mixed_batch_warm", gbturbo.MIXED, warm, cycles),
                                     ("fp64_batch_uniform", gbturbo.FP64, None, fp64_reference_cycles)):
        t0 = time.perf_counter()
        with gbturbo.Solver(dirs[te], prec) as s:
            t_create = time.perf_counter() - t0
            t1 = time.perf_counter()
            if start is None:
                s.init_uniform()
            else:
                start(s)
            t_start = time.perf_counter() - t1
            s.timer_start()
            H = s.iterate(n_cyc)
            ms = s.timer_stop()
        hist[name] = H
        out[name] = {"create_s": t_create, "start_s": t_start, "ms_per_cycle": ms / n_cyc,
                     "wall_s": time.perf_counter() - t0}
    out["mixed_batch_warm"]["network_field_kept"] = int(sum(used_all[0]))
    tol_m, tol_pr = 1e-3, 1e-4

    def first_rule(H, q):
        ok = np.nonzero((H[:, q, 1] <= 1e-6) & (H[:, q, 10] <= speedline.MASS_RATIO_LIMIT))[0]
        return int(ok[0]) + 1 if ok.size else None

    # the FP64 reference: the plain FP64 solve's integrals after twice the cap, for points it converged
    # within the cap (so that they had as long again to settle)
    ref = {q: hist["fp64_batch_uniform"][-1, q] for q in range(n_test)
           if (first_rule(hist["fp64_batch_uniform"], q) or cycles + 1) <= cycles}
    out["fp64_batch_uniform"]["converged"] = len(ref)

    def first_within(H, q):
        r = ref[q]
        bad = np.nonzero((np.abs(H[:, q, 6] - r[6]) > tol_m * abs(r[6])) | (np.abs(H[:, q, 8] - r[8]) > tol_pr * abs(r[8])))[0]
        return 0 if bad.size == 0 else (int(bad[-1]) + 2 if bad[-1] + 1 < H.shape[0] else None)

    per = {}
    for name in ("mixed_batch_uniform", "mixed_batch_warm"):
        H = hist[name]
        rule = [first_rule(H, q) for q in range(n_test)]
        within = [first_within(H, q) if q in ref else None for q in range(n_test)]
        per[name] = (rule, within)
        err_at_rule = [max(abs(H[c - 1, q, 6] - ref[q][6]) / abs(ref[q][6]), 0.0) for q, c in enumerate(rule) if c and q in ref]
        pr_at_rule = [abs(H[c - 1, q, 8] - ref[q][8]) / abs(ref[q][8]) for q, c in enumerate(rule) if c and q in ref]
        out[name].update({
            "converged_by_rule": sum(1 for c in rule if c), "cycles_to_rule": rule,
            "within_tol_of_fp64": sum(1 for c in within if c is not None), "cycles_to_fp64_integrals": within,
            "at_rule_mass_flow_rel_err_max": max(err_at_rule) if err_at_rule else None,
            "at_rule_pressure_ratio_rel_err_max": max(pr_at_rule) if pr_at_rule else None})
    both = [q for q in range(n_test) if per["mixed_batch_uniform"][1][q] is not None and per["mixed_batch_warm"][1][q] is not None]
    out["points_both_reach_fp64_integrals"] = len(both)
    if both:
        cu = [per["mixed_batch_uniform"][1][q] for q in both]
        cw = [per["mixed_batch_warm"][1][q] for q in both]
        out["median_cycles_to_fp64_integrals"] = {"uniform": float(np.median(cu)), "warm": float(np.median(cw))}
        out["sum_cycles_to_fp64_integrals"] = {"uniform": int(sum(cu)), "warm": int(sum(cw))}
    both_r = [q for q in range(n_test) if per["mixed_batch_uniform"][0][q] and per["mixed_batch_warm"][0][q]]
    if both_r:
        out["median_cycles_to_rule"] = {"uniform": float(np.median([per["mixed_batch_uniform"][0][q] for q in both_r])),
                                        "warm": float(np.median([per["mixed_batch_warm"][0][q] for q in both_r]))}
    # solves per hour of a batch that retires each point when it reaches the FP64 integrals (the
    # points that never do count at the cap), from the measured time per cycle of the batch: one
    # point-cycle costs ms_per_cycle / n_test
    for name in ("mixed_batch_uniform", "mixed_batch_warm"):
        pc = sum(c if c is not None else cycles for c in per[name][1])
        t = pc * out[name]["ms_per_cycle"] / n_test / 1000.0 + out[name]["start_s"]
        out[name]["point_cycles"] = pc
        out[name]["retiring_batch_solves_per_hour"] = 3600.0 * n_test / t
    # plain FP64 one solve at a time from the uniform start (a subsample of the held-out points)
    sub = list(range(n_train, n_train + n_test))[:4]
    t_sub = 0.0
    for q in sub:
        t0 = time.perf_counter()
        speedline.run([dirs[q]], gbturbo.FP64, max_iter=cycles, chunk=50, tol=1e-6)
        t_sub += time.perf_counter() - t0
    out["fp64_single_uniform"] = {"subsample": len(sub), "wall_s": t_sub, "solves_per_hour": 3600.0 * len(sub) / t_sub}
    base = out["fp64_single_uniform"]["solves_per_hour"]
    for name in ("mixed_batch_uniform", "mixed_batch_warm"):
        out[name]["retiring_over_plain_fp64_single"] = out[name]["retiring_batch_solves_per_hour"] / base
    amort = out["mixed_batch_warm"]["point_cycles"] * out["mixed_batch_warm"]["ms_per_cycle"] / n_test / 1000.0 + \
        out["mixed_batch_warm"]["start_s"] + out["data_s"] + out["train_s"]
    out["warm_retiring_including_training_solves_per_hour"] = 3600.0 * n_test / amort
    w.close()
    return out


def study_network(gbturbo):
    """the warm-start network's tensor-core kernels alone: device time per forward pass and per
    training pass (forward, loss, backward) at several row counts, the fused inference pass (every
    layer in one kernel), and the dense BF16 rate they
    reach (FLOPs per row: 2 x (64x256 + 4 x 256x256 + 256x16) forward; backward the same again for
    the weight gradients and again less the first layer's 2 x 64x256 for the data gradients)"""
    fwd_flop = 2 * (64 * 256 + 4 * 256 * 256 + 256 * 16)
    step_flop = 3 * fwd_flop - 2 * 64 * 256
    out = {"study": "network", "rows": {}}
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("bf16_tflops", 1900.0))
    with gbturbo.WarmStart(seed=1) as w:
        for rows in (32768, 262144, 1048576):
            ms_f, ms_s, ms_i, dmax = w.benchmark(rows, iters=20)
            tf_f = fwd_flop * rows / (ms_f / 1000.0) / 1e12
            tf_s = step_flop * rows / (ms_s / 1000.0) / 1e12
            tf_i = fwd_flop * rows / (ms_i / 1000.0) / 1e12
            out["rows"][str(rows)] = {"ms_forward": ms_f, "ms_train_step": ms_s, "ms_inference_fused": ms_i,
                                      "tflops_forward": tf_f, "tflops_train_step": tf_s,
                                      "tflops_inference_fused": tf_i, "frac_of_bf16_peak_forward": tf_f / peak,
                                      "frac_of_bf16_peak_inference_fused": tf_i / peak,
                                      "fused_vs_layer_by_layer_max_abs_diff": dmax}
    out["bf16_peak_tflops"] = peak
    return out


def study_multigrid(gbturbo, tmp, cycles):
    """the 129 x 49 x 49 passage at 1.10 x p_t with two levels (the reference's cycle) and with the
    three-level V-cycle extension, both forms: density residual and mass-flow imbalance at
    checkpoints, device time per cycle"""
    dirs, cells = make_cases(os.path.join(tmp, "mg"), 1, back_pressures=[1.10])
    out = {"study": "multigrid", "cycles": cycles, "cells": cells, "runs": {}}
    for levels in (2, 3):
        for name, prec in (("fp64", gbturbo.FP64), ("mixed", gbturbo.MIXED)):
            with gbturbo.Solver(dirs, prec, levels=levels) as s:
                s.init_uniform()
                s.timer_start()
                h = s.iterate(cycles)[:, 0, :]
                ms = s.timer_stop()
            marks = [c for c in (50, 100, 200, 300, 500, 1000, 1500, 2000, 3000) if c <= cycles]
            out["runs"][f"{levels}_levels_{name}"] = {
                "ms_per_cycle": ms / cycles,
                "res_dens": {str(c): float(h[c - 1, 1]) for c in marks},
                "mass_ratio": {str(c): float(h[c - 1, 10]) for c in marks},
                "min_res_dens": float(h[:, 1].min()), "first_below_1e-4": int(np.argmax(h[:, 1] < 1e-4)) + 1 if (h[:, 1] < 1e-4).any() else None}
    return out


def run_study(args):
    import build as pkg_build
    pkg_build.build()
    import gbturbo
    tmp = tempfile.mkdtemp(prefix="gbt_study_")
    try:
        if args.study == "precision":
            res = study_precision(gbturbo, tmp, args.cycles or 3000)
        elif args.study == "multigrid":
            res = study_multigrid(gbturbo, tmp, args.cycles or 1000)
        elif args.study == "network":
            res = study_network(gbturbo)
        elif args.study == "warmstart":
            res = study_warmstart(gbturbo, tmp, args.cycles or 2000, args.points)
        else:
            res = study_solves(gbturbo, tmp, args.cycles or 4000, args.points)
        print(json.dumps(res), flush=True)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return 0


def config_block(args, cells, nsolve):
    if getattr(args, "sampled", False):
        wl, mesh = "sampled_rotor_passages_2level_multigrid", "97x41x41 / 129x49x49 / 161x65x65 (seeded sampler)"
    elif getattr(args, "variant", "default") != "default":
        wl = {"jst": "rotor_passage_129x49x49_jst_2level_multigrid", "sa": "rotor_passage_129x49x49_spalart_allmaras_single_grid",
              "stage": "rotor_stator_stage_129x49x49_65x49x49_mixing_plane_2level"}[args.variant]
        mesh = "129x49x49 rotor + 65x49x49 stator" if args.variant == "stage" else "129x49x49 (axial x pitch x span)"
    elif getattr(args, "blocks", 1) == 3:
        wl, mesh = "rotor_passage_129x49x49_3block_2level_multigrid", "129x49x49 as blocks of 41/49/41 axial nodes"
    else:
        wl, mesh = "rotor_passage_129x49x49_2level_multigrid", "129x49x49 (axial x pitch x span)"
    if getattr(args, "levels", 2) == 3:
        wl = wl.replace("2level_multigrid", "3level_vcycle")
    return {"workload": wl, "mesh_nodes": mesh,
            "cells_per_solve": cells, "solves_per_gpu": nsolve, "precision": args.precision,
            "levels": getattr(args, "levels", 2),
            "scheme": {"default": "Roe + MUSCL3 (primitive), Baldwin-Lomax, LU-SGS, 2-level FAS (reference maximum)",
                       "jst": "JST (k2 0.5, k4 1/32), Baldwin-Lomax, LU-SGS, 2-level FAS",
                       "sa": "Roe + MUSCL3 (primitive), Spalart-Allmaras, LU-SGS, single grid",
                       "stage": "Roe + MUSCL3 (primitive), Baldwin-Lomax, LU-SGS, 2-level FAS, mixing plane"}[
                           getattr(args, "variant", "default")],
            "l2": "inputs larger than L2 (FP64 working set well above 129 MB), no flush",
            "parallelism": "replicas"}


# ---------------------------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------------------------
def run_gpu(args, rank, world, dist):
    import build as pkg_build
    pkg_build.build()
    import gbturbo
    prec = gbturbo.FP64 if args.precision == "fp64" else gbturbo.MIXED
    wsize = 8 if prec == gbturbo.FP64 else 4
    tmp = tempfile.mkdtemp(prefix=f"gbt_bench_{rank}_")
    try:
        if args.sampled:
            dirs, cell_list = make_sampled_cases(tmp, args.batch, seed=2024 + rank)
            cells = sum(cell_list) / len(cell_list)     # mean per solve; totals below multiply by nsolve
        else:
            dirs, cells = make_cases(tmp, args.batch, seed_offset=rank, blocks=args.blocks, variant=args.variant)
        nsolve = len(dirs)
        grid_bytes = sum(os.path.getsize(os.path.join(d, "grid.dat")) for d in dirs)

        # --- device-resident throughput (value)
        s = gbturbo.Solver(dirs, prec, levels=args.levels)
        s.init_uniform()
        s.iterate(max(args.warmup, 3), history=False)
        s.sync()
        barrier(dist)
        clk = ClockSampler()
        clk.start()
        s.timer_start()
        s.iterate(args.steps, history=False)
        ms = s.timer_stop()
        clocks = clk.stop()
        barrier(dist)
        ms = allmax(dist, ms)
        value = cells * nsolve * world * args.steps / (ms / 1000.0)
        status = [int(x) for x in s.status()]

        # --- stage profile of a few cycles (eager launches, events around every stage)
        nprof = min(5, args.steps)
        s.profile_begin()
        s.iterate(nprof, history=False)
        prof = s.profile_end()
        slot_dims = [[s.dims(q, l)[:3] for q in range(s.n_slots)] for l in range(1, s.ng + 1)]
        tuning = {f"level{l}": list(s.sweep_tuning(l)) for l in range(1, s.ng + 1)}
        total_prof = sum(v[0] for v in prof.values())
        launches_per_step = sum(v[1] for v in prof.values()) / nprof
        dom = max((k for k in prof if k in ALG), key=lambda k: prof[k][0])
        dom_ms, dom_launches, dom_evals = prof[dom]
        units_step = alg_units_per_step(dom, slot_dims, dom_evals, nprof)
        # algorithmic bytes of the stage per cycle / its device time per cycle (events around the
        # stage's launches, eager); per launch = per cycle / launches per cycle
        bytes_per_step = units_step * alg_bytes_per_unit(dom, wsize)
        achieved = bytes_per_step / (dom_ms / nprof / 1000.0) / 1e9
        bytes_per_launch = bytes_per_step / (dom_launches / nprof)
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except Exception:
            pass
        peak = float(peaks.get("hbm_gbs", 6800.0))
        traffic = None
        try:
            for line in open(os.path.join(ROOT, "profiles", "dram_traffic_per_launch.txt")):
                f = line.split()
                if len(f) >= 4 and not line.startswith("#") and f[0] == dom and f[1] == args.precision and int(f[2]) == nsolve:
                    traffic = float(f[3])        # DRAM read + write bytes per launch (ncu), same averaging
        except FileNotFoundError:
            pass
        roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "traffic": traffic, "alg_bytes_per_launch": bytes_per_launch,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6800 GB/s"}
        counts = fp64_ops_per_unit().get(dom) if prec == gbturbo.FP64 else None
        if counts is not None:
            # the FP64 form is bound by the FP64 pipe: counted FP64 operations of the stage (ncu, per
            # face or plane cell) over its device time, against the FP64 rate measured in this run.
            # DADD and DMUL hold the pipe as long as an FMA, so beside the FLOP fraction the line
            # gives the pipe's occupancy: FP64 instructions issued per second against the FMA-chain
            # loop's instructions per second (half its FLOP rate).
            flops_unit, inst_unit = counts
            rate = gbturbo.fp64_rate() / 1e12
            sec = dom_ms / nprof / 1000.0
            flop_step = units_step * flops_unit
            tf = flop_step / sec / 1e12
            ti = units_step * inst_unit / sec / 1e12
            roofline = {"bound": "fp64", "kernel": dom, "achieved": tf, "peak": rate, "unit": "TFLOP/s",
                        "frac": tf / rate, "traffic": traffic, "flop_per_launch": flop_step / (dom_launches / nprof),
                        "flop_per_unit": flops_unit,
                        "fp64_pipe": {"achieved": ti, "peak": rate / 2.0, "unit": "T FP64 instructions/s",
                                      "frac": ti / (rate / 2.0), "inst_per_unit": inst_unit},
                        "peak_source": "FP64 FMA-chain loop timed in this run (gb_fp64_rate); "
                                       "MEASURED_PEAKS.json holds no FP64 figure",
                        "hbm": {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                                "alg_bytes_per_launch": bytes_per_launch}}
        forms = None
        if (rank == 0 and world == 1 and not args.no_forms and prec == gbturbo.FP64 and nsolve == 1 and args.blocks == 1
                and args.variant == "default" and args.levels == 2):
            n_ref = max(args.warmup, 3) + args.steps + nprof
            forms = measure_forms(gbturbo, dirs, cells, n_ref, s.integrals(1)[0], min(args.steps, 50), tmp)
            if not args.no_solves:
                forms["solves_per_hour"] = measure_solves(gbturbo, os.path.join(tmp, "solves"))
        s.close()

        # --- end to end through the C-ABI: case files on the host -> handle (upload + geometry)
        # -> iterations with the history row read back every step
        barrier(dist)
        t0 = time.perf_counter()
        e = gbturbo.Solver(dirs, prec, levels=args.levels)
        e.init_uniform()
        e.iterate(max(args.warmup, 3), history=True)
        for _ in range(args.steps):
            e.iterate(1, history=True)
        e.close()
        t_e2e = allmax(dist, time.perf_counter() - t0)
        barrier(dist)
        n_e2e = max(args.warmup, 3) + args.steps
        e2e_value = cells * nsolve * world * n_e2e / t_e2e

        base = None
        if rank == 0 and not args.no_cpu_baseline and args.blocks == 1 and args.variant == "default" and args.levels == 2:
            # (the CPU oracle port is single-block)
            base = cpu_baseline(dirs[0], cells, warm=3, steps=2, fp32=prec == gbturbo.MIXED)

        if rank == 0:
            stages = {k: {"ms_per_step": round(v[0] / nprof, 4), "launches_per_step": round(v[1] / nprof, 1),
                          "share": round(v[0] / total_prof, 4)} for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}
            line = {
                "metric": "cell_updates_per_s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
                "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if prec == gbturbo.FP64 else "f32+f64", "data": "synthetic",
                "config": config_block(args, cells, nsolve),
                "clocks": clocks,
                "e2e": {"value": e2e_value, "unit": "cell-updates/s",
                        "h2d_bytes_per_step": int(grid_bytes / n_e2e), "d2h_bytes_per_step": 96 * nsolve},
                "gpu_launches": int(round(launches_per_step * args.steps)),
                "roofline": roofline,
                "sweep_shape_cells_per_warp_warps_per_block": tuning,
                "stages": stages,
                "forms": forms,
                "cpu_baseline": base,
                "status": status,
            }
            print(json.dumps(line), flush=True)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return 0


def main():
    args = parse()
    if args.study:
        return run_study(args)
    rank, world, dist = dist_init()
    if args.impl == "reference":
        rc = run_reference(args, rank, world, dist)
    else:
        rc = run_gpu(args, rank, world, dist)
    if dist is not None:
        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
