"""Regenerates the golden fixtures of tests/golden/ from the reference solver itself.

For each case below: writes the case files (config.dat, BoundaryDefinition.dat, grid.dat) with
the package's mesh generator into tests/golden/<name>/, runs the reference's own CPU code through
oracle/_ref/ref_harness (built by oracle/build_ref.sh from the reference sources) for the given
number of driver iterations, and stores the history, the final state and one residual
evaluation at that state (every intermediate array) in tests/golden/<name>.npz.

Only runs where the reference sources and a C++ compiler exist; the fixtures it writes are
committed so the tests need neither.

    python tests/golden/make_golden.py [name ...]      (default: every short case, the restart case,
                                                        the multi-block and stage cases and the FP32-build
                                                        histories; long cases by name)
"""
from __future__ import annotations

import importlib.util
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PKG = os.path.join(ROOT, "3d-fluid-numerical-simulation-software_gb300")
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def _meshgen():
    spec = importlib.util.spec_from_file_location("gb_meshgen", os.path.join(PKG, "meshgen.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["gb_meshgen"] = mod
    spec.loader.exec_module(mod)
    return mod


# name -> (generator, kwargs, options, iterations)
CASES = {
    "duct_9x9x17": ("annular_duct", dict(IM=9, JM=9, KM=17), {}, 20),
    "duct_9x9x17_sw_nnd": ("annular_duct", dict(IM=9, JM=9, KM=17), {"scheme": "200", "recon": "100"}, 12),
    "duct_9x9x17_laminar_cons": ("annular_duct", dict(IM=9, JM=9, KM=17),
                                 {"recon_var": "100", "recon": "400", "turb": "0"}, 12),
    "duct_9x9x17_muscl2u_global": ("annular_duct", dict(IM=9, JM=9, KM=17),
                                   {"recon": "200", "timestep": "G", "limiter": "N"}, 10),
    "rotor_9x9x33": ("rotor_passage", dict(IM=9, JM=9, KM=33), {}, 20),
    "rotor_9x9x33_mg": ("rotor_passage", dict(IM=9, JM=9, KM=33), {"multigrid": "Y", "coarse_iter": "5"}, 14),
    # JST central scheme with artificial dissipation (k2 0.6, k4 1/100), three dummy layers
    "duct_9x9x17_jst": ("annular_duct", dict(IM=9, JM=9, KM=17), {"scheme": "100"}, 12),
    "rotor_9x9x33_jst_mg": ("rotor_passage", dict(IM=9, JM=9, KM=33),
                            {"scheme": "100", "k2": "0.5", "k4": "32.0", "multigrid": "Y", "coarse_iter": "4"}, 12),
    # Spalart-Allmaras (wall distances, the eddy-viscosity equation in the residual and the
    # LU-SGS sweeps), single grid
    "duct_9x9x17_sa": ("annular_duct", dict(IM=9, JM=9, KM=17), {"turb": "200"}, 12),
    "rotor_9x9x33_sa": ("rotor_passage", dict(IM=9, JM=9, KM=33), {"turb": "200"}, 12),
    # imposed mass flow: 25 kg/s, relaxation 0.2, every 2 iterations, residual gate 1.0
    "rotor_9x9x33_massflow": ("rotor_passage", dict(IM=9, JM=9, KM=33),
                              {"mass_imposed": "Y", "mass_line": "25.0 0.2 2 1.0"}, 20),
}

# long runs: only the driver history is kept, and the case is regenerated by the tests from the
# same generator call (its grid file is several MB)
LONG = {
    "duct_33x33x65_2000": ("annular_duct", dict(IM=33, JM=33, KM=65), {}, 2000),
    # the rotor blade family on a 25x25x65 mesh at 1.05 x p_t, two-level FAS: the reference's driver
    # runs it until its convergence rule stops it (cycle 1371 of at most 6000)
    "rotor_25x25x65_converged": ("rotor_passage", dict(IM=25, JM=25, KM=65),
                                 {"Pout": "%.1f" % (1.05 * 101325.0), "multigrid": "Y", "coarse_iter": "2",
                                  "Ma0": "0.45", "maxiter": "6000"}, 6000),
    # the benchmark's passage (129x49x49 nodes, 1.20 x p_t, two-level FAS) run for 2000 cycles: the
    # reference's own solution leaves the converging branch (mass flow falls from about 28.6 to 10
    # between cycles 800 and 1800 and the outlet flow reverses); single-threaded about 80 minutes
    "rotor_129x49x49_2000": ("rotor_passage", dict(IM=49, JM=49, KM=129),
                             {"Pout": "%.1f" % (1.20 * 101325.0), "multigrid": "Y", "coarse_iter": "2",
                              "Ma0": "0.45"}, 2000),
}

# multi-block: the rotor passage cut at the blade's leading- and trailing-edge planes into three
# blocks joined by interfaces (meshgen.split_axial); every array per block ("b<block>_" prefix),
# and the reference's solution and restart files written at the end
MULTI = {
    "rotor_9x9x33_3block": (dict(IM=9, JM=9, KM=33), [9, 25], {}, 12),
    "rotor_9x9x33_3block_mg": (dict(IM=9, JM=9, KM=33), [9, 25], {"multigrid": "Y", "coarse_iter": "4"}, 12),
}

# rotor-stator stage: a rotor passage of 22 blades at 16000 rpm and a stationary row of 30 blades,
# joined by a mixing plane (meshgen.stage_passage)
STAGE = {
    "stage_9x9x17": (dict(), {}, 12),
    "stage_9x9x17_mg": (dict(), {"multigrid": "Y", "coarse_iter": "4"}, 12),
}

# restart round trip: the reference runs n1 iterations and writes its solution and restart files,
# then a second run of the same case with "use previous solution" reads the restart file and runs
# n2 more; both case directories are kept (the second holds the restart file it starts from)
RESTART = {
    "rotor_9x9x33_restart": ("rotor_passage", dict(IM=9, JM=9, KM=33), {}, 10, 10),
}

# the reference's default FP32 build (REAL = float; oracle/_ref32, FP32=1 oracle/build_ref.sh):
# driver history only, on the case directory of an FP64 fixture. It pins the oracle's FP32 build,
# which is the CPU timing beside the GPU's mixed form, to FP32 round-off (not bit for bit).
FP32_RUNS = {
    "duct_9x9x17_fp32": ("duct_9x9x17", 20),
    "rotor_9x9x33_mg_fp32": ("rotor_9x9x33_mg", 14),
}
HARNESS32 = os.path.join(ROOT, "oracle", "_ref32", "ref_harness")

KEEP_R = ["cv", "pv", "mut", "ev", "res_ev", "omega", "lamcI", "lamcJ", "lamcK", "lamvI", "lamvJ", "lamvK", "dt", "FcI", "FcJ",
          "FcK", "FvI", "FvJ", "FvK", "res", "dIS_pv", "dIP_pv", "dJS_pv", "dJP_pv", "dKS_pv", "dKP_pv", "dIS_cv",
          "dKP_cv"]


def make_long(name: str) -> None:
    mg = _meshgen()
    gen, kw, opts, n_iter = LONG[name]
    case = getattr(mg, gen)(**kw, options=opts, name=name)
    with tempfile.TemporaryDirectory() as tmp:
        mg.write_case(case, tmp)
        out = os.path.join(tmp, "out")
        subprocess.run([HARNESS, str(n_iter), out, "0"], cwd=tmp, check=True, stdout=subprocess.DEVNULL)
        hist = np.load(os.path.join(out, "history.npy"))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), history=hist)
    print(name, "iterations:", int(hist.shape[0]))


def make_restart(name: str) -> None:
    mg = _meshgen()
    gen, kw, opts, n1, n2 = RESTART[name]
    cdir, rdir = os.path.join(HERE, name), os.path.join(HERE, name + "_reuse")
    for d in (cdir, rdir):
        if os.path.isdir(d):
            shutil.rmtree(d)
    mg.write_case(getattr(mg, gen)(**kw, options=dict(opts), name=name), cdir)
    mg.write_case(getattr(mg, gen)(**kw, options=dict(opts, restart="Y"), name=name), rdir)
    data = {}
    with tempfile.TemporaryDirectory() as tmp:
        for f in os.listdir(cdir):
            shutil.copy(os.path.join(cdir, f), tmp)
        out = os.path.join(tmp, "out")
        subprocess.run([HARNESS, str(n1), out, "0", "1"], cwd=tmp, check=True, stdout=subprocess.DEVNULL)
        data["history1"] = np.load(os.path.join(out, "history.npy"))
        for key, f in (("restart_file", "RestartSolution.dat"), ("solution_file", "RelativeSolution.plt")):
            data[key] = np.frombuffer(open(os.path.join(tmp, f), "rb").read(), dtype=np.uint8)
        shutil.copy(os.path.join(tmp, "RestartSolution.dat"), rdir)
    with tempfile.TemporaryDirectory() as tmp:
        for f in os.listdir(rdir):
            shutil.copy(os.path.join(rdir, f), tmp)
        out = os.path.join(tmp, "out")
        subprocess.run([HARNESS, str(n2), out, "0"], cwd=tmp, check=True, stdout=subprocess.DEVNULL)
        data["history2"] = np.load(os.path.join(out, "history.npy"))
        data["s1_cv"] = np.load(os.path.join(out, "s1_cv.npy"))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
    print(name, "iterations:", n1, "+", n2)


def make_multi(name: str) -> None:
    mg = _meshgen()
    if name in STAGE:
        kw, opts, n_iter = STAGE[name]
        case = mg.stage_passage(**kw, options=dict(opts), name=name)
    else:
        kw, cuts, opts, n_iter = MULTI[name]
        case = mg.split_axial(mg.rotor_passage(**kw, options=dict(opts), name=name), cuts, name=name)
    cdir = os.path.join(HERE, name)
    if os.path.isdir(cdir):
        shutil.rmtree(cdir)
    mg.write_multiblock_case(case, cdir)
    keep = ("cv", "pv", "mut", "omega", "lamcK", "lamvK", "dt", "FcK", "FvK", "FcJ", "res", "dKS_pv", "dKP_pv")
    with tempfile.TemporaryDirectory() as tmp:
        for f in os.listdir(cdir):
            shutil.copy(os.path.join(cdir, f), tmp)
        out = os.path.join(tmp, "out")
        subprocess.run([HARNESS, str(n_iter), out, "1", "1"], cwd=tmp, check=True, stdout=subprocess.DEVNULL)
        data = {"history": np.load(os.path.join(out, "history.npy"))}
        for f in sorted(os.listdir(out)):
            key = f[:-4]
            parts = key.split("_", 2)
            if not key.startswith("b") or len(parts) < 3:
                continue
            kind, field = parts[1], parts[2]
            if (kind == "r1" and field in keep) or (kind == "g1" and field in ("faceK", "cell", "totalvol")):
                data[key] = np.load(os.path.join(out, f))
        for key, f in (("restart_file", "RestartSolution.dat"), ("solution_file", "RelativeSolution.plt")):
            data[key] = np.frombuffer(open(os.path.join(tmp, f), "rb").read(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
    print(name, "iterations:", int(data["history"].shape[0]))


def make_fp32(name: str) -> None:
    src, n_iter = FP32_RUNS[name]
    with tempfile.TemporaryDirectory() as tmp:
        for f in os.listdir(os.path.join(HERE, src)):
            shutil.copy(os.path.join(HERE, src, f), tmp)
        out = os.path.join(tmp, "out")
        subprocess.run([HARNESS32, str(n_iter), out, "0"], cwd=tmp, check=True, stdout=subprocess.DEVNULL)
        hist = np.load(os.path.join(out, "history.npy"))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), history=hist, case=np.array(src))
    print(name, "iterations:", int(hist.shape[0]))


def make(name: str) -> None:
    if name in FP32_RUNS:
        make_fp32(name)
        return
    if name in MULTI or name in STAGE:
        make_multi(name)
        return
    if name in RESTART:
        make_restart(name)
        return
    if name in LONG:
        make_long(name)
        return
    mg = _meshgen()
    gen, kw, opts, n_iter = CASES[name]
    case = getattr(mg, gen)(**kw, options=opts, name=name)
    cdir = os.path.join(HERE, name)
    if os.path.isdir(cdir):
        shutil.rmtree(cdir)
    mg.write_case(case, cdir)
    with tempfile.TemporaryDirectory() as tmp:
        for f in os.listdir(cdir):
            shutil.copy(os.path.join(cdir, f), tmp)
        out = os.path.join(tmp, "out")
        subprocess.run([HARNESS, str(n_iter), out, "1"], cwd=tmp, check=True, stdout=subprocess.DEVNULL)
        data = {}
        base_case = name in ("duct_9x9x17", "rotor_9x9x33")
        for f in sorted(os.listdir(out)):
            key = f[:-4]
            if key.startswith("r1_") and key[3:] not in KEEP_R:
                continue
            if key.startswith("s") or key.startswith("g2_"):
                continue                       # state after the loop is r1_cv's interior
            if key.startswith("g1_") and not base_case and key != "g1_dwall":
                continue                       # geometry is pinned on the two base cases
            if not base_case and key.startswith("r1_d"):
                continue
            data[key] = np.load(os.path.join(out, f))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **data)
    print(name, "iterations:", int(data["history"].shape[0]))


if __name__ == "__main__":
    if not os.path.exists(HARNESS):
        sys.exit("build the reference harness first: oracle/build_ref.sh")
    for n in (sys.argv[1:] or list(CASES) + list(RESTART) + list(MULTI) + list(STAGE) + list(FP32_RUNS)):
        make(n)
