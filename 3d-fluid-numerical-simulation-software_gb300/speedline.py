"""Speedline driver: the operating points of one compressor speed line (the back pressure swept at
fixed speed) run as one batch on the GPU, each reported where the reference's driver would stop
it (source/Structured_FV3D.cpp:214-218: density residual at or below the convergence tolerance
and |m_in - m_out| / m_in <= 0.003, or the iteration cap).

A point is a copy of a template case directory in the reference's formats whose config.dat has
the outlet static pressure replaced; the grid and boundary files are linked, not copied. The
config file is positional (the reference reads it line by line, source/UserInput.cpp:20-140), so
the value lines are addressed by their position.

    import speedline
    dirs = speedline.make_points("rotor_case", [1.05, 1.10, 1.15, 1.20, 1.25], "points", ratio_of="Ptin")
    table = speedline.run(dirs)           # one dict per point
"""
from __future__ import annotations

import os
import shutil
from typing import Dict, List, Optional, Sequence

import numpy as np

import gbturbo

# 0-based line numbers of config.dat values used here
LINE_GRID = 1
LINE_BC = 4
LINE_PTIN = 18
LINE_POUT = 20
LINE_MAXITER = 32
LINE_CONVTOL = 35

MASS_RATIO_LIMIT = 0.003


def _lines(path: str) -> List[str]:
    with open(path, newline="") as f:
        return f.read().splitlines(keepends=True)


def _value(line: str) -> str:
    return line.split("#")[0].split()[0]


def _replace_value(line: str, value: str) -> str:
    """the first token of a config line replaced, the rest (comment, line ending) kept"""
    head = line.lstrip()
    indent = line[:len(line) - len(head)]
    tok = head.split()[0]
    return indent + value + head[len(tok):]


def make_points(template: str, back_pressures: Sequence[float], root: str, ratio_of: Optional[str] = None,
                overrides: Optional[Dict[int, str]] = None) -> List[str]:
    """One case directory per back pressure under root. back_pressures are in Pa, or, with
    ratio_of="Ptin", ratios to the template's inlet total pressure. overrides: further config
    values by 0-based line number (e.g. {LINE_CONVTOL: "1.0E-4"})."""
    cfg = _lines(os.path.join(template, "config.dat"))
    grid, bc = _value(cfg[LINE_GRID]), _value(cfg[LINE_BC])
    scale = float(_value(cfg[LINE_PTIN])) if ratio_of == "Ptin" else 1.0
    dirs = []
    for q, pb in enumerate(back_pressures):
        d = os.path.join(root, f"point{q:03d}")
        os.makedirs(d, exist_ok=True)
        lines = list(cfg)
        lines[LINE_POUT] = _replace_value(lines[LINE_POUT], "%.6f" % (pb * scale))
        for ln, v in (overrides or {}).items():
            lines[ln] = _replace_value(lines[ln], v)
        with open(os.path.join(d, "config.dat"), "w", newline="") as f:
            f.write("".join(lines))
        for name in (grid, bc):
            src, dst = os.path.abspath(os.path.join(template, name)), os.path.join(d, name)
            if os.path.lexists(dst):
                os.remove(dst)
            try:
                os.symlink(src, dst)
            except OSError:
                shutil.copy(src, dst)
        dirs.append(d)
    return dirs


def run(dirs: Sequence[str], precision: int = gbturbo.MIXED, max_iter: Optional[int] = None, chunk: int = 50,
        tol: Optional[float] = None, start=None) -> List[Dict]:
    """Runs the points as one batch until every point met the reference's convergence rule or the
    iteration cap (default: the template's maxiter), and reports each point at its first
    converged iteration (its last iteration if it never converged). start(solver), if given, sets
    the starting field in place of the uniform start (e.g. a WarmStart's apply)."""
    cfg = _lines(os.path.join(dirs[0], "config.dat"))
    tol = float(_value(cfg[LINE_CONVTOL])) if tol is None else tol
    max_iter = int(_value(cfg[LINE_MAXITER])) if max_iter is None else max_iter
    pouts = [float(_value(_lines(os.path.join(d, "config.dat"))[LINE_POUT])) for d in dirs]
    n = len(dirs)
    done = [None] * n                      # history row at convergence
    last = None
    with gbturbo.Solver(list(dirs), precision) as s:
        if start is None:
            s.init_uniform()
        else:
            start(s)
        it = 0
        while it < max_iter and any(r is None for r in done):
            h = s.iterate(min(chunk, max_iter - it))          # (chunk, n, 12)
            it += h.shape[0]
            last = h[-1]
            for q in range(n):
                if done[q] is not None:
                    continue
                ok = np.nonzero((h[:, q, 1] <= tol) & (h[:, q, 10] <= MASS_RATIO_LIMIT))[0]
                if ok.size:
                    done[q] = h[ok[0], q].copy()
        status = s.status()
    table = []
    for q in range(n):
        row = done[q] if done[q] is not None else last[q]
        table.append({"case": dirs[q], "pout_pa": pouts[q], "converged": done[q] is not None,
                      "iteration": int(row[0]), "res_dens": float(row[1]), "m_in": float(row[6]),
                      "m_out": float(row[7]), "pressure_ratio": float(row[8]), "efficiency": float(row[9]),
                      "mass_ratio": float(row[10]), "status": int(status[q])})
    return table
