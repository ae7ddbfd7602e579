"""Synthetic turbomachinery cases written in the reference solver's own input formats.

A *case* is the triple the reference reads from its working directory:

* ``config.dat``            -- positional option file (``source/UserInput.cpp:17-239``)
* the grid file             -- text multi-block node list (``source/UserInput.cpp:241-334``)
* ``BoundaryDefinition.dat`` -- patch list (``source/UserInput.cpp:336-446``)

Axis convention of the reference: rotation about **z**, ``(i, j, k) = (span, pitch,
axial)``; inlet on the ``k = 1`` face, outlet on ``k = KM`` (``source/BndCondOutlet.cpp:34-79``).
Pitch angle increases with ``j`` so that the periodic pair (j-min face listed first) never
flips the sign of ``delta_th`` (``source/BndCondInteriorPeriodic.cpp:54-59``).

Two geometry families are generated:

* ``annular_duct``  -- single-block annular sector with a 3-D hub bump (plain-method case).
* ``rotor_passage`` -- single-block H-grid around one compressor blade: circular-arc camber,
  linear radial stagger, NACA-style thickness, blade surfaces as j-face walls over the blade's
  axial range and periodic j-faces upstream and downstream.

Both use a two-sided tanh stretching with a prescribed first spacing at the walls.
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np


# ----------------------------------------------------------------------------------------
# point distributions
# ----------------------------------------------------------------------------------------
def two_sided_spacing(n_int: int, length: float, d1: float) -> np.ndarray:
    """Node positions in [0, length] with ``n_int`` intervals and first spacing ``d1`` at both
    ends, from the symmetric tanh stretching s(x) = 1/2 (1 + tanh(b (x - 1/2)) / tanh(b/2)).
    ``b`` is found by bisection so the first interval equals ``d1`` (uniform if ``d1`` is not
    smaller than the uniform spacing)."""
    x = np.linspace(0.0, 1.0, n_int + 1)
    if d1 >= length / n_int:
        return x * length

    def first(b: float) -> float:
        s = 0.5 * (1.0 + np.tanh(b * (x[1] - 0.5)) / np.tanh(0.5 * b))
        return s * length

    lo, hi = 1e-6, 60.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if first(mid) > d1:
            lo = mid
        else:
            hi = mid
    b = 0.5 * (lo + hi)
    s = 0.5 * (1.0 + np.tanh(b * (x - 0.5)) / np.tanh(0.5 * b))
    s[0], s[-1] = 0.0, 1.0
    return s * length


# ----------------------------------------------------------------------------------------
# case description
# ----------------------------------------------------------------------------------------
@dataclasses.dataclass
class Patch:
    """One boundary patch in ``BoundaryDefinition.dat`` numbering (1-based, face types 1..6 =
    i-, i+, j-, j+, k-, k+; the face index is a node index, the other two are cell ranges)."""
    kind: str                      # inlet | outlet | wall | periodic
    face: int
    rng: Tuple[int, int, int, int, int, int]
    rotate: int = 0                # walls: 1 = rotates with the block
    face2: int = 0                 # periodic partner
    rng2: Tuple[int, int, int, int, int, int] = (0, 0, 0, 0, 0, 0)
    orient: int = 2


@dataclasses.dataclass
class Case:
    name: str
    nodes: np.ndarray              # (IM, JM, KM, 3) float64, [i-1, j-1, k-1]
    patches: List[Patch]
    nblade: int
    rpm: float
    options: Dict[str, str]

    @property
    def dims(self) -> Tuple[int, int, int]:
        return tuple(int(v) for v in self.nodes.shape[:3])  # type: ignore

    @property
    def n_cells(self) -> int:
        IM, JM, KM = self.dims
        return (IM - 1) * (JM - 1) * (KM - 1)


DEFAULT_OPTIONS: Dict[str, str] = {
    "turbo": "A", "equation": "N", "init": "U",
    "Rgas": "287.06", "gamma": "1.4", "Pr_lam": "0.72", "Pr_tur": "0.90",
    "Ptin": "101325.0", "Ttin": "288.15", "Pout": "93219.0", "P21": "1.0",
    "Ma0": "0.5", "Len_ref": "1.0", "ev_ratio": "3.0",
    "inlet_dir": "0.0 0.0 1.0", "outlet_dir": "0.0 0.0 0.0",
    "mass_imposed": "N", "mass_line": "1.0 1.0 100 0.0001",
    "maxiter": "2000", "coarse_iter": "0", "outstep": "100000", "convtol": "1.0E-6",
    "nt": "1", "multigrid": "N", "restart": "N", "walldist": "N",
    "CFL": "3.0", "C_timestep": "1.0", "relax": "1.0", "epsEntr": "0.05",
    "k2": "0.6", "k4": "100.0", "IRS": "N", "limiter": "Y", "timestep": "L",
    "recon_var": "200", "recon": "500", "scheme": "300", "time": "500", "turb": "100",
}


def _config_text(opt: Dict[str, str], gridfile: str, bcfile: str) -> str:
    o = dict(DEFAULT_OPTIONS)
    o.update(opt)
    lines = [
        "# grid file", gridfile, "#", "# boundary condition file", bcfile, "#",
        "# Physics - general", "#--------------------------",
        f"{o['turbo']}               # axial(A) / centrifugal(C) / general(G)",
        f"{o['equation']}               # Euler(E) / Navier-Stokes(N)",
        f"{o['init']}               # uniform(U) / interpolate(I)",
        f"{o['Rgas']}          # Gas_Constant [J/(kg.k)]",
        f"{o['gamma']}             # Specific_Heat_Ratio",
        f"{o['Pr_lam']}            # laminar Prandtl number",
        f"{o['Pr_tur']}            # turbulence Prandtl number",
        "#", "# Physics - internal flow", "#--------------------------",
        f"{o['Ptin']}        # total pressure at inlet [Pa]",
        f"{o['Ttin']}          # total temperature at inlet [K]",
        f"{o['Pout']}         # static pressure at outlet [Pa]",
        f"{o['P21']}             # approximate ratio of inlet to outlet static pressure",
        f"{o['Ma0']}             # Mach number for initial",
        f"{o['Len_ref']}             # reference length [m]",
        f"{o['ev_ratio']}             # reference eddy viscous ratio",
        f"{o['inlet_dir']}     # flow direction at inlet",
        f"{o['outlet_dir']}     # flow direction at outlet",
        f"{o['mass_imposed']}               # use flow mass outlet (Y=yes, N=no)",
        f"{o['mass_line']}    # mass imposed, relax_press, iter control, res control",
        "#", "# Iteration control", "# -------------------------",
        f"{o['maxiter']}      # max. number of iterations",
        f"{o['coarse_iter']}      # number of iterations on coarse grid",
        f"{o['outstep']}      # number of iterations for save",
        f"{o['convtol']}    # convergence tolerance",
        f"{o['nt']}         # number of threads",
        f"{o['multigrid']}         # use multigrid method",
        f"{o['restart']}         # use previous solution for restart",
        f"{o['walldist']}         # use previous Wall Distance for restart",
        "#", "# Numerical parameters", "# -------------------------",
        f"{o['CFL']}       # CFL-number",
        f"{o['C_timestep']}       # time step coefficient",
        f"{o['relax']}       # relax factor in LU_SGS",
        f"{o['epsEntr']}      # entropy correction coefficient",
        f"{o['k2']}       # k2 used for artificial Dissipation",
        f"{o['k4']}     # k4 used for artificial Dissipation",
        f"{o['IRS']}         # use implict res smooth",
        f"{o['limiter']}         # limit (dens,vel, press) flow variables",
        f"{o['timestep']}         # local(L) / global(G) time-stepping",
        f"{o['recon_var']}       # cons(100) / prim(200) / charact(300)",
        f"{o['recon']}       # none(0)/NND(100)/MUSCL2u(200)/MUSCL2c(300)/MUSCL2o(400)/MUSCL3(500)",
        f"{o['scheme']}       # JST(100)/SW(200)/Roe(300)/...",
        f"{o['time']}       # RK3(100)/.../LU-SGS(500)",
        f"{o['turb']}       # none(0) / BL(100) / SA(200) / SST(300)",
        "",
    ]
    return "\n".join(lines)


def _bc_text(case: Case) -> str:
    IM, JM, KM = case.dims
    inl = [p for p in case.patches if p.kind == "inlet"]
    out = [p for p in case.patches if p.kind == "outlet"]
    wal = [p for p in case.patches if p.kind == "wall"]
    per = [p for p in case.patches if p.kind == "periodic"]
    L = ["# Boundary definition", "#", "# inlet", "#---------------------------",
         f" {len(inl)}\t\t# number of inlets", "#ID_BID FT_Ista_Iend_Jsta_Jend_Ksta_Kend"]
    for n, p in enumerate(inl, 1):
        L.append(f"{n}\t1\t{p.face}\t" + "\t".join(str(v) for v in p.rng))
    L += ["#", "# outlet", "#---------------------------",
          f" {len(out)}\t\t# number of outlets", "#ID_BID_FT_Ista_Iend_Jsta_Jend_Ksta_Kend"]
    for n, p in enumerate(out, 1):
        L.append(f"{n}\t1\t{p.face}\t" + "\t".join(str(v) for v in p.rng))
    L += ["#", "# wall", "#---------------------------",
          f" {len(wal)}\t\t# number of Walls", "#ID_BID_FT_wrot_Ista_Iend_Jsta_Jend_Ksta_Kend"]
    for n, p in enumerate(wal, 1):
        L.append(f"{n}\t1\t{p.face}\t{p.rotate}\t" + "\t".join(str(v) for v in p.rng))
    L += ["#", "# periodic", "#---------------------------",
          f"{len(per)}\t\t# number of Periodics",
          "#ID_ori_BID1_FT1_Ista1_Iend1_Jsta1_Jend1_Ksta1_Kend1_BID2_FT2_..."]
    for n, p in enumerate(per, 1):
        L.append(f"{n}\t{p.orient}\t1\t{p.face}\t" + "\t".join(str(v) for v in p.rng)
                 + f"\t1\t{p.face2}\t" + "\t".join(str(v) for v in p.rng2))
    L += ["#", "# interior", "#--------------------------", " 0\t\t# number of Interiors",
          "#ID_ori_BID1_FT1_...", "#", "# mixing plane", "#--------------------------",
          " 0\t\t# number of MixingPlanes", "#ID_ori_BID1_FT1_...", "#", "# Blocks",
          "#--------------------------", "1\t\t# number of Blocks", "#BID_IM_JM_KM_Nblade_rpm",
          f"1    {IM} {JM} {KM}\t{case.nblade}  {case.rpm:.17g}", ""]
    return "\n".join(L)


def write_grid(path: str, nodes: np.ndarray) -> None:
    """Grid file: block count, block id, ``IM JM KM``, then one ``x y z`` line per node with
    k outermost and i innermost (``source/UserInput.cpp:275-285``). 17 significant digits so the
    reference's ``stringstream`` parse recovers the exact doubles."""
    IM, JM, KM = nodes.shape[:3]
    arr = np.ascontiguousarray(np.transpose(nodes, (2, 1, 0, 3)).reshape(-1, 3))
    with open(path, "w") as f:
        f.write("1\n1\n%d %d %d\n" % (IM, JM, KM))
        np.savetxt(f, arr, fmt="%.17g")


def write_case(case: Case, directory: str, gridfile: str = "grid.dat") -> None:
    os.makedirs(directory, exist_ok=True)
    write_grid(os.path.join(directory, gridfile), case.nodes)
    with open(os.path.join(directory, "BoundaryDefinition.dat"), "w") as f:
        f.write(_bc_text(case))
    with open(os.path.join(directory, "config.dat"), "w") as f:
        f.write(_config_text(case.options, gridfile, "BoundaryDefinition.dat"))


# ----------------------------------------------------------------------------------------
# plain-method case: annular-sector duct
# ----------------------------------------------------------------------------------------
def annular_duct(IM: int = 33, JM: int = 33, KM: int = 65, r_hub: float = 0.20,
                 r_tip: float = 0.30, sector_deg: float = 10.0, length: float = 0.30,
                 bump: float = 0.10, d1: float = 1e-4, options: Optional[Dict[str, str]] = None,
                 name: str = "duct") -> Case:
    """Annular sector duct (i = span, j = pitch, k = axial), 3-D sinusoidal hub bump of
    ``bump`` x span over the middle third of the length, modulated in pitch, two-sided tanh
    clustering with first spacing ``d1`` at hub and casing. Stationary (rpm 0)."""
    span = r_tip - r_hub
    s_i = two_sided_spacing(IM - 1, 1.0, d1 / span)
    th = np.deg2rad(np.linspace(-0.5 * sector_deg, 0.5 * sector_deg, JM))
    z = np.linspace(0.0, length, KM)
    nodes = np.zeros((IM, JM, KM, 3))
    for k in range(KM):
        zz = z[k]
        t = (zz - length / 3.0) / (length / 3.0)
        hb = math.sin(math.pi * t) ** 2 if 0.0 <= t <= 1.0 else 0.0
        for j in range(JM):
            mod = 0.75 + 0.25 * math.cos(2.0 * math.pi * th[j] / np.deg2rad(sector_deg))
            rh = r_hub + bump * span * hb * mod
            r = rh + (r_tip - rh) * s_i
            nodes[:, j, k, 0] = r * math.cos(th[j])
            nodes[:, j, k, 1] = r * math.sin(th[j])
            nodes[:, j, k, 2] = zz
    patches = [
        Patch("inlet", 5, (1, IM - 1, 1, JM - 1, 1, 1)),
        Patch("outlet", 6, (1, IM - 1, 1, JM - 1, KM, KM)),
        Patch("wall", 1, (1, 1, 1, JM - 1, 1, KM - 1), rotate=1),
        Patch("wall", 2, (IM, IM, 1, JM - 1, 1, KM - 1), rotate=0),
        Patch("periodic", 3, (1, IM - 1, 1, 1, 1, KM - 1), face2=4,
              rng2=(1, IM - 1, JM, JM, 1, KM - 1), orient=2),
    ]
    nblade = int(round(360.0 / sector_deg))
    opt = {"Pout": "%.1f" % (0.92 * 101325.0)}
    opt.update(options or {})
    return Case(name, nodes, patches, nblade, 0.0, opt)


# ----------------------------------------------------------------------------------------
# rotor passage: single-block H-grid around one blade
# ----------------------------------------------------------------------------------------
def _naca_thickness(x: np.ndarray, tmax: float) -> np.ndarray:
    """Closed-trailing-edge 4-digit thickness polynomial scaled to ``tmax`` (fraction of
    chord); zero at both ends of the chord."""
    x = np.clip(x, 0.0, 1.0)
    return 5.0 * tmax * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x ** 2
                         + 0.2843 * x ** 3 - 0.1036 * x ** 4)


def rotor_passage(IM: int = 49, JM: int = 49, KM: int = 129, nblade: int = 22,
                  r_hub: float = 0.10, r_tip: float = 0.25, chord_ax: float = 0.06,
                  camber_hub: float = 40.0, camber_tip: float = 25.0,
                  stagger_hub: float = 30.0, stagger_tip: float = 60.0, tmax: float = 0.06,
                  rpm: float = 16000.0, d1: float = 1e-5, stagger_offset: float = 0.0,
                  k_le: Optional[int] = None, k_te: Optional[int] = None,
                  options: Optional[Dict[str, str]] = None, name: str = "rotor") -> Case:
    """H-grid passage of a compressor rotor rotating about z.

    Nodes ``k_le .. k_te`` (1-based) carry the blade; the camber line has a metal angle that
    varies linearly along the chord from ``stagger + camber/2`` at the leading edge to
    ``stagger - camber/2`` at the trailing edge (circular arc), with stagger and camber linear in
    span. The blade leans against the rotation (d(r theta)/dz < 0 for rpm > 0) so that it does
    work on the flow. Up- and downstream the camber line continues with a slope that decays to
    axial at the inlet/outlet planes, and the two j-faces there are exactly one pitch apart
    (periodic). Clustering: first spacing ``d1`` at hub, casing and blade surfaces."""
    if k_le is None or k_te is None:
        n_up = (KM - 1) // 3
        n_up -= n_up % 4
        k_le = n_up + 1
        k_te = KM - n_up
    pitch = 2.0 * math.pi / nblade
    span = r_tip - r_hub
    s_i = two_sided_spacing(IM - 1, 1.0, d1 / span)
    n_up, n_bl, n_dn = k_le - 1, k_te - k_le, KM - k_te
    dz = chord_ax / n_bl
    z_le, z_te = n_up * dz, n_up * dz + chord_ax
    # axial node positions: uniform over the blade, stretched up/downstream
    z = np.zeros(KM)
    up_len, dn_len = 1.0 * chord_ax, 1.0 * chord_ax
    for k in range(KM):
        if k < k_le - 1:
            t = (k_le - 1 - k) / n_up
            z[k] = z_le - up_len * (0.35 * t + 0.65 * t * t)
        elif k <= k_te - 1:
            z[k] = z_le + (k - (k_le - 1)) * dz
        else:
            t = (k - (k_te - 1)) / n_dn
            z[k] = z_te + dn_len * (0.35 * t + 0.65 * t * t)
    z -= z[0]
    z_le, z_te = z[k_le - 1], z[k_te - 1]
    nodes = np.zeros((IM, JM, KM, 3))
    sgn = -1.0 if rpm >= 0 else 1.0
    for i in range(IM):
        frac = s_i[i]
        r = r_hub + span * frac
        stagger = math.radians(stagger_hub + (stagger_tip - stagger_hub) * frac + stagger_offset)
        camber = math.radians(camber_hub + (camber_tip - camber_hub) * frac)
        b_le, b_te = stagger + 0.5 * camber, stagger - 0.5 * camber
        # camber line r*theta(z) over the blade, integrated from the linear metal angle
        xb = (z[k_le - 1:k_te] - z_le) / chord_ax
        beta = b_le + (b_te - b_le) * xb
        slope = np.tan(beta)
        rth_b = np.concatenate([[0.0], np.cumsum(0.5 * (slope[1:] + slope[:-1]) * np.diff(z[k_le - 1:k_te]))])
        rth = np.zeros(KM)
        rth[k_le - 1:k_te] = rth_b
        # upstream: slope decays linearly from tan(b_le) at the LE to 0 at the inlet plane
        for k in range(k_le - 2, -1, -1):
            a = (z[k] - z[0]) / (z_le - z[0])
            a1 = (z[k + 1] - z[0]) / (z_le - z[0])
            rth[k] = rth[k + 1] - 0.5 * (a + a1) * math.tan(b_le) * (z[k + 1] - z[k])
        for k in range(k_te, KM):
            a = (z[-1] - z[k]) / (z[-1] - z_te)
            a1 = (z[-1] - z[k - 1]) / (z[-1] - z_te)
            rth[k] = rth[k - 1] + 0.5 * (a + a1) * math.tan(b_te) * (z[k] - z[k - 1])
        th_c = sgn * rth / r
        th_c -= 0.5 * (th_c.max() + th_c.min())
        # circumferential half-thickness over the blade (normal thickness / cos(beta))
        half = np.zeros(KM)
        cos_b = np.cos(beta)
        half[k_le - 1:k_te] = 0.5 * _naca_thickness(xb, tmax) * (chord_ax / math.cos(stagger)) / cos_b / r
        th_lo = th_c + half           # suction/pressure surface of the blade at j = 1
        th_hi = th_c + pitch - half   # surface of the next blade at j = JM
        s_j = np.zeros((KM, JM))
        for k in range(KM):
            if k_le - 1 <= k <= k_te - 1:
                wdth = r * (th_hi[k] - th_lo[k])
                s_j[k] = two_sided_spacing(JM - 1, 1.0, min(d1 / max(wdth, 1e-9), 1.0 / (JM - 1)))
            else:
                s_j[k] = np.linspace(0.0, 1.0, JM)
        # blend the blade clustering smoothly into the uniform up/downstream distribution
        for k in range(KM):
            if k < k_le - 1:
                w = max(0.0, 1.0 - (k_le - 1 - k) / 6.0)
                s_j[k] = w * s_j[k_le - 1] + (1 - w) * s_j[k]
            elif k > k_te - 1:
                w = max(0.0, 1.0 - (k - (k_te - 1)) / 6.0)
                s_j[k] = w * s_j[k_te - 1] + (1 - w) * s_j[k]
        for k in range(KM):
            th_row = th_lo[k] + (th_hi[k] - th_lo[k]) * s_j[k]
            nodes[i, :, k, 0] = r * np.cos(th_row)
            nodes[i, :, k, 1] = r * np.sin(th_row)
            nodes[i, :, k, 2] = z[k]
    c_le, c_te = k_le, k_te - 1        # blade cell range in k (1-based cells)
    patches = [
        Patch("inlet", 5, (1, IM - 1, 1, JM - 1, 1, 1)),
        Patch("outlet", 6, (1, IM - 1, 1, JM - 1, KM, KM)),
        Patch("wall", 1, (1, 1, 1, JM - 1, 1, KM - 1), rotate=1),
        Patch("wall", 2, (IM, IM, 1, JM - 1, 1, KM - 1), rotate=0),
        Patch("wall", 3, (1, IM - 1, 1, 1, c_le, c_te), rotate=1),
        Patch("wall", 4, (1, IM - 1, JM, JM, c_le, c_te), rotate=1),
        Patch("periodic", 3, (1, IM - 1, 1, 1, 1, c_le - 1), face2=4,
              rng2=(1, IM - 1, JM, JM, 1, c_le - 1), orient=2),
        Patch("periodic", 3, (1, IM - 1, 1, 1, c_te + 1, KM - 1), face2=4,
              rng2=(1, IM - 1, JM, JM, c_te + 1, KM - 1), orient=2),
    ]
    opt = {"Pout": "%.1f" % (1.20 * 101325.0), "Ma0": "0.45"}
    opt.update(options or {})
    return Case(name, nodes, patches, nblade, rpm, opt)


def sample_operating_points(n: int, seed: int = 2024) -> List[Dict[str, float]]:
    """Seeded operating-point sampler of the batched form: back pressure U[1.05, 1.30] x p_t,
    speed in {0.8, 0.9, 1.0} x 16000 rpm, mesh in {97x41x41, 129x49x49, 161x65x65} (axial x
    pitch x span), stagger perturbed by N(0, 1 deg)."""
    rng = np.random.default_rng(seed)
    meshes = [(41, 41, 97), (49, 49, 129), (65, 65, 161)]
    pts = []
    for _ in range(n):
        m = meshes[int(rng.integers(0, 3))]
        pts.append({"pb": float(rng.uniform(1.05, 1.30)),
                    "rpm": float(16000.0 * [0.8, 0.9, 1.0][int(rng.integers(0, 3))]),
                    "IM": m[0], "JM": m[1], "KM": m[2],
                    "stagger_offset": float(rng.normal(0.0, 1.0))})
    return pts


# ----------------------------------------------------------------------------------------
# multi-block cases: blocks stacked along the axis, joined by interfaces
# ----------------------------------------------------------------------------------------
@dataclasses.dataclass
class BlockPatch:
    """A patch of a multi-block case: ``block`` (1-based) owns it; interfaces and periodic pairs
    name the partner block in ``block2``."""
    patch: Patch
    block: int
    block2: int = 0


@dataclasses.dataclass
class MultiBlockCase:
    name: str
    blocks: List[np.ndarray]       # per block (IM, JM, KM, 3) nodes
    patches: List[BlockPatch]      # inlets, outlets, walls, periodic pairs and interfaces
    nblade: int
    rpm: float
    options: Dict[str, str]
    block_nblade: Optional[List[int]] = None     # per block, when the blocks differ (stages)
    block_rpm: Optional[List[float]] = None

    @property
    def n_cells(self) -> int:
        return sum((b.shape[0] - 1) * (b.shape[1] - 1) * (b.shape[2] - 1) for b in self.blocks)


def split_axial(case: Case, cuts: Sequence[int], name: Optional[str] = None) -> MultiBlockCase:
    """The single-block case cut into blocks at the node planes ``k = cuts`` (1-based), in the
    H-H-H arrangement of the reference's rotor-67 example (``run_rotor67/BoundaryDefinition.dat``):
    neighbouring blocks share their cut plane and are joined by an interface between the k+ face
    of the upstream block and the k- face of the downstream one (orientation 2: the i index of one
    face runs along the j index of the other's shadow order). Patches on i- and j-faces are split
    at the cuts; the inlet goes to the first block, the outlet to the last."""
    IM, JM, KM = case.dims
    edges = [1] + list(cuts) + [KM]
    if any(b <= a for a, b in zip(edges, edges[1:])):
        raise ValueError("cuts must increase strictly inside (1, KM)")
    blocks = [np.ascontiguousarray(case.nodes[:, :, k0 - 1:k1, :]) for k0, k1 in zip(edges, edges[1:])]
    out: List[BlockPatch] = []
    nb = len(blocks)
    for p in case.patches:
        if p.kind in ("inlet", "outlet") or p.face in (5, 6):
            b = 1 if p.face == 5 else nb
            k = 1 if p.face == 5 else blocks[-1].shape[2]
            r = list(p.rng)
            r[4] = r[5] = k
            out.append(BlockPatch(dataclasses.replace(p, rng=tuple(r)), b))
            continue
        for b, (k0, k1) in enumerate(zip(edges, edges[1:]), 1):
            # cells k0 .. k1-1 of the single block are cells 1 .. k1-k0 of block b
            lo, hi = max(p.rng[4], k0), min(p.rng[5], k1 - 1)
            if lo > hi:
                continue
            r = list(p.rng)
            r[4], r[5] = lo - k0 + 1, hi - k0 + 1
            q = dataclasses.replace(p, rng=tuple(r))
            if p.kind == "periodic":
                r2 = list(p.rng2)
                r2[4], r2[5] = r[4], r[5]
                q = dataclasses.replace(q, rng2=tuple(r2))
                out.append(BlockPatch(q, b, b))
            else:
                out.append(BlockPatch(q, b))
    for b in range(1, nb):
        kb = blocks[b - 1].shape[2]
        face = Patch("interior", 6, (1, IM - 1, 1, JM - 1, kb, kb), face2=5, rng2=(1, IM - 1, 1, JM - 1, 1, 1), orient=2)
        out.append(BlockPatch(face, b, b + 1))
    return MultiBlockCase(name or case.name + "_mb", blocks, out, case.nblade, case.rpm, dict(case.options))


def _bc_text_multi(case: MultiBlockCase) -> str:
    def sel(kind):
        return [p for p in case.patches if p.patch.kind == kind]

    def rng(t):
        return "\t".join(str(v) for v in t)

    inl, out, wal, per, itf = sel("inlet"), sel("outlet"), sel("wall"), sel("periodic"), sel("interior")
    mix = sel("mixing")
    L = ["# Boundary definition", "#", "# inlet", "#---------------------------",
         f" {len(inl)}\t\t# number of inlets", "#ID_BID FT_Ista_Iend_Jsta_Jend_Ksta_Kend"]
    L += [f"{n}\t{p.block}\t{p.patch.face}\t{rng(p.patch.rng)}" for n, p in enumerate(inl, 1)]
    L += ["#", "# outlet", "#---------------------------",
          f" {len(out)}\t\t# number of outlets", "#ID_BID_FT_Ista_Iend_Jsta_Jend_Ksta_Kend"]
    L += [f"{n}\t{p.block}\t{p.patch.face}\t{rng(p.patch.rng)}" for n, p in enumerate(out, 1)]
    L += ["#", "# wall", "#---------------------------",
          f" {len(wal)}\t\t# number of Walls", "#ID_BID_FT_wrot_Ista_Iend_Jsta_Jend_Ksta_Kend"]
    L += [f"{n}\t{p.block}\t{p.patch.face}\t{p.patch.rotate}\t{rng(p.patch.rng)}" for n, p in enumerate(wal, 1)]
    L += ["#", "# periodic", "#---------------------------", f"{len(per)}\t\t# number of Periodics",
          "#ID_ori_BID1_FT1_Ista1_Iend1_Jsta1_Jend1_Ksta1_Kend1_BID2_FT2_..."]
    L += [f"{n}\t{p.patch.orient}\t{p.block}\t{p.patch.face}\t{rng(p.patch.rng)}\t{p.block2}\t{p.patch.face2}\t"
          f"{rng(p.patch.rng2)}" for n, p in enumerate(per, 1)]
    L += ["#", "# interior", "#--------------------------", f" {len(itf)}\t\t# number of Interiors",
          "#ID_ori_BID1_FT1_Ista1_Iend1_Jsta1_Jend1_Ksta1_Kend1_BID2_FT2_..."]
    L += [f"{n}\t{p.patch.orient}\t{p.block}\t{p.patch.face}\t{rng(p.patch.rng)}\t{p.block2}\t{p.patch.face2}\t"
          f"{rng(p.patch.rng2)}" for n, p in enumerate(itf, 1)]
    L += ["#", "# mixing plane", "#--------------------------", f" {len(mix)}\t\t# number of MixingPlanes",
          "#ID_ori_BID1_FT1_..."]
    L += [f"{n}\t{p.patch.orient}\t{p.block}\t{p.patch.face}\t{rng(p.patch.rng)}\t{p.block2}\t{p.patch.face2}\t"
          f"{rng(p.patch.rng2)}" for n, p in enumerate(mix, 1)]
    L += ["#", "# Blocks", "#--------------------------",
          f"{len(case.blocks)}\t\t# number of Blocks", "#BID_IM_JM_KM_Nblade_rpm"]
    for b, nodes in enumerate(case.blocks, 1):
        IM, JM, KM = nodes.shape[:3]
        nbl = case.block_nblade[b - 1] if case.block_nblade else case.nblade
        rpm = case.block_rpm[b - 1] if case.block_rpm else case.rpm
        L.append(f"{b}    {IM} {JM} {KM}\t{nbl}  {rpm:.17g}")
    L.append("")
    return "\n".join(L)


def write_multiblock_case(case: MultiBlockCase, directory: str, gridfile: str = "grid.dat") -> None:
    """Grid file with every block (block count, then per block its id, ``IM JM KM`` and nodes),
    BoundaryDefinition.dat with block ids, config.dat."""
    os.makedirs(directory, exist_ok=True)
    with open(os.path.join(directory, gridfile), "w") as f:
        f.write("%d\n" % len(case.blocks))
        for b, nodes in enumerate(case.blocks, 1):
            IM, JM, KM = nodes.shape[:3]
            f.write("%d\n%d %d %d\n" % (b, IM, JM, KM))
            np.savetxt(f, np.ascontiguousarray(np.transpose(nodes, (2, 1, 0, 3)).reshape(-1, 3)), fmt="%.17g")
    with open(os.path.join(directory, "BoundaryDefinition.dat"), "w") as f:
        f.write(_bc_text_multi(case))
    with open(os.path.join(directory, "config.dat"), "w") as f:
        f.write(_config_text(case.options, gridfile, "BoundaryDefinition.dat"))


def stage_passage(IM: int = 9, JM1: int = 9, KM1: int = 17, JM2: int = 9, KM2: int = 17, nblade1: int = 22,
                  nblade2: int = 30, rpm: float = 16000.0, options: Optional[Dict[str, str]] = None,
                  name: str = "stage") -> MultiBlockCase:
    """A rotor passage followed by a stator passage, joined by a mixing plane (the reference's
    CMesh::BndCondMixingPlane between the k+ face of block 1 and the k- face of block 2): block 1 is
    ``rotor_passage`` with ``nblade1`` blades at ``rpm``, block 2 a stationary blade row of
    ``nblade2`` blades (the same generator with its stagger mirrored and no rotation) placed
    downstream, with the same radial node distribution so that the rows of the mixing plane match.
    The rotor's outlet face and the stator's inlet face become the mixing plane."""
    opts = dict(options or {})
    rot = rotor_passage(IM=IM, JM=JM1, KM=KM1, nblade=nblade1, rpm=rpm, options=opts, name=name)
    sta = rotor_passage(IM=IM, JM=JM2, KM=KM2, nblade=nblade2, rpm=0.0, stagger_hub=-30.0, stagger_tip=-20.0,
                        camber_hub=-30.0, camber_tip=-20.0, options=opts, name=name)
    n2 = sta.nodes.copy()
    n2[..., 2] += rot.nodes[..., 2].max() - n2[..., 2].min()
    patches: List[BlockPatch] = []
    for p in rot.patches:
        if p.kind == "outlet":
            continue
        patches.append(BlockPatch(p, 1, 1 if p.kind == "periodic" else 0))
    for p in sta.patches:
        if p.kind == "inlet":
            continue
        if p.kind == "wall" and p.face in (1, 2):
            p = dataclasses.replace(p, rotate=0)           # stator hub and casing do not rotate
        patches.append(BlockPatch(p, 2, 2 if p.kind == "periodic" else 0))
    mp = Patch("mixing", 6, (1, IM - 1, 1, JM1 - 1, KM1, KM1), face2=5, rng2=(1, IM - 1, 1, JM2 - 1, 1, 1), orient=2)
    patches.append(BlockPatch(mp, 1, 2))
    return MultiBlockCase(name, [rot.nodes, n2], patches, nblade1, rpm, opts, block_nblade=[nblade1, nblade2],
                          block_rpm=[rpm, 0.0])
