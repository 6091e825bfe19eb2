"""Writer for the reference's ``$KEY`` input decks.

Emits the region, control, initial, material, time-step and main input files
in the formats the reference parses, so that the same synthetic mesh can be run
through the reference solver (parity oracle, CPU baseline) and through this
library.  Formats:

* region file: ``np ne 0``, node records ``name x y z``, element records
  ``name mat tri n1..n6`` (Grid.cpp:159-298, :1159-1167)
* control file: ``0 ne``, records ``name lineNo line c1 c2 mid`` (Grid.cpp:398-424)
* initial file: ``# time x 40700 U V S`` header, ``np 0``, records
  ``name U V S`` (Grid.cpp:510-760; element count 0 means no element records)
* material file: ``$BOTTOM no MANN n 0 1.0``, ``$TURBULENCE no vt ...``
  (Type.cpp:502-520, :670-690)
* time-step file keys (Timeint.cpp:2003-2345) and main-file keys
  (Project.cpp:1706-1860)
"""

from __future__ import annotations

import os

import numpy as np

from .meshgen import Mesh


def fmt(v: float) -> str:
    return repr(float(v))


def write_deck(mesh: Mesh, out_dir: str, *, steady: bool = True, dt: float = 3600.0,
               nsteps: int = 1, theta: float = 1.0, maxiter: int = 60, hydrograph=None,
               solver_maxiter: int = 1000, solver_maxdiff: float = 1.0e-8,
               conv_uv: float = 1.0e-9, conv_s: float = 1.0e-9,
               relax=(2, 0.001, 0.1, 0.5, 0.5, 0.1),
               dryrew=(2, 10, 0.01, 0.02, 100, 5), report_level: int = 3,
               restart_file: str | None = None) -> str:
    """Write a complete deck; returns the main input file path.

    ``hydrograph`` is a list of ``(t, Q, S)`` rows; when given the inlet is a
    QTINLET discharge hydrograph, otherwise a constant QINLET with the mesh's Q.
    """
    os.makedirs(out_dir, exist_ok=True)
    npn, ne = mesh.np, mesh.ne
    with open(os.path.join(out_dir, "region.2dm"), "w") as f:
        f.write(f"{npn} {ne} 0\n")
        for k in range(npn):
            f.write(f"{k + 1} {fmt(mesh.x[k])} {fmt(mesh.y[k])} {fmt(mesh.z[k])}\n")
        for e in range(ne):
            nd = " ".join(str(int(n) + 1) for n in mesh.elems[e])
            f.write(f"{e + 1} {int(mesh.elem_type[e])} tri {nd}\n")
    ctl = []
    for no, seg in sorted(mesh.lines.items()):
        for s in seg:
            ctl.append((no, s))
    with open(os.path.join(out_dir, "control.2dm"), "w") as f:
        f.write(f"0 {len(ctl)}\n")
        for e, (no, s) in enumerate(ctl):
            f.write(f"{e + 1} {no} line {s[0] + 1} {s[1] + 1} {s[2] + 1}\n")
    with open(os.path.join(out_dir, "init.dat"), "w") as f:
        f.write("# 0.0 x 40700 U V S\n")
        f.write(f"{npn} 0\n")
        for k in range(npn):
            f.write(f"{k + 1} {fmt(mesh.U0[k])} {fmt(mesh.V0[k])} {fmt(mesh.S0[k])}\n")
    with open(os.path.join(out_dir, "mat.inp"), "w") as f:
        f.write("$RISMO2D 40700\n")
        for no, n, _vt in mesh.materials:
            f.write(f"$BOTTOM {no} MANN {fmt(n)} 0 1.0\n")
        for no, _n, vt in mesh.materials:
            f.write(f"$TURBULENCE {no} {fmt(vt)} 1.0 0.0 0.0 0.0 0.0 0.0\n")
    Q = mesh.meta["Q"]
    S_out = mesh.meta["S_out"]
    xo = float(mesh.x[mesh.lines[2][0][0]])
    lines = ["$RISMO2D 40700",
             f"$TM_STEPS 1 {nsteps} 0",
             f"$TM_INTERVAL {fmt(dt)} 100.0 100.0",
             f"$TM_WEIGHT {fmt(theta)} 1.0 1.0",
             f"$TM_OUTPUT 1 to {nsteps} step {nsteps}",
             "$TM_STEP_NO 1",
             "$TM_CYCLE 1",
             f"$TM_STATIONARY {1 if steady else 0}",
             "$TM_TURBULENCE 1",
             "$TM_DISPERSION 0",
             f"$TM_MAXITER {maxiter}",
             "$TM_SOLVER 1"]
    if hydrograph is None:
        lines.append(f"$TM_LINE QINLET 1 {fmt(Q)} {fmt(mesh.meta.get('S_in', S_out))}")
    else:
        for t, q, s in hydrograph:
            lines.append(f"$TM_LINE QTINLET 1 {fmt(q)} {fmt(s)} {fmt(t)}")
    lines.append(f"$TM_LINE OUTLET 2 {fmt(S_out)} {fmt(xo)} 0.0 0 0.0")
    with open(os.path.join(out_dir, "steps.inp"), "w") as f:
        f.write("\n".join(lines) + "\n")
    main = ["$RISMO2D 40700",
            f"$REPORTLEVEL {report_level}",
            "$REPORTFILE report.txt",
            "$TIMESTEPFILE steps.inp",
            "$MATERIALFILE mat.inp",
            "$REGIONFILE region.2dm",
            "$CONTROLFILE control.2dm",
            "$ASC_INITFILE init.dat",
            f"$SOLVER 1 5 1 0 100 {solver_maxiter} {fmt(solver_maxdiff)}",
            f"$CONVERGENCE {fmt(conv_uv)} {fmt(conv_s)} 1.0e-4 1.0e-4",
            "$RELAX " + " ".join(str(v) for v in relax),
            "$DRYREW " + " ".join(str(v) for v in dryrew),
            "$GPDEGREE 5"]
    if restart_file:
        main.append(f"$ASC_RESTFILE {restart_file}")
    path = os.path.join(out_dir, "main.inp")
    with open(path, "w") as f:
        f.write("\n".join(main) + "\n")
    return path
