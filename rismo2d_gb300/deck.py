"""Writer and reader of the reference's ``$KEY`` input decks.

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

import dataclasses
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


# ---- reading decks -------------------------------------------------------------

@dataclasses.dataclass
class DeckRun:
    """A deck read back: mesh and initial state, parameters, line boundary
    conditions and the time-step control of the time-step file."""

    mesh: Mesh
    params: object                 # sim.Params
    line_bcs: list                 # [(kind, line, rows)]: QINLET [(Q, S)], QTINLET [(t, Q, S)], OUTLET [(S,)]
    steady: bool
    dt: float
    first_step: int
    last_step: int
    max_newton: int
    time0: float                   # time of the initial file (s)
    initial: dict | None           # the initial file's node values (None: no initial file)
    files: dict                    # key -> path of the files the main deck names


def parse_time(t: str) -> float:
    """Seconds of a reference time string: "s", "m:s", "h:m:s", "d:h:m:s" or
    "dTh:m:s" (TIME::Set, Times.h:240-290)."""
    t = t.strip()
    if "T" in t:
        d, rest = t.split("T", 1)
        h, m, s = rest.split(":")
        return ((int(d) * 24 + int(h)) * 60 + int(m)) * 60 + float(s)
    parts = t.split(":")
    val = [0, 0, 0]
    sec = float(parts[-1])
    for i, p in enumerate(reversed(parts[:-1])):
        val[2 - i] = int(p)
    return ((val[0] * 24 + val[1]) * 60 + val[2]) * 60 + sec


def format_time(sec: float) -> str:
    """The reference's time string (TIME::Get, Times.h:331-335): [dT]HH:MM:SS.micro."""
    micro_total = int(round(sec * 1e6))
    s, micro = divmod(micro_total, 1000000)
    m, s = divmod(s, 60)
    h, m = divmod(m, 60)
    d, h = divmod(h, 24)
    if d > 0:
        return f"{d}T{h:02d}:{m:02d}:{s:02d}.{micro:06d}"
    return f"{h:02d}:{m:02d}:{s:02d}.{micro:06d}"


def _lines(path: str):
    with open(path) as f:
        for ln in f:
            ln = ln.strip()
            if ln:
                yield ln


def _keys(path: str) -> list:
    """($KEY, tokens) of every $-line of a key file, in file order."""
    out = []
    for ln in _lines(path):
        if ln.startswith("$"):
            tok = ln.split()
            out.append((tok[0][1:], tok[1:]))
    return out


def read_region(path: str):
    """Region file (GRID::InputRegion, Grid.cpp:159-298): ``np ne 0``, node
    records ``name x y z``, element records ``name mat tri n1..n6``; node and
    element names are 1-based and select the slot."""
    it = _lines(path)
    npn, ne = (int(v) for v in next(it).split()[:2])
    x, y, z = np.zeros(npn), np.zeros(npn), np.zeros(npn)
    for _ in range(npn):
        tok = next(it).split()
        k = int(tok[0]) - 1
        x[k], y[k], z[k] = float(tok[1]), float(tok[2]), float(tok[3])
    elems = np.zeros((ne, 6), np.int32)
    etype = np.zeros(ne, np.int32)
    for _ in range(ne):
        tok = next(it).split()
        e = int(tok[0]) - 1
        if tok[2] != "tri" or len(tok) < 9:
            raise ValueError(f"{path}: only six-node triangles are supported ({' '.join(tok[:3])})")
        etype[e] = int(tok[1])
        elems[e] = [int(v) - 1 for v in tok[3:9]]
    return x, y, z, elems, etype


def read_control(path: str) -> dict:
    """Control file (Grid.cpp:398-424): ``0 ne``, records ``name lineNo line c1 c2 mid``."""
    it = _lines(path)
    _np0, ne = (int(v) for v in next(it).split()[:2])
    lines: dict = {}
    for _ in range(ne):
        tok = next(it).split()
        if tok[2] != "line":
            raise ValueError(f"{path}: only line elements are supported")
        lines.setdefault(int(tok[1]), []).append([int(v) - 1 for v in tok[3:6]])
    return {no: np.asarray(seg, np.int32) for no, seg in lines.items()}


def read_initial(path: str) -> dict:
    """Initial / restart file (GRID::InputInitial, Grid.cpp:508-760): header
    ``# time x release var,var,...`` -- variables by name from release 40000
    on, else the fixed columns of release 280 -- then ``np ne``, node records
    ``name values...`` and, when ``ne`` > 0, element records (skipped here).
    Returns the time (s), the release and per-node arrays indexed by name - 1
    (U, V, W, S, dUdt, dVdt, dSdt, K, D, C, qb, Zb; absent ones are None)."""
    names = ("U", "V", "W", "S", "dUdt", "dVdt", "dSdt", "K", "D", "C", "qb", "Zb")
    it = _lines(path)
    head = next(it)[1:].replace(",", " ").split()
    time = parse_time(head[0])
    release = int(head[2]) if len(head) > 2 else 0
    if release >= 40000:
        cols = [v for v in head[3:]]
    elif release >= 280:
        cols = ["U", "V", "S", "K", "D", "C", "dUdt", "dVdt", "dSdt"]
    else:
        cols = ["U", "V", "W", "S", "K", "D", "C", "dUdt", "dVdt", "dSdt"]
    npn = int(next(it).split()[0])
    vals = {n: None for n in names}
    present = [c if c in names else None for c in cols]
    for c in present:
        if c is not None:
            vals[c] = np.zeros(npn)
    for _ in range(npn):
        tok = next(it).replace(",", " ").split()
        k = int(tok[0]) - 1
        for c, v in zip(present, tok[1:]):
            if c is not None:
                vals[c][k] = float(v)
    vals["time"] = time
    vals["release"] = release
    return vals


def bed_zor(mesh: Mesh) -> np.ndarray:
    """The reference's bed NODE::zor of a mesh: the region file's elevation at the
    corners, the mean of the two corners at the mid-side nodes."""
    zor = np.asarray(mesh.z, np.float64).copy()
    for k, (a, b) in enumerate(((0, 1), (1, 2), (2, 0))):
        zor[mesh.elems[:, 3 + k]] = 0.5 * (mesh.z[mesh.elems[:, a]] + mesh.z[mesh.elems[:, b]])
    return zor


def write_restart(path: str, time: float, state: dict, release: int = 40700):
    """The reference's ASCII restart layout (GRID::OutputData, Grid.cpp:1183-1240):
    header with the variable list, ``np 0`` (no element records) and one record
    per node ``name U V S dUdt dVdt dSdt K D C qb Zb`` -- readable as an
    ``$ASC_INITFILE`` by the reference and by read_initial.  ``state`` holds
    U, V, S and optionally dUdt, dVdt, dSdt (zero when absent: a restart with
    theta = 1 does not read them) and z, the bed NODE::zor written as Zb
    (bed_zor); values are written to full double precision."""
    npn = len(state["U"])
    zero = np.zeros(npn)
    cols = [state["U"], state["V"], state["S"], state.get("dUdt", zero), state.get("dVdt", zero),
            state.get("dSdt", zero), zero, zero, zero, zero, state.get("z", zero)]
    with open(path, "w") as f:
        f.write(f"# {format_time(time):>22s}   Release {release}   U,V,S,dUdt,dVdt,dSdt,K,D,C,qb,Zb\n")
        f.write(f"{npn}  0\n")
        for k in range(npn):
            f.write(f"{k + 1:7d} " + " ".join(repr(float(c[k])) for c in cols) + "\n")


def read_deck(main_path: str) -> DeckRun:
    """Read a main deck and the files it names ($REGIONFILE, $CONTROLFILE,
    $MATERIALFILE, $TIMESTEPFILE, $ASC_INITFILE; keys of Project.cpp:1706-1860
    and Timeint.cpp:1530-2345).  Supported: six-node triangles, Manning
    friction, constant eddy viscosity, QINLET / QTINLET / OUTLET lines,
    BiCGStab with ILU(0) -- the subset of include/rg300_sim.h."""
    from .sim import Params
    base = os.path.dirname(os.path.abspath(main_path))
    files, params = {}, Params()
    for key, tok in _keys(main_path):
        if key in ("REGIONFILE", "CONTROLFILE", "MATERIALFILE", "TIMESTEPFILE", "ASC_INITFILE", "ASC_RESTFILE"):
            files[key] = os.path.join(base, tok[0])
        elif key == "SOLVER":
            if int(tok[1]) != 5:
                raise ValueError("only $SOLVER type 5 (BiCGStab) is supported")
            params.solver_maxiter, params.solver_maxdiff = int(tok[5]), float(tok[6])
        elif key == "CONVERGENCE":
            params.conv_uv, params.conv_s = float(tok[0]), float(tok[1])
        elif key == "RELAX":
            params.relax_method = int(tok[0])
            params.max_delta_uv, params.max_delta_s = float(tok[3]), float(tok[4])
        elif key == "DRYREW":
            params.dryrew_method, params.dryrew_freq = int(tok[0]), int(tok[1])
            params.dry_limit, params.rewet_limit = float(tok[2]), float(tok[3])
            params.countdown = int(tok[5])
            params.rewet_limit = max(params.rewet_limit, params.dry_limit)   # Project.cpp:1851
        elif key == "MAX_Us":
            params.max_us = float(tok[0])
    x, y, z, elems, etype = read_region(files["REGIONFILE"])
    lines = read_control(files["CONTROLFILE"]) if "CONTROLFILE" in files else {}
    nmat, vt = {}, {}
    for key, tok in _keys(files["MATERIALFILE"]):
        if key == "BOTTOM":
            if tok[1] != "MANN":
                raise ValueError("only Manning friction ($BOTTOM no MANN n) is supported")
            nmat[int(tok[0])] = float(tok[2])
        elif key == "TURBULENCE":
            vt[int(tok[0])] = float(tok[1])
    materials = [(no, nmat[no], vt.get(no, 0.0)) for no in sorted(nmat)]
    steady, dt, first, last, maxit = False, 0.0, 1, 1, params.max_newton
    bcs: dict = {}
    for key, tok in _keys(files["TIMESTEPFILE"]):
        if key == "TM_STEPS":
            first, last = int(tok[0]), int(tok[1])
        elif key == "TM_INTERVAL":
            dt = float(tok[0])                                    # seconds (Timeint.cpp:1567)
        elif key == "TM_WEIGHT":
            params.theta = float(tok[0])
        elif key == "TM_STATIONARY":
            steady = int(tok[0]) != 0
        elif key == "TM_MAXITER":
            maxit = int(tok[0])
        elif key == "TM_CYCLE":
            # cycles of a time step (Timeint.cpp:2003-2019): only the Taylor-Hood flow
            # cycle (kUVSCyc = 1, Project.h:102) is on this path; e.g. the element
            # reordering cycle 95 (Compute.cpp:666-680) is not
            cyc = [int(v) for v in " ".join(tok).replace(",", " ").split()]
            if any(c != 1 for c in cyc):
                raise ValueError(f"$TM_CYCLE {' '.join(map(str, cyc))}: only cycle 1 (UVS flow) is supported")
        elif key == "TM_LINE":
            kind, no = tok[0], int(tok[1])
            v = [float(a) for a in tok[2:]]
            if kind == "QINLET":
                bcs[(kind, no)] = [(v[0], v[1])]                  # one row, later ones overwrite
            elif kind == "QTINLET":
                bcs.setdefault((kind, no), []).append((v[2], v[0], v[1]))
            elif kind == "OUTLET":
                bcs.setdefault((kind, no), []).append((v[0],))
            else:
                raise ValueError(f"$TM_LINE {kind} is not supported")
    params.max_newton = maxit
    line_bcs = [(k, no, rows) for (k, no), rows in bcs.items()]
    init = read_initial(files["ASC_INITFILE"]) if "ASC_INITFILE" in files else None
    npn = len(x)
    if init is not None:
        S0 = init["S"] if init["S"] is not None else z.copy()
        U0 = init["U"] if init["U"] is not None else np.zeros(npn)
        V0 = init["V"] if init["V"] is not None else np.zeros(npn)
    else:
        S0, U0, V0 = z.copy(), np.zeros(npn), np.zeros(npn)   # GRID::InputInitial without a file
    meta = dict(kind="deck", main=os.path.abspath(main_path))
    for kind, no, rows in line_bcs:
        if kind == "OUTLET":
            meta.setdefault("S_out", rows[0][0])
        elif kind == "QINLET":
            meta.setdefault("Q", rows[0][0])
            meta.setdefault("S_in", rows[0][1])
    mesh = Mesh(x=x, y=y, z=z, elems=elems, elem_type=etype, lines=lines, S0=S0, U0=U0, V0=V0,
                materials=materials, meta=meta)
    return DeckRun(mesh=mesh, params=params, line_bcs=line_bcs, steady=steady, dt=dt, first_step=first,
                   last_step=last, max_newton=maxit, time0=init["time"] if init else 0.0, initial=init,
                   files=files)
