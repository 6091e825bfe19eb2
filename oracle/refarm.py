"""CPU baseline of the reference solver on the benchmark workload.

TEST INFRASTRUCTURE ONLY: used by bench.py's `--impl reference` arm and its
`cpu_baseline` field, never by the shipped library; nothing here loads
librg300.so.  The reference itself (a serial C++ program) cannot run on the
GPU host: its sources do not travel there and this build may not copy them.
What runs instead is this repository's C restatement of the reference's Newton
iteration arithmetic (oracle/rg_oracle.c, pinned bit-exact against the
reference's own dumps by tests/test_oracle_golden.py), on one host core as the
reference runs:

  * the system of the workload's initial wet model: U, V at every node of the
    wet triangles and S at their corners, numbered node by node (the
    reference's last-occurrence order changes where entries sit, not how many
    there are), CRS pattern in EQS::SetIndexMat's layout (orc_pattern);
  * element assembly (EQS_UVS2D::Region + CRSMAT::AssembleEqs_im, FP32 matrix
    as the reference stores it), CRSMAT::ScaleL2Norm and PRECO_ILU0::Factor,
    each timed once;
  * BICGSTAB::Iterate iterations with the ILU(0) preconditioner, timed one
    iteration per sample.

A time step of the reference is then N_newton x (assembly + scaling + factor)
+ N_krylov x (one BiCGStab iteration), with N_newton and N_krylov the
reference's OWN counts to ||B_k||/||B_0|| <= 1e-8 on the same kind of mesh:
the compiled reference's run recorded in tests/golden (the 2 km x 2 km window
of the braided river at the same resolution for the braided workload; the
200k meander itself for the meander workload).  The counts of the full 4M
mesh would be larger (Krylov iterations grow with the system), so the
estimate favours the reference.
"""

from __future__ import annotations

import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.abspath(os.path.join(HERE, ".."))
GOLDEN = os.path.join(REPO, "tests", "golden")
COUNTS_FIXTURE = {"braided4m": "braided_tile.npz", "meander200k": "meander200k.npz"}
DRY_LIMIT = 0.01


def reference_counts(workload: str, tol: float = 1e-8) -> dict | None:
    """Newton iterations per time step until ||B_k|| / ||B_0|| <= tol, and the BiCGStab
    iterations of those Newton iterations, from the compiled reference's recorded run."""
    path = os.path.join(GOLDEN, COUNTS_FIXTURE[workload])
    if not os.path.exists(path):
        return None
    g = np.load(path)
    newton, krylov, reached = [], [], []
    for k in range(int(g["steps"])):
        sc = g[f"scales_{k}"]
        kr = g[f"krylov_{k}"]
        r = sc / sc[0]
        hit = np.nonzero(r[1:] <= tol)[0]
        n = int(hit[0]) + 1 if len(hit) else len(sc)
        newton.append(n)
        krylov.append(int(np.sum(kr[:n])))
        reached.append(bool(len(hit)))
    return {"newton_per_step": float(np.mean(newton)), "krylov_per_step": float(np.mean(krylov)),
            "steps": len(newton), "tol_reached": all(reached), "fixture": os.path.basename(path)}


def build_system(wl):
    """The workload's initial wet model as the oracle's inputs, and its CRS pattern."""
    import oracle
    mesh = wl["mesh"]()
    t0 = time.perf_counter()
    H = mesh.S0 - mesh.z
    en = np.ascontiguousarray(mesh.elems, np.int32)
    wet_tri = np.all(H[en[:, :3]] > DRY_LIMIT, axis=1)
    els = np.ascontiguousarray(en[wet_tri])
    corner = np.zeros(mesh.np, bool)
    corner[els[:, :3].ravel()] = True
    used = np.zeros(mesh.np, bool)
    used[els.ravel()] = True
    eqno = np.full((mesh.np, 3), -1, np.int32)
    nodes = np.nonzero(used)[0]
    ndof = 2 + corner[nodes].astype(np.int64)
    first = np.concatenate([[0], np.cumsum(ndof)[:-1]])
    eqno[nodes, 0] = first
    eqno[nodes, 1] = first + 1
    cn = corner[nodes]
    eqno[nodes[cn], 2] = first[cn] + 2
    neq = int(ndof.sum())
    ptr, idx = oracle.pattern(mesh.np, els, eqno, neq)
    t1 = time.perf_counter()
    # nodal Manning friction of the initial state (MODEL::DoFriction)
    import ctypes as C
    mats = {no: n for no, n, _vt in mesh.materials}
    vts = {no: vt for no, _n, vt in mesh.materials}
    etype = np.asarray(mesh.elem_type)[wet_tri]
    elem_n = np.ascontiguousarray([mats[int(t)] for t in etype], np.float64)
    evt = np.ascontiguousarray([vts[int(t)] for t in etype], np.float64)
    af = np.ones(len(els))
    cf = np.zeros(mesh.np)
    nnd = np.full(len(els), 6, np.int32)
    zero = np.zeros(mesh.np)
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    oracle.lib().orc_friction(C.c_int(mesh.np), C.c_int(len(els)), P(els), P(nnd), P(elem_n), P(af), P(zero),
                              P(zero), P(np.ascontiguousarray(mesh.S0)), P(np.ascontiguousarray(mesh.z)),
                              C.c_double(0.5 * DRY_LIMIT), C.c_double(9.81), P(cf))
    m = oracle.Model(x=mesh.x, y=mesh.y, z=mesh.z, U=mesh.U0, V=mesh.V0, S=mesh.S0, dUdt=zero, dVdt=zero,
                     dSdt=zero, cf=cf, cfw=zero, uu=zero, uv=zero, vv=zero, rot=np.zeros((mesh.np, 4)),
                     niox=zero, nioy=zero, bcU=zero, bcS=zero, evt=evt, nflag=np.zeros(mesh.np, np.int32),
                     bckind=np.zeros(mesh.np, np.int32), eqno=eqno, enodes=els, ennd=nnd,
                     eflag=np.zeros(len(els), np.int32), g=9.81, hmin=0.5 * DRY_LIMIT,
                     vk=1.78e-6 / (1.0 + 0.0337 * 10.0 + 0.00022 * 100.0),
                     relaxThdt_UV=1.0 / wl["dt"], relaxThdt_H=1.0 / wl["dt"])
    return {"model": m, "mesh": mesh, "ptr": ptr, "idx": idx, "neq": neq, "nnz": int(ptr[-1]),
            "wet_triangles": int(len(els)), "pattern_s": t1 - t0}


def newton_parts(sysd) -> dict:
    """One Newton iteration's fixed parts with the reference's arithmetic: assembly (FP32
    matrix, FP64 residual), ScaleL2Norm, ILU(0) factorisation."""
    import oracle
    t0 = time.perf_counter()
    A, B = oracle.assemble(sysd["model"], sysd["ptr"], sysd["idx"], np.float32)
    t1 = time.perf_counter()
    oracle.scale_l2(sysd["ptr"], A, B)
    t2 = time.perf_counter()
    _rc, ILU = oracle.ilu0_factor(sysd["ptr"], sysd["idx"], A)
    t3 = time.perf_counter()
    sysd.update(A=A, B=B, ILU=ILU)
    return {"assemble_s": t1 - t0, "scale_s": t2 - t1, "factor_s": t3 - t2}


def krylov_iteration(sysd) -> float:
    """Seconds of one BiCGStab iteration (two ILU(0) applies, two SpMV, vector updates)."""
    import oracle
    t0 = time.perf_counter()
    oracle.bicgstab(sysd["ptr"], sysd["idx"], sysd["A"], sysd["ILU"], sysd["B"], 1, 1e-30)
    return time.perf_counter() - t0


def host_cpu() -> str:
    """The host's CPU model (x86 `model name`; on Arm the implementer/part codes), and the
    machine type: the reference arm runs on one of its cores."""
    import platform
    info = {}
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if ":" in line:
                    k, v = (t.strip() for t in line.split(":", 1))
                    info.setdefault(k, v)
    except OSError:
        pass
    if "model name" in info:
        return f"{info['model name']} ({platform.machine()})"
    if "CPU part" in info:
        return f"{platform.machine()} CPU implementer {info.get('CPU implementer', '?')} part {info['CPU part']}"
    return platform.machine()


def estimate(parts: dict, t_kry: float, counts: dict) -> float:
    fixed = parts["assemble_s"] + parts["scale_s"] + parts["factor_s"]
    return counts["newton_per_step"] * fixed + counts["krylov_per_step"] * t_kry


def _sample_text(workload, sysd, parts, t_kry, nk, counts):
    return (f"oracle C restatement of the reference's arithmetic, 1 host core (the reference is serial): the "
            f"{workload} workload's initial wet model (neq={sysd['neq']}, nnz={sysd['nnz']}): assembly "
            f"{parts['assemble_s']:.2f} s + ScaleL2Norm {parts['scale_s']:.2f} s + ILU(0) factor "
            f"{parts['factor_s']:.2f} s per Newton iteration, {t_kry:.3f} s per BiCGStab iteration (mean of {nk}); "
            f"scaled by the compiled reference's own {counts['newton_per_step']:.1f} Newton and "
            f"{counts['krylov_per_step']:.0f} BiCGStab iterations per step to 1e-8 ({counts['fixture']})")


def cpu_baseline(workload: str, wl, budget_s: float) -> dict:
    counts = reference_counts(workload)
    if counts is None:
        return {"unavailable": f"no recorded reference run for {workload}"}
    sysd = build_system(wl)
    parts = newton_parts(sysd)
    ts = []
    t0 = time.perf_counter()
    while not ts or (time.perf_counter() - t0 < budget_s and len(ts) < 50):
        ts.append(krylov_iteration(sysd))
    t_kry = float(np.mean(ts))
    value = estimate(parts, t_kry, counts)
    return {"value": round(value, 3), "unit": "s/step", "cores": 1, "kind": "port", "host_cpu": host_cpu(),
            "sample": _sample_text(workload, sysd, parts, t_kry, len(ts), counts)}


def bench_line(workload: str, wl, steps: int, warmup: int, metric: str) -> dict:
    """The `--impl reference` line: each of the `steps` timed samples is one BiCGStab
    iteration of the reference's solver on the workload's system (the assembly,
    scaling and factorisation are timed once, in the warm-up); value = the time step
    those samples imply with the reference's own iteration counts."""
    counts = reference_counts(workload)
    if counts is None:
        return {"impl": "reference", "unavailable": f"no recorded reference run for {workload}"}
    sysd = build_system(wl)
    parts = newton_parts(sysd)
    for _ in range(max(0, warmup - 1)):
        krylov_iteration(sysd)
    t0 = time.perf_counter()
    ts = [krylov_iteration(sysd) for _ in range(steps)]
    wall = time.perf_counter() - t0
    t_kry = float(np.mean(ts))
    value = round(estimate(parts, t_kry, counts), 3)
    text = _sample_text(workload, sysd, parts, t_kry, len(ts), counts)
    return {"impl": "reference", "metric": metric, "value": value, "unit": "s/step", "steps": steps,
            "warmup": warmup, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 matrix / f64 vectors", "data": "synthetic",
            "config": {"workload": wl["desc"], "workload_name": workload, "parallelism": "replicas only"},
            "timed_region_s": round(wall, 3),
            "reference_counts": counts,
            "cpu_baseline": {"value": value, "unit": "s/step", "cores": 1, "kind": "port", "host_cpu": host_cpu(),
                             "sample": text},
            "e2e": {"value": value, "unit": "s/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
