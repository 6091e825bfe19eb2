#!/usr/bin/env python3
"""Seconds per shallow-water time step on one GB300, Newton iterated to 1e-8.

Workload (synthetic, seeded): the meander valley of rismo2d_gb300.meshgen --
10 km sinusoidal main channel (wavelength 400 m, amplitude 80 m, 60 m wide,
4 m deep) between 200 m flood plains, log-normal Strickler roughness (median
20, sigma 0.3, 16 bands), 200,028 six-node triangles / 402,747 nodes, constant
eddy viscosity 0.5 m^2/s.  Unsteady, dt = 10 s, theta = 1, inflow hydrograph
Q(t) = 300 + 500 sin^2(pi t / 7200) m^3/s, outlet level fixed, dry/rewet
method 2 every 10 Newton iterations.  Every time step runs Newton until the
scaled residual ||B_k|| / ||B_0|| <= 1e-8.

A "step" is one such time step.  Default arm (the headline): the
mixed-precision solver (FP32 Krylov / SpMV / ILU(0) inside FP64 iterative
refinement, FP64 residual and update) started from the learned warm start,
as an inexact Newton iteration (BiCGStab to relative residual 0.5, ILU(0)
factors reused for up to 64 Newton iterations); the Newton convergence test
is the same ||B_k|| / ||B_0|| <= 1e-8.
The network is trained on the GPU, before the timed region, on a trajectory
of the plain mixed solver under a different hydrograph (Q(t) = 250 + 700
sin^2(pi t / 5400), 12 steps from rest); the timed steps are held out.  Each
timed step includes the prediction (features + forward pass, host copies in
and out).  The same time steps also run cold-started (mixed, same Newton-
Krylov options, no warm start), cold with the reference's linear solves, and
with the plain FP64 GPU path (the reference's algorithm) for comparison; the
CPU restatement of the
reference's solver is timed on a bounded sample on the host cores.
`--impl reference` times that CPU solver alone.  One JSON line on stdout.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

STEP_DT = 10.0
RESIDUAL_TOL = 1.0e-8
METRIC = "s per time step at 1e-8 Newton residual: mixed+learned vs plain FP64, 1 GB300"
WORKLOAD = ("meander 10 km x 601 m, 200,028 P2 triangles (402,747 nodes), unsteady dt=10 s, "
            "Q(t)=300+500 sin^2(pi t/7200), dry/rewet on, Newton to ||B||/||B0||<=1e-8")
# training trajectory of the warm-start network: another hydrograph, from rest
TRAIN_HYDROGRAPH = dict(Q0=250.0, dQ=700.0, period=5400.0, t_end=7200.0)
TRAIN_STEPS = 12
# Newton-Krylov options of the mixed arms (the FP64 arm runs the reference's
# linear solves: ILU(0) factored and BiCGStab to maxDiff in every iteration)
LINEAR_FORCING = 0.5
ILU_REUSE = 64
TRAIN_EPOCHS = 30
TRAIN_BATCH = 8192
PEAKS_FILE = os.path.join(REPO, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0

# Newton and Krylov iterations per time step of the plain FP64 GPU path on this
# workload's first timed steps (time steps 4 and 5, after 3 warm-up steps;
# measured on GB300: 33 / 801 per step); used only to scale the CPU solver's
# per-iteration time when the FP64 arm does not run in the same process.
FP64_NEWTON_PER_STEP = 33.0
FP64_KRYLOV_PER_STEP = 801.0

# DRAM bytes (read + write) of one k_trsv_wave<float, LOWER> launch on this
# workload, from the ncu capture summarised in
# profiles/k_trsv_wave_meander200k.txt (cold L2, kernel replay)
NCU_TRSV_TRAFFIC_BYTES = 14.733312e6


def workload():
    from rismo2d_gb300 import meshgen
    from rismo2d_gb300.sim import Params
    mesh = meshgen.meander()
    hyd = meshgen.sin2_hydrograph()
    return mesh, hyd, Params()


# ---- distributed setup: replicas only (the ILU(0) chain does not shard) ----

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Dist:
    def __init__(self, backend: str):
        self.world, self.rank, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        dev = f"cuda:{self.local}" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---- clocks sampled during the timed region ---------------------------------

class Clocks:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, local_rank: int):
        self.proc = None
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        ids = [v for v in vis.split(",") if v.strip()]
        self.index = ids[local_rank] if local_rank < len(ids) else str(local_rank)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.index, f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out = self.proc.communicate(timeout=10)[0]
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out = self.proc.communicate()[0]
        sm, smax, reasons = [], [], set()
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for name, v in zip(self.NAMES, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- GPU arm ------------------------------------------------------------------

def l2_flush(buf):
    import torch
    buf.zero_()
    torch.cuda.synchronize()


def train_net(device: int, max_newton: int = 0):
    """The warm-start network of the workload's mesh, trained on the GPU on the plain mixed
    solver's trajectory under the training hydrograph (not the timed one)."""
    from rismo2d_gb300 import _lib, meshgen
    from rismo2d_gb300 import warmstart as ws
    from rismo2d_gb300.sim import Simulation, RG_CRIT_RESIDUAL
    mesh, _hyd, params = workload()
    hyd = meshgen.sin2_hydrograph(**TRAIN_HYDROGRAPH)
    t0 = time.perf_counter()
    sim = Simulation(mesh, params, hydrograph=hyd, precision=_lib.PREC_MIXED, device=device)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    states, times, reps = ws.collect_trajectory(sim, hyd, 0.0, STEP_DT, TRAIN_STEPS, criterion=RG_CRIT_RESIDUAL,
                                                residual_tol=RESIDUAL_TOL, max_newton=max_newton)
    sim.close()
    t1 = time.perf_counter()
    net = ws.WarmStartNet(mesh, device=device, seed=7)
    net.set_scales((4.0, 1.0, 1.0), *ws.trajectory_scales(states))
    nsamp = ws.add_trajectory(net, states, times, hyd, STEP_DT)
    losses = net.train(epochs=TRAIN_EPOCHS, batch=TRAIN_BATCH, lr=1e-3, seed=3)
    t2 = time.perf_counter()
    info = {"hydrograph": "Q(t)=250+700 sin^2(pi t/5400) from rest (held out from the timed steps)",
            "trajectory_steps": TRAIN_STEPS, "samples": int(nsamp), "epochs": TRAIN_EPOCHS, "batch": TRAIN_BATCH,
            "loss_first_last": [round(float(losses[0]), 4), round(float(losses[-1]), 4)],
            "trajectory_s": round(t1 - t0, 2), "train_s": round(t2 - t1, 2),
            "converged": all(r["converged"] for r in reps)}
    return net, info


def run_gpu(prec: int, warmup: int, steps: int, device: int, profile: bool, clocks: Clocks | None, dist: Dist,
            flush_buf, max_newton: int = 0, net=None, linear_forcing: float = 0.0, ilu_reuse: int = 0):
    """W warm-up and K timed time steps through Simulation.step; per-step device time by
    CUDA events on the library's stream, host wall time of step + state download.  With
    `net`, every step after the first starts from the network's prediction; the
    prediction's wall time (its kernels on the network's stream, copies in and out)
    is added to the step's device time."""
    import torch
    from rismo2d_gb300 import warmstart as ws
    from rismo2d_gb300.sim import Simulation, RG_CRIT_RESIDUAL
    mesh, hyd, params = workload()
    sim = Simulation(mesh, params, hydrograph=hyd, precision=prec, device=device)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    t = 0.0
    reps = []
    hist = [sim.get_state()] if net else []

    def predict():
        if net is None or len(hist) < 2:
            return 0.0, 0, 0
        p0 = time.perf_counter()
        sim.set_warm_start(*ws.predict_next(net, hist[-2], hist[-1], t, hyd, STEP_DT))
        nwet = int(np.count_nonzero(ws.wet(hist[-1])))
        # network copies: 6 state arrays + node list in, 4 floats per wet node out
        return (time.perf_counter() - p0) * 1e3, 6 * 8 * mesh.np + 4 * nwet, 16 * nwet

    kw = dict(criterion=RG_CRIT_RESIDUAL, residual_tol=RESIDUAL_TOL, max_newton=max_newton,
              linear_forcing=linear_forcing, ilu_reuse=ilu_reuse)
    for _ in range(warmup):
        predict()
        reps.append(sim.step(t, STEP_DT, **kw))
        t += STEP_DT
        if net:
            hist = [hist[-1], sim.get_state()]
    st0 = sim.stats()
    sim.stage_ms(reset=True)
    if profile:
        sim.profile(True, reset=True)
    dev_ms, e2e_ms, timed = [], [], []
    pred_h2d = pred_d2h = 0
    states = []
    dist.barrier()
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    if profile:
        torch.cuda.profiler.start()          # profiler range = the timed steps (no-op without a profiler)
    wall0 = time.perf_counter()
    for _ in range(steps):
        l2_flush(flush_buf)
        h0 = time.perf_counter()
        pred_ms, bi, bo = predict()
        pred_h2d += bi
        pred_d2h += bo
        sim.event_record(0)
        rep = sim.step(t, STEP_DT, **kw)
        sim.event_record(1)
        state = sim.get_state()               # result to host memory (numpy)
        h1 = time.perf_counter()
        if net:
            hist = [hist[-1], state]
        dev_ms.append(sim.event_elapsed(0, 1) + pred_ms)
        e2e_ms.append((h1 - h0) * 1e3)
        timed.append(rep)
        states.append({k: state[k] for k in ("U", "V", "S", "flag")})
        t += STEP_DT
    torch.cuda.synchronize()
    if profile:
        torch.cuda.profiler.stop()
    dist.barrier()
    wall1 = time.perf_counter()
    clk = clocks.stop() if clocks else None
    st1 = sim.stats()
    stage = {k: round(v / steps, 2) for k, v in sim.stage_ms().items()}
    prof = sim.profile_read() if profile else None
    if profile:
        sim.profile(False)
    # the network's launches per prediction: features + forward
    mod = sim.model()
    wet_tri = int(np.count_nonzero(np.asarray(mod["elem_nnd"]) == 6))
    wet_nodes = int(np.count_nonzero((states[-1]["flag"] & 64) == 0)) if states else 0
    out = dict(dev_ms=dev_ms, e2e_ms=e2e_ms, wall_s=wall1 - wall0, reps=timed, warm_reps=reps, states=states,
               wet_tri=wet_tri, wet_nodes=wet_nodes,
               stats=st1.tolist(), h2d=int(st1[12] - st0[12]) + pred_h2d, d2h=int(st1[13] - st0[13]) + pred_d2h,
               launches=int(st1[14] - st0[14]) + (2 * steps if net else 0), prof=prof, clocks=clk, stage=stage)
    sim.close()
    return out


# ---- CPU solver (oracle restatement of the reference) on a bounded sample -----

def cpu_newton_system():
    """The first Newton system of the workload, built on the host: the host model's
    numbering/boundary set-up and the oracle's friction and element assembly."""
    import ctypes as C
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from rismo2d_gb300.sim import Simulation, RG_DEVICE_NONE
    mesh, hyd, params = workload()
    sim = Simulation(mesh, params, hydrograph=hyd, device=RG_DEVICE_NONE)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    sim.dry_rewet_pass()
    s0 = sim.get_state()
    # nodal friction of the current state (oracle restatement of MODEL::DoFriction)
    en = np.ascontiguousarray(mesh.elems, np.int32)
    mats = {no: n for no, n, _vt in mesh.materials}
    elem_n = np.ascontiguousarray([mats[int(t)] for t in mesh.elem_type], np.float64)
    zor = mesh.z.copy()
    mid = en[:, 3:6]
    cor = en[:, :3]
    for k, (a, b) in enumerate(((0, 1), (1, 2), (2, 0))):
        zor[mid[:, k]] = 0.5 * (mesh.z[cor[:, a]] + mesh.z[cor[:, b]])
    x0, y0, z0 = mesh.x[cor[:, 0]], mesh.y[cor[:, 0]], zor[cor[:, 0]]
    xx = [mesh.x[cor[:, i]] - x0 for i in (1, 2)]
    yy = [mesh.y[cor[:, i]] - y0 for i in (1, 2)]
    zz = [zor[cor[:, i]] - z0 for i in (1, 2)]
    t1 = yy[0] * zz[1] - yy[1] * zz[0]
    t2 = zz[0] * xx[1] - zz[1] * xx[0]
    t3 = xx[0] * yy[1] - xx[1] * yy[0]
    af = np.ascontiguousarray(np.sqrt(t1 * t1 + t2 * t2 + t3 * t3) / t3)
    cf = np.zeros(mesh.np)
    nnd = np.full(len(en), 6, np.int32)
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    oracle.lib().orc_friction(C.c_int(mesh.np), C.c_int(len(en)), P(en), P(nnd), P(elem_n), P(af), P(s0["U"]),
                              P(s0["V"]), P(s0["S"]), P(s0["z"]), C.c_double(0.5 * params.dry_limit),
                              C.c_double(params.g), P(cf))
    sim.prepare_iteration(STEP_DT, cf)
    st = sim.get_state()
    num = sim.numbering()
    bnd = sim.boundary()
    mod = sim.model()
    z0v = np.zeros(mesh.np)
    m = oracle.Model(x=mesh.x, y=mesh.y, z=st["z"], U=st["U"], V=st["V"], S=st["S"], dUdt=z0v, dVdt=z0v,
                     dSdt=z0v, cf=cf, cfw=z0v, uu=z0v, uv=z0v, vv=z0v, rot=bnd["rot4"], niox=mod["niox"],
                     nioy=mod["nioy"], bcU=bnd["bcU"], bcS=bnd["bcS"], evt=mod["elem_vt"], nflag=bnd["nflag"],
                     bckind=bnd["bckind"], eqno=num["eqno"], enodes=mod["elem_nodes"], ennd=mod["elem_nnd"],
                     eflag=mod["elem_flag"], g=params.g, hmin=0.5 * params.dry_limit, vk=params.vk,
                     relaxThdt_UV=1.0 / STEP_DT / params.theta, relaxThdt_H=1.0 / STEP_DT / params.theta)
    n = num["neq"]
    ptr = np.zeros(n + 1, np.int64)
    ptr[1:] = np.cumsum(num["width"])
    index = np.ascontiguousarray(num["index"], np.int32)
    t0 = time.perf_counter()
    A, B = oracle.assemble(m, ptr, index, np.float32)
    t_asm = time.perf_counter() - t0
    sim.close()
    return dict(ptr=ptr, index=index, A=A, B=B, neq=n, nnz=len(index), t_assemble=t_asm)


def cpu_newton_once(sysd):
    """One Newton iteration's linear algebra with the reference's arithmetic (float
    matrix and ILU(0), double vectors): ScaleL2Norm, ILU(0) factor, BiCGStab to 1e-8."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    A = sysd["A"].copy()
    B = sysd["B"].copy()
    t0 = time.perf_counter()
    oracle.scale_l2(sysd["ptr"], A, B)
    rc, ILU = oracle.ilu0_factor(sysd["ptr"], sysd["index"], A)
    t1 = time.perf_counter()
    ok, X, its, acc = oracle.bicgstab(sysd["ptr"], sysd["index"], A, ILU, B, 1000, RESIDUAL_TOL)
    t2 = time.perf_counter()
    return dict(t_factor=t1 - t0, t_krylov=t2 - t1, its=its, ok=bool(ok))


def cpu_estimate(samples, sysd, newton_per_step, krylov_per_step):
    t_fac = statistics.mean(s["t_factor"] for s in samples) + sysd["t_assemble"]
    per_kry = sum(s["t_krylov"] for s in samples) / max(1, sum(s["its"] for s in samples))
    return newton_per_step * t_fac + krylov_per_step * per_kry, t_fac, per_kry


def cpu_baseline(budget_s: float, newton_per_step: float, krylov_per_step: float):
    sysd = cpu_newton_system()
    samples = []
    t0 = time.perf_counter()
    while not samples or (time.perf_counter() - t0 < budget_s and len(samples) < 20):
        samples.append(cpu_newton_once(sysd))
    value, t_fac, per_kry = cpu_estimate(samples, sysd, newton_per_step, krylov_per_step)
    its = [s["its"] for s in samples]
    return {"value": round(value, 3), "unit": "s/step", "cores": 1, "kind": "port",
            "sample": (f"oracle C restatement (1 host core): element assembly + ScaleL2Norm + ILU(0) factor + "
                       f"BiCGStab(1e-8) of the workload's first Newton system (neq={sysd['neq']}, "
                       f"nnz={sysd['nnz']}), {len(samples)} solve(s) of {its[0]} Krylov its; scaled to a time "
                       f"step by {newton_per_step:.1f} Newton and {krylov_per_step:.1f} Krylov iterations "
                       f"per step: {t_fac:.3f} s per Newton + {per_kry * 1e3:.2f} ms per Krylov iteration")}


# ---- roofline of the dominant kernel ---------------------------------------------

def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def trsv_roofline(prof, neq: int, nnz: int, w: int, wx: int):
    """ILU(0) apply (L and U launches): z(w+4) + 4(n+1) + 3 n wx algorithmic bytes per apply."""
    launches, ms = prof["trsv"]
    if launches == 0 or ms <= 0:
        return None
    apply_bytes = nnz * (w + 4) + 4 * (neq + 1) + 3 * neq * wx
    per_launch = apply_bytes / 2.0
    avg_s = ms / launches / 1e3
    achieved = per_launch / avg_s / 1e9
    peak, kind = hbm_peak()
    return {"bound": "hbm", "kernel": "k_trsv_wave<float> (ILU(0) L and U solves)", "achieved": round(achieved, 2),
            "peak": peak, "peak_kind": kind, "unit": "GB/s", "frac": round(achieved / peak, 5),
            "traffic": NCU_TRSV_TRAFFIC_BYTES, "algorithmic_bytes_per_launch": per_launch,
            "launches": launches, "avg_launch_ms": round(ms / launches, 4),
            "share_of_step_device_time": None}


def class_rooflines(prof, neq: int, nnz: int, tri: int, nodes: int, w: int = 4, wx: int = 4):
    """Achieved bandwidth of every profiled kernel class from the live event timing, with the
    algorithmic bytes per launch of its formula: SpMV z(w+4) + 4(n+1) + 2n wx; ILU(0) apply
    z(w+4) + 4(n+1) + 3n wx per L+U pair; factor 2zw + 4z + 4(n+1); assembly zw + 8n + 120N
    + 24T + 900T (T wet triangles, N wet nodes).  The refinement residual's SpMV reads FP64
    vectors, so the SpMV class figure is a lower bound."""
    peak, kind = hbm_peak()
    per_launch = {"spmv": nnz * (w + 4) + 4 * (neq + 1) + 2 * neq * wx,
                  "trsv": (nnz * (w + 4) + 4 * (neq + 1) + 3 * neq * wx) / 2.0,
                  "factor": 2 * nnz * w + 4 * nnz + 4 * (neq + 1),
                  "assemble": nnz * w + 8 * neq + 120 * nodes + 24 * tri + 900 * tri}
    out = {}
    for cls, (launches, ms) in prof.items():
        if cls not in per_launch or launches == 0 or ms <= 0:
            continue
        gbs = per_launch[cls] * launches / (ms / 1e3) / 1e9
        out[cls] = {"launches": launches, "avg_launch_ms": round(ms / launches, 4),
                    "algorithmic_bytes_per_launch": int(per_launch[cls]), "achieved_gbs": round(gbs, 2),
                    "frac": round(gbs / peak, 5)}
    return {"peak_gbs": peak, "peak_kind": kind, "classes": out}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--fp64-steps", type=int, default=2, help="timed steps of the plain FP64 comparison (0: skip)")
    ap.add_argument("--cold-steps", type=int, default=5,
                    help="timed steps of the mixed solver without warm start (0: skip)")
    ap.add_argument("--exact-steps", type=int, default=2,
                    help="timed steps of the mixed solver, cold, with the reference's linear solves: every Newton "
                         "iteration factors ILU(0) and solves to maxDiff (0: skip)")
    ap.add_argument("--linear-forcing", type=float, default=LINEAR_FORCING,
                    help="inexact Newton: BiCGStab to max(maxDiff, this) relative residual (0: maxDiff)")
    ap.add_argument("--ilu-reuse", type=int, default=ILU_REUSE,
                    help="Newton iterations an ILU(0) factorisation is reused for (0: factor every iteration)")
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU solver sampling (0: skip)")
    ap.add_argument("--max-newton", type=int, default=0,
                    help="cap on Newton iterations per step, for short profiling runs only (0: none; a capped "
                         "run is not a benchmark result)")
    args = ap.parse_args()
    warmup = max(3, args.warmup)

    if args.impl == "reference":
        world, rank, _local = dist_env()
        if rank != 0:
            return 0
        sysd = cpu_newton_system()
        samples = []
        for _ in range(warmup):
            cpu_newton_once(sysd)
        for _ in range(args.steps):
            samples.append(cpu_newton_once(sysd))
        value, t_fac, per_kry = cpu_estimate(samples, sysd, FP64_NEWTON_PER_STEP, FP64_KRYLOV_PER_STEP)
        line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "s/step",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": warmup, "higher_is_better": False,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 matrix / f64 vectors", "data": "synthetic",
                "config": {"workload": WORKLOAD, "parallelism": "replicas only"},
                "cpu_baseline": {"value": round(value, 3), "unit": "s/step", "cores": 1, "kind": "port",
                                 "sample": (f"each step: one Newton iteration's element assembly + ScaleL2Norm + "
                                            f"ILU(0) + BiCGStab(1e-8) of the first Newton system (neq="
                                            f"{sysd['neq']}), scaled by {FP64_NEWTON_PER_STEP} Newton / "
                                            f"{FP64_KRYLOV_PER_STEP} Krylov iterations per time step")},
                "e2e": {"value": round(value, 3), "unit": "s/step", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0

    import torch
    dist = Dist("nccl")
    device = dist.local
    torch.cuda.set_device(device)
    flush_buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{device}")   # 256 MiB > L2
    from rismo2d_gb300 import _lib
    clocks = Clocks(device)
    net, learned_info = train_net(device, args.max_newton)
    solver_kw = dict(linear_forcing=args.linear_forcing, ilu_reuse=args.ilu_reuse)
    mixed = run_gpu(_lib.PREC_MIXED, warmup, args.steps, device, True, clocks, dist, flush_buf, args.max_newton,
                    net=net, **solver_kw)
    net.close()
    k = args.steps
    dev_s = sum(mixed["dev_ms"]) / 1e3
    dev_s_max = dist.max(dev_s)
    value = dev_s_max / (k * dist.world)                         # whole-job seconds per time step
    e2e_s = dist.max(sum(mixed["e2e_ms"]) / 1e3) / (k * dist.world)
    newton = [r["newton_iterations"] for r in mixed["reps"]]
    krylov = [r["krylov_iterations"] for r in mixed["reps"]]
    conv = all(r["converged"] for r in mixed["reps"])

    def rel_errs(sa, sb):
        errs = []
        for a, b in zip(sa, sb):
            wet = (b["flag"] & 64) == 0               # NODE::kDry
            rel = {v: float(np.max(np.abs(a[v][wet] - b[v][wet])) / max(1e-30, np.max(np.abs(b[v][wet]))))
                   for v in ("U", "V", "S")}
            rel["flags_identical"] = bool(np.array_equal(a["flag"], b["flag"]))
            errs.append(rel)
        return errs

    cold = None
    if args.cold_steps > 0:
        kc = min(args.cold_steps, k)
        c = run_gpu(_lib.PREC_MIXED, warmup, kc, device, False, None, dist, flush_buf, args.max_newton, **solver_kw)
        cs = sum(c["dev_ms"]) / 1e3 / kc
        cold = {"s_per_step": round(cs, 4), "steps": kc,
                "newton_per_step": statistics.mean(r["newton_iterations"] for r in c["reps"]),
                "krylov_per_step": statistics.mean(r["krylov_iterations"] for r in c["reps"]),
                "converged": all(r["converged"] for r in c["reps"]),
                "learned_speedup": round(cs / (sum(mixed["dev_ms"][:kc]) / 1e3 / kc), 3),
                "learned_vs_cold_max_rel_err": rel_errs(mixed["states"][:kc], c["states"])}
    exact = None
    if args.exact_steps > 0:
        ke = min(args.exact_steps, k)
        x = run_gpu(_lib.PREC_MIXED, warmup, ke, device, False, None, dist, flush_buf, args.max_newton)
        exact = {"s_per_step": round(sum(x["dev_ms"]) / 1e3 / ke, 4), "steps": ke,
                 "newton_per_step": statistics.mean(r["newton_iterations"] for r in x["reps"]),
                 "krylov_per_step": statistics.mean(r["krylov_iterations"] for r in x["reps"]),
                 "converged": all(r["converged"] for r in x["reps"]),
                 "host_stage_ms_per_step": x["stage"]}
    fp64 = None
    if args.fp64_steps > 0:
        kf = min(args.fp64_steps, k)
        f = run_gpu(_lib.PREC_FP64, warmup, kf, device, False, None, dist, flush_buf, args.max_newton)
        fs = sum(f["dev_ms"]) / 1e3 / kf
        errs = rel_errs(mixed["states"][:kf], f["states"])
        fp64 = {"s_per_step": round(fs, 4), "steps": kf,
                "newton_per_step": statistics.mean(r["newton_iterations"] for r in f["reps"]),
                "krylov_per_step": statistics.mean(r["krylov_iterations"] for r in f["reps"]),
                "converged": all(r["converged"] for r in f["reps"]),
                "learned_mixed_speedup": round(fs / (sum(mixed["dev_ms"][:kf]) / 1e3 / kf), 3),
                "learned_mixed_vs_fp64_max_rel_err": errs}
    cpu = None
    if dist.rank == 0 and args.cpu_budget > 0:
        nps = fp64["newton_per_step"] if fp64 else statistics.mean(newton)
        kps = fp64["krylov_per_step"] if fp64 else statistics.mean(krylov)
        cpu = cpu_baseline(args.cpu_budget, nps, kps)
    # roofline of the dominant kernel (ILU(0) triangular solves) from the live event timing
    st = mixed["stats"]
    roof = trsv_roofline(mixed["prof"], int(st[0]), int(st[1]), 4, 4)
    if roof:
        roof["share_of_step_device_time"] = round(mixed["prof"]["trsv"][1] / sum(mixed["dev_ms"]), 4)
    if dist.rank == 0:
        line = {"metric": METRIC, "value": round(value, 4), "unit": "s/step", "n_gpus": dist.world, "steps": k,
                "warmup": warmup, "ms_per_step": round(1e3 * dev_s_max / k, 2), "higher_is_better": False,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 Krylov/ILU(0) + f64 refinement",
                "data": "synthetic (seeded meander mesh, no external dataset)",
                "config": {"workload": WORKLOAD, "solver": "mixed: FP32 BiCGStab/ILU(0)/SpMV in FP64 iterative "
                           "refinement, started from the learned warm start (prediction inside each timed step); "
                           f"inexact Newton: BiCGStab to relative residual {args.linear_forcing:g}; ILU(0) factors "
                           f"reused for up to {args.ilu_reuse} Newton iterations; the Newton test stays "
                           "||B_k||/||B_0|| <= 1e-8",
                           "precision_arm": "mixed+learned",
                           "linear_forcing": args.linear_forcing, "ilu_reuse": args.ilu_reuse,
                           "parallelism": "replicas only" if dist.world > 1 else "1 GPU",
                           "l2": "256 MiB buffer written between timed steps (the ~60 MB system stays "
                                 "L2-resident within a step)",
                           "neq": int(st[0]), "nnz": int(st[1])},
                "newton_per_step": statistics.mean(newton), "krylov_per_step": statistics.mean(krylov),
                "converged": conv, "warm_start_accepted": sum(r["warm_start"] for r in mixed["reps"]),
                "learned": learned_info, "cold_start": cold, "mixed_reference_solves": exact, "fp64": fp64,
                "host_stage_ms_per_step": mixed["stage"],
                "clocks": mixed["clocks"],
                "e2e": {"value": round(e2e_s, 4), "unit": "s/step",
                        "h2d_bytes_per_step": mixed["h2d"] // k, "d2h_bytes_per_step": mixed["d2h"] // k,
                        "api": "Simulation.step + get_state (host numpy state out)"},
                "gpu_launches": mixed["launches"],
                "device_ms_by_kernel_class": {kk: [v[0], round(v[1], 2)] for kk, v in mixed["prof"].items()},
                "roofline": roof,
                "roofline_by_kernel_class": class_rooflines(mixed["prof"], int(st[0]), int(st[1]), mixed["wet_tri"],
                                                            mixed["wet_nodes"]),
                "cpu_baseline": cpu}
        if args.max_newton:
            line["profiling_case"] = f"Newton capped at {args.max_newton} per step: not a benchmark result"
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
