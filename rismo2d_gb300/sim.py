"""Python front end of the standalone time stepper (include/rg300_sim.h).

`Simulation` mirrors the reference's run of EQS_UVS2D::Execute per time step
(EqsUVS2D.cpp:71): construct it from a mesh (rismo2d_gb300.meshgen.Mesh or the
same arrays read from reference decks), set the initial state, call `step`.
All numerical work happens in librg300.so; this module only marshals arrays.
"""

from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np

from . import _lib
from ._lib import p

RG_BC_QINLET, RG_BC_QTINLET, RG_BC_OUTLET = 1, 2, 3
RG_CRIT_CORRECTION, RG_CRIT_RESIDUAL = 0, 1
RG_DEVICE_NONE = -2


class LineBc(C.Structure):
    _fields_ = [("kind", C.c_int), ("line", C.c_int), ("npts", C.c_int), ("t", C.c_void_p),
                ("Q", C.c_void_p), ("S", C.c_void_p)]


class DeckParams(C.Structure):
    _fields_ = [("g", C.c_double), ("vk", C.c_double), ("dry_limit", C.c_double), ("rewet_limit", C.c_double),
                ("dryrew_method", C.c_int), ("dryrew_freq", C.c_int), ("countdown", C.c_int),
                ("relax_method", C.c_int), ("max_delta_uv", C.c_double), ("max_delta_s", C.c_double),
                ("max_us", C.c_double), ("conv_uv", C.c_double), ("conv_s", C.c_double), ("max_newton", C.c_int),
                ("solver_maxiter", C.c_int), ("solver_maxdiff", C.c_double), ("theta", C.c_double)]


class Deck(C.Structure):
    _fields_ = [("np", C.c_int), ("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p), ("ne", C.c_int),
                ("elem_nodes", C.c_void_p), ("elem_mat", C.c_void_p), ("nmat", C.c_int), ("mat_n", C.c_void_p),
                ("mat_vt", C.c_void_p), ("nseg", C.c_int), ("seg_nodes", C.c_void_p), ("seg_line", C.c_void_p),
                ("nbc", C.c_int), ("bc", C.c_void_p), ("params", DeckParams)]


class StepCtl(C.Structure):
    _fields_ = [("steady", C.c_int), ("first_step", C.c_int), ("criterion", C.c_int),
                ("residual_tol", C.c_double), ("max_newton", C.c_int), ("linear_forcing", C.c_double),
                ("ilu_reuse", C.c_int), ("friction_jacobian", C.c_int)]


class StepReport(C.Structure):
    _fields_ = [("newton_iterations", C.c_int), ("krylov_iterations", C.c_int), ("converged", C.c_int),
                ("neq", C.c_int), ("dryrew_events", C.c_int), ("dry_nodes", C.c_int), ("solver_status", C.c_int),
                ("n_hist", C.c_int), ("residual_first", C.c_double), ("residual_ratio", C.c_double),
                ("wall_ms", C.c_double), ("residual_hist", C.c_double * 64), ("warm_start", C.c_int),
                ("residual_warm", C.c_double)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "residual_hist"}
        d["residual_hist"] = [self.residual_hist[i] for i in range(self.n_hist)]
        return d


@dataclasses.dataclass
class Params:
    """Deck parameters; defaults are the $RELAX/$DRYREW/$SOLVER lines deck.write_deck writes."""
    g: float = 9.81
    vk: float = 1.78e-6 / (1.0 + 0.0337 * 10.0 + 0.00022 * 100.0)   # Project.cpp:110, 10 degC
    dry_limit: float = 0.01
    rewet_limit: float = 0.02
    dryrew_method: int = 2
    dryrew_freq: int = 10
    countdown: int = 5
    relax_method: int = 2
    max_delta_uv: float = 0.5
    max_delta_s: float = 0.5
    max_us: float = 100.0
    conv_uv: float = 1.0e-9
    conv_s: float = 1.0e-9
    max_newton: int = 60
    solver_maxiter: int = 1000
    solver_maxdiff: float = 1.0e-8
    theta: float = 1.0


class Simulation:
    """A mesh, its boundary conditions and the GPU state of one run."""

    def __init__(self, mesh, params: Params | None = None, hydrograph=None, precision: int = _lib.PREC_FP64,
                 device: int = 0, line_bcs=None):
        """``line_bcs`` (optional): [(kind, line, rows)] with kind "QINLET" (rows [(Q, S)]),
        "QTINLET" (rows [(t, Q, S)]) or "OUTLET" (rows [(S,)]) -- the $TM_LINE conditions
        of a deck (deck.read_deck).  Without it: the inlet on line 1 (QINLET with the
        mesh's Q, or QTINLET with ``hydrograph``) and the outlet level on line 2."""
        self.lib = _lib.load()
        self.lib.rg_sim_last_error.restype = C.c_char_p
        self.params = params or Params()
        self.mesh = mesh
        m = mesh
        mats = sorted(m.materials)
        mat_index = {no: i for i, (no, _n, _vt) in enumerate(mats)}
        self._arr = dict(
            x=np.ascontiguousarray(m.x, np.float64), y=np.ascontiguousarray(m.y, np.float64),
            z=np.ascontiguousarray(m.z, np.float64),
            en=np.ascontiguousarray(m.elems, np.int32).reshape(-1),
            emat=np.ascontiguousarray([mat_index[int(t)] for t in m.elem_type], np.int32),
            mat_n=np.ascontiguousarray([n for _no, n, _vt in mats], np.float64),
            mat_vt=np.ascontiguousarray([vt for _no, _n, vt in mats], np.float64))
        segs, lines = [], []
        for no, seg in sorted(m.lines.items()):
            for s in seg:
                segs.append(s)
                lines.append(no)
        self._arr["segs"] = np.ascontiguousarray(np.asarray(segs, np.int32).reshape(-1))
        self._arr["lines"] = np.ascontiguousarray(lines, np.int32)
        bcs = []
        if line_bcs is not None:
            kinds = {"QINLET": RG_BC_QINLET, "QTINLET": RG_BC_QTINLET, "OUTLET": RG_BC_OUTLET}
            for i, (kind, line, rows) in enumerate(line_bcs):
                r = np.asarray(rows, np.float64).reshape(len(rows), -1)
                if kind == "QTINLET":
                    t, Q, S = r[:, 0], r[:, 1], r[:, 2]
                elif kind == "QINLET":
                    t, Q, S = np.zeros(1), r[:1, 0], r[:1, 1]
                else:
                    t, Q, S = np.zeros(1), np.zeros(1), r[:1, 0]
                for nm, arr in (("t", t), ("Q", Q), ("S", S)):
                    self._arr[f"bc{i}_{nm}"] = np.ascontiguousarray(arr, np.float64)
                a_ = self._arr
                bcs.append(LineBc(kinds[kind], int(line), len(a_[f"bc{i}_t"]), p(a_[f"bc{i}_t"]), p(a_[f"bc{i}_Q"]),
                                  p(a_[f"bc{i}_S"])))
        elif hydrograph is None:
            S_in = m.meta.get("S_in", m.meta["S_out"])
            self._arr["q_t"] = np.array([0.0])
            self._arr["q_Q"] = np.array([float(m.meta["Q"])])
            self._arr["q_S"] = np.array([float(S_in)])
            bcs.append(LineBc(RG_BC_QINLET, 1, 1, p(self._arr["q_t"]), p(self._arr["q_Q"]), p(self._arr["q_S"])))
        else:
            h = np.asarray(hydrograph, np.float64)
            self._arr["q_t"] = np.ascontiguousarray(h[:, 0])
            self._arr["q_Q"] = np.ascontiguousarray(h[:, 1])
            self._arr["q_S"] = np.ascontiguousarray(h[:, 2])
            bcs.append(LineBc(RG_BC_QTINLET, 1, len(h), p(self._arr["q_t"]), p(self._arr["q_Q"]),
                              p(self._arr["q_S"])))
        if line_bcs is None:
            self._arr["o_S"] = np.array([float(m.meta["S_out"])])
            bcs.append(LineBc(RG_BC_OUTLET, 2, 1, None, None, p(self._arr["o_S"])))
        self._bcs = (LineBc * len(bcs))(*bcs)
        pp = self.params
        dp = DeckParams(pp.g, pp.vk, pp.dry_limit, pp.rewet_limit, pp.dryrew_method, pp.dryrew_freq, pp.countdown,
                        pp.relax_method, pp.max_delta_uv, pp.max_delta_s, pp.max_us, pp.conv_uv, pp.conv_s,
                        pp.max_newton, pp.solver_maxiter, pp.solver_maxdiff, pp.theta)
        a = self._arr
        self._deck = Deck(len(a["x"]), p(a["x"]), p(a["y"]), p(a["z"]), len(a["emat"]), p(a["en"]), p(a["emat"]),
                          len(a["mat_n"]), p(a["mat_n"]), p(a["mat_vt"]), len(a["lines"]), p(a["segs"]),
                          p(a["lines"]), len(bcs), C.cast(self._bcs, C.c_void_p), dp)
        self.ptr = C.c_void_p()
        st = self.lib.rg_sim_create(C.byref(self._deck), C.c_int(precision), C.c_int(device), C.byref(self.ptr))
        if st != _lib.RG_OK:
            raise _lib.RgError(st, "rg_sim_create: " + self._err())
        self.np = len(a["x"])
        self.precision = precision
        self.step_no = 0

    def _err(self) -> str:
        if not self.ptr:
            return ""
        e = self.lib.rg_sim_last_error(self.ptr)
        return e.decode() if e else ""

    def close(self):
        if self.ptr:
            self.lib.rg_sim_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, U, V, S):
        U, V, S = (np.ascontiguousarray(v, np.float64) for v in (U, V, S))
        st = self.lib.rg_sim_set_state(self.ptr, p(U), p(V), p(S))
        if st != _lib.RG_OK:
            raise _lib.RgError(st, "rg_sim_set_state: " + self._err())
        self.step_no = 0

    def set_warm_start(self, U, V, S):
        """Starting state of the next step's Newton iteration (kept only if its residual is smaller)."""
        U, V, S = (np.ascontiguousarray(v, np.float64) for v in (U, V, S))
        st = self.lib.rg_sim_set_warm_start(self.ptr, p(U), p(V), p(S))
        if st != _lib.RG_OK:
            raise _lib.RgError(st, "rg_sim_set_warm_start: " + self._err())

    def get_state(self) -> dict:
        out = {k: np.zeros(self.np) for k in ("U", "V", "S", "z")}
        flags = np.zeros(self.np, np.int32)
        self.lib.rg_sim_get_state(self.ptr, p(out["U"]), p(out["V"]), p(out["S"]), p(out["z"]), p(flags))
        out["flag"] = flags
        return out

    def step(self, t: float, dt: float, steady: bool = False, criterion: int = RG_CRIT_RESIDUAL,
             residual_tol: float = 1e-8, max_newton: int = 0, linear_forcing: float = 0.0,
             ilu_reuse: int = 0, friction_jacobian: bool = False) -> dict:
        ctl = StepCtl(1 if steady else 0, 1 if self.step_no == 0 else 0, criterion, residual_tol, max_newton,
                      linear_forcing, ilu_reuse, 1 if friction_jacobian else 0)
        rep = StepReport()
        st = self.lib.rg_sim_step(self.ptr, C.c_double(t), C.c_double(dt), C.byref(ctl), C.byref(rep))
        if st not in (_lib.RG_OK, _lib.RG_NOT_CONVERGED):
            raise _lib.RgError(st, "rg_sim_step: " + self._err())
        self.step_no += 1
        return rep.as_dict()

    STAGES = ("dry_rewet", "friction", "bcon", "numbering", "upload", "download", "assemble", "factor", "krylov",
              "update", "warm_start")

    def stage_ms(self, reset: bool = False) -> dict:
        """Host wall time per stage of the steps since the last reset (ms)."""
        ms = np.zeros(len(self.STAGES))
        st = self.lib.rg_sim_stage_ms(self.ptr, p(ms), C.c_int(len(ms)), C.c_int(1 if reset else 0))
        if st != _lib.RG_OK:
            raise _lib.RgError(st, "rg_sim_stage_ms")
        return dict(zip(self.STAGES, ms.tolist()))

    def continuity(self) -> dict:
        """MODEL::Continuity (Contin.cpp:43-170) of the current state, FP64 on the GPU:
        per control line k+1 the discharge Q = Qx + Qy and its parts."""
        ns = C.c_int()
        st = self.lib.rg_sim_continuity(self.ptr, C.byref(ns), None, None)
        if st != _lib.RG_OK:
            raise _lib.RgError(st, "rg_sim_continuity: " + self._err())
        qx, qy = np.zeros(ns.value), np.zeros(ns.value)
        st = self.lib.rg_sim_continuity(self.ptr, None, p(qx), p(qy))
        if st != _lib.RG_OK:
            raise _lib.RgError(st, "rg_sim_continuity: " + self._err())
        return {"Q": qx + qy, "Qx": qx, "Qy": qy}

    # -- inspection of the host model (numbering, pattern, boundary data) ----
    def prepare_iteration(self, t_bc: float, cf=None):
        cf = None if cf is None else np.ascontiguousarray(cf, np.float64)
        st = self.lib.rg_sim_prepare_iteration(self.ptr, C.c_double(t_bc), p(cf))
        if st != _lib.RG_OK:
            raise _lib.RgError(st, "rg_sim_prepare_iteration: " + self._err())

    def dry_rewet_pass(self):
        d, w = C.c_int(), C.c_int()
        st = self.lib.rg_sim_dry_rewet(self.ptr, C.byref(d), C.byref(w))
        if st != _lib.RG_OK:
            raise _lib.RgError(st, "rg_sim_dry_rewet: " + self._err())
        return d.value, w.value

    def numbering(self) -> dict:
        neq = C.c_int()
        nnz = C.c_int64()
        self.lib.rg_sim_get_numbering(self.ptr, C.byref(neq), None, None, C.byref(nnz))
        eqno = np.zeros(3 * self.np, np.int32)
        width = np.zeros(neq.value, np.int32)
        self.lib.rg_sim_get_numbering(self.ptr, None, p(eqno), p(width), None)
        index = np.zeros(nnz.value, np.int32)
        self.lib.rg_sim_get_pattern(self.ptr, p(index))
        return dict(neq=neq.value, eqno=eqno.reshape(-1, 3), width=width, index=index)

    def model(self) -> dict:
        """Model element list and open-boundary normals of the last model build."""
        ne = C.c_int()
        self.lib.rg_sim_get_model(self.ptr, C.byref(ne), None, None, None, None, None, None)
        m = ne.value
        out = dict(elem_nodes=np.zeros((m, 6), np.int32), elem_nnd=np.zeros(m, np.int32),
                   elem_flag=np.zeros(m, np.int32), elem_vt=np.zeros(m), niox=np.zeros(self.np),
                   nioy=np.zeros(self.np))
        st = self.lib.rg_sim_get_model(self.ptr, None, p(out["elem_nodes"]), p(out["elem_nnd"]),
                                       p(out["elem_flag"]), p(out["elem_vt"]), p(out["niox"]), p(out["nioy"]))
        if st != _lib.RG_OK:
            raise _lib.RgError(st, "rg_sim_get_model: " + self._err())
        return out

    # -- the GPU context: structure, copy counters, per-kernel device time ----
    def context(self) -> C.c_void_p:
        self.lib.rg_sim_context.restype = C.c_void_p
        return C.c_void_p(self.lib.rg_sim_context(self.ptr))

    def stats(self) -> np.ndarray:
        out = np.zeros(15, np.int64)
        self.lib.rg_get_stats(self.context(), p(out), C.c_int(15))
        return out

    def profile(self, enable: bool, reset: bool = True):
        st = self.lib.rg_profile(self.context(), C.c_int(1 if enable else 0), C.c_int(1 if reset else 0))
        if st != _lib.RG_OK:
            raise _lib.RgError(st, "rg_profile")

    def profile_read(self) -> dict:
        out = np.zeros(8)
        self.lib.rg_profile_read(self.context(), p(out), C.c_int(8))
        names = ("trsv", "spmv", "factor", "assemble")
        return {k: (int(out[2 * i]), float(out[2 * i + 1])) for i, k in enumerate(names)}

    def event_record(self, slot: int):
        st = self.lib.rg_event_record(self.context(), C.c_int(slot))
        if st != _lib.RG_OK:
            raise _lib.RgError(st, "rg_event_record")

    def event_elapsed(self, a: int, b: int) -> float:
        ms = C.c_double()
        st = self.lib.rg_event_elapsed(self.context(), C.c_int(a), C.c_int(b), C.byref(ms))
        if st != _lib.RG_OK:
            raise _lib.RgError(st, "rg_event_elapsed")
        return ms.value

    def boundary(self) -> dict:
        out = dict(nflag=np.zeros(self.np, np.int32), bckind=np.zeros(self.np, np.int32),
                   rot4=np.zeros((self.np, 4)), bcU=np.zeros(self.np), bcS=np.zeros(self.np))
        self.lib.rg_sim_get_boundary(self.ptr, p(out["nflag"]), p(out["bckind"]), p(out["rot4"]), p(out["bcU"]),
                                     p(out["bcS"]))
        return out
