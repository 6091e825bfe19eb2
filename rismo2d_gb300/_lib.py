"""ctypes bindings of the rg300 C ABI (include/rg300.h).

Loads the in-tree librg300.so; there is no fallback: if the library is missing
or cannot be loaded the import of this module fails with the loader's error.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librg300.so")

RG_OK = 0
RG_NOT_CONVERGED = 1
RG_ERR_ARG = 10
RG_ERR_CUDA = 11
RG_ERR_ZERO_PIVOT = 12
RG_ERR_DEVICE_WAIT = 13
RG_ERR_NONFINITE = 14

PREC_FP64 = 0
PREC_REF32 = 1
PREC_MIXED = 2

# every symbol the public header declares (checked by the CPU test suite)
EXPORTS = ["rg_create", "rg_destroy", "rg_last_error", "rg_version", "rg_set_pattern", "rg_set_boundary",
           "rg_set_state", "rg_get_state", "rg_set_relax", "rg_set_jacobian", "rg_set_wait_limit", "rg_set_fp64_pivots", "rg_assemble", "rg_load_system", "rg_scale",
           "rg_ilu0_factor", "rg_ilu0_apply", "rg_ilu0_apply_f32", "rg_spmv", "rg_bicgstab", "rg_solve", "rg_set_update_lists",
           "rg_newton_update", "rg_set_friction", "rg_friction", "rg_continuity", "rg_get_timings",
           "rg_sim_create", "rg_sim_destroy", "rg_sim_last_error", "rg_sim_set_state", "rg_sim_get_state",
           "rg_sim_step", "rg_sim_prepare_iteration", "rg_sim_get_numbering", "rg_sim_get_pattern",
           "rg_sim_get_boundary", "rg_set_elements", "rg_set_old", "rg_get_dt", "rg_timegrad",
           "rg_zero_velocity", "rg_sim_dry_rewet", "rg_get_stats", "rg_event_record", "rg_event_elapsed",
           "rg_sim_context", "rg_profile", "rg_profile_read", "rg_sim_get_model",
           "rg_ilu0_apply_dev_noalloc",
           "rg_mlp_create", "rg_mlp_destroy", "rg_mlp_last_error", "rg_mlp_set_mesh", "rg_mlp_set_scales",
           "rg_mlp_get_params", "rg_mlp_set_params", "rg_mlp_features", "rg_mlp_add_samples",
           "rg_mlp_clear_samples", "rg_mlp_train", "rg_mlp_loss_grad", "rg_mlp_predict",
           "rg_sim_set_warm_start", "rg_sim_stage_ms", "rg_sim_continuity"]


class RgMesh(C.Structure):
    _fields_ = [("np", C.c_int), ("x", C.c_void_p), ("y", C.c_void_p), ("ne", C.c_int),
                ("elem_nodes", C.c_void_p), ("elem_nnd", C.c_void_p), ("elem_flag", C.c_void_p),
                ("elem_vt", C.c_void_p), ("g", C.c_double), ("hmin", C.c_double), ("vk", C.c_double)]


class RgUpdateOpts(C.Structure):
    _fields_ = [("relax_method", C.c_int), ("max_delta_uv", C.c_double), ("max_delta_s", C.c_double),
                ("max_us", C.c_double), ("dry_limit", C.c_double), ("dryrew_method", C.c_int)]


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"rg300 CUDA library not built: {LIB_PATH} is missing "
                              "(run `python -c 'import __graft_entry__ as g; g.build()'`)")
        lib = C.CDLL(LIB_PATH)
        for name in EXPORTS:
            getattr(lib, name)
        lib.rg_last_error.restype = C.c_char_p
        lib.rg_version.restype = C.c_char_p
        _lib = lib
    return _lib


def p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class RgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"rg300 status {status}: {msg}")
        self.status = status


class Context:
    """One rg_ctx: mesh, pattern and device buffers on one GPU."""

    def __init__(self, x, y, elem_nodes, elem_nnd, elem_flag, elem_vt, g, hmin, vk,
                 precision: int = PREC_FP64, device: int = 0):
        self.lib = load()
        self._keep = [np.ascontiguousarray(x, np.float64), np.ascontiguousarray(y, np.float64),
                      np.ascontiguousarray(elem_nodes, np.int32).reshape(-1, 6),
                      np.ascontiguousarray(elem_nnd, np.int32), np.ascontiguousarray(elem_flag, np.int32),
                      np.ascontiguousarray(elem_vt, np.float64)]
        xx, yy, en, ennd, ef, evt = self._keep
        m = RgMesh(len(xx), p(xx), p(yy), len(ennd), p(en), p(ennd), p(ef), p(evt), g, hmin, vk)
        self.ptr = C.c_void_p()
        st = self.lib.rg_create(C.byref(m), C.c_int(precision), C.c_int(device), C.byref(self.ptr))
        if st != RG_OK:
            msg = self.lib.rg_last_error(self.ptr).decode() if self.ptr else ""
            raise RgError(st, "rg_create: " + msg)
        self.np = len(xx)
        self.precision = precision
        self.neq = 0
        self.nnz = 0

    def _check(self, st: int, what: str, ok=(RG_OK,)):
        if st not in ok:
            raise RgError(st, f"{what}: {self.lib.rg_last_error(self.ptr).decode()}")
        return st

    def close(self):
        if self.ptr:
            self.lib.rg_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_pattern(self, width, index, eqno):
        width = np.ascontiguousarray(width, np.int32)
        index = np.ascontiguousarray(index, np.int32)
        eqno = np.ascontiguousarray(eqno, np.int32).reshape(-1)
        self._check(self.lib.rg_set_pattern(self.ptr, C.c_int(len(width)), p(width), p(index), p(eqno)),
                    "rg_set_pattern")
        self.neq = len(width)
        self.nnz = int(width.sum())

    def set_boundary(self, nflag, bckind, rot, niox, nioy, bcU, bcS):
        arrs = [np.ascontiguousarray(nflag, np.int32), np.ascontiguousarray(bckind, np.int32),
                np.ascontiguousarray(rot, np.float64).reshape(-1), np.ascontiguousarray(niox, np.float64),
                np.ascontiguousarray(nioy, np.float64), np.ascontiguousarray(bcU, np.float64),
                np.ascontiguousarray(bcS, np.float64)]
        self._check(self.lib.rg_set_boundary(self.ptr, *[p(a) for a in arrs]), "rg_set_boundary")

    def set_state(self, U=None, V=None, S=None, dUdt=None, dVdt=None, dSdt=None, z=None, cf=None, cfw=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64)
                for a in (U, V, S, dUdt, dVdt, dSdt, z, cf, cfw)]
        self._check(self.lib.rg_set_state(self.ptr, *[p(a) for a in arrs]), "rg_set_state")

    def get_state(self):
        out = [np.zeros(self.np) for _ in range(4)]
        self._check(self.lib.rg_get_state(self.ptr, *[p(a) for a in out]), "rg_get_state")
        return dict(zip(["U", "V", "S", "z"], out))

    def set_fp64_pivots(self, depth: float):
        self._check(self.lib.rg_set_fp64_pivots(self.ptr, C.c_double(depth)), "rg_set_fp64_pivots")

    def set_wait_limit(self, polls: int):
        self._check(self.lib.rg_set_wait_limit(self.ptr, C.c_longlong(polls)), "rg_set_wait_limit")

    def set_relax(self, r_uv, r_h):
        self._check(self.lib.rg_set_relax(self.ptr, C.c_double(r_uv), C.c_double(r_h)), "rg_set_relax")

    def assemble(self, want_A=True):
        B = np.zeros(self.neq)
        A32 = np.zeros(self.nnz, np.float32) if (want_A and self.precision != PREC_FP64) else None
        A64 = np.zeros(self.nnz, np.float64) if (want_A and self.precision == PREC_FP64) else None
        self._check(self.lib.rg_assemble(self.ptr, p(B), p(A32), p(A64)), "rg_assemble")
        return (A64 if A64 is not None else A32), B

    def load_system(self, A, B):
        A = np.ascontiguousarray(A)
        B = np.ascontiguousarray(B, np.float64)
        if A.dtype == np.float32:
            st = self.lib.rg_load_system(self.ptr, p(A), None, p(B))
        else:
            A = A.astype(np.float64)
            st = self.lib.rg_load_system(self.ptr, None, p(A), p(B))
        self._check(st, "rg_load_system")

    def scale(self):
        s = C.c_double()
        self._check(self.lib.rg_scale(self.ptr, C.byref(s)), "rg_scale")
        return s.value

    def ilu0_factor(self, want_LU=False):
        LU32 = LU64 = None
        if want_LU:
            if self.precision == PREC_FP64:
                LU64 = np.zeros(self.nnz)
            else:
                LU32 = np.zeros(self.nnz, np.float32)
        self._check(self.lib.rg_ilu0_factor(self.ptr, p(LU32), p(LU64)), "rg_ilu0_factor")
        return LU64 if LU64 is not None else LU32

    def ilu0_apply(self, b):
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros(self.neq)
        self._check(self.lib.rg_ilu0_apply(self.ptr, p(b), p(x)), "rg_ilu0_apply")
        return x

    def ilu0_apply_f32(self, b):
        b = np.ascontiguousarray(b, np.float32)
        x = np.zeros(self.neq, np.float32)
        self._check(self.lib.rg_ilu0_apply_f32(self.ptr, p(b), p(x)), "rg_ilu0_apply_f32")
        return x

    def spmv(self, x):
        x = np.ascontiguousarray(x, np.float64)
        r = np.zeros(self.neq)
        self._check(self.lib.rg_spmv(self.ptr, p(x), p(r)), "rg_spmv")
        return r

    def bicgstab(self, maxiter=1000, maxdiff=1e-8):
        X = np.zeros(self.neq)
        it = C.c_int()
        acc = C.c_double()
        st = self._check(self.lib.rg_bicgstab(self.ptr, C.c_int(maxiter), C.c_double(maxdiff), p(X),
                                              C.byref(it), C.byref(acc)), "rg_bicgstab",
                         ok=(RG_OK, RG_NOT_CONVERGED))
        return st == RG_OK, X, it.value, acc.value

    def solve(self, maxiter=1000, maxdiff=1e-8):
        X = np.zeros(self.neq)
        sc = C.c_double()
        it = C.c_int()
        st = self._check(self.lib.rg_solve(self.ptr, C.c_int(maxiter), C.c_double(maxdiff), p(X), C.byref(sc),
                                           C.byref(it)), "rg_solve", ok=(RG_OK, RG_NOT_CONVERGED))
        return st == RG_OK, X, sc.value, it.value

    def set_update_lists(self, model_nodes, region_nodes, zor):
        mn = np.ascontiguousarray(model_nodes, np.int32)
        rn = np.ascontiguousarray(region_nodes, np.int32).reshape(-1)
        zo = np.ascontiguousarray(zor, np.float64)
        self._keep_upd = (mn, rn, zo)
        self._check(self.lib.rg_set_update_lists(self.ptr, C.c_int(len(mn)), p(mn), C.c_int(len(rn) // 6), p(rn),
                                                 p(zo)), "rg_set_update_lists")

    def newton_update(self, relax_method=2, max_delta_uv=0.5, max_delta_s=0.5, max_us=100.0, dry_limit=0.01,
                      dryrew_method=2):
        o = RgUpdateOpts(relax_method, max_delta_uv, max_delta_s, max_us, dry_limit, dryrew_method)
        stats = np.zeros(6)
        self._check(self.lib.rg_newton_update(self.ptr, C.byref(o), p(stats)), "rg_newton_update")
        return stats

    def set_friction(self, elem_n, elem_areafact):
        en = np.ascontiguousarray(elem_n, np.float64)
        ea = np.ascontiguousarray(elem_areafact, np.float64)
        self._check(self.lib.rg_set_friction(self.ptr, p(en), p(ea)), "rg_set_friction")

    def friction(self):
        cf = np.zeros(self.np)
        self._check(self.lib.rg_friction(self.ptr, p(cf)), "rg_friction")
        return cf

    def timings(self):
        ms = np.zeros(8)
        self._check(self.lib.rg_get_timings(self.ptr, p(ms), C.c_int(8)), "rg_get_timings")
        return ms
