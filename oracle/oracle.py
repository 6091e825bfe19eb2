"""ctypes bindings of the oracle restatement (liboracle.so built from rg_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and
by the CPU-baseline leg of bench.py, always as the checker.  The shipped library
never imports this module.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")


def reference_sources() -> str:
    """Directory of the reference's C++ sources: $RG_REFERENCE_SOURCES, else the
    REFSRC default of oracle/Makefile (the recipe that compiles them)."""
    env = os.environ.get("RG_REFERENCE_SOURCES")
    if env:
        return env
    with open(os.path.join(HERE, "Makefile")) as f:
        for line in f:
            if line.startswith("REFSRC"):
                return line.split("=", 1)[1].strip()
    return ""

_lib = None


def build(force: bool = False) -> str:
    src = [os.path.join(HERE, "rg_oracle.c")]
    deps = src + [os.path.join(HERE, "rg_oracle_la.inc"), os.path.join(HERE, "rg_oracle.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-std=c99", "-o", LIB] + src + ["-lm"])
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
    return _lib


class OrcModel(C.Structure):
    _fields_ = [("np", C.c_int),
                ("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
                ("U", C.c_void_p), ("V", C.c_void_p), ("S", C.c_void_p),
                ("dUdt", C.c_void_p), ("dVdt", C.c_void_p), ("dSdt", C.c_void_p),
                ("cf", C.c_void_p), ("cfw", C.c_void_p), ("uu", C.c_void_p),
                ("uv", C.c_void_p), ("vv", C.c_void_p),
                ("nflag", C.c_void_p), ("bckind", C.c_void_p), ("rot", C.c_void_p),
                ("niox", C.c_void_p), ("nioy", C.c_void_p), ("bcU", C.c_void_p), ("bcS", C.c_void_p),
                ("eqno", C.c_void_p),
                ("ne", C.c_int), ("enodes", C.c_void_p), ("ennd", C.c_void_p),
                ("eflag", C.c_void_p), ("evt", C.c_void_p),
                ("g", C.c_double), ("hmin", C.c_double), ("vk", C.c_double),
                ("relaxThdt_UV", C.c_double), ("relaxThdt_H", C.c_double)]


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class Model:
    """Holds contiguous arrays and the orc_model struct pointing into them."""

    DBL = ["x", "y", "z", "U", "V", "S", "dUdt", "dVdt", "dSdt", "cf", "cfw", "uu", "uv", "vv",
           "rot", "niox", "nioy", "bcU", "bcS", "evt"]
    INT = ["nflag", "bckind", "eqno", "enodes", "ennd", "eflag"]

    def __init__(self, **kw):
        self.arrays = {}
        for k in self.DBL:
            self.arrays[k] = np.ascontiguousarray(kw[k], dtype=np.float64)
        for k in self.INT:
            self.arrays[k] = np.ascontiguousarray(kw[k], dtype=np.int32)
        s = OrcModel()
        s.np = int(self.arrays["x"].shape[0])
        s.ne = int(self.arrays["ennd"].shape[0])
        for k in self.DBL + self.INT:
            if hasattr(s, k):
                setattr(s, k, _p(self.arrays[k]))
        for k in ("g", "hmin", "vk", "relaxThdt_UV", "relaxThdt_H"):
            setattr(s, k, float(kw[k]))
        self.struct = s

    @property
    def neq(self) -> int:
        return int(self.arrays["eqno"].max()) + 1


def model_from_state(st: dict) -> Model:
    """orc_model inputs from a STATE record of the reference dump."""
    mats = st["materials"]
    evt = mats[:, 3][np.clip(st["elem_type"] - 1, 0, len(mats) - 1)]   # 1-based TYPE ids
    rot = np.stack([st["r00"], st["r01"], st["r10"], st["r11"]], axis=1)
    eqno = np.stack([st["eq0"], st["eq1"], st["eq2"]], axis=1)
    return Model(x=st["x"], y=st["y"], z=st["z"], U=st["U"], V=st["V"], S=st["S"],
                 dUdt=st["dUdt"], dVdt=st["dVdt"], dSdt=st["dSdt"], cf=st["cf"], cfw=st["cfw"],
                 uu=st["uu"], uv=st["uv"], vv=st["vv"], rot=rot, niox=st["niox"], nioy=st["nioy"],
                 bcU=st["bcU"], bcS=st["bcS"], evt=evt, nflag=st["flag"], bckind=st["bckind"],
                 eqno=eqno, enodes=st["elem_nodes"], ennd=st["elem_nnd"], eflag=st["elem_flag"],
                 g=st["g"], hmin=st["hmin"], vk=st["vk"], relaxThdt_UV=st["relaxThdt_UV"],
                 relaxThdt_H=st["relaxThdt_H"])


def coefs(m: Model, e: int):
    K = np.zeros((24, 24))
    f = np.zeros(24)
    ok = lib().orc_coefs(C.byref(m.struct), C.c_int(e), _p(K), _p(f))
    return ok, K, f


def assemble(m: Model, ptr: np.ndarray, index: np.ndarray, dtype=np.float32):
    neq = ptr.shape[0] - 1
    ptr = np.ascontiguousarray(ptr, np.int64)
    index = np.ascontiguousarray(index, np.int32)
    A = np.zeros(int(ptr[-1]), dtype)
    B = np.zeros(neq)
    fn = lib().orc_assemble_f32 if dtype == np.float32 else lib().orc_assemble_f64
    fn(C.byref(m.struct), C.c_int(neq), _p(ptr), _p(index), _p(A), _p(B))
    return A, B


def _sfx(dtype):
    return "f32" if np.dtype(dtype) == np.float32 else "f64"


def scale_l2(ptr, A, B):
    fn = getattr(lib(), "orc_scale_l2_" + _sfx(A.dtype))
    fn.restype = C.c_double
    return fn(C.c_int(len(B)), _p(ptr), _p(A), _p(B))


def spmv(ptr, index, A, x):
    r = np.zeros(len(x))
    getattr(lib(), "orc_spmv_" + _sfx(A.dtype))(C.c_int(len(x)), _p(ptr), _p(index), _p(A), _p(x), _p(r))
    return r


def ilu0_factor(ptr, index, A):
    ILU = np.zeros_like(A)
    rc = getattr(lib(), "orc_ilu0_factor_" + _sfx(A.dtype))(C.c_int(len(ptr) - 1), _p(ptr), _p(index),
                                                           _p(A), _p(ILU))
    return rc, ILU


def ilu0_solve(ptr, index, ILU, B):
    X = np.zeros(len(B))
    getattr(lib(), "orc_ilu0_solve_" + _sfx(ILU.dtype))(C.c_int(len(B)), _p(ptr), _p(index), _p(ILU),
                                                       _p(np.ascontiguousarray(B)), _p(X))
    return X


def bicgstab(ptr, index, A, ILU, b, maxiter=1000, maxdiff=1e-8, x0=None):
    x = np.zeros(len(b)) if x0 is None else np.array(x0, dtype=np.float64)
    it = C.c_int(0)
    acc = C.c_double(0)
    ok = getattr(lib(), "orc_bicgstab_" + _sfx(A.dtype))(
        C.c_int(len(b)), _p(ptr), _p(index), _p(A), _p(ILU), _p(np.ascontiguousarray(b)), _p(x),
        C.c_int(maxiter), C.c_double(maxdiff), C.byref(it), C.byref(acc))
    return ok, x, it.value, acc.value


def continuity(seg_nodes, seg_section, nsect, x, y, U, V, S, z):
    """Discharge through the control sections (MODEL::Continuity, Contin.cpp:43-170)."""
    L = lib()
    seg_nodes = np.ascontiguousarray(seg_nodes, np.int32).reshape(-1)
    seg_section = np.ascontiguousarray(seg_section, np.int32)
    arrs = [np.ascontiguousarray(a, np.float64) for a in (x, y, U, V, S, z)]
    qx, qy = np.zeros(nsect), np.zeros(nsect)
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    L.orc_continuity(C.c_int(len(seg_section)), P(seg_nodes), P(seg_section), C.c_int(nsect),
                     *[P(a) for a in arrs], P(qx), P(qy))
    return qx, qy


def pattern(np_, enodes, eqno, neq):
    """CRS pattern in the layout of EQS::SetIndexMat (IndexMat.cpp:91-342) for six-node
    elements `enodes` (ne, 6) and equation numbers `eqno` (np, 3; -1 none)."""
    L = lib()
    L.orc_pattern.restype = C.c_int64
    en = np.ascontiguousarray(enodes, np.int32).reshape(-1)
    eq = np.ascontiguousarray(eqno, np.int32).reshape(-1)
    ptr = np.zeros(neq + 1, np.int64)
    nnz = L.orc_pattern(C.c_int(np_), C.c_int(len(en) // 6), _p(en), _p(eq), C.c_int(neq), _p(ptr), None)
    idx = np.zeros(nnz, np.int32)
    L.orc_pattern(C.c_int(np_), C.c_int(len(en) // 6), _p(en), _p(eq), C.c_int(neq), _p(ptr), _p(idx))
    return ptr, idx
