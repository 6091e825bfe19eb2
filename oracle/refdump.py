"""Reader for the binary records written by oracle/ref_hooks.cpp.

Test infrastructure: used by the golden-fixture generator and by tests that run
the reference build (oracle/_ref) in this container.  The layout of each record
mirrors the order of the ``put``/``arr`` calls in ref_hooks.cpp.
"""

from __future__ import annotations

import struct

import numpy as np

NODE_INT = ["no", "name", "flag", "bckind", "rot", "countdown"]
NODE_DBL = ["x", "y", "z", "zor", "U", "V", "S", "dUdt", "dVdt", "dSdt",
            "oU", "oV", "oS", "odUdt", "odVdt", "odSdt",
            "cf", "cfw", "vt", "uu", "uv", "vv",
            "r00", "r01", "r10", "r11", "niox", "nioy", "nx", "ny",
            "bcU", "bcV", "bcS", "bcQ", "bcA"]
NODE_EQ = ["eq0", "eq1", "eq2"]
SCALARS = ["relaxThdt_UV", "relaxThdt_H", "g", "hmin", "vk", "actualTurb", "actualDisp",
           "neq", "time", "dt", "timestep"]


class _Cursor:
    def __init__(self, buf: bytes):
        self.buf = buf
        self.pos = 0

    def scalar(self, fmt: str):
        v = struct.unpack_from(fmt, self.buf, self.pos)[0]
        self.pos += struct.calcsize(fmt)
        return v

    def arr(self, dtype):
        n = self.scalar("<q")
        dt = np.dtype(dtype)
        a = np.frombuffer(self.buf, dtype=dt, count=n, offset=self.pos).copy()
        self.pos += n * dt.itemsize
        return a


def _state(c: _Cursor) -> dict:
    d = {"np": c.scalar("<i")}
    for k in NODE_INT:
        d[k] = c.arr("<i4")
    for k in NODE_DBL:
        d[k] = c.arr("<f8")
    for k in NODE_EQ:
        d[k] = c.arr("<i4")
    d["elem_flag"] = c.arr("<i4")
    d["elem_type"] = c.arr("<i4")
    d["elem_nnd"] = c.arr("<i4")
    d["elem_name"] = c.arr("<i4")
    d["elem_areafact"] = c.arr("<f8")
    d["elem_nodes"] = c.arr("<i4").reshape(-1, 6)
    d["region_flag"] = c.arr("<i4")
    d["region_type"] = c.arr("<i4")
    d["region_areafact"] = c.arr("<f8")
    d["region_nodes"] = c.arr("<i4").reshape(-1, 6)
    d["model_nodes"] = c.arr("<i4")
    sc = c.arr("<f8")
    for k, v in zip(SCALARS, sc):
        d[k] = float(v)
    d["materials"] = c.arr("<f8").reshape(-1, 4)
    return d


def _crs(c: _Cursor) -> dict:
    neq = c.scalar("<i")
    width = c.arr("<i4")
    index = c.arr("<i4")
    A = c.arr("<f4")
    B = c.arr("<f8")
    ptr = np.zeros(neq + 1, np.int64)
    ptr[1:] = np.cumsum(width)
    return {"neq": neq, "width": width, "ptr": ptr, "index": index, "A": A, "B": B}


def read_dump(path: str) -> list:
    """Return the list of ``(tag, record)`` pairs in file order."""
    data = open(path, "rb").read()
    out = []
    pos = 0
    while pos < len(data):
        tag = data[pos:pos + 8].rstrip(b"\0").decode()
        n = struct.unpack_from("<q", data, pos + 8)[0]
        payload = data[pos + 16:pos + 16 + n]
        pos += 16 + n
        c = _Cursor(payload)
        if tag in ("STATE", "FINAL"):
            rec = _state(c)
        elif tag == "CRS":
            rec = _crs(c)
        elif tag == "SCALE":
            rec = {"scale": c.scalar("<d")}
        elif tag == "X":
            err = c.scalar("<i")
            its = c.scalar("<i")
            rec = {"err": err, "iters": its, "X": c.arr("<f8")}
        elif tag == "XL":
            err = c.scalar("<i")
            its = c.scalar("<i")
            rec = {"err": err, "iters": its, "seconds": c.scalar("<d")}
        elif tag == "ASML":
            rec = {"seconds": c.scalar("<d"), "neq": c.scalar("<i")}
        elif tag == "FINALL":
            rec = {"seconds": c.scalar("<d"), "np": c.scalar("<i")}
            for k, dt in (("U", "<f8"), ("V", "<f8"), ("S", "<f8"), ("z", "<f8"), ("flag", "<i4")):
                rec[k] = c.arr(dt)
        else:
            raise ValueError(f"unknown record {tag!r}")
        out.append((tag, rec))
    return out


def newton_iterations(records: list) -> list:
    """Group records into Newton iterations: dicts with state, crs, scale, x."""
    its = []
    cur = None
    for tag, rec in records:
        if tag == "STATE":
            cur = {"state": rec}
            its.append(cur)
        elif tag == "CRS":
            cur["crs"] = rec
        elif tag == "SCALE":
            cur["scale"] = rec["scale"]
        elif tag == "X":
            cur["x"] = rec
        elif tag == "FINAL":
            its.append({"final": rec})
    return its


def light_steps(records: list) -> list:
    """Group the records of a light dump (RG_DUMP_LIGHT=1) into time steps: per step the
    Newton residual norms, BiCGStab counts, solve and assembly seconds, equation counts,
    the step's wall time and its end state."""
    steps, cur = [], None
    for tag, rec in records:
        if cur is None:
            cur = {"scales": [], "iters": [], "solve_s": [], "assemble_s": [], "neq": []}
        if tag == "SCALE":
            cur["scales"].append(rec["scale"])
        elif tag == "XL":
            cur["iters"].append(rec["iters"])
            cur["solve_s"].append(rec["seconds"])
        elif tag == "ASML":
            cur["assemble_s"].append(rec["seconds"])
            cur["neq"].append(rec["neq"])
        elif tag == "FINALL":
            cur.update(rec)
            steps.append(cur)
            cur = None
    return steps
