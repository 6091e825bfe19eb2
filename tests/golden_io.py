"""Helpers that turn a golden fixture (tests/golden/*.npz) into the inputs of
the oracle and of the rg300 C ABI."""

from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name: str) -> dict:
    d = np.load(os.path.join(GOLDEN, name))
    return {k: d[k] for k in d.files}


def state(g: dict, it) -> dict:
    pre = f"it{it}_" if it != "final" else "final_"
    out = {k[len(pre):]: v for k, v in g.items() if k.startswith(pre)}
    width = out.pop("crs_width", g["crs_width"])
    out["width"] = width
    out["index"] = out.pop("crs_index", g["crs_index"])
    ptr = np.zeros(len(width) + 1, np.int64)
    ptr[1:] = np.cumsum(width)
    out["ptr"] = ptr
    out["eqno"] = np.stack([out["eq0"], out["eq1"], out["eq2"]], axis=1).astype(np.int32)
    out["rot4"] = np.stack([out["r00"], out["r01"], out["r10"], out["r11"]], axis=1)
    mats = out["materials"]
    # element types are 1-based TYPE ids (TYPE::Getid(i + 1), Type.cpp:409)
    out["elem_vt"] = mats[:, 3][np.clip(out["elem_type"] - 1, 0, len(mats) - 1)]
    out["region_n"] = mats[:, 2][np.clip(out["region_type"] - 1, 0, len(mats) - 1)]
    return out


def oracle_model(st: dict):
    import oracle
    return oracle.Model(x=st["x"], y=st["y"], z=st["z"], U=st["U"], V=st["V"], S=st["S"],
                        dUdt=st["dUdt"], dVdt=st["dVdt"], dSdt=st["dSdt"], cf=st["cf"], cfw=st["cfw"],
                        uu=st["uu"], uv=st["uv"], vv=st["vv"], rot=st["rot4"], niox=st["niox"],
                        nioy=st["nioy"], bcU=st["bcU"], bcS=st["bcS"], evt=st["elem_vt"], nflag=st["flag"],
                        bckind=st["bckind"], eqno=st["eqno"], enodes=st["elem_nodes"], ennd=st["elem_nnd"],
                        eflag=st["elem_flag"], g=float(st["g"]), hmin=float(st["hmin"]), vk=float(st["vk"]),
                        relaxThdt_UV=float(st["relaxThdt_UV"]), relaxThdt_H=float(st["relaxThdt_H"]))


def gpu_context(st: dict, precision: int):
    from rismo2d_gb300 import _lib
    ctx = _lib.Context(st["x"], st["y"], st["elem_nodes"], st["elem_nnd"], st["elem_flag"], st["elem_vt"],
                       float(st["g"]), float(st["hmin"]), float(st["vk"]), precision=precision)
    ctx.set_pattern(st["width"], st["index"], st["eqno"])
    load_iteration(ctx, st)
    return ctx


def load_iteration(ctx, st: dict):
    ctx.set_boundary(st["flag"], st["bckind"], st["rot4"], st["niox"], st["nioy"], st["bcU"], st["bcS"])
    ctx.set_state(U=st["U"], V=st["V"], S=st["S"], dUdt=st["dUdt"], dVdt=st["dVdt"], dSdt=st["dSdt"],
                  z=st["z"], cf=st["cf"], cfw=st["cfw"])
    ctx.set_relax(float(st["relaxThdt_UV"]), float(st["relaxThdt_H"]))
