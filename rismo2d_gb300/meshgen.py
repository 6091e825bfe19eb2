"""Seeded synthetic Taylor-Hood meshes for the shallow-water Newton step.

The reference ships no example decks, so the solver is exercised on generated
meshes of the shapes its workloads name:

* ``channel`` -- straight rectangular channel, structured quads split into two
  six-node triangles, bed slope plus Gaussian bumps.
* ``meander`` -- straight valley with a sinusoidal main channel cut into sloping
  flood plains; the channel is carved into the bed elevation, the mesh is a
  structured grid over the valley.

Node and element layout follow the reference's region-file conventions
(``GRID::InputRegion``, Grid.cpp:159-298): six-node triangles list the three
corners counter-clockwise, then the mid-side nodes of edges 0-1, 1-2, 2-0
(``SHAPE::getCornerNodes``, Shape.cpp:455-461).  Elements are emitted in a
frontal order that sweeps along the channel and across its width at each
station, which is the order the reference's element reordering produces for a
strip and therefore the order its ILU(0) runs in.
"""

from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class Mesh:
    """A P2 triangle mesh with boundary control lines and initial state."""

    x: np.ndarray            # (np,) float64
    y: np.ndarray
    z: np.ndarray            # bed elevation
    elems: np.ndarray        # (ne, 6) int32, zero-based node indices
    elem_type: np.ndarray    # (ne,) int32 material number (1-based)
    lines: dict              # line number -> (nl, 3) int32 (corner, corner, mid)
    S0: np.ndarray           # initial water surface elevation
    U0: np.ndarray
    V0: np.ndarray
    materials: list          # [(no, manning_n, vt)]
    meta: dict

    @property
    def np(self) -> int:
        return int(self.x.shape[0])

    @property
    def ne(self) -> int:
        return int(self.elems.shape[0])


def _strip(nx: int, ny: int):
    """Structured (2nx+1) x (2ny+1) P2 node grid and its triangles.

    Returns node (i, j) index arrays, element connectivity (zero-based) and the
    inlet (i=0) / outlet (i=2nx) boundary line elements.  Quads are visited
    station by station along i, across j inside a station.
    """
    px, py = 2 * nx + 1, 2 * ny + 1

    def nid(i, j):
        return i * py + j            # node numbering also sweeps across first

    ii, jj = np.meshgrid(np.arange(px), np.arange(py), indexing="ij")
    els = []
    for i in range(nx):
        for j in range(ny):
            a, b = nid(2 * i, 2 * j), nid(2 * i + 2, 2 * j)
            c, d = nid(2 * i + 2, 2 * j + 2), nid(2 * i, 2 * j + 2)
            mab, mbc = nid(2 * i + 1, 2 * j), nid(2 * i + 2, 2 * j + 1)
            mcd, mda = nid(2 * i + 1, 2 * j + 2), nid(2 * i, 2 * j + 1)
            mac = nid(2 * i + 1, 2 * j + 1)
            els.append((a, b, c, mab, mbc, mac))
            els.append((a, c, d, mac, mcd, mda))
    inlet = [(nid(0, 2 * j), nid(0, 2 * j + 2), nid(0, 2 * j + 1)) for j in range(ny)]
    outlet = [(nid(2 * nx, 2 * j), nid(2 * nx, 2 * j + 2), nid(2 * nx, 2 * j + 1)) for j in range(ny)]
    return (ii.ravel(), jj.ravel(), np.asarray(els, dtype=np.int32),
            np.asarray(inlet, dtype=np.int32), np.asarray(outlet, dtype=np.int32))


def channel(nx: int = 50, ny: int = 10, length: float = 1000.0, width: float = 100.0,
            slope: float = 0.001, nbumps: int = 8, seed: int = 1, depth0: float = 3.0,
            manning_n: float = 1.0 / 30.0, vt: float = 0.5, Q: float = 200.0,
            S_out: float = 3.0) -> Mesh:
    """Straight channel: bed slope plus seeded Gaussian bumps (sigma 20 m)."""
    rng = np.random.default_rng(seed)
    ii, jj, els, inlet, outlet = _strip(nx, ny)
    x = length * ii / (2 * nx)
    y = width * jj / (2 * ny)
    z = slope * (length - x)
    cx = rng.uniform(0.0, length, nbumps)
    cy = rng.uniform(0.0, width, nbumps)
    amp = rng.uniform(0.05, 0.2, nbumps)
    for k in range(nbumps):
        z = z + amp[k] * np.exp(-((x - cx[k]) ** 2 + (y - cy[k]) ** 2) / (2.0 * 20.0 ** 2))
    S0 = z + depth0
    return Mesh(x=x.astype(np.float64), y=y.astype(np.float64), z=z, elems=els,
                elem_type=np.ones(els.shape[0], np.int32),
                lines={1: inlet, 2: outlet}, S0=S0, U0=np.zeros_like(x), V0=np.zeros_like(x),
                materials=[(1, manning_n, vt)],
                meta=dict(kind="channel", nx=nx, ny=ny, Q=Q, S_out=S_out, steady=True))


def sin2_hydrograph(Q0: float = 300.0, dQ: float = 500.0, period: float = 7200.0, t_end: float = 7200.0,
                    every: float = 600.0, S: float = 4.0) -> list:
    """QTINLET table of Q(t) = Q0 + dQ sin^2(pi t / period), one row per `every` seconds."""
    ts = np.arange(0.0, t_end + 0.5 * every, every)
    return [(float(t), Q0 + dQ * np.sin(np.pi * t / period) ** 2, S) for t in ts]


def meander(nx: int = 1266, ny: int = 79, length: float = 10000.0, amplitude: float = 80.0,
            wavelength: float = 400.0, channel_width: float = 60.0, channel_depth: float = 4.0,
            plain_width: float = 200.0, plain_rise: float = 1.0, valley_slope: float = 5.0e-4,
            kst_median: float = 20.0, kst_sigma: float = 0.3, nbands: int = 16, seed: int = 2,
            vt: float = 0.5, Q0: float = 300.0, depth_out: float = 3.5) -> Mesh:
    """Meandering main channel inside a straight valley with flood plains.

    The valley is ``2*(amplitude + channel_width/2 + plain_width)`` wide.  The
    channel bed lies ``channel_depth`` below the flood-plain surface at the
    bank; the flood plains rise by ``plain_rise`` over ``plain_width`` towards
    the valley edge.  Roughness is log-normal per along-valley band.
    """
    rng = np.random.default_rng(seed)
    half = amplitude + 0.5 * channel_width + plain_width
    width = 2.0 * half
    ii, jj, els, inlet, outlet = _strip(nx, ny)
    x = length * ii / (2 * nx)
    y = width * jj / (2 * ny) - half
    yc = amplitude * np.sin(2.0 * np.pi * x / wavelength)
    d = np.abs(y - yc)                      # lateral distance from the centreline
    valley = valley_slope * (length - x)
    bank = 0.5 * channel_width
    plain = channel_depth + plain_rise * np.clip((d - bank) / plain_width, 0.0, 1.0)
    z = np.where(d <= bank, 0.0, plain) + valley
    # per-element material band along the valley, log-normal Strickler
    kst = kst_median * np.exp(kst_sigma * rng.standard_normal(nbands))
    mats = [(k + 1, 1.0 / kst[k], vt) for k in range(nbands)]
    elx = x[els[:, :3]].mean(axis=1)
    etype = (np.minimum((elx / length * nbands).astype(np.int32), nbands - 1) + 1).astype(np.int32)
    S_out = depth_out                         # outlet level above the channel bed at x=length
    S0 = np.maximum(valley + depth_out, z)    # water surface parallel to the valley, dry where the bed is higher
    return Mesh(x=x.astype(np.float64), y=y.astype(np.float64), z=z, elems=els, elem_type=etype,
                lines={1: inlet, 2: outlet}, S0=S0, U0=np.zeros_like(x), V0=np.zeros_like(x),
                materials=mats,
                meta=dict(kind="meander", nx=nx, ny=ny, Q=Q0, S_out=S_out, steady=False))
