"""Seeded synthetic Taylor-Hood meshes for the shallow-water Newton step.

The reference ships no example decks, so the solver is exercised on generated
meshes of the shapes its workloads name:

* ``channel`` -- straight rectangular channel, structured quads split into two
  six-node triangles, bed slope plus Gaussian bumps.
* ``meander`` -- straight valley with a sinusoidal main channel cut into sloping
  flood plains; the channel is carved into the bed elevation, the mesh is a
  structured grid over the valley.
* ``braided`` -- 20 km x 2 km braided river: intersecting anabranches between
  bars whose bed is three octaves of gradient noise; the bars start dry.

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
    station by station along i, across j inside a station; each quad gives the
    triangles (a, b, c) and (a, c, d) with a, b, c, d its corners counter-
    clockwise from (i, j).  Node numbering also sweeps across first.
    """
    px, py = 2 * nx + 1, 2 * ny + 1
    ii, jj = np.meshgrid(np.arange(px), np.arange(py), indexing="ij")
    qi, qj = np.meshgrid(np.arange(nx, dtype=np.int64), np.arange(ny, dtype=np.int64), indexing="ij")
    qi, qj = qi.ravel(), qj.ravel()

    def nid(i, j):
        return i * py + j

    a, b = nid(2 * qi, 2 * qj), nid(2 * qi + 2, 2 * qj)
    c, d = nid(2 * qi + 2, 2 * qj + 2), nid(2 * qi, 2 * qj + 2)
    mab, mbc = nid(2 * qi + 1, 2 * qj), nid(2 * qi + 2, 2 * qj + 1)
    mcd, mda = nid(2 * qi + 1, 2 * qj + 2), nid(2 * qi, 2 * qj + 1)
    mac = nid(2 * qi + 1, 2 * qj + 1)
    els = np.empty((2 * nx * ny, 6), np.int32)
    els[0::2] = np.stack([a, b, c, mab, mbc, mac], axis=1)
    els[1::2] = np.stack([a, c, d, mac, mcd, mda], axis=1)
    j = np.arange(ny, dtype=np.int64)
    inlet = np.stack([nid(0, 2 * j), nid(0, 2 * j + 2), nid(0, 2 * j + 1)], axis=1).astype(np.int32)
    outlet = np.stack([nid(2 * nx, 2 * j), nid(2 * nx, 2 * j + 2), nid(2 * nx, 2 * j + 1)], axis=1).astype(np.int32)
    return ii.ravel(), jj.ravel(), els, inlet, outlet


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
            vt: float = 0.5, Q0: float = 300.0, depth_out: float = 3.5, bumps: int = 0,
            bump_seed: int = 0, bump_amp: tuple = (0.1, 0.5), bump_sigma: float = 30.0) -> Mesh:
    """Meandering main channel inside a straight valley with flood plains.

    The valley is ``2*(amplitude + channel_width/2 + plain_width)`` wide.  The
    channel bed lies ``channel_depth`` below the flood-plain surface at the
    bank; the flood plains rise by ``plain_rise`` over ``plain_width`` towards
    the valley edge.  Roughness is log-normal per along-valley band.  With
    ``bumps`` > 0, a field of that many Gaussian bumps (amplitude uniform in
    ``bump_amp``, positive or negative, width ``bump_sigma``, centres uniform
    over the valley; seeded by ``bump_seed``) is added to the bed.
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
    if bumps > 0:
        brng = np.random.default_rng(bump_seed)
        cx = brng.uniform(0.0, length, bumps)
        cy = brng.uniform(-half, half, bumps)
        amp = brng.uniform(*bump_amp, bumps) * brng.choice([-1.0, 1.0], bumps)
        order = np.argsort(x, kind="stable")
        xs = x[order]
        for k in range(bumps):
            lo, hi = np.searchsorted(xs, [cx[k] - 4.0 * bump_sigma, cx[k] + 4.0 * bump_sigma])
            sel = order[lo:hi]
            z[sel] += amp[k] * np.exp(-((x[sel] - cx[k]) ** 2 + (y[sel] - cy[k]) ** 2) / (2.0 * bump_sigma ** 2))
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


def perlin(x: np.ndarray, y: np.ndarray, cell_x: float, cell_y: float, rng) -> np.ndarray:
    """Gradient noise (Perlin's construction) on a lattice of cell_x x cell_y.

    Every lattice vertex gets a random unit gradient; a point takes the dot
    products of the four surrounding gradients with its offsets to those
    vertices, blended with the quintic fade 6t^5 - 15t^4 + 10t^3.  The value is
    zero on the lattice and lies in about [-0.7, 0.7].
    """
    u, v = x / cell_x, y / cell_y
    i0 = np.floor(u).astype(np.int64)
    j0 = np.floor(v).astype(np.int64)
    fu, fv = u - i0, v - j0
    i0 -= i0.min()
    j0 -= j0.min()
    ang = rng.uniform(0.0, 2.0 * np.pi, (int(i0.max()) + 2, int(j0.max()) + 2))
    gx, gy = np.cos(ang), np.sin(ang)

    def corner(di, dj):
        return gx[i0 + di, j0 + dj] * (fu - di) + gy[i0 + di, j0 + dj] * (fv - dj)

    def fade(t):
        return t * t * t * (t * (6.0 * t - 15.0) + 10.0)

    su, sv = fade(fu), fade(fv)
    n0 = corner(0, 0) + su * (corner(1, 0) - corner(0, 0))
    n1 = corner(0, 1) + su * (corner(1, 1) - corner(0, 1))
    return n0 + sv * (n1 - n0)


def braided_hydrograph(Q0: float = 500.0, Qpeak: float = 3000.0, duration: float = 86400.0,
                       every: float = 600.0, S: float = 0.0) -> list:
    """QTINLET table of a flood wave Q(t) = Q0 + (Qpeak - Q0) sin^2(pi t / duration)."""
    return sin2_hydrograph(Q0=Q0, dQ=Qpeak - Q0, period=duration, t_end=duration, every=every, S=S)


def braided(nx: int = 4000, ny: int = 500, length: float = 20000.0, width: float = 2000.0,
            valley_slope: float = 5.0e-4, anabranches: int = 5, branch_width=(80.0, 160.0),
            branch_depth: float = 3.0, bar_rise: float = 1.0, relief: float = 2.0, octaves: int = 3,
            cell_x: float = 1600.0, cell_y: float = 400.0, bed_relief: float = 0.3, depth0: float = 0.5,
            kst: float = 30.0, vt: float = 0.5, seed: int = 5, Q0: float = 500.0) -> Mesh:
    """Braided river: intersecting anabranches between bars on a fractal bed.

    ``anabranches`` sinuous channels (seeded amplitudes, wavelengths and phases,
    widths in ``branch_width``) wander across the valley and cross each other;
    their beds lie ``branch_depth`` below the valley line with a gradient-noise
    roughness of +-``bed_relief``.  Between them the bars rise ``bar_rise`` to
    ``bar_rise + relief`` above the valley line: gradient noise of ``octaves``
    octaves (lattice cells and amplitudes halve per octave, cells elongated
    along the valley), scaled to [0, 1] times ``relief``.  Banks are steps
    between neighbouring nodes, as in ``meander``: the reference's Newton
    iteration (Jacobian with the friction coefficient held fixed, bed clamped
    under nodes shallower than the dry limit) stalls on wide shallow fringes,
    which a smooth fractal bed under a shallow sheet of water produces.
    The initial water surface lies ``depth0`` above the valley line, so the
    bars start dry and flood as the hydrograph rises.  Defaults: 20 km x 2 km,
    4,000,000 six-node triangles, 8,009,001 nodes (5 m x 4 m quads).
    """
    rng = np.random.default_rng(seed)
    ii, jj, els, inlet, outlet = _strip(nx, ny)
    x = length * ii / (2 * nx)
    y = width * jj / (2 * ny)
    valley = valley_slope * (length - x)
    # bars: fractal relief scaled to [0, 1]
    noise = np.zeros_like(x)
    amp = 1.0
    for k in range(octaves):
        noise += amp * perlin(x, y, cell_x / 2 ** k, cell_y / 2 ** k, rng)
        amp *= 0.5
    lo, hi = float(np.min(noise)), float(np.max(noise))
    bars = bar_rise + relief * (noise - lo) / max(1e-12, hi - lo)
    # anabranch beds: a finer noise field of +-bed_relief
    fine = perlin(x, y, cell_x / 4, cell_y / 4, rng)
    fine *= bed_relief / max(1e-12, float(np.max(np.abs(fine))))
    inside = np.zeros(x.shape, bool)
    for _ in range(anabranches):
        a = rng.uniform(0.2, 0.4) * width
        lam = rng.uniform(2500.0, 6000.0)
        phase = rng.uniform(0.0, 2.0 * np.pi)
        w = rng.uniform(*branch_width)
        yc = 0.5 * width + a * np.sin(2.0 * np.pi * x / lam + phase)
        inside |= np.abs(y - yc) <= 0.5 * w
    z = valley + np.where(inside, -branch_depth + fine, bars)
    S0 = np.maximum(valley + depth0, z)
    return Mesh(x=x.astype(np.float64), y=y.astype(np.float64), z=z, elems=els,
                elem_type=np.ones(els.shape[0], np.int32), lines={1: inlet, 2: outlet}, S0=S0,
                U0=np.zeros_like(x), V0=np.zeros_like(x), materials=[(1, 1.0 / kst, vt)],
                meta=dict(kind="braided", nx=nx, ny=ny, Q=Q0, S_out=depth0, S_in=valley_slope * length + depth0,
                          steady=False))
