"""Known-answer checks of the discretisation the path solves, on the oracle's
restatement of the element assembly (CPU): a lake at rest -- flat water
surface over a bumpy bed, no flow, no inflow, the outlet level equal to the
lake level -- and Manning uniform flow down a plane slope are exact steady
solutions of the reference's weak form (the seven-point rule integrates the
hydrostatic terms exactly and the boundary lines close the pressure
integral), so the assembled residual vanishes to rounding while the Jacobian
does not."""

import ctypes as C

import numpy as np

import oracle
from rismo2d_gb300 import deck, meshgen
from rismo2d_gb300.sim import Params, Simulation, RG_DEVICE_NONE


def _area_factors(mesh):
    """GRID::AreaFactors (ArFact.cpp:41-97): |normal| / n_z of each triangle on the bed zor."""
    en = np.ascontiguousarray(mesh.elems, np.int32)
    zor = deck.bed_zor(mesh)
    cor = en[:, :3]
    x0, y0, z0 = mesh.x[cor[:, 0]], mesh.y[cor[:, 0]], zor[cor[:, 0]]
    xx = [mesh.x[cor[:, i]] - x0 for i in (1, 2)]
    yy = [mesh.y[cor[:, i]] - y0 for i in (1, 2)]
    zz = [zor[cor[:, i]] - z0 for i in (1, 2)]
    t1 = yy[0] * zz[1] - yy[1] * zz[0]
    t2 = zz[0] * xx[1] - zz[1] * xx[0]
    t3 = xx[0] * yy[1] - xx[1] * yy[0]
    return np.ascontiguousarray(np.sqrt(t1 * t1 + t2 * t2 + t3 * t3) / t3)


def _system(mesh, params, line_bcs, S, dt=None, U=None):
    sim = Simulation(mesh, params, line_bcs=line_bcs, device=RG_DEVICE_NONE)
    zero = np.zeros(mesh.np)
    sim.set_state(zero if U is None else U, zero, S)
    sim.dry_rewet_pass()
    s0 = sim.get_state()
    en = np.ascontiguousarray(mesh.elems, np.int32)
    mats = {no: n for no, n, _vt in mesh.materials}
    elem_n = np.ascontiguousarray([mats[int(t)] for t in mesh.elem_type], np.float64)
    af = _area_factors(mesh)
    cf = np.zeros(mesh.np)
    nnd = np.full(len(en), 6, np.int32)
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    oracle.lib().orc_friction(C.c_int(mesh.np), C.c_int(len(en)), P(en), P(nnd), P(elem_n), P(af), P(s0["U"]),
                              P(s0["V"]), P(s0["S"]), P(s0["z"]), C.c_double(0.5 * params.dry_limit),
                              C.c_double(params.g), P(cf))
    sim.prepare_iteration(0.0, cf)
    st, num, bnd, mod = sim.get_state(), sim.numbering(), sim.boundary(), sim.model()
    r = 0.0 if dt is None else 1.0 / dt / params.theta
    m = oracle.Model(x=mesh.x, y=mesh.y, z=st["z"], U=st["U"], V=st["V"], S=st["S"], dUdt=zero, dVdt=zero,
                     dSdt=zero, cf=cf, cfw=zero, uu=zero, uv=zero, vv=zero, rot=bnd["rot4"], niox=mod["niox"],
                     nioy=mod["nioy"], bcU=bnd["bcU"], bcS=bnd["bcS"], evt=mod["elem_vt"], nflag=bnd["nflag"],
                     bckind=bnd["bckind"], eqno=num["eqno"], enodes=mod["elem_nodes"], ennd=mod["elem_nnd"],
                     eflag=mod["elem_flag"], g=params.g, hmin=0.5 * params.dry_limit, vk=params.vk,
                     relaxThdt_UV=r, relaxThdt_H=r)
    n = num["neq"]
    ptr = np.zeros(n + 1, np.int64)
    ptr[1:] = np.cumsum(num["width"])
    A, B = oracle.assemble(m, ptr, np.ascontiguousarray(num["index"], np.int32), np.float64)
    sim.close()
    return A, B


def test_lake_at_rest_has_zero_residual():
    mesh = meshgen.channel(nx=20, ny=4, length=400.0, width=50.0, nbumps=6, seed=5, Q=10.0)
    S_lake = float(np.max(mesh.z)) + 2.0
    bcs = [("QINLET", 1, [(0.0, S_lake)]), ("OUTLET", 2, [(S_lake,)])]
    A, B = _system(mesh, Params(), bcs, np.full(mesh.np, S_lake))
    H = S_lake - deck.bed_zor(mesh)
    scale = Params().g * float(np.max(H)) ** 2 * 400.0        # a hydrostatic force times a length
    assert np.max(np.abs(A)) > 0.0
    assert np.max(np.abs(B)) <= 1e-12 * scale, np.max(np.abs(B)) / scale


def test_lake_at_rest_unsteady_and_with_inflow():
    """With the time term the lake stays a solution; an inflow breaks the balance
    only through the inlet rows (specified minus actual discharge)."""
    mesh = meshgen.channel(nx=20, ny=4, length=400.0, width=50.0, nbumps=6, seed=5, Q=10.0)
    S_lake = float(np.max(mesh.z)) + 2.0
    H = S_lake - deck.bed_zor(mesh)
    scale = Params().g * float(np.max(H)) ** 2 * 400.0
    _A, B = _system(mesh, Params(), [("QINLET", 1, [(0.0, S_lake)]), ("OUTLET", 2, [(S_lake,)])],
                    np.full(mesh.np, S_lake), dt=10.0)
    assert np.max(np.abs(B)) <= 1e-12 * scale
    _A, B = _system(mesh, Params(), [("QINLET", 1, [(25.0, S_lake)]), ("OUTLET", 2, [(S_lake,)])],
                    np.full(mesh.np, S_lake))
    nz = np.flatnonzero(np.abs(B) > 1e-9 * scale)
    assert 0 < len(nz) <= 2 * (mesh.meta["ny"] * 2 + 1)           # the inlet nodes' rows only


def test_manning_uniform_flow_has_zero_residual():
    """Uniform flow down a plane slope: depth H, velocity U with g H S0 = cf U^2, where
    cf = areaFact g n^2 / H^0.333333 is the reference's nodal Manning coefficient
    (DoFriction.cpp:87-206) -- U is Manning's H^(2/3) S0^(1/2) / n to 1e-5.  Inlet
    discharge U H W, outlet level H: the assembled residual vanishes to rounding."""
    L, W, slope, Hd = 400.0, 50.0, 0.001, 2.0
    mesh = meshgen.channel(nx=20, ny=4, length=L, width=W, slope=slope, nbumps=0, depth0=Hd)
    p = Params()
    n = mesh.materials[0][1]
    af = float(np.sqrt(1.0 + slope * slope))                 # inclined-element area factor
    U = float(np.sqrt(p.g * Hd * slope / (af * p.g * n * n / Hd ** 0.333333)))
    assert abs(U - Hd ** (2.0 / 3.0) * slope ** 0.5 / n) <= 1e-5 * U
    bcs = [("QINLET", 1, [(U * Hd * W, slope * L + Hd)]), ("OUTLET", 2, [(Hd,)])]
    A, B = _system(mesh, p, bcs, deck.bed_zor(mesh) + Hd, U=np.full(mesh.np, U))
    scale = p.g * Hd * slope * (L / 20.0) * (W / 4.0)         # friction / slope force on one quad
    assert np.max(np.abs(A)) > 0.0
    assert np.max(np.abs(B)) <= 1e-10 * scale, np.max(np.abs(B)) / scale


def _model(mesh, p, S, U, V, relax):
    sim = Simulation(mesh, p, device=RG_DEVICE_NONE)
    sim.set_state(U, V, S)
    sim.dry_rewet_pass()
    s0 = sim.get_state()
    en = np.ascontiguousarray(mesh.elems, np.int32)
    cf = np.zeros(mesh.np)
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    elem_n = np.full(len(en), mesh.materials[0][1])
    af = _area_factors(mesh)
    oracle.lib().orc_friction(C.c_int(mesh.np), C.c_int(len(en)), P(en), P(np.full(len(en), 6, np.int32)),
                              P(elem_n), P(af), P(s0["U"]), P(s0["V"]), P(s0["S"]), P(s0["z"]),
                              C.c_double(0.5 * p.dry_limit), C.c_double(p.g), P(cf))
    sim.prepare_iteration(0.0, cf)
    st, num, bnd, mod = sim.get_state(), sim.numbering(), sim.boundary(), sim.model()
    Z = lambda: np.zeros(mesh.np)        # separate arrays: the model points into each
    m = oracle.Model(x=mesh.x, y=mesh.y, z=st["z"], U=st["U"], V=st["V"], S=st["S"], dUdt=Z(), dVdt=Z(),
                     dSdt=Z(), cf=cf, cfw=Z(), uu=Z(), uv=Z(), vv=Z(), rot=bnd["rot4"], niox=mod["niox"],
                     nioy=mod["nioy"], bcU=bnd["bcU"], bcS=bnd["bcS"], evt=mod["elem_vt"], nflag=bnd["nflag"],
                     bckind=bnd["bckind"], eqno=num["eqno"], enodes=mod["elem_nodes"], ennd=mod["elem_nnd"],
                     eflag=mod["elem_flag"], g=p.g, hmin=0.5 * p.dry_limit, vk=p.vk, relaxThdt_UV=relax,
                     relaxThdt_H=relax)
    sim.close()
    return m, np.asarray(bnd["nflag"]), np.asarray(mod["elem_nodes"]), np.asarray(mod["elem_nnd"])


def test_element_jacobian_matches_finite_differences():
    """EQS_UVS2D::Region's 15x15 Jacobian (CoefsUVS2D.cpp:740-1060) against central
    differences of its own element residual, on a non-uniform flow over a bumpy bed, for
    interior triangles, steady and with the time term (the state's time derivative moved
    with U, V, S at relaxThdt): every block agrees to 1e-8 of the matrix's largest entry
    when the nodal friction coefficient is held fixed -- the Jacobian is exact apart from
    the friction coefficient's dependence on the depth, which the reference recomputes
    every iteration and does not differentiate."""
    mesh = meshgen.channel(nx=20, ny=4, length=400.0, width=50.0, nbumps=6, seed=5, Q=100.0)
    p = Params()
    x, y = mesh.x, mesh.y
    U = 1.0 + 0.3 * np.sin(x / 50.0) * np.cos(y / 20.0)
    V = 0.2 * np.sin(x / 30.0)
    S = deck.bed_zor(mesh) + 2.0 + 0.1 * np.cos(x / 40.0)
    N_BOUND = 16
    h = 1e-6
    for relax in (0.0, 0.1):
        m, nflag, men, mnnd = _model(mesh, p, S, U, V, relax)
        interior = [e for e in range(len(mnnd)) if mnnd[e] == 6 and not np.any(nflag[men[e]] & N_BOUND)]
        assert len(interior) >= 8
        for e in interior[:8]:
            _ok, K, _f = oracle.coefs(m, e)
            nd = men[e]
            scale = np.max(np.abs(K[:15, :15]))
            for c in range(15):
                var, k = c // 6, c % 6
                if var == 2 and k >= 3:
                    continue                              # S lives on the corners only
                arr, drv = ("U", "dUdt") if var == 0 else (("V", "dVdt") if var == 1 else ("S", "dSdt"))
                fs = []
                for sgn in (1.0, -1.0):
                    m.arrays[arr][nd[k]] += sgn * h
                    m.arrays[drv][nd[k]] += sgn * h * relax
                    fs.append(oracle.coefs(m, e)[2])
                    m.arrays[arr][nd[k]] -= sgn * h
                    m.arrays[drv][nd[k]] -= sgn * h * relax
                fd = -(fs[0] - fs[1]) / (2.0 * h)
                assert np.max(np.abs(K[:15, c] - fd[:15])) <= 1e-8 * scale, (relax, e, c)
