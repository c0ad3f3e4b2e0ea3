"""Writes the golden fixtures of tests/golden -- TEST INFRASTRUCTURE ONLY.

    python tests/golden/make_golden.py

Each fixture stores a small seeded problem and the answers of the reference path on it:
the oracle's restatement of the reference solver (band Cholesky, as the reference's
``cholesky`` algorithm) and, for the Static3D case, the reference's own NSPCG
(``iterative`` algorithm, IC-preconditioned CG from the reference's ``extlib/nspcg``,
compiled into ``oracle/_ref`` by ``make -C oracle ref``) driven to zeta = 1e-12.  The
fixtures are committed; the tests replay them without the reference tree.

Fixtures:
* ``static3d_layered_aniso_12x10x18``: Static3D (therm3d.cpp), anisotropic layers,
  convective top, ORDER_201; Cholesky and NSPCG temperatures, loops, toterr.
* ``static3d_mesa_faces_12x11x16``: an etched mesa (masked mesh) with heat-flux,
  convective and radiative faces in the reference's placement, ORDER_012.
* ``staticcyl_etched_aniso_35x52``: StaticCyl (therm2d.cpp), an etched mesa (masked
  mesh), anisotropic layers, ORDER_01.
* ``static2d_etched_aniso_33x47``: Static2D (therm2d.cpp), an etched mesa, anisotropic
  layers, ORDER_10.
* ``dynamic3d_consistent_12x11x16``: Dynamic3D (femT3d.cpp), consistent capacity,
  theta = 0.75, 2 ns in 0.2 ns steps.
* ``dynamiccyl_lumped_24x30``: DynamicCyl (femT2d.cpp), lumped capacity,
  Crank-Nicolson, k(T) rebuilt every 3 steps, 2 ns in 0.2 ns steps, ORDER_10.
* ``shockley3d_junction_21x19x30``: Shockley3D (electr3d.cpp), a layered junction
  structure, 5 loops, ORDER_102.
* ``thermoelectric3d_19x19x28``: the ThermoElectric3D loop (thermoelectric.py:181-219):
  electrical compute(6), its Joule heat to the thermal problem, thermal compute(1),
  until both errors are within maxerr, ORDER_012.
* ``thermoelectric3d_betaT_19x19x28``: the same loop with a temperature-dependent junction
  beta(T) = 18 (300/T)^1.5, each round's element temperatures fed back into the electrical
  problem (the thermal -> electrical direction of the coupling).
"""
from __future__ import annotations

import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))

import golden_io as G  # noqa: E402
from oracle import dynamic2d as D2  # noqa: E402
from oracle import dynamic3d as D3  # noqa: E402
from oracle import electr3d as E  # noqa: E402
from oracle import fem2d as O2  # noqa: E402
from oracle import fem3d as O  # noqa: E402
from oracle import nspcg as N  # noqa: E402
from plask_gb300 import structures as S  # noqa: E402
from plask_gb300.mesh import RectangularMesh2D  # noqa: E402


def mesa_with_faces(seed, n):
    """Layers etched into a mesa in the top 4 element layers (an EMPTY material around
    it) with heat flux, convection and radiation on several faces."""
    s = S.layered_c0(seed=seed, n=n, power=1e15)
    n_mat = s.k300.size
    s.k300 = np.append(s.k300, 0.026)
    s.p = np.append(s.p, 0.0)
    s.kz_ratio = np.append(s.kz_ratio, 1.0)
    s.hexp = np.append(s.hexp, 0.0)
    s.empty = np.append(s.empty, True)
    ne2 = s.mat.shape[0]
    xm = 0.5 * (s.axes[0][1:] + s.axes[0][:-1])
    ym = 0.5 * (s.axes[1][1:] + s.axes[1][:-1])
    outside = (xm[None, :] > 20.0) | (ym[:, None] > 20.0)
    mat = s.mat.copy()
    for k in range(ne2 - 4, ne2):
        mat[k][outside] = n_mat
    s.mat = mat
    s.heatflux = [("left", -2e3)]
    s.convection = [("top", 80.0, 295.0), ("right", 40.0, 300.0)]
    s.radiation = [("front", 0.7, 310.0), ("top", 0.5, 280.0)]
    return s


def problem2d(s, geometry, order, bc_compat=True, empty_elements="exclude"):
    """oracle.fem2d.Problem2D of a 2D structure with side conditions."""
    mats = O.Materials(s.k300, s.p, s.kz_ratio, s.hexp, s.empty)
    mesh = RectangularMesh2D(*s.axes, ordering=order)

    def place(side):
        return RectangularMesh2D.side(side).mask(mesh)

    return O2.Problem2D(axes=s.axes, mat=s.mat, materials=mats, heat=s.heat, geometry=geometry,
                        temperature=[(place(a), v) for a, v in s.temperature],
                        heatflux=[(place(a), v) for a, v in s.heatflux],
                        convection=[(place(a), h, t) for a, h, t in s.convection],
                        radiation=[(place(a), e, t) for a, e, t in s.radiation],
                        order=order, inittemp=s.inittemp, maxerr=s.maxerr, empty_elements=empty_elements,
                        bc_compat=bc_compat)


def records(rec):
    return [[r.loop, r.maxT, r.err] for r in rec]


def static3d_layered():
    s = S.layered_c1(seed=5, n=(12, 10, 18))
    order = "201"
    p = O.from_structure(s, order=order)
    T, toterr, rec = O.compute(p)
    Tn, toterr_n, rec_n, iters = N.compute_iterative(p, zeta=1e-12, maxit=5000)
    arr, meta = G.pack_thermal(s)
    arr.update(T_cholesky=T, T_nspcg=Tn)
    meta.update(kind="static3d", order=order, empty_elements="exclude", toterr=toterr, records=records(rec),
                nspcg={"zeta": 1e-12, "toterr": toterr_n, "records": records(rec_n), "iterations": iters})
    G.save("static3d_layered_aniso_12x10x18", arr, meta)
    return float(np.max(np.abs(T - Tn)))


def static3d_mesa():
    s = mesa_with_faces(seed=12, n=(12, 11, 16))
    order = "012"
    p = O.from_structure(s, order=order)
    T, toterr, rec = O.compute(p)
    arr, meta = G.pack_thermal(s)
    arr.update(T_cholesky=T)
    meta.update(kind="static3d", order=order, empty_elements="exclude", toterr=toterr, records=records(rec))
    G.save("static3d_mesa_faces_12x11x16", arr, meta)


def staticcyl():
    s = S.layered_2d(seed=22, n=(35, 52), etch=True, anisotropic=True)
    order = "01"
    p = problem2d(s, "cylindrical", order)
    T, toterr, rec = O2.compute(p)
    arr, meta = G.pack_thermal(s)
    arr.update(T_cholesky=T)
    meta.update(kind="static2d", geometry="cylindrical", order=order, bc_compat=True, empty_elements="exclude",
                toterr=toterr, records=records(rec))
    G.save("staticcyl_etched_aniso_35x52", arr, meta)


def static2d():
    s = S.layered_2d(seed=12, n=(33, 47), etch=True, anisotropic=True)
    order = "10"
    p = problem2d(s, "cartesian", order)
    T, toterr, rec = O2.compute(p)
    arr, meta = G.pack_thermal(s)
    arr.update(T_cholesky=T)
    meta.update(kind="static2d", geometry="cartesian", order=order, bc_compat=True, empty_elements="exclude",
                toterr=toterr, records=records(rec))
    G.save("static2d_etched_aniso_33x47", arr, meta)


def dynamiccyl():
    s = S.layered_2d(seed=73, n=(24, 30))
    s.heatflux, s.convection, s.radiation = [], [], []
    rng = np.random.default_rng(73)
    cp = rng.uniform(300.0, 900.0, s.k300.size)
    dens = rng.uniform(2000.0, 7000.0, s.k300.size)
    order = "10"
    p = problem2d(s, "cylindrical", order)
    T, elaps, steps = D2.compute(p, 2.0, cp, dens, timestep=0.2, theta=0.5, lumping=True, rebuildfreq=3)
    node_id, _ = O2.masked_numbering(p)
    arr, meta = G.pack_thermal(s)
    arr.update(T_direct=O2.to_full(p, node_id, T, fill=np.nan), cp=cp, dens=dens)
    meta.update(kind="dynamic2d", geometry="cylindrical", order=order, bc_compat=True, empty_elements="exclude",
                time=2.0, timestep=0.2, theta=0.5, lumping=True, rebuildfreq=3, elapsed=elaps, steps=steps)
    G.save("dynamiccyl_lumped_24x30", arr, meta)


def dynamic3d():
    s = S.layered_c0(seed=5, n=(12, 11, 16))
    rng = np.random.default_rng(5 + 77)
    cp = rng.uniform(300.0, 900.0, s.k300.size)
    dens = rng.uniform(2000.0, 7000.0, s.k300.size)
    order = "201"
    p = O.from_structure(s, order=order, empty_elements="include")
    T, elaps, steps = D3.compute(p, 2.0, cp, dens, timestep=0.2, theta=0.75, lumping=False)
    node_id, _ = O.masked_numbering(p)
    arr, meta = G.pack_thermal(s)
    arr.update(T_direct=O.to_full(p, node_id, T), cp=cp, dens=dens)
    meta.update(kind="dynamic3d", order=order, empty_elements="include", time=2.0, timestep=0.2, theta=0.75,
                lumping=False, rebuildfreq=0, elapsed=elaps, steps=steps)
    G.save("dynamic3d_consistent_12x11x16", arr, meta)


def shockley3d():
    s = S.shockley_c4(seed=4001, n=(21, 19, 30), voltage=1.9)
    s.thermal = None
    order, loops = "102", 5
    p = E.from_structure(s, order=order, convergence="fast")
    V, conds, toterr, rec = E.compute(p, loops=loops)
    arr, meta = G.pack_elec(s)
    arr.update(V_cholesky=V)
    meta.update(kind="shockley3d", order=order, convergence="fast", loops=loops, toterr=toterr,
                total_current=4 * E.total_current(p, V, conds))
    G.save("shockley3d_junction_21x19x30", arr, meta)


def thermoelectric3d():
    s = S.shockley_c4(seed=4003, n=(19, 19, 28), voltage=2.1)
    order, tfreq = "012", 6
    p = E.from_structure(s, order=order)
    tp = O.from_structure(s.thermal, order=order)
    state, T, rounds = {}, None, []
    ve, tt = 2 * s.maxerr, 2 * tp.maxerr
    while tt > tp.maxerr or ve > s.maxerr:
        V, conds, ve, _ = E.compute(p, loops=tfreq, state=state)
        tp.heat = E.heat(p, V, conds)
        T, tt, _ = O.compute(tp, loops=1, T=T)
        rounds.append([ve, tt])
    arr, meta = G.pack_elec(s)
    arr.update(T_cholesky=T, V_cholesky=V)
    meta.update(kind="thermoelectric3d", order=order, tfreq=tfreq, rounds=rounds)
    G.save("thermoelectric3d_19x19x28", arr, meta)


def element_mean(T):
    """Element-average temperatures (the 8-node mean) of a canonical node field."""
    return 0.125 * (T[:-1, :-1, :-1] + T[:-1, :-1, 1:] + T[:-1, 1:, :-1] + T[:-1, 1:, 1:]
                    + T[1:, :-1, :-1] + T[1:, :-1, 1:] + T[1:, 1:, :-1] + T[1:, 1:, 1:])


BETA_T = (18.0, 1.5)  # beta(T) = 18 (300/T)^1.5 1/V


def beta_of_t(b0, bp):
    return lambda T: b0 * (300.0 / T) ** bp


def thermoelectric3d_beta_t():
    """The ThermoElectric3D loop with a temperature-dependent junction beta(T): each round the
    electrical problem reads the element temperatures of the last thermal solve, as the
    reference's electrical solver reads its inTemperature receiver (thermoelectric.py:209-211,
    electr3d.cpp:203-237)."""
    s = S.shockley_c4(seed=4005, n=(19, 19, 28), voltage=2.2)
    order, tfreq = "012", 6
    packed_beta = list(s.beta)
    s.beta = [beta_of_t(*BETA_T)]
    p = E.from_structure(s, order=order)
    tp = O.from_structure(s.thermal, order=order)
    state, T, rounds = {}, None, []
    ve, tt = 2 * s.maxerr, 2 * tp.maxerr
    while tt > tp.maxerr or ve > s.maxerr:
        p.temperature = np.full(tuple(n - 1 for n in tp.shape), tp.inittemp) if T is None else element_mean(T)
        V, conds, ve, _ = E.compute(p, loops=tfreq, state=state)
        tp.heat = E.heat(p, V, conds)
        T, tt, _ = O.compute(tp, loops=1, T=T)
        rounds.append([ve, tt])
    s.beta = packed_beta
    arr, meta = G.pack_elec(s)
    arr.update(T_cholesky=T, V_cholesky=V)
    meta.update(kind="thermoelectric3d", order=order, tfreq=tfreq, rounds=rounds, beta_T=list(BETA_T))
    G.save("thermoelectric3d_betaT_19x19x28", arr, meta)


def main():
    if not N.available():
        raise SystemExit("oracle/_ref/libnspcg_ref.so is not built: make -C oracle ref (needs the reference tree)")
    d = static3d_layered()
    print(f"static3d layered: Cholesky vs the reference's NSPCG max |dT| = {d:.3e} K")
    static3d_mesa()
    staticcyl()
    static2d()
    dynamic3d()
    dynamiccyl()
    shockley3d()
    thermoelectric3d()
    thermoelectric3d_beta_t()
    for n in G.names():
        print(n, (HERE / f"{n}.npz").stat().st_size, "bytes")


if __name__ == "__main__":
    main()
