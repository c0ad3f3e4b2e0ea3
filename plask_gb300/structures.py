"""Seeded synthetic layered structures for the Static3D thermal solver.

PLaSK builds these inputs from a geometry tree and a mesh generator; here they
are generated directly as what the FEM path consumes: three rectilinear axes
(micrometres), one material id per element, a small material table with
k(T) = k300 * (300/T)**p, one heat density per element (W/m^3) and boundary
conditions on named mesh sides.

Every generator takes a ``seed`` and draws from ``numpy.random.default_rng``
(PCG64), so a seed names a structure exactly.

Lateral refinement: the lateral axes span 0..50 um and are refined
geometrically toward x = y = 0.  With 40 nodes the cell ratio is 1.15; for
other node counts the ratio is ``1.15 ** (39 / (n - 1))`` so that the largest
to smallest cell ratio (1.15**39 ~ 233) -- the grading of the 40-node mesh --
is kept when the mesh is scaled.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

LATERAL_SPAN = 50.0
SUBSTRATE = 150.0


@dataclasses.dataclass
class Structure:
    """Everything one Static3D solve needs, in plain arrays.

    * ``axes``: (axis0, axis1, axis2) node coordinates in um, axis 2 vertical
    * ``mat``: int32 element material ids, shape (n2-1, n1-1, n0-1), axis 0 fastest
    * ``k300``, ``p``, ``kz_ratio``, ``hexp``, ``empty``: per-material model
      k_xy(T, h) = k300 * (300/T)**p * h**hexp,  k_z = kz_ratio * k_xy
    * ``heat``: element heat density in W/m^3, same shape as ``mat``
    * ``temperature``/``heatflux``/``convection``/``radiation``: boundary
      conditions as (side, values...) with side one of
      "bottom", "top", "back", "front", "left", "right"
    * ``ktables``: tabulated k(T) replacing the power law of some materials
    """

    axes: tuple
    mat: np.ndarray
    k300: np.ndarray
    p: np.ndarray
    kz_ratio: np.ndarray
    hexp: np.ndarray
    empty: np.ndarray
    heat: np.ndarray
    temperature: list = dataclasses.field(default_factory=list)
    heatflux: list = dataclasses.field(default_factory=list)
    convection: list = dataclasses.field(default_factory=list)
    radiation: list = dataclasses.field(default_factory=list)
    maxerr: float = 0.05
    inittemp: float = 300.0
    name: str = ""
    # tabulated k(T) of some materials: {material id: (T, k_xy, k_z or None)}
    ktables: dict | None = None

    @property
    def shape(self):
        """Node-grid shape (n2, n1, n0)."""
        return tuple(len(a) for a in self.axes[::-1])

    @property
    def nodes(self):
        return int(np.prod(self.shape))


def side_mask(shape, side):
    """Boolean node mask (n2, n1, n0) of a mesh side.

    Names follow PLaSK's 3D rectangular mesh boundaries
    (plask/mesh/rectilinear3d.cpp:158-190): back/front = axis 0 lo/hi,
    left/right = axis 1 lo/hi, bottom/top = axis 2 lo/hi.
    """
    m = np.zeros(shape, bool)
    if side == "bottom":
        m[0] = True
    elif side == "top":
        m[-1] = True
    elif side == "left":
        m[:, 0] = True
    elif side == "right":
        m[:, -1] = True
    elif side == "back":
        m[:, :, 0] = True
    elif side == "front":
        m[:, :, -1] = True
    else:
        raise ValueError(f"unknown side {side!r}")
    return m


def graded_axis(n, span=LATERAL_SPAN, ratio40=1.15):
    """n nodes on [0, span] with cells growing geometrically away from 0."""
    if n < 2:
        raise ValueError("an axis needs at least 2 nodes")
    r = ratio40 ** (39.0 / (n - 1))
    h = r ** np.arange(n - 1)
    h *= span / h.sum()
    x = np.concatenate([[0.0], np.cumsum(h)])
    x[-1] = span
    return x


def _geometric_fill(length, cells, first):
    """Cells on a segment of given length, growing from ``first`` by a common ratio."""
    if cells * first >= length:
        return np.full(cells, length / cells)
    lo, hi = 1.0, 2.0
    while first * (hi ** cells - 1) / (hi - 1) < length:
        hi *= 2
    for _ in range(200):
        q = 0.5 * (lo + hi)
        if first * (q ** cells - 1) / (q - 1) < length:
            lo = q
        else:
            hi = q
    h = first * q ** np.arange(cells)
    return h * (length / h.sum())


def _allocate(weights, total, minimum=1):
    """Largest-remainder allocation of ``total`` cells with a per-entry minimum."""
    n = len(weights)
    base = np.full(n, minimum, np.int64)
    rest = total - base.sum()
    if rest < 0:
        raise ValueError("not enough cells for the layers")
    w = np.asarray(weights, np.float64)
    share = rest * w / w.sum()
    extra = np.floor(share).astype(np.int64)
    left = rest - extra.sum()
    order = np.argsort(-(share - extra), kind="stable")
    extra[order[:left]] += 1
    return base + extra


def vertical_axis(thicknesses, n_nodes, substrate=SUBSTRATE, substrate_share=0.25):
    """Node coordinates: a graded substrate under uniformly meshed layers.

    Returns (z, layer_of_element) where layer 0 is the substrate and layer i >= 1
    the i-th epitaxial layer from the bottom.
    """
    cells = n_nodes - 1
    nl = len(thicknesses)
    n_sub = max(1, int(round(substrate_share * cells)))
    per_layer = _allocate(np.sqrt(np.asarray(thicknesses)), cells - n_sub)
    hs = []
    layer = []
    first = 2.0 * thicknesses[0] / per_layer[0]
    sub = _geometric_fill(substrate, n_sub, first)[::-1]
    hs.append(sub)
    layer.append(np.zeros(n_sub, np.int64))
    for i, (t, c) in enumerate(zip(thicknesses, per_layer)):
        hs.append(np.full(c, t / c))
        layer.append(np.full(c, i + 1, np.int64))
    h = np.concatenate(hs)
    z = np.concatenate([[0.0], np.cumsum(h)])
    return z, np.concatenate(layer)


def _layered(rng, n, n_layers, active_thickness, anisotropic, source_radius, power):
    thick = np.exp(rng.uniform(math.log(0.05), math.log(3.0), n_layers))
    active = int(rng.integers(n_layers // 3, max(n_layers // 3 + 1, 2 * n_layers // 3)))
    thick[active] = active_thickness
    x0 = graded_axis(n[0])
    x1 = graded_axis(n[1])
    z, layer_of = vertical_axis(thick, n[2])
    n_mat = n_layers + 1
    k300 = np.exp(rng.uniform(math.log(1.0), math.log(150.0), n_mat))
    p = rng.uniform(0.5, 1.5, n_mat)
    kz = rng.uniform(0.5, 1.0, n_mat) if anisotropic else np.ones(n_mat)
    mat = np.broadcast_to(layer_of[:, None, None], (n[2] - 1, n[1] - 1, n[0] - 1)).astype(np.int32)
    xm = 0.5 * (x0[1:] + x0[:-1])
    ym = 0.5 * (x1[1:] + x1[:-1])
    r2 = xm[None, :] ** 2 + ym[:, None] ** 2
    disc = r2 <= source_radius ** 2
    heat = np.zeros(mat.shape)
    heat[layer_of == active + 1] = np.where(disc, power, 0.0)[None]
    return dict(axes=(x0, x1, z), mat=np.ascontiguousarray(mat), k300=k300, p=p, kz_ratio=kz,
                hexp=np.zeros(n_mat), empty=np.zeros(n_mat, bool), heat=heat)


def _fit_layers(n, n_layers):
    """Number of layers that fits n[2] - 1 vertical cells next to the substrate."""
    cells = n[2] - 1
    return max(1, min(n_layers, cells - max(1, int(round(0.25 * cells)))))


def layered_c0(seed=0, n=(40, 40, 60), power=1e16, n_layers=12):
    """Plain Static3D case: 12 layers on a 150 um substrate, isotropic k(T),
    a 4 um-radius disc source at 1e16 W/m^3 in a 0.1 um layer, bottom at 300 K.

    Meshes with fewer than ``n_layers + 2`` vertical cells get fewer layers.  At the
    full 40x40x60 size seed 0 runs away thermally (k falls as (300/T)^p: max T 1339,
    3890, 9406, 20545 K over the first four outer loops, for the model as for the
    reference); seeds 1 to 5 settle at 424-716 K."""
    rng = np.random.default_rng(seed)
    d = _layered(rng, n, _fit_layers(n, n_layers), 0.1, False, 4.0, power)
    return Structure(**d, temperature=[("bottom", 300.0)], name=f"layered-{n[0]}x{n[1]}x{n[2]}-s{seed}")


def layered_c1(seed=1000, n=(128, 128, 200), power=1e16, n_layers=12):
    """The scaled case: same generator at 128x128x200 nodes with lateral
    anisotropy k_z/k_xy ~ U[0.5, 1] and a convective top (h = 10 W/m^2K, 300 K)."""
    rng = np.random.default_rng(seed)
    d = _layered(rng, n, _fit_layers(n, n_layers), 0.1, True, 4.0, power)
    return Structure(**d, temperature=[("bottom", 300.0)], convection=[("top", 10.0, 300.0)],
                     name=f"layered-aniso-{n[0]}x{n[1]}x{n[2]}-s{seed}")


def learned_c2(seed=2000, n=None, oxide_factor=1e-2):
    """Structures of the learned preconditioner's configuration: 8..40 random layers on the
    150 um substrate (thickness log-uniform in 0.05..3 um, k300 log-uniform in 1..150 W/mK,
    p in 0.5..1.5, k_z / k_xy in 0.5..1), a cylindrical mesa of radius 5..30 um about
    x = y = 0 etched through the upper part of the layers (EMPTY outside it: a masked mesh),
    an annular oxide aperture inside the mesa -- one layer whose material between the
    aperture radius and the mesa radius has ``oxide_factor`` times its host's conductivity
    (the reference's HollowCylinder, plask/geometry/cylinder.hpp:95), a contrast of up to
    1e3 against the other layers -- and 1..3 Gaussian heat blobs in the aperture, their total
    power scaled to a temperature rise of the order of 40 K.  Grids
    of 96..160 nodes per axis (``n`` overrides), multiples of 4; bottom at 300 K, the other
    faces adiabatic, the quarter device mirrored in x and y."""
    rng = np.random.default_rng(seed)
    if n is None:
        n = tuple(int(4 * round(rng.uniform(96, 160) / 4)) for _ in range(3))
    n_layers = min(int(rng.integers(8, 41)), _fit_layers(n, 40))
    thick = np.exp(rng.uniform(math.log(0.05), math.log(3.0), n_layers))
    x0 = graded_axis(n[0])
    x1 = graded_axis(n[1])
    z, layer_of = vertical_axis(thick, n[2])
    n_lay = n_layers + 1  # substrate + layers
    k300 = np.exp(rng.uniform(math.log(1.0), math.log(150.0), n_lay))
    pexp = rng.uniform(0.5, 1.5, n_lay)
    kz = rng.uniform(0.5, 1.0, n_lay)
    mesa_r = rng.uniform(5.0, 30.0)
    first_etched = int(rng.integers(max(1, n_layers // 2), n_layers)) + 1  # layer ids first_etched..n_layers
    ox_layer = int(rng.integers(first_etched, n_layers + 1))
    ap_r = rng.uniform(0.2, 0.7) * mesa_r
    ox_id, empty_id = n_lay, n_lay + 1
    k300 = np.append(k300, [k300[ox_layer] * oxide_factor, 0.026])
    pexp = np.append(pexp, [pexp[ox_layer], 0.0])
    kz = np.append(kz, [kz[ox_layer], 1.0])
    empty = np.zeros(n_lay + 2, bool)
    empty[empty_id] = True
    xm = 0.5 * (x0[1:] + x0[:-1])
    ym = 0.5 * (x1[1:] + x1[:-1])
    zm = 0.5 * (z[1:] + z[:-1])
    r = np.sqrt(xm[None, :] ** 2 + ym[:, None] ** 2)  # (n1 - 1, n0 - 1)
    mat = np.broadcast_to(layer_of[:, None, None], (n[2] - 1, n[1] - 1, n[0] - 1)).astype(np.int32).copy()
    etched = layer_of >= first_etched
    mat[etched] = np.where(r > mesa_r, empty_id, mat[etched])
    ox = layer_of == ox_layer
    mat[ox] = np.where((r > ap_r) & (r <= mesa_r), ox_id, mat[ox])
    # heat: 1..3 Gaussian blobs near the aperture layer, inside the aperture
    heat = np.zeros(mat.shape)
    z_ox = 0.5 * (z[np.flatnonzero(ox)[0]] + z[np.flatnonzero(ox)[-1] + 1])
    for _ in range(int(rng.integers(1, 4))):
        ang = rng.uniform(0.0, 0.5 * math.pi)
        rad = rng.uniform(0.0, 0.8) * ap_r
        cx, cy = rad * math.cos(ang), rad * math.sin(ang)
        cz = z_ox + rng.uniform(-1.0, 1.0)
        sxy, sz = rng.uniform(1.0, 4.0), rng.uniform(0.2, 1.0)
        peak = rng.uniform(0.5, 2.0)  # relative weights; the total is scaled below
        g = np.exp(-((xm[None, None, :] - cx) ** 2 + (ym[None, :, None] - cy) ** 2) / (2 * sxy ** 2)
                   - (zm[:, None, None] - cz) ** 2 / (2 * sz ** 2))
        heat += peak * g
    heat[mat == empty_id] = 0.0
    # total power of the quarter device scaled so that the heat would raise a half-space of the
    # weaker of the substrate and the blobs' host layer by about 40 K at 300 K through a 4 um
    # disc (dT = P / (pi k r) for the full disc: P_quarter = dT pi k r / 4), which keeps the
    # k(T) loop away from thermal runaway whatever the drawn conductivities
    vol = (np.diff(z)[:, None, None] * np.diff(x1)[None, :, None] * np.diff(x0)[None, None, :]) * 1e-18
    k_weak = min(k300[0], k300[ox_layer])
    target = 40.0 * math.pi * k_weak * 4e-6 / 4.0
    total = float((heat * vol).sum())
    if total > 0:
        heat *= target / total
    return Structure(axes=(x0, x1, z), mat=np.ascontiguousarray(mat), k300=k300, p=pexp, kz_ratio=kz,
                     hexp=np.zeros(k300.size), empty=empty, heat=heat, temperature=[("bottom", 300.0)],
                     name=f"learned_c2-{seed}")


def sweep_c3(seed=3000, count=256, lo=32, hi=96, power=(1e15, 1e16)):
    """Batched sweep: ``count`` layered structures with per-axis node counts
    uniform in [lo, hi] and source power uniform in ``power`` W/m^3.

    The default power range stops at 1e16 W/m^3: above a few 1e16 the k(T) =
    k300 (300/T)^p layers of this generator run away thermally (the outer loop of
    the reference algorithm climbs past 1e4 K or the Cholesky factorisation meets a
    non-positive pivot), so a sweep up to 1e17 would time diverging loops."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = tuple(int(v) for v in rng.integers(lo, hi + 1, 3))
        pw = float(rng.uniform(*power))
        out.append(layered_c0(seed=seed + 1 + i, n=n, power=pw))
    return out


@dataclasses.dataclass
class ElecStructure:
    """Everything one Shockley3D solve needs, in plain arrays.

    * ``axes``: node coordinates in um (axis 2 vertical)
    * ``mat``: int32 element material ids, shape (n2-1, n1-1, n0-1), axis 0 fastest
    * ``cond_xy``, ``cond_z``: per-material conductivity tensor (S/m); ``eps``:
      relative permittivity; ``empty``: EMPTY materials; ``noheat``: no Joule heat
    * ``junction``: element junction number + 1 (0 outside), same shape as ``mat``
    * ``beta`` (1/V), ``js`` (A/m^2): per junction
    * ``voltage``: [(node mask (n2, n1, n0), volts)] in list order
    * ``symmetric``: (axis 0, axis 1) mirror symmetry at the low end, which doubles
      the reference's total current and heat per symmetric direction
    * ``thermal``: the matching Static3D structure of a coupled problem, or None
    """

    axes: tuple
    mat: np.ndarray
    cond_xy: np.ndarray
    cond_z: np.ndarray
    eps: np.ndarray
    empty: np.ndarray
    noheat: np.ndarray
    junction: np.ndarray
    beta: list
    js: list
    voltage: list
    symmetric: tuple = (False, False)
    maxerr: float = 0.05
    thermal: Structure | None = None
    name: str = ""

    @property
    def shape(self):
        return tuple(len(a) for a in self.axes[::-1])

    def element_cond(self):
        """(ne2, ne1, ne0, 2) table conductivities per element."""
        return np.stack([self.cond_xy[self.mat], self.cond_z[self.mat]], axis=-1)


def _divide(points, parts):
    """Every interval between consecutive points split into ``parts`` equal cells."""
    out = [points[0]]
    for a, b in zip(points[:-1], points[1:]):
        out.extend(a + (b - a) * np.arange(1, parts + 1) / parts)
    return np.asarray(out, np.float64)


def shockley_diode(prediv=(3, 3, 2), junction_eps=12.9):
    """A p-n junction between two ideal conductors, 1000 x 1000 um, 0.02 um thick:
    300 um conductor blocks (1e9 S/m) on both sides of the junction and 700 x 700 x 1 um
    contacts at the top (0 V on its top face) and bottom (1 V on its bottom face),
    surrounded by air.  Each interval between object edges is divided into ``prediv``
    equal cells.  With beta = 10 1/V and js = 1 A/m^2 the current is
    1e-9 S js (e^beta - 1) mA with S = 1e6 um^2, and the Joule heat that times 1 V.
    """
    x = _divide([-500.0, -350.0, 350.0, 500.0], prediv[0])
    y = _divide([-500.0, -350.0, 350.0, 500.0], prediv[1])
    zb = [0.0, 1.0, 301.0, 301.02, 601.02, 602.02]
    z = _divide(zb, prediv[2])
    ne = (len(z) - 1, len(y) - 1, len(x) - 1)
    xm, ym, zm = (0.5 * (a[1:] + a[:-1]) for a in (x, y, z))
    mat = np.zeros(ne, np.int32)  # conductor
    in_contact = (np.abs(xm)[None, :] < 350.0) & (np.abs(ym)[:, None] < 350.0)
    for k, zc in enumerate(zm):
        if zc < 1.0 or zc > 601.02:
            mat[k] = np.where(in_contact, 0, 2)
        elif 301.0 < zc < 301.02:
            mat[k] = 1
    junction = (mat == 1).astype(np.int32)
    shape = (len(z), len(y), len(x))
    on_contact = (np.abs(x)[None, :] <= 350.0) & (np.abs(y)[:, None] <= 350.0)
    top = np.zeros(shape, bool)
    top[-1] = on_contact
    bottom = np.zeros(shape, bool)
    bottom[0] = on_contact
    return ElecStructure(axes=(x, y, z), mat=mat, cond_xy=np.array([1e9, 5.0, 0.55e-14]),
                         cond_z=np.array([1e9, 5.0, 0.55e-14]), eps=np.array([1.0, junction_eps, 1.0]),
                         empty=np.array([False, False, True]), noheat=np.zeros(3, bool), junction=junction,
                         beta=[10.0], js=[1.0], voltage=[(top, 0.0), (bottom, 1.0)], maxerr=1e-3,
                         name=f"shockley-diode-{prediv[0]}{prediv[1]}{prediv[2]}")


def shockley_c4(seed=4000, n=(200, 200, 120), voltage=None, n_layers=12, contact_radius=6.0):
    """Coupled thermal-electrical case: the layered generator with a 20 nm junction
    layer (js = 1 A/m^2, beta = 18 1/V), per-layer electrical conductivity log-uniform
    in 1e-1..1e5 S/m, ``voltage`` (uniform in 1.6..2.2 V when None) on a top disc contact
    of radius 6 um at x = y = 0 (a quarter of the device: symmetric in axes 0 and 1)
    and 0 V on the bottom face.  The thermal structure has the bottom at 300 K and no
    heat sources of its own: its heat comes from the electrical solution."""
    rng = np.random.default_rng(seed)
    nl = _fit_layers(n, n_layers)
    d = _layered(rng, n, nl, 0.02, True, 0.0, 0.0)
    x0, x1, z = d["axes"]
    layer_of = d["mat"][:, 0, 0]
    dz = np.diff(z)
    thickness = np.array([dz[layer_of == m].sum() for m in range(nl + 1)])
    thickness[0] = np.inf  # the substrate
    junction_layer = int(np.argmin(np.abs(thickness - 0.02)))
    n_mat = nl + 1
    sigma = np.exp(rng.uniform(math.log(1e-1), math.log(1e5), n_mat))
    volts = float(rng.uniform(1.6, 2.2)) if voltage is None else float(voltage)
    mat = d["mat"]
    junction = (mat == junction_layer).astype(np.int32)
    shape = (len(z), len(x1), len(x0))
    top = np.zeros(shape, bool)
    top[-1] = (x0[None, :] ** 2 + x1[:, None] ** 2) <= contact_radius ** 2
    bottom = np.zeros(shape, bool)
    bottom[0] = True
    thermal = Structure(**d, temperature=[("bottom", 300.0)], name=f"shockley-thermal-{n[0]}x{n[1]}x{n[2]}-s{seed}")
    return ElecStructure(axes=(x0, x1, z), mat=mat, cond_xy=sigma, cond_z=sigma.copy(), eps=np.full(n_mat, 12.0),
                         empty=np.zeros(n_mat, bool), noheat=np.zeros(n_mat, bool), junction=junction, beta=[18.0],
                         js=[1.0], voltage=[(top, volts), (bottom, 0.0)], symmetric=(True, True), maxerr=0.1,
                         thermal=thermal, name=f"shockley-{n[0]}x{n[1]}x{n[2]}-s{seed}")


def layered_2d(seed=0, n=(60, 80), power=1e15, n_layers=10, etch=False, anisotropic=False):
    """2D layered structure for Static2D / StaticCyl: the 3D generator's vertical stack on
    a 0..50 um horizontal axis refined toward 0 (the axis or the symmetry plane), a
    source within 4 um of it in a 0.1 um layer, bottom at 300 K.  The default power is a
    tenth of the 3D generator's: a 2D strip source (infinite along the depth) heats far
    more than a disc, and at 1e16 W/m^3 the k(T) layers run away thermally.

    ``etch``: the layers above the active one are removed beyond x = 15 um (an EMPTY
    material there, a mesa), which exercises the masked mesh.  ``anisotropic``: k_1/k_0
    ~ U[0.5, 1] per material.  Axes are (axis0, axis1), ``mat``/``heat`` of shape
    (n1-1, n0-1), boundary sides "left", "right", "bottom", "top"."""
    rng = np.random.default_rng(seed)
    n_layers = max(1, min(n_layers, (n[1] - 1) - max(1, int(round(0.25 * (n[1] - 1))))))
    thick = np.exp(rng.uniform(math.log(0.05), math.log(3.0), n_layers))
    active = int(rng.integers(n_layers // 3, max(n_layers // 3 + 1, 2 * n_layers // 3)))
    thick[active] = 0.1
    x0 = graded_axis(n[0])
    y, layer_of = vertical_axis(thick, n[1])
    n_mat = n_layers + 1
    k300 = np.exp(rng.uniform(math.log(1.0), math.log(150.0), n_mat))
    p = rng.uniform(0.5, 1.5, n_mat)
    kz = rng.uniform(0.5, 1.0, n_mat) if anisotropic else np.ones(n_mat)
    mat = np.broadcast_to(layer_of[:, None], (n[1] - 1, n[0] - 1)).astype(np.int32).copy()
    xm = 0.5 * (x0[1:] + x0[:-1])
    empty = np.zeros(n_mat, bool)
    if etch:
        k300 = np.append(k300, 0.026)
        p = np.append(p, 0.0)
        kz = np.append(kz, 1.0)
        empty = np.append(empty, True)
        mat[(layer_of > active + 1)[:, None] & (xm > 15.0)[None, :]] = n_mat
        n_mat += 1
    heat = np.zeros(mat.shape)
    heat[layer_of == active + 1] = np.where(np.abs(xm) <= 4.0, power, 0.0)[None]
    return Structure(axes=(x0, y), mat=np.ascontiguousarray(mat), k300=k300, p=p, kz_ratio=kz,
                     hexp=np.zeros(n_mat), empty=empty, heat=heat, temperature=[("bottom", 300.0)],
                     name=f"layered2d-{n[0]}x{n[1]}-s{seed}")
