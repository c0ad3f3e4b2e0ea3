"""Golden fixtures -- TEST INFRASTRUCTURE ONLY: (de)serialisation of the seeded structures
and of the problems built from them, shared by ``make_golden.py`` (which writes the
fixtures) and ``tests/test_regression_golden.py`` (which replays them on the oracle and the GPU).

A fixture is one ``.npz`` file holding the solver inputs (axes, element materials, the
material table, heat, boundary conditions as mesh sides or node masks) and the outputs
the reference path produces on them, with a JSON ``meta`` entry for the scalars and the
lists.  Nothing here regenerates a structure from its seed: the stored arrays are the
inputs, so a fixture keeps pinning the same problem if a generator changes.
"""
from __future__ import annotations

import json
import pathlib

import numpy as np

from plask_gb300 import structures as S

HERE = pathlib.Path(__file__).resolve().parent

_MATERIAL_FIELDS = ("k300", "p", "kz_ratio", "hexp", "empty")
_ELEC_FIELDS = ("cond_xy", "cond_z", "eps", "empty", "noheat")


def pack_thermal(s, prefix=""):
    """Arrays and JSON-able metadata of a :class:`plask_gb300.structures.Structure`."""
    arr = {f"{prefix}mat": np.asarray(s.mat, np.int32), f"{prefix}heat": np.asarray(s.heat, np.float64)}
    for d, a in enumerate(s.axes):
        arr[f"{prefix}axis{d}"] = np.asarray(a, np.float64)
    for f in _MATERIAL_FIELDS:
        arr[f"{prefix}{f}"] = np.asarray(getattr(s, f))
    meta = {"dims": len(s.axes), "temperature": [list(c) for c in s.temperature],
            "heatflux": [list(c) for c in s.heatflux], "convection": [list(c) for c in s.convection],
            "radiation": [list(c) for c in s.radiation], "maxerr": s.maxerr, "inittemp": s.inittemp,
            "name": s.name}
    return arr, meta


def unpack_thermal(data, meta, prefix=""):
    axes = tuple(np.array(data[f"{prefix}axis{d}"]) for d in range(meta["dims"]))
    kw = {f: np.array(data[f"{prefix}{f}"]) for f in _MATERIAL_FIELDS}
    return S.Structure(axes=axes, mat=np.array(data[f"{prefix}mat"]), heat=np.array(data[f"{prefix}heat"]),
                       temperature=[tuple(c) for c in meta["temperature"]],
                       heatflux=[tuple(c) for c in meta["heatflux"]],
                       convection=[tuple(c) for c in meta["convection"]],
                       radiation=[tuple(c) for c in meta["radiation"]], maxerr=meta["maxerr"],
                       inittemp=meta["inittemp"], name=meta["name"], **kw)


def pack_elec(s):
    """Arrays and metadata of a :class:`plask_gb300.structures.ElecStructure` (with its
    thermal structure, when it has one)."""
    arr = {"mat": np.asarray(s.mat, np.int32), "junction": np.asarray(s.junction, np.int32)}
    for d, a in enumerate(s.axes):
        arr[f"axis{d}"] = np.asarray(a, np.float64)
    for f in _ELEC_FIELDS:
        arr[f] = np.asarray(getattr(s, f))
    for i, (mask, _) in enumerate(s.voltage):
        arr[f"voltage_mask{i}"] = np.asarray(mask, bool)
    meta = {"beta": list(map(float, s.beta)), "js": list(map(float, s.js)),
            "voltage": [float(v) for _, v in s.voltage], "symmetric": list(s.symmetric), "maxerr": s.maxerr,
            "name": s.name, "thermal": None}
    if s.thermal is not None:
        ta, tm = pack_thermal(s.thermal, prefix="thermal_")
        arr.update(ta)
        meta["thermal"] = tm
    return arr, meta


def unpack_elec(data, meta):
    axes = tuple(np.array(data[f"axis{d}"]) for d in range(3))
    kw = {f: np.array(data[f]) for f in _ELEC_FIELDS}
    voltage = [(np.array(data[f"voltage_mask{i}"]), v) for i, v in enumerate(meta["voltage"])]
    thermal = None if meta["thermal"] is None else unpack_thermal(data, meta["thermal"], prefix="thermal_")
    return S.ElecStructure(axes=axes, mat=np.array(data["mat"]), junction=np.array(data["junction"]),
                           beta=list(meta["beta"]), js=list(meta["js"]), voltage=voltage,
                           symmetric=tuple(meta["symmetric"]), maxerr=meta["maxerr"], thermal=thermal,
                           name=meta["name"], **kw)


def save(name, arrays, meta):
    np.savez_compressed(HERE / f"{name}.npz", meta=np.array(json.dumps(meta, sort_keys=True)), **arrays)


def load(name):
    with np.load(HERE / f"{name}.npz") as f:
        data = {k: np.array(f[k]) for k in f.files}
    meta = json.loads(str(data.pop("meta")))
    return data, meta


# fixtures that store answers at a subset of nodes of a regenerated structure instead of the
# inputs (make_golden_c1.py); replayed by their own tests, not by the generic replay
SUBSET_FIXTURES = ("static3d_layered_c1_128x128x200_nspcg",)


def names():
    return sorted(p.stem for p in HERE.glob("*.npz") if p.stem not in SUBSET_FIXTURES)
