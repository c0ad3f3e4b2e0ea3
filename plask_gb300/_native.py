"""ctypes binding of the native library ``libplgpu_fem3d.so`` (include/plgpu_fem3d.h,
plgpu_fem2d.h, plgpu_elec3d.h, plgpu_unet.h).

The library is the only compute path: importing this module fails loudly when
it is missing or cannot be loaded, and every call checks the returned status
and raises with the handle's error text.
"""
from __future__ import annotations

import ctypes as C
import pathlib

import numpy as np

_LIB_PATH = pathlib.Path(__file__).resolve().parent / "lib" / "libplgpu_fem3d.so"

OK = 0
ERR_ARG, ERR_CUDA, ERR_NOT_SPD, ERR_NOCONV, ERR_STATE, ERR_NONFINITE = -1, -2, -3, -4, -5, -6

ORDERS = {"012": 0, "021": 1, "102": 2, "120": 3, "201": 4, "210": 5}
BC_TEMPERATURE, BC_HEATFLUX, BC_CONVECTION, BC_RADIATION = 0, 1, 2, 3
ALGORITHMS = {"cholesky": 0, "gauss": 1, "iterative": 2, "gpu-pcg": 3, "gpu-mixed": 4, "gpu-learned": 5}
NOCONV = {"error": 0, "warning": 1, "continue": 2}
EMPTY = {"default": 0, "exclude": 1, "excluded": 1, "include": 2, "included": 2}
NORMS = {"scaled": 0, "plain": 1}
ORDERS2D = {"10": 0, "01": 1}
GEOMETRY2D = {"cartesian": 1, "cylindrical": 2}


class Stats(C.Structure):
    _fields_ = [
        ("loops", C.c_int),
        ("total_loops", C.c_int),
        ("inner_iterations", C.c_int),
        ("refinements", C.c_int),
        ("converged", C.c_int),
        ("fallbacks", C.c_int),
        ("err", C.c_double),
        ("toterr", C.c_double),
        ("max_t", C.c_double),
        ("last_rel_residual", C.c_double),
        ("solve_ms", C.c_double),
        ("total_ms", C.c_double),
        ("kernel_launches", C.c_longlong),
        ("learned_iterations", C.c_int),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


LOG_CB = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_char_p)

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)
_up = C.POINTER(C.c_uint8)
_h = C.c_void_p

# name -> (restype, argtypes); every entry point declared in include/plgpu_fem3d.h
SIGNATURES = {
    "plgpu_fem3d_create": (C.c_int, [_dp, C.c_int, _dp, C.c_int, _dp, C.c_int, C.c_int, C.POINTER(_h)]),
    "plgpu_fem3d_destroy": (C.c_int, [_h]),
    "plgpu_fem3d_last_error": (C.c_char_p, [_h]),
    "plgpu_fem3d_set_materials": (C.c_int, [_h, C.c_int, _dp, _dp, _dp, _dp, _up]),
    "plgpu_fem3d_set_elements": (C.c_int, [_h, _ip, _dp, _dp]),
    "plgpu_fem3d_set_heat": (C.c_int, [_h, _dp]),
    "plgpu_fem3d_clear_bc": (C.c_int, [_h, C.c_int]),
    "plgpu_fem3d_add_bc": (C.c_int, [_h, C.c_int, _lp, C.c_size_t, C.c_double, C.c_double]),
    "plgpu_fem3d_set_solver": (C.c_int, [_h, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int]),
    "plgpu_fem3d_set_loop": (C.c_int, [_h, C.c_double, C.c_double]),
    "plgpu_fem3d_set_residual_norm": (C.c_int, [_h, C.c_int]),
    "plgpu_fem3d_set_dynamic": (C.c_int, [_h, _dp, _dp, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int]),
    "plgpu_fem3d_compute_dynamic": (C.c_int, [_h, C.c_double, _dp, C.POINTER(Stats)]),
    "plgpu_fem3d_compute": (C.c_int, [_h, C.c_int, _dp, C.POINTER(Stats)]),
    "plgpu_fem3d_invalidate": (C.c_int, [_h]),
    "plgpu_fem3d_sizes": (C.c_int, [_h, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "plgpu_fem3d_get_temperature": (C.c_int, [_h, _dp]),
    "plgpu_fem3d_set_temperature": (C.c_int, [_h, _dp]),
    "plgpu_fem3d_get_heat_flux": (C.c_int, [_h, _dp]),
    "plgpu_fem3d_get_conductivity": (C.c_int, [_h, _dp]),
    "plgpu_fem3d_get_thickness": (C.c_int, [_h, _dp]),
    "plgpu_fem3d_stream": (C.c_void_p, [_h]),
    "plgpu_fem3d_set_log_callback": (C.c_int, [_h, LOG_CB, C.c_void_p]),
    "plgpu_fem3d_time_operator": (C.c_int, [_h, C.c_int, C.c_int, C.c_int, _dp, _dp]),
    # include/plgpu_unet.h
    "plgpu_unet_create": (C.c_int, [C.c_ulonglong, C.POINTER(_h)]),
    "plgpu_unet_destroy": (C.c_int, [_h]),
    "plgpu_unet_last_error": (C.c_char_p, [_h]),
    "plgpu_unet_num_params": (C.c_int, [_h, C.POINTER(C.c_size_t)]),
    "plgpu_unet_get_weights": (C.c_int, [_h, C.POINTER(C.c_float)]),
    "plgpu_unet_set_weights": (C.c_int, [_h, C.POINTER(C.c_float)]),
    "plgpu_unet_save": (C.c_int, [_h, C.c_char_p]),
    "plgpu_unet_load": (C.c_int, [_h, C.c_char_p]),
    "plgpu_unet_train": (C.c_int, [_h, _h, C.c_int, C.c_float, C.c_ulonglong, C.c_int, C.c_int, C.c_int,
                                   C.POINTER(C.c_float)]),
    "plgpu_unet_loss_grad": (C.c_int, [_h, _h, _dp, _dp, C.POINTER(C.c_float), _dp, _dp]),
    "plgpu_unet_apply": (C.c_int, [_h, _h, _dp, _dp]),
    "plgpu_unet_time_apply": (C.c_int, [_h, _h, C.c_int, _dp, _dp]),
    "plgpu_fem3d_set_preconditioner": (C.c_int, [_h, _h]),
    "plgpu_fem3d_mult": (C.c_int, [_h, C.c_int, _dp, _dp]),
    "plgpu_fem3d_mult_noalloc": (C.c_int, [_h, C.c_int, _dp, _dp]),
    "plgpu_fem3d_set_material_table": (C.c_int, [_h, C.c_int, C.c_int, _dp, _dp, _dp]),
    "plgpu_fem3d_cg_operator": (C.c_int, [_h, _dp, _dp, _dp, C.POINTER(C.c_int)]),
    # include/plgpu_elec3d.h
    "plgpu_elec3d_create": (C.c_int, [_dp, C.c_int, _dp, C.c_int, _dp, C.c_int, C.c_int, C.POINTER(_h)]),
    "plgpu_elec3d_destroy": (C.c_int, [_h]),
    "plgpu_elec3d_last_error": (C.c_char_p, [_h]),
    "plgpu_elec3d_set_materials": (C.c_int, [_h, C.c_int, _dp, _dp, _dp, _up, _up]),
    "plgpu_elec3d_set_elements": (C.c_int, [_h, _ip, _ip]),
    "plgpu_elec3d_set_element_conductivity": (C.c_int, [_h, _dp]),
    "plgpu_elec3d_set_junction": (C.c_int, [_h, C.c_int, C.c_double, C.c_double]),
    "plgpu_elec3d_set_junction_params": (C.c_int, [_h, _dp]),
    "plgpu_elec3d_set_junction_conductivity": (C.c_int, [_h, C.c_double, C.c_double]),
    "plgpu_elec3d_clear_voltage": (C.c_int, [_h]),
    "plgpu_elec3d_add_voltage": (C.c_int, [_h, _lp, C.c_size_t, C.c_double]),
    "plgpu_elec3d_set_solver": (C.c_int, [_h, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int]),
    "plgpu_elec3d_set_loop": (C.c_int, [_h, C.c_double, C.c_int]),
    "plgpu_elec3d_compute": (C.c_int, [_h, C.c_int, _dp, C.POINTER(Stats)]),
    "plgpu_elec3d_invalidate": (C.c_int, [_h]),
    "plgpu_elec3d_get_potential": (C.c_int, [_h, _dp]),
    "plgpu_elec3d_get_current_density": (C.c_int, [_h, _dp]),
    "plgpu_elec3d_get_heat": (C.c_int, [_h, _dp]),
    "plgpu_elec3d_get_conductivity": (C.c_int, [_h, _dp]),
    "plgpu_elec3d_total_current": (C.c_int, [_h, C.c_int, _dp]),
    "plgpu_elec3d_total_heat": (C.c_int, [_h, _dp]),
    "plgpu_elec3d_total_energy": (C.c_int, [_h, _dp]),
    "plgpu_elec3d_capacitance": (C.c_int, [_h, _dp]),
    "plgpu_elec3d_stream": (C.c_void_p, [_h]),
    "plgpu_fem3d_heat_from": (C.c_int, [_h, _h]),
    "plgpu_fem3d_set_grid_share": (C.c_int, [_h, C.c_int]),
    "plgpu_fem3d_batch_compute": (C.c_int, [C.POINTER(_h), C.c_int, C.c_int, C.c_int, _dp, C.POINTER(Stats),
                                            C.POINTER(C.c_int)]),
    "plgpu_fem3d_batch_tune": (C.c_int, [C.POINTER(_h), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                         C.POINTER(C.c_int), _dp]),
    "plgpu_fem3d_get_element_temperature": (C.c_int, [_h, _dp]),
    # include/plgpu_fem2d.h
    "plgpu_fem2d_create": (C.c_int, [_dp, C.c_int, _dp, C.c_int, C.c_int, C.c_int, C.POINTER(_h)]),
}

_lib = None


def library_path():
    return _LIB_PATH


def load():
    """Load the native library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        from . import build as _build

        _build.build()
    if not _LIB_PATH.exists():
        raise RuntimeError(f"native library {_LIB_PATH} is missing; run python -m plask_gb300.build")
    lib = C.CDLL(str(_LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class NativeError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"[{code}] {message}")
        self.code = code


class ComputationError(NativeError):
    """Linear-solve failure (non-SPD breakdown, no convergence with noconv=error, NaN)."""


class BadInput(NativeError, ValueError):
    """Invalid argument passed to the solver."""


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64) if a is not None else None


class Fem3D:
    """Owning wrapper of one ``plgpu_fem3d`` handle.

    Arrays exchanged with it use the mesh iteration order given at creation.
    """

    def __init__(self, axes, ordering="012"):
        lib = load()
        self._lib = lib
        ax = [_f64(a) for a in axes]
        h = _h()
        rc = lib.plgpu_fem3d_create(_ptr(ax[0], C.c_double), len(ax[0]), _ptr(ax[1], C.c_double), len(ax[1]),
                                    _ptr(ax[2], C.c_double), len(ax[2]), ORDERS[ordering], C.byref(h))
        if rc != OK:
            msg = lib.plgpu_fem3d_last_error(None)
            raise (BadInput if rc == ERR_ARG else NativeError)(rc, (msg or b"").decode())
        self._h = h
        self.shape = tuple(len(a) for a in ax[::-1])
        self.ordering = ordering
        self._log_cb = None

    def close(self):
        if getattr(self, "_h", None):
            self._lib.plgpu_fem3d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc == OK:
            return
        msg = (self._lib.plgpu_fem3d_last_error(self._h) or b"").decode()
        if rc == ERR_ARG:
            raise BadInput(rc, msg)
        if rc in (ERR_NOT_SPD, ERR_NOCONV, ERR_NONFINITE):
            raise ComputationError(rc, msg)
        raise NativeError(rc, msg)

    def set_log_callback(self, fn):
        """fn(level, message) receives the solver's log lines."""
        if fn is None:
            self._log_cb = None
            self._check(self._lib.plgpu_fem3d_set_log_callback(self._h, LOG_CB(), None))
            return
        cb = LOG_CB(lambda user, level, msg: fn(level, msg.decode()))
        self._log_cb = cb
        self._check(self._lib.plgpu_fem3d_set_log_callback(self._h, cb, None))

    def set_materials(self, k300, p, kz_ratio=None, hexp=None, empty=None):
        k300, p = _f64(k300), _f64(p)
        kz, he = _f64(kz_ratio), _f64(hexp)
        em = np.ascontiguousarray(empty, dtype=np.uint8) if empty is not None else None
        self._check(self._lib.plgpu_fem3d_set_materials(self._h, len(k300), _ptr(k300, C.c_double), _ptr(p, C.c_double),
                                                        _ptr(kz, C.c_double), _ptr(he, C.c_double),
                                                        _ptr(em, C.c_uint8)))

    def set_material_table(self, material, T, k_xy, k_z=None):
        """Tabulated k(T) of one material (piecewise linear, constant beyond the ends)."""
        t, kx, kz = _f64(T), _f64(k_xy), _f64(k_z)
        n = 0 if t is None else len(t)
        if n and (len(kx) != n or (kz is not None and len(kz) != n)):
            raise BadInput(-1, "table arrays must have the same length")
        self._check(self._lib.plgpu_fem3d_set_material_table(self._h, int(material), n, _ptr(t, C.c_double),
                                                             _ptr(kx, C.c_double), _ptr(kz, C.c_double)))

    def set_elements(self, material, heat=None, leaf_height=None):
        m = np.ascontiguousarray(material, dtype=np.int32).ravel()
        q, lh = _f64(heat), _f64(leaf_height)
        self._check(self._lib.plgpu_fem3d_set_elements(self._h, _ptr(m, C.c_int32), _ptr(q, C.c_double),
                                                       _ptr(lh, C.c_double)))

    def set_heat(self, heat):
        q = _f64(heat)
        self._check(self._lib.plgpu_fem3d_set_heat(self._h, _ptr(q, C.c_double)))

    def clear_bc(self, kind):
        self._check(self._lib.plgpu_fem3d_clear_bc(self._h, kind))

    def add_bc(self, kind, nodes, v0, v1=0.0):
        nd = np.ascontiguousarray(nodes, dtype=np.int64).ravel()
        self._check(self._lib.plgpu_fem3d_add_bc(self._h, kind, _ptr(nd, C.c_int64), nd.size, float(v0), float(v1)))

    def set_solver(self, algorithm="iterative", rtol=1e-14, maxit=0, noconv="warning", empty_elements="default",
                   bc_compat=True):
        self._check(self._lib.plgpu_fem3d_set_solver(self._h, ALGORITHMS[algorithm], float(rtol), int(maxit),
                                                     NOCONV[noconv], EMPTY[empty_elements], 1 if bc_compat else 0))

    def set_loop(self, inittemp=300.0, maxerr=0.05):
        self._check(self._lib.plgpu_fem3d_set_loop(self._h, float(inittemp), float(maxerr)))

    def set_dynamic(self, cp, dens, timestep=0.1, methodparam=0.5, lumping=True, rebuildfreq=0, logfreq=500):
        """Heat capacities per material and the time-stepping parameters (Dynamic3D)."""
        c, d = _f64(cp), _f64(dens)
        self._check(self._lib.plgpu_fem3d_set_dynamic(self._h, _ptr(c, C.c_double), _ptr(d, C.c_double),
                                                      float(timestep), float(methodparam), 1 if lumping else 0,
                                                      int(rebuildfreq), int(logfreq)))

    def compute_dynamic(self, time):
        """Time steps over ``time`` ns; returns (elapsed time [ns], stats dict)."""
        el = C.c_double(0.0)
        st = Stats()
        self._check(self._lib.plgpu_fem3d_compute_dynamic(self._h, float(time), C.byref(el), C.byref(st)))
        return el.value, st.as_dict()

    def set_residual_norm(self, norm="scaled"):
        """Residual norm of the linear solves: "scaled" (Jacobi-weighted) or "plain"."""
        self._check(self._lib.plgpu_fem3d_set_residual_norm(self._h, NORMS[norm]))

    def compute(self, loops=0):
        """Run compute(loops); returns (toterr, stats dict)."""
        tot = C.c_double(0.0)
        st = Stats()
        self._check(self._lib.plgpu_fem3d_compute(self._h, int(loops), C.byref(tot), C.byref(st)))
        return tot.value, st.as_dict()

    def invalidate(self):
        self._check(self._lib.plgpu_fem3d_invalidate(self._h))

    def sizes(self):
        nn, ne = C.c_size_t(0), C.c_size_t(0)
        self._check(self._lib.plgpu_fem3d_sizes(self._h, C.byref(nn), C.byref(ne)))
        return nn.value, ne.value

    def temperature(self, out=None):
        nn, _ = self.sizes()
        out = np.empty(nn) if out is None else out
        self._check(self._lib.plgpu_fem3d_get_temperature(self._h, _ptr(out, C.c_double)))
        return out

    def set_temperature(self, values):
        v = _f64(values).ravel()
        self._check(self._lib.plgpu_fem3d_set_temperature(self._h, _ptr(v, C.c_double)))

    def heat_flux(self):
        _, ne = self.sizes()
        out = np.empty((ne, 3))
        self._check(self._lib.plgpu_fem3d_get_heat_flux(self._h, _ptr(out, C.c_double)))
        return out

    def conductivity(self):
        _, ne = self.sizes()
        out = np.empty((ne, 2))
        self._check(self._lib.plgpu_fem3d_get_conductivity(self._h, _ptr(out, C.c_double)))
        return out

    def thickness(self):
        _, ne = self.sizes()
        out = np.empty(ne)
        self._check(self._lib.plgpu_fem3d_get_thickness(self._h, _ptr(out, C.c_double)))
        return out

    def mult(self, x, precision=64):
        """y = A x with the current system matrix; x, y full node arrays in mesh order."""
        xv = _f64(x).ravel()
        y = np.empty_like(xv)
        self._check(self._lib.plgpu_fem3d_mult(self._h, int(precision), _ptr(xv, C.c_double), _ptr(y, C.c_double)))
        return y

    def mult_noalloc(self, x, precision=64):
        """A x like :meth:`mult`, staged in the library's static device buffer (no device allocation).

        For callers that cannot allocate device memory during the call; meshes of at most
        2,097,152 nodes, handle already set up by compute() or mult()."""
        xv = _f64(x).ravel()
        y = np.empty_like(xv)
        self._check(self._lib.plgpu_fem3d_mult_noalloc(self._h, int(precision), _ptr(xv, C.c_double),
                                                       _ptr(y, C.c_double)))
        return y

    def cg_operator(self, x):
        """(A x, (x, A x), staged) with the FP32 operator of the inner CG iteration.

        ``staged`` is True when the TMA-staged kernel ran.  No Dirichlet replacement."""
        xv = _f64(x).ravel()
        y = np.empty_like(xv)
        xax = C.c_double(0.0)
        st = C.c_int(0)
        self._check(self._lib.plgpu_fem3d_cg_operator(self._h, _ptr(xv, C.c_double), _ptr(y, C.c_double),
                                                      C.byref(xax), C.byref(st)))
        return y, xax.value, bool(st.value)

    def time_operator(self, precision=32, reps=20, flush_l2=True):
        """(mean ms per launch, algorithmic bytes per launch) of the stiffness-operator kernel."""
        ms, by = C.c_double(0.0), C.c_double(0.0)
        self._check(self._lib.plgpu_fem3d_time_operator(self._h, int(precision), int(reps), 1 if flush_l2 else 0,
                                                        C.byref(ms), C.byref(by)))
        return ms.value, by.value

    def stream(self):
        return self._lib.plgpu_fem3d_stream(self._h)

    def set_grid_share(self, share):
        """Aim the stencil kernel's grid at 1/share of the GPU (batched solves)."""
        self._check(self._lib.plgpu_fem3d_set_grid_share(self._h, int(share)))


class Fem2D(Fem3D):
    """Owning wrapper of a planar ``plgpu_fem3d`` handle made by ``plgpu_fem2d_create``
    (include/plgpu_fem2d.h): Static2D (geometry "cartesian") or StaticCyl ("cylindrical").

    Arrays exchanged with it use the 2D mesh iteration order ("10": axis 0 fastest,
    "01": axis 1 fastest); heat fluxes have 2 components per element."""

    def __init__(self, axes, ordering="01", geometry="cartesian"):
        lib = load()
        self._lib = lib
        ax = [_f64(a) for a in axes]
        h = _h()
        rc = lib.plgpu_fem2d_create(_ptr(ax[0], C.c_double), len(ax[0]), _ptr(ax[1], C.c_double), len(ax[1]),
                                    ORDERS2D[ordering], GEOMETRY2D[geometry], C.byref(h))
        if rc != OK:
            msg = lib.plgpu_fem3d_last_error(None)
            raise (BadInput if rc == ERR_ARG else NativeError)(rc, (msg or b"").decode())
        self._h = h
        self.shape = (len(ax[1]), len(ax[0]))
        self.ordering = ordering
        self.geometry = geometry
        self._log_cb = None

    def heat_flux(self):
        _, ne = self.sizes()
        out = np.empty((ne, 2))
        self._check(self._lib.plgpu_fem3d_get_heat_flux(self._h, _ptr(out, C.c_double)))
        return out


class Elec3D:
    """Owning wrapper of one ``plgpu_elec3d`` handle (include/plgpu_elec3d.h): the Shockley3D core.

    Arrays exchanged with it use the mesh iteration order given at creation."""

    def __init__(self, axes, ordering="012"):
        lib = load()
        self._lib = lib
        ax = [_f64(a) for a in axes]
        h = _h()
        rc = lib.plgpu_elec3d_create(_ptr(ax[0], C.c_double), len(ax[0]), _ptr(ax[1], C.c_double), len(ax[1]),
                                     _ptr(ax[2], C.c_double), len(ax[2]), ORDERS[ordering], C.byref(h))
        if rc != OK:
            msg = lib.plgpu_elec3d_last_error(None)
            raise (BadInput if rc == ERR_ARG else NativeError)(rc, (msg or b"").decode())
        self._h = h
        self.shape = tuple(len(a) for a in ax[::-1])
        self.n_elements = int(np.prod([len(a) - 1 for a in ax]))
        self.ordering = ordering

    def close(self):
        if getattr(self, "_h", None):
            self._lib.plgpu_elec3d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc == OK:
            return
        msg = (self._lib.plgpu_elec3d_last_error(self._h) or b"").decode()
        if rc == ERR_ARG:
            raise BadInput(rc, msg)
        if rc in (ERR_NOT_SPD, ERR_NOCONV, ERR_NONFINITE):
            raise ComputationError(rc, msg)
        raise NativeError(rc, msg)

    def set_materials(self, cond_xy, cond_z, eps=None, empty=None, noheat=None):
        cx, cz, ep = _f64(cond_xy), _f64(cond_z), _f64(eps)
        em = np.ascontiguousarray(empty, dtype=np.uint8) if empty is not None else None
        nh = np.ascontiguousarray(noheat, dtype=np.uint8) if noheat is not None else None
        self._check(self._lib.plgpu_elec3d_set_materials(self._h, len(cx), _ptr(cx, C.c_double), _ptr(cz, C.c_double),
                                                         _ptr(ep, C.c_double), _ptr(em, C.c_uint8),
                                                         _ptr(nh, C.c_uint8)))

    def set_elements(self, material, junction=None):
        m = np.ascontiguousarray(material, dtype=np.int32).ravel()
        j = np.ascontiguousarray(junction, dtype=np.int32).ravel() if junction is not None else None
        self._check(self._lib.plgpu_elec3d_set_elements(self._h, _ptr(m, C.c_int32), _ptr(j, C.c_int32)))

    def set_element_conductivity(self, cond2):
        c = _f64(cond2).ravel() if cond2 is not None else None
        self._check(self._lib.plgpu_elec3d_set_element_conductivity(self._h, _ptr(c, C.c_double)))

    def set_junction(self, n, beta, js):
        self._check(self._lib.plgpu_elec3d_set_junction(self._h, int(n), float(beta), float(js)))

    def set_junction_params(self, beta_js):
        """Per-element (beta, js) pairs (mesh order) or None."""
        v = _f64(beta_js).ravel() if beta_js is not None else None
        self._check(self._lib.plgpu_elec3d_set_junction_params(self._h, _ptr(v, C.c_double)))

    def set_junction_conductivity(self, c00, c11):
        self._check(self._lib.plgpu_elec3d_set_junction_conductivity(self._h, float(c00), float(c11)))

    def clear_voltage(self):
        self._check(self._lib.plgpu_elec3d_clear_voltage(self._h))

    def add_voltage(self, nodes, volts):
        nd = np.ascontiguousarray(nodes, dtype=np.int64).ravel()
        self._check(self._lib.plgpu_elec3d_add_voltage(self._h, _ptr(nd, C.c_int64), nd.size, float(volts)))

    def set_solver(self, algorithm="iterative", rtol=1e-14, maxit=0, noconv="warning", empty_elements="default"):
        self._check(self._lib.plgpu_elec3d_set_solver(self._h, ALGORITHMS[algorithm], float(rtol), int(maxit),
                                                      NOCONV[noconv], EMPTY[empty_elements]))

    def set_loop(self, maxerr=0.05, convergence="fast"):
        self._check(self._lib.plgpu_elec3d_set_loop(self._h, float(maxerr), {"fast": 0, "stable": 1}[convergence]))

    def compute(self, loops=0):
        """Run compute(loops); returns (toterr [%], stats dict; max_t holds max |j| [kA/cm2])."""
        tot = C.c_double(0.0)
        st = Stats()
        self._check(self._lib.plgpu_elec3d_compute(self._h, int(loops), C.byref(tot), C.byref(st)))
        return tot.value, st.as_dict()

    def invalidate(self):
        self._check(self._lib.plgpu_elec3d_invalidate(self._h))

    def potential(self, n_nodes):
        out = np.empty(int(n_nodes))
        self._check(self._lib.plgpu_elec3d_get_potential(self._h, _ptr(out, C.c_double)))
        return out

    def current_density(self):
        out = np.empty((self.n_elements, 3))
        self._check(self._lib.plgpu_elec3d_get_current_density(self._h, _ptr(out, C.c_double)))
        return out

    def heat(self):
        out = np.empty(self.n_elements)
        self._check(self._lib.plgpu_elec3d_get_heat(self._h, _ptr(out, C.c_double)))
        return out

    def conductivity(self):
        out = np.empty((self.n_elements, 2))
        self._check(self._lib.plgpu_elec3d_get_conductivity(self._h, _ptr(out, C.c_double)))
        return out

    def _scalar(self, fn, *args):
        v = C.c_double(0.0)
        self._check(fn(self._h, *args, C.byref(v)))
        return v.value

    def total_current(self, n=0):
        return self._scalar(self._lib.plgpu_elec3d_total_current, int(n))

    def total_heat(self):
        return self._scalar(self._lib.plgpu_elec3d_total_heat)

    def total_energy(self):
        return self._scalar(self._lib.plgpu_elec3d_total_energy)

    def capacitance(self):
        return self._scalar(self._lib.plgpu_elec3d_capacitance)

    def stream(self):
        return self._lib.plgpu_elec3d_stream(self._h)


def _handle_array(fems):
    arr = (_h * len(fems))()
    for i, f in enumerate(fems):
        arr[i] = f._h
    return arr


def batch_compute(fems, loops=0, threads=8):
    """compute(loops) of independent Fem3D handles, run concurrently (include/plgpu_fem3d.h).

    Returns (toterr array, list of stats dicts, status array)."""
    lib = load()
    n = len(fems)
    tot = np.zeros(n)
    st = (Stats * max(n, 1))()
    status = (C.c_int * max(n, 1))()
    rc = lib.plgpu_fem3d_batch_compute(_handle_array(fems), n, int(loops), int(threads), _ptr(tot, C.c_double), st,
                                       status)
    for i in range(n):
        if status[i] != OK:
            fems[i]._check(status[i])
    if rc != OK:
        raise NativeError(rc, "batched compute failed")
    return tot, [st[i].as_dict() for i in range(n)], np.array(status[:n])


def batch_tune(fems, loops=0, max_threads=32):
    """Autotune the batched path on these handles: (threads, grid share, solves/s per trial)."""
    lib = load()
    n = len(fems)
    bt, bs = C.c_int(0), C.c_int(0)
    ntr = 2 * (int(np.floor(np.log2(max(1, min(max_threads, n))))) + 1)
    tim = np.zeros(ntr)
    rc = lib.plgpu_fem3d_batch_tune(_handle_array(fems), n, int(loops), int(max_threads), C.byref(bt), C.byref(bs),
                                    _ptr(tim, C.c_double))
    if rc != OK:
        for f in fems:
            f._check(rc)
        raise NativeError(rc, "batch tuning failed")
    return bt.value, bs.value, tim


def heat_from(thermal, electrical):
    """Device-side coupling: the thermal handle's heat sources := the electrical handle's Joule heat."""
    thermal._check(thermal._lib.plgpu_fem3d_heat_from(thermal._h, electrical._h))


def element_temperature(thermal):
    """Element-average temperatures of a thermal handle (mesh order)."""
    _, ne = thermal.sizes()
    out = np.empty(ne)
    thermal._check(thermal._lib.plgpu_fem3d_get_element_temperature(thermal._h, _ptr(out, C.c_double)))
    return out


class UNet:
    """Owning wrapper of a ``plgpu_unet`` (include/plgpu_unet.h): the learned preconditioner."""

    def __init__(self, seed=0):
        lib = load()
        self._lib = lib
        h = _h()
        rc = lib.plgpu_unet_create(int(seed), C.byref(h))
        if rc != OK:
            raise NativeError(rc, (lib.plgpu_unet_last_error(None) or b"").decode())
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.plgpu_unet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, fem=None):
        if rc == OK:
            return
        if fem is not None:
            fem._check(rc)
        msg = (self._lib.plgpu_unet_last_error(self._h) or b"").decode()
        raise (BadInput if rc == ERR_ARG else NativeError)(rc, msg)

    @property
    def num_params(self):
        n = C.c_size_t(0)
        self._check(self._lib.plgpu_unet_num_params(self._h, C.byref(n)))
        return n.value

    @property
    def weights(self):
        w = np.empty(self.num_params, np.float32)
        self._check(self._lib.plgpu_unet_get_weights(self._h, w.ctypes.data_as(C.POINTER(C.c_float))))
        return w

    @weights.setter
    def weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        if w.size != self.num_params:
            raise BadInput(ERR_ARG, f"expected {self.num_params} weights, got {w.size}")
        self._check(self._lib.plgpu_unet_set_weights(self._h, w.ctypes.data_as(C.POINTER(C.c_float))))

    def save(self, path):
        self._check(self._lib.plgpu_unet_save(self._h, str(path).encode()))

    def load(self, path):
        self._check(self._lib.plgpu_unet_load(self._h, str(path).encode()))

    def train(self, fem, steps, lr=1e-3, seed=0, smooth=(5, 60), pairs="jacobi"):
        """Adam steps on pairs generated by the system matrix of ``fem`` (a Fem3D); returns the losses.

        pairs: "jacobi" (noise after damped-Jacobi sweeps) or "cg" (error after Jacobi-PCG
        iterations on A e = 0); ``smooth`` bounds the number of sweeps or iterations."""
        losses = np.empty(max(int(steps), 1), np.float32)
        kind = {"jacobi": 0, "cg": 1}[pairs]
        rc = self._lib.plgpu_unet_train(self._h, fem._h, int(steps), float(lr), int(seed), int(smooth[0]),
                                        int(smooth[1]), kind, losses.ctypes.data_as(C.POINTER(C.c_float)))
        self._check(rc, fem)
        return losses[: int(steps)]

    def loss_grad(self, fem, e):
        """(loss, gradient, r, z) for error ``e`` (full node array in mesh order)."""
        e = _f64(e).ravel()
        loss = C.c_double(0.0)
        g = np.empty(self.num_params, np.float32)
        r = np.empty_like(e)
        z = np.empty_like(e)
        rc = self._lib.plgpu_unet_loss_grad(self._h, fem._h, _ptr(e, C.c_double), C.byref(loss),
                                            g.ctypes.data_as(C.POINTER(C.c_float)), _ptr(r, C.c_double),
                                            _ptr(z, C.c_double))
        self._check(rc, fem)
        return loss.value, g, r, z

    def apply(self, fem, r):
        """z = P(r) for a residual (full node array in mesh order)."""
        r = _f64(r).ravel()
        z = np.empty_like(r)
        self._check(self._lib.plgpu_unet_apply(self._h, fem._h, _ptr(r, C.c_double), _ptr(z, C.c_double)), fem)
        return z

    def time_apply(self, fem, reps=20):
        """(forward ms, whole preconditioner application ms), device time on ``fem``'s mesh."""
        a, b = C.c_double(0.0), C.c_double(0.0)
        self._check(self._lib.plgpu_unet_time_apply(self._h, fem._h, int(reps), C.byref(a), C.byref(b)), fem)
        return a.value, b.value


def attach_preconditioner(fem, net):
    """Use ``net`` (a UNet or None) in the learned solve of ``fem``."""
    fem._check(fem._lib.plgpu_fem3d_set_preconditioner(fem._h, net._h if net is not None else None))
    fem._pre = net
