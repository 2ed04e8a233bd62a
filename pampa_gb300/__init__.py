"""pampa_gb300: GB300-native k-eigenvalue solver for pampa's diffusion and SN hot path.

The product is ``libpampa_gb300.so`` (built in-tree by ``pampa_gb300.build``).  This
module binds its C-ABI with ctypes:

* :class:`Pampa` mirrors the reference's C driver API (``pampa_initialize`` ...
  ``pampa_finalize``, ``pampa_get_field``); it reads ``.pmp`` inputs exactly as the
  reference does and runs the solve on the GPU.
* :class:`DiffusionProblem` / :class:`SNProblem` wrap the lower-level ``pgpu_*`` operator
  API (operator arrays in, device-resident solve, results out).

There is no CPU fallback: if the library is missing, importing the bindings raises.
"""

from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libpampa_gb300.so")

PGPU_OK, PGPU_ERR_INVALID, PGPU_ERR_CUDA, PGPU_ERR_NOT_CONVERGED, PGPU_ERR_NEGATIVE_FLUX, \
    PGPU_ERR_NAN, PGPU_ERR_NO_MEMORY, PGPU_ERR_TIMEOUT = range(8)
PGPU_FP64, PGPU_MIXED = 0, 1
FACE_INTERIOR, FACE_VACUUM, FACE_REFLECTIVE, FACE_NONE = range(4)

_lib = None


class PampaError(RuntimeError):
    pass


class pgpu_options(C.Structure):
    _fields_ = [("precision", C.c_int), ("tol_k", C.c_double), ("tol_flux", C.c_double),
                ("max_outer", C.c_int), ("max_inner", C.c_int), ("power", C.c_double),
                ("verbose", C.c_int), ("profile", C.c_int), ("shift", C.c_double)]


class pgpu_stats(C.Structure):
    _fields_ = [("keff", C.c_double), ("outer_iterations", C.c_int), ("inner_iterations", C.c_int),
                ("sweeps", C.c_int), ("residual", C.c_double), ("seconds", C.c_double),
                ("status", C.c_int), ("launches", C.c_longlong), ("kernel_seconds", C.c_double),
                ("kernel_launches", C.c_longlong), ("kernel_bytes", C.c_double),
                ("kernel_name", C.c_char * 32)]


_P = C.POINTER
_pd = _P(C.c_double)
_pi = _P(C.c_int)


class pgpu_diffusion_operator(C.Structure):
    _fields_ = [("num_cells", C.c_int), ("num_groups", C.c_int), ("num_faces", C.c_int),
                ("num_materials", C.c_int), ("neighbors", _pi), ("offdiag", _pd), ("diag", _pd),
                ("materials", _pi), ("volumes", _pd), ("sigma_s", _pd), ("chi", _pd),
                ("nu_sigma_f", _pd), ("kappa_sigma_f", _pd)]


class pgpu_sn_operator(C.Structure):
    _fields_ = [("num_cells", C.c_int), ("num_groups", C.c_int), ("num_dirs", C.c_int),
                ("num_faces", C.c_int), ("num_materials", C.c_int), ("use_ls", C.c_int),
                ("num_cell_faces", _pi), ("face_kind", _pi), ("neighbors", _pi), ("areas", _pd),
                ("normals", _pd), ("gauss", _pd), ("reflect_axis", _pi), ("ls_weight", _pd),
                ("materials", _pi), ("volumes", _pd), ("directions", _pd), ("weights", _pd),
                ("reflected", _pi), ("sigma_t", _pd), ("sigma_s", _pd), ("chi", _pd),
                ("nu_sigma_f", _pd), ("kappa_sigma_f", _pd), ("cart_nx", C.c_int), ("cart_ny", C.c_int),
                ("cart_nz", C.c_int)]


# Every C symbol declared in include/pampa_gb300.h, with its ctypes signature.
SYMBOLS = {
    "pampa_initialize": (None, [C.c_int, _P(C.c_char_p), _P(_pd), _pi, _pi]),
    "pampa_initialize_steady_state": (None, [C.c_int, _P(C.c_char_p), _pi]),
    "pampa_solve": (None, [C.c_int, C.c_double, C.c_double, _pi]),
    "pampa_solve_steady_state": (None, [_pi]),
    "pampa_finalize": (None, [_P(_pd), _pi]),
    "pampa_finalize_steady_state": (None, [_pi]),
    "pampa_get_field": (None, [_pd, C.c_char_p, _pi]),
    "pampa_set_field": (None, [_pd, C.c_char_p, _pi]),
    "pampa_get_keff": (None, [_pd, _pi]),
    "pampa_get_field_size": (None, [C.c_char_p, _pi, _pi]),
    "pampa_get_solve_stats": (None, [_pi, _pi, _pd, _pi]),
    "pampa_get_problem": (None, [_P(C.c_void_p), _pi]),
    "pgpu_default_options": (None, [_P(pgpu_options)]),
    "pgpu_last_error": (C.c_char_p, []),
    "pgpu_diffusion_create": (C.c_int, [C.c_int, _P(pgpu_diffusion_operator), _P(C.c_void_p)]),
    "pgpu_diffusion_apply": (C.c_int, [C.c_void_p, _pd, _pd]),
    "pgpu_sn_create": (C.c_int, [C.c_int, _P(pgpu_sn_operator), _P(C.c_void_p)]),
    "pgpu_sn_apply": (C.c_int, [C.c_void_p, _pd, _pd]),
    "pgpu_problem_solve": (C.c_int, [C.c_void_p, _P(pgpu_options), _P(pgpu_stats)]),
    "pgpu_problem_solve_linear": (C.c_int, [C.c_void_p, C.c_double, _pd, _pd, _P(pgpu_options), _P(pgpu_stats)]),
    "pgpu_problem_get_keff": (C.c_int, [C.c_void_p, _pd]),
    "pgpu_problem_get_scalar_flux": (C.c_int, [C.c_void_p, _pd]),
    "pgpu_problem_get_angular_flux": (C.c_int, [C.c_void_p, _pd]),
    "pgpu_problem_get_power": (C.c_int, [C.c_void_p, _pd, _pd, _pd]),
    "pgpu_problem_device_bytes": (C.c_longlong, [C.c_void_p]),
    "pgpu_problem_set_sm_share": (C.c_int, [C.c_void_p, C.c_int]),
    "pgpu_problem_upload_bytes": (C.c_longlong, [C.c_void_p]),
    "pgpu_problem_destroy": (None, [C.c_void_p]),
    "pgpu_normalize_power_noalloc": (C.c_int, [C.c_int, C.c_int] + [C.c_void_p] * 5 + [C.c_double, C.c_double]
                                     + [C.c_void_p] * 6),
    "pgpu_serve_create": (C.c_int, [C.c_int, C.c_int, C.c_double, _P(C.c_void_p)]),
    "pgpu_serve_budget_bytes": (C.c_longlong, [C.c_void_p]),
    "pgpu_serve_set_sm_share": (C.c_int, [C.c_void_p, C.c_int]),
    "pgpu_serve_submit_diffusion": (C.c_int, [C.c_void_p, _P(pgpu_diffusion_operator), _P(pgpu_options), C.c_int,
                                              _P(C.c_longlong)]),
    "pgpu_serve_submit_sn": (C.c_int, [C.c_void_p, _P(pgpu_sn_operator), _P(pgpu_options), C.c_int,
                                       _P(C.c_longlong)]),
    "pgpu_serve_poll": (C.c_int, [C.c_void_p, C.c_longlong, _pi]),
    "pgpu_serve_wait": (C.c_int, [C.c_void_p, C.c_longlong, _P(pgpu_stats), _pd, _pd, _pd]),
    "pgpu_serve_destroy": (C.c_int, [C.c_void_p]),
}


def lib() -> C.CDLL:
    """Load libpampa_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise PampaError(f"{LIB_PATH} is missing: run `python -m pampa_gb300.build` first")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SYMBOLS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    return lib().pgpu_last_error().decode()


def default_options(**kw) -> pgpu_options:
    o = pgpu_options()
    lib().pgpu_default_options(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_pd)


def _ip(a: np.ndarray):
    return a.ctypes.data_as(_pi)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


# --------------------------------------------------------------------------------------
# Drop-in driver API
# --------------------------------------------------------------------------------------


class Pampa:
    """The reference's C driver API (pampa.hxx) over libpampa_gb300.so.

    One instance at a time (the C API drives a single global driver, as the reference's
    does).  Errors raise :class:`PampaError` carrying the library's message.
    """

    def __init__(self, input_path: str, *args: str):
        self._argv = [b"pampa", input_path.encode()] + [a.encode() for a in args]
        argv = (C.c_char_p * len(self._argv))(*self._argv)
        err = C.c_int(0)
        self._dt = _pd()
        ndt = C.c_int(0)
        lib().pampa_initialize(len(self._argv), argv, C.byref(self._dt), C.byref(ndt), C.byref(err))
        if err.value:
            raise PampaError(f"pampa_initialize failed for {input_path}")
        self.dt = [self._dt[i] for i in range(ndt.value)]
        self._open = True

    def solve(self, n: int = 0, dt: float = 0.0, t: float = 0.0):
        err = C.c_int(0)
        lib().pampa_solve(n, dt, t, C.byref(err))
        if err.value:
            raise PampaError(f"pampa_solve failed: {last_error()}")

    @property
    def keff(self) -> float:
        k = C.c_double(0)
        err = C.c_int(0)
        lib().pampa_get_keff(C.byref(k), C.byref(err))
        if err.value:
            raise PampaError("pampa_get_keff failed")
        return k.value

    def field(self, name: str) -> np.ndarray:
        size = C.c_int(0)
        err = C.c_int(0)
        lib().pampa_get_field_size(name.encode(), C.byref(size), C.byref(err))
        if err.value:
            raise PampaError(f"unknown field {name}")
        out = np.zeros(size.value)
        lib().pampa_get_field(_dp(out), name.encode(), C.byref(err))
        if err.value:
            raise PampaError(f"pampa_get_field({name}) failed")
        return out

    def set_field(self, name: str, values) -> None:
        v = _f64(values)
        err = C.c_int(0)
        lib().pampa_set_field(_dp(v), name.encode(), C.byref(err))
        if err.value:
            raise PampaError(f"pampa_set_field({name}) failed")

    def stats(self) -> dict:
        o, i, s, e = C.c_int(0), C.c_int(0), C.c_double(0), C.c_int(0)
        lib().pampa_get_solve_stats(C.byref(o), C.byref(i), C.byref(s), C.byref(e))
        return dict(outer_iterations=o.value, inner_iterations=i.value, seconds=s.value)

    def apply_operator(self, x) -> np.ndarray:
        """y = R x on the GPU for the operator the driver assembled from the input."""
        h = C.c_void_p(None)
        err = C.c_int(0)
        lib().pampa_get_problem(C.byref(h), C.byref(err))
        if err.value:
            raise PampaError(f"pampa_get_problem failed: {last_error()}")
        x = _f64(x)
        y = np.zeros_like(x)
        # a vector of the scalar flux's length is a diffusion vector, anything else an SN
        # angular flux (the library checks the problem's kind either way)
        fn = lib().pgpu_diffusion_apply if x.size == self.field_size("scalar-flux") else lib().pgpu_sn_apply
        st = fn(h, _dp(x), _dp(y))
        if st != PGPU_OK:
            raise PampaError(f"operator apply failed: {last_error()}")
        return y

    def field_size(self, name: str) -> int:
        size = C.c_int(0)
        err = C.c_int(0)
        lib().pampa_get_field_size(name.encode(), C.byref(size), C.byref(err))
        return size.value if err.value == 0 else 0

    def finalize(self):
        if self._open:
            err = C.c_int(0)
            lib().pampa_finalize(C.byref(self._dt), C.byref(err))
            self._open = False
            if err.value:
                raise PampaError("pampa_finalize failed")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.finalize()


# --------------------------------------------------------------------------------------
# GPU operator API
# --------------------------------------------------------------------------------------


@dataclass
class SolveResult:
    keff: float
    stats: dict


class _Problem:
    _keep: list

    def __init__(self):
        self._h = C.c_void_p(None)

    def _check(self, st: int, what: str):
        if st != PGPU_OK:
            raise PampaError(f"{what} failed ({st}): {last_error()}")

    def solve(self, **opts) -> SolveResult:
        o = default_options(**opts)
        s = pgpu_stats()
        st = lib().pgpu_problem_solve(self._h, C.byref(o), C.byref(s))
        stats = {k: getattr(s, k) for k, _ in pgpu_stats._fields_}
        if st != PGPU_OK:
            raise PampaError(f"pgpu_problem_solve failed ({st}): {last_error()} stats={stats}")
        return SolveResult(s.keff, stats)

    def solve_linear(self, lam: float, b, x0=None, **opts) -> tuple[np.ndarray, dict]:
        """x with (R - lam F) x = b (diffusion problems), from the guess x0 (zeros)."""
        o = default_options(**opts)
        s = pgpu_stats()
        bb = _f64(b)
        x = np.array(x0, dtype=np.float64) if x0 is not None else np.zeros_like(bb)
        st = lib().pgpu_problem_solve_linear(self._h, lam, _dp(bb), _dp(x), C.byref(o), C.byref(s))
        stats = {k: getattr(s, k) for k, _ in pgpu_stats._fields_}
        if st != PGPU_OK:
            raise PampaError(f"pgpu_problem_solve_linear failed ({st}): {last_error()} stats={stats}")
        return x, stats

    def scalar_flux(self) -> np.ndarray:
        out = np.zeros(self.num_cells * self.num_groups)
        self._check(lib().pgpu_problem_get_scalar_flux(self._h, _dp(out)), "get_scalar_flux")
        return out

    def power(self):
        q = np.zeros(self.num_cells)
        P = np.zeros(self.num_cells)
        tot = C.c_double(0)
        self._check(lib().pgpu_problem_get_power(self._h, _dp(q), _dp(P), C.byref(tot)), "get_power")
        return q, P, tot.value

    @property
    def device_bytes(self) -> int:
        return int(lib().pgpu_problem_device_bytes(self._h))

    def close(self):
        if self._h:
            lib().pgpu_problem_destroy(self._h)
            self._h = C.c_void_p(None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class DiffusionProblem(_Problem):
    """Device-resident diffusion operator (pgpu_diffusion_operator)."""

    def __init__(self, *, neighbors, offdiag, diag, materials, volumes, sigma_s, chi,
                 nu_sigma_f, kappa_sigma_f, device: int = 0):
        super().__init__()
        nbr = _i32(neighbors)
        F, n = nbr.shape
        G = np.asarray(diag).size // n
        nm = np.asarray(chi).size // G
        self.num_cells, self.num_groups = n, G
        arrs = dict(neighbors=nbr, offdiag=_f64(offdiag), diag=_f64(diag), materials=_i32(materials),
                    volumes=_f64(volumes), sigma_s=_f64(sigma_s), chi=_f64(chi),
                    nu_sigma_f=_f64(nu_sigma_f), kappa_sigma_f=_f64(kappa_sigma_f))
        op = pgpu_diffusion_operator(n, G, F, nm)
        for k, a in arrs.items():
            setattr(op, k, _ip(a) if a.dtype == np.int32 else _dp(a))
        self._keep = list(arrs.values())
        self._check(lib().pgpu_diffusion_create(device, C.byref(op), C.byref(self._h)), "pgpu_diffusion_create")

    def apply(self, x) -> np.ndarray:
        x = _f64(x)
        y = np.zeros_like(x)
        self._check(lib().pgpu_diffusion_apply(self._h, _dp(x), _dp(y)), "pgpu_diffusion_apply")
        return y


class SNProblem(_Problem):
    """Device-resident discrete-ordinates operator (pgpu_sn_operator)."""

    def __init__(self, *, num_cell_faces, face_kind, neighbors, areas, normals, gauss, reflect_axis,
                 materials, volumes, directions, weights, reflected, sigma_t, sigma_s, chi,
                 nu_sigma_f, kappa_sigma_f, ls_weight=None, device: int = 0):
        super().__init__()
        kind = _i32(face_kind)
        F, n = kind.shape
        w = _f64(weights)
        M = w.size
        if np.asarray(sigma_s).ndim != 3:
            raise ValueError("sigma_s must have shape (materials, G, G)")
        nm, G = np.asarray(sigma_s).shape[:2]
        self.num_cells, self.num_groups, self.num_dirs = n, G, M
        arrs = dict(num_cell_faces=_i32(num_cell_faces), face_kind=kind, neighbors=_i32(neighbors),
                    areas=_f64(areas), normals=_f64(normals), gauss=_f64(gauss),
                    reflect_axis=_i32(reflect_axis), materials=_i32(materials), volumes=_f64(volumes),
                    directions=_f64(directions), weights=w, reflected=_i32(reflected),
                    sigma_t=_f64(sigma_t), sigma_s=_f64(sigma_s), chi=_f64(chi),
                    nu_sigma_f=_f64(nu_sigma_f), kappa_sigma_f=_f64(kappa_sigma_f))
        use_ls = ls_weight is not None
        if use_ls:
            arrs["ls_weight"] = _f64(ls_weight)
        op = pgpu_sn_operator(n, G, M, F, nm, int(use_ls))
        for k, a in arrs.items():
            setattr(op, k, _ip(a) if a.dtype == np.int32 else _dp(a))
        self._keep = list(arrs.values())
        self._check(lib().pgpu_sn_create(device, C.byref(op), C.byref(self._h)), "pgpu_sn_create")

    def apply(self, x) -> np.ndarray:
        x = _f64(x)
        y = np.zeros_like(x)
        self._check(lib().pgpu_sn_apply(self._h, _dp(x), _dp(y)), "pgpu_sn_apply")
        return y

    def angular_flux(self) -> np.ndarray:
        out = np.zeros(self.num_cells * self.num_groups * self.num_dirs)
        self._check(lib().pgpu_problem_get_angular_flux(self._h, _dp(out)), "get_angular_flux")
        return out


def diffusion_operator_struct(*, neighbors, offdiag, diag, materials, volumes, sigma_s, chi, nu_sigma_f,
                              kappa_sigma_f):
    """(pgpu_diffusion_operator, arrays to keep alive) from numpy arrays."""
    nbr = _i32(neighbors)
    F, n = nbr.shape
    G = np.asarray(diag).size // n
    nm = np.asarray(chi).size // G
    arrs = dict(neighbors=nbr, offdiag=_f64(offdiag), diag=_f64(diag), materials=_i32(materials),
                volumes=_f64(volumes), sigma_s=_f64(sigma_s), chi=_f64(chi),
                nu_sigma_f=_f64(nu_sigma_f), kappa_sigma_f=_f64(kappa_sigma_f))
    op = pgpu_diffusion_operator(n, G, F, nm)
    for k, a in arrs.items():
        setattr(op, k, _ip(a) if a.dtype == np.int32 else _dp(a))
    return op, list(arrs.values())


def sn_operator_struct(*, num_cell_faces, face_kind, neighbors, areas, normals, gauss, reflect_axis, materials,
                       volumes, directions, weights, reflected, sigma_t, sigma_s, chi, nu_sigma_f, kappa_sigma_f,
                       ls_weight=None, cart=(0, 0, 0)):
    """(pgpu_sn_operator, arrays to keep alive) from numpy arrays (layouts of the header)."""
    kind = _i32(face_kind)
    F, n = kind.shape
    w = _f64(weights)
    nm, G = np.asarray(sigma_s).shape[:2]
    arrs = dict(num_cell_faces=_i32(num_cell_faces), face_kind=kind, neighbors=_i32(neighbors),
                areas=_f64(areas), normals=_f64(normals), gauss=_f64(gauss), reflect_axis=_i32(reflect_axis),
                materials=_i32(materials), volumes=_f64(volumes), directions=_f64(directions), weights=w,
                reflected=_i32(reflected), sigma_t=_f64(sigma_t), sigma_s=_f64(sigma_s), chi=_f64(chi),
                nu_sigma_f=_f64(nu_sigma_f), kappa_sigma_f=_f64(kappa_sigma_f))
    if ls_weight is not None:
        arrs["ls_weight"] = _f64(ls_weight)
    op = pgpu_sn_operator(n, G, w.size, F, nm, int(ls_weight is not None))
    for k, a in arrs.items():
        setattr(op, k, _ip(a) if a.dtype == np.int32 else _dp(a))
    op.cart_nx, op.cart_ny, op.cart_nz = cart
    return op, list(arrs.values())


class Server:
    """Continuous-batching solve server (pgpu_serve_*): submit operators, wait for results."""

    def __init__(self, device: int = 0, slots: int = 8, hbm_fraction: float = 0.8, sm_share: int | None = None):
        self._h = C.c_void_p(None)
        st = lib().pgpu_serve_create(device, slots, hbm_fraction, C.byref(self._h))
        if st != PGPU_OK:
            raise PampaError(f"pgpu_serve_create failed ({st}): {last_error()}")
        self._sizes = {}
        if sm_share is not None and lib().pgpu_serve_set_sm_share(self._h, sm_share) != PGPU_OK:
            raise PampaError("pgpu_serve_set_sm_share failed")

    @property
    def budget_bytes(self) -> int:
        return int(lib().pgpu_serve_budget_bytes(self._h))

    def submit_diffusion(self, op: dict, options: pgpu_options | None = None, want_flux: bool = False) -> int:
        o, _keep = diffusion_operator_struct(**op)
        rid = C.c_longlong(0)
        st = lib().pgpu_serve_submit_diffusion(self._h, C.byref(o), C.byref(options) if options else None,
                                               int(want_flux), C.byref(rid))
        if st != PGPU_OK:
            raise PampaError(f"pgpu_serve_submit_diffusion failed ({st})")
        self._sizes[rid.value] = o.num_cells * o.num_groups if want_flux else 0
        return rid.value

    def submit_sn(self, op: dict, options: pgpu_options | None = None, want_flux: bool = False) -> int:
        o, _keep = sn_operator_struct(**op)
        rid = C.c_longlong(0)
        st = lib().pgpu_serve_submit_sn(self._h, C.byref(o), C.byref(options) if options else None,
                                        int(want_flux), C.byref(rid))
        if st != PGPU_OK:
            raise PampaError(f"pgpu_serve_submit_sn failed ({st})")
        self._sizes[rid.value] = o.num_cells * o.num_groups if want_flux else 0
        return rid.value

    def done(self, rid: int) -> bool:
        d = C.c_int(0)
        if lib().pgpu_serve_poll(self._h, rid, C.byref(d)) != PGPU_OK:
            raise PampaError(f"unknown request {rid}")
        return bool(d.value)

    def wait(self, rid: int) -> dict:
        """Result of a request: status, keff, stats, phi (when asked for) and times."""
        stats = pgpu_stats()
        k = C.c_double(0.0)
        times = np.zeros(3)
        nphi = self._sizes.pop(rid, 0)
        phi = np.zeros(nphi) if nphi else None
        st = lib().pgpu_serve_wait(self._h, rid, C.byref(stats), C.byref(k), _dp(phi) if phi is not None else None,
                                   _dp(times))
        return dict(status=st, keff=k.value, phi=phi, queue_s=times[0], run_s=times[1], latency_s=times[2],
                    error=last_error() if st != PGPU_OK else "",
                    stats={f: getattr(stats, f) for f, _ in pgpu_stats._fields_})

    def close(self):
        if self._h:
            lib().pgpu_serve_destroy(self._h)
            self._h = C.c_void_p(None)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
