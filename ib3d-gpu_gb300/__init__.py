"""GB300 IB3D hot path: Python mirror of the C ABI in include/ib3d.h.

The reference drives its hot path as Fortran subroutine calls (main.f90:29-66:
nsMomentum, velocityBC, solidCellBC, velocityForcing1, poissonSolver,
pressureForcing1, stressCal1/2). `Solver` exposes the same calls, in the same
names, over ctypes bindings of libib3d.so; arrays are numpy arrays in the
reference's Fortran layout (shape (nx+2, ny+2, nz+2), order='F').

The library is the CUDA implementation; there is no CPU fallback. Importing this
module works without a GPU (so the build and the ABI can be checked anywhere),
but creating a Solver needs the built libib3d.so and a CUDA device and raises
IB3DError otherwise.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib
import re

import numpy as np

from . import grids  # noqa: F401  (re-exported)

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "libib3d.so"
HEADER = HERE.parent / "include" / "ib3d.h"

OK, ERR_ARG, ERR_CUDA, ERR_MESH, ERR_PROBE, ERR_NOCONV, ERR_NONFINITE, ERR_MEMORY, ERR_TOO_LARGE = 0, -1, -2, -3, -4, -5, -6, -7, -8
ERR_IO = -9
CRIT_UPDATE, CRIT_RESIDUAL = 0, 1
PREC_FP64, PREC_FP32DC, PREC_FP64_FAST = 0, 1, 2
WARM_ZERO, WARM_PREV, WARM_LEARNED = 0, 1, 2
INNER_FIXED, INNER_ADAPTIVE, INNER_TAIL = 0, 1, 2
MESH_GMSH, MESH_GAMBIT = 0, 1
OUTLET_ZERO_GRADIENT, OUTLET_CONVECTIVE = 0, 1
MOMENTUM_EULER, MOMENTUM_AB2 = 0, 1
FIELDS = {"u": 0, "v": 1, "w": 2, "ut": 3, "vt": 4, "wt": 5, "p": 6, "pc": 7, "b": 8}
_ERRNAMES = {ERR_ARG: "IB3D_ERR_ARG", ERR_CUDA: "IB3D_ERR_CUDA", ERR_MESH: "IB3D_ERR_MESH",
             ERR_PROBE: "IB3D_ERR_PROBE", ERR_NOCONV: "IB3D_ERR_NOCONV", ERR_NONFINITE: "IB3D_ERR_NONFINITE",
             ERR_MEMORY: "IB3D_ERR_MEMORY", ERR_TOO_LARGE: "IB3D_ERR_TOO_LARGE", ERR_IO: "IB3D_ERR_IO"}


class IB3DError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERRNAMES.get(code, code)}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [("re", C.c_double), ("deltat", C.c_double), ("omega", C.c_double), ("eps", C.c_double),
                ("max_sweeps", C.c_int64), ("criterion", C.c_int32), ("precision", C.c_int32),
                ("warm_start", C.c_int32), ("check_every", C.c_int32), ("inner_sweeps", C.c_int32),
                ("sweep_kernel", C.c_int32), ("omega_inner", C.c_double), ("inner_schedule", C.c_int32),
                ("outlet", C.c_int32), ("momentum", C.c_int32), ("smooth_sweeps", C.c_int32),
                ("ramp_sweeps", C.c_int32)]


class SolveStats(C.Structure):
    _fields_ = [("sweeps", C.c_int64), ("outer", C.c_int64), ("divmax", C.c_double), ("derr_std_st", C.c_double),
                ("final_err", C.c_double), ("solve_seconds", C.c_double), ("initial_err", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Timers(C.Structure):
    _fields_ = [("ms", C.c_double * 10), ("sweeps64", C.c_int64), ("sweeps32", C.c_int64), ("outer", C.c_int64),
                ("launches", C.c_int64), ("steps", C.c_int64), ("launches32", C.c_int64)]
    PHASES = ("momentum", "bc", "forcing", "divergence", "sor64", "sor32", "residual", "correct", "stress", "net")

    def as_dict(self) -> dict:
        d = {f"{n}_ms": self.ms[q] for q, n in enumerate(self.PHASES)}
        for k in ("sweeps64", "sweeps32", "outer", "launches", "steps", "launches32"):
            d[k] = getattr(self, k)
        return d


_lib = None
_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_F = C.POINTER(C.c_float)
_VP = C.c_void_p


def header_functions() -> list[str]:
    """Names of the functions include/ib3d.h declares."""
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?(?:int|int64_t|void\*?|char\*?|const char\*)\s*\**\s*(ib3d_\w+)\s*\(",
                                 text, re.M)))


def lib() -> C.CDLL:
    """Loads libib3d.so (built by build.py); raises when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise IB3DError(ERR_CUDA, f"{LIB_PATH} is missing: run build() (the CUDA library is required)")
    L = C.CDLL(str(LIB_PATH))
    sig = {
        "ib3d_default_params": (None, [C.POINTER(Params)]),
        "ib3d_create": (C.c_int, [C.POINTER(_VP), C.POINTER(Params), C.c_int64, C.c_int64, C.c_int64, _D, _D, _D]),
        "ib3d_destroy": (None, [_VP]),
        "ib3d_last_error": (C.c_char_p, [_VP]),
        "ib3d_set_params": (C.c_int, [_VP, C.POINTER(Params)]),
        "ib3d_set_mesh": (C.c_int, [_VP, C.c_int64, _D, _D, _D, C.c_int64, _I64, _I64, _I64, C.c_double,
                                    C.c_double, C.c_double, C.c_int64]),
        "ib3d_search": (C.c_int, [_VP, _I64, _I64]),
        "ib3d_selective_retag": (C.c_int, [_VP, _I64]),
        "ib3d_move_body": (C.c_int, [_VP] + [C.c_double] * 6),
        "ib3d_move_body_free": (C.c_int, [_VP, C.c_double, C.c_double, C.c_double, _D]),
        "ib3d_read_surface_mesh": (C.c_int, [C.c_char_p, C.c_int32, C.c_int64, _I64, _D, _D, _D, _I64, _I64, _I64,
                                             _I64]),
        "ib3d_set_mesh_file": (C.c_int, [_VP, C.c_char_p, C.c_int32, C.c_int64, C.c_double, C.c_double,
                                         C.c_double, C.c_int64]),
        "ib3d_write_restart": (C.c_int, [_VP, C.c_char_p, C.c_double, C.c_int64, C.c_int64]),
        "ib3d_read_restart": (C.c_int, [_VP, C.c_char_p, _D, _I64, _I64]),
        "ib3d_write_result_text": (C.c_int, [_VP, C.c_char_p, C.c_double, C.c_int64, C.c_int64]),
        "ib3d_read_result_text": (C.c_int, [_VP, C.c_char_p, _D, _I64, _I64]),
        "ib3d_set_poisson_coefficients": (C.c_int, [_VP, _D, _D, _D]),
        "ib3d_get_search": (C.c_int, [_VP, _I64, _I64, _I64, _D]),
        "ib3d_initial_conditions": (C.c_int, [_VP]),
        "ib3d_upload_fields": (C.c_int, [_VP, _D, _D, _D, _D]),
        "ib3d_download_fields": (C.c_int, [_VP, _D, _D, _D, _D, _D, _D, _D]),
        "ib3d_download_fields_async": (C.c_int, [_VP, _D, _D, _D, _D, _D, _D, _D]),
        "ib3d_download_wait": (C.c_int, [_VP]),
        "ib3d_get_field": (C.c_int, [_VP, C.c_int, _D]),
        "ib3d_set_field": (C.c_int, [_VP, C.c_int, _D]),
        "ib3d_ns_momentum": (C.c_int, [_VP]),
        "ib3d_ns_momentum_ab": (C.c_int, [_VP]),
        "ib3d_calculate_uc": (C.c_int, [_VP, _D]),
        "ib3d_velocity_bc": (C.c_int, [_VP]),
        "ib3d_solid_cell_bc": (C.c_int, [_VP]),
        "ib3d_velocity_forcing": (C.c_int, [_VP]),
        "ib3d_pressure_forcing": (C.c_int, [_VP]),
        "ib3d_poisson_solver": (C.c_int, [_VP, C.POINTER(SolveStats)]),
        "ib3d_redblack_sor": (C.c_int, [_VP, C.POINTER(SolveStats)]),
        "ib3d_stress": (C.c_int, [_VP, C.c_int, _D]),
        "ib3d_step": (C.c_int, [_VP, C.c_int, C.POINTER(SolveStats), _D]),
        "ib3d_device_field": (_VP, [_VP, C.c_int]),
        "ib3d_timers_enable": (C.c_int, [_VP, C.c_int]),
        "ib3d_timers_read": (C.c_int, [_VP, C.POINTER(Timers)]),
        "ib3d_stream": (_VP, [_VP]),
        "ib3d_net_create": (C.c_int, [C.POINTER(_VP), C.c_uint64]),
        "ib3d_net_destroy": (None, [_VP]),
        "ib3d_net_last_error": (C.c_char_p, [_VP]),
        "ib3d_net_num_params": (C.c_int64, [_VP]),
        "ib3d_net_get_params": (C.c_int, [_VP, _F]),
        "ib3d_net_set_params": (C.c_int, [_VP, _F]),
        "ib3d_net_loss_grad": (C.c_int, [_VP, C.c_int, C.c_int, _F, _F, _D, _F, _F]),
        "ib3d_net_dataset_reserve": (C.c_int, [_VP, C.c_int, C.c_int64]),
        "ib3d_net_dataset_size": (C.c_int64, [_VP]),
        "ib3d_net_capture": (C.c_int, [_VP, _VP, C.c_int, C.c_uint64]),
        "ib3d_net_set_coarsening": (C.c_int, [_VP, C.c_int]),
        "ib3d_net_train": (C.c_int, [_VP, C.c_int, C.c_int, C.c_double, C.c_uint64, _D]),
        "ib3d_net_set_wgrad_tensor_cores": (C.c_int, [_VP, C.c_int]),
        "ib3d_enable_history": (C.c_int, [_VP]),
        "ib3d_attach_net": (C.c_int, [_VP, _VP]),
        "ib3d_pressure_solve_noalloc": (C.c_int, [C.c_int64, C.c_int64, C.c_int64, _VP, _VP, _VP, _VP, _VP,
                                                  C.c_double, _VP, C.c_double, C.c_double, C.c_int64, C.c_int32,
                                                  _VP, _I64, _D]),
        "ib3d_synchronize": (C.c_int, [_VP]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def default_params(**kw) -> Params:
    p = Params()
    lib().ib3d_default_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _ip(a: np.ndarray):
    return a.ctypes.data_as(_I64)


class Solver:
    """One device-resident solver context (ib3d_ctx)."""

    def __init__(self, x: np.ndarray, y: np.ndarray, z: np.ndarray, params: Params | None = None, **kw):
        self.L = lib()
        self.params = params if params is not None else default_params(**kw)
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.y = np.ascontiguousarray(y, dtype=np.float64)
        self.z = np.ascontiguousarray(z, dtype=np.float64)
        self.nx, self.ny, self.nz = len(x) - 1, len(y) - 1, len(z) - 1
        self.shape = (self.nx + 2, self.ny + 2, self.nz + 2)
        self._h = _VP()
        rc = self.L.ib3d_create(C.byref(self._h), C.byref(self.params), self.nx, self.ny, self.nz, _dp(self.x),
                                _dp(self.y), _dp(self.z))
        if rc != OK:
            raise IB3DError(rc, "ib3d_create failed (no CUDA device, bad grid or bad parameters)")
        self.nelems = 0

    # -- plumbing
    def _check(self, rc: int, what: str):
        if rc != OK:
            msg = self.L.ib3d_last_error(self._h)
            raise IB3DError(rc, f"{what}: {msg.decode() if msg else ''}")
        return rc

    def close(self):
        if self._h:
            self.L.ib3d_destroy(self._h)
            self._h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_params(self, params: Params | None = None, **kw):
        p = params if params is not None else self.params
        for k, v in kw.items():
            setattr(p, k, v)
        self._check(self.L.ib3d_set_params(self._h, C.byref(p)), "ib3d_set_params")
        self.params = p

    # -- set-up
    def set_mesh(self, nodes: np.ndarray, tris: np.ndarray, shift=(0.0, 0.0, 0.0), inor: int = 1):
        nodes = np.asarray(nodes, dtype=np.float64)
        tris = np.asarray(tris, dtype=np.int64)
        xn, yn, zn = (np.ascontiguousarray(nodes[:, q]) for q in range(3))
        e1, e2, e3 = (np.ascontiguousarray(tris[:, q]) for q in range(3))
        self._check(self.L.ib3d_set_mesh(self._h, len(nodes), _dp(xn), _dp(yn), _dp(zn), len(tris), _ip(e1), _ip(e2),
                                         _ip(e3), float(shift[0]), float(shift[1]), float(shift[2]), int(inor)),
                    "ib3d_set_mesh")
        self.nelems = len(tris)

    def search(self, box) -> dict:
        b = np.asarray(box, dtype=np.int64)
        counts = np.zeros(5, dtype=np.int64)
        self._check(self.L.ib3d_search(self._h, _ip(b), _ip(counts)), "ib3d_search")
        self.counts = dict(zip(("fluid", "solid", "ib", "red", "black"), (int(v) for v in counts)))
        return self.counts

    def selective_retag(self) -> dict:
        """selectiveRetagging: re-tag the 6^3 neighbourhoods of the current IB cells
        (after move_body, in place of search)."""
        counts = np.zeros(5, dtype=np.int64)
        self._check(self.L.ib3d_selective_retag(self._h, _ip(counts)), "ib3d_selective_retag")
        self.counts = dict(zip(("fluid", "solid", "ib", "red", "black"), (int(v) for v in counts)))
        return self.counts

    def set_poisson_coefficients(self, acx, acy, acz):
        """Replaces Acx/Acy/Acz ((n,3) arrays, the layout coefficientMatrix builds)."""
        a = [np.asfortranarray(v, dtype=np.float64) for v in (acx, acy, acz)]
        self._check(self.L.ib3d_set_poisson_coefficients(self._h, *(_dp(v) for v in a)),
                    "ib3d_set_poisson_coefficients")

    def write_restart(self, path, totime: float = 0.0, ita: int = 0, ita1: int = 0, text: bool = False):
        """Binary restart (or, text=True, the reference's formatted `result` file)."""
        fn = self.L.ib3d_write_result_text if text else self.L.ib3d_write_restart
        self._check(fn(self._h, str(path).encode(), float(totime), int(ita), int(ita1)), "write restart")

    def read_restart(self, path, text: bool = False) -> tuple:
        """Loads u, v, w, p (and ut = u ...); returns (totime, ita, ita1)."""
        t = np.zeros(1)
        it = np.zeros(2, dtype=np.int64)
        fn = self.L.ib3d_read_result_text if text else self.L.ib3d_read_restart
        self._check(fn(self._h, str(path).encode(), _dp(t), _ip(it[0:1]), _ip(it[1:2])), "read restart")
        return float(t[0]), int(it[0]), int(it[1])

    def move_body_free(self, fx: float, fy: float, fz: float) -> np.ndarray:
        """Force-driven motion (shiftSurfaceNodesMovingbody); returns the new body velocity."""
        v = np.zeros(3)
        self._check(self.L.ib3d_move_body_free(self._h, fx, fy, fz, _dp(v)), "ib3d_move_body_free")
        return v

    def set_mesh_file(self, path, fmt: int = 0, sur_geo_points: int = 0, shift=(0.0, 0.0, 0.0), inor: int = 1):
        self._check(self.L.ib3d_set_mesh_file(self._h, str(path).encode(), fmt, sur_geo_points, float(shift[0]),
                                              float(shift[1]), float(shift[2]), inor), "ib3d_set_mesh_file")

    def move_body(self, dx: float, dy: float, dz: float, us: float = 0.0, vs: float = 0.0, ws: float = 0.0):
        """Prescribed motion: shift the body, set its velocity; search again before stepping."""
        self._check(self.L.ib3d_move_body(self._h, dx, dy, dz, us, vs, ws), "ib3d_move_body")

    def get_search(self) -> dict:
        nib = self.counts["ib"]
        cell = np.zeros(self.shape, dtype=np.int64, order="F")
        ib = np.zeros((nib, 3), dtype=np.int64, order="F")
        nelp = np.zeros(nib, dtype=np.int64)
        nd = np.zeros((nib, 7), dtype=np.float64, order="F")
        self._check(self.L.ib3d_get_search(self._h, _ip(cell), _ip(ib), _ip(nelp), _dp(nd)), "ib3d_get_search")
        return {"cell": cell, "ib": ib, "nelp": nelp, "normdis": nd}

    def initial_conditions(self):
        self._check(self.L.ib3d_initial_conditions(self._h), "ib3d_initial_conditions")

    # -- fields
    def get_field(self, name: str) -> np.ndarray:
        out = np.empty(self.shape, dtype=np.float64, order="F")
        self._check(self.L.ib3d_get_field(self._h, FIELDS[name], _dp(out)), "ib3d_get_field")
        return out

    def set_field(self, name: str, arr: np.ndarray):
        a = np.asfortranarray(arr, dtype=np.float64)
        assert a.shape == self.shape
        self._check(self.L.ib3d_set_field(self._h, FIELDS[name], _dp(a)), "ib3d_set_field")

    def upload_fields(self, u=None, v=None, w=None, p=None):
        arrs = [None if a is None else np.asfortranarray(a, dtype=np.float64) for a in (u, v, w, p)]
        ptrs = [None if a is None else _dp(a) for a in arrs]
        self._check(self.L.ib3d_upload_fields(self._h, *ptrs), "ib3d_upload_fields")

    def download_fields(self, out: dict | None = None) -> dict:
        names = ("u", "v", "w", "ut", "vt", "wt", "p")
        out = out if out is not None else {n: np.empty(self.shape, dtype=np.float64, order="F") for n in names}
        self._check(self.L.ib3d_download_fields(self._h, *(_dp(out[n]) for n in names)), "ib3d_download_fields")
        return out

    def download_fields_async(self, out: dict) -> dict:
        """Starts the download of the seven fields into `out` (arrays that stay alive and
        unread until download_wait); returns at once."""
        names = ("u", "v", "w", "ut", "vt", "wt", "p")
        self._check(self.L.ib3d_download_fields_async(self._h, *(_dp(out[n]) for n in names)),
                    "ib3d_download_fields_async")
        return out

    def download_wait(self):
        self._check(self.L.ib3d_download_wait(self._h), "ib3d_download_wait")

    def device_field(self, name: str) -> int:
        return self.L.ib3d_device_field(self._h, FIELDS[name]) or 0

    def synchronize(self):
        self._check(self.L.ib3d_synchronize(self._h), "ib3d_synchronize")

    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        return self.L.ib3d_stream(self._h) or 0

    def enable_history(self):
        self._check(self.L.ib3d_enable_history(self._h), "ib3d_enable_history")

    def attach_net(self, net: "Net | None"):
        self._check(self.L.ib3d_attach_net(self._h, net._h if net is not None else None), "ib3d_attach_net")
        self._net = net

    def timers_enable(self, on: bool = True):
        self._check(self.L.ib3d_timers_enable(self._h, 1 if on else 0), "ib3d_timers_enable")

    def timers_read(self) -> dict:
        t = Timers()
        self._check(self.L.ib3d_timers_read(self._h, C.byref(t)), "ib3d_timers_read")
        return t.as_dict()

    # -- the reference's per-step calls (main.f90:46-66)
    def ns_momentum(self):
        self._check(self.L.ib3d_ns_momentum(self._h), "ib3d_ns_momentum")

    def velocity_bc(self):
        self._check(self.L.ib3d_velocity_bc(self._h), "ib3d_velocity_bc")

    def solid_cell_bc(self):
        self._check(self.L.ib3d_solid_cell_bc(self._h), "ib3d_solid_cell_bc")

    def velocity_forcing(self):
        self._check(self.L.ib3d_velocity_forcing(self._h), "ib3d_velocity_forcing")

    def pressure_forcing(self):
        self._check(self.L.ib3d_pressure_forcing(self._h), "ib3d_pressure_forcing")

    def poisson_solver(self, allow_noconv: bool = False) -> dict:
        st = SolveStats()
        rc = self.L.ib3d_poisson_solver(self._h, C.byref(st))
        if not (allow_noconv and rc == ERR_NOCONV):
            self._check(rc, "ib3d_poisson_solver")
        d = st.as_dict()
        d["rc"] = rc
        return d

    def ns_momentum_ab(self):
        self._check(self.L.ib3d_ns_momentum_ab(self._h), "ib3d_ns_momentum_ab")

    def calculate_uc(self) -> float:
        uc = np.zeros(1)
        self._check(self.L.ib3d_calculate_uc(self._h, _dp(uc)), "ib3d_calculate_uc")
        return float(uc[0])

    def redblack_sor(self, allow_noconv: bool = False) -> dict:
        """REDBLACKSOR alone on the b already set (set_field("b", ...))."""
        st = SolveStats()
        rc = self.L.ib3d_redblack_sor(self._h, C.byref(st))
        if not (allow_noconv and rc == ERR_NOCONV):
            self._check(rc, "ib3d_redblack_sor")
        d = st.as_dict()
        d["rc"] = rc
        return d

    def stress(self, first: bool) -> np.ndarray:
        coef = np.zeros(4, dtype=np.float64)
        self._check(self.L.ib3d_stress(self._h, 1 if first else 0, _dp(coef)), "ib3d_stress")
        return coef

    def step(self, first: bool, allow_noconv: bool = False):
        st = SolveStats()
        coef = np.zeros(4, dtype=np.float64)
        rc = self.L.ib3d_step(self._h, 1 if first else 0, C.byref(st), _dp(coef))
        if not (allow_noconv and rc == ERR_NOCONV):
            self._check(rc, "ib3d_step")
        d = st.as_dict()
        d["rc"] = rc
        return d, coef


class Net:
    """The learned warm start's 3-D U-Net (ib3d_net)."""

    def __init__(self, seed: int = 0):
        self.L = lib()
        self._h = _VP()
        rc = self.L.ib3d_net_create(C.byref(self._h), seed)
        if rc != OK:
            raise IB3DError(rc, "ib3d_net_create failed")
        self.nparams = int(self.L.ib3d_net_num_params(self._h))
        self.coarsen = 2

    def _check(self, rc: int, what: str):
        if rc != OK:
            msg = self.L.ib3d_net_last_error(self._h)
            raise IB3DError(rc, f"{what}: {msg.decode() if msg else ''}")

    def close(self):
        if self._h:
            self.L.ib3d_net_destroy(self._h)
            self._h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.nparams, np.float32)
        self._check(self.L.ib3d_net_get_params(self._h, out.ctypes.data_as(_F)), "ib3d_net_get_params")
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparams
        self._check(self.L.ib3d_net_set_params(self._h, p.ctypes.data_as(_F)), "ib3d_net_set_params")

    def loss_grad(self, x: np.ndarray, target: np.ndarray):
        """x: [B, S, S, S, 4] (z, y, x, channel: previous correction, b/dt, previous
        pressure, residual of the previous correction), target: [B, S, S, S]."""
        B, S = x.shape[0], x.shape[1]
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(target, dtype=np.float32)
        loss = np.zeros(1)
        grad = np.zeros(self.nparams, np.float32)
        out = np.zeros(t.shape, np.float32)
        self._check(self.L.ib3d_net_loss_grad(self._h, B, S, x.ctypes.data_as(_F), t.ctypes.data_as(_F),
                                              loss.ctypes.data_as(_D), grad.ctypes.data_as(_F),
                                              out.ctypes.data_as(_F)), "ib3d_net_loss_grad")
        return float(loss[0]), grad, out

    def reserve(self, patch: int, capacity: int):
        self._check(self.L.ib3d_net_dataset_reserve(self._h, patch, capacity), "ib3d_net_dataset_reserve")

    def set_coarsening(self, f: int):
        """1: full resolution; 2 (default): 2x2x2 cells per voxel; 4: 4x4x4."""
        self._check(self.L.ib3d_net_set_coarsening(self._h, f), "ib3d_net_set_coarsening")
        self.coarsen = f

    def dataset_size(self) -> int:
        return int(self.L.ib3d_net_dataset_size(self._h))

    def capture(self, solver: "Solver", npatches: int, seed: int = 0):
        self._check(self.L.ib3d_net_capture(self._h, solver._h, npatches, seed), "ib3d_net_capture")

    def set_wgrad_tensor_cores(self, on: bool = True):
        """Weight gradients on the tensor cores (default) or on the CUDA cores (reference)."""
        self._check(self.L.ib3d_net_set_wgrad_tensor_cores(self._h, 1 if on else 0),
                    "ib3d_net_set_wgrad_tensor_cores")

    def train(self, steps: int, batch: int = 8, lr: float = 1e-3, seed: int = 0) -> float:
        loss = np.zeros(1)
        self._check(self.L.ib3d_net_train(self._h, steps, batch, lr, seed, loss.ctypes.data_as(_D)), "ib3d_net_train")
        return float(loss[0])


def read_surface_mesh(path, fmt: int = 0, sur_geo_points: int = 0):
    """Nodes (N,3) and 1-based triangles (M,3) of a Gmsh 2 or Gambit surface mesh file."""
    L = lib()
    nn = np.zeros(1, np.int64)
    ne = np.zeros(1, np.int64)
    null = C.POINTER(C.c_double)()
    rc = L.ib3d_read_surface_mesh(str(path).encode(), fmt, sur_geo_points, _ip(nn), null, null, null, _ip(ne),
                                  C.POINTER(C.c_int64)(), C.POINTER(C.c_int64)(), C.POINTER(C.c_int64)())
    if rc != OK:
        raise IB3DError(rc, "ib3d_read_surface_mesh")
    xyz = [np.zeros(int(nn[0])) for _ in range(3)]
    e = [np.zeros(int(ne[0]), np.int64) for _ in range(3)]
    rc = L.ib3d_read_surface_mesh(str(path).encode(), fmt, sur_geo_points, _ip(nn), *(_dp(a) for a in xyz), _ip(ne),
                                  *(_ip(a) for a in e))
    if rc != OK:
        raise IB3DError(rc, "ib3d_read_surface_mesh")
    return np.stack(xyz, axis=1), np.stack(e, axis=1)


def setup_case(cs, params: Params | None = None, **kw) -> Solver:
    """Solver for a grids.Case: grid, icosphere body, search and initial conditions."""
    p = params if params is not None else default_params(re=cs.re, deltat=cs.dt, omega=cs.omega, eps=cs.eps)
    for k, v in kw.items():
        setattr(p, k, v)
    s = Solver(cs.x, cs.y, cs.z, p)
    nodes, tris = grids.icosphere(cs.subdivisions, cs.radius)
    s.set_mesh(nodes, tris)
    s.search(cs.box)
    s.initial_conditions()
    return s


def build(verbose: bool = False):
    from . import buildlib as _b
    return _b.build(verbose=verbose)
