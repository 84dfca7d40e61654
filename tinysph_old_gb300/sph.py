"""Python front-end of the C ABI (``include/tsph.h``), shaped like the
reference's interface: a particle system object plus free functions named
after the reference functions they replace (``Divide_To_Cells``,
``Particle_To_Cell``, ``Compute_Forces``, ...).

There is no fallback: if ``libtsph.so`` cannot be loaded (or built) every
call raises, and every non-zero status of the library raises
:class:`TsphError`.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

# status codes (tsph.h)
N_TILE_SHAPES = 3  # pair-kernel variants (TSPH_N_TILE_SHAPES)
TILE_SHAPES = {"wide": 0, "deep": 1, "rec": 2}
OK, ERR_ARG, ERR_CUDA, ERR_STATE, ERR_NOMEM, ERR_NUMERIC, ERR_DENSITY, ERR_ESCAPED, \
    ERR_UNSUPPORTED = range(9)
FLUID, WALL = 0, 1
WALL_MDBC, WALL_DBC, WALL_BT = 0, 1, 2
PREC_FP32, PREC_FP64 = 0, 1
F_R, F_V, F_A, F_RHO, F_DRHO, F_P, F_INDEX, F_TYPE = (1 << k for k in range(8))
F_ALL = F_R | F_V | F_A | F_RHO | F_DRHO | F_P | F_INDEX | F_TYPE
HEALTH_NAN, HEALTH_DENSITY, HEALTH_ESCAPED, HEALTH_REMOVED = 1, 2, 4, 8
HEALTH_STALL, HEALTH_UPLOAD = 0x10, 0x20

# the C entry points declared in include/tsph.h
ABI_SYMBOLS = (
    "tsph_abi_version", "tsph_last_error", "tsph_status_string", "tsph_device_count",
    "tsph_create", "tsph_destroy", "tsph_add_particles", "tsph_np", "tsph_grid",
    "tsph_particle_mass", "tsph_divide_to_cells", "tsph_clear_cells", "tsph_particle_to_cell",
    "tsph_get_cells", "tsph_pair_digest", "tsph_grid_tables", "tsph_particle_to_cell_noalloc",
    "tsph_density_to_pressure", "tsph_mdbc_density", "tsph_bt_density",
    "tsph_add_buffer_zone", "tsph_set_zone_capacity", "tsph_bz_inlet", "tsph_bz_outlet",
    "tsph_compute_forces", "tsph_symplectic_predictor", "tsph_symplectic_corrector",
    "tsph_remove_out_of_domain", "tsph_step", "tsph_download", "tsph_upload", "tsph_sync",
    "tsph_download_async", "tsph_download_wait", "tsph_upload_async",
    "tsph_health", "tsph_kernel_launches", "tsph_fluid_totals", "tsph_set_profiling",
    "tsph_get_profile",
    "tsph_water_level", "tsph_point_fields", "tsph_water_front", "tsph_autotune",
    "tsph_set_tile_shape", "tsph_get_tile_shape", "tsph_set_cases", "tsph_write_vtk", "tsph_save_checkpoint", "tsph_load_checkpoint",
    "tsph_export_graph", "tsph_apply_update", "tsph_window_check", "tsph_get_stream",
    "tsph_state_save", "tsph_state_restore", "tsph_gnn_n_params", "tsph_gnn_create",
    "tsph_gnn_destroy", "tsph_gnn_set_params", "tsph_gnn_get_params", "tsph_gnn_get_grads",
    "tsph_gnn_forward", "tsph_gnn_infer", "tsph_gnn_loss_grad", "tsph_gnn_adam",
    "tsph_ale_create", "tsph_ale_destroy", "tsph_ale_add_particles", "tsph_ale_set_scheme",
    "tsph_ale_set_keep_cells", "tsph_ale_sort_count",
    "tsph_ale_np", "tsph_ale_divide_to_cells", "tsph_ale_particle_to_cell", "tsph_ale_gradient",
    "tsph_ale_forces", "tsph_ale_leapfrog_one", "tsph_ale_leapfrog_two", "tsph_ale_step",
    "tsph_ale_download", "tsph_ale_upload", "tsph_ale_sync", "tsph_ale_health",
    "tsph_ale_download_async", "tsph_ale_download_wait", "tsph_ale_upload_async",
)

ALE_AS_WRITTEN = 0
ALE_MUSCL = 1
ALE_FIRST_ORDER = 2
(ALE_F_R, ALE_F_V, ALE_F_RHO, ALE_F_P, ALE_F_OMEGA, ALE_F_OMEGARHO, ALE_F_OMEGAV, ALE_F_RATES,
 ALE_F_GRAD, ALE_F_INDEX, ALE_F_TYPE) = (1 << k for k in range(11))
ALE_F_ALL = (1 << 11) - 1


class TsphError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"tsph status {status}: {message}")
        self.status = status


class _Constants(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("h", "kap", "cs", "rho0", "visco", "delta", "dp")]


class _Domain(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("x_0", "x_m", "y_0", "y_m")]


class _HostState(C.Structure):
    _fields_ = [("r", C.c_void_p), ("v", C.c_void_p), ("a", C.c_void_p), ("rho", C.c_void_p),
                ("drho", C.c_void_p), ("p", C.c_void_p), ("index", C.c_void_p),
                ("type", C.c_void_p)]


class _AleHostState(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("r", "v", "rho", "p", "omega", "omegarho", "omegav",
                                          "domega", "domegarho", "domegav", "grad", "index",
                                          "type")]


class GnnGraph(C.Structure):
    """tsph_gnn_graph: device pointers of an exported particle graph."""
    _fields_ = [("pos", C.c_void_p), ("vel", C.c_void_p), ("srho", C.c_void_p),
                ("wall", C.c_void_p), ("deg", C.c_void_p), ("nbr", C.c_void_p),
                ("n_nodes", C.c_int32), ("k_slots", C.c_int32), ("h", C.c_double),
                ("u_scale", C.c_double), ("s_scale", C.c_double)]


class _Profile(C.Structure):
    _fields_ = [("pair_us", C.c_double), ("pair_launches", C.c_int),
                ("sort_us", C.c_double), ("sort_launches", C.c_int),
                ("mdbc_us", C.c_double), ("mdbc_launches", C.c_int),
                ("other_us", C.c_double), ("other_launches", C.c_int)]


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load ``libtsph.so`` (building it with nvcc if it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise RuntimeError(f"{_build.LIB} is missing: run tinysph_old_gb300/build.py")
    L = C.CDLL(_build.LIB)
    P, I, D = C.c_void_p, C.c_int, C.c_double
    L.tsph_abi_version.restype = I
    L.tsph_last_error.restype = C.c_char_p
    L.tsph_status_string.restype = C.c_char_p
    L.tsph_status_string.argtypes = [I]
    L.tsph_device_count.argtypes = [C.POINTER(I)]
    L.tsph_create.argtypes = [C.POINTER(_Constants), C.POINTER(_Domain), I, P, C.POINTER(P)]
    L.tsph_destroy.argtypes = [P]
    L.tsph_add_particles.argtypes = [P, I, P, P, P, P, P, P]
    L.tsph_np.argtypes = [P, C.POINTER(I)]
    L.tsph_grid.argtypes = [P, C.POINTER(I), C.POINTER(I)]
    L.tsph_particle_mass.argtypes = [P, C.POINTER(D)]
    for f in ("tsph_divide_to_cells", "tsph_clear_cells", "tsph_particle_to_cell",
              "tsph_density_to_pressure", "tsph_mdbc_density", "tsph_bt_density", "tsph_sync"):
        getattr(L, f).argtypes = [P]
    L.tsph_get_cells.argtypes = [P, P, P]
    L.tsph_pair_digest.argtypes = [P, P, P, P]
    L.tsph_grid_tables.argtypes = [C.POINTER(_Constants), C.POINTER(_Domain), C.POINTER(I),
                                   C.POINTER(I), P, P]
    L.tsph_particle_to_cell_noalloc.argtypes = [C.POINTER(_Constants), C.POINTER(_Domain), I, P,
                                                P, P, P, C.POINTER(I)]
    L.tsph_compute_forces.argtypes = [P, I]
    L.tsph_add_buffer_zone.argtypes = [P, D, D, D, D, I, D, D, D, D, I]
    L.tsph_set_zone_capacity.argtypes = [P, I, I]
    L.tsph_bz_inlet.argtypes = [P, I, D]
    L.tsph_bz_outlet.argtypes = [P, I, D]
    L.tsph_symplectic_predictor.argtypes = [P, D]
    L.tsph_symplectic_corrector.argtypes = [P, D]
    L.tsph_remove_out_of_domain.argtypes = [P, C.POINTER(I)]
    L.tsph_step.argtypes = [P, I, D, I]
    L.tsph_download.argtypes = [P, I, C.POINTER(_HostState)]
    L.tsph_upload.argtypes = [P, I, C.POINTER(_HostState)]
    L.tsph_download_async.argtypes = [P, I, C.POINTER(_HostState)]
    L.tsph_download_wait.argtypes = [P]
    L.tsph_upload_async.argtypes = [P, I, C.POINTER(_HostState)]
    L.tsph_health.argtypes = [P, C.POINTER(C.c_uint32), I]
    L.tsph_kernel_launches.argtypes = [P, C.POINTER(C.c_longlong), I]
    L.tsph_fluid_totals.argtypes = [P, P]
    L.tsph_set_profiling.argtypes = [P, I]
    L.tsph_get_profile.argtypes = [P, C.POINTER(_Profile), I]
    L.tsph_water_level.argtypes = [P, I, P, P, P, P]
    L.tsph_point_fields.argtypes = [P, I, P, P]
    L.tsph_water_front.argtypes = [P, D, C.POINTER(D)]
    L.tsph_autotune.argtypes = [P, P, P]
    L.tsph_set_tile_shape.argtypes = [P, I]
    L.tsph_get_tile_shape.argtypes = [P, P]
    L.tsph_set_cases.argtypes = [P, I, P, P, P]
    L.tsph_write_vtk.argtypes = [P, C.c_char_p]
    L.tsph_export_graph.argtypes = [P, I, I] + [P] * 9 + [C.POINTER(C.c_int32)] * 2
    L.tsph_apply_update.argtypes = [P, P, D, D, D, I, I]
    L.tsph_window_check.argtypes = [P, D, C.POINTER(C.c_double)]
    L.tsph_get_stream.argtypes = [P, C.POINTER(P)]
    L.tsph_state_save.argtypes = [P]
    L.tsph_state_restore.argtypes = [P]
    L.tsph_gnn_n_params.restype = I
    L.tsph_gnn_create.argtypes = [I, P, C.POINTER(P)]
    L.tsph_gnn_destroy.argtypes = [P]
    L.tsph_gnn_set_params.argtypes = [P, P]
    L.tsph_gnn_get_params.argtypes = [P, P]
    L.tsph_gnn_get_grads.argtypes = [P, P]
    L.tsph_gnn_forward.argtypes = [P, C.POINTER(GnnGraph), P]
    L.tsph_gnn_infer.argtypes = [P, C.POINTER(GnnGraph), P]
    L.tsph_gnn_loss_grad.argtypes = [P, C.POINTER(GnnGraph), P, C.POINTER(D)]
    L.tsph_gnn_adam.argtypes = [P, D, D, D, D]
    L.tsph_save_checkpoint.argtypes = [P, C.c_char_p]
    L.tsph_load_checkpoint.argtypes = [C.c_char_p, P, C.POINTER(P)]
    L.tsph_ale_create.argtypes = [C.POINTER(_Constants), C.POINTER(_Domain), P, C.POINTER(P)]
    for f in ("tsph_ale_destroy", "tsph_ale_divide_to_cells", "tsph_ale_particle_to_cell",
              "tsph_ale_gradient", "tsph_ale_sync"):
        getattr(L, f).argtypes = [P]
    L.tsph_ale_add_particles.argtypes = [P, I, P, P, P, P, P, P]
    L.tsph_ale_set_scheme.argtypes = [P, I]
    L.tsph_ale_set_keep_cells.argtypes = [P, I]
    L.tsph_ale_sort_count.argtypes = [P, C.POINTER(C.c_longlong)]
    L.tsph_ale_np.argtypes = [P, C.POINTER(I)]
    L.tsph_ale_forces.argtypes = [P, D]
    L.tsph_ale_leapfrog_one.argtypes = [P, D]
    L.tsph_ale_leapfrog_two.argtypes = [P, D, I]
    L.tsph_ale_step.argtypes = [P, D, I, I]
    L.tsph_ale_download.argtypes = [P, I, C.POINTER(_AleHostState)]
    L.tsph_ale_upload.argtypes = [P, I, C.POINTER(_AleHostState)]
    L.tsph_ale_download_async.argtypes = [P, I, C.POINTER(_AleHostState)]
    L.tsph_ale_download_wait.argtypes = [P]
    L.tsph_ale_upload_async.argtypes = [P, I, C.POINTER(_AleHostState)]
    L.tsph_ale_health.argtypes = [P, C.POINTER(C.c_uint32), I]
    _lib = L
    return L


def device_count() -> int:
    n = C.c_int(0)
    load().tsph_device_count(C.byref(n))
    return n.value


def grid_tables(h, kap, domain):
    """Host-only: (ncx, ncy, bx, by) of ``tsph_grid_tables`` (no GPU needed)."""
    L = load()
    c = _Constants(h, kap, 1.0, 1000.0, 0.0, 0.0, h)
    d = _Domain(*domain)
    ncx, ncy = C.c_int(), C.c_int()
    _check(L.tsph_grid_tables(C.byref(c), C.byref(d), C.byref(ncx), C.byref(ncy), None, None))
    bx = np.empty(ncx.value + 1, dtype=np.int64)
    by = np.empty(ncy.value + 1, dtype=np.int64)
    _check(L.tsph_grid_tables(C.byref(c), C.byref(d), C.byref(ncx), C.byref(ncy), _p(bx), _p(by)))
    return ncx.value, ncy.value, bx, by


def _check(rc: int):
    if rc != OK:
        msg = load().tsph_last_error().decode(errors="replace")
        raise TsphError(rc, msg)


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class ParticleSystem:
    """``Particle_system`` + ``Simulation_data`` on the GPU (src/SPH_particle_system.h,
    src/SPH_data.h).  ``precision`` is ``"fp32"`` (FP32 pair math, FP64
    positions) or ``"fp64"``."""

    def __init__(self, h, kap, cs, rho0, visco, delta, dp, domain, precision="fp32",
                 stream=None):
        L = load()
        self._L = L
        c = _Constants(h, kap, cs, rho0, visco, delta, dp)
        d = _Domain(*domain)
        prec = {"fp32": PREC_FP32, "fp64": PREC_FP64}[precision]
        h_ = C.c_void_p()
        _check(L.tsph_create(C.byref(c), C.byref(d), prec, stream, C.byref(h_)))
        self._h = h_
        self.precision = precision
        self.domain = tuple(domain)

    @classmethod
    def from_case(cls, case, precision="fp32", divide=True, bin_particles=True):
        """Build a system from a :class:`tinysph_old_gb300.cases.Case` (INIT of the
        reference drivers: add particles, Divide_To_Cells, Particle_To_Cell)."""
        s = cls(case.h, case.kap, case.cs, case.rho0, case.visco, case.delta, case.dp,
                case.domain, precision)
        a = case.particles.arrays()
        gnr = np.zeros((case.np, 2))
        gn = a["gnr"]
        if len(gn):
            # the reference indexes gnr by particle index (walls first)
            gnr[:len(gn)] = gn
        s.add_particles(a["type"], a["r"], a["v"], a["rho"], a["p"], gnr if len(gn) else None)
        for z in case.meta.get("zones", []):
            s.add_buffer_zone(**z)
        if divide:
            s.divide_to_cells()
            if bin_particles:
                s.particle_to_cell()
        return s

    def close(self):
        if getattr(self, "_h", None):
            self._L.tsph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- particles
    def add_particles(self, ptype, r, v=None, rho=None, p=None, gnr=None):
        n = len(ptype)
        t = np.ascontiguousarray(ptype, dtype=np.int32)
        r = np.ascontiguousarray(r, dtype=np.float64).reshape(n, 2)
        v = None if v is None else np.ascontiguousarray(v, dtype=np.float64).reshape(n, 2)
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        p = None if p is None else np.ascontiguousarray(p, dtype=np.float64)
        g = None if gnr is None else np.ascontiguousarray(gnr, dtype=np.float64).reshape(n, 2)
        _check(self._L.tsph_add_particles(self._h, n, _p(t), _p(r), _p(v), _p(rho), _p(p), _p(g)))

    @property
    def np(self) -> int:
        n = C.c_int()
        _check(self._L.tsph_np(self._h, C.byref(n)))
        return n.value

    def grid(self):
        a, b = C.c_int(), C.c_int()
        _check(self._L.tsph_grid(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    @property
    def mass(self) -> float:
        m = C.c_double()
        _check(self._L.tsph_particle_mass(self._h, C.byref(m)))
        return m.value

    # ---- find pairs
    def divide_to_cells(self):
        _check(self._L.tsph_divide_to_cells(self._h))

    def clear_cells(self):
        _check(self._L.tsph_clear_cells(self._h))

    def particle_to_cell(self):
        _check(self._L.tsph_particle_to_cell(self._h))

    def get_cells(self):
        ncx, ncy = self.grid()
        start = np.empty(ncx * ncy + 1, dtype=np.int32)
        lst = np.empty(max(self.np, 1), dtype=np.int32)
        _check(self._L.tsph_get_cells(self._h, _p(start), _p(lst)))
        return start, lst[:start[-1]]

    def pair_digest(self):
        n = self.np
        cnt = np.empty(n, dtype=np.int32)
        sm = np.empty(n, dtype=np.int64)
        xr = np.empty(n, dtype=np.int32)
        _check(self._L.tsph_pair_digest(self._h, _p(cnt), _p(sm), _p(xr)))
        return cnt, sm, xr

    # ---- physics
    def density_to_pressure(self):
        _check(self._L.tsph_density_to_pressure(self._h))

    def mdbc_density(self):
        _check(self._L.tsph_mdbc_density(self._h))

    def add_buffer_zone(self, x0, xm, y0, ym, nbl, vx, vy, ox, oy, btype):
        """A buffer zone (tsph_add_buffer_zone; before the first step)."""
        _check(self._L.tsph_add_buffer_zone(self._h, x0, xm, y0, ym, int(nbl), vx, vy, ox, oy,
                                            int(btype)))

    def set_zone_capacity(self, extra_rows, extra_ids):
        _check(self._L.tsph_set_zone_capacity(self._h, int(extra_rows), int(extra_ids)))

    def bz_inlet(self, zone, dt):
        _check(self._L.tsph_bz_inlet(self._h, int(zone), float(dt)))

    def bz_outlet(self, zone, dt):
        _check(self._L.tsph_bz_outlet(self._h, int(zone), float(dt)))

    def bt_density(self):
        """BT_compute_density_BTGeo (src/SPH_BT.h)."""
        _check(self._L.tsph_bt_density(self._h))

    def compute_forces(self, wall_model=WALL_MDBC):
        _check(self._L.tsph_compute_forces(self._h, int(wall_model)))

    def predictor(self, dt):
        _check(self._L.tsph_symplectic_predictor(self._h, float(dt)))

    def corrector(self, dt):
        _check(self._L.tsph_symplectic_corrector(self._h, float(dt)))

    def remove_out_of_domain(self) -> int:
        n = C.c_int()
        _check(self._L.tsph_remove_out_of_domain(self._h, C.byref(n)))
        return n.value

    def step(self, wall_model, dt, nsteps=1):
        _check(self._L.tsph_step(self._h, int(wall_model), float(dt), int(nsteps)))

    # ---- state
    def download(self, fields=F_ALL, out=None):
        """State in the reference's order as a dict of numpy arrays."""
        n = self.np
        res = {} if out is None else out
        spec = [(F_R, "r", (n, 2), np.float64), (F_V, "v", (n, 2), np.float64),
                (F_A, "a", (n, 2), np.float64), (F_RHO, "rho", (n,), np.float64),
                (F_DRHO, "drho", (n,), np.float64), (F_P, "p", (n,), np.float64),
                (F_INDEX, "index", (n,), np.int32), (F_TYPE, "type", (n,), np.int32)]
        hs = _HostState()
        for bit, name, shape, dt in spec:
            if fields & bit:
                if name not in res:
                    res[name] = np.empty(shape, dtype=dt)
                setattr(hs, name, res[name].ctypes.data)
        _check(self._L.tsph_download(self._h, int(fields), C.byref(hs)))
        return res

    def upload(self, **fields):
        hs = _HostState()
        mask = 0
        keep = []
        bits = dict(r=F_R, v=F_V, a=F_A, rho=F_RHO, drho=F_DRHO, p=F_P)
        for name, arr in fields.items():
            if arr is None:
                continue
            a = np.ascontiguousarray(arr, dtype=np.float64)
            keep.append(a)
            setattr(hs, name, a.ctypes.data)
            mask |= bits[name]
        _check(self._L.tsph_upload(self._h, mask, C.byref(hs)))

    def upload_ptrs(self, mask, **ptrs):
        """Upload from raw host pointers (e.g. pinned buffers)."""
        hs = _HostState()
        for k, v in ptrs.items():
            setattr(hs, k, v)
        _check(self._L.tsph_upload(self._h, int(mask), C.byref(hs)))

    def download_ptrs(self, mask, **ptrs):
        hs = _HostState()
        for k, v in ptrs.items():
            setattr(hs, k, v)
        _check(self._L.tsph_download(self._h, int(mask), C.byref(hs)))

    def download_async(self, mask, **ptrs):
        """Start a download into raw host pointers (pinned buffers, kept
        valid until download_wait); r, v, a, rho, drho and p only."""
        hs = _HostState()
        for k, v in ptrs.items():
            setattr(hs, k, v)
        _check(self._L.tsph_download_async(self._h, int(mask), C.byref(hs)))

    def download_wait(self):
        _check(self._L.tsph_download_wait(self._h))

    def upload_async(self, mask, **ptrs):
        """Stage an upload from raw host pointers (pinned buffers, kept valid
        until particle_to_cell, which applies it); r, v, a, rho, drho, p."""
        hs = _HostState()
        for k, v in ptrs.items():
            setattr(hs, k, v)
        _check(self._L.tsph_upload_async(self._h, int(mask), C.byref(hs)))

    def sync(self):
        _check(self._L.tsph_sync(self._h))

    def kernel_launches(self, reset=False) -> int:
        """Kernels launched for this system (graph steps counted per kernel,
        the conditional re-binning only when it ran)."""
        n = C.c_longlong()
        _check(self._L.tsph_kernel_launches(self._h, C.byref(n), 1 if reset else 0))
        return n.value

    def health(self, clear=False) -> int:
        f = C.c_uint32()
        _check(self._L.tsph_health(self._h, C.byref(f), 1 if clear else 0))
        return f.value

    def fluid_totals(self):
        out = np.zeros(4)
        _check(self._L.tsph_fluid_totals(self._h, _p(out)))
        return dict(mass=out[0], ekin=out[1], px=out[2], py=out[3])

    # ---- probes (src/SPH_water_level.h, src/testing.h)
    def water_level(self, x, y0, inverse=None):
        """Water_Elevation (inverse=False) / Water_Elevation_inverse at gauges."""
        x = np.ascontiguousarray(np.atleast_1d(x), dtype=np.float64)
        y0 = np.ascontiguousarray(np.broadcast_to(y0, x.shape), dtype=np.float64)
        inv = None
        if inverse is not None:
            inv = np.ascontiguousarray(np.broadcast_to(inverse, x.shape), dtype=np.int32)
        out = np.empty(len(x))
        _check(self._L.tsph_water_level(self._h, len(x), _p(x), _p(y0), _p(inv), _p(out)))
        return out

    def point_fields(self, xy):
        """Shepard {rho, p, vx, vy} at points (n, 2); Pressure_in_point = [:, 1]."""
        xy = np.ascontiguousarray(np.asarray(xy, dtype=np.float64).reshape(-1, 2))
        out = np.empty((len(xy), 4))
        _check(self._L.tsph_point_fields(self._h, len(xy), _p(xy), _p(out)))
        return out

    def water_front(self, y_max):
        x = C.c_double()
        _check(self._L.tsph_water_front(self._h, float(y_max), C.byref(x)))
        return x.value

    def write_vtk(self, path):
        """write_to_ASCII_VTK (src/SPH_data_to_vtk.h)."""
        _check(self._L.tsph_write_vtk(self._h, os.fsencode(path)))

    def save_checkpoint(self, path):
        _check(self._L.tsph_save_checkpoint(self._h, os.fsencode(path)))

    @classmethod
    def load_checkpoint(cls, path, stream=None):
        """A new system restarted from a checkpoint."""
        L = load()
        h_ = C.c_void_p()
        _check(L.tsph_load_checkpoint(os.fsencode(path), stream, C.byref(h_)))
        s = cls.__new__(cls)
        s._L = L
        s._h = h_
        s.precision = None
        s.domain = None
        return s

    def export_graph(self, k_slots, capacity, pos, vel, srho, wall, id_, deg, nbr, acc=None,
                     rate=None):
        """Device pointers (ints) -> (n_nodes, n_wall); see tsph_export_graph."""
        n, nw = C.c_int32(), C.c_int32()
        _check(self._L.tsph_export_graph(self._h, int(k_slots), int(capacity), pos, vel, srho,
                                         wall, id_, deg, nbr, acc, rate, C.byref(n),
                                         C.byref(nw)))
        return n.value, nw.value

    def apply_update(self, y, u_scale, s_scale, k_dt, add_rates=True, phase=0,
                     zero_momentum=False):
        """The surrogate's window update from the device array y (3 floats per
        node of the last export); phase 0 explicit, 1 kick, 2 drift; see
        tsph_apply_update."""
        flags = (1 if add_rates else 0) | (2 if zero_momentum else 0)
        _check(self._L.tsph_apply_update(self._h, y, float(u_scale), float(s_scale), float(k_dt),
                                         flags, int(phase)))

    def window_check(self, k_dt):
        """(max, rms) density error / rho0, the momentum error, the count and
        the worst particle of the last window; see tsph_window_check."""
        out = (C.c_double * 5)()
        _check(self._L.tsph_window_check(self._h, float(k_dt), out))
        return out[0], out[1], out[2], int(out[3]), int(out[4])

    def stream_ptr(self):
        """The CUDA stream (as an int) the system's kernels run on."""
        p = C.c_void_p()
        _check(self._L.tsph_get_stream(self._h, C.byref(p)))
        return p.value

    def state_save(self):
        _check(self._L.tsph_state_save(self._h))

    def state_restore(self):
        _check(self._L.tsph_state_restore(self._h))

    def autotune(self):
        """Time every variant of the pair kernel, keep the fastest:
        (variant, [median us of each variant])."""
        c = C.c_int32()
        us = np.zeros(N_TILE_SHAPES)
        _check(self._L.tsph_autotune(self._h, C.byref(c), _p(us)))
        return c.value, us

    def set_tile_shape(self, shape: int):
        _check(self._L.tsph_set_tile_shape(self._h, int(shape)))

    def set_cases(self, x_range, gravity, removal):
        """Cases packed into this system (tsph_set_cases): per case the x
        range [lo, hi) of its columns, its gravity and its removal thresholds
        (x_lo, x_hi, y_lo, y_hi); before particle_to_cell."""
        xr = np.ascontiguousarray(x_range, dtype=np.float64).reshape(-1, 2)
        g = np.ascontiguousarray(gravity, dtype=np.float64).reshape(-1)
        bx = np.ascontiguousarray(removal, dtype=np.float64).reshape(-1, 4)
        if not (len(xr) == len(g) == len(bx)):
            raise ValueError("one x range, gravity and removal box per case")
        _check(self._L.tsph_set_cases(self._h, len(g), _p(xr), _p(g), _p(bx)))

    @property
    def tile_shape(self) -> int:
        """The pair-kernel variant in use (-1 before the first step)."""
        c = C.c_int32()
        _check(self._L.tsph_get_tile_shape(self._h, C.byref(c)))
        return c.value

    def set_profiling(self, on: bool):
        _check(self._L.tsph_set_profiling(self._h, 1 if on else 0))

    def profile(self, reset=True):
        p = _Profile()
        _check(self._L.tsph_get_profile(self._h, C.byref(p), 1 if reset else 0))
        return {k: getattr(p, k) for k, _ in _Profile._fields_}


# ---- free functions under the reference's names (src/*.h)
def Divide_To_Cells(particles: ParticleSystem, simulation_data=None):
    particles.divide_to_cells()


def Clear_cells(particles: ParticleSystem):
    particles.clear_cells()


def Particle_To_Cell(particles: ParticleSystem, simulation_data=None):
    particles.particle_to_cell()


def Density_to_pressure(particles: ParticleSystem):
    particles.density_to_pressure()


def mDBC_compute_density_mdbcGeo(particles: ParticleSystem, simulation_data=None):
    particles.mdbc_density()


def Compute_Forces(particles: ParticleSystem, wall_model=WALL_MDBC):
    particles.compute_forces(wall_model)


def Integrate_SymplecticPredictor(particles: ParticleSystem, dt):
    particles.predictor(dt)


def Integrate_SymplecticCorrector(particles: ParticleSystem, dt):
    particles.corrector(dt)


def RemoveParticlesOutOfDomain(particles: ParticleSystem, simulation_data=None) -> int:
    return particles.remove_out_of_domain()


def Water_Elevation(particles: ParticleSystem, simulation_data, x, y0) -> float:
    return float(particles.water_level(x, y0, 0)[0])


def Water_Elevation_inverse(particles: ParticleSystem, simulation_data, x, y0) -> float:
    return float(particles.water_level(x, y0, 1)[0])


def Pressure_in_point(particles: ParticleSystem, simulation_data, ar) -> float:
    return float(particles.point_fields([ar])[0, 1])


class AleSystem:
    """Riemann / ALE-SPH ``Particle_system`` on the GPU (the path of
    cases/ALESPH_dambreakLong/MUSCL.h): leap-frog in omega, omega*rho,
    omega*v (src/RALESPH_integration.h), one-sided MUSCL gradients and the
    linearised-Riemann flux loop (src/_testMUSCL_interaction.h); BT walls with
    a normal each.  ``scheme`` is :data:`ALE_AS_WRITTEN` (the reference's
    MUSCL.h fluxes), :data:`ALE_MUSCL` or :data:`ALE_FIRST_ORDER` (the
    SPH_simulationINT.h driver, src/RALESPH_interaction.h)."""

    def __init__(self, h, kap, cs, rho0, visco, delta, dp, domain, stream=None):
        L = load()
        self._L = L
        c = _Constants(h, kap, cs, rho0, visco, delta, dp)
        d = _Domain(*domain)
        h_ = C.c_void_p()
        _check(L.tsph_ale_create(C.byref(c), C.byref(d), stream, C.byref(h_)))
        self._h = h_
        self.domain = tuple(domain)

    @classmethod
    def from_case(cls, case, scheme=ALE_AS_WRITTEN, divide=True, bin_particles=True):
        """INIT of the ALE driver: ALESPH_Add_particle for every particle
        (normals of the walls from the generators), Divide_To_Cells,
        Particle_To_Cell."""
        s = cls(case.h, case.kap, case.cs, case.rho0, case.visco, case.delta, case.dp,
                case.domain)
        a = case.particles.arrays()
        nrm = np.zeros((case.np, 2))
        nn = np.asarray(case.particles.normals, dtype=np.float64).reshape(-1, 2)
        # special.n is indexed by particle index: walls come first
        nrm[:len(nn)] = nn
        s.add_particles(a["type"], a["r"], a["v"], a["rho"], a["p"], nrm)
        s.set_scheme(scheme)
        if divide:
            s.divide_to_cells()
            if bin_particles:
                s.particle_to_cell()
        return s

    def close(self):
        if getattr(self, "_h", None):
            self._L.tsph_ale_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add_particles(self, ptype, r, v=None, rho=None, p=None, normal=None):
        n = len(ptype)
        t = np.ascontiguousarray(ptype, dtype=np.int32)
        r = np.ascontiguousarray(r, dtype=np.float64).reshape(n, 2)
        v = None if v is None else np.ascontiguousarray(v, dtype=np.float64).reshape(n, 2)
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        p = None if p is None else np.ascontiguousarray(p, dtype=np.float64)
        nr = None if normal is None else np.ascontiguousarray(normal, dtype=np.float64).reshape(n, 2)
        _check(self._L.tsph_ale_add_particles(self._h, n, _p(t), _p(r), _p(v), _p(rho), _p(p),
                                              _p(nr)))

    def set_scheme(self, scheme):
        _check(self._L.tsph_ale_set_scheme(self._h, int(scheme)))

    def set_keep_cells(self, on: bool):
        """Kept cells for :meth:`step` (default on): the sort runs only when a
        particle moved more than the skin since its binning or left the
        domain; off, every step sorts (the reference's cell order)."""
        _check(self._L.tsph_ale_set_keep_cells(self._h, 1 if on else 0))

    def sort_count(self) -> int:
        """Sorts that :meth:`step` ran on kept cells since the system was built."""
        n = C.c_longlong()
        _check(self._L.tsph_ale_sort_count(self._h, C.byref(n)))
        return int(n.value)

    @property
    def np(self) -> int:
        n = C.c_int()
        _check(self._L.tsph_ale_np(self._h, C.byref(n)))
        return n.value

    def divide_to_cells(self):
        _check(self._L.tsph_ale_divide_to_cells(self._h))

    def particle_to_cell(self):
        _check(self._L.tsph_ale_particle_to_cell(self._h))

    def gradient(self):
        _check(self._L.tsph_ale_gradient(self._h))

    def forces(self, dt):
        _check(self._L.tsph_ale_forces(self._h, float(dt)))

    def leapfrog_one(self, dt):
        _check(self._L.tsph_ale_leapfrog_one(self._h, float(dt)))

    def leapfrog_two(self, dt, step):
        _check(self._L.tsph_ale_leapfrog_two(self._h, float(dt), int(step)))

    def step(self, dt, step0, nsteps=1):
        _check(self._L.tsph_ale_step(self._h, float(dt), int(step0), int(nsteps)))

    def download(self, fields=ALE_F_ALL):
        """State in the reference's order as a dict of numpy arrays."""
        n = self.np
        spec = [(ALE_F_R, "r", (n, 2), np.float64), (ALE_F_V, "v", (n, 2), np.float64),
                (ALE_F_RHO, "rho", (n,), np.float64), (ALE_F_P, "p", (n,), np.float64),
                (ALE_F_OMEGA, "omega", (n,), np.float64),
                (ALE_F_OMEGARHO, "omegarho", (n,), np.float64),
                (ALE_F_OMEGAV, "omegav", (n, 2), np.float64),
                (ALE_F_RATES, "domega", (n,), np.float64),
                (ALE_F_RATES, "domegarho", (n,), np.float64),
                (ALE_F_RATES, "domegav", (n, 2), np.float64),
                (ALE_F_GRAD, "grad", (n, 12), np.float64),
                (ALE_F_INDEX, "index", (n,), np.int32), (ALE_F_TYPE, "type", (n,), np.int32)]
        hs = _AleHostState()
        res = {}
        for bit, name, shape, dt in spec:
            if fields & bit:
                res[name] = np.empty(shape, dtype=dt)
                setattr(hs, name, res[name].ctypes.data)
        _check(self._L.tsph_ale_download(self._h, int(fields), C.byref(hs)))
        return res

    def upload(self, r=None, v=None, rho=None, omega=None):
        """Set fluid positions, velocities, densities and volumes (omega*v and
        omega*rho follow), arrays in the reference's particle order."""
        hs = _AleHostState()
        mask = 0
        keep = []
        for name, arr, bit in (("r", r, ALE_F_R), ("v", v, ALE_F_V), ("rho", rho, ALE_F_RHO),
                               ("omega", omega, ALE_F_OMEGA)):
            if arr is None:
                continue
            a = np.ascontiguousarray(arr, dtype=np.float64)
            keep.append(a)
            setattr(hs, name, a.ctypes.data)
            mask |= bit
        _check(self._L.tsph_ale_upload(self._h, mask, C.byref(hs)))

    def upload_ptrs(self, mask, **ptrs):
        """Upload from raw host pointers (e.g. pinned buffers), arrays in the
        reference's particle order."""
        hs = _AleHostState()
        for k, v in ptrs.items():
            setattr(hs, k, v)
        _check(self._L.tsph_ale_upload(self._h, int(mask), C.byref(hs)))

    def download_ptrs(self, mask, **ptrs):
        """Download into raw host pointers (e.g. pinned buffers)."""
        hs = _AleHostState()
        for k, v in ptrs.items():
            setattr(hs, k, v)
        _check(self._L.tsph_ale_download(self._h, int(mask), C.byref(hs)))

    def download_async(self, mask, **ptrs):
        """Pipelined download of r, v, rho into raw host pointers (pinned for
        an overlap); valid after :meth:`download_wait`."""
        hs = _AleHostState()
        for k, v in ptrs.items():
            setattr(hs, k, v)
        _check(self._L.tsph_ale_download_async(self._h, int(mask), C.byref(hs)))

    def download_wait(self):
        _check(self._L.tsph_ale_download_wait(self._h))

    def upload_async(self, mask, **ptrs):
        """Staged upload of r, v, rho from raw host pointers (pinned for an
        overlap), applied by the next :meth:`particle_to_cell`."""
        hs = _AleHostState()
        for k, v in ptrs.items():
            setattr(hs, k, v)
        _check(self._L.tsph_ale_upload_async(self._h, int(mask), C.byref(hs)))

    def sync(self):
        _check(self._L.tsph_ale_sync(self._h))

    def health(self, clear=False) -> int:
        f = C.c_uint32()
        _check(self._L.tsph_ale_health(self._h, C.byref(f), 1 if clear else 0))
        return f.value


def Kernel_gradient_approx(particles: AleSystem):
    particles.gradient()


def Integrate_LeapFrog_partOne(particles: AleSystem, dt):
    particles.leapfrog_one(dt)


def Integrate_LeapFrog_partTwo(particles: AleSystem, dt, step):
    particles.leapfrog_two(dt, step)


class Gnn:
    """The surrogate's graph network on the device (tsph_gnn_*)."""

    def __init__(self, capacity, stream=None):
        self._L = load()
        h_ = C.c_void_p()
        _check(self._L.tsph_gnn_create(int(capacity), stream, C.byref(h_)))
        self._h = h_
        self.n_params = self._L.tsph_gnn_n_params()

    def close(self):
        if getattr(self, "_h", None):
            self._L.tsph_gnn_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, flat):
        a = np.ascontiguousarray(flat, dtype=np.float32)
        assert a.size == self.n_params
        _check(self._L.tsph_gnn_set_params(self._h, _p(a)))

    def params(self):
        out = np.empty(self.n_params, dtype=np.float32)
        _check(self._L.tsph_gnn_get_params(self._h, _p(out)))
        return out

    def grads(self):
        out = np.empty(self.n_params, dtype=np.float32)
        _check(self._L.tsph_gnn_get_grads(self._h, _p(out)))
        return out

    def forward(self, graph, y_ptr=None):
        _check(self._L.tsph_gnn_forward(self._h, C.byref(graph), y_ptr))

    def infer(self, graph, y_ptr):
        """The BF16 tensor-core forward (tsph_gnn_infer)."""
        _check(self._L.tsph_gnn_infer(self._h, C.byref(graph), y_ptr))

    def loss_grad(self, graph, target_ptr):
        l = C.c_double()
        _check(self._L.tsph_gnn_loss_grad(self._h, C.byref(graph), target_ptr, C.byref(l)))
        return l.value

    def adam(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        _check(self._L.tsph_gnn_adam(self._h, float(lr), float(beta1), float(beta2), float(eps)))
