"""ctypes front-end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Two back-ends with one interface:

* ``PortSystem``: ``oracle/liboracle.so``, the plain-C restatement
  (``oracle/tsph_oracle.c``), built on any host by ``oracle/Makefile``.
* ``RefSystem``: ``oracle/_ref/libtsph_ref.so``, the reference's own headers
  compiled by ``make -C oracle ref`` (only where the reference sources exist).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module.  The product never does.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libtsph_ref.so")
REF_ALE_LIB = os.path.join(HERE, "_ref", "libtsph_ref_ale.so")
REF_BT_LIB = os.path.join(HERE, "_ref", "libtsph_ref_bt.so")

F_RX, F_RY, F_VX, F_VY, F_AX, F_AY, F_RHO, F_DRHO, F_P = range(9)
F_ROX, F_ROY, F_VOX, F_VOY, F_RHO_O = range(9, 14)

_D = C.c_double
_P = C.c_void_p
_I = C.c_int
_DP = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_IP = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build_port(force: bool = False) -> str:
    if force or not os.path.exists(PORT_LIB):
        subprocess.run(["make", "-s", "-C", HERE, "all"],
                       check=True)
    return PORT_LIB


def build_ref() -> str | None:
    """Build the reference harness where the reference sources are present
    (oracle/Makefile's `ref-if-present`; REF in the environment overrides the
    Makefile's location of the reference checkout)."""
    subprocess.run(["make", "-s", "-C", HERE, "ref-if-present"], check=True)
    return REF_LIB if os.path.exists(REF_LIB) else None


def ref_available() -> bool:
    if not os.path.exists(REF_LIB):
        return False
    try:
        C.CDLL(REF_LIB)
        return True
    except OSError:
        return False


_port = None
_ref = None


def _load_port():
    global _port
    if _port is None:
        build_port()
        L = C.CDLL(PORT_LIB)
        L.orc_create.restype = _P
        L.orc_create.argtypes = [_D] * 11
        L.orc_destroy.argtypes = [_P]
        L.orc_set_threads.argtypes = [_I]
        L.orc_get_threads.restype = _I
        L.orc_add_particle.argtypes = [_P, _I] + [_D] * 8
        L.orc_add_gnr.argtypes = [_P, _D, _D]
        L.orc_np.argtypes = [_P]
        L.orc_np.restype = _I
        L.orc_grid.argtypes = [_P, C.POINTER(_I), C.POINTER(_I)]
        L.orc_const.argtypes = [_P, _I]
        L.orc_const.restype = _D
        L.orc_get_field.argtypes = [_P, _I, _DP]
        L.orc_set_field.argtypes = [_P, _I, _DP]
        L.orc_get_meta.argtypes = [_P, _IP, _IP]
        L.orc_get_cells.argtypes = [_P, _IP, _IP]
        L.orc_get_cells.restype = _I
        for f in ("orc_divide_to_cells", "orc_clear_cells", "orc_particle_to_cell",
                  "orc_density_to_pressure", "orc_mdbc_density", "orc_bt_density"):
            getattr(L, f).argtypes = [_P]
        L.orc_compute_forces.argtypes = [_P, _I]
        L.orc_predictor.argtypes = [_P, _D]
        L.orc_corrector.argtypes = [_P, _D]
        L.orc_remove_out_of_domain.argtypes = [_P]
        L.orc_remove_out_of_domain.restype = _I
        L.orc_step.argtypes = [_P, _I, _D, _I]
        L.orc_add_zone.argtypes = [_P, _D, _D, _D, _D, _I, _D, _D, _D, _D, _I]
        L.orc_add_zone.restype = _I
        L.orc_bz_inlet.argtypes = [_P, _I, _D]
        L.orc_bz_outlet.argtypes = [_P, _I, _D]
        L.orc_step_zones.argtypes = [_P, _I, _D, _I]
        L.orc_pair_digest.argtypes = [_P, _IP, np.ctypeslib.ndpointer(dtype=np.int64, flags='C_CONTIGUOUS'), _IP]
        L.orc_water_level.argtypes = [_P, _D, _D, _I]
        L.orc_water_level.restype = _D
        L.orc_point_fields.argtypes = [_P, _D, _D, _DP]
        L.orc_wendland.argtypes = [_D, _D, C.POINTER(_D), C.POINTER(_D)]
        L.orc_pressure.argtypes = [_D, _D, _D]
        L.orc_pressure.restype = _D
        L.orc_pressure_to_density.argtypes = [_D, _D, _D]
        L.orc_pressure_to_density.restype = _D
        L.orc_ale_add_particle.argtypes = [_P, _I] + [_D] * 6
        L.orc_ale_add_normal.argtypes = [_P, _D, _D]
        L.orc_ale_get_field.argtypes = [_P, _I, _DP]
        L.orc_ale_set_field.argtypes = [_P, _I, _DP]
        L.orc_ale_set_scheme.argtypes = [_P, _I]
        L.orc_ale_gradient.argtypes = [_P]
        L.orc_ale_forces.argtypes = [_P, _D]
        L.orc_ale_forces_first_order.argtypes = [_P]
        L.orc_ale_leapfrog_one.argtypes = [_P, _D]
        L.orc_ale_leapfrog_two.argtypes = [_P, _D, _I]
        L.orc_ale_step.argtypes = [_P, _D, _I, _I]
        _port = L
    return _port


def _load_ref():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_LIB)
        L.ref_create.restype = _P
        L.ref_create.argtypes = [_D] * 11
        L.ref_destroy.argtypes = [_P]
        L.ref_set_threads.argtypes = [_I]
        L.ref_add_particle.argtypes = [_P, _I] + [_D] * 6
        L.ref_add_gnr.argtypes = [_P, _D, _D]
        L.ref_create_block_of_fluid.argtypes = [_P] + [_D] * 4
        L.ref_create_block_of_fluid_wp.argtypes = [_P] + [_D] * 4
        L.ref_create_wall_x_mdbc.argtypes = [_P, _D, _D, _D, _I, _D]
        L.ref_create_wall_y_mdbc.argtypes = [_P, _D, _D, _D, _I, _D]
        L.ref_create_corner_mdbc.argtypes = [_P, _I, _I, _D, _D]
        L.ref_create_wall_x.argtypes = [_P, _D, _D, _D, _I]
        L.ref_create_wall_y.argtypes = [_P, _D, _D, _D, _I]
        L.ref_np.argtypes = [_P]
        L.ref_np.restype = _I
        L.ref_grid.argtypes = [_P, C.POINTER(_I), C.POINTER(_I)]
        L.ref_get_state.argtypes = [_P] + [_P] * 8
        L.ref_set_state.argtypes = [_P] + [_P] * 6
        L.ref_get_gnr.argtypes = [_P, _DP]
        L.ref_ngnr.argtypes = [_P]
        L.ref_ngnr.restype = _I
        L.ref_get_cells.argtypes = [_P, _P, _P]
        L.ref_get_cells.restype = _I
        for f in ("ref_divide_to_cells", "ref_clear_cells", "ref_particle_to_cell",
                  "ref_density_to_pressure", "ref_mdbc_density",
                  "ref_remove_out_of_domain"):
            getattr(L, f).argtypes = [_P]
        L.ref_compute_forces.argtypes = [_P, _I]
        L.ref_predictor.argtypes = [_P, _D]
        L.ref_corrector.argtypes = [_P, _D]
        L.ref_step.argtypes = [_P, _I, _D, _I]
        L.ref_add_zone.argtypes = [_P, _D, _D, _D, _D, _I, _D, _D, _D, _D, _I]
        L.ref_create_inlet_y.argtypes = [_P, _D, _D, _D, _I, _I, _D, _D, _I]
        L.ref_create_outlet_y.argtypes = [_P, _D, _D, _D, _I, _I, _D, _D, _I, _I]
        L.ref_create_inlet_x.argtypes = [_P, _D, _D, _D, _I, _I, _D, _D, _I]
        L.ref_nzones.argtypes = [_P]
        L.ref_nzones.restype = _I
        L.ref_get_zone.argtypes = [_P, _I, _DP]
        L.ref_bz_inlet.argtypes = [_P, _I, _D]
        L.ref_bz_outlet.argtypes = [_P, _I, _D]
        L.ref_step_zones.argtypes = [_P, _D, _I]
        L.ref_water_level.argtypes = [_P, _D, _D, _I]
        L.ref_water_level.restype = _D
        L.ref_point_fields.argtypes = [_P, _D, _D, _DP]
        L.ref_pressure_in_point.argtypes = [_P, _D, _D]
        L.ref_pressure_in_point.restype = _D
        L.ref_wendland.argtypes = [_D, _D, C.POINTER(_D), C.POINTER(_D)]
        _ref = L
    return _ref


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class _Base:
    """Common state accessors; ``state()`` returns the reference-order fields."""

    def ncells(self):
        ncx, ncy = self.grid()
        return ncx * ncy


class PortSystem(_Base):
    """The plain-C oracle."""

    def __init__(self, h, kap, cs, rho0, visco, delta, dp, domain):
        self.L = _load_port()
        self.s = self.L.orc_create(h, kap, cs, rho0, visco, delta, dp, *domain)

    @classmethod
    def from_case(cls, case, divide=True):
        o = cls(case.h, case.kap, case.cs, case.rho0, case.visco, case.delta, case.dp,
                case.domain)
        ps = case.particles
        for i in range(ps.np):
            o.L.orc_add_particle(o.s, ps.type[i], ps.p[i], ps.rho[i], ps.rx[i], ps.ry[i],
                                 ps.vx[i], ps.vy[i], 0.0, 0.0)
        for g in ps.gnr:
            o.L.orc_add_gnr(o.s, g[0], g[1])
        for z in case.meta.get("zones", []):
            o.L.orc_add_zone(o.s, z["x0"], z["xm"], z["y0"], z["ym"], z["nbl"], z["vx"], z["vy"],
                             z["ox"], z["oy"], z["btype"])
        if divide:
            o.divide_to_cells()
            o.particle_to_cell()
        return o

    def step_zones(self, dt, n=1, model=0):
        """RUN of cases/inflowSlab_mDBC (mDBC step with the zones' inlet and
        outlet after the predictor); model 2 (BT) is cases/flowDrop_BT."""
        self.L.orc_step_zones(self.s, int(model), dt, int(n))

    def __del__(self):
        try:
            self.L.orc_destroy(self.s)
        except Exception:
            pass

    @staticmethod
    def set_threads(n):
        _load_port().orc_set_threads(int(n))

    @staticmethod
    def get_threads():
        return _load_port().orc_get_threads()

    def np(self):
        return self.L.orc_np(self.s)

    def grid(self):
        a, b = _I(), _I()
        self.L.orc_grid(self.s, C.byref(a), C.byref(b))
        return a.value, b.value

    def const(self, which):
        return self.L.orc_const(self.s, which)

    def field(self, f):
        out = np.empty(self.np(), dtype=np.float64)
        self.L.orc_get_field(self.s, f, out)
        return out

    def set_field(self, f, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        assert a.shape == (self.np(),)
        self.L.orc_set_field(self.s, f, a)

    def state(self):
        n = self.np()
        idx = np.empty(n, dtype=np.int32)
        typ = np.empty(n, dtype=np.int32)
        self.L.orc_get_meta(self.s, idx, typ)
        g = self.field
        return dict(r=np.stack([g(F_RX), g(F_RY)], 1), v=np.stack([g(F_VX), g(F_VY)], 1),
                    a=np.stack([g(F_AX), g(F_AY)], 1), rho=g(F_RHO), drho=g(F_DRHO),
                    p=g(F_P), index=idx, type=typ)

    def set_state(self, r=None, v=None, a=None, rho=None, drho=None, p=None):
        if r is not None:
            self.set_field(F_RX, r[:, 0]); self.set_field(F_RY, r[:, 1])
        if v is not None:
            self.set_field(F_VX, v[:, 0]); self.set_field(F_VY, v[:, 1])
        if a is not None:
            self.set_field(F_AX, a[:, 0]); self.set_field(F_AY, a[:, 1])
        if rho is not None:
            self.set_field(F_RHO, rho)
        if drho is not None:
            self.set_field(F_DRHO, drho)
        if p is not None:
            self.set_field(F_P, p)

    def cells(self):
        nc = self.ncells()
        start = np.empty(nc + 1, dtype=np.int32)
        lst = np.empty(max(self.np(), 1), dtype=np.int32)
        n = self.L.orc_get_cells(self.s, start, lst)
        if n < 0:
            raise RuntimeError("cells not built")
        return start, lst[:n]

    def water_level(self, x, y0, inverse=False):
        return self.L.orc_water_level(self.s, float(x), float(y0), 1 if inverse else 0)

    def point_fields(self, x, y):
        out = np.zeros(4)
        self.L.orc_point_fields(self.s, float(x), float(y), out)
        return out

    def pair_digest(self):
        n = self.np()
        c = np.empty(n, dtype=np.int32)
        s = np.empty(n, dtype=np.int64)
        x = np.empty(n, dtype=np.int32)
        self.L.orc_pair_digest(self.s, c, s, x)
        return c, s, x

    def divide_to_cells(self):
        self.L.orc_divide_to_cells(self.s)

    def clear_cells(self):
        self.L.orc_clear_cells(self.s)

    def particle_to_cell(self):
        self.L.orc_particle_to_cell(self.s)

    def density_to_pressure(self):
        self.L.orc_density_to_pressure(self.s)

    def compute_forces(self, model):
        self.L.orc_compute_forces(self.s, int(model))

    def mdbc_density(self):
        self.L.orc_mdbc_density(self.s)

    def predictor(self, dt):
        self.L.orc_predictor(self.s, dt)

    def corrector(self, dt):
        self.L.orc_corrector(self.s, dt)

    def remove_out_of_domain(self):
        return self.L.orc_remove_out_of_domain(self.s)

    def step(self, model, dt, n=1):
        self.L.orc_step(self.s, int(model), dt, int(n))


class RefSystem(_Base):
    """The reference's own code (oracle/_ref/libtsph_ref.so)."""

    def __init__(self, h, kap, cs, rho0, visco, delta, dp, domain):
        self.L = _load_ref()
        self.s = self.L.ref_create(h, kap, cs, rho0, visco, delta, dp, *domain)

    @classmethod
    def from_case(cls, case, divide=True):
        o = cls(case.h, case.kap, case.cs, case.rho0, case.visco, case.delta, case.dp,
                case.domain)
        ps = case.particles
        for i in range(ps.np):
            o.L.ref_add_particle(o.s, ps.type[i], ps.p[i], ps.rho[i], ps.rx[i], ps.ry[i],
                                 ps.vx[i], ps.vy[i])
        for g in ps.gnr:
            o.L.ref_add_gnr(o.s, g[0], g[1])
        for z in case.meta.get("zones", []):
            o.L.ref_add_zone(o.s, z["x0"], z["xm"], z["y0"], z["ym"], z["nbl"], z["vx"], z["vy"],
                             z["ox"], z["oy"], z["btype"])
        if divide:
            o.divide_to_cells()
            o.particle_to_cell()
        return o

    def step_zones(self, dt, n=1):
        self.L.ref_step_zones(self.s, dt, int(n))

    def zones(self):
        out = []
        for k in range(self.L.ref_nzones(self.s)):
            z = np.empty(12)
            self.L.ref_get_zone(self.s, k, z)
            out.append(z)
        return out

    def __del__(self):
        try:
            self.L.ref_destroy(self.s)
        except Exception:
            pass

    @staticmethod
    def set_threads(n):
        _load_ref().ref_set_threads(int(n))

    def np(self):
        return self.L.ref_np(self.s)

    def grid(self):
        a, b = _I(), _I()
        self.L.ref_grid(self.s, C.byref(a), C.byref(b))
        return a.value, b.value

    def state(self):
        n = self.np()
        r = np.empty((n, 2)); v = np.empty((n, 2)); a = np.empty((n, 2))
        rho = np.empty(n); drho = np.empty(n); p = np.empty(n)
        idx = np.empty(n, dtype=np.int32); typ = np.empty(n, dtype=np.int32)
        self.L.ref_get_state(self.s, _ptr(r), _ptr(v), _ptr(a), _ptr(rho), _ptr(drho),
                             _ptr(p), _ptr(idx), _ptr(typ))
        return dict(r=r, v=v, a=a, rho=rho, drho=drho, p=p, index=idx, type=typ)

    def set_state(self, r=None, v=None, a=None, rho=None, drho=None, p=None):
        c = lambda x, shp: None if x is None else np.ascontiguousarray(x, dtype=np.float64)
        r, v, a = c(r, 2), c(v, 2), c(a, 2)
        rho, drho, p = c(rho, 1), c(drho, 1), c(p, 1)
        self.L.ref_set_state(self.s, _ptr(r), _ptr(v), _ptr(a), _ptr(rho), _ptr(drho),
                             _ptr(p))

    def gnr(self):
        out = np.empty((self.L.ref_ngnr(self.s), 2))
        self.L.ref_get_gnr(self.s, out.reshape(-1))
        return out

    def cells(self):
        nc = self.ncells()
        start = np.empty(nc + 1, dtype=np.int32)
        lst = np.empty(max(self.np(), 1), dtype=np.int32)
        n = self.L.ref_get_cells(self.s, _ptr(start), _ptr(lst))
        return start, lst[:n]

    def divide_to_cells(self):
        self.L.ref_divide_to_cells(self.s)

    def clear_cells(self):
        self.L.ref_clear_cells(self.s)

    def particle_to_cell(self):
        self.L.ref_particle_to_cell(self.s)

    def density_to_pressure(self):
        self.L.ref_density_to_pressure(self.s)

    def compute_forces(self, model):
        self.L.ref_compute_forces(self.s, int(model))

    def mdbc_density(self):
        self.L.ref_mdbc_density(self.s)

    def predictor(self, dt):
        self.L.ref_predictor(self.s, dt)

    def corrector(self, dt):
        self.L.ref_corrector(self.s, dt)

    def remove_out_of_domain(self):
        self.L.ref_remove_out_of_domain(self.s)

    def step(self, model, dt, n=1):
        self.L.ref_step(self.s, int(model), dt, int(n))

    def water_level(self, x, y0, inverse=False):
        return self.L.ref_water_level(self.s, float(x), float(y0), 1 if inverse else 0)

    def point_fields(self, x, y):
        out = np.zeros(4)
        self.L.ref_point_fields(self.s, float(x), float(y), out)
        return out

    def pressure_in_point(self, x, y):
        return self.L.ref_pressure_in_point(self.s, float(x), float(y))


def ref_wendland(r, h):
    L = _load_ref()
    w, f = _D(), _D()
    L.ref_wendland(r, h, C.byref(w), C.byref(f))
    return w.value, f.value


def wendland(r, h):
    L = _load_port()
    w, f = _D(), _D()
    L.orc_wendland(r, h, C.byref(w), C.byref(f))
    return w.value, f.value


# ---------------------------------------------------------------- ALE-SPH
_ref_ale = None


def _load_ref_ale():
    global _ref_ale
    if _ref_ale is None:
        L = C.CDLL(REF_ALE_LIB)
        L.refale_create.restype = _P
        L.refale_create.argtypes = [_D] * 11
        L.refale_destroy.argtypes = [_P]
        L.refale_set_threads.argtypes = [_I]
        L.refale_add_particle.argtypes = [_P, _I] + [_D] * 6
        L.refale_add_normal.argtypes = [_P, _D, _D]
        L.refale_create_wall_x_bt.argtypes = [_P, _D, _D, _D, _I, _D, _D]
        L.refale_create_wall_y_bt.argtypes = [_P, _D, _D, _D, _I, _D, _D]
        L.refale_create_corner_bt.argtypes = [_P, _I, _I, _D, _D, _D, _D]
        L.refale_create_block_of_fluid.argtypes = [_P] + [_D] * 4
        L.refale_np.argtypes = [_P]
        L.refale_np.restype = _I
        L.refale_nn.argtypes = [_P]
        L.refale_nn.restype = _I
        L.refale_get_normals.argtypes = [_P, _DP]
        L.refale_get_state.argtypes = [_P] + [_P] * 13
        L.refale_set_velocity_density.argtypes = [_P, _DP, _DP]
        for f in ("refale_divide_to_cells", "refale_particle_to_cell",
                  "refale_density_to_pressure", "refale_gradient"):
            getattr(L, f).argtypes = [_P]
        L.refale_forces.argtypes = [_P, _D]
        L.refale_leapfrog_one.argtypes = [_P, _D]
        L.refale_leapfrog_two.argtypes = [_P, _D, _I]
        L.refale_step.argtypes = [_P, _D, _I, _I]
        L.refale_forces_first_order.argtypes = [_P]
        L.refale_step_first_order.argtypes = [_P, _D, _I, _I]
        _ref_ale = L
    return _ref_ale


def ref_ale_available() -> bool:
    if not os.path.exists(REF_ALE_LIB):
        return False
    try:
        C.CDLL(REF_ALE_LIB)
        return True
    except OSError:
        return False


ALE_FIELDS = ("omega", "omegarho", "omegavx", "omegavy", "domega", "domegarho", "domegavx",
              "domegavy")


class PortAle(PortSystem):
    """The oracle's ALE-SPH functions on a PortSystem."""

    @classmethod
    def from_case(cls, case, divide=True):
        o = cls(case.h, case.kap, case.cs, case.rho0, case.visco, case.delta, case.dp,
                case.domain)
        ps = case.particles
        for i in range(ps.np):
            o.L.orc_ale_add_particle(o.s, ps.type[i], ps.p[i], ps.rho[i], ps.rx[i], ps.ry[i],
                                     ps.vx[i], ps.vy[i])
        for n in ps.normals:
            o.L.orc_ale_add_normal(o.s, n[0], n[1])
        if divide:
            o.divide_to_cells()
            o.particle_to_cell()
        return o

    def ale_field(self, f):
        out = np.empty(self.np(), dtype=np.float64)
        self.L.orc_ale_get_field(self.s, f, out)
        return out

    def set_ale_field(self, f, arr):
        self.L.orc_ale_set_field(self.s, f, np.ascontiguousarray(arr, dtype=np.float64))

    def ale_state(self):
        st = self.state()
        g = self.ale_field
        st.update(omega=g(0), omegarho=g(1), omegav=np.stack([g(2), g(3)], 1), domega=g(4),
                  domegarho=g(5), domegav=np.stack([g(6), g(7)], 1),
                  grad=np.stack([g(12 + k) for k in range(12)], 1))
        return st

    def set_velocity_density(self, v, rho):
        """Fluid v and rho with omega*v, omega*rho kept consistent."""
        st = self.state()
        fl = st["type"] == 0
        om = self.ale_field(0)
        vv = st["v"].copy(); rr = st["rho"].copy()
        vv[fl] = v[fl]; rr[fl] = rho[fl]
        self.set_state(v=vv, rho=rr)
        omv = np.stack([self.ale_field(2), self.ale_field(3)], 1)
        omv[fl] = vv[fl] * om[fl, None]
        omr = self.ale_field(1)
        omr[fl] = rr[fl] * om[fl]
        self.set_ale_field(2, omv[:, 0]); self.set_ale_field(3, omv[:, 1])
        self.set_ale_field(1, omr)

    def set_scheme(self, scheme):
        self.L.orc_ale_set_scheme(self.s, int(scheme))

    def gradient(self):
        self.L.orc_ale_gradient(self.s)

    def ale_forces(self, dt):
        self.L.orc_ale_forces(self.s, dt)

    def ale_forces_first_order(self):
        self.L.orc_ale_forces_first_order(self.s)

    def leapfrog_one(self, dt):
        self.L.orc_ale_leapfrog_one(self.s, dt)

    def leapfrog_two(self, dt, step):
        self.L.orc_ale_leapfrog_two(self.s, dt, int(step))

    def ale_step(self, dt, step0, n):
        self.L.orc_ale_step(self.s, dt, int(step0), int(n))


class RefAle:
    """The reference's ALE-SPH code (oracle/_ref/libtsph_ref_ale.so)."""

    def __init__(self, case):
        self.L = _load_ref_ale()
        self.s = self.L.refale_create(case.h, case.kap, case.cs, case.rho0, case.visco,
                                      case.delta, case.dp, *case.domain)

    @classmethod
    def from_case(cls, case, divide=True):
        o = cls(case)
        ps = case.particles
        for i in range(ps.np):
            o.L.refale_add_particle(o.s, ps.type[i], ps.p[i], ps.rho[i], ps.rx[i], ps.ry[i],
                                    ps.vx[i], ps.vy[i])
        for n in ps.normals:
            o.L.refale_add_normal(o.s, n[0], n[1])
        if divide:
            o.L.refale_divide_to_cells(o.s)
            o.L.refale_particle_to_cell(o.s)
        return o

    def __del__(self):
        try:
            self.L.refale_destroy(self.s)
        except Exception:
            pass

    @staticmethod
    def set_threads(n):
        _load_ref_ale().refale_set_threads(int(n))

    def np(self):
        return self.L.refale_np(self.s)

    def ale_state(self):
        n = self.np()
        out = dict(r=np.empty((n, 2)), v=np.empty((n, 2)), rho=np.empty(n), p=np.empty(n),
                   type=np.empty(n, dtype=np.int32), index=np.empty(n, dtype=np.int32),
                   omega=np.empty(n), omegarho=np.empty(n), omegav=np.empty((n, 2)),
                   domega=np.empty(n), domegarho=np.empty(n), domegav=np.empty((n, 2)),
                   grad=np.empty((n, 12)))
        k = ("r", "v", "rho", "p", "type", "index", "omega", "omegarho", "omegav", "domega",
             "domegarho", "domegav", "grad")
        self.L.refale_get_state(self.s, *[_ptr(out[x]) for x in k])
        return out

    def normals(self):
        out = np.empty((self.L.refale_nn(self.s), 2))
        self.L.refale_get_normals(self.s, out.reshape(-1))
        return out

    def set_velocity_density(self, v, rho):
        self.L.refale_set_velocity_density(self.s, np.ascontiguousarray(v, dtype=np.float64).reshape(-1),
                                           np.ascontiguousarray(rho, dtype=np.float64))

    def particle_to_cell(self):
        self.L.refale_particle_to_cell(self.s)

    def density_to_pressure(self):
        self.L.refale_density_to_pressure(self.s)

    def gradient(self):
        self.L.refale_gradient(self.s)

    def ale_forces(self, dt):
        self.L.refale_forces(self.s, dt)

    def ale_forces_first_order(self):
        self.L.refale_forces_first_order(self.s)

    def ale_step_first_order(self, dt, step0, n):
        self.L.refale_step_first_order(self.s, dt, int(step0), int(n))

    def leapfrog_one(self, dt):
        self.L.refale_leapfrog_one(self.s, dt)

    def leapfrog_two(self, dt, step):
        self.L.refale_leapfrog_two(self.s, dt, int(step))

    def ale_step(self, dt, step0, n):
        self.L.refale_step(self.s, dt, int(step0), int(n))


# ---------------------------------------------------------------- BT walls
ORC_BT = 2  # oracle/tsph_oracle.h


class PortBt(PortSystem):
    """The oracle with boundary-integral walls (src/SPH_interactionBT.h,
    src/SPH_BT.h): the wall normals of the case are added with
    orc_ale_add_normal (walls first)."""

    @classmethod
    def from_case(cls, case, divide=True):
        o = PortSystem.from_case.__func__(cls, case, divide=False)
        for n in case.particles.normals:
            o.L.orc_ale_add_normal(o.s, n[0], n[1])
        if divide:
            o.divide_to_cells()
            o.particle_to_cell()
        return o

    def bt_density(self):
        self.L.orc_bt_density(self.s)


_ref_bt = None


def _load_ref_bt():
    global _ref_bt
    if _ref_bt is None:
        L = C.CDLL(REF_BT_LIB)
        L.refbt_create.restype = _P
        L.refbt_create.argtypes = [_D] * 11
        L.refbt_destroy.argtypes = [_P]
        L.refbt_set_threads.argtypes = [_I]
        L.refbt_add_particle.argtypes = [_P, _I] + [_D] * 6
        L.refbt_add_normal.argtypes = [_P, _D, _D]
        L.refbt_create_wall_x_bt.argtypes = [_P, _D, _D, _D, _I, _D, _D]
        L.refbt_create_wall_y_bt.argtypes = [_P, _D, _D, _D, _I, _D, _D]
        L.refbt_create_corner_bt.argtypes = [_P, _I, _I, _D, _D, _D, _D]
        L.refbt_create_block_of_fluid_wp.argtypes = [_P] + [_D] * 4
        L.refbt_np.argtypes = [_P]
        L.refbt_np.restype = _I
        L.refbt_nn.argtypes = [_P]
        L.refbt_nn.restype = _I
        L.refbt_get_normals.argtypes = [_P, _DP]
        L.refbt_get_state.argtypes = [_P] + [_P] * 8
        L.refbt_set_velocity_density.argtypes = [_P, _DP, _DP]
        for f in ("refbt_divide_to_cells", "refbt_particle_to_cell", "refbt_density_to_pressure",
                  "refbt_wall_density", "refbt_forces"):
            getattr(L, f).argtypes = [_P]
        L.refbt_step.argtypes = [_P, _D, _I]
        L.refbt_add_zone.argtypes = [_P, _D, _D, _D, _D, _I, _D, _D, _D, _D, _I]
        L.refbt_create_inlet_x.argtypes = [_P, _D, _D, _D, _I, _I, _D, _D, _I]
        L.refbt_create_outlet_y.argtypes = [_P, _D, _D, _D, _I, _I, _D, _D, _I, _I]
        L.refbt_step_zones.argtypes = [_P, _D, _I]
        _ref_bt = L
    return _ref_bt


def ref_bt_available() -> bool:
    if not os.path.exists(REF_BT_LIB):
        return False
    try:
        C.CDLL(REF_BT_LIB)
        return True
    except OSError:
        return False


class RefBt:
    """The reference's BT-wall WCSPH code (oracle/_ref/libtsph_ref_bt.so)."""

    def __init__(self, case):
        self.L = _load_ref_bt()
        self.s = self.L.refbt_create(case.h, case.kap, case.cs, case.rho0, case.visco,
                                     case.delta, case.dp, *case.domain)

    @classmethod
    def from_case(cls, case, divide=True):
        o = cls(case)
        ps = case.particles
        for i in range(ps.np):
            o.L.refbt_add_particle(o.s, ps.type[i], ps.p[i], ps.rho[i], ps.rx[i], ps.ry[i],
                                   ps.vx[i], ps.vy[i])
        for n in ps.normals:
            o.L.refbt_add_normal(o.s, n[0], n[1])
        for z in case.meta.get("zones", []):
            o.L.refbt_add_zone(o.s, z["x0"], z["xm"], z["y0"], z["ym"], z["nbl"], z["vx"],
                               z["vy"], z["ox"], z["oy"], z["btype"])
        if divide:
            o.L.refbt_divide_to_cells(o.s)
            o.L.refbt_particle_to_cell(o.s)
        return o

    def step_zones(self, dt, n=1):
        """RUN of cases/flowDrop_BT (the BT step with the zones' inlet and
        outlet after the predictor)."""
        self.L.refbt_step_zones(self.s, dt, int(n))

    @classmethod
    def generated(cls, case, dp, L=1.61, wall_height=1.0, column=(0.6, 0.3)):
        """The same tank built by the reference's own generators
        (cases/damBreakLong_BT/geometry.h)."""
        import math

        o = cls(case)
        s2 = math.sqrt(2)
        o.L.refbt_create_wall_x_bt(o.s, 0.0 + dp, L - dp, 0.0, -1, 0.0, 1.0)
        o.L.refbt_create_wall_y_bt(o.s, 0.0, 0.0 + dp, wall_height, -1, 1.0, 0.0)
        o.L.refbt_create_wall_y_bt(o.s, L, 0.0 + dp, wall_height, +1, -1.0, 0.0)
        o.L.refbt_create_corner_bt(o.s, -1, -1, 0.0, 0.0, s2, s2)
        o.L.refbt_create_corner_bt(o.s, +1, -1, L, 0.0, -s2, s2)
        o.L.refbt_create_block_of_fluid_wp(o.s, 0.0 + dp, 0 + dp, column[0], column[1])
        return o

    def __del__(self):
        try:
            self.L.refbt_destroy(self.s)
        except Exception:
            pass

    @staticmethod
    def set_threads(n):
        _load_ref_bt().refbt_set_threads(int(n))

    def np(self):
        return self.L.refbt_np(self.s)

    def state(self):
        n = self.np()
        out = dict(r=np.empty((n, 2)), v=np.empty((n, 2)), a=np.empty((n, 2)), rho=np.empty(n),
                   drho=np.empty(n), p=np.empty(n), type=np.empty(n, dtype=np.int32),
                   index=np.empty(n, dtype=np.int32))
        k = ("r", "v", "a", "rho", "drho", "p", "type", "index")
        self.L.refbt_get_state(self.s, *[_ptr(out[x]) for x in k])
        return out

    def normals(self):
        out = np.empty((self.L.refbt_nn(self.s), 2))
        self.L.refbt_get_normals(self.s, out.reshape(-1))
        return out

    def set_velocity_density(self, v, rho):
        self.L.refbt_set_velocity_density(self.s, np.ascontiguousarray(v, dtype=np.float64).reshape(-1),
                                          np.ascontiguousarray(rho, dtype=np.float64))

    def divide_to_cells(self):
        self.L.refbt_divide_to_cells(self.s)

    def particle_to_cell(self):
        self.L.refbt_particle_to_cell(self.s)

    def density_to_pressure(self):
        self.L.refbt_density_to_pressure(self.s)

    def bt_density(self):
        self.L.refbt_wall_density(self.s)

    def compute_forces(self):
        self.L.refbt_forces(self.s)

    def step(self, dt, n=1):
        self.L.refbt_step(self.s, dt, int(n))
