"""Particle generators of the reference, restated for the host side.

Each function appends particles to a :class:`ParticleSet` in exactly the order
and with exactly the IEEE double arithmetic of the reference generator it
names (``src/SPH_create.h``), so a case built here is bit-identical to the same
case built by the reference (checked against the reference's own generators in
``tests/test_geometry.py``).  Python floats are IEEE binary64 and Python never
contracts ``a*b+c`` into an FMA, so the expressions below round exactly like
the reference's C++.

The mDBC generators also record each wall particle's ghost node (the
reference's ``special.gnr``, ``src/SPH_data.h:51``); walls must be created
before fluid, as in every reference case, because ``gnr`` is indexed by the
particle index (``src/SPH_mDBC.h:26``).
"""

from __future__ import annotations

import math

import numpy as np

FLUID = 0  # src/SPH_defs.h:46
WALL = 1   # src/SPH_defs.h:47


class ParticleSet:
    """Host-side particle list in the reference's order (``Add_particle``,
    ``src/SPH_particle_system.h:25-50``)."""

    def __init__(self, dp: float, h: float, kap: float, cs: float, rho0: float = 1000.0):
        self.dp = dp
        self.h = h
        self.kap = kap
        self.cs = cs
        self.rho0 = rho0
        self.type: list[int] = []
        self.p: list[float] = []
        self.rho: list[float] = []
        self.rx: list[float] = []
        self.ry: list[float] = []
        self.vx: list[float] = []
        self.vy: list[float] = []
        self.gnr: list[tuple[float, float]] = []

    def add(self, ptype: int, p: float, rho: float, r, v=(0.0, 0.0)):
        self.type.append(ptype)
        self.p.append(p)
        self.rho.append(rho)
        self.rx.append(r[0])
        self.ry.append(r[1])
        self.vx.append(v[0])
        self.vy.append(v[1])

    @property
    def np(self) -> int:
        return len(self.type)

    def arrays(self):
        """Return a dict of numpy arrays (r and v as (n, 2) float64)."""
        n = self.np
        out = {
            "type": np.asarray(self.type, dtype=np.int32),
            "p": np.asarray(self.p, dtype=np.float64),
            "rho": np.asarray(self.rho, dtype=np.float64),
            "r": np.stack([np.asarray(self.rx, dtype=np.float64),
                           np.asarray(self.ry, dtype=np.float64)], axis=1).reshape(n, 2),
            "v": np.stack([np.asarray(self.vx, dtype=np.float64),
                           np.asarray(self.vy, dtype=np.float64)], axis=1).reshape(n, 2),
            "gnr": np.asarray(self.gnr, dtype=np.float64).reshape(-1, 2),
        }
        return out


def _len(x0, y0, x1, y1):
    # LEN macro, src/SPH_defs.h:34
    return math.sqrt((x1 - x0) * (x1 - x0) + (y1 - y0) * (y1 - y0))


def _kh(ps: ParticleSet) -> float:
    # kh = h * kap as written in the generators (src/SPH_create.h:550)
    return ps.h * ps.kap


def create_block_of_fluid(ps: ParticleSet, x_0, y_0, x_1, y_1):
    """``Create_Block_of_Fluid``, src/SPH_create.h:105-139 (column-major loop,
    x outer, y inner; rho = rho0, p = 0)."""
    dp = ps.dp
    npart_x = int(_len(x_0, y_0, x_1, y_0) / dp)
    npart_y = int(_len(x_0, y_0, x_0, y_1) / dp)
    for i in range(npart_x + 1):
        rx = x_0 + i * dp
        for j in range(npart_y + 1):
            ry = y_0 + j * dp
            ps.add(FLUID, 0.0, ps.rho0, (rx, ry))


def pressure_to_density(p, rho0, c0):
    """``Pressure_to_density``, src/SPH_pressure.h:37-51."""
    b_const = c0 * c0 * rho0 / 7.0
    return (math.pow(p / b_const + 1, 1.0 / 7)) * rho0


def create_block_of_fluid_wp(ps: ParticleSet, x_0, y_0, x_1, y_1):
    """``Create_Block_of_FluidWP`` (hydrostatic p and rho),
    src/SPH_create.h:689-727."""
    dp = ps.dp
    npart_x = int(_len(x_0, y_0, x_1, y_0) / dp)
    npart_y = int(_len(x_0, y_0, x_0, y_1) / dp)
    for i in range(npart_x + 1):
        rx = x_0 + i * dp
        for j in range(npart_y + 1):
            ry = y_0 + j * dp
            rhoin = pressure_to_density(9.81 * (y_1 - ry) * 1000, 1000.0, ps.cs)
            ps.add(FLUID, 9.81 * (y_1 - ry) * 1000, rhoin, (rx, ry))


def create_wall_x_mdbc(ps: ParticleSet, x_0, x_1, y, orientation, y_w):
    """``Create_Wall_x_mdbc``, src/SPH_create.h:546-581."""
    dp = ps.dp
    npart = int(_len(x_0, y, x_1, y) / dp)
    nvl = int(math.ceil(_kh(ps) / dp) - 0)
    for l in range(nvl):
        ry = y + dp * l * orientation
        for i in range(npart + 1):
            rx = x_0 + i * dp
            ps.add(WALL, 0.0, ps.rho0, (rx, ry))
            ps.gnr.append((rx, y_w + math.fabs(ry - y_w)))


def create_wall_y_mdbc(ps: ParticleSet, x, y_0, y_1, orientation, x_w):
    """``Create_Wall_y_mdbc``, src/SPH_create.h:583-619."""
    dp = ps.dp
    npart = int(_len(x, y_0, x, y_1) / dp)
    nvl = int(math.ceil(_kh(ps) / dp) - 0)
    for l in range(nvl):
        rx = x + dp * l * orientation
        for i in range(npart + 1):
            ry = y_0 + i * dp
            ps.add(WALL, 0.0, ps.rho0, (rx, ry))
            ps.gnr.append((x_w + math.fabs(rx - x_w) * (-1) * orientation, ry))


def create_corner_mdbc(ps: ParticleSet, orientation_x, orientation_y, xyv):
    """``Create_corner_mdbc``, src/SPH_create.h:621-652."""
    dp = ps.dp
    nvl = int(math.ceil(_kh(ps) / dp) - 0)
    for l in range(nvl):
        ry = xyv[1] + dp * l * orientation_y + dp / 2 * orientation_y
        for i in range(nvl):
            rx = xyv[0] + dp * i * orientation_x + dp / 2 * orientation_x
            ps.add(WALL, 0.0, ps.rho0, (rx, ry))
            ps.gnr.append((xyv[0] + math.fabs(rx - xyv[0]) * (-1) * orientation_x,
                           xyv[1] + math.fabs(ry - xyv[1]) * (-1) * orientation_y))


def create_wall_x(ps: ParticleSet, x_0, x_1, y, orientation):
    """``Create_Wall_x`` (DBC, ceil(kh/dp)+1 layers), src/SPH_create.h:37-69."""
    dp = ps.dp
    npart = int(_len(x_0, y, x_1, y) / dp)
    nvl = int(math.ceil(_kh(ps) / dp) + 1)
    for l in range(nvl):
        ry = y + dp * l * orientation
        for i in range(npart + 1):
            ps.add(WALL, 0.0, ps.rho0, (x_0 + i * dp, ry))


def create_wall_y(ps: ParticleSet, x, y_0, y_1, orientation):
    """``Create_Wall_y`` (DBC, ceil(kh/dp)+1 layers), src/SPH_create.h:71-103."""
    dp = ps.dp
    npart = int(_len(x, y_0, x, y_1) / dp)
    nvl = int(math.ceil(_kh(ps) / dp) + 1)
    for l in range(nvl):
        rx = x + dp * l * orientation
        for i in range(npart + 1):
            ps.add(WALL, 0.0, ps.rho0, (rx, y_0 + i * dp))


class AleParticleSet(ParticleSet):
    """Particles of the ALE-SPH path: ``ALESPH_Add_particle``
    (src/SPH_particle_system.h:51-108) plus the BT wall normals
    (``special.n``, src/SPH_data.h:52), indexed by particle index."""

    def __init__(self, dp, h, kap, cs, rho0=1000.0):
        super().__init__(dp, h, kap, cs, rho0)
        self.normals: list[tuple[float, float]] = []


def create_wall_x_bt(ps: AleParticleSet, x_0, x_1, y, orientation, n):
    """``Create_Wall_x_bt`` (one layer, normal n), src/ALESPH_create.h:690-725."""
    dp = ps.dp
    npart = int(_len(x_0, y, x_1, y) / dp)
    for l in range(1):
        ry = y + dp * l * orientation
        for i in range(npart + 1):
            ps.add(WALL, 0.0, ps.rho0, (x_0 + i * dp, ry))
            ps.normals.append((n[0], n[1]))


def create_wall_y_bt(ps: AleParticleSet, x, y_0, y_1, orientation, n):
    """``Create_Wall_y_bt``, src/ALESPH_create.h:727-761."""
    dp = ps.dp
    npart = int(_len(x, y_0, x, y_1) / dp)
    for l in range(1):
        rx = x + dp * l * orientation
        for i in range(npart + 1):
            ps.add(WALL, 0.0, ps.rho0, (rx, y_0 + i * dp))
            ps.normals.append((n[0], n[1]))


def create_corner_bt(ps: AleParticleSet, orientation_x, orientation_y, xyv, n):
    """``Create_corner_bt``, src/ALESPH_create.h:763-792."""
    dp = ps.dp
    for l in range(1):
        ry = xyv[1] + dp * l * orientation_y
        for i in range(1):
            rx = xyv[0] + dp * i * orientation_x
            ps.add(WALL, 0.0, ps.rho0, (rx, ry))
            ps.normals.append((n[0], n[1]))


# ------------------------------------------------------------ open boundaries
INLET1 = 7    # src/SPH_defs.h:53
OUTLET1 = 12  # src/SPH_defs.h:59
OUTLET2 = 13  # src/SPH_defs.h:60


def buffer_zone(x0, xm, y0, ym, nbl, v0, orientation, btype):
    """``BufferZone`` (src/SPH_inlet_outlet_data.h): region, layers, velocity,
    orientation and the type of its buffer particles."""
    return dict(x0=x0, xm=xm, y0=y0, ym=ym, nbl=nbl, vx=v0[0], vy=v0[1], ox=orientation[0],
                oy=orientation[1], btype=btype)


def create_inlet_y(ps: ParticleSet, x, y_0, y_1, orientation, nbl, v0, btype):
    """``DRAW_CreateInletY``, src/SPH_create.h:439-471: nbl columns of buffer
    particles of type btype moving with v0, and the zone (returned)."""
    dp = ps.dp
    npart = int(math.ceil(_len(x, y_0, x, y_1) / dp)) + 1
    for l in range(nbl):
        rx = x + dp * l * orientation
        for hh in range(npart):
            ps.add(btype, 0.0, ps.rho0, (rx, y_0 + hh * dp), (v0[0], v0[1]))
    return buffer_zone(x, x + nbl * dp * orientation, y_0, y_1, nbl, v0, (float(orientation), 0.0),
                       btype)


def create_inlet_x(ps: ParticleSet, y, x_0, x_1, orientation, nbl, v0, btype):
    """``DRAW_CreateInletX``, src/SPH_create.h:472-504: nbl rows of buffer
    particles above (+1) or below (-1) the line y, and the zone (returned)."""
    dp = ps.dp
    npart = int(math.ceil(_len(x_0, y, x_1, y) / dp)) + 1
    for l in range(nbl):
        ry = y + dp * l * orientation
        for hh in range(npart):
            ps.add(btype, 0.0, ps.rho0, (x_0 + hh * dp, ry), (v0[0], v0[1]))
    return buffer_zone(x_0, x_1, y, y + nbl * dp * orientation, nbl, v0, (0.0, float(orientation)),
                       btype)


def create_outlet_y(ps: ParticleSet, x, y_0, y_1, orientation, nbl, v0, btype, empty=True):
    """``DRAW_CreateOutletY``, src/SPH_create.h:508-540 (with empty = false the
    reference fills the zone with particles of type `inlet`)."""
    dp = ps.dp
    if not empty:
        npart = int(math.ceil(_len(x, y_0, x, y_1) / dp)) + 1
        for l in range(nbl):
            rx = x + dp * l * orientation
            for hh in range(npart):
                ps.add(6, 0.0, ps.rho0, (rx, y_0 + hh * dp), (v0[0], v0[1]))
    return buffer_zone(x, x + nbl * dp * orientation, y_0, y_1, nbl, v0, (float(orientation), 0.0),
                       btype)
