"""Case builders with the constants of the reference's case drivers: dam
breaks with mDBC, DBC and boundary-integral walls, still water with mDBC,
DBC and boundary-integral walls, the ALE-SPH dam break, and open-boundary
cases.

A case is a :class:`Case`: particles in the reference's order, the SPH
constants of ``SPH_constants`` (``src/SPH_data.h:124-140``), the padded domain
of ``Simulation_data`` (``src/SPH_data.h:205-219``, padded as in
``PREP_SIMULATION_DATA``, e.g. ``cases/damBreakLong_mDBC/
SPH_simulationSymplectic.h:206-221``), the wall model and the time step.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import geometry as geo

WALL_MDBC = 0
WALL_DBC = 1
WALL_BT = 2


@dataclass
class Case:
    name: str
    particles: geo.ParticleSet
    h: float
    kap: float
    cs: float
    rho0: float
    visco: float
    delta: float
    dp: float
    domain: tuple  # padded (x_0, x_m, y_0, y_m)
    wall_model: int
    dt: float
    meta: dict = field(default_factory=dict)

    @property
    def np(self) -> int:
        return self.particles.np

    def constants(self):
        return dict(h=self.h, kap=self.kap, cs=self.cs, rho0=self.rho0,
                    visco=self.visco, delta=self.delta, dp=self.dp)


def _pad(x_0, x_1, y_0, y_1, nvl, dp):
    # PREP_SIMULATION_DATA: x_0 -= nvl*dp etc.
    return (x_0 - nvl * dp, x_1 + nvl * dp, y_0 - nvl * dp, y_1 + nvl * dp)


def dam_break_mdbc(dp: float = 0.005, cs: float = 34.3, wall_height: float = 1.0,
                   tank_length: float = 1.61, column=(0.6, 0.3),
                   dt: float | None = None) -> Case:
    """Dam break with mDBC walls: ``cases/damBreakLong_mDBC/constants.h`` and
    ``geometry.h:9-23``.

    Reference values: dp = 0.005, h = sqrt(2 dp^2) (constants.h:17), kap = 2.1,
    cs = 34.3 (constants.h:26), visco = 0.02, delta = 0.1, dt = 5e-5
    (constants.h:21), walls up to y = 1.0 m, domain [0, 2] x [0, 1].  The
    benchmark configuration uses cs = 35, walls to 0.8 m and dt scaled with dp
    (dt = 5e-5 * dp / 0.005).
    """
    x_0, x_1, y_0, y_1 = 0.0, 2.0, 0.0, 1.0
    kap = 2.1
    hh = 1.0 * math.sqrt(2 * dp * dp)
    if dt is None:
        dt = 0.00005 * (dp / 0.005)
    nvl = int(math.ceil(kap * hh / dp))
    ps = geo.ParticleSet(dp, hh, kap, cs)
    L = tank_length
    geo.create_wall_x_mdbc(ps, 0.0 + dp, L, 0.0, -1, dp / 2)
    geo.create_wall_y_mdbc(ps, 0.0, 0 + dp, wall_height, -1, dp / 2)
    geo.create_wall_y_mdbc(ps, L, 0 + dp, wall_height, +1, L - dp / 2)
    geo.create_corner_mdbc(ps, -1, -1, (0.0 + dp / 2, 0.0 + dp / 2))
    geo.create_corner_mdbc(ps, +1, -1, (L - dp / 2, 0.0 + dp / 2))
    geo.create_block_of_fluid(ps, 0 + dp, 0 + dp, column[0], column[1])
    return Case(name=f"dam_break_mdbc_dp{dp:g}", particles=ps, h=hh, kap=kap, cs=cs,
                rho0=1000.0, visco=0.02, delta=0.1, dp=dp,
                domain=_pad(x_0, x_1, y_0, y_1, nvl, dp), wall_model=WALL_MDBC,
                dt=dt, meta=dict(nvl=nvl, wall_height=wall_height, tank_length=L,
                                 column=tuple(column)))


def dam_break_dbc(dp: float = 0.005, dt: float | None = None) -> Case:
    """Dam break with DBC walls: ``cases/damBreakLong_DBC/constants.h`` and
    ``geometry.h`` (the walls of the mDBC case, whose ghost nodes the DBC
    interaction of src/SPH_interactionDBC.h does not use; a hydrostatic
    column, Create_Block_of_FluidWP, 0.6 x 0.3 m).  Reference values: dp =
    0.005, h = sqrt(2 dp^2), kap = 2.1, cs = 34.3, visco = 0.02, delta = 0.1,
    dt = 5e-5 (scaled with dp here), walls to y = 1.0 m, domain [0, 2] x [0, 1].
    """
    base = dam_break_mdbc(dp=dp, dt=dt)
    ps = geo.ParticleSet(dp, base.h, base.kap, base.cs)
    L = 1.61
    geo.create_wall_x_mdbc(ps, 0.0 + dp, L, 0.0, -1, dp / 2)
    geo.create_wall_y_mdbc(ps, 0.0, 0 + dp, 1.0, -1, dp / 2)
    geo.create_wall_y_mdbc(ps, L, 0 + dp, 1.0, +1, L - dp / 2)
    geo.create_corner_mdbc(ps, -1, -1, (0.0 + dp / 2, 0.0 + dp / 2))
    geo.create_corner_mdbc(ps, +1, -1, (L - dp / 2, 0.0 + dp / 2))
    geo.create_block_of_fluid_wp(ps, 0 + dp, 0 + dp, 0.6, 0.3)
    return Case(name=f"dam_break_dbc_dp{dp:g}", particles=ps, h=base.h, kap=base.kap,
                cs=base.cs, rho0=1000.0, visco=0.02, delta=0.1, dp=dp, domain=base.domain,
                wall_model=WALL_DBC, dt=base.dt, meta=dict(base.meta))


def still_water_mdbc(dp: float = 0.02, dt: float | None = None) -> Case:
    """Still water with mDBC walls: ``cases/stillWater_mDBC/constants.h`` and
    ``geometry.h`` (tank 0.8 m wide, walls to 1 m, a hydrostatic block
    0.8 - 2 dp wide and 0.5 m deep, Create_Block_of_FluidWP).  Reference
    values: dp = 0.02, h = 2 dp, kap = 2.1, cs = 42.48, visco = 0.01,
    delta = 0.1, dt = 2e-4 (scaled with dp here), domain [0, 1] x [0, 1]."""
    x_0, x_1, y_0, y_1 = 0.0, 1.0, 0.0, 1.0
    kap = 2.1
    hh = 2.0 * dp
    if dt is None:
        dt = 0.0002 * (dp / 0.02)
    cs = 42.48
    nvl = int(math.ceil(kap * hh / dp))
    ps = geo.ParticleSet(dp, hh, kap, cs)
    W = 0.8
    geo.create_wall_x_mdbc(ps, 0.0 + dp, W - dp, 0.0, -1, dp / 2)
    geo.create_wall_y_mdbc(ps, 0.0, 0 + dp, 1.0, -1, dp / 2)
    geo.create_wall_y_mdbc(ps, W, 0 + dp, 1.0, +1, W - dp / 2)
    geo.create_corner_mdbc(ps, -1, -1, (0.0 + dp / 2, 0.0 + dp / 2))
    geo.create_corner_mdbc(ps, +1, -1, (W - dp / 2, 0.0 + dp / 2))
    geo.create_block_of_fluid_wp(ps, 0 + dp, 0 + dp, W - dp, 0.5)
    return Case(name=f"still_water_mdbc_dp{dp:g}", particles=ps, h=hh, kap=kap, cs=cs,
                rho0=1000.0, visco=0.01, delta=0.1, dp=dp,
                domain=_pad(x_0, x_1, y_0, y_1, nvl, dp), wall_model=WALL_MDBC, dt=dt,
                meta=dict(nvl=nvl, depth=0.5))


def still_water_tank_mdbc(dp: float = 0.004, width: float = 0.8, depth: float = 0.3,
                          wall_height: float = 0.4, cs: float = 35.0) -> Case:
    """Still water with mDBC walls in a tank of a given size, with the dam
    break's numerics (the batched workload's still-water cases): the walls
    and corners of ``cases/stillWater_mDBC/geometry.h`` for a tank ``width``
    wide with walls ``wall_height`` high, a hydrostatic block
    (Create_Block_of_FluidWP) from (dp, dp) to (width - dp, depth);
    h = sqrt(2 dp^2), kap = 2.1, visco = 0.02, delta = 0.1,
    dt = 5e-5 * dp / 0.005; domain [0, width + 0.1] x [0, wall_height + 0.1]
    padded."""
    kap = 2.1
    hh = 1.0 * math.sqrt(2 * dp * dp)
    dt = 0.00005 * (dp / 0.005)
    nvl = int(math.ceil(kap * hh / dp))
    ps = geo.ParticleSet(dp, hh, kap, cs)
    W = width
    geo.create_wall_x_mdbc(ps, 0.0 + dp, W - dp, 0.0, -1, dp / 2)
    geo.create_wall_y_mdbc(ps, 0.0, 0 + dp, wall_height, -1, dp / 2)
    geo.create_wall_y_mdbc(ps, W, 0 + dp, wall_height, +1, W - dp / 2)
    geo.create_corner_mdbc(ps, -1, -1, (0.0 + dp / 2, 0.0 + dp / 2))
    geo.create_corner_mdbc(ps, +1, -1, (W - dp / 2, 0.0 + dp / 2))
    geo.create_block_of_fluid_wp(ps, 0 + dp, 0 + dp, W - dp, depth)
    return Case(name=f"still_water_tank_mdbc_dp{dp:g}", particles=ps, h=hh, kap=kap, cs=cs,
                rho0=1000.0, visco=0.02, delta=0.1, dp=dp,
                domain=_pad(0.0, W + 0.1, 0.0, wall_height + 0.1, nvl, dp),
                wall_model=WALL_MDBC, dt=dt, meta=dict(nvl=nvl, depth=depth))


def still_water_dbc(dp: float = 0.005, width: float = 0.5, depth: float = 0.3,
                    tank_height: float = 0.4, cs: float = 20.0, visco: float = 0.02,
                    delta: float = 0.1, layers: int = 3,
                    hydrostatic: bool = True) -> Case:
    """Still water in a tank with dynamic (DBC) walls.

    Water ``width`` x ``depth`` on a regular lattice at (i + 1/2) dp, filling
    the tank's interior width, ``layers`` layers of wall particles below and on
    both sides up to ``tank_height``; h = 1.5 dp, kap = 2.1, dt = 0.2 h / cs.
    Initial fluid state is hydrostatic (``Create_Block_of_FluidWP``,
    src/SPH_create.h:689-727: p = 9.81 (H - y) 1000, rho from the inverse EOS);
    wall particles get the hydrostatic value of their depth (rho0 above the
    free surface).  The pair loop is the DBC flavour
    (``src/SPH_interactionDBC.h``).
    """
    kap = 2.1
    hh = 1.5 * dp
    dt = 0.2 * hh / cs
    ps = geo.ParticleSet(dp, hh, kap, cs)
    nx = int(round(width / dp))
    ny = int(round(depth / dp))
    nyw = int(round(tank_height / dp))

    def hydro(y):
        if not hydrostatic or y >= depth:
            return 0.0, 1000.0
        p = 9.81 * (depth - y) * 1000
        return p, geo.pressure_to_density(p, 1000.0, cs)

    # walls first (bottom layers incl. corners, then the two sides)
    for l in range(layers):
        y = -(l + 0.5) * dp
        for i in range(-layers, nx + layers):
            x = (i + 0.5) * dp
            p, r = hydro(y)
            ps.add(geo.WALL, p, r, (x, y))
    for side in (0, 1):
        for l in range(layers):
            x = -(l + 0.5) * dp if side == 0 else width + (l + 0.5) * dp
            for j in range(nyw):
                y = (j + 0.5) * dp
                p, r = hydro(y)
                ps.add(geo.WALL, p, r, (x, y))
    for i in range(nx):
        x = (i + 0.5) * dp
        for j in range(ny):
            y = (j + 0.5) * dp
            p, r = hydro(y)
            ps.add(geo.FLUID, p, r, (x, y))
    pad = (layers + 2) * dp
    domain = (0.0 - pad, width + pad, 0.0 - pad, tank_height + pad)
    return Case(name=f"still_water_dbc_dp{dp:g}", particles=ps, h=hh, kap=kap, cs=cs,
                rho0=1000.0, visco=visco, delta=delta, dp=dp, domain=domain,
                wall_model=WALL_DBC, dt=dt,
                meta=dict(width=width, depth=depth, tank_height=tank_height,
                          layers=layers, nfluid=nx * ny))


def dam_break_benchmark(dp: float = 0.0005) -> Case:
    """The benchmark dam break: tank 1.61 x 0.8 m, column 0.6 x 0.3 m, mDBC,
    cs = 35 m/s, delta = 0.1, dt = 5e-5 * dp / 0.005 (about 0.24 h / cs)."""
    return dam_break_mdbc(dp=dp, cs=35.0, wall_height=0.8)


def dam_break_bt(dp: float = 0.005, cs: float = 34.3, dt: float | None = None,
                 tank_length: float = 1.61, wall_height: float = 1.0,
                 column=(0.6, 0.3)) -> Case:
    """WCSPH dam break with boundary-integral (BT) walls:
    ``cases/damBreakLong_BT/constants_smallDeltaT.h`` and ``geometry.h``
    (one wall layer with normals, corners with normals (+-sqrt 2, sqrt 2),
    hydrostatic column ``Create_Block_of_FluidWP``).  Reference values:
    dp = 0.005, h = sqrt(2 dp^2), cs = 34.3, dt = 2.5e-5 (scaled with dp
    here).  The wall normals travel in the per-wall vector of
    ``tsph_add_particles``."""
    x_0, x_1, y_0, y_1 = 0.0, 2.0, 0.0, 1.0
    kap = 2.1
    hh = 1.0 * math.sqrt(2 * dp * dp)
    if dt is None:
        dt = 0.000025 * (dp / 0.005)
    nvl = int(math.ceil(kap * hh / dp))
    ps = geo.AleParticleSet(dp, hh, kap, cs)
    L = tank_length
    geo.create_wall_x_bt(ps, 0.0 + dp, L - dp, 0.0, -1, (0.0, 1.0))
    geo.create_wall_y_bt(ps, 0.0, 0.0 + dp, wall_height, -1, (1.0, 0.0))
    geo.create_wall_y_bt(ps, L, 0.0 + dp, wall_height, +1, (-1.0, 0.0))
    geo.create_corner_bt(ps, -1, -1, (0.0, 0.0), (math.sqrt(2), math.sqrt(2)))
    geo.create_corner_bt(ps, +1, -1, (L, 0.0), (-math.sqrt(2), math.sqrt(2)))
    nw = ps.np
    geo.create_block_of_fluid_wp(ps, 0.0 + dp, 0 + dp, column[0], column[1])
    ps.gnr = list(ps.normals)  # walls come first: normal k belongs to particle k
    return Case(name=f"dam_break_bt_dp{dp:g}", particles=ps, h=hh, kap=kap, cs=cs,
                rho0=1000.0, visco=0.02, delta=0.1, dp=dp,
                domain=_pad(x_0, x_1, y_0, y_1, nvl, dp), wall_model=WALL_BT, dt=dt,
                meta=dict(nvl=nvl, nwalls=nw, wall_height=wall_height))


def still_water_bt(dp: float = 0.02) -> Case:
    """Still water with boundary-integral (BT) walls:
    ``cases/stillWater_BT/constants.h`` and ``geometry.h`` (tank 0.8 m wide,
    walls to 1 m, water 0.8 - dp wide and 0.5 m deep with hydrostatic p and
    rho, h = 2 dp, kap = 2.1, cs = 42.48, visco = 0.01, delta = 0.1,
    dt = 2e-4 at dp = 0.02, scaled with dp)."""
    x_0, x_1, y_0, y_1 = 0.0, 1.0, 0.0, 1.0
    kap = 2.1
    hh = 2.0 * dp
    dt = 0.0002 * (dp / 0.02)
    cs = 42.48
    nvl = int(math.ceil(kap * hh / dp))
    ps = geo.AleParticleSet(dp, hh, kap, cs)
    W = 0.8
    geo.create_wall_x_bt(ps, 0.0 + dp, W - dp, 0.0, -1, (0.0, 1.0))
    geo.create_wall_y_bt(ps, 0.0, 0.0 + dp, 1.0, -1, (1.0, 0.0))
    geo.create_wall_y_bt(ps, W, 0.0 + dp, 1.0, +1, (-1.0, 0.0))
    geo.create_corner_bt(ps, -1, -1, (0.0, 0.0), (math.sqrt(2), math.sqrt(2)))
    geo.create_corner_bt(ps, +1, -1, (W, 0.0), (-math.sqrt(2), math.sqrt(2)))
    nw = ps.np
    geo.create_block_of_fluid_wp(ps, 0 + dp, 0 + dp, W - dp, 0.5)
    ps.gnr = list(ps.normals)
    return Case(name=f"still_water_bt_dp{dp:g}", particles=ps, h=hh, kap=kap, cs=cs,
                rho0=1000.0, visco=0.01, delta=0.1, dp=dp,
                domain=_pad(x_0, x_1, y_0, y_1, nvl, dp), wall_model=WALL_BT, dt=dt,
                meta=dict(nvl=nvl, nwalls=nw, depth=0.5))


def still_water_ale(dp: float = 0.02) -> Case:
    """Riemann / ALE-SPH still water: ``cases/ALESPH_stillWater/constants.h``
    and ``geometry.h``, the tank, walls, hydrostatic block and constants of
    ``cases/stillWater_BT`` (h = 2 dp, cs = 42.48, visco = 0.01, dt = 2e-4)
    run by the ALE driver."""
    c = still_water_bt(dp)
    c.name = f"still_water_ale_dp{dp:g}"
    return c


def inflow_slab_mdbc(dp: float = 0.005, dt: float | None = None) -> Case:
    """Flow from an inlet over a step, mDBC walls, open boundaries:
    ``cases/inflowSlab_mDBC/constants.h`` and ``geometry.h`` (inlet buffer
    of 4 columns at x = 0.1 m, y in (0.1, 0.2], v = 0.75 m/s, zone 0; empty
    outlet zone at x = 1.0 m, zone 1).  Reference values: dp = 0.005,
    h = sqrt(2 dp^2), cs = 42.48, visco = 0.1, delta = 0.1, dt = 5e-5 (scaled
    with dp here).  The zones travel in ``meta["zones"]``."""
    x_0, x_1, y_0, y_1 = 0.0, 2.0, 0.0, 1.0
    kap = 2.1
    hh = 1.0 * math.sqrt(2 * dp * dp)
    if dt is None:
        dt = 0.00005 * (dp / 0.005)
    cs = 42.48
    nvl = int(math.ceil(kap * hh / dp))
    ps = geo.ParticleSet(dp, hh, kap, cs)
    geo.create_wall_x_mdbc(ps, 0.0, 0.4 - 3 * dp, 0.1, -1, 0.1 + dp / 2)
    geo.create_wall_y_mdbc(ps, 0.4, 0 + dp, 0.1 - 3 * dp, -1, 0.4 + dp / 2)
    geo.create_wall_x_mdbc(ps, 0.4 + dp, 1.2, 0.0, -1, 0 + dp / 2)
    geo.create_corner_mdbc(ps, -1, -1, (0.4 + dp / 2, 0.0 + dp / 2))
    geo.create_corner_mdbc(ps, -1, -1, (0.4 + dp / 2, 0.1 + dp / 2))
    nw = ps.np
    zones = [geo.create_inlet_y(ps, 0.1, 0.1 + dp, 0.2, -1, 4, (0.75, 0.0), geo.INLET1),
             geo.create_outlet_y(ps, 1.0, 0.0 + dp, 0.5, +1, 4, (0.5, 0.0), geo.OUTLET1, True)]
    return Case(name=f"inflow_slab_mdbc_dp{dp:g}", particles=ps, h=hh, kap=kap, cs=cs,
                rho0=1000.0, visco=0.1, delta=0.1, dp=dp,
                domain=_pad(x_0, x_1, y_0, y_1, nvl, dp), wall_model=WALL_MDBC, dt=dt,
                meta=dict(nvl=nvl, nwalls=nw, zones=zones))


def flow_drop_mdbc(dp: float = 0.005, dt: float | None = None) -> Case:
    """A jet falling from an inlet onto a floor, draining through two outlets:
    ``cases/flowDrop_mDBC/constants.h`` and ``geometry2.h`` (inlet rows above
    y = 0.3 + 4 dp, x in (0.8, 1.0], v = (0, -3) m/s, zone 0; outlets at
    x = 1.3 - 4 dp (+x, zone 1) and x = 0.5 (-x, zone 2)).  Reference
    values: dp = 0.005, h = sqrt(2 dp^2), cs = 34.3, visco = 0.02,
    delta = 0.1, dt = 5e-5 (scaled with dp here)."""
    x_0, x_1, y_0, y_1 = 0.0, 2.0, 0.0, 1.0
    kap = 2.1
    hh = 1.0 * math.sqrt(2 * dp * dp)
    if dt is None:
        dt = 0.00005 * (dp / 0.005)
    cs = 34.3
    nvl = int(math.ceil(kap * hh / dp))
    ps = geo.ParticleSet(dp, hh, kap, cs)
    geo.create_wall_x_mdbc(ps, 0.0 + dp, 1.61, 0.0, -1, dp / 2)
    nw = ps.np
    zones = [geo.create_inlet_x(ps, 0.3 + 4 * dp, 0.8 + dp, 1.0, +1, 4, (0.0, -3.0), geo.INLET1),
             geo.create_outlet_y(ps, 1.3 - 4 * dp, 0.0 + dp, 0.2, +1, 4, (2.0, 0.0), geo.OUTLET1),
             geo.create_outlet_y(ps, 0.5, 0.0 + dp, 0.2, -1, 4, (-2.0, 0.0), geo.OUTLET2)]
    return Case(name=f"flow_drop_mdbc_dp{dp:g}", particles=ps, h=hh, kap=kap, cs=cs,
                rho0=1000.0, visco=0.02, delta=0.1, dp=dp,
                domain=_pad(x_0, x_1, y_0, y_1, nvl, dp), wall_model=WALL_MDBC, dt=dt,
                meta=dict(nvl=nvl, nwalls=nw, zones=zones))


def inflow_tank_bottom_mdbc(dp: float = 0.005, dt: float | None = None) -> Case:
    """Inflow over a ledge into a tank, mDBC walls:
    ``cases/inflowTankBottom_mDBC/constants.h`` and ``geometry.h`` (tank
    floor x in (0.2, 1.2), left wall to 0.4 m, right wall to 0.8 m, a ledge
    at y = 0.4 + 3 dp from x = dp to 0.4, a hydrostatic layer 0.15 m deep in
    the tank, an inlet at x = 0.1 between y = 0.4 + 4 dp and 0.5 blowing +x
    at 1.5 m/s).  Reference values: dp = 0.005, h = sqrt(2 dp^2), kap = 2.1,
    cs = 34.3, visco = 0.02, delta = 0.1, dt = 5e-5 (scaled with dp here)."""
    x_0, x_1, y_0, y_1 = 0.0, 2.0, 0.0, 1.0
    kap = 2.1
    hh = 1.0 * math.sqrt(2 * dp * dp)
    if dt is None:
        dt = 0.00005 * (dp / 0.005)
    cs = 34.3
    nvl = int(math.ceil(kap * hh / dp))
    ps = geo.ParticleSet(dp, hh, kap, cs)
    geo.create_wall_x_mdbc(ps, 0.2 + dp, 1.2 - dp, 0.0, -1, dp / 2)
    geo.create_wall_y_mdbc(ps, 0.2, 0 + dp, 0.4, -1, dp / 2)
    geo.create_wall_y_mdbc(ps, 1.2, 0 + dp, 0.8, +1, 1.2 - dp / 2)
    geo.create_corner_mdbc(ps, -1, -1, (0.2 + dp / 2, 0.0 + dp / 2))
    geo.create_corner_mdbc(ps, +1, -1, (1.2 - dp / 2, 0.0 + dp / 2))
    geo.create_wall_x_mdbc(ps, 0.0 + dp, 0.4, 0.4 + 3 * dp, -1, dp / 2)
    nw = ps.np
    geo.create_block_of_fluid_wp(ps, 0.2 + dp, 0 + dp, 1.2, 0.15)
    zones = [geo.create_inlet_y(ps, 0.1, 0.4 + 4 * dp, 0.5, -1, 4, (1.5, 0.0), geo.INLET1)]
    return Case(name=f"inflow_tank_bottom_mdbc_dp{dp:g}", particles=ps, h=hh, kap=kap, cs=cs,
                rho0=1000.0, visco=0.02, delta=0.1, dp=dp,
                domain=_pad(x_0, x_1, y_0, y_1, nvl, dp), wall_model=WALL_MDBC, dt=dt,
                meta=dict(nvl=nvl, nwalls=nw, zones=zones))


def flow_drop_bt(dp: float = 0.005, dt: float | None = None) -> Case:
    """The falling jet of ``cases/flowDrop_BT`` (``constantsBT.h``,
    ``geometry.h``): one boundary-integral floor from x = -2 dp to 2 + 2 dp
    with normal (0, 1), the inlet and the two outlets of flowDrop_mDBC.
    Reference values: dp = 0.005, h = sqrt(2 dp^2), kap = 2.1, cs = 34.3,
    visco = 0.02, delta = 0.1, dt = 4e-5 (scaled with dp here)."""
    x_0, x_1, y_0, y_1 = 0.0, 2.0, 0.0, 1.0
    kap = 2.1
    hh = 1.0 * math.sqrt(2 * dp * dp)
    if dt is None:
        dt = 0.00004 * (dp / 0.005)
    cs = 34.3
    nvl = int(math.ceil(kap * hh / dp))
    ps = geo.AleParticleSet(dp, hh, kap, cs)
    geo.create_wall_x_bt(ps, 0.0 - dp * 2, 2.0 + dp * 2, 0.0, -1, (0.0, 1.0))
    nw = ps.np
    zones = [geo.create_inlet_x(ps, 0.3 + 4 * dp, 0.8 + dp, 1.0, +1, 4, (0.0, -3.0), geo.INLET1),
             geo.create_outlet_y(ps, 1.3 - 4 * dp, 0.0 + dp, 0.2, +1, 4, (2.0, 0.0), geo.OUTLET1),
             geo.create_outlet_y(ps, 0.5, 0.0 + dp, 0.2, -1, 4, (-2.0, 0.0), geo.OUTLET2)]
    ps.gnr = list(ps.normals)
    return Case(name=f"flow_drop_bt_dp{dp:g}", particles=ps, h=hh, kap=kap, cs=cs,
                rho0=1000.0, visco=0.02, delta=0.1, dp=dp,
                domain=_pad(x_0, x_1, y_0, y_1, nvl, dp), wall_model=WALL_BT, dt=dt,
                meta=dict(nvl=nvl, nwalls=nw, zones=zones))


def outlet_channel_mdbc(dp: float = 0.005, speed: float = 2.0) -> Case:
    """A fluid slab driven along a floor into an outlet zone (no counterpart
    case in the reference; it exercises BZ_Integrate_outlet's retyping and
    removal, src/SPH_buffer_zones.h:111-206): mDBC floor from x = 0 to 1.2
    m, fluid x in [0.40, 0.48], y in [dp, 0.05] moving at `speed`, an empty
    inlet zone (zone 0) far upstream and the outlet zone at x = 0.5 m
    (zone 1, 4 layers, +x)."""
    x_0, x_1, y_0, y_1 = 0.0, 2.0, 0.0, 1.0
    kap = 2.1
    hh = 1.0 * math.sqrt(2 * dp * dp)
    dt = 0.00005 * (dp / 0.005)
    cs = 42.48
    nvl = int(math.ceil(kap * hh / dp))
    ps = geo.ParticleSet(dp, hh, kap, cs)
    geo.create_wall_x_mdbc(ps, 0.0, 1.2, 0.0, -1, 0 + dp / 2)
    nw = ps.np
    n0 = ps.np
    geo.create_block_of_fluid(ps, 0.40, 0.0 + dp, 0.48, 0.05)
    for k in range(n0, ps.np):
        ps.vx[k] = speed
    zones = [geo.buffer_zone(0.05, 0.05 - 4 * dp, dp, 0.05, 4, (speed, 0.0), (-1.0, 0.0), geo.INLET1),
             geo.create_outlet_y(ps, 0.5, 0.0 + dp, 0.5, +1, 4, (speed, 0.0), geo.OUTLET1, True)]
    return Case(name=f"outlet_channel_mdbc_dp{dp:g}", particles=ps, h=hh, kap=kap, cs=cs,
                rho0=1000.0, visco=0.1, delta=0.1, dp=dp,
                domain=_pad(x_0, x_1, y_0, y_1, nvl, dp), wall_model=WALL_MDBC, dt=dt,
                meta=dict(nvl=nvl, nwalls=nw, zones=zones))


def dam_break_ale(dp: float = 0.005, cs: float = 34.3, dt: float | None = None,
                  tank_length: float = 1.61, wall_height: float = 1.0,
                  column=(0.6, 0.3)) -> Case:
    """Riemann / ALE-SPH dam break with boundary-integral (BT) walls:
    ``cases/ALESPH_dambreakLong/constants.h`` and ``geometry.h:16-24``
    (one wall layer with normals, corners with normals (+-sqrt 2, sqrt 2)).
    Reference values: dp = 0.005, h = sqrt(2 dp^2), cs = 34.3, dt = 5e-5; the
    benchmark configuration uses dp = 0.0004 and dt scaled with dp."""
    x_0, x_1, y_0, y_1 = 0.0, 2.0, 0.0, 1.0
    kap = 2.1
    hh = 1.0 * math.sqrt(2 * dp * dp)
    if dt is None:
        dt = 0.00005 * (dp / 0.005)
    nvl = int(math.ceil(kap * hh / dp))
    ps = geo.AleParticleSet(dp, hh, kap, cs)
    L = tank_length
    geo.create_wall_x_bt(ps, 0.0 + dp, L - dp, 0.0, -1, (0.0, 1.0))
    geo.create_wall_y_bt(ps, 0.0, 0.0 + dp, wall_height, -1, (1.0, 0.0))
    geo.create_wall_y_bt(ps, L, 0.0 + dp, wall_height, +1, (-1.0, 0.0))
    geo.create_corner_bt(ps, -1, -1, (0.0, 0.0), (math.sqrt(2), math.sqrt(2)))
    geo.create_corner_bt(ps, +1, -1, (L, 0.0), (-math.sqrt(2), math.sqrt(2)))
    nw = ps.np
    geo.create_block_of_fluid(ps, 0.0 + dp, 0 + dp, column[0], column[1])
    return Case(name=f"dam_break_ale_dp{dp:g}", particles=ps, h=hh, kap=kap, cs=cs,
                rho0=1000.0, visco=0.02, delta=0.1, dp=dp,
                domain=_pad(x_0, x_1, y_0, y_1, nvl, dp), wall_model=2, dt=dt,
                meta=dict(nvl=nvl, nwalls=nw, wall_height=wall_height))
