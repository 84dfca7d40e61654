"""Many independent WCSPH cases stepped together on one GPU.

The batched workload is a set of seeded dam-break and still-water tanks of
different sizes and resolutions (particle spacing dp in {0.004, 0.003,
0.002} m), all with mDBC walls and the dam-break constants (h = sqrt(2) dp,
c0 = 35 m/s, dt = 0.01 dp s).

:class:`Batch` packs every case into ONE particle system, so each kernel
launch of a step covers the whole batch.  Case k is scaled by
lambda_k = dp_sys / dp_k (dp_sys the smallest spacing) and shifted along x:
in that frame every case has the system's spacing, h, particle mass, sound
speed and time step, and the SPH equations are those of the unscaled case
with velocity and density unchanged, time scaled by lambda_k (one system step
dt_sys advances case k by its own dt_k = dt_sys / lambda_k) and gravity
g / lambda_k.  Gravity and RemoveParticlesOutOfDomain's box
(src/SPH_btdebug.h:4-31) are therefore per case: the system's case table
(``tsph_set_cases``) gives each grid column its case.  Cases sit side by side
with gaps of several cells; a particle leaves its case only through that
case's removal box, so no pair ever spans two cases.  Per-case results agree
with separate runs of each case up to FP32 rounding (the scaled positions
round differently).

:class:`GroupedBatch` is the packing used before the case table: cases with
identical constants side by side in one system per group, groups on their
own streams (one launch per kernel per group).

The case generators here are vectorised restatements of the ones in
``cases`` (bit-identical particles, tested), because a batch holds millions
of particles.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import cases as _cases

DAM_BREAK = "dam_break"
STILL_WATER = "still_water"
FLUID, WALL = 0, 1


@dataclass
class CaseSpec:
    """One case of the batch.  Dam break: tank of length ``tank`` and walls
    0.8 m high, water column ``col_w`` x ``col_h`` at the left wall.  Still
    water: a tank ``col_w`` wide with walls ``col_h`` + 0.1 m high, filled
    ``col_h`` deep at rest (hydrostatic start).  Both with mDBC walls,
    c0 = 35 m/s, h = sqrt(2) dp, dt = 0.01 dp."""

    kind: str
    dp: float
    tank: float
    col_w: float
    col_h: float

    def group(self):
        return (self.kind, self.dp)


def sample_specs(n: int = 512, seed: int = 0, dps=(0.004, 0.003, 0.002)):
    """Seeded batch: kind uniform over {dam break, still water}, tank width
    U(0.8, 2.0) m, column width U(0.2, 0.8) m (at most the tank width less
    0.1 m), height U(0.1, 0.5) m, dp uniform over `dps`."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        kind = DAM_BREAK if rng.random() < 0.5 else STILL_WATER
        dp = float(dps[int(rng.integers(len(dps)))])
        tank = float(rng.uniform(0.8, 2.0))
        col_w = float(min(rng.uniform(0.2, 0.8), tank - 0.1))
        col_h = float(rng.uniform(0.1, 0.5))
        out.append(CaseSpec(kind, dp, tank, col_w, col_h))
    return out


# ---------------------------------------------------------------- generators
# Vectorised restatements of geometry.create_* (same IEEE operations in the
# same order per element, so the particles are bit-identical).

def _block(dp, x_0, y_0, x_1, y_1):
    npx = int(math.sqrt((x_1 - x_0) * (x_1 - x_0)) / dp)
    npy = int(math.sqrt((y_1 - y_0) * (y_1 - y_0)) / dp)
    rx = x_0 + np.arange(npx + 1, dtype=np.float64) * dp
    ry = y_0 + np.arange(npy + 1, dtype=np.float64) * dp
    return np.repeat(rx, npy + 1), np.tile(ry, npx + 1)


def _wall_x_mdbc(dp, kh, x_0, x_1, y, o, y_w):
    npart = int(math.sqrt((x_1 - x_0) * (x_1 - x_0)) / dp)
    nvl = int(math.ceil(kh / dp))
    rx0 = x_0 + np.arange(npart + 1, dtype=np.float64) * dp
    xs, ys, gx, gy = [], [], [], []
    for l in range(nvl):
        ry = y + dp * l * o
        xs.append(rx0)
        ys.append(np.full(npart + 1, ry))
        gx.append(rx0)
        gy.append(np.full(npart + 1, y_w + math.fabs(ry - y_w)))
    return map(np.concatenate, (xs, ys, gx, gy))


def _wall_y_mdbc(dp, kh, x, y_0, y_1, o, x_w):
    npart = int(math.sqrt((y_1 - y_0) * (y_1 - y_0)) / dp)
    nvl = int(math.ceil(kh / dp))
    ry0 = y_0 + np.arange(npart + 1, dtype=np.float64) * dp
    xs, ys, gx, gy = [], [], [], []
    for l in range(nvl):
        rx = x + dp * l * o
        xs.append(np.full(npart + 1, rx))
        ys.append(ry0)
        gx.append(np.full(npart + 1, x_w + math.fabs(rx - x_w) * (-1) * o))
        gy.append(ry0)
    return map(np.concatenate, (xs, ys, gx, gy))


def _corner_mdbc(dp, kh, ox, oy, xv, yv):
    nvl = int(math.ceil(kh / dp))
    xs, ys, gx, gy = [], [], [], []
    for l in range(nvl):
        ry = yv + dp * l * oy + dp / 2 * oy
        for i in range(nvl):
            rx = xv + dp * i * ox + dp / 2 * ox
            xs.append(rx)
            ys.append(ry)
            gx.append(xv + math.fabs(rx - xv) * (-1) * ox)
            gy.append(yv + math.fabs(ry - yv) * (-1) * oy)
    return map(np.asarray, (xs, ys, gx, gy))


@dataclass
class CaseArrays:
    """Particles of one case in the reference's order, its constants and its
    own padded domain (case-local coordinates)."""

    spec: CaseSpec
    type: np.ndarray
    r: np.ndarray
    rho: np.ndarray
    p: np.ndarray
    gnr: np.ndarray
    h: float
    kap: float
    cs: float
    dt: float
    wall_model: int
    domain: tuple
    extent: tuple = field(default=(0.0, 0.0))  # x range the tank occupies

    @property
    def np(self):
        return len(self.type)


def case_arrays(spec: CaseSpec) -> CaseArrays:
    """The particles of `spec` (identical to ``cases.dam_break_mdbc`` /
    ``cases.still_water_dbc`` with the same parameters)."""
    dp = spec.dp
    if spec.kind == DAM_BREAK:
        kap, cs, L, wall_h = 2.1, 35.0, spec.tank, 0.8
        h = 1.0 * math.sqrt(2 * dp * dp)
        kh = h * kap
        parts = [
            _wall_x_mdbc(dp, kh, 0.0 + dp, L, 0.0, -1, dp / 2),
            _wall_y_mdbc(dp, kh, 0.0, 0 + dp, wall_h, -1, dp / 2),
            _wall_y_mdbc(dp, kh, L, 0 + dp, wall_h, +1, L - dp / 2),
            _corner_mdbc(dp, kh, -1, -1, 0.0 + dp / 2, 0.0 + dp / 2),
            _corner_mdbc(dp, kh, +1, -1, L - dp / 2, 0.0 + dp / 2),
        ]
        wx, wy, gx, gy = (np.concatenate(list(c)) for c in zip(*[tuple(p) for p in parts]))
        fx, fy = _block(dp, 0 + dp, 0 + dp, spec.col_w, spec.col_h)
        nw, nf = len(wx), len(fx)
        r = np.stack([np.concatenate([wx, fx]), np.concatenate([wy, fy])], 1)
        typ = np.concatenate([np.full(nw, WALL, np.int32), np.full(nf, FLUID, np.int32)])
        gnr = np.zeros((nw + nf, 2))
        gnr[:nw, 0], gnr[:nw, 1] = gx, gy
        rho = np.full(nw + nf, 1000.0)
        p = np.zeros(nw + nf)
        nvl = int(math.ceil(kap * h / dp))
        dom = _cases._pad(0.0, max(2.0, L + 0.1), 0.0, 1.0, nvl, dp)
        return CaseArrays(spec, typ, r, rho, p, gnr, h, kap, cs, 0.00005 * (dp / 0.005),
                          _cases.WALL_MDBC, dom, (dom[0], L + nvl * dp))
    # still water (cases.still_water_tank_mdbc: a tank col_w wide, walls
    # col_h + 0.1 high, filled col_h deep at rest, hydrostatic start)
    kap, cs, L, wall_h, depth = 2.1, 35.0, spec.col_w, spec.col_h + 0.1, spec.col_h
    h = 1.0 * math.sqrt(2 * dp * dp)
    kh = h * kap
    parts = [
        _wall_x_mdbc(dp, kh, 0.0 + dp, L - dp, 0.0, -1, dp / 2),
        _wall_y_mdbc(dp, kh, 0.0, 0 + dp, wall_h, -1, dp / 2),
        _wall_y_mdbc(dp, kh, L, 0 + dp, wall_h, +1, L - dp / 2),
        _corner_mdbc(dp, kh, -1, -1, 0.0 + dp / 2, 0.0 + dp / 2),
        _corner_mdbc(dp, kh, +1, -1, L - dp / 2, 0.0 + dp / 2),
    ]
    wx, wy, gx, gy = (np.concatenate(list(c)) for c in zip(*[tuple(p) for p in parts]))
    fx, fy = _block(dp, 0 + dp, 0 + dp, L - dp, depth)
    # Create_Block_of_FluidWP (src/SPH_create.h:689-727): p = 9.81 (H - y) 1000,
    # rho from Pressure_to_density with libm pow, per distinct height
    b = cs * cs * 1000.0 / 7.0
    uy, inv = np.unique(fy, return_inverse=True)
    up = 9.81 * (depth - uy) * 1000
    ur = np.array([math.pow(q / b + 1, 1.0 / 7) * 1000.0 for q in up])
    nw, nf = len(wx), len(fx)
    r = np.stack([np.concatenate([wx, fx]), np.concatenate([wy, fy])], 1)
    typ = np.concatenate([np.full(nw, WALL, np.int32), np.full(nf, FLUID, np.int32)])
    gnr = np.zeros((nw + nf, 2))
    gnr[:nw, 0], gnr[:nw, 1] = gx, gy
    rho = np.concatenate([np.full(nw, 1000.0), ur[inv]])
    p = np.concatenate([np.zeros(nw), up[inv]])
    nvl = int(math.ceil(kap * h / dp))
    dom = _cases._pad(0.0, L + 0.1, 0.0, wall_h + 0.1, nvl, dp)
    return CaseArrays(spec, typ, r, rho, p, gnr, h, kap, cs, 0.00005 * (dp / 0.005),
                      _cases.WALL_MDBC, dom, (dom[0], L + nvl * dp))


# ---------------------------------------------------------------- packing
# Horizontal gap between packed tanks: still water never leaves its tank, so
# 4 kh (no pair can span it) is enough; a dam-break particle can be thrown over
# a 0.8 m wall, and anything above the domain top (1 m + padding) is removed,
# so it falls at most ~1.1 m before it drops below the floor and is removed:
# at < 5 m/s that is < 2.4 m of travel.
SPLASH_GAP = 2.5


@dataclass
class PackedGroup:
    """Cases with identical constants, side by side in one particle system.
    ``offset[k]``: the x shift of case k; ``base[k]``: its first particle
    index in the system (particles keep the reference's order per case)."""

    cases: list
    offset: np.ndarray
    base: np.ndarray
    domain: tuple
    system: object = None

    @property
    def np(self):
        return int(sum(c.np for c in self.cases))

    @property
    def dt(self):
        return self.cases[0].dt

    @property
    def wall_model(self):
        return self.cases[0].wall_model


def pack(case_list, splash_gap=SPLASH_GAP) -> PackedGroup:
    c0 = case_list[0]
    kh = c0.h * c0.kap
    gap = splash_gap if c0.spec.kind == DAM_BREAK else 4.0 * kh
    offs, bases = [], []
    x, base = 0.0, 0
    for k, c in enumerate(case_list):
        if k:
            x += case_list[k - 1].extent[1] - c.extent[0] + gap
        offs.append(x)
        bases.append(base)
        base += c.np
    last = case_list[-1]
    dom = (c0.domain[0], offs[-1] + last.domain[1], min(c.domain[2] for c in case_list),
           max(c.domain[3] for c in case_list))
    return PackedGroup(list(case_list), np.array(offs), np.array(bases, dtype=np.int64), dom)


def group_specs(specs):
    """Specs grouped by constants: {(kind, dp): [(batch index, spec), ...]}."""
    groups = {}
    for k, s in enumerate(specs):
        groups.setdefault(s.group(), []).append((k, s))
    return groups


class GroupedBatch:
    """Cases packed one particle system per group of equal constants, each
    group on its own stream (``step(n)``: every group advances by n of its
    own time steps).  Used to generate the surrogate's training windows,
    whose cases share one spacing."""

    def __init__(self, specs, precision="fp32", streams=True):
        from . import sph

        self.specs = list(specs)
        self.groups = []
        self.where = {}  # batch index -> (group, position in group)
        self._streams = []
        for key, members in sorted(group_specs(self.specs).items()):
            g = pack([case_arrays(s) for _, s in members])
            g.key = key
            for pos, (k, _) in enumerate(members):
                self.where[k] = (len(self.groups), pos)
            stream = None
            if streams:
                import torch

                st = torch.cuda.Stream()
                self._streams.append(st)
                stream = st.cuda_stream
            c0 = g.cases[0]
            s = sph.ParticleSystem(c0.h, c0.kap, c0.cs, 1000.0, 0.02, 0.1, c0.spec.dp, g.domain,
                                   precision, stream=stream)
            typ = np.concatenate([c.type for c in g.cases])
            r = np.concatenate([c.r + np.array([off, 0.0]) for c, off in zip(g.cases, g.offset)])
            rho = np.concatenate([c.rho for c in g.cases])
            p = np.concatenate([c.p for c in g.cases])
            gnr = None
            if c0.wall_model == _cases.WALL_MDBC:
                gnr = np.concatenate([c.gnr + np.array([off, 0.0]) * (c.type[:, None] == WALL)
                                      for c, off in zip(g.cases, g.offset)])
            s.add_particles(typ, r, None, rho, p, gnr)
            s.divide_to_cells()
            s.particle_to_cell()
            g.system = s
            self.groups.append(g)

    @property
    def np(self):
        return sum(g.np for g in self.groups)

    def step(self, n=1):
        for g in self.groups:
            g.system.step(g.wall_model, g.dt, n)

    def sync(self):
        for g in self.groups:
            g.system.sync()

    def case_state(self, k):
        """State of batch case k in its own coordinates and particle order."""
        gi, pos = self.where[k]
        g = self.groups[gi]
        st = g.system.download()
        lo, hi = g.base[pos], g.base[pos] + g.cases[pos].np
        sel = (st["index"] >= lo) & (st["index"] < hi)
        out = {f: st[f][sel] for f in st}
        out["index"] = out["index"] - lo
        out["r"] = out["r"] - np.array([g.offset[pos], 0.0])
        return out


# ------------------------------------------------------- one system, scaled
# Gap between the column ranges of two packed cases, in cells: more than the
# 2h support plus the distance a particle can travel past its case's removal
# box in the step before the corrector erases it.
CASE_GAP_CELLS = 4
# margin of a case's column range beyond its removal thresholds (m, unscaled)
CASE_MARGIN = 0.02


@dataclass
class ScaledPacking:
    """Where the cases of a batch go in one system (see :class:`Batch`)."""

    cases: list
    dp: float           # the system's spacing (the finest case's)
    h: float
    dt: float
    scale: np.ndarray   # lambda_k = dp / dp_k
    offset: np.ndarray  # x shift of case k in the system's frame
    base: np.ndarray    # first particle index of case k
    ranges: np.ndarray  # [lo, hi) of case k's grid columns
    boxes: np.ndarray   # removal thresholds (x_lo, x_hi, y_lo, y_hi) of case k
    gravity: np.ndarray
    domain: tuple


def pack_scaled(case_list, kap=2.1) -> ScaledPacking:
    """Case k scaled by dp / dp_k and placed along x with CASE_GAP_CELLS
    cells between the column ranges of neighbouring cases; its removal box is
    RemoveParticlesOutOfDomain's (src/SPH_btdebug.h:16-19, eps = 0.01 m) in
    the system's frame."""
    dp = min(c.spec.dp for c in case_list)
    h = 1.0 * math.sqrt(2 * dp * dp)
    kh = h * kap
    gap = CASE_GAP_CELLS * kh
    scale = np.array([dp / c.spec.dp for c in case_list])
    offs, bases, ranges, boxes = [], [], [], []
    x, base = 0.0, 0
    for k, (c, lam) in enumerate(zip(case_list, scale)):
        x0, x1, y0, y1 = c.domain
        lo, hi = lam * (x0 - CASE_MARGIN), lam * (x1 + CASE_MARGIN)
        off = (x + gap if k else 0.0) - lo
        offs.append(off)
        bases.append(base)
        base += c.np
        ranges.append((lo + off, hi + off))
        boxes.append((lam * (x0 - 0.01) + off, lam * (x1 - 0.01) + off, lam * (y0 - 0.01),
                      lam * (y1 + 0.01)))
        x = hi + off
    ranges = np.array(ranges)
    ylo = min(lam * (c.domain[2] - CASE_MARGIN) for c, lam in zip(case_list, scale))
    yhi = max(lam * (c.domain[3] + CASE_MARGIN) for c, lam in zip(case_list, scale))
    return ScaledPacking(list(case_list), dp, h, 0.00005 * (dp / 0.005), scale, np.array(offs),
                         np.array(bases, dtype=np.int64), ranges, np.array(boxes),
                         9.81 / scale, (ranges[0, 0], ranges[-1, 1], ylo, yhi))


class Batch:
    """The batched workload in ONE particle system (module docstring): case k
    scaled by ``scale[k]`` = dp_sys / dp_k and shifted by ``offset[k]`` along
    x, its particles at ``base[k]`` .. ``base[k] + np_k`` of the system's
    numbering, its gravity 9.81 / scale[k] and its removal box in the
    system's case table.  One ``step`` advances every case by its own dt_k
    (= dt / scale[k]) with one launch per kernel for the whole batch."""

    def __init__(self, specs, precision="fp32", stream=None, arrays=None, kap=2.1):
        from . import sph

        self.specs = list(specs)
        # `arrays`: the cases' particles when not those of case_arrays(spec)
        self.cases = list(arrays) if arrays is not None else [case_arrays(sp) for sp in self.specs]
        pk = pack_scaled(self.cases, kap)
        self.packing = pk
        self.dp, self.h, self.dt = pk.dp, pk.h, pk.dt
        self.kap, self.cs = kap, 35.0
        self.wall_model = _cases.WALL_MDBC
        self.scale, self.offset, self.base = pk.scale, pk.offset, pk.base
        self.ranges, self.boxes, self.gravity, self.domain = pk.ranges, pk.boxes, pk.gravity, pk.domain
        typ = np.concatenate([c.type for c in self.cases])
        r = np.concatenate([c.r * lam + np.array([off, 0.0])
                            for c, lam, off in zip(self.cases, self.scale, self.offset)])
        rho = np.concatenate([c.rho for c in self.cases])
        p = np.concatenate([c.p for c in self.cases])
        gnr = np.concatenate([(c.gnr * lam + np.array([off, 0.0])) * (c.type[:, None] == WALL)
                              for c, lam, off in zip(self.cases, self.scale, self.offset)])
        s = sph.ParticleSystem(self.h, self.kap, self.cs, 1000.0, 0.02, 0.1, self.dp,
                               self.domain, precision, stream=stream)
        s.add_particles(typ, r, None, rho, p, gnr)
        s.divide_to_cells()
        s.set_cases(self.ranges, self.gravity, self.boxes)
        s.particle_to_cell()
        self.system = s

    @property
    def np(self):
        return int(sum(c.np for c in self.cases))

    def step(self, n=1):
        self.system.step(self.wall_model, self.dt, n)

    def sync(self):
        self.system.sync()

    def case_dt(self, k):
        """The physical time step of case k (one system step)."""
        return self.dt / self.scale[k]

    def case_state(self, k, st=None):
        """State of batch case k in its own units, coordinates and particle
        order (``st``: a download of the system to reuse)."""
        st = self.system.download() if st is None else st
        lo, hi = self.base[k], self.base[k] + self.cases[k].np
        sel = (st["index"] >= lo) & (st["index"] < hi)
        out = {f: st[f][sel] for f in st}
        lam = self.scale[k]
        out["index"] = out["index"] - lo
        out["r"] = (out["r"] - np.array([self.offset[k], 0.0])) / lam
        if "a" in out:
            out["a"] = out["a"] * lam
        if "drho" in out:
            out["drho"] = out["drho"] * lam
        return out
