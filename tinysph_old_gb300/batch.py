"""Many independent WCSPH cases stepped together on one GPU.

The batched workload is a set of seeded dam-break and still-water tanks of
different sizes and resolutions.  Cases that share every SPH constant (the
same kind and particle spacing, hence the same h, dt, mass, sound speed and
wall model) form a group.  A group is packed into one domain: the tanks sit
side by side along x, each shifted by an entry of the group's case table and
separated by an empty gap, and the group runs as one particle system, so
every kernel launch of a step covers all of its cases at once (one counting
sort, one pair pass over all cells of all tanks).  A particle interacts only
with particles within 2h of it, so tanks more than 2h apart never see each
other; the gap is wide enough that a particle thrown over a tank wall falls
below the floor level (and leaves the domain) before it can reach the next
tank.  Per-case results therefore agree with separate runs of each case up to
FP32 rounding (the cell grid is aligned differently and the positions are
shifted by the case offset).

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
    0.8 m high, water column ``col_w`` x ``col_h`` at the left wall, mDBC,
    c0 = 35 m/s, h = sqrt(2) dp.  Still water: water ``tank`` wide and
    ``col_h`` deep filling a tank of the same width, 3 DBC wall layers,
    c0 = 20 m/s, h = 1.5 dp."""

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
    # still water (cases.still_water_dbc: water col_w wide filling the tank,
    # col_h deep, tank col_h + 0.1 high, 3 wall layers, hydrostatic start)
    return _still_water(spec, dp, spec.col_w, spec.col_h, spec.col_h + 0.1, 20.0, 3)


def _still_water(spec, dp, width, depth, tank_height, cs, layers):
    kap = 2.1
    h = 1.5 * dp
    nx, ny, nyw = int(round(width / dp)), int(round(depth / dp)), int(round(tank_height / dp))
    b = cs * cs * 1000.0 / 7.0

    def hydro(y):
        # per distinct height, with math.pow (libm pow, as geometry.pressure_to_density)
        uy, inv = np.unique(y, return_inverse=True)
        up = np.array([0.0 if v >= depth else 9.81 * (depth - v) * 1000 for v in uy])
        ur = np.array([1000.0 if v >= depth else math.pow(q / b + 1, 1.0 / 7) * 1000.0
                       for v, q in zip(uy, up)])
        return up[inv], ur[inv]

    xs, ys = [], []
    for l in range(layers):
        i = np.arange(-layers, nx + layers, dtype=np.float64)
        xs.append((i + 0.5) * dp)
        ys.append(np.full(len(i), -(l + 0.5) * dp))
    jw = np.arange(nyw, dtype=np.float64)
    for side in (0, 1):
        for l in range(layers):
            x = -(l + 0.5) * dp if side == 0 else width + (l + 0.5) * dp
            xs.append(np.full(nyw, x))
            ys.append((jw + 0.5) * dp)
    wx, wy = np.concatenate(xs), np.concatenate(ys)
    i = np.arange(nx, dtype=np.float64)
    j = np.arange(ny, dtype=np.float64)
    fx, fy = np.repeat((i + 0.5) * dp, ny), np.tile((j + 0.5) * dp, nx)
    x, y = np.concatenate([wx, fx]), np.concatenate([wy, fy])
    p, rho = hydro(y)
    typ = np.concatenate([np.full(len(wx), WALL, np.int32), np.full(len(fx), FLUID, np.int32)])
    pad = (layers + 2) * dp
    dom = (0.0 - pad, width + pad, 0.0 - pad, tank_height + pad)
    return CaseArrays(spec, typ, np.stack([x, y], 1), rho, p, np.zeros((len(x), 2)), h, kap, cs,
                      0.2 * h / cs, _cases.WALL_DBC, dom, (dom[0], dom[1]))


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


class Batch:
    """The batched workload: one packed particle system per group of equal
    constants.  ``step(n)`` advances every group by n of its own time steps
    (all graph launches enqueued before any synchronisation, one stream per
    group)."""

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
