"""Edge cases of the step through the C ABI against the oracle: no walls, no
fluid, one isolated particle (free fall, and the boundary-integral flavour's
empty Shepard sum), and a particle thrown out of the domain inside the fused
step."""

import math

import numpy as np
import pytest

from tinysph_old_gb300 import cases
from tinysph_old_gb300 import geometry as geo

DP = 0.02


def _case(ps, model, dt=4e-4, name="edge"):
    h = math.sqrt(2 * DP * DP)
    nvl = int(math.ceil(2.1 * h / DP))
    return cases.Case(name=name, particles=ps, h=h, kap=2.1, cs=34.3, rho0=1000.0, visco=0.02,
                      delta=0.1, dp=DP, domain=cases._pad(0.0, 1.0, 0.0, 1.0, nvl, DP),
                      wall_model=model, dt=dt, meta={})


def _set(kind="plain"):
    h = math.sqrt(2 * DP * DP)
    return (geo.AleParticleSet if kind == "bt" else geo.ParticleSet)(DP, h, 2.1, 34.3)


def _compare(gpu, orc, precision, scale_tol=1e-9):
    a, b = gpu.download(), orc.state()
    ob = np.argsort(b["index"])
    assert np.array_equal(a["index"], b["index"][ob])
    for f in ("r", "v", "rho", "p"):
        x, y = a[f], b[f][ob]
        tol = (scale_tol if precision == "fp64" else 1e-4) * max(1.0, float(np.max(np.abs(y))))
        assert float(np.max(np.abs(x - y))) <= tol, (f, float(np.max(np.abs(x - y))), tol)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_fluid_without_walls(gpu_tsph, oracle_mod, precision):
    ps = _set()
    geo.create_block_of_fluid(ps, 0.3, 0.3, 0.5, 0.5)
    case = _case(ps, 0)
    g = gpu_tsph.ParticleSystem.from_case(case, precision)
    o = oracle_mod.PortSystem.from_case(case)
    g.step(0, case.dt, 20)
    o.step(0, case.dt, 20)
    _compare(g, o, precision)


@pytest.mark.gpu
def test_walls_without_fluid(gpu_tsph, oracle_mod):
    ps = _set()
    geo.create_wall_x_mdbc(ps, 0.2, 0.8, 0.2, -1, 0.2 + DP / 2)
    case = _case(ps, 0)
    g = gpu_tsph.ParticleSystem.from_case(case, "fp64")
    o = oracle_mod.PortSystem.from_case(case)
    g.step(0, case.dt, 5)
    o.step(0, case.dt, 5)
    _compare(g, o, "fp64")
    assert g.np == case.np


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_single_particle_falls_freely(gpu_tsph, oracle_mod, precision):
    ps = _set()
    ps.add(geo.FLUID, 0.0, 1000.0, (0.5, 0.8))
    case = _case(ps, 0)
    g = gpu_tsph.ParticleSystem.from_case(case, precision)
    o = oracle_mod.PortSystem.from_case(case)
    n = 50
    g.step(0, case.dt, n)
    o.step(0, case.dt, n)
    _compare(g, o, precision, 1e-12)
    st = g.download()
    t = n * case.dt
    # the symplectic scheme is exact for a constant acceleration
    assert abs(st["v"][0, 1] + 9.81 * t) <= 1e-6 and abs(st["r"][0, 1] - (0.8 - 0.5 * 9.81 * t * t)) <= 1e-8


@pytest.mark.gpu
def test_boundary_integral_isolated_particle(gpu_tsph, oracle_mod):
    """A fluid particle with no fluid neighbour: the Shepard sum is 0, so
    a = -g and drho = 0 (src/SPH_interactionBT.h:180-186)."""
    ps = _set("bt")
    geo.create_wall_x_bt(ps, 0.2, 0.8, 0.2, -1, (0.0, 1.0))
    ps.add(geo.FLUID, 0.0, 1000.0, (0.5, 0.6))
    ps.gnr = list(ps.normals)
    case = _case(ps, 2)
    g = gpu_tsph.ParticleSystem.from_case(case, "fp64")
    o = oracle_mod.PortBt.from_case(case)
    g.bt_density()
    g.density_to_pressure()
    g.compute_forces(2)
    o.bt_density()
    o.density_to_pressure()
    o.compute_forces(2)
    a, b = g.download(), o.state()
    fl = a["type"] == 0
    assert np.allclose(a["a"][fl], [[0.0, -9.81]]) and np.all(a["drho"][fl] == 0.0)
    assert np.allclose(a["a"], b["a"]) and np.allclose(a["rho"], b["rho"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision,variant", [("fp64", None), ("fp32", 0), ("fp32", 2)])
def test_particle_thrown_out_inside_the_fused_step(gpu_tsph, oracle_mod, precision, variant):
    ps = _set()
    geo.create_block_of_fluid(ps, 0.3, 0.3, 0.4, 0.4)
    case = _case(ps, 0)
    g = gpu_tsph.ParticleSystem.from_case(case, precision)
    if variant is not None:
        g.set_tile_shape(variant)
    o = oracle_mod.PortSystem.from_case(case)
    st = g.download()
    v = st["v"].copy()
    r = st["r"].copy()
    k = len(r) - 1
    r[k] = (0.4, case.domain[3] - 0.03)
    v[k] = (0.0, 40.0)  # leaves through the top within two steps
    g.upload(r=r, v=v)
    g.particle_to_cell()
    o.set_state(r=r, v=v)
    o.clear_cells()
    o.particle_to_cell()
    g.step(0, case.dt, 4)
    o.step(0, case.dt, 4)
    assert g.np == case.np - 1 and o.np() == case.np - 1
    _compare(g, o, precision)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,variant", [("fp64", None), ("fp32", 0), ("fp32", 2)])
def test_fused_step_erase_skips_the_particle_after_an_erased_one(gpu_tsph, oracle_mod, precision,
                                                                 variant):
    """Three particles of consecutive indices leave the domain in the same
    fused step.  RemoveParticlesOutOfDomain erases inside a forward loop
    (src/SPH_btdebug.h:14-29), so the first is erased, the second is not
    examined in that step (it goes on, outside the domain, and is erased in
    the next one) and the third is erased: the fused step keeps the oracle's
    survivor set step by step."""
    ps = _set()
    geo.create_block_of_fluid(ps, 0.3, 0.3, 0.4, 0.4)
    case = _case(ps, 0)
    g = gpu_tsph.ParticleSystem.from_case(case, precision)
    if variant is not None:
        g.set_tile_shape(variant)
    o = oracle_mod.PortSystem.from_case(case)
    st = g.download()
    v = st["v"].copy()
    r = st["r"].copy()
    n = len(r)
    # The right edge is the one side where a point can lie outside the box
    # (x > xm - 0.01) and still inside the cell grid, which reaches
    # x0 - 0.273 h + ncx kh: there the skipped particle stays binned until the
    # next step erases it.  All three reach that band in the first step.
    xm, eps = case.domain[1], 0.01
    kh, of = case.kap * case.h, 0.273 * case.h
    ncx = int((xm - case.domain[0] + of) / kh) + 1
    grid_right = case.domain[0] - of + ncx * kh
    x_start, vx = xm - eps - 0.005, 20.0
    x_next = x_start + vx * case.dt
    assert xm - eps + 1e-3 < x_next < grid_right - 1e-3
    for k, y in zip((n - 3, n - 2, n - 1), (0.40, 0.44, 0.48)):
        assert st["type"][k] == 0
        r[k] = (x_start, y)
        v[k] = (vx, 0.0)
    g.upload(r=r, v=v)
    g.particle_to_cell()
    o.set_state(r=r, v=v)
    o.clear_cells()
    o.particle_to_cell()
    counts = []
    for _ in range(4):
        g.step(0, case.dt, 1)
        o.step(0, case.dt, 1)
        assert g.np == o.np()
        counts.append(g.np)
        _compare(g, o, precision)
    # the erase with the skip: n -> n - 2 in one step, n - 3 in the next
    assert counts[:2] == [n - 2, n - 3] and counts[-1] == n - 3


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_remove_skips_the_particle_after_an_erased_one(gpu_tsph, oracle_mod, precision):
    """RemoveParticlesOutOfDomain erases inside a forward loop
    (src/SPH_btdebug.h:4-31): of three consecutive particles outside the box
    the first and the third go, the second stays until the next call."""
    ps = _set()
    geo.create_block_of_fluid(ps, 0.3, 0.3, 0.4, 0.4)
    case = _case(ps, 0)
    g = gpu_tsph.ParticleSystem.from_case(case, precision)
    o = oracle_mod.PortSystem.from_case(case)
    st = g.download()
    r = st["r"].copy()
    for k in (10, 11, 12, 20):
        r[k] = (0.5, case.domain[3] + 0.05)
    g.upload(r=r)
    o.set_state(r=r)
    assert g.remove_out_of_domain() == o.remove_out_of_domain() == 3
    assert g.np == case.np - 3
    # the skipped one goes in the next call
    assert g.remove_out_of_domain() == o.remove_out_of_domain() == 1
    assert g.np == case.np - 4
