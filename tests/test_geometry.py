"""Host-side case builders against the reference's own generators
(tests/golden/geometry.npz, produced by the reference's src/SPH_create.h)."""

import os

import numpy as np
import pytest

from tinysph_old_gb300 import cases, geometry

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "geometry.npz"))


@pytest.mark.parametrize("dp", [0.02, 0.01])
def test_dam_break_geometry_bit_exact(dp):
    case = cases.dam_break_mdbc(dp=dp)
    a = case.particles.arrays()
    assert np.array_equal(a["r"], GOLD[f"dam_dp{dp:g}_r"])
    assert np.array_equal(a["type"], GOLD[f"dam_dp{dp:g}_type"])
    assert np.array_equal(a["rho"], GOLD[f"dam_dp{dp:g}_rho"])
    assert np.array_equal(a["gnr"], GOLD[f"dam_dp{dp:g}_gnr"])


def test_fluid_wp_and_dbc_walls_bit_exact():
    dp = 0.02
    ps = geometry.ParticleSet(dp, 1.5 * dp, 2.1, 20.0)
    geometry.create_wall_x(ps, 0.0, 0.5, 0.0, -1)
    geometry.create_wall_y(ps, 0.0, 0.0 + dp, 0.4, -1)
    geometry.create_block_of_fluid_wp(ps, 0 + dp, 0 + dp, 0.5 - dp, 0.3)
    a = ps.arrays()
    assert np.array_equal(a["r"], GOLD["wp_dp0.02_r"])
    assert np.array_equal(a["type"], GOLD["wp_dp0.02_type"])
    assert np.array_equal(a["rho"], GOLD["wp_dp0.02_rho"])
    assert np.array_equal(a["p"], GOLD["wp_dp0.02_p"])


def test_benchmark_case_sizes():
    """The dam-break sweep of the benchmark: ~45k / 180k / 720k fluid."""
    sizes = {}
    for dp in (0.002, 0.001, 0.0005):
        c = cases.dam_break_benchmark(dp)
        nf = int(np.sum(np.asarray(c.particles.type) == 0))
        sizes[dp] = (nf, c.np)
    assert 44_000 < sizes[0.002][0] < 46_000
    assert 178_000 < sizes[0.001][0] < 182_000
    assert 715_000 < sizes[0.0005][0] < 722_000
    # walls are a few percent
    assert sizes[0.0005][1] - sizes[0.0005][0] < 0.05 * sizes[0.0005][1]


def test_still_water_case():
    c = cases.still_water_dbc(dp=0.005)
    t = np.asarray(c.particles.type)
    assert int(np.sum(t == 0)) == 6000
    assert abs(c.dt - 0.2 * 1.5 * 0.005 / 20.0) < 1e-15
    # three wall layers below the water
    ry = np.asarray(c.particles.ry)
    assert np.isclose(ry[t == 1].min(), -2.5 * 0.005)
