"""Probes of the case drivers: water level (src/SPH_water_level.h) and the
Shepard point fields behind Pressure_in_point (src/testing.h), on the
reference's own state after 20 steps of the dp = 0.01 dam break
(tests/golden/make_golden.py probes).

Oracle: bit-exact against the reference.  GPU (FP64 probe arithmetic on the
device state): FP64 build within 1e-9; FP32 build (densities stored in FP32)
within a few of the reference's sampling steps for the water level and 1e-5
relative for the point fields.
"""

import os

import numpy as np
import pytest

from tinysph_old_gb300 import cases

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _gold():
    return np.load(os.path.join(GOLD, "probes_dam_break_dp0.01.npz"))


def test_probe_oracle_matches_reference(oracle_mod):
    g = _gold()
    case = cases.dam_break_mdbc(dp=0.01)
    P = oracle_mod.PortSystem.from_case(case)
    P.set_state(r=g["r"], v=g["v"], rho=g["rho"], p=g["p"])
    P.particle_to_cell()
    for (x, y0, inv), wl in zip(g["gauges"], g["water_level"]):
        assert P.water_level(x, y0, bool(inv)) == wl, (x, y0, inv)
    for (x, y), f in zip(g["points"], g["point_fields"]):
        assert np.array_equal(P.point_fields(x, y), f), (x, y)
    assert np.array_equal(g["point_fields"][:, 1], g["pressure_in_point"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_probes_gpu_vs_reference(gpu_tsph, precision):
    g = _gold()
    case = cases.dam_break_mdbc(dp=0.01)
    s = gpu_tsph.ParticleSystem.from_case(case, precision)
    s.upload(r=g["r"], v=g["v"], rho=g["rho"], p=g["p"])
    s.particle_to_cell()
    gauges = g["gauges"]
    wl = s.water_level(gauges[:, 0], gauges[:, 1], gauges[:, 2].astype(np.int32))
    dp_wl = case.dp * 0.00005
    i_cross = np.sqrt(2.0 * 0.5 / dp_wl)  # sampling step near the top of the tank
    tol_wl = 1e-9 if precision == "fp64" else 4 * dp_wl * i_cross
    assert np.max(np.abs(wl - g["water_level"])) <= tol_wl, (wl, g["water_level"])
    pf = s.point_fields(g["points"])
    ref = g["point_fields"]
    for k, scale in enumerate((1000.0, max(1.0, np.max(np.abs(ref[:, 1]))), 1.0, 1.0)):
        tol = (1e-9 if precision == "fp64" else 1e-5) * scale
        assert np.max(np.abs(pf[:, k] - ref[:, k])) <= tol, (k, pf[:, k], ref[:, k])
    assert gpu_tsph.Pressure_in_point(s, None, g["points"][4]) == pytest.approx(
        ref[4, 1], rel=1e-5, abs=1e-6)


@pytest.mark.gpu
def test_water_front_is_the_largest_x_below_the_height(gpu_tsph):
    g = _gold()
    case = cases.dam_break_mdbc(dp=0.01)
    s = gpu_tsph.ParticleSystem.from_case(case, "fp32")
    s.upload(r=g["r"], v=g["v"], rho=g["rho"], p=g["p"])
    s.particle_to_cell()
    fl = g["type"] == 0
    for ymax in (0.02, 0.1, 1.0):
        sel = fl & (g["r"][:, 1] <= ymax)
        assert s.water_front(ymax) == np.max(g["r"][sel, 0])
    assert np.isnan(s.water_front(-1.0))
