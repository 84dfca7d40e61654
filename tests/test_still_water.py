"""Still water with DBC walls (tank 0.6 x 0.4 m, water 0.5 x 0.3 m, dp =
0.005 m: 6,000 fluid particles, 3 wall layers, h = 1.5 dp, c0 = 20 m/s,
dt = 0.2 h / c0): the hydrostatic pressure profile after 20,000 steps and
the fields after 2,000 steps against the oracle (the reference's algorithm
in FP64 on the host cores).

Bars (measured on a GB300: mean / max hydrostatic error 0.69 % / 2.0 % of
rho0 g H in both precisions after 20,000 steps; after 2,000 steps the FP64
build is within 3e-9 m of the oracle, the FP32 build within 7e-8 m):
mean <= 1.5 %, max <= 4 % of rho0 g H below 3 cm under the surface; fields
within the stated FP32 / FP64 tolerances.
"""

import os

import numpy as np
import pytest

from tinysph_old_gb300 import cases

G = 9.81
H = 0.3


def _hydro_error(st):
    fl = st["type"] == 0
    y = st["r"][fl, 1]
    p = st["p"][fl]
    err = np.abs(p - 1000.0 * G * (H - y))[y < H - 0.03] / (1000.0 * G * H)
    return float(np.mean(err)), float(np.max(err))


@pytest.mark.gpu
def test_still_water_stays_hydrostatic_20000_steps(gpu_tsph):
    case = cases.still_water_dbc(dp=0.005)
    s = gpu_tsph.ParticleSystem.from_case(case, "fp32")
    for _ in range(4):
        s.step(case.wall_model, case.dt, 5000)
        mean, mx = _hydro_error(s.download())
        assert mean <= 0.015 and mx <= 0.04, (mean, mx)
    st = s.download()
    assert s.health() == 0
    assert s.np == case.np  # nothing leaves the tank
    fl = st["type"] == 0
    assert np.max(np.abs(st["v"][fl])) < 0.05  # at rest up to the WCSPH noise


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol_r,tol_v,tol_rho,tol_p",
                         [("fp64", 1e-7, 2e-6, 2e-5, 1e-2), ("fp32", 1e-6, 2e-5, 1e-3, 0.5)])
def test_still_water_2000_steps_vs_oracle(gpu_tsph, oracle_mod, precision, tol_r, tol_v, tol_rho,
                                          tol_p):
    case = cases.still_water_dbc(dp=0.005)
    P = oracle_mod.PortSystem.from_case(case)
    P.set_threads(os.cpu_count() or 1)
    P.step(case.wall_model, case.dt, 2000)
    ref = P.state()
    s = gpu_tsph.ParticleSystem.from_case(case, precision)
    s.step(case.wall_model, case.dt, 2000)
    st = s.download()
    assert np.array_equal(st["index"], ref["index"])
    for f, tol in (("r", tol_r), ("v", tol_v), ("rho", tol_rho), ("p", tol_p)):
        e = float(np.max(np.abs(st[f] - ref[f])))
        assert e <= tol, (f, e, tol)
