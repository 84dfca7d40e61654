"""The ALE-SPH oracle (oracle/tsph_oracle_ale.c) against golden vectors the
reference produced (tests/golden/make_golden.py ale) and, where the reference
sources are present, against the reference live.  Bit-exact comparisons."""

import os

import numpy as np
import pytest

from tinysph_old_gb300 import cases

GOLD = os.path.join(os.path.dirname(__file__), "golden")
FIELDS = ("r", "v", "rho", "p", "omega", "omegarho", "omegav", "domega", "domegarho", "domegav",
          "index")


def _gold():
    return np.load(os.path.join(GOLD, "dam_break_ale_dp0.02.npz"))


def _port(O, case, g):
    P = O.PortAle.from_case(case)
    P.set_threads(1)
    P.set_velocity_density(g["init_v"], g["init_rho"])
    return P


def test_ale_geometry_matches_reference_generators():
    """Create_Wall_x_bt / Create_Wall_y_bt / Create_corner_bt /
    Create_Block_of_Fluid (src/ALESPH_create.h:690-793) restated in
    geometry.py give the reference's particles and normals bit for bit."""
    g = _gold()
    case = cases.dam_break_ale(dp=0.02)
    a = case.particles.arrays()
    assert np.array_equal(a["r"], g["geom_r"])
    assert np.array_equal(a["type"], g["geom_type"])
    assert np.array_equal(np.asarray(case.particles.normals), g["geom_normals"])
    assert np.array_equal(np.full(case.np, 0.02 * 0.02), g["geom_omega"])


def test_ale_oracle_matches_reference_golden(oracle_mod):
    O = oracle_mod
    g = _gold()
    case = cases.dam_break_ale(dp=0.02)
    P = _port(O, case, g)
    st = P.ale_state()
    for k in ("r", "v", "rho", "omega", "omegarho", "omegav"):
        assert np.array_equal(st[k], g[f"init_{k}"]), k
    P.density_to_pressure()
    P.gradient()
    P.ale_forces(float(g["dt"]))
    st = P.ale_state()
    for k in ("grad", "domega", "domegarho", "domegav"):
        assert np.array_equal(st[k], g[f"forces_{k}"]), k
    P2 = _port(O, case, g)
    every = int(g["snap_every"])
    for k in range(every, int(g["nsteps"]) + 1, every):
        P2.ale_step(float(g["dt"]), k - every, every)
        st = P2.ale_state()
        for f in FIELDS:
            assert np.array_equal(st[f], g[f"step{k}_{f}"]), (k, f)


def test_ale_oracle_thread_independent(oracle_mod):
    """The oracle's OpenMP loops write disjoint particles: results do not
    depend on the thread count."""
    O = oracle_mod
    g = _gold()
    case = cases.dam_break_ale(dp=0.02)
    out = []
    for t in (1, 4):
        P = _port(O, case, g)
        P.set_threads(t)
        P.ale_step(float(g["dt"]), 0, 4)
        out.append(P.ale_state())
    for f in FIELDS:
        assert np.array_equal(out[0][f], out[1][f]), f


def test_ale_muscl_scheme_reduces_to_first_order_for_linear_fields(oracle_mod):
    """The MUSCL scheme (no counterpart in the reference) with all gradients
    zero and a uniform velocity gives the reference's fluxes up to rounding:
    both reconstructions collapse to the particle states."""
    O = oracle_mod
    case = cases.dam_break_ale(dp=0.02)
    res = []
    for scheme in (0, 1):
        P = O.PortAle.from_case(case)
        P.set_threads(1)
        st = P.state()
        fl = st["type"] == 0
        v = np.zeros_like(st["v"])
        v[fl] = (0.1, -0.05)
        rho = st["rho"].copy()
        rho[fl] = 1000.0 + 0.01 * st["r"][fl, 1]
        P.set_velocity_density(v, rho)
        P.set_scheme(scheme)
        P.density_to_pressure()
        P.ale_forces(case.dt)  # gradients stay zero: no gradient pass
        res.append(P.ale_state())
    for k in ("domega", "domegarho", "domegav"):
        a, b = res[0][k], res[1][k]
        assert np.allclose(a, b, rtol=1e-9, atol=1e-9 * np.max(np.abs(a))), k


def test_ale_oracle_matches_live_reference_dp001(oracle_mod):
    """Where the reference sources are present: 5 steps at dp = 0.01."""
    O = oracle_mod
    if not O.ref_ale_available():
        pytest.skip("reference ALE harness not built (needs the reference sources)")
    case = cases.dam_break_ale(dp=0.01)
    R = O.RefAle.from_case(case)
    P = O.PortAle.from_case(case)
    rng = np.random.default_rng(7)
    a = case.particles.arrays()
    fl = a["type"] == 0
    v = np.zeros((case.np, 2))
    v[fl] = rng.normal(0, 0.05, (fl.sum(), 2))
    rho = np.full(case.np, 1000.0)
    rho[fl] *= 1 + 1e-3 * rng.standard_normal(fl.sum())
    R.set_velocity_density(v, rho)
    P.set_velocity_density(v, rho)
    O.RefAle.set_threads(1)
    R.ale_step(case.dt, 0, 5)
    P.set_threads(4)
    P.ale_step(case.dt, 0, 5)
    x, y = R.ale_state(), P.ale_state()
    for f in FIELDS + ("grad",):
        assert np.array_equal(x[f], y[f]), f


def test_first_order_oracle_matches_reference_golden(oracle_mod):
    """The first-order driver (cases/ALESPH_dambreakLong/SPH_simulationINT.h,
    src/RALESPH_interaction.h): fluxes and 6 steps, bit for bit."""
    O = oracle_mod
    g = np.load(os.path.join(GOLD, "dam_break_ale_first_order_dp0.02.npz"))
    case = cases.dam_break_ale(dp=0.02)
    P = _port(O, case, g)
    P.density_to_pressure()
    P.ale_forces_first_order()
    st = P.ale_state()
    for k in ("domega", "domegarho", "domegav"):
        assert np.array_equal(st[k], g[f"forces_{k}"]), k
    P2 = _port(O, case, g)
    P2.set_scheme(2)
    every = int(g["snap_every"])
    for k in range(every, int(g["nsteps"]) + 1, every):
        P2.ale_step(float(g["dt"]), k - every, every)
        st = P2.ale_state()
        for f in FIELDS:
            assert np.array_equal(st[f], g[f"step{k}_{f}"]), (k, f)


def test_ale_still_water_matches_reference_golden(oracle_mod):
    """cases/ALESPH_stillWater (the stillWater_BT tank, hydrostatic start,
    h = 2 dp): per-function outputs and 6 steps of the MUSCL.h RUN loop from a
    seeded perturbation, bit for bit (tests/golden/still_water_ale_dp0.02.npz)."""
    O = oracle_mod
    g = np.load(os.path.join(GOLD, "still_water_ale_dp0.02.npz"))
    case = cases.still_water_ale(dp=0.02)
    P = _port(O, case, g)
    st = P.ale_state()
    for k in ("r", "v", "rho", "omega", "omegarho", "omegav"):
        assert np.array_equal(st[k], g[f"init_{k}"]), k
    P.density_to_pressure()
    P.gradient()
    P.ale_forces(float(g["dt"]))
    st = P.ale_state()
    for k in ("grad", "domega", "domegarho", "domegav"):
        assert np.array_equal(st[k], g[f"forces_{k}"]), k
    P2 = _port(O, case, g)
    every = int(g["snap_every"])
    for k in range(every, int(g["nsteps"]) + 1, every):
        P2.ale_step(float(g["dt"]), k - every, every)
        st = P2.ale_state()
        for f in FIELDS:
            assert np.array_equal(st[f], g[f"step{k}_{f}"]), (k, f)
