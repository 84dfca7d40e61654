"""The oracle's boundary-integral (BT) walls against the reference's own
outputs (tests/golden/dam_break_bt_dp0.02.npz and still_water_bt_dp0.02.npz, made by
tests/golden/make_golden.py from src/SPH_interactionBT.h, src/SPH_BT.h and
the RUN loop of cases/damBreakLong_BT/SPH_simulationSymplectic.h), and the
case generator against the reference's generators."""

import os
import sys

import numpy as np

from tinysph_old_gb300 import cases

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import oracle as O  # noqa: E402

GOLD = np.load(os.path.join(HERE, "golden", "dam_break_bt_dp0.02.npz"))


def _rel(a, b):
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


def test_bt_generator_matches_the_reference_generators():
    case = cases.dam_break_bt(dp=0.02)
    a = case.particles.arrays()
    assert np.array_equal(a["r"], GOLD["geom_r"])
    assert np.array_equal(a["type"], GOLD["geom_type"])
    assert np.array_equal(a["rho"], GOLD["geom_rho"])
    assert np.array_equal(a["p"], GOLD["geom_p"])
    assert np.array_equal(np.array(case.particles.normals), GOLD["geom_normals"])


def _port():
    case = cases.dam_break_bt(dp=0.02)
    o = O.PortBt.from_case(case)
    o.set_state(v=GOLD["init_v"], rho=GOLD["init_rho"])
    return case, o


def test_bt_density_and_forces_match_the_reference():
    case, o = _port()
    o.bt_density()
    o.density_to_pressure()
    o.compute_forces(O.ORC_BT)
    st = o.state()
    for f in ("rho", "p", "a", "drho"):
        assert _rel(st[f], GOLD[f"forces_{f}"]) <= 1e-12, f


def test_bt_steps_match_the_reference():
    case, o = _port()
    for k in (10, 20):
        o.step(O.ORC_BT, float(GOLD["dt"]), 10)
        st = o.state()
        assert np.array_equal(st["index"], GOLD[f"step{k}_index"])
        for f in ("r", "v", "rho", "p", "a", "drho"):
            assert _rel(st[f], GOLD[f"step{k}_{f}"]) <= 1e-10, (k, f)


def test_bt_still_water_steps_match_the_reference():
    """cases/stillWater_BT from its hydrostatic start: the reference's RUN
    loop (tests/golden/still_water_bt_dp0.02.npz) against the oracle."""
    g = np.load(os.path.join(HERE, "golden", "still_water_bt_dp0.02.npz"))
    case = cases.still_water_bt(dp=0.02)
    o = O.PortBt.from_case(case)
    done = 0
    for n in g["snaps"]:
        o.step(O.ORC_BT, float(g["dt"]), int(n) - done)
        done = int(n)
        st = o.state()
        assert np.array_equal(st["index"], g[f"step{n}_index"])
        for f in ("r", "v", "rho", "p", "a", "drho"):
            assert _rel(st[f], g[f"step{n}_{f}"]) <= 1e-10, (int(n), f)
