"""The oracle's open boundaries (inlet / outlet buffer zones,
src/SPH_buffer_zones.h) against the reference's own runs
(tests/golden/inflow_slab_mdbc_dp0.005.npz, outlet_channel_mdbc_dp0.005.npz,
flow_drop_mdbc_dp0.02.npz, made by tests/golden/make_golden.py): particle counts, types and state at
every snapshot, bit for bit (x86 here; 1e-12 relative allowed for libm)."""

import os
import sys

import numpy as np
import pytest

from tinysph_old_gb300 import cases

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import oracle as O  # noqa: E402


@pytest.mark.parametrize("fname,builder", [
    ("inflow_slab_mdbc_dp0.005.npz", lambda: cases.inflow_slab_mdbc(dp=0.005)),
    ("outlet_channel_mdbc_dp0.005.npz", lambda: cases.outlet_channel_mdbc(dp=0.005)),
    ("flow_drop_mdbc_dp0.02.npz", lambda: cases.flow_drop_mdbc(dp=0.02)),
])
def test_zones_match_the_reference(fname, builder):
    g = np.load(os.path.join(HERE, "golden", fname))
    case = builder()
    P = O.PortSystem.from_case(case)
    done = 0
    for n in g["snaps"]:
        P.step_zones(float(g["dt"]), int(n) - done)
        done = int(n)
        st = P.state()
        assert np.array_equal(st["type"], g[f"step{n}_type"]), n
        for f in ("r", "v", "rho", "p"):
            ref = g[f"step{n}_{f}"]
            assert np.max(np.abs(st[f] - ref)) <= 1e-12 * max(1.0, float(np.max(np.abs(ref)))), (n, f)


def test_flow_drop_bt_matches_the_reference():
    """cases/flowDrop_BT: the case generator against the reference's
    generators, and the RUN loop (BT wall density and forces with the inlet
    and the two outlets after the predictor) bit for bit while the reference
    is defined: until its first erasure, whose Remove_particle also erases
    past the end of a vector the BT generators leave short
    (tests/golden/flow_drop_bt_dp0.02.npz)."""
    g = np.load(os.path.join(HERE, "golden", "flow_drop_bt_dp0.02.npz"))
    case = cases.flow_drop_bt(dp=0.02)
    a = case.particles.arrays()
    assert np.array_equal(a["r"], g["geom_r"])
    assert np.array_equal(a["type"], g["geom_type"])
    assert np.array_equal(a["v"], g["geom_v"])
    assert np.array_equal(np.asarray(case.particles.normals), g["geom_normals"])
    P = O.PortBt.from_case(case)
    done = 0
    for n in g["snaps"]:
        P.step_zones(float(g["dt"]), int(n) - done, model=O.ORC_BT)
        done = int(n)
        st = P.state()
        assert np.array_equal(st["type"], g[f"step{n}_type"]), n
        for f in ("r", "v", "rho", "p", "a", "drho"):
            assert np.array_equal(st[f], g[f"step{n}_{f}"]), (int(n), f)


def test_inflow_tank_bottom_matches_the_reference():
    """cases/inflowTankBottom_mDBC (an inlet feeding a ledge above a tank): the
    case generator against the reference's generators and the RUN loop bit
    for bit over 1500 steps (tests/golden/inflow_tank_bottom_mdbc_dp0.02.npz)."""
    g = np.load(os.path.join(HERE, "golden", "inflow_tank_bottom_mdbc_dp0.02.npz"))
    case = cases.inflow_tank_bottom_mdbc(dp=0.02)
    a = case.particles.arrays()
    for k in ("r", "v", "rho", "p", "type"):
        assert np.array_equal(a[k], g[f"geom_{k}"]), k
    P = O.PortSystem.from_case(case)
    done = 0
    for n in g["snaps"]:
        P.step_zones(float(g["dt"]), int(n) - done)
        done = int(n)
        st = P.state()
        assert np.array_equal(st["type"], g[f"step{n}_type"]), n
        for f in ("r", "v", "rho", "p"):
            assert np.array_equal(st[f], g[f"step{n}_{f}"]), (int(n), f)
