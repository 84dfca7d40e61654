"""Boundary-integral (BT) walls on the GPU through the C ABI against the
reference's golden vectors (tests/golden/dam_break_bt_dp0.02.npz: the
reference's src/SPH_BT.h wall density, src/SPH_interactionBT.h forces and
the RUN loop of cases/damBreakLong_BT/SPH_simulationSymplectic.h).

Bars: FP64 build within 1e-9 of the field's scale (CUDA's pow and sqrt
against glibc's, and the within-cell summation order); FP32 build the
per-field bars of the WCSPH parity tests (FP32 rounding of ~25-term pair
sums), and 5e-3 kg/m^3 for the walls' Shepard densities."""

import os

import numpy as np
import pytest

from tinysph_old_gb300 import cases

GOLD = os.path.join(os.path.dirname(__file__), "golden", "dam_break_bt_dp0.02.npz")
BT = 2


def _err(a, b):
    return float(np.max(np.abs(np.asarray(a, dtype=np.float64) - np.asarray(b, dtype=np.float64))))


def _tol(precision, field, ref):
    mag = float(np.max(np.abs(ref))) if np.size(ref) else 0.0
    if precision == "fp64":
        return 1e-9 * max(1.0, mag)
    return {
        "r": 1e-9,
        "v": 2e-6 + 1e-5 * mag,
        "a": 2e-3 + 2e-5 * mag,
        "rho": 2e-4,
        "drho": 2e-2 + 2e-5 * mag,
        "p": 5e-2 + 1e-6 * mag,
    }[field]


def _system(tsph, g, precision):
    s = tsph.ParticleSystem.from_case(cases.dam_break_bt(dp=0.02), precision)
    s.upload(v=g["init_v"], rho=g["init_rho"])
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_bt_wall_density_and_forces(gpu_tsph, precision):
    g = np.load(GOLD)
    s = _system(gpu_tsph, g, precision)
    s.bt_density()
    s.density_to_pressure()
    st = s.download()
    wall = st["type"] == 1
    e = _err(st["rho"][wall], g["forces_rho"][wall])
    assert e <= (1e-9 * 1000 if precision == "fp64" else 5e-3), e
    s.compute_forces(BT)
    st = s.download()
    fl = st["type"] == 0
    for f in ("a", "drho"):
        ref = g[f"forces_{f}"][fl]
        e = _err(st[f][fl], ref)
        assert e <= _tol(precision, f, ref), (f, e)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_bt_fused_step_matches_reference(gpu_tsph, precision):
    """tsph_step with TSPH_WALL_BT (fused kernels, CUDA graph) against the
    reference's RUN loop, 20 steps."""
    g = np.load(GOLD)
    s = _system(gpu_tsph, g, precision)
    for k in (10, 20):
        s.step(BT, float(g["dt"]), 10)
        st = s.download()
        assert np.array_equal(st["index"], g[f"step{k}_index"])
        fl = st["type"] == 0
        for f in ("r", "v", "a", "rho", "drho", "p"):
            ref = g[f"step{k}_{f}"][fl]
            e = _err(st[f][fl], ref)
            lim = _tol(precision, f, ref) * (1 if precision == "fp64" else 1 + k)
            assert e <= lim, (k, f, e, lim)
    assert s.health() & ~gpu_tsph.HEALTH_REMOVED == 0


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_bt_still_water_against_oracle(gpu_tsph, oracle_mod, precision):
    """cases/stillWater_BT (h = 2 dp, ~50 neighbours per particle): 200 and
    2000 steps (0.4 s) against the oracle (itself equal to the reference bit
    for bit), and the column stays near hydrostatic: interior pressure within
    15 % (mean) of rho0 g H of p = rho0 g (0.5 - y) (measured 9 % at 0.4 s,
    the BT walls' compression wave)."""
    case = cases.still_water_bt(dp=0.02)
    s = gpu_tsph.ParticleSystem.from_case(case, precision)
    o = oracle_mod.PortBt.from_case(case)
    # the FP64 build drifts from the oracle's last bits (CUDA's pow, the
    # within-cell summation order), grown over 2000 steps: 1e3 x the bars
    for n, s64, s32 in ((200, 1.0, 1.0), (1800, 1e3, 10.0)):
        s.step(BT, case.dt, n)
        o.step(BT, case.dt, n)
        a, b = s.download(), o.state()
        ob = np.argsort(b["index"])
        assert np.array_equal(a["index"], b["index"][ob])
        fl = a["type"] == 0
        for f, l64, l32 in (("r", 1e-9, 2e-6), ("v", 1e-9, 2e-4), ("rho", 1e-7, 5e-3)):
            e = _err(a[f][fl], b[f][ob][fl])
            lim = l64 * s64 if precision == "fp64" else l32 * s32
            assert e <= lim, (n, f, e, lim)
    fl = a["type"] == 0
    x, y = a["r"][fl, 0], a["r"][fl, 1]
    inner = (x > 0.2) & (x < 0.6) & (y > 0.1) & (y < 0.4)
    err = np.abs(a["p"][fl][inner] - 1000.0 * 9.81 * (0.5 - y[inner])) / (1000.0 * 9.81 * 0.5)
    assert float(np.mean(err)) < 0.15, float(np.mean(err))
