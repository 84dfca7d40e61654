"""Precision of the FP32 build over physical time, asserted.

* The benchmark dam break (739,278 particles, dp = 0.0005, mDBC): the FP32
  build against the FP64 build of the same kernels after 200 steps, per
  field.  Measured on a GB300: fluid r 6.0e-12 m, v 2.0e-8 m/s (1.2e-6 of the
  largest |v|), rho 6.4e-7 kg/m^3, p 7.9e-4 Pa (3.2e-6 of the largest |p|);
  the bars below are about ten times that.
* The same dam break at dp = 0.004 (13,674 particles) to t = 0.5 s: the water
  front (largest fluid x below 5 cm, src/SPH_water_level.h) and the water
  level at the four gauges of cases/damBreakLong_mDBC/constants.h:58-80 every
  0.05 s, FP32 against FP64.  Measured: front within 6.5e-4 relative (before
  the impact on the far wall at ~0.4 s: within 1.1e-4), gauges within
  3.7e-4 m.  After the impact the splash is chaotic, so the bars are a few
  times the measured spread: front 2e-3 relative (5e-4 before t = 0.4 s),
  gauges dp / 2.
* Riemann / ALE-SPH dam break at dp = 0.004 (12,153 particles) to t = 0.05 s
  (1,250 steps of the as-written scheme, src/_testMUSCL_interaction.h:13-324,
  src/RALESPH_integration.h:10-107): the FP32-flux GPU path against the FP64
  oracle.  Measured: r 2.4e-8 m, v 6.9e-7 m/s (5.6e-7 of the largest |v|),
  rho 2.2e-6 kg/m^3, p 3.5e-3 Pa (8.4e-7 of the largest |p|).

The FP64 runs take about a minute in all (GB300 FP64 rate), the oracle about
20 s on 16 host cores.
"""

import os

import numpy as np
import pytest

from tinysph_old_gb300 import cases

GAUGES_X = np.array([0.3, 0.865, 1.114, 1.3625])  # constants.h: h1-h4


def _maxdiff(a, b):
    d = np.asarray(a, dtype=np.float64) - np.asarray(b, dtype=np.float64)
    if d.ndim == 2:
        d = np.linalg.norm(d, axis=1)
    return float(np.max(np.abs(d))) if d.size else 0.0


@pytest.mark.gpu
def test_fp32_against_fp64_at_benchmark_size(gpu_tsph):
    case = cases.dam_break_benchmark(0.0005)
    a = gpu_tsph.ParticleSystem.from_case(case, "fp32")
    b = gpu_tsph.ParticleSystem.from_case(case, "fp64")
    a.step(case.wall_model, case.dt, 200)
    b.step(case.wall_model, case.dt, 200)
    sa, sb = a.download(), b.download()
    assert np.array_equal(sa["index"], sb["index"])
    assert a.health() == 0 and b.health() == 0
    fl = sb["type"] == 0
    vmax = float(np.max(np.linalg.norm(sb["v"][fl], axis=1)))
    bars = {
        ("r", True): 2e-7 * case.dp,        # 1e-10 m
        ("v", True): 1e-5 * vmax,
        ("rho", True): 1e-8 * case.rho0,    # 1e-5 kg/m^3
        ("rho", False): 1e-8 * case.rho0,
        ("p", True): 4e-5 * float(np.max(np.abs(sb["p"][fl]))),
        ("p", False): 4e-5 * float(np.max(np.abs(sb["p"][~fl]))),
    }
    errs = {}
    for (f, fluid), bar in bars.items():
        m = fl if fluid else ~fl
        errs[(f, fluid)] = (_maxdiff(sa[f][m], sb[f][m]), bar)
    print({f"{f}{'' if fl_ else '_wall'}": f"{e:.3g}/{b:.3g}" for (f, fl_), (e, b) in errs.items()})
    for k, (e, bar) in errs.items():
        assert e <= bar, (k, e, bar)
    # walls do not move
    assert np.array_equal(sa["r"][~fl], sb["r"][~fl])


@pytest.mark.gpu
def test_front_and_gauges_over_half_a_second(gpu_tsph):
    case = cases.dam_break_benchmark(0.004)
    a = gpu_tsph.ParticleSystem.from_case(case, "fp32")
    b = gpu_tsph.ParticleSystem.from_case(case, "fp64")
    every = int(round(0.05 / case.dt))
    nsteps = int(round(0.5 / case.dt))
    done = 0
    fronts = []
    while done < nsteps:
        a.step(case.wall_model, case.dt, every)
        b.step(case.wall_model, case.dt, every)
        done += every
        t = done * case.dt
        fa, fb = a.water_front(0.05), b.water_front(0.05)
        wa, wb = a.water_level(GAUGES_X, 0.0), b.water_level(GAUGES_X, 0.0)
        rel = abs(fa - fb) / fb
        print(f"t {t:.2f} front {fa:.5f} {fb:.5f} rel {rel:.2e} gauges {np.round(wa, 4)} "
              f"{np.round(wb, 4)} max {np.max(np.abs(wa - wb)):.2e}")
        assert rel <= (5e-4 if t <= 0.4 + 1e-9 else 2e-3), (t, fa, fb)
        assert np.max(np.abs(wa - wb)) <= case.dp / 2, (t, wa, wb)
        fronts.append(fb)
    assert a.health() == 0 and b.health() == 0
    # the surge runs the length of the tank: the front advances until it
    # meets the far wall (x = 1.61 - dp) by t = 0.45 s
    fronts = np.array(fronts)
    assert np.all(np.diff(fronts[:8]) > 0)
    assert fronts[8] > 1.6 - 2 * case.dp


@pytest.mark.gpu
def test_ale_against_the_fp64_oracle_over_fifty_milliseconds(gpu_tsph, oracle_mod):
    case = cases.dam_break_ale(dp=0.004)
    nsteps = int(round(0.05 / case.dt))
    P = oracle_mod.PortAle.from_case(case)
    P.set_threads(os.cpu_count() or 1)
    s = gpu_tsph.AleSystem.from_case(case)
    every = nsteps // 5
    done = 0
    while done < nsteps:
        P.ale_step(case.dt, done, every)
        s.step(case.dt, done, every)
        done += every
        st, ref = s.download(), P.ale_state()
        assert np.array_equal(st["index"], ref["index"]), done
        fl = ref["type"] == 0
        bars = {
            "r": 5e-5 * case.dp,           # 2e-7 m
            "v": 1e-5 * float(np.max(np.linalg.norm(ref["v"][fl], axis=1))),
            "rho": 2e-8 * case.rho0,       # 2e-5 kg/m^3
            "p": 1e-5 * float(np.max(np.abs(ref["p"][fl]))),
        }
        errs = {f: (_maxdiff(st[f][fl], ref[f][fl]), bar) for f, bar in bars.items()}
        print(f"t {done * case.dt:.3f}", {f: f"{e:.3g}/{b:.3g}" for f, (e, b) in errs.items()})
        for f, (e, bar) in errs.items():
            assert e <= bar, (done, f, e, bar)
        assert np.array_equal(st["r"][~fl], ref["r"][~fl])
    assert s.health() & ~gpu_tsph.HEALTH_REMOVED == 0
