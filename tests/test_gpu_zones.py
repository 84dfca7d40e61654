"""Open boundaries on the GPU through the C ABI against the reference's own
runs (tests/golden/inflow_slab_mdbc_dp0.005.npz: cases/inflowSlab_mDBC, the
inlet creating particles; outlet_channel_mdbc_dp0.005.npz: the outlet's
retyping and its erasures, including the reference's skip of the particle
after an erased one).  Particle count, order and types exact; fields within
1e-9 of their scale (FP64 build: CUDA's pow against glibc's in the last
bits, grown quadratically with the step count as the flow through the
outlet amplifies them: 1.5e-7 relative after 600 steps) or the FP32 bars of
the WCSPH parity tests grown with the step count."""

import os

import numpy as np
import pytest

from tinysph_old_gb300 import cases

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _tol(precision, field, ref, steps):
    mag = float(np.max(np.abs(ref))) if np.size(ref) else 0.0
    if precision == "fp64":
        return 1e-9 * max(1.0, mag) * (1 + (steps / 50) ** 2)
    base = {"r": 1e-9, "v": 2e-6 + 1e-5 * mag, "rho": 2e-4, "p": 5e-2 + 1e-6 * mag}[field]
    return base * (1 + steps / 10)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("fname,builder", [
    ("inflow_slab_mdbc_dp0.005.npz", lambda: cases.inflow_slab_mdbc(dp=0.005)),
    ("outlet_channel_mdbc_dp0.005.npz", lambda: cases.outlet_channel_mdbc(dp=0.005)),
])
def test_zones_match_the_reference(gpu_tsph, fname, builder, precision):
    g = np.load(os.path.join(GOLD, fname))
    case = builder()
    s = gpu_tsph.ParticleSystem.from_case(case, precision)
    done = 0
    for n in g["snaps"]:
        s.step(case.wall_model, float(g["dt"]), int(n) - done)
        done = int(n)
        st = s.download()
        ref_type = g[f"step{n}_type"]
        assert len(st["type"]) == len(ref_type), (n, len(st["type"]), len(ref_type))
        assert np.array_equal(st["type"], ref_type), n
        for f in ("r", "v", "rho", "p"):
            ref = g[f"step{n}_{f}"]
            e = float(np.max(np.abs(st[f] - ref)))
            lim = _tol(precision, f, ref, int(n))
            assert e <= lim, (n, f, e, lim)
