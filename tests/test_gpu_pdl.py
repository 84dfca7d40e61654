"""Programmatic dependent launch changes when kernels launch, never what they
compute: every engine kernel waits for its predecessor before touching
memory.  Runs with it on and off (TSPH_PDL, read when a system's engine is
created) must agree bit for bit; a kernel that read its predecessor's output
early would show up here as a difference."""

import os

import numpy as np
import pytest

from tinysph_old_gb300 import cases


def _run(gpu_tsph, case, precision, steps, pdl, variant=None):
    old = os.environ.get("TSPH_PDL")
    os.environ["TSPH_PDL"] = "1" if pdl else "0"
    try:
        s = gpu_tsph.ParticleSystem.from_case(case, precision)
        if variant is not None:
            s.set_tile_shape(variant)
        s.step(case.wall_model, case.dt, steps)
        return s.download()
    finally:
        if old is None:
            os.environ.pop("TSPH_PDL", None)
        else:
            os.environ["TSPH_PDL"] = old


@pytest.mark.gpu
@pytest.mark.parametrize("precision,variant", [("fp32", 0), ("fp32", 2), ("fp64", None)])
@pytest.mark.parametrize("builder,steps", [
    (lambda: cases.dam_break_mdbc(dp=0.005), 300),
    (lambda: cases.still_water_dbc(dp=0.01), 300),
    (lambda: cases.outlet_channel_mdbc(dp=0.005), 300),
])
def test_pdl_on_and_off_agree_bit_for_bit(gpu_tsph, builder, steps, precision, variant):
    a = _run(gpu_tsph, builder(), precision, steps, True, variant)
    b = _run(gpu_tsph, builder(), precision, steps, False, variant)
    for f in ("r", "v", "rho", "p", "type"):
        assert np.array_equal(a[f], b[f]), f
