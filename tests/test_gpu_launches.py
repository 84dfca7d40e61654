"""tsph_kernel_launches: the kernels a system launched.  A graph step counts
its kernels, so the count grows by the same amount per step (the conditional
re-binning and sort stay off at these speeds: four kernels per FP32 mDBC step
over pair records with kept lists, mDBC + predictor, two pair passes and the
wall rows, more with the tiled kernels); the equation of state that brings
the stored pressure up to date runs once, at the first call that reads the
state after the steps; reset clears it."""

import pytest

from tinysph_old_gb300 import cases


@pytest.mark.gpu
def test_kernel_launch_count_per_graph_step(gpu_tsph):
    case = cases.dam_break_mdbc(dp=0.01)
    s = gpu_tsph.ParticleSystem.from_case(case)
    s.step(case.wall_model, case.dt, 2)  # captures the graph
    s.kernel_launches(reset=True)
    s.step(case.wall_model, case.dt, 5)
    c5 = s.kernel_launches(reset=True)
    s.step(case.wall_model, case.dt, 15)
    c15 = s.kernel_launches(reset=True)
    per_step = (c15 - c5) / 10
    assert per_step == int(per_step) and 4 <= per_step <= 12, (c5, c15)
    assert c5 == 5 * per_step  # no equation of state between the steps
    assert s.kernel_launches() == 0
    # a download after steps runs the equation of state once before its own
    # kernels; a second download finds the pressure up to date
    s.download()
    stale = s.kernel_launches(reset=True)
    s.download()
    fresh = s.kernel_launches(reset=True)
    assert stale == fresh + 1, (stale, fresh)
    # a download that does not ask for the pressure leaves it stale: the
    # full download after it still runs the equation of state
    s.step(case.wall_model, case.dt, 1)
    s.kernel_launches(reset=True)
    s.download(gpu_tsph.F_R | gpu_tsph.F_V | gpu_tsph.F_RHO)
    no_p = s.kernel_launches(reset=True)
    s.download()
    with_p = s.kernel_launches(reset=True)
    assert with_p == fresh + 1 and no_p < with_p, (no_p, with_p, fresh)
