"""tsph_download_async / tsph_download_wait: a pipelined loop (upload a
state, re-bin, step, start the result's download, wait for it one step
later) leaves in the host buffers exactly what tsph_download returns, in
both precisions; a state with erased particles falls back to the
synchronous download; other fields are refused."""

import numpy as np
import pytest

from tinysph_old_gb300 import cases


def _buffers(n, torch):
    return tuple(torch.empty(shape, dtype=torch.float64, pin_memory=True)
                 for shape in ((n, 2), (n, 2), (n,)))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_pipelined_download_matches_the_synchronous_one(gpu_tsph, precision):
    torch = pytest.importorskip("torch")
    case = cases.dam_break_mdbc(dp=0.01)
    s = gpu_tsph.ParticleSystem.from_case(case, precision)
    n = s.np
    mask = gpu_tsph.F_R | gpu_tsph.F_V | gpu_tsph.F_RHO
    inp = _buffers(n, torch)
    s.download_ptrs(mask, r=inp[0].data_ptr(), v=inp[1].data_ptr(), rho=inp[2].data_ptr())
    outs = [_buffers(n, torch) for _ in range(2)]
    expect = []
    for k in range(4):
        s.upload_ptrs(mask, r=inp[0].data_ptr(), v=inp[1].data_ptr(), rho=inp[2].data_ptr())
        s.particle_to_cell()
        s.step(case.wall_model, case.dt, 3 + k)  # a different result every call
        o = outs[k % 2]
        s.download_async(mask, r=o[0].data_ptr(), v=o[1].data_ptr(), rho=o[2].data_ptr())
        if k > 0:
            # the previous result, complete once the next download has started
            prev = outs[(k - 1) % 2]
            want = expect[-1]
            assert np.array_equal(prev[0].numpy(), want["r"])
            assert np.array_equal(prev[1].numpy(), want["v"])
            assert np.array_equal(prev[2].numpy(), want["rho"])
        s.download_wait()
        expect.append(s.download())
        # a second wait is a no-op
        s.download_wait()
    last = outs[3 % 2]
    assert np.array_equal(last[0].numpy(), expect[-1]["r"])
    assert np.array_equal(last[2].numpy(), expect[-1]["rho"])


@pytest.mark.gpu
def test_download_async_with_erased_particles_and_bad_fields(gpu_tsph):
    case = cases.dam_break_mdbc(dp=0.02)
    s = gpu_tsph.ParticleSystem.from_case(case, "fp32")
    st = s.download()
    r = st["r"].copy()
    fl = np.flatnonzero(st["type"] == 0)
    r[fl[5]] = (0.5, case.domain[3] + 0.5)  # leaves the domain
    s.upload(r=r)
    assert s.remove_out_of_domain() == 1
    s.particle_to_cell()
    n = s.np
    assert n == case.np - 1
    out_r = np.zeros((n, 2))
    out_p = np.zeros(n)
    s.download_async(gpu_tsph.F_R | gpu_tsph.F_P, r=out_r.ctypes.data, p=out_p.ctypes.data)
    s.download_wait()
    want = s.download()
    assert np.array_equal(out_r, want["r"]) and np.array_equal(out_p, want["p"])
    with pytest.raises(gpu_tsph.TsphError):
        s.download_async(gpu_tsph.F_INDEX, index=np.zeros(n, dtype=np.int32).ctypes.data)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_staged_upload_matches_the_synchronous_one(gpu_tsph, precision):
    """tsph_upload_async + tsph_particle_to_cell leaves the state that
    tsph_upload + tsph_particle_to_cell leaves (FP64 bit for bit, FP32 to
    rounding), also when the upload is staged while a step is in flight and
    the previous result is still being read back; between staging and
    binning only downloads of the asynchronous kind are accepted."""
    torch = pytest.importorskip("torch")
    case = cases.dam_break_mdbc(dp=0.01)
    a = gpu_tsph.ParticleSystem.from_case(case, precision)
    b = gpu_tsph.ParticleSystem.from_case(case, precision)
    if precision == "fp32":
        a.set_tile_shape(2)
        b.set_tile_shape(2)
    n = a.np
    # a step's whole input: positions, velocities, densities and the rates of
    # the last forces pass (the predictor's a, drho)
    mask = gpu_tsph.F_R | gpu_tsph.F_V | gpu_tsph.F_A | gpu_tsph.F_RHO | gpu_tsph.F_DRHO
    a.step(case.wall_model, case.dt, 5)
    inp = _buffers(n, torch) + tuple(torch.empty(sh, dtype=torch.float64, pin_memory=True)
                                     for sh in ((n, 2), (n,)))
    ptrs = dict(r=inp[0].data_ptr(), v=inp[1].data_ptr(), rho=inp[2].data_ptr(),
                a=inp[3].data_ptr(), drho=inp[4].data_ptr())
    a.download_ptrs(mask, **ptrs)
    # reference: synchronous upload of the same state, then the same steps
    b.upload_ptrs(mask, **ptrs)
    b.particle_to_cell()
    b.step(case.wall_model, case.dt, 3)
    want = b.download()
    # pipelined: stage the upload while a's steps run, read a's result back
    outs = [_buffers(n, torch) for _ in range(2)]
    a.step(case.wall_model, case.dt, 2)
    a.upload_async(mask, **ptrs)
    o = outs[0]
    m3 = gpu_tsph.F_R | gpu_tsph.F_V | gpu_tsph.F_RHO
    a.download_async(m3, r=o[0].data_ptr(), v=o[1].data_ptr(), rho=o[2].data_ptr())
    with pytest.raises(gpu_tsph.TsphError):
        a.download()
    with pytest.raises(gpu_tsph.TsphError):
        a.upload_ptrs(mask, **ptrs)
    with pytest.raises(gpu_tsph.TsphError):
        a.step(case.wall_model, case.dt, 1)
    a.download_wait()
    a.particle_to_cell()
    a.step(case.wall_model, case.dt, 3)
    got = a.download()
    assert a.health() == 0
    for f in ("r", "v", "rho", "p", "a"):
        if precision == "fp64":
            assert np.array_equal(got[f], want[f]), f
        else:
            # the FP32 pair-record step keeps a's cells (every particle within
            # sigma of where a binned it) while b bins afresh: the pair sums
            # run in another order, equal to FP32 rounding
            d = float(np.max(np.abs(got[f] - want[f])))
            assert d <= 1e-5 * max(1.0, float(np.max(np.abs(want[f])))), (f, d)


@pytest.mark.gpu
def test_staged_upload_with_erased_particles_is_dropped(gpu_tsph):
    case = cases.dam_break_mdbc(dp=0.02)
    s = gpu_tsph.ParticleSystem.from_case(case, "fp32")
    st = s.download()
    r = st["r"].copy()
    r[np.flatnonzero(st["type"] == 0)[3]] = (0.5, case.domain[3] + 0.5)
    s.upload(r=r)
    assert s.remove_out_of_domain() == 1
    s.particle_to_cell()
    before = s.download()
    n = s.np
    r2 = np.ascontiguousarray(before["r"] + 1e-4)
    s.upload_async(gpu_tsph.F_R, r=r2.ctypes.data)
    s.particle_to_cell()
    assert s.health() & gpu_tsph.HEALTH_UPLOAD
    after = s.download()
    assert np.array_equal(after["r"], before["r"]) and n == s.np


@pytest.mark.gpu
def test_binning_after_an_upload_keeps_cells_within_sigma(gpu_tsph):
    """On the FP32 pair-record step, Particle_To_Cell after an upload keeps
    the cells and lists when every particle is within sigma of where it was
    binned: uploading a system's own state changes nothing (the next steps
    are bit for bit those of the system left alone).  A particle moved
    further re-bins the state (gated on the device's check): the exact cell
    lists then equal a fresh system's, and stepping goes on healthily."""
    case = cases.dam_break_mdbc(dp=0.01)
    a = gpu_tsph.ParticleSystem.from_case(case, "fp32")
    b = gpu_tsph.ParticleSystem.from_case(case, "fp32")
    for s in (a, b):
        s.set_tile_shape(2)
        s.step(case.wall_model, case.dt, 6)
    mask = gpu_tsph.F_R | gpu_tsph.F_V | gpu_tsph.F_A | gpu_tsph.F_RHO | gpu_tsph.F_DRHO
    st = a.download()
    bufs = {k: np.ascontiguousarray(st[k]) for k in ("r", "v", "a", "rho", "drho")}
    a.upload_async(mask, **{k: v.ctypes.data for k, v in bufs.items()})
    a.particle_to_cell()
    a.step(case.wall_model, case.dt, 4)
    b.step(case.wall_model, case.dt, 4)
    ga, gb = a.download(), b.download()
    for f in ("r", "v", "a", "rho", "drho", "p"):
        assert np.array_equal(ga[f], gb[f]), f
    # one fluid particle moved half a spacing: re-binned
    r = ga["r"].copy()
    k = int(np.flatnonzero(ga["type"] == 0)[17])
    r[k, 0] += 0.5 * case.dp
    r = np.ascontiguousarray(r)
    a.upload_async(gpu_tsph.F_R, r=r.ctypes.data)
    a.particle_to_cell()
    c = gpu_tsph.ParticleSystem.from_case(case, "fp32")
    c.upload(r=r)
    c.particle_to_cell()
    sa, la = a.get_cells()
    sc, lc = c.get_cells()
    assert np.array_equal(sa, sc) and np.array_equal(la, lc)
    a.step(case.wall_model, case.dt, 3)
    assert a.health() == 0
