"""The allocation-free binning entry point, tsph_particle_to_cell_noalloc.

It serves callers that cannot allocate device memory: a host framework that
binds this library through its FFI and owns every device buffer in its own
pool, or a time loop that must not call cudaMalloc/cudaFree because they
synchronise the device.  The caller passes its positions and output buffers;
the counting sort's working memory is a static array inside the library.
These tests call it through the C ABI twice in a row (a larger case, then a
smaller one, so stale contents of the shared array would show) and compare
its cell lists with the ones the regular entry point, tsph_particle_to_cell,
returns for the same positions.  Cell lists are integers: the bar is exact
equality, as for every cell-list test.  Further cases: particles outside the
grid (left out of the lists, TSPH_ERR_ESCAPED), a call on a non-default
stream, positions at an 8-byte (not 16-byte) aligned address, misaligned
pointers refused, and device memory unchanged across a call.
"""

import ctypes as C

import numpy as np
import pytest

from tinysph_old_gb300 import cases


def _perturbed_case(dp, seed):
    case = cases.dam_break_mdbc(dp=dp)
    a = case.particles.arrays()
    r = a["r"].copy()
    fl = a["type"] == 0
    rng = np.random.default_rng(seed)
    r[fl] += rng.uniform(-0.3 * dp, 0.3 * dp, size=(int(fl.sum()), 2))
    return case, r


def _reference_lists(tsph, case, r):
    s = tsph.ParticleSystem.from_case(case, "fp32")
    try:
        s.upload(r=r)
        s.particle_to_cell()
        start_ref, list_ref = s.get_cells()
        ncx, ncy = s.grid()
    finally:
        s.close()
    return start_ref, list_ref, ncx * ncy


def _args(tsph, case):
    c = tsph._Constants(case.h, case.kap, case.cs, case.rho0, case.visco, case.delta, case.dp)
    d = tsph._Domain(*case.domain)
    return c, d


def _call(L, c, d, n, r_ptr, start_dev, list_dev, stream=None):
    nb = C.c_int(-1)
    rc = L.tsph_particle_to_cell_noalloc(C.byref(c), C.byref(d), n, r_ptr, start_dev.data_ptr(),
                                         list_dev.data_ptr(), stream, C.byref(nb))
    return rc, nb.value


@pytest.mark.gpu
def test_noalloc_binning_matches_particle_to_cell(gpu_tsph):
    torch = pytest.importorskip("torch")
    L = gpu_tsph.load()
    for call, (dp, seed) in enumerate(((0.01, 5), (0.02, 6))):
        case, r = _perturbed_case(dp, seed)
        start_ref, list_ref, ncells = _reference_lists(gpu_tsph, case, r)
        # the caller's own device buffers
        r_dev = torch.from_numpy(np.ascontiguousarray(r)).to("cuda")
        start_dev = torch.full((ncells + 1,), -7, dtype=torch.int32, device="cuda")
        list_dev = torch.full((len(r),), -7, dtype=torch.int32, device="cuda")
        c, d = _args(gpu_tsph, case)
        torch.cuda.synchronize()
        rc, nb = _call(L, c, d, len(r), r_dev.data_ptr(), start_dev, list_dev)
        assert rc == 0, (call, L.tsph_last_error())
        assert nb == len(r)
        assert np.array_equal(start_dev.cpu().numpy(), start_ref), call
        assert np.array_equal(list_dev.cpu().numpy(), list_ref), call


@pytest.mark.gpu
def test_noalloc_binning_escaped_stream_alignment_and_memory(gpu_tsph):
    torch = pytest.importorskip("torch")
    L = gpu_tsph.load()
    case, r = _perturbed_case(0.01, 11)
    start_ref, list_ref, ncells = _reference_lists(gpu_tsph, case, r)
    c, d = _args(gpu_tsph, case)
    n = len(r)

    # positions at an address that is 8- but not 16-byte aligned: one double
    # of padding in front of the caller's array
    padded = torch.zeros(2 * n + 1, dtype=torch.float64, device="cuda")
    padded[1:] = torch.from_numpy(np.ascontiguousarray(r).reshape(-1)).to("cuda")
    r_ptr = padded.data_ptr() + 8
    assert r_ptr % 16 == 8
    start_dev = torch.full((ncells + 1,), -7, dtype=torch.int32, device="cuda")
    list_dev = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    rc, nb = _call(L, c, d, n, r_ptr, start_dev, list_dev, C.c_void_p(stream.cuda_stream))
    assert rc == 0, L.tsph_last_error()
    assert nb == n
    assert np.array_equal(start_dev.cpu().numpy(), start_ref)
    assert np.array_equal(list_dev.cpu().numpy(), list_ref)

    # no device allocation: free device memory and torch's allocator are
    # unchanged across a second call
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    alloc0 = torch.cuda.memory_allocated()
    rc, nb = _call(L, c, d, n, r_ptr, start_dev, list_dev, C.c_void_p(stream.cuda_stream))
    assert rc == 0, L.tsph_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_allocated() == alloc0

    # a few fluid particles moved outside the grid: they are left out, the
    # other lists are those of the regular path without them
    fl = np.flatnonzero(case.particles.arrays()["type"] == 0)
    gone = fl[[3, 400, 401, len(fl) - 1]]
    r2 = r.copy()
    r2[gone, 1] = case.domain[3] + 50.0
    padded[1:] = torch.from_numpy(np.ascontiguousarray(r2).reshape(-1)).to("cuda")
    start_dev.fill_(-7)
    list_dev.fill_(-7)
    rc, nb = _call(L, c, d, n, r_ptr, start_dev, list_dev, C.c_void_p(stream.cuda_stream))
    assert rc == gpu_tsph.ERR_ESCAPED, L.tsph_last_error()
    assert nb == n - len(gone)
    keep = ~np.isin(list_ref, gone)
    want_list = list_ref[keep]
    cell_of = np.repeat(np.arange(ncells), np.diff(start_ref))
    want_start = np.zeros(ncells + 1, dtype=np.int64)
    np.add.at(want_start, cell_of[keep] + 1, 1)
    want_start = np.cumsum(want_start)
    assert np.array_equal(start_dev.cpu().numpy(), want_start)
    assert np.array_equal(list_dev.cpu().numpy()[:nb], want_list)

    # misaligned pointers are refused before anything is queued
    rc, _ = _call(L, c, d, n, padded.data_ptr() + 4, start_dev, list_dev)
    assert rc == gpu_tsph.ERR_ARG
    assert b"misaligned" in L.tsph_last_error()


@pytest.mark.gpu
def test_noalloc_binning_rejects_sizes_beyond_its_scratch(gpu_tsph):
    L = gpu_tsph.load()
    case = cases.dam_break_mdbc(dp=0.02)
    c, d = _args(gpu_tsph, case)
    rc = L.tsph_particle_to_cell_noalloc(C.byref(c), C.byref(d), (1 << 20) + 1, 8, 8, 8, None,
                                         None)
    assert rc == gpu_tsph.ERR_ARG
    assert b"max" in L.tsph_last_error()
    big = gpu_tsph._Domain(0.0, 100.0, 0.0, 100.0)  # far more cells than the scratch holds
    rc = L.tsph_particle_to_cell_noalloc(C.byref(c), C.byref(big), 10, 8, 8, 8, None, None)
    assert rc == gpu_tsph.ERR_ARG
