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
equality, as for every cell-list test.
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


@pytest.mark.gpu
def test_noalloc_binning_matches_particle_to_cell(gpu_tsph):
    torch = pytest.importorskip("torch")
    L = gpu_tsph.load()
    for call, (dp, seed) in enumerate(((0.01, 5), (0.02, 6))):
        case, r = _perturbed_case(dp, seed)
        # the regular path
        s = gpu_tsph.ParticleSystem.from_case(case, "fp32")
        s.upload(r=r)
        s.particle_to_cell()
        start_ref, list_ref = s.get_cells()
        ncx, ncy = s.grid()
        # the caller's own device buffers
        r_dev = torch.from_numpy(np.ascontiguousarray(r)).to("cuda")
        start_dev = torch.full((ncx * ncy + 1,), -7, dtype=torch.int32, device="cuda")
        list_dev = torch.full((len(r),), -7, dtype=torch.int32, device="cuda")
        c = gpu_tsph._Constants(case.h, case.kap, case.cs, case.rho0, case.visco, case.delta,
                                case.dp)
        d = gpu_tsph._Domain(*case.domain)
        nb = C.c_int(-1)
        torch.cuda.synchronize()
        rc = L.tsph_particle_to_cell_noalloc(C.byref(c), C.byref(d), len(r), r_dev.data_ptr(),
                                             start_dev.data_ptr(), list_dev.data_ptr(), None,
                                             C.byref(nb))
        assert rc == 0, (call, L.tsph_last_error())
        assert nb.value == len(r)
        assert np.array_equal(start_dev.cpu().numpy(), start_ref), call
        assert np.array_equal(list_dev.cpu().numpy(), list_ref), call
        s.close()


@pytest.mark.gpu
def test_noalloc_binning_rejects_sizes_beyond_its_scratch(gpu_tsph):
    L = gpu_tsph.load()
    case = cases.dam_break_mdbc(dp=0.02)
    c = gpu_tsph._Constants(case.h, case.kap, case.cs, case.rho0, case.visco, case.delta, case.dp)
    d = gpu_tsph._Domain(*case.domain)
    rc = L.tsph_particle_to_cell_noalloc(C.byref(c), C.byref(d), (1 << 20) + 1, 8, 8, 8, None,
                                         None)
    assert rc == gpu_tsph.ERR_ARG
    assert b"max" in L.tsph_last_error()
    big = gpu_tsph._Domain(0.0, 100.0, 0.0, 100.0)  # far more cells than the scratch holds
    rc = L.tsph_particle_to_cell_noalloc(C.byref(c), C.byref(big), 10, 8, 8, 8, None, None)
    assert rc == gpu_tsph.ERR_ARG
