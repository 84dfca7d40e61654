"""VTK output (the reference's write_to_ASCII_VTK layout) and checkpoint /
restart of a system."""

import numpy as np
import pytest

from tinysph_old_gb300 import cases


def test_load_rejects_a_file_that_is_not_a_checkpoint(tsph, tmp_path):
    p = tmp_path / "junk.bin"
    p.write_bytes(b"not a checkpoint at all")
    with pytest.raises(tsph.TsphError) as e:
        tsph.ParticleSystem.load_checkpoint(str(p))
    assert e.value.status == tsph.ERR_ARG


@pytest.mark.gpu
def test_vtk_has_the_reference_layout(gpu_tsph, tmp_path):
    case = cases.dam_break_mdbc(dp=0.02)
    s = gpu_tsph.ParticleSystem.from_case(case)
    s.step(0, case.dt, 5)
    st = s.download()
    p = tmp_path / "out.vtk"
    s.write_vtk(str(p))
    lines = p.read_text().splitlines()
    n = s.np
    assert lines[:5] == ["# vtk DataFile Version 3.0", "vtk output", "ASCII", "DATASET POLYDATA",
                         f"POINTS {n} float"]
    pts = np.array([[float(t) for t in ln.split()] for ln in lines[5:5 + n]])
    assert np.allclose(pts[:, :2], st["r"], rtol=1e-5, atol=1e-6) and np.all(pts[:, 2] == 0)
    k = 5 + n
    assert lines[k:k + 3] == [f"POINT_DATA {n}", "FIELDS FieldData 4", f"type 1 {n} int"]
    assert np.array_equal(np.array([int(t) for t in lines[k + 3:k + 3 + n]]), st["type"])
    k += 3 + n
    assert lines[k] == f"pressure 1 {n} float"
    assert np.allclose([float(t) for t in lines[k + 1:k + 1 + n]], st["p"], rtol=1e-5, atol=1e-3)
    k += 1 + n
    assert lines[k] == f"density 1 {n} float"
    assert np.allclose([float(t) for t in lines[k + 1:k + 1 + n]], st["rho"], rtol=1e-5)
    k += 1 + n
    assert lines[k] == f"velocity 3 {n} float"
    vel = np.array([[float(t) for t in ln.split()] for ln in lines[k + 1:k + 1 + n]])
    assert np.allclose(vel[:, :2], st["v"], rtol=1e-5, atol=1e-6)
    assert len(lines) == k + 1 + n


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_checkpoint_restart_continues_bit_for_bit(gpu_tsph, tmp_path, precision):
    case = cases.dam_break_mdbc(dp=0.02)
    a = gpu_tsph.ParticleSystem.from_case(case, precision)
    a.step(0, case.dt, 10)
    p = tmp_path / "run.ckp"
    a.save_checkpoint(str(p))
    a.step(0, case.dt, 10)
    b = gpu_tsph.ParticleSystem.load_checkpoint(str(p))
    b.step(0, case.dt, 10)
    x, y = a.download(), b.download()
    for f in ("r", "v", "a", "rho", "drho", "p", "type"):
        assert np.array_equal(x[f], y[f]), f


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_checkpoint_of_a_system_with_buffer_zones(gpu_tsph, tmp_path, precision):
    """The outlet channel saved after its outlet has retyped and erased
    particles (indices past the initial ones, gaps left by erasures): the
    restarted system keeps the zones and continues bit for bit, appends and
    erasures included."""
    case = cases.outlet_channel_mdbc(dp=0.005)
    a = gpu_tsph.ParticleSystem.from_case(case, precision)
    a.step(case.wall_model, case.dt, 450)
    n_saved = a.np
    p = tmp_path / "zones.ckp"
    a.save_checkpoint(str(p))
    a.step(case.wall_model, case.dt, 150)
    b = gpu_tsph.ParticleSystem.load_checkpoint(str(p))
    assert b.np == n_saved
    b.step(case.wall_model, case.dt, 150)
    x, y = a.download(), b.download()
    assert len(x["type"]) == len(y["type"]) and len(x["type"]) < n_saved
    for f in ("r", "v", "a", "rho", "drho", "p", "type"):
        assert np.array_equal(x[f], y[f]), f
