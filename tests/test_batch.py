"""Batched cases: the vectorised generators, the seeded batch, the packing of
every case into one particle system (scaled to the system's particle spacing,
with a column range, a gravity and a removal box per case), and (GPU)
per-case results of the packed batch against the oracle run on each case in
its own units, including erasures at a case's own removal box."""

import numpy as np
import pytest

from tinysph_old_gb300 import batch as B
from tinysph_old_gb300 import cases


@pytest.mark.parametrize("spec", [
    B.CaseSpec(B.DAM_BREAK, 0.004, 1.3, 0.55, 0.37),
    B.CaseSpec(B.DAM_BREAK, 0.003, 2.0, 0.8, 0.5),
    B.CaseSpec(B.STILL_WATER, 0.004, 1.3, 0.55, 0.37),
    B.CaseSpec(B.STILL_WATER, 0.002, 1.9, 0.79, 0.49),
])
def test_vectorised_generators_match_the_reference_order(spec):
    a = B.case_arrays(spec)
    if spec.kind == B.DAM_BREAK:
        c = cases.dam_break_mdbc(dp=spec.dp, cs=35.0, wall_height=0.8, tank_length=spec.tank,
                                 column=(spec.col_w, spec.col_h))
    else:
        c = cases.still_water_tank_mdbc(dp=spec.dp, width=spec.col_w, depth=spec.col_h,
                                        wall_height=spec.col_h + 0.1)
    ca = c.particles.arrays()
    assert a.np == c.np
    for k in ("r", "type", "rho", "p"):
        assert np.array_equal(getattr(a, k), ca[k]), k
    assert np.array_equal(a.gnr[:len(ca["gnr"])], ca["gnr"])
    assert (a.h, a.kap, a.cs, a.dt, a.wall_model) == (c.h, c.kap, c.cs, c.dt, c.wall_model)
    if spec.kind == B.STILL_WATER:  # (a dam break's domain grows with its tank: x_1 = max(2, L + 0.1))
        assert a.domain == c.domain


def test_seeded_batch_spans_the_stated_sizes():
    specs = B.sample_specs(512, seed=0)
    n = np.array([B.case_arrays(s).np for s in specs])
    assert len(specs) == 512
    assert n.min() >= 2000 and n.max() <= 100_000
    assert {s.dp for s in specs} == {0.004, 0.003, 0.002}
    assert {s.kind for s in specs} == {B.DAM_BREAK, B.STILL_WATER}
    assert specs == B.sample_specs(512, seed=0)  # deterministic


def test_scaled_packing_keeps_cases_apart():
    specs = B.sample_specs(64, seed=3)
    cs = [B.case_arrays(s) for s in specs]
    pk = B.pack_scaled(cs)
    kh = pk.h * 2.1
    # column ranges in order, CASE_GAP_CELLS cells apart
    assert np.all(pk.ranges[1:, 0] - pk.ranges[:-1, 1] >= B.CASE_GAP_CELLS * kh * (1 - 1e-12))
    for k, c in enumerate(cs):
        lam = pk.scale[k]
        # the system's spacing, h and step for every scaled case; gravity g / lambda
        assert np.isclose(c.spec.dp * lam, pk.dp) and np.isclose(c.h * lam, pk.h)
        assert np.isclose(c.dt * lam, pk.dt) and np.isclose(pk.gravity[k], 9.81 / lam)
        r = c.r * lam + np.array([pk.offset[k], 0.0])
        assert pk.ranges[k, 0] <= r[:, 0].min() and r[:, 0].max() < pk.ranges[k, 1]
        # the removal box lies inside the case's columns: a fluid particle
        # leaves them only by being erased, so no pair spans two cases
        x_lo, x_hi, y_lo, y_hi = pk.boxes[k]
        assert pk.ranges[k, 0] < x_lo and x_hi < pk.ranges[k, 1]
        fl = c.type == B.FLUID
        assert np.all((r[fl, 0] >= x_lo) & (r[fl, 0] <= x_hi))
        assert np.all((r[fl, 1] >= y_lo) & (r[fl, 1] <= y_hi))
        assert y_lo >= pk.domain[2] and y_hi <= pk.domain[3]


def _oracle_case(oracle_mod, a):
    P = oracle_mod.PortSystem(a.h, a.kap, a.cs, 1000.0, 0.02, 0.1, a.spec.dp, a.domain)
    for i in range(a.np):
        P.L.orc_add_particle(P.s, int(a.type[i]), float(a.p[i]), float(a.rho[i]),
                             float(a.r[i, 0]), float(a.r[i, 1]), 0.0, 0.0, 0.0, 0.0)
    for i in np.nonzero(a.type == B.WALL)[0]:  # walls come first
        P.L.orc_add_gnr(P.s, float(a.gnr[i, 0]), float(a.gnr[i, 1]))
    P.divide_to_cells()
    P.particle_to_cell()
    return P


@pytest.mark.gpu
def test_batch_in_one_system_matches_the_oracle_per_case(gpu_tsph, oracle_mod):
    """Five cases of three spacings in one system (one launch per kernel per
    step) against the oracle run on each case alone in its own units.  Two
    consecutive fluid particles of the still-water case start beyond its
    removal threshold x > x_m - 0.01 (inside its columns and the system's
    grid): the first step erases the first and, as the reference's erase loop
    does, skips the second, which goes one step later."""
    import os

    oracle_mod.PortSystem.set_threads(os.cpu_count() or 1)
    # a shallow tank (15 particles per column) before a second case: chunks of
    # 128 targets there span more columns than the window table holds, and
    # the last window (global path) crosses into the next case
    specs = [B.CaseSpec(B.DAM_BREAK, 0.004, 1.0, 0.4, 0.3),
             B.CaseSpec(B.STILL_WATER, 0.003, 1.0, 0.5, 0.25),
             B.CaseSpec(B.STILL_WATER, 0.004, 1.0, 0.5, 0.06),
             B.CaseSpec(B.DAM_BREAK, 0.002, 0.9, 0.25, 0.2),
             B.CaseSpec(B.STILL_WATER, 0.004, 1.0, 0.4, 0.2)]
    arrays = [B.case_arrays(s) for s in specs]
    sw = arrays[1]
    fl = np.nonzero(sw.type == B.FLUID)[0]
    out = fl[40:42]
    xm = sw.domain[1]
    sw.r[out[0]] = (xm - 0.005, 0.05)
    sw.r[out[1]] = (xm - 0.004, 0.06)
    bt = B.Batch(specs, arrays=arrays)
    assert bt.system.tile_shape == 2
    refs = [_oracle_case(oracle_mod, a) for a in arrays]
    done = 0
    for nsteps in (1, 1, 98):
        bt.step(nsteps)
        for P, a in zip(refs, arrays):
            P.step(a.wall_model, a.dt, nsteps)
        done += nsteps
        st = bt.system.download()
        for k, (P, a) in enumerate(zip(refs, arrays)):
            got, ref = bt.case_state(k, st), P.state()
            assert np.array_equal(got["index"], ref["index"]), (done, k)
            f = ref["type"] == B.FLUID
            er = float(np.max(np.abs(got["r"][f] - ref["r"][f])))
            ev = float(np.max(np.abs(got["v"][f] - ref["v"][f])))
            erho = float(np.max(np.abs(got["rho"] - ref["rho"])))
            print(done, k, specs[k].kind, specs[k].dp, er, ev, erho)
            assert er <= 1e-7 and ev <= 1e-4 and erho <= 1e-3, (done, k, er, ev, erho)
            # walls do not move (equal up to the rounding of the scaling)
            assert np.max(np.abs(got["r"][~f] - ref["r"][~f])) <= 1e-12
        if done == 1:  # the first erased, the second skipped
            ids = bt.case_state(1, st)["index"]
            assert out[0] not in ids and out[1] in ids
    ids = bt.case_state(1, st)["index"]
    assert out[0] not in ids and out[1] not in ids
    assert bt.system.np == sum(a.np for a in arrays) - 2


@pytest.mark.gpu
def test_batch_pipelined_transfers_equal_synchronous(gpu_tsph):
    """The case-table system through the pipelined transfers (the staged
    upload applied by particle_to_cell, the step, the download read back a
    step later) gives bit for bit the synchronous loop's results."""
    torch = pytest.importorskip("torch")
    specs = [B.CaseSpec(B.DAM_BREAK, 0.004, 1.0, 0.4, 0.3),
             B.CaseSpec(B.STILL_WATER, 0.002, 1.0, 0.4, 0.2)]
    a, b = B.Batch(specs), B.Batch(specs)
    a.step(3)
    b.step(3)
    sa, sb = a.system, b.system
    n = sa.np
    mask = gpu_tsph.F_R | gpu_tsph.F_V | gpu_tsph.F_RHO
    hin = [torch.empty(shape, dtype=torch.float64, pin_memory=True)
           for shape in ((n, 2), (n, 2), (n,))]
    ptr = dict(r=hin[0].data_ptr(), v=hin[1].data_ptr(), rho=hin[2].data_ptr())
    sa.download_ptrs(mask, **ptr)
    sync = []
    for _ in range(3):
        sa.upload_ptrs(mask, **ptr)
        sa.particle_to_cell()
        a.step(1)
        sync.append(sa.download(mask))
    outs = [[torch.empty_like(t, pin_memory=True) for t in hin] for _ in range(3)]
    sb.upload_async(mask, **ptr)
    for k in range(3):
        if k:
            sb.upload_async(mask, **ptr)
        sb.particle_to_cell()
        b.step(1)
        o = outs[k]
        sb.download_async(mask, r=o[0].data_ptr(), v=o[1].data_ptr(), rho=o[2].data_ptr())
    sb.download_wait()
    for k in range(3):
        o = [t.numpy() for t in outs[k]]
        assert np.array_equal(o[0], sync[k]["r"]), k
        assert np.array_equal(o[1], sync[k]["v"]), k
        assert np.array_equal(o[2], sync[k]["rho"]), k


@pytest.mark.gpu
def test_case_table_rules(gpu_tsph, tmp_path):
    """tsph_set_cases: FP32 only, non-empty ranges; on a system with a case
    table the per-function force, corrector and removal calls and checkpoints
    are refused (they would apply the system's gravity and box)."""
    specs = [B.CaseSpec(B.DAM_BREAK, 0.004, 1.0, 0.4, 0.3),
             B.CaseSpec(B.STILL_WATER, 0.002, 1.0, 0.4, 0.2)]
    bt = B.Batch(specs)
    s = bt.system
    E = gpu_tsph.TsphError
    for call in (lambda: s.compute_forces(gpu_tsph.WALL_MDBC), lambda: s.corrector(bt.dt),
                 lambda: s.remove_out_of_domain(),
                 lambda: s.save_checkpoint(str(tmp_path / "c.bin"))):
        with pytest.raises(E) as e:
            call()
        assert e.value.status == gpu_tsph.ERR_UNSUPPORTED
    with pytest.raises(E) as e:  # only the mDBC fused step reads the table
        s.step(gpu_tsph.WALL_DBC, bt.dt, 1)
    assert e.value.status == gpu_tsph.ERR_UNSUPPORTED
    with pytest.raises(E) as e:
        s.set_tile_shape(0)
    assert e.value.status == gpu_tsph.ERR_ARG
    a = B.case_arrays(specs[0])
    f = gpu_tsph.ParticleSystem(a.h, a.kap, a.cs, 1000.0, 0.02, 0.1, a.spec.dp, a.domain, "fp32")
    with pytest.raises(E) as e:  # an empty range
        f.set_cases([[1.0, 1.0]], [9.81], [[0.0, 1.0, 0.0, 1.0]])
    assert e.value.status == gpu_tsph.ERR_ARG
    with pytest.raises(E) as e:  # two cases sharing columns
        f.set_cases([[0.0, 1.0], [0.5, 2.0]], [9.81, 9.81],
                    [[0.1, 0.9, 0.0, 1.0], [0.6, 1.9, 0.0, 1.0]])
    assert e.value.status == gpu_tsph.ERR_ARG
    d = gpu_tsph.ParticleSystem(a.h, a.kap, a.cs, 1000.0, 0.02, 0.1, a.spec.dp, a.domain, "fp64")
    with pytest.raises(E) as e:
        d.set_cases([[0.0, 1.0]], [9.81], [[0.0, 1.0, 0.0, 1.0]])
    assert e.value.status == gpu_tsph.ERR_UNSUPPORTED
    s.step(bt.wall_model, bt.dt, 2)
    assert s.health() == 0


@pytest.mark.gpu
def test_batched_water_front_matches_plain_runs(gpu_tsph):
    """The metric's bar for the batched form: three dam breaks of three
    spacings in one system, 5,000 system steps (0.1-0.2 s of each case's own
    time, well into the collapse), against each case run alone by the plain
    step for the same steps: the water front (largest fluid x at most 5 cm up)
    within 1 % (measured: well below), the case's mass unchanged."""
    specs = [B.CaseSpec(B.DAM_BREAK, 0.004, 1.0, 0.3, 0.3),
             B.CaseSpec(B.DAM_BREAK, 0.003, 1.2, 0.4, 0.3),
             B.CaseSpec(B.DAM_BREAK, 0.002, 0.8, 0.25, 0.25)]
    nsteps = 5000
    bt = B.Batch(specs)
    bt.step(nsteps)
    st = bt.system.download()
    assert bt.system.health() & ~gpu_tsph.HEALTH_REMOVED == 0
    for k, spec in enumerate(specs):
        a = B.case_arrays(spec)
        s = gpu_tsph.ParticleSystem(a.h, a.kap, a.cs, 1000.0, 0.02, 0.1, spec.dp, a.domain, "fp32")
        s.add_particles(a.type, a.r, None, a.rho, a.p, a.gnr)
        s.divide_to_cells()
        s.particle_to_cell()
        s.step(a.wall_model, a.dt, nsteps)
        ref = s.download()
        got = bt.case_state(k, st)

        def front(x):
            fl = (x["type"] == B.FLUID) & (x["r"][:, 1] <= 0.05)
            return float(np.max(x["r"][fl, 0]))

        fb, fp = front(got), front(ref)
        print(k, spec.dp, nsteps * a.dt, fb, fp, abs(fb - fp) / fp)
        assert abs(fb - fp) / fp <= 0.01, (k, fb, fp)
        assert abs(fp - s.water_front(0.05)) <= 1e-12  # the device's own front agrees
        assert np.sum(got["type"] == B.FLUID) == np.sum(ref["type"] == B.FLUID)
        s.close()
