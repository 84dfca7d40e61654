"""Batched cases: the vectorised generators, the seeded batch, the packing of
equal-constant cases into one domain, and (GPU) per-case results of a packed
group against separate runs of the same cases."""

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
        c = cases.still_water_dbc(dp=spec.dp, width=spec.col_w, depth=spec.col_h,
                                  tank_height=spec.col_h + 0.1)
    ca = c.particles.arrays()
    assert a.np == c.np
    for k in ("r", "type", "rho", "p"):
        assert np.array_equal(getattr(a, k), ca[k]), k
    if len(ca["gnr"]):
        assert np.array_equal(a.gnr[:len(ca["gnr"])], ca["gnr"])
    assert (a.h, a.kap, a.cs, a.dt, a.wall_model) == (c.h, c.kap, c.cs, c.dt, c.wall_model)


def test_seeded_batch_spans_the_stated_sizes():
    specs = B.sample_specs(512, seed=0)
    n = np.array([B.case_arrays(s).np for s in specs])
    assert len(specs) == 512
    assert n.min() >= 2000 and n.max() <= 100_000
    assert {s.dp for s in specs} == {0.004, 0.003, 0.002}
    assert {s.kind for s in specs} == {B.DAM_BREAK, B.STILL_WATER}
    assert specs == B.sample_specs(512, seed=0)  # deterministic


def test_packing_keeps_cases_apart():
    specs = B.sample_specs(64, seed=3)
    for key, members in B.group_specs(specs).items():
        g = B.pack([B.case_arrays(s) for _, s in members])
        c0 = g.cases[0]
        kh = c0.h * c0.kap
        gap = B.SPLASH_GAP if key[0] == B.DAM_BREAK else 4 * kh
        for k in range(len(g.cases) - 1):
            right = g.offset[k] + g.cases[k].extent[1]
            left = g.offset[k + 1] + g.cases[k + 1].extent[0]
            assert left - right >= gap * (1 - 1e-12)
            # no particle of one case within 2h of the next one
            xr = (g.cases[k].r[:, 0] + g.offset[k]).max()
            xl = (g.cases[k + 1].r[:, 0] + g.offset[k + 1]).min()
            assert xl - xr > 2 * c0.h
        assert all(len({(c.h, c.kap, c.cs, c.dt, c.wall_model) for c in g.cases}) == 1 for _ in [0])


@pytest.mark.gpu
def test_packed_group_matches_separate_runs(gpu_tsph):
    specs = [B.CaseSpec(B.DAM_BREAK, 0.004, 1.0, 0.4, 0.3), B.CaseSpec(B.DAM_BREAK, 0.004, 1.6, 0.6, 0.25),
             B.CaseSpec(B.STILL_WATER, 0.004, 1.0, 0.5, 0.3), B.CaseSpec(B.STILL_WATER, 0.004, 1.0, 0.3, 0.2),
             B.CaseSpec(B.DAM_BREAK, 0.004, 0.9, 0.3, 0.45)]
    bt = B.Batch(specs, streams=False)
    assert len(bt.groups) == 2
    nsteps = 200
    bt.step(nsteps)
    for k, spec in enumerate(specs):
        a = B.case_arrays(spec)
        s = gpu_tsph.ParticleSystem(a.h, a.kap, a.cs, 1000.0, 0.02, 0.1, spec.dp, a.domain, "fp32")
        s.add_particles(a.type, a.r, None, a.rho, a.p, a.gnr if a.wall_model == 0 else None)
        s.divide_to_cells()
        s.particle_to_cell()
        s.step(a.wall_model, a.dt, nsteps)
        ref = s.download()
        got = bt.case_state(k)
        assert np.array_equal(got["index"], ref["index"]), k
        er = float(np.max(np.abs(got["r"] - ref["r"])))
        ev = float(np.max(np.abs(got["v"] - ref["v"])))
        erho = float(np.max(np.abs(got["rho"] - ref["rho"])))
        print(k, spec.kind, er, ev, erho)
        assert er <= 1e-5 and ev <= 2e-3 and erho <= 2e-2, (k, er, ev, erho)
