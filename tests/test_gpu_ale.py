"""GPU parity of the Riemann / ALE-SPH path (tsph_ale_*) through the C ABI
against the reference's golden vectors and the oracle.

FP32 fluxes, FP64 integration of omega, omega*rho, omega*v.  Bars, per field:
rates and gradients within 2e-5 of the field's largest magnitude (FP32
rounding of ~20-term pair sums whose terms are ~1e3 times the result);
conserved variables within the integrated rate error (dt * steps * rate
bar) plus 1e-7 relative; derived v, rho, p and positions as in the WCSPH
parity tests.  Cell order and the particle set: exact.
"""

import os

import numpy as np
import pytest

from tinysph_old_gb300 import cases

GOLD = os.path.join(os.path.dirname(__file__), "golden")
RATES = ("domega", "domegarho", "domegav")


def _gold():
    return np.load(os.path.join(GOLD, "dam_break_ale_dp0.02.npz"))


def _err(a, b):
    return float(np.max(np.abs(np.asarray(a, dtype=np.float64) - np.asarray(b, dtype=np.float64))))


def _rate_tol(ref):
    return 2e-5 * float(np.max(np.abs(ref))) + 1e-12


def _check_state(st, ref, dt, nsteps, rates_ref, c0, tag=""):
    """Compare a downloaded ALE state with a reference state (dict of the
    same fields)."""
    fl = ref["type"] == 0 if "type" in ref else st["type"] == 0
    assert np.array_equal(st["index"], ref["index"]), tag
    errs = {}
    for f in RATES:
        e = _err(st[f][fl], ref[f][fl])
        lim = _rate_tol(rates_ref[f][fl])
        errs[f] = (e, lim)
    integ = {f: dt * nsteps * _rate_tol(rates_ref["d" + f][fl])
             for f in ("omega", "omegarho", "omegav")}
    for f in ("omega", "omegarho", "omegav"):
        e = _err(st[f][fl], ref[f][fl])
        lim = integ[f] * 4 + 1e-7 * float(np.max(np.abs(ref[f][fl])))
        errs[f] = (e, lim)
    vmag = float(np.max(np.abs(ref["v"][fl])))
    errs["v"] = (_err(st["v"][fl], ref["v"][fl]), 2e-6 + 1e-5 * vmag)
    errs["rho"] = (_err(st["rho"][fl], ref["rho"][fl]), 2e-4)
    errs["p"] = (_err(st["p"][fl], ref["p"][fl]), 2e-4 * c0 * c0 + 1e-6 * float(np.max(np.abs(ref["p"][fl]))))
    errs["r"] = (_err(st["r"], ref["r"]), 1e-9)
    print(tag, {f: f"{e:.3g}/{lim:.3g}" for f, (e, lim) in errs.items()})
    for f, (e, lim) in errs.items():
        assert e <= lim, (tag, f, e, lim)
    return errs


def _gpu(tsph, case, g, scheme=0):
    s = tsph.AleSystem.from_case(case, scheme=scheme)
    s.upload(v=g["init_v"], rho=g["init_rho"])
    return s


@pytest.mark.gpu
def test_ale_gradient_and_forces_vs_reference_golden(gpu_tsph):
    g = _gold()
    case = cases.dam_break_ale(dp=0.02)
    s = _gpu(gpu_tsph, case, g)
    st = s.download()
    fl = st["type"] == 0
    for k in ("r", "omega", "omegarho", "omegav"):  # FP64 on the device
        assert _err(st[k], g[f"init_{k}"]) <= 1e-15 * max(1.0, float(np.max(np.abs(g[f"init_{k}"])))), k
    # v and rho - rho0 are FP32 copies
    assert _err(st["v"], g["init_v"]) <= 1e-7 * float(np.max(np.abs(g["init_v"])))
    assert _err(st["rho"], g["init_rho"]) <= 1e-6
    s.gradient()
    s.forces(float(g["dt"]))
    st = s.download()
    e = _err(st["grad"][fl], g["forces_grad"][fl])
    assert e <= _rate_tol(g["forces_grad"][fl]), e
    for k in RATES:
        e = _err(st[k][fl], g[f"forces_{k}"][fl])
        assert e <= _rate_tol(g[f"forces_{k}"][fl]), (k, e)


@pytest.mark.gpu
def test_ale_step_vs_reference_golden(gpu_tsph):
    """The fused step (leap-frog one, fluxes, leap-frog two + removal +
    re-binning) against the reference's RUN loop, snapshot by snapshot."""
    g = _gold()
    case = cases.dam_break_ale(dp=0.02)
    s = _gpu(gpu_tsph, case, g)
    every = int(g["snap_every"])
    dt = float(g["dt"])
    rates = {f: g[f"forces_{f}"] for f in RATES}
    for k in range(every, int(g["nsteps"]) + 1, every):
        s.step(dt, k - every, every)
        st = s.download()
        ref = {f: g[f"step{k}_{f}"] for f in ("r", "v", "rho", "p", "omega", "omegarho",
                                              "omegav", "domega", "domegarho", "domegav",
                                              "index")}
        ref["type"] = g["init_type"]
        _check_state(st, ref, dt, k, rates, case.cs, tag=f"step{k}")
    assert s.health() & ~gpu_tsph.HEALTH_REMOVED == 0


@pytest.mark.gpu
def test_ale_muscl_scheme_vs_oracle(gpu_tsph, oracle_mod):
    """The MUSCL interface states (superbee-limited reconstruction of both
    particles, no counterpart in the reference) against the oracle's
    restatement of the same scheme."""
    O = oracle_mod
    g = _gold()
    case = cases.dam_break_ale(dp=0.02)
    dt = float(g["dt"])
    P = O.PortAle.from_case(case)
    P.set_threads(4)
    P.set_velocity_density(g["init_v"], g["init_rho"])
    P.set_scheme(1)
    s = _gpu(gpu_tsph, case, g, scheme=gpu_tsph.ALE_MUSCL)
    P.density_to_pressure()
    P.gradient()
    P.ale_forces(dt)
    s.gradient()
    s.forces(dt)
    ref = P.ale_state()
    st = s.download()
    fl = ref["type"] == 0
    assert _err(st["grad"][fl], ref["grad"][fl]) <= _rate_tol(ref["grad"][fl])
    for k in RATES:
        assert _err(st[k][fl], ref[k][fl]) <= _rate_tol(ref[k][fl]), k
    rates = {f: ref[f] for f in RATES}
    P2 = O.PortAle.from_case(case)
    P2.set_threads(4)
    P2.set_velocity_density(g["init_v"], g["init_rho"])
    P2.set_scheme(1)
    s2 = _gpu(gpu_tsph, case, g, scheme=gpu_tsph.ALE_MUSCL)
    P2.ale_step(dt, 0, 4)
    s2.step(dt, 0, 4)
    _check_state(s2.download(), P2.ale_state(), dt, 4, rates, case.cs, tag="muscl")


@pytest.mark.gpu
def test_ale_first_order_vs_reference_golden(gpu_tsph):
    """The first-order driver (SPH_simulationINT.h, src/RALESPH_interaction.h):
    fluxes at the initial state and 6 fused steps against the reference."""
    g = np.load(os.path.join(GOLD, "dam_break_ale_first_order_dp0.02.npz"))
    case = cases.dam_break_ale(dp=0.02)
    s = _gpu(gpu_tsph, case, g, scheme=gpu_tsph.ALE_FIRST_ORDER)
    s.forces(float(g["dt"]))
    st = s.download()
    fl = st["type"] == 0
    for k in RATES:
        e = _err(st[k][fl], g[f"forces_{k}"][fl])
        assert e <= _rate_tol(g[f"forces_{k}"][fl]), (k, e)
    s = _gpu(gpu_tsph, case, g, scheme=gpu_tsph.ALE_FIRST_ORDER)
    every = int(g["snap_every"])
    dt = float(g["dt"])
    rates = {f: g[f"forces_{f}"] for f in RATES}
    for k in range(every, int(g["nsteps"]) + 1, every):
        s.step(dt, k - every, every)
        ref = {f: g[f"step{k}_{f}"] for f in ("r", "v", "rho", "p", "omega", "omegarho",
                                              "omegav", "domega", "domegarho", "domegav",
                                              "index")}
        ref["type"] = g["init_type"]
        _check_state(s.download(), ref, dt, k, rates, case.cs, tag=f"first-order step{k}")


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [0, 1, 2])
def test_ale_fused_equals_per_function_sequence(gpu_tsph, scheme):
    """tsph_ale_step with a sort every step (kept cells off) and the
    reference's RUN order through the per-function entry points give
    bit-identical states (same kernels, same order)."""
    g = _gold()
    case = cases.dam_break_ale(dp=0.02)
    dt = float(g["dt"])
    a = _gpu(gpu_tsph, case, g, scheme)
    b = _gpu(gpu_tsph, case, g, scheme)
    a.set_keep_cells(False)
    b.set_keep_cells(False)
    a.step(dt, 0, 4)
    for stp in range(1, 5):
        if stp > 1:
            b.leapfrog_one(dt)
        b.particle_to_cell()
        if scheme == 1:
            b.gradient()
        b.forces(dt)
        b.leapfrog_two(dt, stp)
    b.particle_to_cell()
    x, y = a.download(), b.download()
    for f in ("r", "v", "rho", "omega", "omegarho", "omegav", "domega", "domegarho", "domegav",
              "index"):
        assert np.array_equal(x[f], y[f]), f


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [0, 2])
def test_ale_kept_cells_vs_sort_every_step(gpu_tsph, scheme):
    """Kept cells (the default) against a sort every step: the dp = 0.004 dam
    break from rest (densities perturbed by 1e-3) over 400 steps (16 ms):
    the collapse moves the column's front past the skin (2.7e-4 m) after
    ~185 steps, then every few tens of steps.  The states agree within the
    FP32 bars (summation order only), the same particles are live, and the
    sort ran on some steps and not on most."""
    case = cases.dam_break_ale(dp=0.004)
    rng = np.random.default_rng(5)
    a = case.particles.arrays()
    fl = a["type"] == 0
    rho = np.full(case.np, 1000.0)
    rho[fl] *= 1 + 1e-3 * rng.standard_normal(fl.sum())
    nsteps = 400
    runs = []
    for keep in (True, False):
        s = gpu_tsph.AleSystem.from_case(case, scheme=scheme)
        s.upload(rho=rho)
        s.set_keep_cells(keep)
        s.step(case.dt, 0, nsteps)
        runs.append((s.download(), s.sort_count()))
    (kept, nk), (ref, ne) = runs
    ref["type"] = kept["type"]
    # the bars' scale: the rates of the final state (from rest, the first
    # step's are zero)
    rates = {f: ref[f] for f in RATES}
    assert ne == 0
    assert 0 < nk < nsteps // 4, nk
    _check_state(kept, ref, case.dt, nsteps, rates, case.cs, tag=f"kept cells, scheme {scheme}")


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [0, 2])
def test_ale_removal_on_kept_cells(gpu_tsph, scheme):
    """Removal inside the fused step on kept cells: six fluid particles put
    just outside the domain box (inside the cell grid) leave the system at
    the next step, as with a sort every step (src/SPH_btdebug.h:4-31); the
    rest agrees within the FP32 bars."""
    case = cases.dam_break_ale(dp=0.004)
    a = case.particles.arrays()
    fl = np.flatnonzero(a["type"] == 0)
    r = a["r"].copy()
    moved = fl[:: len(fl) // 6][:6]
    r[moved, 0] = case.domain[1] + 0.1 * case.h
    runs = []
    for keep in (True, False):
        s = gpu_tsph.AleSystem.from_case(case, scheme=scheme)
        s.set_keep_cells(keep)
        s.upload(r=r)
        s.particle_to_cell()
        s.step(case.dt, 0, 3)
        runs.append((s.download(), s.health()))
    (kept, hk), (ref, he) = runs
    assert hk & gpu_tsph.HEALTH_REMOVED and he & gpu_tsph.HEALTH_REMOVED
    assert len(kept["index"]) == case.np - 6
    assert not np.isin(moved, kept["index"]).any()
    rates = {f: ref[f] for f in RATES}
    _check_state(kept, ref, case.dt, 3, rates, case.cs, tag=f"removal, scheme {scheme}")


@pytest.mark.gpu
def test_ale_part_one_ahead_is_exact(gpu_tsph):
    """On kept cells a step ends with the next step's part one applied; the
    state seen by a download, a second call of the step, or a per-function
    part one is the same bit for bit: ten steps in one call, in two calls,
    and in two calls with a download between them; six steps in one call
    and five followed by the per-function part one, fluxes and part two."""
    g = _gold()
    case = cases.dam_break_ale(dp=0.02)
    dt = float(g["dt"])
    fields = ("r", "v", "rho", "omega", "omegarho", "omegav", "domega", "domegarho",
              "domegav", "index")
    a, b, c, d, e = (_gpu(gpu_tsph, case, g) for _ in range(5))
    a.step(dt, 0, 10)
    b.step(dt, 0, 5)
    b.step(dt, 5, 5)
    c.step(dt, 0, 5)
    mid = c.download()
    c.step(dt, 5, 5)
    x = a.download()
    for other in (b, c):
        y = other.download()
        for f in fields:
            assert np.array_equal(x[f], y[f]), f
    assert not np.array_equal(mid["r"], x["r"])
    d.step(dt, 0, 6)
    e.step(dt, 0, 5)
    e.leapfrog_one(dt)
    e.forces(dt)
    e.leapfrog_two(dt, 6)
    x, y = d.download(), e.download()
    for f in fields:
        assert np.array_equal(x[f], y[f]), f


@pytest.mark.gpu
def test_ale_pipelined_transfers_equal_synchronous(gpu_tsph):
    """The pipelined loop (staged upload applied by particle_to_cell, step,
    download read back a step later) gives bit for bit the synchronous
    loop's results; a staged upload blocks the calls that use the state."""
    torch = pytest.importorskip("torch")
    case = cases.dam_break_ale(dp=0.004)
    dt = case.dt
    a, b = gpu_tsph.AleSystem.from_case(case), gpu_tsph.AleSystem.from_case(case)
    a.step(dt, 0, 3)
    b.step(dt, 0, 3)
    n = a.np
    mask = gpu_tsph.ALE_F_R | gpu_tsph.ALE_F_V | gpu_tsph.ALE_F_RHO
    hin = [torch.empty(shape, dtype=torch.float64, pin_memory=True)
           for shape in ((n, 2), (n, 2), (n,))]
    a.download_ptrs(mask, r=hin[0].data_ptr(), v=hin[1].data_ptr(), rho=hin[2].data_ptr())
    ptr = dict(r=hin[0].data_ptr(), v=hin[1].data_ptr(), rho=hin[2].data_ptr())
    outs = [[torch.empty_like(t, pin_memory=True) for t in hin] for _ in range(4)]
    sync = []
    for k in range(4):
        a.upload_ptrs(mask, **ptr)
        a.particle_to_cell()
        a.step(dt, 3 + k, 1)
        sync.append(a.download(gpu_tsph.ALE_F_R | gpu_tsph.ALE_F_V | gpu_tsph.ALE_F_RHO))
    b.upload_async(mask, **ptr)
    with pytest.raises(gpu_tsph.TsphError):
        b.step(dt, 3, 1)
    for k in range(4):
        if k:
            b.upload_async(mask, **ptr)
        b.particle_to_cell()
        b.step(dt, 3 + k, 1)
        o = outs[k]
        b.download_async(mask, r=o[0].data_ptr(), v=o[1].data_ptr(), rho=o[2].data_ptr())
    b.download_wait()
    for k in range(4):
        o = [t.numpy() for t in outs[k]]
        assert np.array_equal(o[0], sync[k]["r"]), k
        assert np.array_equal(o[1], sync[k]["v"]), k
        assert np.array_equal(o[2], sync[k]["rho"]), k
    assert b.health() & ~gpu_tsph.HEALTH_REMOVED == 0


@pytest.mark.gpu
def test_ale_particle_to_cell_on_kept_cells(gpu_tsph):
    """particle_to_cell on kept cells: positions moved within the skin keep
    the cells (no sort), a move past it sorts; the fluxes then equal those
    of a full re-binning within the FP32 bars."""
    case = cases.dam_break_ale(dp=0.004)
    s = gpu_tsph.AleSystem.from_case(case)
    ref = gpu_tsph.AleSystem.from_case(case)
    ref.set_keep_cells(False)
    st = s.download()
    fl = st["type"] == 0
    skin = 0.95 * 0.5 * (case.kap * case.h - 2.0 * case.h)
    rng = np.random.default_rng(3)
    for move, sorts in ((0.3 * skin, 0), (3.0 * skin, 1)):
        r = st["r"].copy()
        d = rng.normal(size=(int(fl.sum()), 2))
        d *= move / np.linalg.norm(d, axis=1, keepdims=True)
        r[fl] += d
        n0 = s.sort_count()
        for sys_ in (s, ref):
            sys_.upload(r=r)
            sys_.particle_to_cell()
            sys_.forces(case.dt)
        assert s.sort_count() - n0 == sorts, move
        x, y = s.download(), ref.download()
        for f in RATES:
            assert _err(x[f][fl], y[f][fl]) <= _rate_tol(y[f][fl]), (move, f)


@pytest.mark.gpu
def test_ale_stale_cells_and_bad_arguments(gpu_tsph):
    case = cases.dam_break_ale(dp=0.02)
    s = gpu_tsph.AleSystem.from_case(case)
    s.leapfrog_two(case.dt, 1)  # moves particles: cell lists stale
    with pytest.raises(gpu_tsph.TsphError):
        s.forces(case.dt)
    with pytest.raises(gpu_tsph.TsphError):
        s.step(case.dt, 1, 1)
    s.particle_to_cell()
    s.forces(case.dt)
    with pytest.raises(gpu_tsph.TsphError):
        s.set_scheme(7)
    with pytest.raises(gpu_tsph.TsphError):
        s.step(case.dt, -1, 1)


@pytest.mark.gpu
def test_ale_larger_case_vs_oracle(gpu_tsph, oracle_mod):
    """dp = 0.004 (11,476 fluid particles), 3 steps of the as-written scheme
    against the oracle; every fluid particle accounted for."""
    O = oracle_mod
    case = cases.dam_break_ale(dp=0.004)
    rng = np.random.default_rng(11)
    a = case.particles.arrays()
    fl = a["type"] == 0
    v = np.zeros((case.np, 2))
    v[fl] = rng.normal(0, 0.05, (fl.sum(), 2))
    rho = np.full(case.np, 1000.0)
    rho[fl] *= 1 + 1e-3 * rng.standard_normal(fl.sum())
    P = O.PortAle.from_case(case)
    P.set_threads(8)
    P.set_velocity_density(v, rho)
    s = gpu_tsph.AleSystem.from_case(case)
    s.upload(v=v, rho=rho)
    P.density_to_pressure()
    P.gradient()
    P.ale_forces(case.dt)
    s.gradient()
    s.forces(case.dt)
    ref0, st0 = P.ale_state(), s.download()
    for k in RATES + ("grad",):
        assert _err(st0[k][fl], ref0[k][fl]) <= _rate_tol(ref0[k][fl]), k
    rates = {f: ref0[f] for f in RATES}
    P2 = O.PortAle.from_case(case)
    P2.set_threads(8)
    P2.set_velocity_density(v, rho)
    s2 = gpu_tsph.AleSystem.from_case(case)
    s2.upload(v=v, rho=rho)
    P2.ale_step(case.dt, 0, 3)
    s2.step(case.dt, 0, 3)
    _check_state(s2.download(), P2.ale_state(), case.dt, 3, rates, case.cs, tag="dp0.004")


@pytest.mark.gpu
def test_ale_still_water_vs_reference_golden(gpu_tsph):
    """cases/ALESPH_stillWater (boundary-integral tank, hydrostatic start,
    h = 2 dp): gradients and fluxes at the golden input, then the fused step
    against the reference's RUN loop snapshot by snapshot."""
    g = np.load(os.path.join(GOLD, "still_water_ale_dp0.02.npz"))
    case = cases.still_water_ale(dp=0.02)
    s = _gpu(gpu_tsph, case, g)
    st = s.download()
    fl = st["type"] == 0
    s.gradient()
    s.forces(float(g["dt"]))
    st = s.download()
    e = _err(st["grad"][fl], g["forces_grad"][fl])
    assert e <= _rate_tol(g["forces_grad"][fl]), e
    for k in RATES:
        e = _err(st[k][fl], g[f"forces_{k}"][fl])
        assert e <= _rate_tol(g[f"forces_{k}"][fl]), (k, e)
    s = _gpu(gpu_tsph, case, g)
    every = int(g["snap_every"])
    dt = float(g["dt"])
    rates = {f: g[f"forces_{f}"] for f in RATES}
    for k in range(every, int(g["nsteps"]) + 1, every):
        s.step(dt, k - every, every)
        st = s.download()
        ref = {f: g[f"step{k}_{f}"] for f in ("r", "v", "rho", "p", "omega", "omegarho",
                                              "omegav", "domega", "domegarho", "domegav",
                                              "index")}
        ref["type"] = g["init_type"]
        _check_state(st, ref, dt, k, rates, case.cs, tag=f"step{k}")
    assert s.health() & ~gpu_tsph.HEALTH_REMOVED == 0
