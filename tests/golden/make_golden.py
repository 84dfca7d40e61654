"""Generate the golden vectors in this directory from the reference itself.

Runs the reference's own code (oracle/_ref/libtsph_ref.so, compiled from the
reference headers by ``make -C oracle ref``) on small seeded cases and stores
its outputs.  Needs the reference sources; the committed .npz files are what
the tests read.  Usage: python tests/golden/make_golden.py [ale|probes|bt|zones]
(``ale`` / ``probes`` / ``bt`` / ``zones`` regenerate only the ALE-SPH, the
probe, the BT-wall or the open-boundary fixtures)
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from tinysph_old_gb300 import cases  # noqa: E402

SEED = 20261203


def perturb(state, rng, dv=0.05, drho=1e-3):
    """Seeded perturbation of fluid velocity and density (walls untouched)."""
    fl = state["type"] == 0
    v = state["v"].copy()
    rho = state["rho"].copy()
    v[fl] += rng.normal(0.0, dv, size=(fl.sum(), 2))
    rho[fl] *= 1.0 + drho * rng.standard_normal(fl.sum())
    return v, rho


def geometry(ref_case_fn, name, out):
    case = ref_case_fn()
    R = O.RefSystem(case.h, case.kap, case.cs, case.rho0, case.visco, case.delta, case.dp,
                    case.domain)
    return case, R


def dam_break_geometry(dp):
    """The reference's own generators for cases/damBreakLong_mDBC/geometry.h."""
    case = cases.dam_break_mdbc(dp=dp)
    R = O.RefSystem(case.h, case.kap, case.cs, case.rho0, case.visco, case.delta, case.dp,
                    case.domain)
    L, s = R.L, R.s
    L.ref_create_wall_x_mdbc(s, 0.0 + dp, 1.61, 0.0, -1, dp / 2)
    L.ref_create_wall_y_mdbc(s, 0.0, 0 + dp, 1.0, -1, dp / 2)
    L.ref_create_wall_y_mdbc(s, 1.61, 0 + dp, 1.0, +1, 1.61 - dp / 2)
    L.ref_create_corner_mdbc(s, -1, -1, 0.0 + dp / 2, 0.0 + dp / 2)
    L.ref_create_corner_mdbc(s, +1, -1, 1.61 - dp / 2, 0.0 + dp / 2)
    L.ref_create_block_of_fluid(s, 0 + dp, 0 + dp, 0.6, 0.3)
    st = R.state()
    return dict(r=st["r"], type=st["type"], rho=st["rho"], p=st["p"], gnr=R.gnr())


def wp_geometry(dp=0.02):
    """Create_Block_of_FluidWP + DBC walls of the reference (src/SPH_create.h)."""
    case = cases.still_water_dbc(dp=dp)
    R = O.RefSystem(case.h, case.kap, case.cs, case.rho0, case.visco, case.delta, case.dp,
                    case.domain)
    L, s = R.L, R.s
    L.ref_create_wall_x(s, 0.0, 0.5, 0.0, -1)
    L.ref_create_wall_y(s, 0.0, 0.0 + dp, 0.4, -1)
    L.ref_create_block_of_fluid_wp(s, 0 + dp, 0 + dp, 0.5 - dp, 0.3)
    st = R.state()
    return dict(r=st["r"], type=st["type"], rho=st["rho"], p=st["p"])


def run_case(case, model, nsteps, rng, snap_every):
    R = O.RefSystem.from_case(case)
    R.set_threads(1)
    st0 = R.state()
    v, rho = perturb(st0, rng)
    R.set_state(v=v, rho=rho)
    init = R.state()
    # per-function outputs at the perturbed initial state
    R.density_to_pressure()
    p0 = R.state()["p"]
    out = dict(init_r=init["r"], init_v=init["v"], init_rho=init["rho"], init_type=init["type"],
               init_p=p0)
    start, lst = R.cells()
    out["cell_start"] = start
    out["cell_list"] = lst
    if model == 0:
        R.mdbc_density()
        out["mdbc_rho"] = R.state()["rho"]
        R.set_state(rho=init["rho"])
        R.density_to_pressure()
    R.compute_forces(model)
    f = R.state()
    out["forces_a"] = f["a"]
    out["forces_drho"] = f["drho"]
    # back to the perturbed initial state (a = drho = 0) and run the RUN loop
    R2 = O.RefSystem.from_case(case)
    R2.set_state(v=v, rho=rho)
    done = 0
    k = 0
    while done < nsteps:
        R2.step(model, case.dt, snap_every)
        done += snap_every
        st = R2.state()
        for key in ("r", "v", "a", "rho", "drho", "p", "index"):
            out[f"step{done}_{key}"] = st[key]
        k += 1
    out["dt"] = np.float64(case.dt)
    out["nsteps"] = np.int64(nsteps)
    out["snap_every"] = np.int64(snap_every)
    return out


def ale_geometry(dp):
    """The reference's BT generators for cases/ALESPH_dambreakLong/geometry.h."""
    case = cases.dam_break_ale(dp=dp)
    R = O.RefAle(case)
    L, s = R.L, R.s
    L.refale_create_wall_x_bt(s, 0.0 + dp, 1.61 - dp, 0.0, -1, 0.0, 1.0)
    L.refale_create_wall_y_bt(s, 0.0, 0.0 + dp, 1.0, -1, 1.0, 0.0)
    L.refale_create_wall_y_bt(s, 1.61, 0.0 + dp, 1.0, +1, -1.0, 0.0)
    L.refale_create_corner_bt(s, -1, -1, 0.0, 0.0, np.sqrt(2), np.sqrt(2))
    L.refale_create_corner_bt(s, +1, -1, 1.61, 0.0, -np.sqrt(2), np.sqrt(2))
    L.refale_create_block_of_fluid(s, 0.0 + dp, 0 + dp, 0.6, 0.3)
    st = R.ale_state()
    return dict(r=st["r"], type=st["type"], rho=st["rho"], omega=st["omega"],
                normals=R.normals())


def run_ale(case, nsteps, rng, snap_every, first_order=False):
    """Riemann / ALE-SPH dam break (cases/ALESPH_dambreakLong/MUSCL.h RUN loop)
    from a seeded perturbation of the fluid velocity and density."""
    O.RefAle.set_threads(1)
    R = O.RefAle.from_case(case)
    st0 = R.ale_state()
    fl = st0["type"] == 0
    v = st0["v"].copy()
    rho = st0["rho"].copy()
    v[fl] += rng.normal(0.0, 0.05, size=(fl.sum(), 2))
    rho[fl] *= 1.0 + 1e-3 * rng.standard_normal(fl.sum())
    R.set_velocity_density(v, rho)
    init = R.ale_state()
    out = {f"init_{k}": init[k] for k in ("r", "v", "rho", "type", "omega", "omegarho", "omegav")}
    out["normals"] = R.normals()
    # per-function outputs at the perturbed initial state
    R.density_to_pressure()
    if first_order:
        R.ale_forces_first_order()
    else:
        R.gradient()
        R.ale_forces(case.dt)
    f = R.ale_state()
    for k in ("grad", "domega", "domegarho", "domegav"):
        out[f"forces_{k}"] = f[k]
    R2 = O.RefAle.from_case(case)
    R2.set_velocity_density(v, rho)
    done = 0
    while done < nsteps:
        if first_order:
            R2.ale_step_first_order(case.dt, done, snap_every)
        else:
            R2.ale_step(case.dt, done, snap_every)
        done += snap_every
        st = R2.ale_state()
        for k in ("r", "v", "rho", "p", "omega", "omegarho", "omegav", "domega", "domegarho",
                  "domegav", "index"):
            out[f"step{done}_{k}"] = st[k]
    out["dt"] = np.float64(case.dt)
    out["nsteps"] = np.int64(nsteps)
    out["snap_every"] = np.int64(snap_every)
    return out


def wendland_samples():
    rng = np.random.default_rng(SEED)
    h = np.array([0.001, np.sqrt(2) * 0.005, 0.0075, 0.04])
    rows = []
    for hh in h:
        r = np.concatenate([[0.0, 2 * hh, 2 * hh * (1 + 1e-12)], rng.uniform(0, 2.2 * hh, 60)])
        for rr in r:
            w, f = O.ref_wendland(float(rr), float(hh))
            rows.append((rr, hh, w, f))
    return np.array(rows)


def main_ale():
    """ALE-SPH fixtures (own seed, so the WCSPH fixtures do not change)."""
    if not O.ref_ale_available():
        raise SystemExit("reference ALE harness not available (needs the reference sources)")
    rng = np.random.default_rng(SEED + 1)
    out = {}
    for k, v in ale_geometry(0.02).items():
        out[f"geom_{k}"] = v
    out.update(run_ale(cases.dam_break_ale(dp=0.02), 6, rng, 2))
    np.savez_compressed(os.path.join(HERE, "dam_break_ale_dp0.02.npz"), **out)
    # the first-order driver (cases/ALESPH_dambreakLong/SPH_simulationINT.h)
    fo = run_ale(cases.dam_break_ale(dp=0.02), 6, np.random.default_rng(SEED + 2), 2,
                 first_order=True)
    np.savez_compressed(os.path.join(HERE, "dam_break_ale_first_order_dp0.02.npz"), **fo)
    # cases/ALESPH_stillWater (hydrostatic start, h = 2 dp), the MUSCL.h RUN loop
    sw = run_ale(cases.still_water_ale(dp=0.02), 6, np.random.default_rng(SEED + 9), 2)
    np.savez_compressed(os.path.join(HERE, "still_water_ale_dp0.02.npz"), **sw)


def main_bt():
    """WCSPH dam break with boundary-integral walls (cases/damBreakLong_BT,
    SPH_simulationSymplectic.h RUN loop; own seed): the tank from the
    reference's generators, the per-function outputs (BT wall density,
    Compute_Forces of src/SPH_interactionBT.h) at a seeded perturbed state,
    and the state after 20 steps."""
    if not O.ref_bt_available():
        raise SystemExit("reference BT harness not available (needs the reference sources)")
    O.RefBt.set_threads(1)
    case = cases.dam_break_bt(dp=0.02)
    gen = O.RefBt.generated(case, case.dp)
    g = gen.state()
    out = {"geom_r": g["r"], "geom_type": g["type"], "geom_rho": g["rho"], "geom_p": g["p"],
           "geom_normals": gen.normals()}
    rng = np.random.default_rng(SEED + 3)
    R = O.RefBt.from_case(case)
    v, rho = perturb(R.state(), rng, dv=0.1, drho=1e-3)
    R.set_velocity_density(v, rho)
    out["init_v"], out["init_rho"] = v, rho
    R.bt_density()
    R.density_to_pressure()
    R.compute_forces()
    f = R.state()
    for k in ("rho", "p", "a", "drho"):
        out[f"forces_{k}"] = f[k]
    R2 = O.RefBt.from_case(case)
    R2.set_velocity_density(v, rho)
    for done in (10, 20):
        R2.step(case.dt, 10)
        st = R2.state()
        for k in ("r", "v", "rho", "p", "a", "drho", "index"):
            out[f"step{done}_{k}"] = st[k]
    out["dt"] = np.float64(case.dt)
    np.savez_compressed(os.path.join(HERE, "dam_break_bt_dp0.02.npz"), **out)
    # still water with BT walls (cases/stillWater_BT): the reference's RUN
    # loop from the case's hydrostatic start, states after 100 and 300 steps
    case = cases.still_water_bt(dp=0.02)
    R3 = O.RefBt.from_case(case)
    out = {"dt": np.float64(case.dt), "snaps": np.array([100, 300])}
    done = 0
    for n in (100, 300):
        R3.step(case.dt, n - done)
        done = n
        st = R3.state()
        for k in ("r", "v", "rho", "p", "a", "drho", "index"):
            out[f"step{n}_{k}"] = st[k]
    np.savez_compressed(os.path.join(HERE, "still_water_bt_dp0.02.npz"), **out)
    # cases/flowDrop_BT: the inlet jet over a BT floor with two outlets.  The
    # reference is defined only until the first erasure: its Remove_particle
    # also erases special.rhoTemp[p], a vector the BT generators leave shorter
    # than the particle list, so erasing a particle past its end is undefined
    # (the harness crashes once the jet reaches the floor, ~650 steps at
    # dp = 0.02); the snapshots stop before that
    dp = 0.02
    case = cases.flow_drop_bt(dp=dp)
    G = O.RefBt(case)
    G.L.refbt_create_wall_x_bt(G.s, 0.0 - dp * 2, 2.0 + dp * 2, 0.0, -1, 0.0, 1.0)
    G.L.refbt_create_inlet_x(G.s, 0.3 + 4 * dp, 0.8 + dp, 1.0, +1, 4, 0.0, -3.0, 7)
    G.L.refbt_create_outlet_y(G.s, 1.3 - 4 * dp, 0.0 + dp, 0.2, +1, 4, 2.0, 0.0, 12, 1)
    G.L.refbt_create_outlet_y(G.s, 0.5, 0.0 + dp, 0.2, -1, 4, -2.0, 0.0, 13, 1)
    g = G.state()
    out = {"geom_r": g["r"], "geom_type": g["type"], "geom_v": g["v"],
           "geom_normals": G.normals(), "dt": np.float64(case.dt),
           "snaps": np.array([200, 400, 600])}
    R4 = O.RefBt.from_case(case)
    done = 0
    for n in (200, 400, 600):
        R4.step_zones(case.dt, n - done)
        done = n
        st = R4.state()
        for k in ("r", "v", "rho", "p", "a", "drho", "type", "index"):
            out[f"step{n}_{k}"] = st[k]
    np.savez_compressed(os.path.join(HERE, "flow_drop_bt_dp0.02.npz"), **out)


def _perturbed_walls(case, u):
    """The case with every wall particle's x scaled by 1 + k u, k in -6..6
    (a fixed pattern over the particle index): a perturbation of a few units
    of roundoff u that enters the flow only where it meets the walls."""
    ps = case.particles
    for i in range(ps.np):
        if ps.type[i] == 1:
            ps.rx[i] = ps.rx[i] * (1 + u * ((i * 7919) % 13 - 6))
    return case


def main_dbc():
    """cases/damBreakLong_DBC: the DBC interaction on the dam break (mDBC
    walls, hydrostatic column), per-function outputs and 6 steps of the RUN
    loop from a seeded perturbed state (own seed); cases/stillWater_mDBC the
    same way."""
    if O.build_ref() is None or not O.ref_available():
        raise SystemExit("reference harness not available (needs the reference sources)")
    rng = np.random.default_rng(SEED + 7)
    out = run_case(cases.dam_break_dbc(dp=0.02), 1, 6, rng, 2)
    np.savez_compressed(os.path.join(HERE, "dam_break_dbc_dp0.02.npz"), **out)
    # cases/stillWater_mDBC (h = 2 dp: ~50 neighbours), same recipe, own seed
    rng = np.random.default_rng(SEED + 8)
    out = run_case(cases.still_water_mdbc(dp=0.02), 0, 6, rng, 2)
    np.savez_compressed(os.path.join(HERE, "still_water_mdbc_dp0.02.npz"), **out)


def main_inflow_tank_bottom():
    """cases/inflowTankBottom_mDBC at dp = 0.02: the reference's generators
    and its RUN loop (the mDBC step with the inlet after the predictor)."""
    O.RefSystem.set_threads(1)
    dp = 0.02
    case = cases.inflow_tank_bottom_mdbc(dp=dp)
    G = O.RefSystem(case.h, case.kap, case.cs, case.rho0, case.visco, case.delta, case.dp,
                    case.domain)
    L, s = G.L, G.s
    L.ref_create_wall_x_mdbc(s, 0.2 + dp, 1.2 - dp, 0.0, -1, dp / 2)
    L.ref_create_wall_y_mdbc(s, 0.2, 0 + dp, 0.4, -1, dp / 2)
    L.ref_create_wall_y_mdbc(s, 1.2, 0 + dp, 0.8, +1, 1.2 - dp / 2)
    L.ref_create_corner_mdbc(s, -1, -1, 0.2 + dp / 2, 0.0 + dp / 2)
    L.ref_create_corner_mdbc(s, +1, -1, 1.2 - dp / 2, 0.0 + dp / 2)
    L.ref_create_wall_x_mdbc(s, 0.0 + dp, 0.4, 0.4 + 3 * dp, -1, dp / 2)
    L.ref_create_block_of_fluid_wp(s, 0.2 + dp, 0 + dp, 1.2, 0.15)
    L.ref_create_inlet_y(s, 0.1, 0.4 + 4 * dp, 0.5, -1, 4, 1.5, 0.0, 7)
    g = G.state()
    out = {f"geom_{k}": g[k] for k in ("r", "v", "rho", "p", "type")}
    out["dt"] = np.float64(case.dt)
    out["snaps"] = np.array([500, 1000, 1500])
    # the reference's own spread (the jet meets the ledge and the tank: the
    # last bits are amplified), as for cases/flowDrop_mDBC
    runs = [O.RefSystem.from_case(case)]
    runs += [O.RefSystem.from_case(_perturbed_walls(cases.inflow_tank_bottom_mdbc(dp=dp), u))
             for u in (2.0 ** -53, 2.0 ** -24)]
    done = 0
    for n in out["snaps"]:
        for R in runs:
            R.step_zones(case.dt, int(n) - done)
        done = int(n)
        st = runs[0].state()
        for k in ("r", "v", "rho", "p", "type"):
            out[f"step{n}_{k}"] = st[k]
        for R, tag in zip(runs[1:], ("spread64", "spread32")):
            pt = R.state()
            assert np.array_equal(pt["type"], st["type"]), (n, tag)
            for k in ("r", "v", "rho", "p"):
                out[f"step{n}_{k}_{tag}"] = np.float64(np.max(np.abs(pt[k] - st[k])))
    np.savez_compressed(os.path.join(HERE, "inflow_tank_bottom_mdbc_dp0.02.npz"), **out)


def main_zones():
    """Open boundaries: cases/inflowSlab_mDBC (the case's own RUN loop with
    BZ_Integrate_inlet / _outlet), an outlet channel that exercises the
    outlet's retyping and removal, and cases/flowDrop_mDBC (a y-oriented
    inlet jet falling onto a floor that drains through a +x and a -x
    outlet); states at snapshots (particle order of the reference's arrays,
    types included).  For the jet, whose impact on the floor amplifies
    any difference in the last bits, the fixture also holds the reference's
    own spread at each snapshot: the largest difference per field between
    its run and its run with the walls perturbed by a few units of FP64
    (``spread64``) or FP32 (``spread32``) roundoff."""
    if O.build_ref() is None or not O.ref_available():
        raise SystemExit("reference harness not available (needs the reference sources)")
    O.RefSystem.set_threads(1)
    for builder, snaps, fname, spread in (
            (lambda: cases.inflow_slab_mdbc(dp=0.005), (100, 200, 400),
             "inflow_slab_mdbc_dp0.005.npz", False),
            (lambda: cases.outlet_channel_mdbc(dp=0.005), (200, 300, 400, 500, 600),
             "outlet_channel_mdbc_dp0.005.npz", False),
            (lambda: cases.flow_drop_mdbc(dp=0.02), (600, 800, 1000, 1200),
             "flow_drop_mdbc_dp0.02.npz", True)):
        case = builder()
        runs = [O.RefSystem.from_case(case)]
        if spread:
            runs += [O.RefSystem.from_case(_perturbed_walls(builder(), u))
                     for u in (2.0 ** -53, 2.0 ** -24)]
        out = {"dt": np.float64(case.dt), "snaps": np.array(snaps)}
        done = 0
        for n in snaps:
            for R in runs:
                R.step_zones(case.dt, n - done)
            done = n
            st = runs[0].state()
            for k in ("r", "v", "rho", "p", "type"):
                out[f"step{n}_{k}"] = st[k]
            for R, tag in zip(runs[1:], ("spread64", "spread32")):
                pt = R.state()
                assert np.array_equal(pt["type"], st["type"]), (fname, n, tag)
                for k in ("r", "v", "rho", "p"):
                    out[f"step{n}_{k}_{tag}"] = np.float64(np.max(np.abs(pt[k] - st[k])))
        np.savez_compressed(os.path.join(HERE, fname), **out)


WL_GAUGES = [(0.3, 0.0, 0), (0.3, 0.45, 1), (0.865, 0.0, 0), (0.865, 0.45, 1),
             (1.114, 0.0, 0), (1.114, 0.45, 1), (1.3625, 0.0, 0), (1.3625, 0.45, 1)]
PT_PROBES = [(1.61, 0.003), (1.61, 0.015), (1.61, 0.03), (1.61, 0.08), (0.3, 0.1), (0.2, 0.25),
             (0.55, 0.05), (0.7, 0.02), (0.05, 0.29), (1.0, 0.5)]


def main_probes():
    """Probes of cases/damBreakLong_mDBC (water levels h1-h4 and their inverse
    gauges, constants.h:57-80; pressure sensors p1-p4, :84-94, plus interior
    points) on the reference's state after 20 steps at dp = 0.01."""
    if O.build_ref() is None or not O.ref_available():
        raise SystemExit("reference harness not available (needs the reference sources)")
    case = cases.dam_break_mdbc(dp=0.01)
    R = O.RefSystem.from_case(case)
    R.set_threads(1)
    R.step(0, case.dt, 20)
    st = R.state()
    out = {k: st[k] for k in ("r", "v", "rho", "p", "type", "index")}
    out["gauges"] = np.array(WL_GAUGES, dtype=np.float64)
    out["water_level"] = np.array([R.water_level(x, y0, bool(inv)) for x, y0, inv in WL_GAUGES])
    out["points"] = np.array(PT_PROBES, dtype=np.float64)
    out["point_fields"] = np.array([R.point_fields(x, y) for x, y in PT_PROBES])
    out["pressure_in_point"] = np.array([R.pressure_in_point(x, y) for x, y in PT_PROBES])
    np.savez_compressed(os.path.join(HERE, "probes_dam_break_dp0.01.npz"), **out)


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "ale":
        main_ale()
        return
    if len(sys.argv) > 1 and sys.argv[1] == "probes":
        main_probes()
        return
    if len(sys.argv) > 1 and sys.argv[1] == "bt":
        main_bt()
        return
    if len(sys.argv) > 1 and sys.argv[1] == "zones":
        main_zones()
        return
    if len(sys.argv) > 1 and sys.argv[1] == "dbc":
        main_dbc()
        return
    if len(sys.argv) > 1 and sys.argv[1] == "tank_bottom":
        main_inflow_tank_bottom()
        return
    if O.build_ref() is None or not O.ref_available():
        raise SystemExit("reference harness not available (needs the reference sources)")
    rng = np.random.default_rng(SEED)
    # 1. geometry from the reference generators
    g = {}
    for dp in (0.02, 0.01):
        for k, v in dam_break_geometry(dp).items():
            g[f"dam_dp{dp:g}_{k}"] = v
    for k, v in wp_geometry(0.02).items():
        g[f"wp_dp0.02_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "geometry.npz"), **g)
    # 2. dam break, mDBC flavour, 6 steps
    dam = run_case(cases.dam_break_mdbc(dp=0.02), 0, 6, rng, 2)
    np.savez_compressed(os.path.join(HERE, "dam_break_mdbc_dp0.02.npz"), **dam)
    # 3. still water, DBC flavour, 6 steps
    sw = run_case(cases.still_water_dbc(dp=0.02), 1, 6, rng, 2)
    np.savez_compressed(os.path.join(HERE, "still_water_dbc_dp0.02.npz"), **sw)
    # 4. Wendland kernel samples
    np.savez_compressed(os.path.join(HERE, "wendland.npz"), samples=wendland_samples())
    # 5. Riemann / ALE-SPH dam break, 6 steps
    main_ale()
    # 6. probes (water level, point fields)
    main_probes()
    # 7. boundary-integral walls (WCSPH), 20 steps
    main_bt()
    # 8. open boundaries
    main_zones()
    # 9. dam break, DBC flavour
    main_dbc()
    # 10. inflow over a ledge into a tank (open boundary, mDBC)
    main_inflow_tank_bottom()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
