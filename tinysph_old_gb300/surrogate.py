"""The learned surrogate: a graph network that advances the SPH state a window
of k = 8 steps at a time, trained on trajectories of the plain solver, with
the plain step as fallback (no counterpart in the reference).

A window, from a state whose last forces pass gave a_0 and drho_0
(tsph_step leaves the state so):

    graph   tsph_export_graph: nodes = particles, edges = pairs with r <= 2h
    network y = GNN(graph)                                    (tsph_gnn_infer)
    update  kick   v += k dt a_0 + U_out (y0, y1)             (tsph_apply_update 1)
            a forces pass with the kicked velocities gives drho*
            drift  rho += k dt drho* + S_out y2,
                   r += k dt (v_0 + v) / 2                    (tsph_apply_update 2)
            (or, scheme "explicit", one update with drho_0)   (tsph_apply_update 0)
    check   a forces pass at the new state gives a_1, drho_1; the window is
            kept if max |rho - (rho_0 + k dt (drho_0 + drho_1) / 2)| / rho0
            <= 1 % (density check) and the momentum error against
            v_0 + k dt (a_0 + a_1) / 2 stays within its bound; otherwise the
            state saved at the window start is restored and k plain steps
            run instead (tsph_window_check, tsph_state_save/_restore).

So the network predicts the part of the window's change that the rates do
not: y = 0 is the method without it (one symplectic step of k dt).  Device
memory comes from torch (allocation and, for building training targets,
index gathers); every computation of the rollout is a kernel of the
library.  The network's parameter layout and initial weights are in
gnn_params.py.
"""

from __future__ import annotations

import json
import math
import os
import time
from dataclasses import dataclass, field

import numpy as np

from . import gnn_params, sph

K_SLOTS = 48  # neighbour slots per node (the SPH pair set has ~24-36)
# the trained model shipped with the package (python -m tinysph_old_gb300.surrogate)
MODEL_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                          "surrogate_dam_break.npz")
K_STRIDE = 8  # SPH steps per surrogate window


class GraphBuffers:
    """Device arrays of one exported particle graph (capacity `cap` nodes)."""

    def __init__(self, cap, device="cuda", rates=True):
        import torch

        self.cap = int(cap)
        T = torch
        self.pos = T.empty((cap, 2), dtype=T.float64, device=device)
        self.vel = T.empty((cap, 2), dtype=T.float32, device=device)
        self.srho = T.empty(cap, dtype=T.float32, device=device)
        self.wall = T.empty(cap, dtype=T.float32, device=device)
        self.id = T.empty(cap, dtype=T.int32, device=device)
        self.deg = T.empty(cap, dtype=T.int32, device=device)
        self.nbr = T.empty((cap, K_SLOTS), dtype=T.int32, device=device)
        self.acc = T.empty((cap, 2), dtype=T.float32, device=device) if rates else None
        self.rate = T.empty(cap, dtype=T.float32, device=device) if rates else None
        self.n = 0
        self.nw = 0

    def export(self, system):
        """tsph_export_graph of `system`'s current state into these buffers."""
        self.n, self.nw = system.export_graph(
            K_SLOTS, self.cap, self.pos.data_ptr(), self.vel.data_ptr(), self.srho.data_ptr(),
            self.wall.data_ptr(), self.id.data_ptr(), self.deg.data_ptr(), self.nbr.data_ptr(),
            self.acc.data_ptr() if self.acc is not None else None,
            self.rate.data_ptr() if self.rate is not None else None)
        return self

    def clone(self, rates=False):
        """A copy holding only the exported nodes (for a training set)."""
        c = GraphBuffers.__new__(GraphBuffers)
        n = self.n
        c.cap = n
        for f in ("pos", "vel", "srho", "wall", "id", "deg", "nbr"):
            setattr(c, f, getattr(self, f)[:n].clone())
        c.acc = self.acc[:n].clone() if rates and self.acc is not None else None
        c.rate = self.rate[:n].clone() if rates and self.rate is not None else None
        c.n, c.nw = n, self.nw
        return c

    def struct(self, h, u_scale, s_scale):
        g = sph.GnnGraph()
        g.pos = self.pos.data_ptr()
        g.vel = self.vel.data_ptr()
        g.srho = self.srho.data_ptr()
        g.wall = self.wall.data_ptr()
        g.deg = self.deg.data_ptr()
        g.nbr = self.nbr.data_ptr()
        g.n_nodes = self.n
        g.k_slots = K_SLOTS
        g.h = float(h)
        g.u_scale = float(u_scale)
        g.s_scale = float(s_scale)
        return g

    def host(self):
        """numpy copies (for the oracle)."""
        n = self.n
        return dict(pos=self.pos[:n].cpu().numpy(), vel=self.vel[:n].cpu().numpy().astype(np.float64),
                    srho=self.srho[:n].cpu().numpy().astype(np.float64),
                    wall=self.wall[:n].cpu().numpy().astype(np.float64),
                    id=self.id[:n].cpu().numpy(), deg=self.deg[:n].cpu().numpy(),
                    nbr=self.nbr[:n].cpu().numpy())


@dataclass
class Model:
    """Trained parameters and the scales they were trained with."""

    params: np.ndarray  # float32, tsph_gnn_n_params
    u_in: float  # input velocity scale U (m/s)
    s_in: float  # input density scale S (kg/m^3)
    u_out: float  # output velocity scale (m/s per window)
    s_out: float  # output density scale (kg/m^3 per window)
    k: int = K_STRIDE
    meta: dict = field(default_factory=dict)

    def save(self, path):
        np.savez_compressed(path, params=self.params.astype(np.float32),
                            scales=np.array([self.u_in, self.s_in, self.u_out, self.s_out, self.k]),
                            meta=np.array(json.dumps(self.meta)))

    @classmethod
    def load(cls, path):
        z = np.load(path)
        u_in, s_in, u_out, s_out, k = z["scales"]
        return cls(z["params"].astype(np.float32), float(u_in), float(s_in), float(u_out),
                   float(s_out), int(k), json.loads(str(z["meta"])))

    @classmethod
    def zero(cls, k=K_STRIDE):
        """The network that outputs y = 0 (the method without it)."""
        return cls(np.zeros(sph.load().tsph_gnn_n_params(), np.float32), 1.0, 1.0, 1.0, 1.0, k)


def window_update(system, y_ptr, model, kdt, wall_model, scheme="explicit", zero_momentum=True):
    """The update part of a window (after export and the network): the
    single explicit update, or kick, forces pass, drift.  The network's
    velocity correction is taken less its fluid mean (no momentum)."""
    if scheme == "kick_drift":
        system.apply_update(y_ptr, model.u_out, model.s_out, kdt, True, phase=1,
                            zero_momentum=zero_momentum)
        system.compute_forces(wall_model)  # the continuity rate with the kicked velocities
        system.apply_update(y_ptr, model.u_out, model.s_out, kdt, True, phase=2)
    else:
        system.apply_update(y_ptr, model.u_out, model.s_out, kdt, True, phase=0,
                            zero_momentum=zero_momentum)


def end_of_window(system, wall_model):
    """Re-bin and run the forces pass at the window's end state; returns the
    number of particles that left the domain."""
    lost = system.remove_out_of_domain()
    system.particle_to_cell()
    if wall_model == sph.WALL_MDBC:
        system.mdbc_density()
    system.density_to_pressure()
    system.compute_forces(wall_model)
    return lost


# ------------------------------------------------------------------ data

def training_specs(n, seed, dp=0.002, area=0.18, aspect=(0.25, 2.0)):
    """Seeded dam breaks of the benchmark tank (1.61 m x 0.8 m walls, mDBC,
    c0 = 35 m/s) with random column aspect ratios col_h / col_w ~ U(aspect)
    and the column area fixed (0.18 m^2: about 45k fluid particles at
    dp = 0.002 m, like the 0.6 x 0.3 m benchmark column)."""
    from . import batch as B

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        a = float(rng.uniform(*aspect))
        w = math.sqrt(area / a)
        out.append(B.CaseSpec(B.DAM_BREAK, dp, 1.61, w, a * w))
    return out


class Sample:
    """One window of a trajectory: the graph at its start, the target per
    node (the change over k plain steps less the change of the window
    without the network, components du, dv, d(rho)) and that baseline
    change, in physical units (0 on walls)."""

    def __init__(self, graph, target, t, base=None):
        self.graph, self.target, self.t = graph, target, t
        self.base = base


def _by_id(gb, ntot):
    import torch

    n = gb.n
    out = torch.full((ntot, 3), float("nan"), device=gb.vel.device)
    idx = gb.id[:n].long()
    out[idx, :2] = gb.vel[:n]
    out[idx, 2] = gb.srho[:n]
    return out


def window_sample(system, ga, gb, wall_model, dt, k=K_STRIDE, scheme="explicit"):
    """From `system`'s state: export, run the window without the network
    (then restore), run k plain steps; the two changes matched by particle
    index."""
    import torch

    zero = Model.zero(k)
    kdt = k * dt
    ga.export(system)
    n = ga.n
    ntot = int(ga.id[:n].max()) + 1
    start = _by_id(ga, ntot)
    system.state_save()
    y = torch.zeros((n, 3), dtype=torch.float32, device=ga.vel.device)
    torch.cuda.synchronize()  # the system's kernels run on their own stream
    window_update(system, y.data_ptr(), zero, kdt, wall_model, scheme)
    end_of_window(system, wall_model)
    base = _by_id(gb.export(system), ntot) - start
    system.state_restore()
    system.step(wall_model, dt, k)
    true = _by_id(gb.export(system), ntot) - start
    ida = ga.id[:n].long()
    tgt = (true - base)[ida]
    base = base[ida]
    bad = (ga.wall[:n] != 0) | torch.isnan(tgt).any(1) | torch.isnan(base).any(1)
    tgt[bad] = 0.0
    base[bad] = 0.0
    return ga.clone(), tgt.contiguous(), base.contiguous()


def generate(specs, t_end, samples_per_case, cases_per_system=25, k=K_STRIDE, log=None,
             scheme="explicit", rollout_model=None, h=None):
    """Run the specs (packed `cases_per_system` to a particle system) to
    `t_end` and take `samples_per_case` windows from each, at evenly spaced
    times (the first after k steps, when the rates of a forces pass exist).
    The trajectory is the plain solver's, or with `rollout_model` the
    surrogate's own rollout with that model (windows checked, plain
    fallback), so that the samples hold the states the surrogate visits."""
    from . import batch as B

    out = []
    for c0 in range(0, len(specs), cases_per_system):
        bt = B.GroupedBatch(specs[c0:c0 + cases_per_system], streams=False)
        for g in bt.groups:
            s, dt = g.system, g.dt
            nsteps = int(round(t_end / dt))
            times = np.linspace(k, nsteps - k, samples_per_case).astype(int)
            cap = g.np + 64
            ga, gb = GraphBuffers(cap, rates=False), GraphBuffers(cap, rates=False)
            ro = None
            if rollout_model is not None:
                s.step(g.wall_model, dt, k)
                ro = Rollout(s, rollout_model, dt, g.wall_model, h or g.cases[0].h,
                             use_net=bool(np.any(rollout_model.params)), capacity=cap,
                             scheme=scheme)
            done = k if ro is not None else 0
            t0 = time.time()
            for st in times:
                st = int(st)
                if st > done:
                    if ro is not None:
                        nw = (st - done) // k
                        ro.run(nw)
                        done += nw * k
                    else:
                        s.step(g.wall_model, dt, st - done)
                        done = st
                graph, tgt, base = window_sample(s, ga, gb, g.wall_model, dt, k, scheme)
                done += k
                out.append(Sample(graph, tgt, done * dt, base))
            if log:
                fb = f", fallback {ro.fallback_rate:.2f}" if ro is not None else ""
                log(f"cases {c0}..{c0 + len(g.cases) - 1}: {g.np} particles, {done} steps, "
                    f"{len(times)} windows, {time.time() - t0:.1f} s{fb}")
        del bt
    return out


def fit_scales(samples, local=False, direct=False):
    """Input scales U, S and output scales over the fluid nodes: U, S the rms
    of |v| (per component) and of rho - rho0, or with `local` the rms of
    their differences across the graph's edges; the output scales the rms of
    the targets (with `direct`, of the whole change: target + base)."""
    acc = np.zeros(4)
    cnt = 0
    ecnt = 0
    for smp in samples:
        g = smp.graph
        fl = g.wall == 0
        if local:
            nb = g.nbr.long()
            ok = nb >= 0
            j = nb.clamp(min=0)
            dv = (g.vel[:, None, :] - g.vel[j]) * ok[..., None]
            ds = (g.srho[:, None] - g.srho[j]) * ok
            acc[0] += float((dv.double() ** 2).sum()) / 2
            acc[1] += float((ds.double() ** 2).sum())
            ecnt += int(ok.sum())
        else:
            acc[0] += float((g.vel[fl].double() ** 2).sum()) / 2
            acc[1] += float((g.srho[fl].double() ** 2).sum())
        t = smp.target + smp.base if direct else smp.target
        acc[2] += float((t[fl, :2].double() ** 2).sum()) / 2
        acc[3] += float((t[fl, 2].double() ** 2).sum())
        cnt += int(fl.sum())
    den = np.array([max(ecnt if local else cnt, 1)] * 2 + [max(cnt, 1)] * 2)
    return tuple(float(max(x, 1e-12)) for x in np.sqrt(acc / den))


# ------------------------------------------------------------------ training

def train(samples, scales, h, iters=1000, lr=1e-3, lr_end=1e-5, seed=0, params=None,
          log=None, log_every=100, clip=None, direct=False):
    """Adam on the device over the samples (one window per iteration, in a
    seeded shuffled order), cosine learning-rate decay; targets optionally
    clipped to +-clip (normalised units).  Returns (Model, loss history)."""
    import torch

    u_in, s_in, u_out, s_out = scales
    cap = max(smp.graph.n for smp in samples)
    net = sph.Gnn(cap)
    p0 = params if params is not None else gnn_params.initial_params(seed)
    net.set_params(p0)
    inv = torch.tensor([1.0 / u_out, 1.0 / u_out, 1.0 / s_out], device="cuda")
    targets = []
    for smp in samples:
        t = (smp.target + smp.base if direct else smp.target) * inv
        if clip:
            t = t.clamp(-clip, clip)
        targets.append(t.contiguous())
    structs = [smp.graph.struct(h, u_in, s_in) for smp in samples]
    rng = np.random.default_rng(seed)
    order = []
    hist = []
    t0 = time.time()
    for it in range(iters):
        if not order:
            order = list(rng.permutation(len(samples)))
        k = order.pop()
        loss = net.loss_grad(structs[k], targets[k].data_ptr())
        lr_t = lr_end + 0.5 * (lr - lr_end) * (1 + math.cos(math.pi * it / max(iters - 1, 1)))
        net.adam(lr_t)
        hist.append(loss)
        if log and (it % log_every == 0 or it == iters - 1):
            log(f"iter {it}: loss {loss:.4f} (lr {lr_t:.2e}, {time.time() - t0:.1f} s)")
    model = Model(net.params(), u_in, s_in, u_out, s_out, K_STRIDE,
                  dict(iters=iters, lr=lr, samples=len(samples), h=h, clip=clip))
    return model, np.array(hist)


def evaluate(model, samples, h):
    """Per output, the mean squared error of the network on the samples
    (normalised units) and that of y = 0 (the window without the network)."""
    import torch

    cap = max(smp.graph.n for smp in samples)
    net = sph.Gnn(cap)
    net.set_params(model.params)
    y = torch.empty((cap, 3), dtype=torch.float32, device="cuda")
    inv = torch.tensor([1.0 / model.u_out, 1.0 / model.u_out, 1.0 / model.s_out], device="cuda")
    se_net = np.zeros(3)
    se_zero = np.zeros(3)
    cnt = 0
    for smp in samples:
        g = smp.graph
        net.forward(g.struct(h, model.u_in, model.s_in), y.data_ptr())
        fl = g.wall == 0
        t = smp.target * inv
        se_zero += (t[fl] ** 2).sum(0).double().cpu().numpy()
        se_net += ((y[:g.n][fl] - t[fl]) ** 2).sum(0).double().cpu().numpy()
        cnt += int(fl.sum())
    return se_net / max(cnt, 1), se_zero / max(cnt, 1)


# ------------------------------------------------------------------ rollout

class Rollout:
    """A particle system advanced by surrogate windows, each checked and,
    when the check fails, replaced by k plain steps from the saved start.
    ``use_net=False`` runs the same windows with y = 0 (the method without
    the network)."""

    def __init__(self, system, model, dt, wall_model, h, tol_density=0.01, tol_momentum=0.5,
                 use_net=True, capacity=None, scheme="explicit"):
        import torch

        self.s = system
        self.m = model
        self.dt = float(dt)
        self.k = int(model.k)
        self.kdt = self.k * self.dt
        self.wall_model = wall_model
        self.h = float(h)
        self.tol_density = tol_density
        self.tol_momentum = tol_momentum
        self.use_net = use_net
        self.scheme = scheme
        cap = int(capacity or system.np + 64)
        self.gb = GraphBuffers(cap, rates=False)
        self.y = torch.zeros((cap, 3), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        self.net = None
        if use_net:
            # the network runs on the system's stream: its output feeds the
            # system's update and its input is the system's export
            self.net = sph.Gnn(cap, stream=system.stream_ptr())
            self.net.set_params(model.params)
        self.windows = 0
        self.fallbacks = 0
        self.checks = []  # (max density err, rms, momentum err, accepted, worst particle)

    def window(self):
        """One window of k steps; True if the surrogate's update was kept."""
        s = self.s
        s.health(clear=True)
        s.state_save()
        self.gb.export(s)
        if self.use_net:
            # the BF16 tensor-core forward (trained in FP32 by tsph_gnn_loss_grad)
            self.net.infer(self.gb.struct(self.h, self.m.u_in, self.m.s_in), self.y.data_ptr())
        window_update(s, self.y.data_ptr(), self.m, self.kdt, self.wall_model, self.scheme)
        lost = end_of_window(s, self.wall_model)
        mx, rms, mom, _, worst = s.window_check(self.kdt)
        flags = s.health(clear=True)
        ok = (lost == 0 and flags == 0 and mx <= self.tol_density
              and (self.tol_momentum is None or mom <= self.tol_momentum))
        self.checks.append((mx, rms, mom, ok, worst))
        self.windows += 1
        if not ok:
            self.fallbacks += 1
            s.state_restore()
            s.step(self.wall_model, self.dt, self.k)
        return ok

    def run(self, n_windows):
        for _ in range(n_windows):
            self.window()

    @property
    def fallback_rate(self):
        return self.fallbacks / max(self.windows, 1)


def plain_check_floor(system, wall_model, dt, n_windows, k=K_STRIDE):
    """The window check applied to the plain solver's own windows: the
    floor of the check's errors (the trapezoidal rule's error on the plain
    trajectory).  Returns an array of (max, rms, momentum) per window."""
    import torch

    cap = system.np + 64
    gb = GraphBuffers(cap, rates=False)
    y = torch.zeros((cap, 3), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    out = []
    for _ in range(n_windows):
        gb.export(system)
        system.apply_update(y.data_ptr(), 0.0, 0.0, 0.0, False)  # records the start, moves nothing
        system.particle_to_cell()
        system.step(wall_model, dt, k)
        out.append(system.window_check(k * dt)[:3])
    return np.array(out)


# ------------------------------------------------------------------ evaluation

GAUGES_X = (0.3, 0.8, 1.3, 1.5)  # free-surface gauges (Water_Elevation), m
PROBES = ((1.60, 0.02), (1.60, 0.10), (1.60, 0.20))  # pressure probes at the far wall, m


def observe(system, front_y=0.02):
    """The quantities the surrogate is checked on: water front (largest fluid
    x with y <= front_y), free-surface elevation at the gauges, pressure at
    the probes (Shepard, as Pressure_in_point)."""
    return dict(front=system.water_front(front_y),
                level=system.water_level(np.array(GAUGES_X), 0.0).tolist(),
                pressure=system.point_fields(np.array(PROBES))[:, 1].tolist())


def compare_runs(case, model, t_end, marks, log=None, use_net=True):
    """Plain SPH and the surrogate from the same start to `t_end`, observed at
    `marks`; device times of both and the surrogate's fallback rate."""
    import torch

    out = dict(marks=list(marks), np=None)
    for kind in ("plain", "surrogate"):
        s = sph.ParticleSystem.from_case(case)
        s.step(0, case.dt, K_STRIDE)  # a forces pass for the first window
        out["np"] = s.np
        obs = []
        done = K_STRIDE
        ro = None
        if kind == "surrogate":
            ro = Rollout(s, model, case.dt, case.wall_model, case.h, use_net=use_net)
        torch.cuda.synchronize()
        t0 = time.time()
        for t in marks:
            nw = max(0, (int(round(t / case.dt)) - done) // K_STRIDE)
            if ro is None:
                s.step(case.wall_model, case.dt, nw * K_STRIDE)
            else:
                ro.run(nw)
            done += nw * K_STRIDE
            s.sync()
            t1 = time.time()
            obs.append(observe(s))
            t0 += time.time() - t1  # observation time excluded
        torch.cuda.synchronize()
        out[kind] = dict(obs=obs, seconds=time.time() - t0, steps=done - K_STRIDE)
        if ro is not None:
            out[kind]["fallback_rate"] = ro.fallback_rate
            out[kind]["windows"] = ro.windows
        if log:
            log(f"{kind}: {out[kind]['seconds']:.1f} s" +
                (f", fallback {ro.fallback_rate:.3f}" if ro is not None else ""))
    p, q = out["plain"]["obs"], out["surrogate"]["obs"]
    h0 = 0.3
    out["errors"] = dict(
        front=[abs(b["front"] - a["front"]) / a["front"] for a, b in zip(p, q)],
        level=[max(abs(x - y) for x, y in zip(a["level"], b["level"])) / h0 for a, b in zip(p, q)],
        pressure=[max(abs(x - y) for x, y in zip(a["pressure"], b["pressure"])) /
                  (1000.0 * 9.81 * h0) for a, b in zip(p, q)])
    for kind in ("plain", "surrogate"):
        out[kind]["particle_steps_per_s"] = out["np"] * out[kind]["steps"] / out[kind]["seconds"]
    return out


def pipeline(out_model, n_train=400, n_held=50, t_train=0.3, samples=8, cases_per_system=25,
             iters=1500, seed=0, eval_dp=0.0005, t_eval=1.0, log=print):
    """Config 5 end to end: training windows from the surrogate's own rollouts
    (y = 0 model, plain fallback) over `n_train` seeded dam breaks at
    dp = 0.002 m, training on the device, the one-window error on `n_held`
    held-out seeds against the method without the network, and plain versus
    surrogate on the benchmark dam break at `eval_dp` for `t_eval` s."""
    from . import batch as B
    from . import cases as CS

    res = {}
    specs = training_specs(n_train, seed)
    held_specs = training_specs(n_held, seed + 1)
    h = B.case_arrays(specs[0]).h
    zero = Model.zero()
    t0 = time.time()
    data = generate(specs, t_train, samples, cases_per_system, rollout_model=zero, log=log)
    held = generate(held_specs, t_train, samples, cases_per_system, rollout_model=zero, log=log)
    res["generate_s"] = time.time() - t0
    scales = fit_scales(data)
    t0 = time.time()
    model, hist = train(data, scales, h, iters=iters, seed=seed, log=log, log_every=250)
    res["train_s"] = time.time() - t0
    model.meta.update(n_train=n_train, t_train=t_train, dp=0.002)
    model.save(out_model)
    a, z = evaluate(model, held, h)
    res["held_out_mse_net"], res["held_out_mse_without"] = a.tolist(), z.tolist()
    log(f"held-out one-window mse: network {a}, without it {z}")
    del data, held
    case = CS.dam_break_benchmark(dp=eval_dp)
    marks = [round(0.05 * i, 2) for i in range(1, int(round(t_eval / 0.05)) + 1)]
    res["eval"] = compare_runs(case, model, t_eval, marks, log=log)
    return model, res


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description="train and evaluate the surrogate")
    ap.add_argument("--out-model", required=True)
    ap.add_argument("--out-json", required=True)
    ap.add_argument("--n-train", type=int, default=400)
    ap.add_argument("--n-held", type=int, default=50)
    ap.add_argument("--t-train", type=float, default=0.3)
    ap.add_argument("--iters", type=int, default=1500)
    ap.add_argument("--eval-dp", type=float, default=0.0005)
    ap.add_argument("--t-eval", type=float, default=1.0)
    a = ap.parse_args()
    _, r = pipeline(a.out_model, a.n_train, a.n_held, a.t_train, iters=a.iters,
                    eval_dp=a.eval_dp, t_eval=a.t_eval, log=lambda m: print(m, flush=True))
    with open(a.out_json, "w") as f:
        json.dump(r, f, indent=1)
