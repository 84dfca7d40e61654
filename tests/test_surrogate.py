"""The learned surrogate's pieces: the exported particle graph and the graph
network's device kernels (forward and gradients) against the numpy oracle
(oracle/gnn_oracle.py), whose own gradients are checked by central
differences."""

import os
import sys

import numpy as np
import pytest

from tinysph_old_gb300 import cases

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "oracle"))
import gnn_oracle as G  # noqa: E402


def _toy_graph(rng, n=30, K=8, radius=0.35):
    pos = rng.uniform(0, 1, (n, 2))
    d = np.linalg.norm(pos[:, None] - pos[None], axis=2)
    nbr = -np.ones((n, K), int)
    deg = np.zeros(n, int)
    for i in range(n):
        js = [j for j in np.argsort(d[i]) if j != i and d[i, j] < radius][:K]
        nbr[i, :len(js)] = js
        deg[i] = len(js)
    return pos, nbr, deg


def test_oracle_gradients_match_central_differences():
    rng = np.random.default_rng(0)
    pos, nbr, deg = _toy_graph(rng)
    n = len(deg)
    vel = rng.normal(0, 0.3, (n, 2))
    srho = rng.normal(0, 1, n)
    wall = (rng.random(n) < 0.2).astype(float)
    x, ii, jj, e, dg = G.graph_inputs(pos, vel, srho, wall, deg, nbr, 0.2, 1.0, 1.0)
    p = G.init_params(1)
    for k in p:
        p[k] = p[k] + rng.normal(0, 0.05, p[k].shape)
    target = rng.normal(0, 1, (n, 3))
    mask = 1 - wall
    _, g, _ = G.loss_and_grad(p, x, ii, jj, e, dg, target, mask)
    flat, gf = G.flatten(p), G.flatten(g)
    for k in rng.choice(len(flat), 60, replace=False):
        f2 = flat.copy()
        f2[k] += 1e-6
        lp = G.loss_and_grad(G.unflatten(f2), x, ii, jj, e, dg, target, mask)[0]
        f2[k] -= 2e-6
        lm = G.loss_and_grad(G.unflatten(f2), x, ii, jj, e, dg, target, mask)[0]
        fd = (lp - lm) / 2e-6
        assert abs(fd - gf[k]) <= 1e-4 * max(1e-6, abs(fd) + abs(gf[k])), (k, fd, gf[k])


def test_package_parameter_layout_matches_the_oracle():
    """The package's own layout and initial weights (gnn_params) agree block by
    block with the oracle's independent statement of the network."""
    from tinysph_old_gb300 import gnn_params as GP

    assert [(n, tuple(s)) for n, s in GP.param_shapes()] == \
        [(n, tuple(s)) for n, s in G.param_shapes()]
    assert GP.n_params() == G.n_params() == 50819
    for seed in (0, 3):
        ours = GP.initial_params(seed)
        theirs = G.flatten(G.init_params(seed)).astype(np.float32)
        assert ours.dtype == np.float32
        np.testing.assert_array_equal(ours, theirs)
    flat = np.arange(GP.n_params(), dtype=np.float64)
    back = GP.unflatten(flat)
    np.testing.assert_array_equal(GP.flatten(back, dtype=np.float64), flat)
    np.testing.assert_array_equal(G.flatten(G.unflatten(flat)), flat)


@pytest.mark.gpu
def test_exported_graph_is_the_symmetric_pair_set(gpu_tsph):
    from tinysph_old_gb300 import surrogate as S

    case = cases.dam_break_mdbc(dp=0.02)
    s = gpu_tsph.ParticleSystem.from_case(case)
    s.step(0, case.dt, 5)
    gb = S.GraphBuffers(case.np + 16).export(s)
    hst = gb.host()
    st = s.download()
    n = gb.n
    assert n == case.np and gb.nw == int(np.sum(st["type"] == 1))
    # node data against the state (reference order by particle index)
    order = hst["id"]
    assert np.array_equal(np.sort(order), np.arange(n))
    assert np.array_equal(hst["pos"], st["r"][order])
    assert np.allclose(hst["vel"], st["v"][order], atol=1e-7)
    assert np.array_equal(hst["wall"], (st["type"][order] == 1).astype(float))
    # edges: symmetric, within 2h, and every pair within 2h (minus a rounding band)
    edges = {(i, int(j)) for i in range(n) for j in hst["nbr"][i, :hst["deg"][i]]}
    assert all((j, i) in edges for i, j in edges)
    r = hst["pos"]
    d = np.linalg.norm(r[:, None] - r[None], axis=2)
    two_h = 2 * case.h
    inside = {(i, j) for i in range(n) for j in np.nonzero((d[i] < two_h * (1 - 1e-6)) & (d[i] > 0))[0]}
    assert inside <= edges
    assert all(d[i, j] <= two_h * (1 + 1e-6) for i, j in edges)


@pytest.mark.gpu
def test_gnn_forward_and_gradients_match_the_oracle(gpu_tsph):
    import torch

    from tinysph_old_gb300 import surrogate as S

    case = cases.dam_break_mdbc(dp=0.02)
    s = gpu_tsph.ParticleSystem.from_case(case)
    rng = np.random.default_rng(4)
    st = s.download()
    fl = st["type"] == 0
    v = st["v"].copy()
    v[fl] = rng.normal(0, 0.5, (fl.sum(), 2))
    rho = st["rho"].copy()
    rho[fl] += rng.normal(0, 2.0, fl.sum())
    s.upload(v=v, rho=rho)
    gb = S.GraphBuffers(case.np).export(s)
    hst = gb.host()
    U, Sc, h = 1.0, 2.0, case.h
    p = G.init_params(7)
    for k in p:
        p[k] = p[k] + rng.normal(0, 0.05, p[k].shape)
    net = gpu_tsph.Gnn(gb.n)
    net.set_params(G.flatten(p).astype(np.float32))
    p32 = G.unflatten(net.params().astype(np.float64))  # the FP32-rounded weights
    target = rng.normal(0, 1, (gb.n, 3))
    tgt = torch.tensor(target, dtype=torch.float32, device="cuda")
    graph = gb.struct(h, U, Sc)
    loss = net.loss_grad(graph, tgt.data_ptr())
    y_dev = torch.empty((gb.n, 3), dtype=torch.float32, device="cuda")
    net.forward(graph, y_dev.data_ptr())
    torch.cuda.synchronize()
    x, ii, jj, e, dg = G.graph_inputs(hst["pos"], hst["vel"], hst["srho"], hst["wall"],
                                      hst["deg"], hst["nbr"], h, U, Sc)
    lref, gref, yref = G.loss_and_grad(p32, x, ii, jj, e, dg, target, 1 - hst["wall"])
    y = y_dev.cpu().numpy()
    assert np.max(np.abs(y - yref)) <= 1e-4 * max(1.0, np.max(np.abs(yref)))
    assert abs(loss - lref) <= 1e-4 * lref
    gdev = G.unflatten(net.grads().astype(np.float64))
    for name, _ in G.param_shapes():
        ref = gref[name]
        err = np.max(np.abs(gdev[name] - ref))
        assert err <= 2e-3 * max(1e-6, np.max(np.abs(ref))), (name, err, np.max(np.abs(ref)))


def _random_graph_setup(gpu_tsph, seed=4):
    from tinysph_old_gb300 import surrogate as S

    case = cases.dam_break_mdbc(dp=0.02)
    s = gpu_tsph.ParticleSystem.from_case(case)
    rng = np.random.default_rng(seed)
    st = s.download()
    fl = st["type"] == 0
    v = st["v"].copy()
    v[fl] = rng.normal(0, 0.5, (fl.sum(), 2))
    rho = st["rho"].copy()
    rho[fl] += rng.normal(0, 2.0, fl.sum())
    s.upload(v=v, rho=rho)
    gb = S.GraphBuffers(case.np).export(s)
    p = G.init_params(seed)
    for k in p:
        p[k] = p[k] + rng.normal(0, 0.05, p[k].shape)
    return case, s, gb, p


@pytest.mark.gpu
def test_bf16_tensor_core_inference_matches_the_fp32_forward(gpu_tsph):
    """tsph_gnn_infer (BF16 weights and activations on the tensor cores, FP32
    accumulation, hardware tanh in the edge SiLU) against tsph_gnn_forward
    (FP32 throughout): within the BF16 rounding, 2 % of the outputs' rms."""
    import torch

    case, s, gb, p = _random_graph_setup(gpu_tsph)
    net = gpu_tsph.Gnn(gb.n)
    net.set_params(G.flatten(p).astype(np.float32))
    graph = gb.struct(case.h, 1.0, 2.0)
    y32 = torch.empty((gb.n, 3), dtype=torch.float32, device="cuda")
    y16 = torch.empty((gb.n, 3), dtype=torch.float32, device="cuda")
    net.forward(graph, y32.data_ptr())
    net.infer(graph, y16.data_ptr())
    torch.cuda.synchronize()
    a, b = y32.cpu().numpy(), y16.cpu().numpy()
    rms = np.sqrt(np.mean(a * a, 0))
    err = np.sqrt(np.mean((a - b) ** 2, 0))
    assert np.all(err <= 0.02 * rms), (err, rms)
    assert np.max(np.abs(a - b)) <= 0.05 * np.max(np.abs(a))


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [0, 2])
def test_fallback_windows_reproduce_plain_stepping(gpu_tsph, variant):
    """A rollout whose every window fails its check (tolerance below zero)
    restores the saved state and runs the plain steps: bit-identical to plain
    stepping, with the tiled pair kernel and with the pair-records kernel
    (whose kept neighbour lists the window's own binnings overwrite: the
    restore rebuilds them at the saved binning positions)."""
    from tinysph_old_gb300 import surrogate as S

    case = cases.dam_break_mdbc(dp=0.02)
    a = gpu_tsph.ParticleSystem.from_case(case)
    b = gpu_tsph.ParticleSystem.from_case(case)
    a.set_tile_shape(variant)
    b.set_tile_shape(variant)
    a.step(0, case.dt, 8)
    b.step(0, case.dt, 8)
    ro = S.Rollout(a, S.Model.zero(), case.dt, 0, case.h, use_net=False, tol_density=-1.0)
    ro.run(6)
    b.step(0, case.dt, 6 * S.K_STRIDE)
    assert ro.fallbacks == 6
    sa, sb = a.download(), b.download()
    oa, ob = np.argsort(sa["index"]), np.argsort(sb["index"])
    for f in ("r", "v", "rho"):
        assert np.array_equal(sa[f][oa], sb[f][ob]), f


@pytest.mark.gpu
def test_window_check_on_the_plain_trajectory_is_at_its_floor(gpu_tsph):
    """The window check (trapezoidal SPH rates at both ends) applied to the
    plain solver's own windows: far below the 1 % fallback threshold."""
    from tinysph_old_gb300 import surrogate as S

    case = cases.dam_break_mdbc(dp=0.02)
    s = gpu_tsph.ParticleSystem.from_case(case)
    s.step(0, case.dt, 200)
    fl = S.plain_check_floor(s, 0, case.dt, 5)
    assert np.all(fl[:, 0] < 1e-3), fl


def test_training_specs_and_model_file_round_trip(tmp_path):
    """The seeded training tanks keep the column area (about 45k particles at
    dp = 0.002 m) with aspect ratios in range; a model file keeps parameters
    and scales."""
    from tinysph_old_gb300 import surrogate as S

    specs = S.training_specs(20, 3)
    for sp in specs:
        assert abs(sp.col_w * sp.col_h - 0.18) < 1e-12
        assert 0.25 <= sp.col_h / sp.col_w <= 2.0 and sp.col_h < 0.8 and sp.col_w < 1.61
    assert S.training_specs(20, 3) == specs and S.training_specs(20, 4) != specs
    m = S.Model(np.arange(G.n_params(), dtype=np.float32), 0.8, 2.4, 0.027, 1.06, 8, {"a": 1})
    m.save(tmp_path / "m.npz")
    r = S.Model.load(tmp_path / "m.npz")
    assert np.array_equal(r.params, m.params) and r.meta == {"a": 1}
    assert (r.u_in, r.s_in, r.u_out, r.s_out, r.k) == (0.8, 2.4, 0.027, 1.06, 8)


@pytest.mark.gpu
def test_trained_network_gains_over_the_window_without_it(gpu_tsph):
    """The committed model against y = 0 (one explicit window of k dt from the
    rates alone) on windows of held-out tanks (seeds the training never saw),
    taken from the surrogate's own rollout: the network removes most of the
    window's error in dv and in rho."""
    from tinysph_old_gb300 import surrogate as S
    from tinysph_old_gb300 import batch as B

    model = S.Model.load(S.MODEL_PATH)
    specs = S.training_specs(2, 777)
    held = S.generate(specs, 0.15, 3, cases_per_system=2, rollout_model=S.Model.zero())
    h = B.case_arrays(specs[0]).h
    net, zero = S.evaluate(model, held, h)
    ratio = net / zero
    assert ratio[1] < 0.6 and ratio[2] < 0.6, ratio
