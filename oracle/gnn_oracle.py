"""CPU oracle of the learned surrogate's network (TEST INFRASTRUCTURE).

The graph network of the surrogate, restated in numpy (float64) to check the
device kernels' forward pass and gradients (tinysph_old_gb300/csrc/tsph_gnn.cu)
and, by central differences, its own backward pass.  It has no counterpart in
the reference (which has no learned part); it follows the same definitions
as the device code:

    node input   x_i = (u_i / U, v_i / U, (rho_i - rho0) / S, wall_i)
    edge input   e_ij = (dx / h, dy / h, |r| / h, (u_i - u_j) / U, (v_i - v_j) / U),
                 dx = x_i - x_j, for every pair 0 < r <= 2h
    encoder      h_i = SiLU(A0 x_i + a0)
    layer (x2)   P = h Wp^T, Q = h Wq^T
                 S_i = sum_j SiLU(P_i + Q_j + We e_ij + be)
                 m_i = W2 S_i + deg_i b2
                 h_i <- h_i + Wn2 SiLU(Wn1 [h_i, m_i] + bn1) + bn2
    decoder      y_i = Wd h_i + bd

(The edge MLP's second layer is applied after the neighbour sum, which is
the same function: W2 sum_j s_ij + deg b2 = sum_j (W2 s_ij + b2).)
"""

import numpy as np

H = 64
LAYERS = 2
NIN, EIN, NOUT = 4, 5, 3


def param_shapes(hidden=H, layers=LAYERS):
    """(name, shape) in the flat order shared with the device code."""
    out = [("A0", (hidden, NIN)), ("a0", (hidden,))]
    for l in range(layers):
        out += [(f"Wp{l}", (hidden, hidden)), (f"Wq{l}", (hidden, hidden)),
                (f"We{l}", (hidden, EIN)), (f"be{l}", (hidden,)),
                (f"W2{l}", (hidden, hidden)), (f"b2{l}", (hidden,)),
                (f"Wn1{l}", (hidden, 2 * hidden)), (f"bn1{l}", (hidden,)),
                (f"Wn2{l}", (hidden, hidden)), (f"bn2{l}", (hidden,))]
    out += [("Wd", (NOUT, hidden)), ("bd", (NOUT,))]
    return out


def n_params(hidden=H, layers=LAYERS):
    return sum(int(np.prod(s)) for _, s in param_shapes(hidden, layers))


def unflatten(flat, hidden=H, layers=LAYERS):
    p, o = {}, 0
    for name, shape in param_shapes(hidden, layers):
        n = int(np.prod(shape))
        p[name] = np.asarray(flat[o:o + n], dtype=np.float64).reshape(shape)
        o += n
    return p


def flatten(p, hidden=H, layers=LAYERS):
    return np.concatenate([np.asarray(p[name], dtype=np.float64).ravel()
                           for name, _ in param_shapes(hidden, layers)])


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def graph_inputs(pos, vel, srho, wall, deg, nbr, h, U, S):
    """Node and edge inputs from an exported graph (numpy arrays)."""
    n = len(deg)
    x = np.stack([vel[:, 0] / U, vel[:, 1] / U, srho / S, wall], 1).astype(np.float64)
    K = nbr.shape[1]
    ii = np.repeat(np.arange(n), K)
    jj = nbr.reshape(-1)
    keep = jj >= 0
    ii, jj = ii[keep], jj[keep]
    d = pos[ii] - pos[jj]
    r = np.sqrt(np.sum(d * d, 1))
    dv = vel[ii] - vel[jj]
    e = np.stack([d[:, 0] / h, d[:, 1] / h, r / h, dv[:, 0] / U, dv[:, 1] / U], 1)
    return x, ii, jj, e, deg.astype(np.float64)


def forward(p, x, ii, jj, e, deg, layers=LAYERS):
    n = len(x)
    cache = {"x": x, "ii": ii, "jj": jj, "e": e, "deg": deg}
    z0 = x @ p["A0"].T + p["a0"]
    h = silu(z0)
    cache["z0"] = z0
    for l in range(layers):
        P = h @ p[f"Wp{l}"].T
        Q = h @ p[f"Wq{l}"].T
        z = P[ii] + Q[jj] + e @ p[f"We{l}"].T + p[f"be{l}"]
        S = np.zeros((n, P.shape[1]))
        np.add.at(S, ii, silu(z))
        m = S @ p[f"W2{l}"].T + deg[:, None] * p[f"b2{l}"]
        hm = np.concatenate([h, m], 1)
        u = hm @ p[f"Wn1{l}"].T + p[f"bn1{l}"]
        t = silu(u)
        cache[l] = dict(h=h, P=P, Q=Q, z=z, S=S, m=m, hm=hm, u=u, t=t)
        h = h + t @ p[f"Wn2{l}"].T + p[f"bn2{l}"]
    cache["hL"] = h
    y = h @ p["Wd"].T + p["bd"]
    return y, cache


def backward(p, cache, dy, layers=LAYERS):
    g = {}
    h = cache["hL"]
    g["Wd"] = dy.T @ h
    g["bd"] = dy.sum(0)
    dh = dy @ p["Wd"]
    ii, jj, e, deg = cache["ii"], cache["jj"], cache["e"], cache["deg"]
    n = len(dh)
    for l in reversed(range(layers)):
        c = cache[l]
        g[f"bn2{l}"] = dh.sum(0)
        g[f"Wn2{l}"] = dh.T @ c["t"]
        du = (dh @ p[f"Wn2{l}"]) * dsilu(c["u"])
        g[f"bn1{l}"] = du.sum(0)
        g[f"Wn1{l}"] = du.T @ c["hm"]
        dhm = du @ p[f"Wn1{l}"]
        Hh = c["h"].shape[1]
        dh_in = dh + dhm[:, :Hh]
        dm = dhm[:, Hh:]
        g[f"W2{l}"] = dm.T @ c["S"]
        g[f"b2{l}"] = (deg[:, None] * dm).sum(0)
        dS = dm @ p[f"W2{l}"]
        dz = dS[ii] * dsilu(c["z"])
        g[f"We{l}"] = dz.T @ e
        g[f"be{l}"] = dz.sum(0)
        dP = np.zeros_like(c["P"])
        dQ = np.zeros_like(c["Q"])
        np.add.at(dP, ii, dz)
        np.add.at(dQ, jj, dz)
        g[f"Wp{l}"] = dP.T @ c["h"]
        g[f"Wq{l}"] = dQ.T @ c["h"]
        dh = dh_in + dP @ p[f"Wp{l}"] + dQ @ p[f"Wq{l}"]
    dz0 = dh * dsilu(cache["z0"])
    g["A0"] = dz0.T @ cache["x"]
    g["a0"] = dz0.sum(0)
    return g


def loss_and_grad(p, x, ii, jj, e, deg, target, mask):
    """Mean squared error over the masked (fluid) nodes and its gradient."""
    y, cache = forward(p, x, ii, jj, e, deg)
    nm = max(int(mask.sum()), 1)
    r = (y - target) * mask[:, None]
    loss = float(np.sum(r * r) / nm)
    dy = 2.0 * r / nm
    return loss, backward(p, cache, dy), y


def init_params(seed=0, hidden=H, layers=LAYERS):
    """Glorot-uniform weights, zero biases; the residual branches (Wn2) start
    small so the untrained network is close to the identity update."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, shape in param_shapes(hidden, layers):
        if len(shape) == 1:
            p[name] = np.zeros(shape)
        else:
            lim = np.sqrt(6.0 / (shape[0] + shape[1]))
            if name.startswith("Wn2") or name == "Wd":
                lim *= 0.1
            p[name] = rng.uniform(-lim, lim, size=shape)
    return p
