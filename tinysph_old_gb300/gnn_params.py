"""Flat parameter layout and initial weights of the surrogate's graph network.

The device kernels (csrc/tsph_gnn.cu) read the network's parameters as one
float32 vector; this module defines the order of its blocks and the seeded
initial values used to start training.  The layout is:

    A0 (H, 4), a0 (H)                                  node encoder
    per layer: Wp, Wq (H, H), We (H, 5), be (H),       edge MLP, first layer
               W2 (H, H), b2 (H),                      edge MLP, second layer
               Wn1 (H, 2H), bn1 (H), Wn2 (H, H), bn2 (H)   node MLP
    Wd (3, H), bd (3)                                  decoder

with H = 64 and two message-passing layers (50,819 parameters).
"""

from __future__ import annotations

import numpy as np

HIDDEN = 64
LAYERS = 2
N_NODE_IN, N_EDGE_IN, N_OUT = 4, 5, 3


def param_shapes(hidden=HIDDEN, layers=LAYERS):
    """(name, shape) of every block, in the order of the flat vector."""
    blocks = [("A0", (hidden, N_NODE_IN)), ("a0", (hidden,))]
    for layer in range(layers):
        blocks.extend([
            (f"Wp{layer}", (hidden, hidden)), (f"Wq{layer}", (hidden, hidden)),
            (f"We{layer}", (hidden, N_EDGE_IN)), (f"be{layer}", (hidden,)),
            (f"W2{layer}", (hidden, hidden)), (f"b2{layer}", (hidden,)),
            (f"Wn1{layer}", (hidden, 2 * hidden)), (f"bn1{layer}", (hidden,)),
            (f"Wn2{layer}", (hidden, hidden)), (f"bn2{layer}", (hidden,)),
        ])
    blocks.extend([("Wd", (N_OUT, hidden)), ("bd", (N_OUT,))])
    return blocks


def n_params(hidden=HIDDEN, layers=LAYERS):
    return int(sum(np.prod(shape) for _, shape in param_shapes(hidden, layers)))


def flatten(blocks, hidden=HIDDEN, layers=LAYERS, dtype=np.float32):
    """dict of blocks -> flat vector in the device order."""
    return np.concatenate([np.asarray(blocks[name], dtype=dtype).reshape(-1)
                           for name, _ in param_shapes(hidden, layers)])


def unflatten(flat, hidden=HIDDEN, layers=LAYERS):
    """flat vector -> dict of blocks (float64 copies)."""
    out, pos = {}, 0
    for name, shape in param_shapes(hidden, layers):
        size = int(np.prod(shape))
        out[name] = np.asarray(flat[pos:pos + size], dtype=np.float64).reshape(shape)
        pos += size
    return out


def initial_params(seed=0, hidden=HIDDEN, layers=LAYERS):
    """Glorot-uniform matrices and zero biases, drawn block by block in layout
    order from numpy's default_rng(seed); the residual branch (Wn*2) and the
    decoder start ten times smaller, so the untrained network is close to the
    method without it.  Returns the flat float32 vector."""
    rng = np.random.default_rng(seed)
    blocks = {}
    for name, shape in param_shapes(hidden, layers):
        if len(shape) == 1:
            blocks[name] = np.zeros(shape)
            continue
        bound = np.sqrt(6.0 / (shape[0] + shape[1]))
        if name == "Wd" or name.startswith("Wn2"):
            bound = 0.1 * bound
        blocks[name] = rng.uniform(-bound, bound, size=shape)
    return flatten(blocks, hidden, layers)
