"""The learned surrogate: a graph network that advances the SPH state k steps
at a time, trained on trajectories of the plain solver, with the plain step
as fallback.

Device memory comes from torch (allocation only); every computation is a
kernel of the library: the particle graph (tsph_export_graph), the network's
forward / backward / Adam (tsph_gnn_*), the state update (tsph_apply_update)
and the plain SPH step.  The network's definition is in
oracle/gnn_oracle.py's docstring (the oracle the device kernels are checked
against).
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import sph

K_SLOTS = 48  # neighbour slots per node (the SPH pair set has ~24-36)


class GraphBuffers:
    """Device arrays of one exported particle graph (capacity `cap` nodes)."""

    def __init__(self, cap, device="cuda"):
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
        self.n = 0
        self.nw = 0

    def export(self, system):
        """tsph_export_graph of `system`'s current state into these buffers."""
        self.n, self.nw = system.export_graph(
            K_SLOTS, self.cap, self.pos.data_ptr(), self.vel.data_ptr(), self.srho.data_ptr(),
            self.wall.data_ptr(), self.id.data_ptr(), self.deg.data_ptr(), self.nbr.data_ptr())
        return self

    def clone(self):
        """A copy holding only the exported nodes (for a training set)."""
        c = GraphBuffers.__new__(GraphBuffers)
        n = self.n
        c.cap = n
        for f in ("pos", "vel", "srho", "wall", "id", "deg", "nbr"):
            setattr(c, f, getattr(self, f)[:n].clone())
        c.n, c.nw = n, self.nw
        return c

    def struct(self, h, u_scale, s_scale, origin=(0.0, 0.0)):
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
        g.origin = (C.c_double * 2)(*origin)
        return g

    def host(self):
        """numpy copies (for the oracle)."""
        n = self.n
        return dict(pos=self.pos[:n].cpu().numpy(), vel=self.vel[:n].cpu().numpy().astype(np.float64),
                    srho=self.srho[:n].cpu().numpy().astype(np.float64),
                    wall=self.wall[:n].cpu().numpy().astype(np.float64),
                    id=self.id[:n].cpu().numpy(), deg=self.deg[:n].cpu().numpy(),
                    nbr=self.nbr[:n].cpu().numpy())
