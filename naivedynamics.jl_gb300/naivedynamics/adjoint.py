"""Differentiable trajectories (nd_adj_*): a kick-drift-kick run of the engine,
the Gaussian-smoothed pair-distance histogram of its final positions, the
squared deviation from a target histogram, and the hand-written adjoint of
that program -- gradients with respect to the initial positions and
velocities and to the Lennard-Jones sigma and epsilon.

The reference (NaiveDynamics.jl) has no derivative code; a Julia caller would
put these calls behind a ChainRulesCore.rrule, a Python caller behind the
torch.autograd.Function below.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import AdjSpec, MDParams, ptr
from .dynamics import _f64


def adj_spec(steps: int, checkpoint_every: int = 50, bins: int = 64, r_max: float = 2.5,
             width: float = 0.0, r_switch: float = -1.0) -> AdjSpec:
    """nd_adj_spec: `steps` MD steps, checkpoints every `checkpoint_every`,
    `bins` histogram bins on [0, r_max], Gaussian width (0 = bin width),
    pair-weight switch from r_switch to r_max (< 0: r_max - 0.25)."""
    s = AdjSpec()
    s.steps, s.checkpoint_every, s.bins = int(steps), int(checkpoint_every), int(bins)
    s.r_max, s.width, s.r_switch = float(r_max), float(width), float(r_switch)
    return s


class Adjoint:
    """One differentiable trajectory on the GPU.

    forward() -> (loss, hist); backward() -> dict(x0, v0, sigma, epsilon) of
    dL/d(.), valid after a forward pass of the current settings."""

    def __init__(self, params: MDParams, spec: AdjSpec, x0, v0, q=None, m=None, ctx=None):
        from ._lib import default_context
        self.ctx = ctx or default_context()
        x0 = _f64(x0, (-1, 3))
        v0 = _f64(v0, (-1, 3))
        self.n = x0.shape[0]
        self.bins = spec.bins
        self.params = params
        qq = None if q is None else _f64(q)
        mm = None if m is None else _f64(m)
        h = ctypes.c_void_p()
        st = _lib.lib().nd_adj_create(self.ctx.handle, ctypes.byref(params), self.n, ptr(x0),
                                      ptr(v0), ptr(qq), ptr(mm), ctypes.byref(spec),
                                      ctypes.byref(h))
        self.ctx.check(st, "nd_adj_create")
        self.handle = h.value

    def close(self):
        if getattr(self, "handle", None):
            _lib.lib().nd_adj_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, sigma: float, epsilon: float):
        self.ctx.check(_lib.lib().nd_adj_set_params(self.handle, float(sigma), float(epsilon)),
                       "nd_adj_set_params")

    def set_target(self, target):
        t = None if target is None else _f64(target)
        if t is not None and t.shape[0] != self.bins:
            raise ValueError(f"target needs {self.bins} bins")
        self.ctx.check(_lib.lib().nd_adj_set_target(self.handle, ptr(t)), "nd_adj_set_target")

    def forward(self):
        hist = np.empty(self.bins, np.float64)
        loss = ctypes.c_double()
        self.ctx.check(_lib.lib().nd_adj_forward(self.handle, ptr(hist), ctypes.byref(loss)),
                       "nd_adj_forward")
        return loss.value, hist

    def backward(self):
        dx = np.empty((self.n, 3), np.float64)
        dv = np.empty((self.n, 3), np.float64)
        ds, de = ctypes.c_double(), ctypes.c_double()
        self.ctx.check(_lib.lib().nd_adj_backward(self.handle, ptr(dx), ptr(dv), ctypes.byref(ds),
                                                  ctypes.byref(de)), "nd_adj_backward")
        return dict(x0=dx, v0=dv, sigma=ds.value, epsilon=de.value)

    def final_positions(self):
        x = np.empty((self.n, 3), np.float64)
        self.ctx.check(_lib.lib().nd_adj_final(self.handle, ptr(x)), "nd_adj_final")
        return x

    def times(self):
        """Device ms of the last forward and backward passes."""
        f, b = ctypes.c_float(), ctypes.c_float()
        self.ctx.check(_lib.lib().nd_adj_times(self.handle, ctypes.byref(f), ctypes.byref(b)),
                       "nd_adj_times")
        return f.value, b.value


def histogram_loss_function():
    """torch.autograd.Function over an Adjoint: apply(adj, sigma, epsilon) with
    0-d float64 tensors returns the loss; backward fills dL/dsigma, dL/depsilon
    (the initial-state gradients are on adj.last_grad)."""
    import torch

    class HistogramLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, adj, sigma, epsilon):
            adj.set_params(float(sigma), float(epsilon))
            loss, _ = adj.forward()
            ctx.adj = adj
            return torch.tensor(loss, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            g = ctx.adj.backward()
            ctx.adj.last_grad = g
            s = float(gout)
            return (None, torch.tensor(s * g["sigma"], dtype=torch.float64),
                    torch.tensor(s * g["epsilon"], dtype=torch.float64))

    return HistogramLoss
