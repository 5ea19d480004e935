"""Optional PyTorch autograd binding of the forward map and its adjoint kernel.

    p, logj, ok = phase_space(ps, x)          # ps: api.PhaseSpace (FP64), x: [n, n_x] CUDA
    loss = (w * p).sum() + logj.sum()
    loss.backward()                           # x.grad from the hand-written adjoint kernel

``theta`` (optional, [n_out - 2, 2]) stands for the (mass, width) of the Breit-Wigner branch
at each msq x index, as phs.mapping_parameters() returns it; its gradient is the adjoint's
thbar summed over events.  The forward map uses the masses and widths the process was built
with, so theta must hold those values.
"""
from __future__ import annotations

import numpy as np
import torch


def mapping_parameters(ps) -> torch.Tensor:
    """(m, Gamma) per msq x index of channel 0 (zeros where the branch is not Breit-Wigner)."""
    proc = ps.proc
    R = (1 << proc.n_out) - 1
    d1, d2, hc = proc.d1[0], proc.d2[0], proc.has_children[0]
    out = np.zeros((max(1, proc.n_out - 2), 2))
    order = []

    def post(code):
        if not hc[code - 1]:
            return
        post(int(d1[code - 1]))
        post(int(d2[code - 1]))
        if code != R:
            order.append(code)

    post(R)
    for k, code in enumerate(order):
        if proc.map_ids[0, code - 1] == 1:
            out[k] = (proc.map_masses[0, code - 1], proc.map_widths[0, code - 1])
    return torch.tensor(out, dtype=torch.float64)


class _PhaseSpace(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, theta, ps, counts):
        ev = ps.generate(x, counts)
        ok = ev.ok.bool()
        logj = torch.where(ok, torch.log(torch.where(ok, ev.factor, torch.ones_like(ev.factor))),
                           torch.zeros_like(ev.factor))
        ctx.save_for_backward(x)
        ctx.ps, ctx.counts = ps, counts
        ctx.mark_non_differentiable(ev.ok)
        return ev.p, logj, ev.ok

    @staticmethod
    def backward(ctx, pbar, jbar, _okbar):
        (x,) = ctx.saved_tensors
        if pbar is None:
            pbar = torch.zeros((x.shape[0], ctx.ps.proc.n_out, 4), dtype=x.dtype, device=x.device)
        xbar, thbar = ctx.ps.vjp(x, pbar, jbar, ctx.counts)
        return xbar, thbar.sum(0).to(torch.float64).cpu(), None, None


def phase_space(ps, x, theta=None, counts=None):
    """Differentiable forward map: returns (momenta [n, n_out, 4], log(factor) [n], ok [n])."""
    if theta is None:
        theta = mapping_parameters(ps)
    return _PhaseSpace.apply(x, theta, ps, counts)
