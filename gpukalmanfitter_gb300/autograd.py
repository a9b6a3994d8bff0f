"""torch.autograd wrapper of the chi2 adjoint, for gradient checks only.

``Chi2.apply(start, alignment, field_scale, batch)`` returns the total
smoothed chi2 of an :class:`~gpukalmanfitter_gb300.AdjointBatch` as a 0-d
FP64 tensor.  Its backward calls kf_adjoint_batch with the gradient on: the
start-parameter gradient per track, the alignment gradient (converted from
incremental global rotations to the Rx Ry Rz angles at the given alignment)
and the field-scale gradient.  The forward and backward both run on the GPU;
nothing here is on the fit's hot path.
"""
from __future__ import annotations

import numpy as np
import torch

from . import rotation_increment_jacobian


class Chi2(torch.autograd.Function):
    @staticmethod
    def forward(ctx, start: torch.Tensor, alignment: torch.Tensor, field_scale: torch.Tensor,
                batch) -> torch.Tensor:
        batch.set_start(start.detach().cpu().numpy())
        a = alignment.detach().cpu().numpy().astype(np.float64)
        fs = float(field_scale.detach().cpu())
        r = batch.run(grad=False, alignment=a, field_scale=fs)
        ctx.batch, ctx.a, ctx.fs = batch, a, fs
        ctx.start = start.detach().cpu().numpy()
        return torch.tensor(float(r["chi2"][r["status"] == 0].sum()), dtype=torch.float64)

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        batch = ctx.batch
        batch.set_start(ctx.start)
        r = batch.run(grad=True, alignment=ctx.a, field_scale=ctx.fs)
        ga = r["grad_align"].copy()
        for k in range(ga.shape[0]):
            ga[k, 3:] = rotation_increment_jacobian(ctx.a[k, 3:]).T @ ga[k, 3:]
        gs = float(g)
        return (torch.from_numpy(r["grad_start"] * gs), torch.from_numpy(ga * gs),
                torch.tensor(float(r["grad_field_scale"][0]) * gs, dtype=torch.float64), None)
