"""torch.autograd binding of the pair adjoint over the C ABI (gain_adjoint_pair_prec).

The adjoint itself lives behind the C ABI; this module only lets torch drive it, so that the
gradient dL/d(dipole_me) of a loss over line strengths can be checked against central
differences and torch.autograd.gradcheck.  It is test and check tooling: the production
callers are C/C++ (a dipole-surface refinement step calls gain_adjoint_pair_prec directly).

    mu = torch.tensor(piece, dtype=torch.float64, requires_grad=True)   # [3][N][ncontrF]
    S = line_strengths(mu, eng, (jindI, gammaI, jindF, gammaF), lower, upper, block=(0, N))
    loss = ((S.log() - S_target.log()) ** 2).sum()
    loss.backward()                                                   # mu.grad = dL/dmu

Forward: the dipole piece is uploaded and the pair runs through the engine (the plain FP64
path or the split tensor-core path), S = amp^2.  Backward: the piece is uploaded again and
the engine's adjoint recomputes the pair's FP64 forward (half line strengths and amplitudes;
nothing per transition is kept from the forward) and chains dL/dS into dL/dmu.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np
import torch

import gainls


class PairLineStrengths(torch.autograd.Function):
    @staticmethod
    def forward(ctx, mu, eng, pair, lower, upper, block, path, precision):
        nv = int(mu.shape[1])
        s, e = block
        piece = np.ascontiguousarray(mu.detach().cpu().numpy(), np.float64).reshape(-1)
        eng.upload_dipole(piece, nv, s, e, e - s)
        eng.run_pair(*pair, list(lower), list(upper), path)
        amp = eng.fetch_amp().copy()
        ctx.eng, ctx.pair, ctx.lower, ctx.upper = eng, pair, list(lower), list(upper)
        ctx.block, ctx.precision, ctx.nv = block, precision, nv
        ctx.save_for_backward(mu.detach())
        return torch.from_numpy(amp * amp)

    @staticmethod
    def backward(ctx, grad_S):
        (mu,) = ctx.saved_tensors
        s, e = ctx.block
        piece = np.ascontiguousarray(mu.cpu().numpy(), np.float64).reshape(-1)
        ctx.eng.upload_dipole(piece, ctx.nv, s, e, e - s)   # the adjoint's own FP64 forward
        g = np.zeros(piece.size, np.float64)
        ctx.eng.adjoint(*ctx.pair, ctx.lower, ctx.upper, np.ascontiguousarray(grad_S.detach().cpu().numpy()), g,
                        precision=ctx.precision)
        return torch.from_numpy(g).view_as(mu), None, None, None, None, None, None, None


def line_strengths(mu: torch.Tensor, eng, pair: Sequence[int], lower: Sequence[int], upper: Sequence[int],
                   block=None, path: int = gainls.PATH_PLAIN_FP64, precision: str = "f64") -> torch.Tensor:
    """S[l, u] = amp^2 of one block pair as a differentiable function of the dipole piece mu
    (float64, [3][N][endF - startF], the gain_upload_dipole layout; block = (startF, endF),
    default the whole range).  precision ("f64", "f32" or "split": tensor-core digit GEMMs) is
    the arithmetic of the adjoint."""
    if block is None:
        block = (0, int(mu.shape[1]))
    return PairLineStrengths.apply(mu, eng, tuple(pair), tuple(lower), tuple(upper), tuple(block), path, precision)
