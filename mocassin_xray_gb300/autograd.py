"""Forbidden-line luminosities as a differentiable function of the cells'
hydrogen densities (and, for the gradient, of chosen elemental abundances)
for PyTorch, at a frozen radiation field.

Forward: the context's balance from a saved starting state (its slot), with
the given densities, converged tightly, then outputGas's volume sums of the
lines (source/output_mod.f90:393-432); backward: the frozen-field
derivatives dL/dHden and dL/d(elemAbun) formed in the same call, contracted
with the incoming gradient.  They come from the implicit-function adjoint of
the converged balance (mcx_adjoint, method "adjoint") or from perturbed
balances (mcx_line_sensitivities, method "differences").  "Frozen field"
means J is held at the context's: the dependence of J on the densities (the
transport's response) is not in these gradients.
"""
from __future__ import annotations

import numpy as np
import torch

from . import abi


class FrozenFieldLines(torch.autograd.Function):
    """L = f(hden, abun): hden [nCells+1] (entry 0 unused), abun [len(abun_z)]
    the abundances of the elements abun_z as they stand in the context (the
    forward evaluates at the context's abundances; abun carries their
    gradient)."""

    @staticmethod
    def forward(fctx, hden, abun, context, slot, lines, abun_z, h, precision, method):
        context.state_restore(slot)
        context.put(abi.ARR_HDEN, hden.detach().cpu().numpy().astype(np.float32))
        if method == "adjoint":
            r = context.adjoint(lines, abun_z=abun_z, h=h, precision=precision, per_cell=True)
        elif method == "differences":
            r = context.line_sensitivities(lines, abun_z=abun_z, h=h, precision=precision, per_cell=True)
        else:
            raise ValueError(f"unknown method {method!r}")
        fctx.save_for_backward(torch.from_numpy(r["dL_dhden"]), torch.from_numpy(r["dL_dabun"]))
        return torch.from_numpy(r["L"]).to(hden.dtype)

    @staticmethod
    def backward(fctx, grad_L):
        d_hden, d_abun = fctx.saved_tensors
        g = grad_L.detach().to(torch.float64).cpu()
        grad_hden = (g @ d_hden).to(grad_L.dtype)
        grad_abun = (g @ d_abun).to(grad_L.dtype) if d_abun.numel() else None
        return grad_hden, grad_abun, None, None, None, None, None, None, None


def frozen_field_lines(context, hden: torch.Tensor, lines, abun: torch.Tensor | None = None, abun_z=(),
                       slot: int = 0, h: float = 1e-3, precision: int = abi.BAL_MIXED,
                       method: str = "adjoint") -> torch.Tensor:
    """Line luminosities [len(lines)] of the forbidden lines `lines`
    [(elem, ion, lower, upper), ...] for the densities `hden`, differentiable
    with respect to hden and (when given) abun, the abundances of the
    elements abun_z.  `slot` holds the state the balance starts from (saved
    with Context.state_save before the first call).  method: "adjoint" (the
    implicit-function adjoint of the converged balance) or "differences"
    (perturbed balances)."""
    if abun is None:
        abun = torch.zeros(0, dtype=hden.dtype)
    return FrozenFieldLines.apply(hden, abun, context, slot, list(lines), tuple(abun_z), h, precision, method)
