"""Reverse-mode differentiation of the device primitives.

Every operator on the time-step path is linear in its tensor argument: the
DCT along an axis, the derivative recurrence, the Galerkin stencils and their
least-squares inverse, banded / dense operators and the banded and Poisson
solves.  The only nonlinearity of a step is the pointwise product of the
convection terms, which torch differentiates by itself.  So one
``torch.autograd.Function`` covers the whole path: it runs a forward kernel and,
in backward, the hand-written transposed kernel of the same operator
(pgx_dct1 modes FWD_T/BWD_T, pgx_cheb_diff_t, pgx_stencil_transpose,
pgx_stencil_from_chebyshev_t, pgx_fdma_solve_t, pgx_poisson_solve_t, transposed
matrix plans).  The backward of the backward is the forward operator again, so
double backward (Hessian-vector products) works as well.
"""
import torch


def _sane(g):
    """Gradients may arrive as broadcast views (stride 0): give the kernels real memory."""
    if g.dim() and (min(g.stride()) == 0 or not g.is_cuda):
        return g.contiguous()
    return g


class LinearMap(torch.autograd.Function):
    """y = A x for a device linear operator A, with x_bar = A^T y_bar in backward."""

    @staticmethod
    def forward(ctx, x, op, op_t):
        # (not ctx.apply: that name is the autograd node's own entry point)
        ctx.op, ctx.op_t = op, op_t
        return op(x)

    @staticmethod
    def backward(ctx, g):
        return linear(_sane(g), ctx.op_t, ctx.op), None, None


def recording(x):
    return torch.is_grad_enabled() and isinstance(x, torch.Tensor) and x.requires_grad


def linear(x, apply, apply_t):
    """apply(x), recorded for autograd (with apply_t as its transpose) when x needs a gradient."""
    if recording(x):
        return LinearMap.apply(x, apply, apply_t)
    return apply(x)
