"""Discrete adjoint of the Rayleigh-Benard time step: gradients of horizon objectives.

The plain step (``NavierStokes.update``) is differentiable end to end: every
device operator it calls records itself with its transposed kernel
(``pypde_gb300.autodiff``), and the convection products are torch pointwise
products.  This module strings steps into a horizon, recomputes the forward
states segment by segment in the backward pass (``torch.utils.checkpoint``, so
only one state per segment is kept), and defines the steady-state residual
objective

    J(X) = || Phi^H(X) - X ||_2 ,   X = (T, U, V) Galerkin coefficients,

with the pressure starting from zero at the beginning of the horizon.  pypde
has no such objective: its navier/rbc2d_adj.py descends along a continuous
adjoint of the one-step residual (reproduced in ``rbc2d_adj``); this is the
exact gradient of the discrete map, checked against central finite
differences.
"""
import numpy as np
import torch
from torch.utils.checkpoint import checkpoint

STATE = ("T", "U", "V", "pres")


def get_state(ns):
    return tuple(getattr(ns, k).vhat for k in STATE)


def set_state(ns, X):
    for k, x in zip(STATE, X):
        getattr(ns, k).vhat = x


def step(ns, X):
    """One time step X -> Phi(X) on the plain path; differentiable in X."""
    set_state(ns, X)
    ns.update()
    return get_state(ns)


def horizon(ns, X, nsteps, every=20):
    """Phi^nsteps(X); while autograd records, forward states inside each segment of
    ``every`` steps are recomputed in backward instead of being kept."""
    X = tuple(X)

    def segment(k, *Y):
        for _ in range(k):
            Y = step(ns, Y)
        return Y

    done = 0
    while done < nsteps:
        k = min(every, nsteps - done)
        if torch.is_grad_enabled() and any(x.requires_grad for x in X):
            X = checkpoint(segment, k, *X, use_reentrant=False, preserve_rng_state=False)
        else:
            X = segment(k, *X)
        done += k
    return X


class ResidualObjective:
    """J(X) = ||Phi^H(X) - X|| over (T, U, V), pressure zero at the start."""

    def __init__(self, ns, nsteps, every=20):
        self.ns, self.nsteps, self.every = ns, nsteps, every

    def _J(self, X3):
        pres0 = torch.zeros_like(self.ns.pres.vhat)
        Y = horizon(self.ns, (*X3, pres0), self.nsteps, self.every)
        r2 = sum(((y - x) ** 2).sum() for y, x in zip(Y[:3], X3))
        return torch.sqrt(r2)

    def __call__(self, X3):
        with torch.no_grad():
            return float(self._J(tuple(x.detach() for x in X3)))

    def value_and_grad(self, X3):
        X3 = tuple(x.detach().clone().requires_grad_(True) for x in X3)
        with torch.enable_grad():
            J = self._J(X3)
            g = torch.autograd.grad(J, X3)
        return float(J.detach()), tuple(x.detach() for x in g)


def random_directions(shapes, count, seed, device):
    """Unit directions in the joint (T, U, V) coefficient space (numpy default_rng(seed))."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        d = [rng.standard_normal(s) for s in shapes]
        nrm = np.sqrt(sum(float((x ** 2).sum()) for x in d))
        out.append(tuple(torch.as_tensor(x / nrm, device=device) for x in d))
    return out


def fd_check(obj, X3, directions, h=1e-6):
    """Central differences (J(X+hd)-J(X-hd))/2h against <grad J, d> for each direction.

    Returns (J, [(fd, adjoint, relative error), ...])."""
    J, g = obj.value_and_grad(X3)
    rows = []
    for d in directions:
        jp = obj(tuple(x + h * e for x, e in zip(X3, d)))
        jm = obj(tuple(x - h * e for x, e in zip(X3, d)))
        fd = (jp - jm) / (2 * h)
        ad = float(sum((gi * e).sum() for gi, e in zip(g, d)))
        rows.append((fd, ad, abs(fd - ad) / max(abs(ad), 1e-300)))
    return J, rows


def _as_tuple(X):
    return tuple(X) if isinstance(X, (tuple, list)) else (X,)


def descend(value_and_grad, X, iters, alpha=0.5, callback=None):
    """Steady-state search: gradient descent on J with the step alpha J / |grad J|^2 (the step that
    would zero a linear J), enlarged after an accepted step and halved after a rejected one.

    ``value_and_grad(X) -> (J, grad)`` with X a tensor or a tuple of tensors (J a scalar or a
    one-element tensor).  Returns (X, [J of every accepted iterate])."""
    single = not isinstance(X, (tuple, list))
    X = tuple(x.detach().clone() for x in _as_tuple(X))

    def vg(Y):
        J, g = value_and_grad(Y[0] if single else Y)
        return float(J if not torch.is_tensor(J) else J.reshape(-1)[0]), _as_tuple(g)

    J, g = vg(X)
    hist = [J]
    for it in range(iters):
        gn2 = sum(float((gi * gi).sum()) for gi in g)
        if gn2 == 0.0 or J == 0.0:
            break
        t = alpha * J / gn2
        Xn = tuple(x - t * gi for x, gi in zip(X, g))
        Jn, gn = vg(Xn)
        if Jn < J:
            X, J, g = Xn, Jn, gn
            alpha = min(1.0, 1.5 * alpha)
            hist.append(J)
        else:
            alpha *= 0.5
        if callback is not None:
            callback(it, J)
    return (X[0] if single else X), hist
