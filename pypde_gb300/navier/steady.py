"""Steady states of the Rayleigh-Benard step by Newton-Krylov (navier/rbc2d_base.py:260-341).

pypde's ``NavierStokesSteadyState.solve_steady_state`` hands the residual

    F(X) = (Phi_dt(X) - X) / dt,   X = (T, U, V) Galerkin coefficients,

(one ``update()``, or ``iterate(dt)`` for a longer horizon) to SciPy's
``optimize.root(method="krylov")``: inexact Newton with an LGMRES inner solver
and finite-difference Jacobian-vector products.  Every evaluation also advances
the solver's pressure ``NS.pres``, so F depends on the evaluation history.

``solve_steady_state(method="reference")`` (the default) is exactly that: the
same SciPy call on the same residual, each evaluation one step of the GPU path
(the fused passes) with the pressure carried from evaluation to evaluation; it
returns SciPy's result, as the reference does.

``method="augmented"`` is this project's variant, written for the GPU:

- the two evaluations of a central-difference Jacobian-vector product,
  F(X + eps v) and F(X - eps v), are two instances of one fused batch, so each
  Krylov vector costs one batched launch sequence (for a one-step residual the
  map is quadratic in X and the central difference is exact up to rounding);
- restarted GMRES with modified Gram-Schmidt on float64 device vectors;
- Armijo backtracking on |F|.

The reference carries the pressure through its residual (every evaluation
advances ``NS.pres``), which makes F depend on the evaluation history (and
keeps SciPy's iteration from converging on the cases tried).  In the augmented
variant the pressure is an unknown of the Newton iteration next to (T, U, V), with the
residual (pres' - pres) / dt of the step's pressure update, so F is one
deterministic map and its zero is a fixed point of the complete step; the
returned ``x`` keeps the reference's (T, U, V) layout and the solver's
pressure field is left at the converged pressure.
"""
import numpy as np
import torch

from .fused import FusedBatch


class SteadyStateResult(dict):
    """x, success, status, message, nit, nfev, fun_norm (like scipy's OptimizeResult)."""

    __getattr__ = dict.__getitem__


class NavierStokesSteadyState:
    """Mixin for ``NavierStokes``: solve_steady_state, flatten, reshape, vectorify, get_masks, steady_fun."""

    # -- the reference's vector layout [T, U, V] (rbc2d_base.py:296-319)
    def flatten(self):
        return tuple(getattr(self, k).vhat.flatten().clone() for k in ("T", "U", "V"))

    def get_masks(self):
        t, u, v = (getattr(self, k).vhat.numel() for k in ("T", "U", "V"))
        return slice(0, t), slice(t, t + u), slice(t + u, t + u + v)

    def reshape(self, X):
        tm, um, vm = self.get_masks()
        return tuple(X[m].clone().reshape(getattr(self, k).vhat.shape) for m, k in zip((tm, um, vm), "TUV"))

    def vectorify(self):
        return torch.cat(self.flatten())

    def steady_fun(self, X, NS=None, dt=None):
        """(Phi(X) - X) / dt (rbc2d_base.py:321-341): one step, or the time loop over ``dt`` with the
        clock reset around it; advances NS's pressure, as the reference does."""
        NS = self if NS is None else NS
        NS.T.vhat, NS.U.vhat, NS.V.vhat = NS.reshape(X)
        if dt is None:
            dt = NS.dt
            NS.update()
        else:
            NS.reset_time()
            NS.iterate(dt, callback=False)
            NS.reset_time()
        return (NS.vectorify() - X) / dt

    def _solve_reference(self, X0, dt, maxiter, disp, tol, jac_options):
        """SciPy's Newton-Krylov on steady_fun with the reference's options (rbc2d_base.py:266-294);
        x travels between the host iteration and the device step once per evaluation."""
        from scipy import optimize
        options = {"maxiter": maxiter, "disp": disp, "fatol": tol, "jac_options": jac_options}
        x0 = self.vectorify() if X0 is None else X0
        x0 = x0.detach().cpu().numpy() if torch.is_tensor(x0) else np.asarray(x0, dtype=np.float64)
        dev = self.T.vhat.device

        def fun(x, NS, dt):
            return NS.steady_fun(torch.as_tensor(x, dtype=torch.float64, device=dev), NS, dt).cpu().numpy()

        if disp:
            print("\nSolve steady state ...\n")
        return optimize.root(fun, x0, args=(self, dt), method="krylov", options=options)

    # -- Newton-Krylov on the fused step
    def _pair(self):
        if getattr(self, "_steady_pair", None) is None:
            self._steady_pair = FusedBatch([self, self], bind=False)
            self._steady_pair.capture(1)
        return self._steady_pair

    def _residuals(self, Za, Zb, nsteps, dt):
        """F at two augmented points Z = (T, U, V, pres) in one batched evaluation."""
        fb = self._pair()
        tm, um, vm = self.get_masks()
        n3 = vm.stop
        outs = []
        for I, Z in zip(fb.insts, (Za, Zb)):
            A = I.arrays
            for key, m in (("TG", tm), ("UG", um), ("VG", vm)):
                A[key].copy_(Z[m].view(A[key].shape))
            A["PRES"].copy_(Z[n3:].view(A["PRES"].shape))
        for _ in range(nsteps):
            fb.step()
        for I, Z in zip(fb.insts, (Za, Zb)):
            A = I.arrays
            Y = torch.cat([A[k].flatten() for k in ("TG", "UG", "VG", "PRES")])
            outs.append((Y - Z) / dt)
        return outs

    def solve_steady_state(self, X0=None, dt=None, maxiter=300, disp=True, tol=1e-8,
                           jac_options={"inner_maxiter": 30}, method="reference"):  # noqa: B006
        """Newton-Krylov for F = 0 (rbc2d_base.py:266-294); ``tol`` bounds max|F| like scipy's fatol.

        ``method="reference"``: SciPy's iteration on the reference's residual (the pressure carried
        through the evaluations); returns SciPy's OptimizeResult.  ``method="augmented"``: the GPU
        Newton-Krylov with the pressure as an unknown (module docstring); returns a
        SteadyStateResult with x on the device."""
        if method == "reference":
            return self._solve_reference(X0, dt, maxiter, disp, tol, jac_options)
        if method != "augmented":
            raise ValueError("method must be 'reference' or 'augmented'")
        if self.nstage != 1:
            raise NotImplementedError("the fused residual covers IMEX Euler")
        nsteps = 1 if dt is None else int(round(dt / self.dt))
        dt = self.dt if dt is None else dt
        m = int(jac_options.get("inner_maxiter", 30))
        X = self.vectorify() if X0 is None else torch.as_tensor(X0, dtype=torch.float64, device="cuda")
        Z = torch.cat([X.clone(), self.pres.vhat.flatten().clone()])
        F, _ = self._residuals(Z, Z, nsteps, dt)
        nfev, nit, status = 1, 0, 1
        fnorm = float(F.abs().max())
        while fnorm > tol and nit < maxiter:
            nit += 1
            zs = max(1.0, float(Z.norm()))

            def jv(v):
                nv = float(v.norm())
                if nv == 0.0:
                    return torch.zeros_like(v)
                eps = 1e-7 * zs / nv
                fp, fm = self._residuals(Z + eps * v, Z - eps * v, nsteps, dt)
                return (fp - fm) / (2.0 * eps)

            s, evals = _gmres(jv, -F, m, rtol=min(1e-3, 0.5 * fnorm))
            nfev += 2 * evals
            # Armijo backtracking on |F|_2
            f2 = float(F.norm())
            lam = 1.0
            while True:
                Fn, _ = self._residuals(Z + lam * s, Z + lam * s, nsteps, dt)
                nfev += 1
                if float(Fn.norm()) <= (1.0 - 1e-4 * lam) * f2 or lam < 1e-4:
                    break
                lam *= 0.5
            Z, F = Z + lam * s, Fn
            fnorm = float(F.abs().max())
            if disp:
                print("%4d:  |F| = %.6e  step %.3g  (%d Krylov vectors)" % (nit, fnorm, lam, evals))
        if fnorm <= tol:
            status, msg = 0, "A solution was found at the specified tolerance."
        else:
            msg = "The maximum number of iterations allowed has been reached."
        n3 = self.get_masks()[2].stop
        X = Z[:n3].clone()
        self.T.vhat, self.U.vhat, self.V.vhat = self.reshape(X)
        self.pres.vhat = Z[n3:].view(self.pres.vhat.shape).clone()
        if getattr(self, "_fused", None) is not None:
            self._fused.insts[0].sync_in()
        return SteadyStateResult(x=X, success=status == 0, status=status, message=msg, nit=nit, nfev=nfev,
                                 fun_norm=fnorm)


def _gmres(A, b, m, rtol):
    """GMRES(m), one cycle from x0 = 0 with modified Gram-Schmidt; returns (x, matvecs)."""
    beta = float(b.norm())
    if beta == 0.0:
        return torch.zeros_like(b), 0
    V = [b / beta]
    H = np.zeros((m + 1, m))
    g = np.zeros(m + 1)
    g[0] = beta
    cs, sn = np.zeros(m), np.zeros(m)
    k = 0
    for k in range(m):
        w = A(V[k])
        for i in range(k + 1):
            H[i, k] = float((w * V[i]).sum())
            w = w - H[i, k] * V[i]
        H[k + 1, k] = float(w.norm())
        for i in range(k):  # apply the previous rotations to column k
            t = cs[i] * H[i, k] + sn[i] * H[i + 1, k]
            H[i + 1, k] = -sn[i] * H[i, k] + cs[i] * H[i + 1, k]
            H[i, k] = t
        r = np.hypot(H[k, k], H[k + 1, k])
        cs[k], sn[k] = (H[k, k] / r, H[k + 1, k] / r) if r > 0 else (1.0, 0.0)
        H[k, k], H[k + 1, k] = r, 0.0
        g[k + 1] = -sn[k] * g[k]
        g[k] = cs[k] * g[k]
        if abs(g[k + 1]) <= rtol * beta or float(w.norm()) == 0.0:
            break
        V.append(w / float(w.norm()) if float(w.norm()) > 0 else w)
    n = k + 1
    y = np.linalg.solve(np.triu(H[:n, :n]), g[:n])
    x = torch.zeros_like(b)
    for i in range(n):
        x = x + float(y[i]) * V[i]
    return x, n
