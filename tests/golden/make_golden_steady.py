"""Golden vectors of the reference's steady-state search (navier/rbc2d_base.py:260-341).

Run from the repository root in a container that has the reference checked out,
its location given by ``--reference`` or the PYPDE_REFERENCE variable:

    python tests/golden/make_golden_steady.py [--reference PATH]

Case: 17 x 17, Ra 5e3, Pr 1, dt 0.05, 3/2 dealiasing, IMEX Euler, T = conductive
profile + 0.1 U(-1,1) noise (numpy default_rng(1)), 100 steps; that state (T, U, V,
pres) is the start of everything below, so nothing depends on how it was reached.

* ``steady_fun`` evaluated on a fixed sequence of four points (the start, two seeded
  perturbations of it, the start again): the step's output and the pressure after
  every evaluation -- the reference's residual advances ``NS.pres`` each time, so
  the sequence pins those semantics.
* ``solve_steady_state(maxiter=k)`` for k = 1 and 5 from the start: the iterate and
  the pressure.  The reference's solver does not converge on this case (nor on the
  others tried) because its residual depends on the evaluation history; a 1e-14
  relative change of the start moves its iterate by about 1e-8 after 1-3 iterations
  and 6e-8 after 5, so the first iterations are what a rounding-level parity check
  can compare.
"""
import argparse
import contextlib
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_shims  # noqa: E402

SHAPE, RA, DT, SEED, AMP, PRESTEPS = (17, 17), 5e3, 0.05, 1, 1e-1, 100
CFG = dict(case="linear", shape=SHAPE, ra=RA, pr=1.0, dt=DT, dealias=True, integrator="eu", beta=1.0, tsave=None)


def perturbations(n):
    """The two seeded directions of the residual sequence (shared with the GPU test)."""
    rng = np.random.default_rng(44)
    return 1e-3 * rng.uniform(-1, 1, n), 1e-3 * rng.uniform(-1, 1, n)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=ref_shims.REFERENCE)
    args = ap.parse_args()
    ref_shims.install(args.reference)
    from navier import rbc2d as R

    def fresh():
        with contextlib.redirect_stdout(io.StringIO()):
            return R.NavierStokes(**CFG)

    ns = fresh()
    ns.T.v = AMP * np.random.default_rng(SEED).uniform(-1, 1, SHAPE)
    ns.T.forward()
    for _ in range(PRESTEPS):
        ns.update()
    G = {"start_T": ns.T.vhat.copy(), "start_U": ns.U.vhat.copy(), "start_V": ns.V.vhat.copy(),
         "start_pres": ns.pres.vhat.copy()}
    X0 = ns.vectorify()

    def restart():
        s = fresh()
        s.T.vhat[:], s.U.vhat[:], s.V.vhat[:] = G["start_T"], G["start_U"], G["start_V"]
        s.pres.vhat[:] = G["start_pres"]
        return s

    s = restart()
    d1, d2 = perturbations(X0.size)
    for k, X in enumerate((X0, X0 + d1, X0 - d2, X0)):
        F = s.steady_fun(X.copy(), s, None)
        G["seq%d_Y" % k] = X + DT * F
        G["seq%d_pres" % k] = s.pres.vhat.copy()
    for iters in (1, 5):
        s = restart()
        with contextlib.redirect_stdout(io.StringIO()):
            sol = s.solve_steady_state(X0=X0.copy(), tol=1e-8, maxiter=iters, disp=False)
        G["nk%d_x" % iters] = np.asarray(sol.x)
        G["nk%d_pres" % iters] = s.pres.vhat.copy()
        print("maxiter %d: |F| %.3e" % (iters, np.abs(np.asarray(sol.fun)).max()))
    out = os.path.join(HERE, "golden_steady.npz")
    np.savez_compressed(out, **{k: np.asarray(v, dtype=np.float64) for k, v in G.items()})
    print("wrote", out, os.path.getsize(out) // 1024, "KiB,", len(G), "arrays")


if __name__ == "__main__":
    main()
