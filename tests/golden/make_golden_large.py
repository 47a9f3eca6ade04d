"""Golden signatures of the large plain Rayleigh-Benard run, from the unmodified pypde reference.

Workload: 513 x 257 Gauss-Lobatto points (x by y), aspect 2, Ra 1e8, Pr 1, dt 1e-3,
3/2 dealiasing, IMEX Euler, case "linear", T = conductive profile + 1e-3 U(-1,1)
noise with numpy default_rng(2); 1000 steps.

Run from the repository root in a container that has the reference checked out,
its location given by ``--reference`` or the PYPDE_REFERENCE variable:

    python tests/golden/make_golden_large.py [--reference PATH] [--steps 1000]

The full state at this size is 5 MB per snapshot, so ``golden_large.npz`` keeps a
signature of each field (T, U, V, P Galerkin coefficients and the Chebyshev
pressure) after 1, 10, 100 and 1000 steps: its low-mode block, a strided subsample
of every mode, its maximum magnitude and four seeded Gaussian projections
(``signature`` below; the GPU test computes the same numbers), plus Nu, Nuvol and
KE.  The file is rewritten after every snapshot, so an interrupted run still
leaves the earlier ones.
"""
import argparse
import contextlib
import io
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_shims  # noqa: E402

SHAPE, ASPECT, RA, DT, SEED, AMP = (513, 257), 2.0, 1e8, 1e-3, 2, 1e-3
SNAPSHOTS = (1, 10, 100, 1000)
FIELDS = ("T", "U", "V", "P", "pres")
LOW = (32, 16)       # low-mode block kept whole
STRIDE = (8, 8)      # subsample of every mode
NPROJ = 4            # seeded Gaussian projections per field


def signature(a, field):
    """Signature of one 2-D array (shared with the GPU test): low block, strided subsample,
    max |a|, and NPROJ projections on standard normal weights drawn from
    default_rng(1000 + index of the field) in the array's shape."""
    a = np.asarray(a, dtype=np.float64)
    w = np.random.default_rng(1000 + FIELDS.index(field)).standard_normal((NPROJ,) + a.shape)
    return {"low": a[:LOW[0], :LOW[1]].copy(), "sub": a[::STRIDE[0], ::STRIDE[1]].copy(),
            "max": np.array([np.max(np.abs(a))]), "proj": np.einsum("kij,ij->k", w, a)}


def quiet(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=ref_shims.REFERENCE)
    ap.add_argument("--steps", type=int, default=SNAPSHOTS[-1])
    args = ap.parse_args()
    ref_shims.install(args.reference)
    from pypde import field_operations as fo
    from navier import rbc2d as R

    ns = quiet(R.NavierStokes, case="linear", shape=SHAPE, ra=RA, pr=1.0, dt=DT, aspect=ASPECT, dealias=True,
               integrator="eu", beta=1.0, tsave=None)
    ns.T.v = AMP * np.random.default_rng(SEED).uniform(-1, 1, SHAPE)
    ns.T.forward()
    G = {"c3_s0_T_" + k: v for k, v in signature(ns.T.vhat, "T").items()}
    out = os.path.join(HERE, "golden_large.npz")
    t0 = time.time()
    for step in range(1, args.steps + 1):
        ns.update()
        if step not in SNAPSHOTS:
            continue
        arrays = {"T": ns.T.vhat, "U": ns.U.vhat, "V": ns.V.vhat, "P": ns.P.vhat, "pres": ns.pres.vhat}
        for f in FIELDS:
            for k, v in signature(arrays[f], f).items():
                G["c3_s%d_%s_%s" % (step, f, k)] = v
        nu, nuv = quiet(ns.eval_Nu)
        ns.U.backward()
        ns.V.backward()
        ke = 0.5 * fo.avg_vol(ns.U.v ** 2 + ns.V.v ** 2, ns.deriv_field.dx, ns.deriv_field.dy)
        G["c3_s%d_scalars" % step] = np.array([nu, nuv, ke])
        np.savez_compressed(out, **{k: np.asarray(v, dtype=np.float64) for k, v in G.items()})
        print("step %d (%.0f s): Nu %.12f Nuvol %.12f KE %.6e" % (step, time.time() - t0, nu, nuv, ke), flush=True)
    print("wrote", out, os.path.getsize(out) // 1024, "KiB,", len(G), "arrays")


if __name__ == "__main__":
    main()
