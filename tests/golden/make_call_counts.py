"""Record which native kernels the pypde reference calls in one Rayleigh-Benard time step.

Run from the repository root in a container that has the reference checked out,
its location given by ``--reference`` or the PYPDE_REFERENCE variable:

    python tests/golden/make_call_counts.py [--reference PATH]

With ``ref_shims`` installed (as for ``make_golden.py``) it wraps the reference's
native call sites -- ``scipy.fftpack.dctn`` as bound in pypde/bases/chebyshev.py:15
and the f2py modules differentiate_cheby, tdma, twodma and fdma -- runs one warm-up
step and then counts the calls of one ``update()`` by kernel family, transform length
and number of lines.  ``call_counts.json`` holds the result; the oracle's own calls
are checked against it on the CPU: the oracle makes the same native-kernel calls as
the reference, on the same sizes, call for call.
"""
import argparse
import collections
import contextlib
import io
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_shims  # noqa: E402

CASES = [  # tag, case, shape, options (the C1 configuration first)
    ("c1_linear65", "linear", (65, 65), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu")),
    ("linear33x17_nd_aspect2", "linear", (33, 17), dict(ra=3e4, dt=0.01, dealias=False, integrator="eu", aspect=2.0)),
    ("rbc33", "rbc", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu")),
    ("zero33", "zero", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu")),
    ("rk3_33", "linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="rk3")),
    ("beta33", "linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu", beta=0.5)),
]


def _lines(shape, n):
    return int(np.prod(shape)) // n if n else 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=ref_shims.REFERENCE)
    args = ap.parse_args()
    ref_shims.install(args.reference)
    import pypde.bases.chebyshev as cheb
    from navier import rbc2d as R

    counts = collections.Counter()

    def count(family, n, lines):
        counts[(family, int(n), int(lines))] += 1

    def dctn(f, type=1, axes=(0,)):  # noqa: A002
        for ax in axes:
            count("dct", f.shape[ax], _lines(f.shape, f.shape[ax]))
        return dctn0(f, type=type, axes=axes)
    dctn0 = cheb.dctn_scipy
    cheb.dctn_scipy = dctn

    def wrap(modname, fname, shape_of):
        mod = sys.modules[modname]
        f0 = getattr(mod, fname)

        def f(*a, **k):
            fam, n, lines = shape_of(*a, **k)
            count(fam, n, lines)
            return f0(*a, **k)
        setattr(mod, fname, f)

    D, T, W, F = ("pypde.bases.fortran.differentiate_cheby", "pypde.bases.linalg.fortran.tdma",
                  "pypde.solver.linalg.fortran.twodma", "pypde.solver.linalg.fortran.fdma")
    wrap(D, "diff_1d", lambda c: ("diff", len(c), 1))
    wrap(D, "diff_2d", lambda c: ("diff", c.shape[0], c.shape[1]))
    wrap(T, "solve_tdma_1d", lambda a, b, c, d, k: ("tdma", len(b), 1))
    wrap(T, "solve_tdma_2d", lambda a, b, c, d, k: ("tdma", len(b), _lines(d.shape, len(b))))
    wrap(W, "solve_twodma_1d", lambda d, u, x: ("twodma", len(d), 1))
    wrap(W, "solve_twodma_2d", lambda d, u, x, axis: ("twodma", x.shape[axis], _lines(x.shape, x.shape[axis])))
    wrap(F, "solve_fdma_1d", lambda l, d, u1, u2, x: ("fdma", len(d), 1))
    wrap(F, "solve_fdma_2d", lambda l, d, u1, u2, x, axis: ("fdma", x.shape[axis], _lines(x.shape, x.shape[axis])))
    wrap(F, "solve_fdma_type2", lambda A, C, lam, x, axis, singular: ("type2", x.shape[axis],
                                                                       _lines(x.shape, x.shape[axis])))

    out = {}
    for tag, case, shape, cfg in CASES:
        opts = dict(cfg)
        with contextlib.redirect_stdout(io.StringIO()):
            ns = R.NavierStokes(case=case, shape=shape, pr=1.0, beta=opts.pop("beta", 1.0),
                                aspect=opts.pop("aspect", 1.0), tsave=None, **opts)
        ns.T.v = 1e-3 * np.random.default_rng(0).uniform(-1, 1, shape)
        ns.T.forward()
        ns.update()
        counts.clear()
        ns.update()
        out[tag] = {"case": case, "shape": list(shape), **cfg,
                    "calls": sorted([list(k) + [v] for k, v in counts.items()])}
        print(tag, sum(counts.values()), "calls")
    with open(os.path.join(HERE, "call_counts.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
