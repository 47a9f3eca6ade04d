"""Generate golden vectors by running the unmodified pypde reference.

Run from the repository root in a container that has the reference checked
out, its location given by ``--reference`` or the PYPDE_REFERENCE variable:

    python tests/golden/make_golden.py [--reference PATH]

It installs ``ref_shims`` (loop-level restatement of the reference's four
f2py Fortran kernels, matplotlib/h5py stubs, NumPy-1.x eig semantics), runs
the reference's own unittest suite against the shims (recorded in
``reference_tests.json``), then records the reference's outputs for seeded
inputs in ``golden.npz``.  The fixtures travel with the repository; the
reference itself does not.
"""
import argparse
import contextlib
import io
import json
import os
import sys
import unittest

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_shims  # noqa: E402


def quiet(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def run_reference_tests(reference):
    """Run the reference's unittest suites (bases, solver, integration) against the shims."""
    loader = unittest.TestLoader()
    suites = []
    for start in ["pypde/bases/test", "pypde/solver/test", "pypde/test"]:
        suites.append(loader.discover(os.path.join(reference, start), top_level_dir=reference))
    res = unittest.TextTestRunner(stream=io.StringIO(), verbosity=0)
    with contextlib.redirect_stdout(io.StringIO()):
        r = res.run(unittest.TestSuite(suites))
    return {"run": r.testsRun, "failures": len(r.failures), "errors": len(r.errors),
            "skipped": len(r.skipped),
            "failed": [str(t) for t, _ in r.failures + r.errors]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=ref_shims.REFERENCE)
    args = ap.parse_args()
    ref_shims.install(args.reference)
    np.random.seed(1234)  # the reference tests draw from np.random

    summary = run_reference_tests(args.reference)
    print("reference tests:", summary)
    with open(os.path.join(HERE, "reference_tests.json"), "w") as f:
        json.dump(summary, f, indent=1)

    from pypde.bases.spectralbase import Base
    from pypde.field import Field
    from pypde import field_operations as fo
    from pypde.templates.hholtz import solverplan_hholtz2d_adi
    from pypde.templates.poisson import solverplan_poisson2d
    from navier import rbc2d as R
    from navier import rbc2d_adj as RA

    G = {}
    rng = np.random.default_rng(20260101)

    # --- 1-D bases along axis 0 of (N x 5) arrays: DCT-I, stencils, derivative
    for N in (33, 40, 65):
        f = rng.uniform(-1, 1, (N, 5))
        c = rng.uniform(-1, 1, (N, 5))
        CH = Base(N, "CH")
        G[f"ch{N}_f"], G[f"ch{N}_c"] = f, c
        G[f"ch{N}_fwd"] = CH.forward_fft(f.copy())
        G[f"ch{N}_bwd"] = CH.backward_fft(c.copy())
        G[f"ch{N}_d1"] = CH.derivative(c.copy(), 1)
        G[f"ch{N}_d2"] = CH.derivative(c.copy(), 2)
        for key in ("CD", "CN"):
            B = Base(N, key)
            v = rng.uniform(-1, 1, (N - 2, 5))
            G[f"{key}{N}_v"] = v
            G[f"{key}{N}_fwd"] = B.forward_fft(f.copy())
            G[f"{key}{N}_bwd"] = B.backward_fft(v.copy())
            G[f"{key}{N}_toch"] = B.to_chebyshev(v.copy())
            G[f"{key}{N}_fromch"] = B.from_chebyshev(c.copy())
            G[f"{key}{N}_d1"] = B.derivative(v.copy(), 1)
            G[f"{key}{N}_d2"] = B.derivative(v.copy(), 2)

    # --- 2-D field transforms with and without 3/2 dealiasing, grad, conversions
    N, M = 33, 20
    for keys in (("CD", "CN"), ("CD", "CD"), ("CH", "CH")):
        tag = "".join(keys)
        fld = Field([Base(N, keys[0], dealias=3 / 2), Base(M, keys[1], dealias=3 / 2)])
        v = rng.uniform(-1, 1, fld.shape_physical)
        vh = rng.uniform(-1, 1, fld.shape_spectral)
        G[f"f2_{tag}_v"], G[f"f2_{tag}_vh"] = v, vh
        G[f"f2_{tag}_fwd"] = fld.forward(v.copy())
        G[f"f2_{tag}_bwd"] = fld.backward(vh.copy())
        G[f"f2_{tag}_dbwd"] = fld.dealias.backward(vh.copy())
        vd = rng.uniform(-1, 1, fld.dealias.shape_physical)
        G[f"f2_{tag}_vd"] = vd
        G[f"f2_{tag}_dfwd"] = fld.dealias.forward(vd.copy())
        fld.vhat = vh.copy()
        for d in ((1, 0), (0, 1), (2, 0), (0, 2), (1, 1)):
            G[f"f2_{tag}_grad{d[0]}{d[1]}"] = fo.grad(fld, d, scale=(0.5, 0.25))
        ch = rng.uniform(-1, 1, fld.shape_physical)
        G[f"f2_{tag}_ch"] = ch
        G[f"f2_{tag}_g2c"] = fo.galerkin_to_cheby(vh.copy(), fld)
        G[f"f2_{tag}_c2g"] = fo.cheby_to_galerkin(ch.copy(), fld)

    # --- convective term, dealiased and not
    for dealias in (True, False):
        fld = Field([Base(N, "CD", dealias=3 / 2), Base(M, "CD", dealias=3 / 2)])
        dfld = Field([Base(N, "CH", dealias=3 / 2), Base(M, "CH", dealias=3 / 2)])
        fld.vhat = rng.uniform(-1, 1, fld.shape_spectral)
        shp = dfld.dealias.shape_physical if dealias else dfld.shape_physical
        ux, uz, bc = (rng.uniform(-1, 1, shp) for _ in range(3))
        t = f"conv{int(dealias)}"
        G[t + "_vh"], G[t + "_ux"], G[t + "_uz"], G[t + "_bc"] = fld.vhat.copy(), ux, uz, bc
        G[t + "_out"] = fo.convective_term(fld, ux, uz, deriv_field=dfld, add_bc=bc,
                                           dealias=dealias, scale=(0.5, 0.5))

    # --- ADI Helmholtz plan and Poisson plan
    for keys, shape in ((("CD", "CD"), (33, 25)), (("CN", "CD"), (33, 25))):
        tag = "".join(keys)
        fld = Field([Base(shape[0], keys[0]), Base(shape[1], keys[1])])
        sol = solverplan_hholtz2d_adi(fld.xs, lam=0.01, scale=(0.5, 0.5))
        b = rng.uniform(-1, 1, shape)
        old = rng.uniform(-1, 1, fld.shape_spectral)
        G[f"hh_{tag}_b"], G[f"hh_{tag}_old"] = b, old
        r = sol.solve_rhs(b.copy())
        G[f"hh_{tag}_rhs"] = np.array(r)
        r = r + sol.solve_old(old.copy())
        G[f"hh_{tag}_rhsold"] = np.array(r)
        G[f"hh_{tag}_x"] = np.array(sol.solve_lhs(np.asfortranarray(r)))
    for keys, singular in ((("CN", "CN"), True), (("CD", "CD"), False), (("CD", "CN"), False)):
        tag = "".join(keys)
        shape = (33, 25)
        fld = Field([Base(shape[0], keys[0]), Base(shape[1], keys[1])])
        sol = solverplan_poisson2d(fld.xs, singular=singular, scale=(0.5, 0.5))
        b = rng.uniform(-1, 1, shape)
        G[f"po_{tag}_b"] = b
        r = sol.solve_rhs(b.copy())
        G[f"po_{tag}_rhs"] = np.array(r)
        x = np.array(sol.solve_lhs(np.asfortranarray(r)))
        if singular:
            x[0, 0] = 0
        G[f"po_{tag}_x"] = x

    # --- Rayleigh-Benard steps
    def ns_state(ns, tag):
        G[tag + "_T"] = ns.T.vhat.copy()
        G[tag + "_U"] = ns.U.vhat.copy()
        G[tag + "_V"] = ns.V.vhat.copy()
        G[tag + "_P"] = ns.P.vhat.copy()
        G[tag + "_pres"] = ns.pres.vhat.copy()
        nu, nuv = quiet(ns.eval_Nu)
        ns.U.backward()
        ns.V.backward()
        ke = 0.5 * fo.avg_vol(ns.U.v ** 2 + ns.V.v ** 2, ns.deriv_field.dx, ns.deriv_field.dy)
        G[tag + "_scalars"] = np.array([nu, nuv, ke])

    cases = [
        # tag, case, shape, cfg, nsteps, seed, amplitude
        ("rbc_lin33", "linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu"), 10, 0, 1e-2),
        ("rbc_lin33nd", "linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=False, integrator="eu"), 10, 0, 1e-2),
        ("rbc_lin33x17", "linear", (33, 17), dict(ra=3e4, dt=0.01, dealias=True, integrator="eu", aspect=2.0), 10, 5, 1e-2),
        ("rbc_rbc33", "rbc", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu"), 10, 1, 1e-2),
        ("rbc_zero33", "zero", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu"), 10, 2, 1e-2),
        ("rbc_rk3_33", "linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="rk3"), 5, 3, 1e-2),
        ("rbc_beta33", "linear", (33, 33), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu", beta=0.5), 5, 4, 1e-2),
        ("rbc_c1", "linear", (65, 65), dict(ra=1e5, dt=0.01, dealias=True, integrator="eu"), 100, 0, 1e-3),
        ("rbc_c1nd", "linear", (65, 65), dict(ra=1e5, dt=0.01, dealias=False, integrator="eu"), 100, 0, 1e-3),
    ]
    for tag, case, shape, cfg, nsteps, seed, amp in cases:
        ns = quiet(R.NavierStokes, case=case, shape=shape, pr=1.0, beta=cfg.pop("beta", 1.0),
                   aspect=cfg.pop("aspect", 1.0), tsave=None, **cfg)
        noise = amp * np.random.default_rng(seed).uniform(-1, 1, shape)
        ns.T.v = noise.copy()
        ns.T.forward()
        G[tag + "_T0"] = ns.T.vhat.copy()
        ns.update()
        if shape[0] < 65:
            ns_state(ns, tag + "_s1")
        for _ in range(nsteps - 1):
            ns.update()
        ns_state(ns, tag + f"_s{nsteps}")
        print("golden", tag, G[tag + f"_s{nsteps}_scalars"])

    # --- adjoint-descent step (navier/rbc2d_adj.py), for the adjoint comparison
    nsa = quiet(RA.NavierStokesAdjoint, case="linear", shape=(33, 33), ra=1e5, pr=1.0, dt=0.01,
                tsave=None, dealias=True, integrator="eu", beta=1.0)
    noise = 1e-2 * np.random.default_rng(7).uniform(-1, 1, (33, 33))
    nsa.T.v = noise.copy()
    nsa.T.forward()
    G["adj33_T0"] = nsa.T.vhat.copy()
    nsa.update()
    G["adj33_T1"], G["adj33_U1"], G["adj33_V1"] = nsa.T.vhat.copy(), nsa.U.vhat.copy(), nsa.V.vhat.copy()
    G["adj33_FT"], G["adj33_FU"], G["adj33_FV"] = nsa.NS.T.vhat.copy(), nsa.NS.U.vhat.copy(), nsa.NS.V.vhat.copy()
    G["adj33_TA"], G["adj33_UA"], G["adj33_VA"] = nsa.TA.vhat.copy(), nsa.UA.vhat.copy(), nsa.VA.vhat.copy()

    out = os.path.join(HERE, "golden.npz")
    np.savez_compressed(out, **{k: np.asarray(v, dtype=np.float64) for k, v in G.items()})
    print("wrote", out, os.path.getsize(out) // 1024, "KiB,", len(G), "arrays")


if __name__ == "__main__":
    main()
