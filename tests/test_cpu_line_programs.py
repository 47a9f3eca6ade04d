"""CPU checks of the fused line programs with the NumPy interpreter emulator.

The adjoint passes must be the exact transpose of the forward step's
linearisation: <g, Phi'(X) d> == <Phi'(X)^T g, d> for random X, d, g.  The
step is quadratic in the state (bilinear convection), so the central
difference of the emulated forward step is its exact linearisation.
"""
import numpy as np
import pytest

from line_program_emulator import Machine, cheb_diff_matrix
from pypde_gb300.host import pseudoinverse_d2, stencil_matrix
from pypde_gb300.navier.fused import (build_programs, global_tables_host, host_tables, instance_params,
                                      scratch_shapes)
from pypde_gb300.navier.fused_adjoint import adjoint_shapes, build_adjoint_programs
from pypde_gb300.templates import poisson2d_matrices

STATE = ("UG", "VG", "TG", "PRES")


def make_machine(N, M, tk, dealias, seed):
    rng = np.random.default_rng(seed)
    ra, pr, dt, aspect = 3e4, 1.0, 0.01, 1.5
    nu, kappa, scale = np.sqrt(pr / ra), np.sqrt(1.0 / pr / ra), (aspect * 0.5, 0.5)
    lens, par = instance_params(N, M, dealias, dt, nu, kappa, scale)
    Nd, Md = lens[5], lens[6]

    def mats(n):
        return stencil_matrix("CN", n), pseudoinverse_d2(n)[2:, :], np.eye(n)[2:, :]

    fd = poisson2d_matrices(mats(N), mats(M), True, scale)
    tables = global_tables_host()
    tables.update(host_tables(N, M, tk, dt, nu, kappa, scale, fd, adjoint=True))
    shapes = {**scratch_shapes(N, M, Nd, Md), **adjoint_shapes(N, M, Nd, Md)}
    for k in ("UG", "VG", "TG", "PG"):
        shapes[k] = shapes["b" + k] = (N - 2, M - 2)
    shapes["PRES"] = shapes["bPRES"] = (N, M)
    arrays = {k: np.zeros(s) for k, s in shapes.items()}
    arrays["TBCC"] = rng.standard_normal((N, M))
    arrays["DTB1"] = rng.standard_normal((Nd, Md))
    arrays["DTB2"] = rng.standard_normal((N, M))
    return Machine(arrays, tables, lens, par), rng


def test_diff_matrix_matches_recurrence_transpose():
    D = cheb_diff_matrix(9)
    c = np.arange(9.0)
    assert np.allclose(D @ c, np.polynomial.chebyshev.chebder(c).tolist() + [0.0])


CASES = [(13, 11, "CD", True), (12, 13, "CN", True), (11, 9, "CD", False)]


@pytest.mark.parametrize("N,M,tk,dealias", CASES, ids=["13x11-CD", "12x13-CN", "11x9-nodealias"])
@pytest.mark.parametrize("fft", [True, False], ids=["dct-op", "dense-dct"])
def test_adjoint_programs_are_the_transposed_step(N, M, tk, dealias, fft):
    m, rng = make_machine(N, M, tk, dealias, 1)
    fwd, adj = build_programs(tk, fft), build_adjoint_programs(tk, fft)
    X = {k: 1e-1 * rng.standard_normal(m.arrays[k].shape) for k in STATE}
    d = {k: rng.standard_normal(m.arrays[k].shape) for k in STATE}
    g = {k: rng.standard_normal(m.arrays[k].shape) for k in STATE}

    def phi(Y):
        for k in STATE:
            m.arrays[k][...] = Y[k]
        for p in fwd:
            m.run(p)
        return {k: m.arrays[k].copy() for k in STATE}

    h = 1e-3
    yp = phi({k: X[k] + h * d[k] for k in STATE})
    ym = phi({k: X[k] - h * d[k] for k in STATE})
    jd = {k: (yp[k] - ym[k]) / (2 * h) for k in STATE}
    lhs = sum(float((g[k] * jd[k]).sum()) for k in STATE)

    for k in STATE:
        m.arrays[k][...] = X[k]
        m.arrays["b" + k][...] = g[k]
    m.arrays["bPG"][...] = 0.0
    for p in adj:
        m.run(p)
    rhs = sum(float((m.arrays["b" + k] * d[k]).sum()) for k in STATE)
    scale = sum(float(np.abs(g[k] * jd[k]).sum()) for k in STATE)
    assert abs(lhs - rhs) <= 1e-9 * scale, (lhs, rhs)
