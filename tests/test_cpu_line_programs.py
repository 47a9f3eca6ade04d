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


def make_machine(N, M, tk, dealias, seed, beta=1.0):
    rng = np.random.default_rng(seed)
    ra, pr, dt, aspect = 3e4, 1.0, 0.01, 1.5
    nu, kappa, scale = np.sqrt(pr / ra), np.sqrt(1.0 / pr / ra), (aspect * 0.5, 0.5)
    lens, par = instance_params(N, M, dealias, dt, nu, kappa, scale, beta=beta)
    Nd, Md = lens[5], lens[6]

    def mats(n):
        return stencil_matrix("CN", n), pseudoinverse_d2(n)[2:, :], np.eye(n)[2:, :]

    fd = poisson2d_matrices(mats(N), mats(M), True, scale)
    tables = global_tables_host()
    tables.update(host_tables(N, M, tk, dt * beta, nu, kappa, scale, fd, adjoint=True))
    shapes = {**scratch_shapes(N, M, Nd, Md, beta != 1.0), **adjoint_shapes(N, M, Nd, Md, beta != 1.0)}
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


def test_banded_tables_solve_and_transpose():
    """The device factor tables (emulated sweeps) solve A x = b and A^T x = b, incl. a singular
    Poisson line (row and column 0 dropped, x_0 = 0)."""
    from line_program_emulator import _fdma
    from pypde_gb300.navier.fused import _fdma_table, _poisson_table
    rng = np.random.default_rng(3)
    n = 21
    Bx = pseudoinverse_d2(n + 2)[2:, :]
    S = stencil_matrix("CD", n + 2)
    A = Bx @ S - 0.03 * np.eye(n + 2)[2:, :] @ S
    b = rng.standard_normal(n)
    for transpose, M in ((False, A), (True, A.T)):
        x = b.copy()
        _fdma(x, _fdma_table(A), n, transpose)
        assert np.allclose(M @ x, b, rtol=0, atol=1e-12 * np.abs(b).max())
    Sn = stencil_matrix("CN", n + 2)
    Ax, Cx = np.eye(n + 2)[2:, :] @ Sn, pseudoinverse_d2(n + 2)[2:, :] @ Sn
    lam = np.array([0.0, -3.0])
    tab = _poisson_table(Ax, Cx, lam)
    for j, lj in enumerate(lam):
        K = Ax + lj * Cx
        for transpose in (False, True):
            x = b.copy()
            _fdma(x, tab[j * 4 * n:(j + 1) * 4 * n], n, transpose)
            if abs(lj) < 1e-10:
                ref = np.zeros(n)
                ref[1:] = np.linalg.solve((K.T if transpose else K)[1:, 1:], b[1:])
            else:
                ref = np.linalg.solve(K.T if transpose else K, b)
            assert np.allclose(x, ref, rtol=0, atol=1e-10 * np.abs(ref).max()), (j, transpose)


@pytest.mark.parametrize("N,M,tk,dealias", CASES, ids=["13x11-CD", "12x13-CN", "11x9-nodealias"])
@pytest.mark.parametrize("rk3", [False, True], ids=["euler", "rk3-stage1"])
def test_split_programs_give_the_same_step(N, M, tk, dealias, rk3):
    """The per-field (variant) form of the convection passes computes the fused form's step."""
    m, rng = make_machine(N, M, tk, dealias, 2)
    if rk3:  # a middle RK3 stage: b, c and the previous stage's velocities all matter
        m.par[9], m.par[10] = 5.0 / 12.0, -17.0 / 60.0
        for k in ("UX_A", "UZ_A", "UX_B", "UZ_B"):
            m.arrays[k] = rng.standard_normal(m.arrays["UXP"].shape)
        for name, arr in (("UXC", "UX_B"), ("UZC", "UZ_B"), ("UXO", "UX_A"), ("UZO", "UZ_A")):
            m.arrays[name] = m.arrays[arr]
    X = {k: 1e-1 * rng.standard_normal(m.arrays[k].shape) for k in STATE}
    out = []
    for split in (False, True):
        for k in STATE:
            m.arrays[k][...] = X[k]
        for p in build_programs(tk, True, rk3=rk3, split=split):
            m.run(p)
        out.append({k: m.arrays[k].copy() for k in STATE})
    for k in STATE:
        scale = np.abs(out[0][k]).max()
        assert np.abs(out[1][k] - out[0][k]).max() <= 1e-12 * scale, k


@pytest.mark.parametrize("tk", ["CD", "CN"])
def test_adjoint_of_split_form_is_the_transpose(tk):
    """R1 in per-field form: the adjoint passes remain the transpose of the (split) forward step."""
    m, rng = make_machine(12, 13, tk, True, 3)
    fwd, adj = build_programs(tk, True, split=True), build_adjoint_programs(tk, True, split=True)
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
    lhs = sum(float((g[k] * (yp[k] - ym[k])).sum()) / (2 * h) for k in STATE)
    for k in STATE:
        m.arrays[k][...] = X[k]
        m.arrays["b" + k][...] = g[k]
    m.arrays["bPG"][...] = 0.0
    for p in adj:
        m.run(p)
    rhs = sum(float((m.arrays["b" + k] * d[k]).sum()) for k in STATE)
    assert abs(lhs - rhs) <= 1e-9 * abs(lhs), (lhs, rhs)


@pytest.mark.parametrize("sd,dm", [(True, False), (False, True)], ids=["per-slot-dct", "dense-mma"])
def test_launch_rewrites_give_the_same_step(sd, dm):
    """The per-launch op rewrites (multi-slot DCT ops split per slot; DCT ops as the program's dense
    matrices on the tensor cores) compute the same forward and reverse-mode passes."""
    import copy
    from pypde_gb300.navier.fused import launch_ops
    m, rng = make_machine(12, 13, "CN", True, 4)
    progs = build_programs("CN", True) + build_adjoint_programs("CN", True)
    X = {k: 1e-1 * rng.standard_normal(m.arrays[k].shape) for k in STATE}
    G = {k: rng.standard_normal(m.arrays[k].shape) for k in STATE}
    out = []
    for rewrite in (False, True):
        for k in STATE:
            m.arrays[k][...] = X[k]
            m.arrays["b" + k][...] = G[k]
        m.arrays["bPG"][...] = 0.0
        for p in progs:
            if rewrite:
                p = copy.copy(p)
                p.ops = launch_ops(p, sd, dm)
            m.run(p)
        out.append({k: m.arrays[k].copy() for k in STATE + tuple("b" + k for k in STATE)})
    for k in out[0]:
        scale = np.abs(out[0][k]).max()
        assert np.abs(out[1][k] - out[0][k]).max() <= 1e-12 * scale, k


@pytest.mark.parametrize("split", [False, True], ids=["fused", "per-field"])
@pytest.mark.parametrize("tk", ["CD", "CN"])
def test_beta_programs(tk, split):
    """beta != 1: the explicit-diffusion passes give the plain-path step's diffusion term (against
    the same programs with beta = 1 plus the term computed densely), and the reverse-mode passes
    stay the exact transpose."""
    from pypde_gb300.host import stencil_matrix as S
    beta = 0.6
    m, rng = make_machine(12, 13, tk, True, 5, beta)
    fwd = build_programs(tk, True, split=split, beta=True)
    adj = build_adjoint_programs(tk, True, split=split, beta=True)
    names = [p.name for p in fwd]
    assert "P2e" in names and names.index("P2e") < names.index("P3")
    # the x- and y-halves written into the right-hand sides: compare with dense operators
    X = {k: 1e-1 * rng.standard_normal(m.arrays[k].shape) for k in STATE}
    for k in STATE:
        m.arrays[k][...] = X[k]
    for p in fwd:
        if p.name in ("P2e",):
            m.run(p)
    N, M = 12, 13
    sx, sz = 1.5 * 0.5, 0.5
    Dn, Dm = cheb_diff_matrix(N), cheb_diff_matrix(M)
    for F, kind in (("U", "CD"), ("T", tk)):
        Sx, Sy = S(kind, N), S("CD", M)
        ref0 = X[F + "G"] @ Sy.T
        refyy = X[F + "G"] @ (Dm @ Dm @ Sy).T / sz ** 2
        assert np.allclose(m.arrays["EY0_" + F], ref0, atol=1e-12 * np.abs(ref0).max())
        assert np.allclose(m.arrays["EYY_" + F], refyy, atol=1e-12 * np.abs(refyy).max())
        del Sx
    # exact transpose of the whole step
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
    lhs = sum(float((g[k] * (yp[k] - ym[k])).sum()) / (2 * h) for k in STATE)
    for k in STATE:
        m.arrays[k][...] = X[k]
        m.arrays["b" + k][...] = g[k]
    m.arrays["bPG"][...] = 0.0
    for p in adj:
        m.run(p)
    rhs = sum(float((m.arrays["b" + k] * d[k]).sum()) for k in STATE)
    assert abs(lhs - rhs) <= 1e-9 * abs(lhs), (lhs, rhs)


def test_beta_split_matches_fused():
    m, rng = make_machine(11, 13, "CN", True, 6, 0.5)
    X = {k: 1e-1 * rng.standard_normal(m.arrays[k].shape) for k in STATE}
    out = []
    for split in (False, True):
        for k in STATE:
            m.arrays[k][...] = X[k]
        for p in build_programs("CN", True, split=split, beta=True):
            m.run(p)
        out.append({k: m.arrays[k].copy() for k in STATE})
    for k in STATE:
        assert np.abs(out[1][k] - out[0][k]).max() <= 1e-12 * np.abs(out[0][k]).max(), k


def _rk3_machines(N, M, tk, seed):
    """Three stage views of one instance (rbc2d_base.py:86-102 coefficients): shared arrays, per
    stage its parameters, ADI tables, velocity arrays (UXC / UXO) and carried velocity gradients."""
    from pypde_gb300.navier.fused_adjoint import RK3_CARRY
    m, rng = make_machine(N, M, tk, True, seed)
    Nd, Md = m.lens[5], m.lens[6]
    for k in ("UX_A", "UX_B", "UZ_A", "UZ_B"):
        m.arrays[k] = np.zeros((Nd, Md))
    for k, shp in adjoint_shapes(N, M, Nd, Md, rk3=True).items():
        m.arrays.setdefault(k, np.zeros(shp))
    ra, pr, dt, aspect = 3e4, 1.0, 0.01, 1.5
    nu, kappa, scale = np.sqrt(pr / ra), np.sqrt(1.0 / pr / ra), (aspect * 0.5, 0.5)
    a, b, c = (8 / 15, 2 / 15, 1 / 3), (8 / 15, 5 / 12, 3 / 4), (0.0, -17 / 60, -5 / 12)

    def mats(n):
        return stencil_matrix("CN", n), pseudoinverse_d2(n)[2:, :], np.eye(n)[2:, :]

    fd = poisson2d_matrices(mats(N), mats(M), True, scale)
    out = []
    for k in range(3):
        par = instance_params(N, M, True, dt, nu, kappa, scale, a[k], b[k], c[k])[1]
        tables = dict(m.tables)
        tables.update({t: v for t, v in host_tables(N, M, tk, dt * a[k], nu, kappa, scale, fd).items()
                       if t in ("Ax_U", "Ax_T", "Ay_U", "Ay_T")})
        cur, old = ("A", "A") if k == 0 else (("B", "A") if k == 1 else ("A", "B"))
        alias = {"UXC": "UX_" + cur, "UZC": "UZ_" + cur, "UXO": "UX_" + old, "UZO": "UZ_" + old, **RK3_CARRY[k]}
        arrays = dict(m.arrays)
        for name, target in alias.items():
            arrays[name] = m.arrays[target]          # the same array object: in-place updates shared
        out.append(Machine(arrays, tables, m.lens, par))
    return out, m.arrays, rng


@pytest.mark.parametrize("tk", ["CD", "CN"])
def test_rk3_adjoint_is_the_transposed_step(tk):
    """The reverse RK3 step (stages 0, 1 rerun; stages 2, 1, 0 backward with the velocity gradients
    carried between stages) is the transpose of the three-stage step's linearisation."""
    st, arrays, rng = _rk3_machines(12, 13, tk, 7)
    fwd = build_programs(tk, True, rk3=True)
    adj = build_adjoint_programs(tk, True, rk3=True)
    keys = STATE + ("PG",)
    X = {k: 1e-1 * rng.standard_normal(arrays[k].shape) for k in keys}
    d = {k: rng.standard_normal(arrays[k].shape) for k in STATE}
    g = {k: rng.standard_normal(arrays[k].shape) for k in STATE}

    def phi(Y):
        for k in keys:
            arrays[k][...] = Y[k]
        for mk in st:
            for p in fwd:
                mk.run(p)
        return {k: arrays[k].copy() for k in STATE}

    def cd(h):   # central difference of <g, Phi(X + h d)>
        yp = phi({k: X[k] + h * d.get(k, 0.0) for k in keys})
        ym = phi({k: X[k] - h * d.get(k, 0.0) for k in keys})
        return sum(float((g[k] * (yp[k] - ym[k])).sum()) / (2 * h) for k in STATE)

    # the three-stage step is not quadratic: Richardson extrapolation removes the O(h^2) term
    lhs = (4.0 * cd(5e-5) - cd(1e-4)) / 3.0
    for k in keys:
        arrays[k][...] = X[k]
    for k in STATE:
        arrays["b" + k][...] = g[k]
    arrays["bPG"][...] = 0.0
    snap = []
    snap.append({k: arrays[k].copy() for k in keys})
    for p in fwd:
        st[0].run(p)
    snap.append({k: arrays[k].copy() for k in keys})
    for p in fwd:
        st[1].run(p)
    for k in (2, 1, 0):
        if k < 2:
            for key in keys:
                arrays[key][...] = snap[k][key]
        for p in adj:
            st[k].run(p)
    rhs = sum(float((arrays["b" + k] * d[k]).sum()) for k in STATE)
    assert abs(lhs - rhs) <= 1e-9 * abs(lhs), (lhs, rhs)


@pytest.mark.parametrize("beta", [1.0, 0.5])
def test_rk3_step_split_matches_fused(beta):
    """All three RK3 stages (velocities carried between stages through UXC / UXO): the per-field form
    computes the fused form's step."""
    st, arrays, rng = _rk3_machines(12, 13, "CN", 8)
    if beta != 1.0:   # the beta parameters and the explicit-diffusion scratch
        from pypde_gb300.navier.fused import P_EDT, P_EDU, P_MNU, scratch_shapes
        for k, shp in scratch_shapes(12, 13, st[0].lens[5], st[0].lens[6], True).items():
            arrays.setdefault(k, np.zeros(shp))
        for m in st:
            m.par = list(m.par)
            m.par[P_EDU], m.par[P_EDT] = m.par[3] * (1 - beta) * 0.01, m.par[4] * (1 - beta)
            m.par[P_MNU] *= beta
            for k in scratch_shapes(12, 13, st[0].lens[5], st[0].lens[6], True):
                m.arrays[k] = arrays[k]
    keys = STATE + ("PG",)
    X = {k: 1e-1 * rng.standard_normal(arrays[k].shape) for k in keys}
    out = []
    for split in (False, True):
        for k in keys:
            arrays[k][...] = X[k]
        for k in ("UX_A", "UX_B", "UZ_A", "UZ_B"):
            arrays[k][...] = 0.0
        progs = build_programs("CN", True, rk3=True, split=split, beta=beta != 1.0)
        for m in st:
            for p in progs:
                m.run(p)
        out.append({k: arrays[k].copy() for k in STATE})
    for k in STATE:
        assert np.abs(out[1][k] - out[0][k]).max() <= 1e-12 * np.abs(out[0][k]).max(), k


@pytest.mark.parametrize("rk3", [False, True])
@pytest.mark.parametrize("beta", [False, True])
def test_algorithmic_work_of_both_forms_agrees(rk3, beta):
    """The roofline's algorithmic flop count: the fused and the per-field form of the step do the same
    transforms (a multi-slot DCT op counts one transform per slot), so their totals agree to the few
    extra pointwise operations of the per-field form."""
    import types
    from pypde_gb300 import _lib
    from pypde_gb300.navier.fused import Prog, program_work
    lens, _ = instance_params(65, 33, True, 0.01, 1e-3, 1e-3, (0.5, 0.5))
    inst = types.SimpleNamespace(lens=lens)
    tot = []
    for split in (False, True):
        progs = build_programs("CD", True, rk3=rk3, split=split, beta=beta)
        tot.append(sum(program_work(p, inst)[0] * len(p.variants) for p in progs))
    assert abs(tot[1] - tot[0]) <= 0.02 * tot[0], tot
    one, three = Prog("a", 1, 6, 4), Prog("b", 1, 6, 4)
    for p, count in ((one, 1), (three, 3)):
        for s in range(count):
            p.load(s, "X", 6)
        p.dct(0, _lib.DCT_FWD, True, count=count)
    assert program_work(three, inst)[0] == pytest.approx(3 * program_work(one, inst)[0])
