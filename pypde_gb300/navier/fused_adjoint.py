"""Reverse-mode (discrete adjoint) fused step: fourteen line-program passes.

The forward fused step (``fused.build_programs``) maps the state
(U, V, T Galerkin coefficients and the Chebyshev pressure) to the next one.
Its adjoint maps the gradient with respect to the new state to the gradient
with respect to the old state.  Every forward pass is linear in its inputs
except the convection products of P2, so the adjoint is the forward pass
sequence run backwards with every operator replaced by its transpose:

  LOAD <-> STORE / STORE_ADD, S <-> S^T, D -> D^T (DIFF_T), DCT FWD/BWD ->
  FWD_T/BWD_T, pad <-> truncate, banded / dense tables -> transposed tables,
  FDMA -> FDMA_T, POISSON -> POISSON_T, the symmetric (S^T S)^-1 and the
  projection P[0,0] = 0 unchanged.

The products ux * dF/dx and uz * dF/dz are linearised around the forward state
of the step: pass R1 (the forward P1) recomputes A_F0 / A_Fx from that state,
and Q2u / Q2f recompute ux, uz and the physical derivatives.  Q2f and Q1 are
written once for a generic field F and run as three descriptors (U, V, T) of
one launch, which triples the CTAs of a single instance.

  R1  x  forward P1 on the step's input state        -> A_F0, A_Fx
  Q10 y  velocity correction^T                       -> U*bar, V*bar, G1bar, G2bar
  Q9  x  pressure update^T, grad P^T                 -> Y1bar, Y2bar
  Q8  y  D_y^T, S_y^T, [0,0] projection, Q_y^T        -> Xbar
  Q7  x  per-eigenvalue transposed sweep             -> R2bar
  Q6  y  H_y^T                                       -> R1bar
  Q5  x  B_x^T, -nu pres-bar, divergence^T           -> W1bar, W2bar
  Q4  y  S_y^T, D_y^T, A_y^-T, B_y^T, (B S)_y^T      -> Q1bar, Q2bar
  Q3s x  A_x^-T, B_x^T, (B S)_x^T                    -> RHSbar, Ubar Vbar Tbar (old-time part)
         (per-field form: and the pressure / buoyancy terms^T)
  Q3  x  forward-DCT_x^T (per-field form: per field); -> Cbar, DPZbar, TSYbar, pres-bar
         pressure / buoyancy terms^T
  Q2u y  ux, uz (recomputed); D_y^T, S_y^T          -> UXP, UZP, pres-bar, Tbar
  Q2f y  per field: products^T, DCT_y^T chains       -> A_F*bar, uxbar / uzbar parts
  Q2z y  per component: ux / uz bar chains           -> A_U0bar, A_V0bar
  Q1  x  per field: DCT_x^T, D_x^T, S_x^T            -> Ubar, Vbar, Tbar (convection part)

The gradient arrays are updated in place: they hold d/d(new state) on entry
and d/d(old state) on exit, so a horizon is a loop of adjoint steps over the
forward states taken in reverse order.
"""
import torch

from .. import _lib
from .._dev import DTYPE, device, to_dev
from .fused import (L_M, L_MD, L_MG, L_N, L_ND, L_NG, P_B, P_C, P_DT, P_EDT, P_EDU, P_IDT, P_ISX, P_ISZ, P_MDT,
                    P_MDTSX, P_MDTSZ, P_MNU, P_TF, FusedBatch, Prog, _Instance, build_programs, host_tables)

BAR_STATE = ("bUG", "bVG", "bTG", "bPG", "bPRES")


def _explicit_diffusion_x_t(p, s, F, kind, src):
    """Transpose of the x-half of the explicit diffusion (P3): from the right-hand-side gradient
    in slot ``src``, EY0_F bar = P_ED S_x^T (D_x^T)^2 / sx^2 and EYY_F bar = P_ED S_x^T of it."""
    ed = P_EDT if F == "T" else P_EDU
    p.copy(s, src)
    p.scale(s, par=ed)
    p.stencil_t(s, kind)
    p.store(s, "bEYY_" + F)
    p.copy(s, src)
    p.scale(s, par=ed)
    p.scale(s, par=P_ISX)
    p.scale(s, par=P_ISX)
    p.diff_t(s, count=2)
    p.stencil_t(s, kind)
    p.store(s, "bEY0_" + F)


def _explicit_diffusion_y_t():
    """Q2e (y, N-2 lines), the transpose of P2e: F bar += S_y^T EY0_F bar + S_y^T (D_y^T)^2 EYY_F bar / sz^2."""
    p = Prog("Q2e", 1, L_NG, 1)
    for F in "UVT":
        p.load(0, "bEYY_" + F, L_M)
        p.scale(0, par=P_ISZ)
        p.scale(0, par=P_ISZ)
        p.diff_t(0, count=2)
        p.load_add(0, "bEY0_" + F)
        p.stencil_t(0, "CD")
        p.store_add(0, "b" + F + "G")
    return p


def build_adjoint_programs(tkind, fft, split=False, beta=False, rk3=False):
    """R1 and the thirteen transposed passes of one IMEX Euler step; R1 is the forward P1 of
    the same form (``split``: per-field) as the batch's forward passes.  ``beta``: with the
    transposes of the explicit-diffusion terms (in Q3s and the extra pass Q2e).

    ``rk3``: the passes of one stage k of the three-stage step.  The stage's products use the
    velocity w = b_k u_k + c_k u_(k-1) (rbc2d_base.py:86-102): Q2u forms it from this stage's
    velocity and the previous stage's (UXO, UZO), and Q2z splits the gradient on w into
    b_k (u_k's own path, plus the carried c_(k+1) part from stage k+1, bUXC / bUZC) and c_k
    (stored for stage k-1, bUXO / bUZO)."""
    BWD, BWD_T, FWD_T = _lib.DCT_BWD, _lib.DCT_BWD_T, _lib.DCT_FWD_T
    kinds = {"U": "CD", "V": "CD", "T": tkind}
    ax = {"U": "Ax_U", "V": "Ax_U", "T": "Ax_T"}
    Q = []

    r1 = build_programs(tkind, fft, split=split)[0]
    r1.name = "R1"
    Q.append(r1)

    # Q10 (y, N-2 lines): U = U* - T_y S_y^T G1 (and V)
    p = Prog("Q10", 1, L_NG, 2)
    for i, F in enumerate("UV"):
        p.load(i, "b" + F + "G", L_MG)
        p.store(i, "b" + F + "S")
        p.scale(i, alpha=-1.0)
    p.tdma_multi(0, 2, "CD")
    p.stencil(0, "CD")
    p.stencil(1, "CD")
    p.store(0, "bG1")
    p.store(1, "bG2")
    Q.append(p)

    # Q9 (x, M lines): pres += S_x Y1 / dt; G1 = T_x S_x^T D_x S_x Y1 / sx; G2 = T_x S_x^T S_x Y2
    p = Prog("Q9", 0, L_M, 2)
    p.load(0, "bG1", L_NG)
    p.load(1, "bG2", L_NG)
    p.tdma_multi(0, 2, "CD")
    p.stencil(0, "CD")
    p.stencil(1, "CD")
    p.scale(0, par=P_ISX)
    p.diff_t(0)
    p.load_add(0, "bPRES", par=P_IDT)
    p.stencil_t(0, "CN")
    p.stencil_t(1, "CN")
    p.store(0, "bY1")
    p.store(1, "bY2")
    Q.append(p)

    # Q8 (y, N-2 lines): PG = Z Q_y X; Y1 = S_y PG; Y2 = D_y Y1 / sz
    p = Prog("Q8", 1, L_NG, 1)
    p.load(0, "bY2", L_M)
    p.scale(0, par=P_ISZ)
    p.diff_t(0)
    p.load_add(0, "bY1")
    p.stencil_t(0, "CN")
    p.add("ZERO00", 0)
    p.dense(0, "QyT", L_MG)
    p.store(0, "bX")
    Q.append(p)

    # Q7 (x, M-2 lines): transposed per-eigenvalue sweep
    p = Prog("Q7", 0, L_MG, 1)
    p.load(0, "bX", L_NG)
    p.add("POISSON_T", 0, mat="Pois")
    p.store(0, "bR2")
    Q.append(p)

    # Q6 (y, N-2 lines): H_y^T
    p = Prog("Q6", 1, L_NG, 1)
    p.load(0, "bR2", L_MG)
    p.dense(0, "HyT", L_M)
    p.store(0, "bR1")
    Q.append(p)

    # Q5 (x, M lines): div = D_x S_x W1 / sx + S_x W2; pres -= nu div; R1 = B_x div
    p = Prog("Q5", 0, L_M, 2)
    p.load(0, "bR1", L_NG)
    p.banded(0, "BxT", -4, 3, L_N)
    p.load_add(0, "bPRES", par=P_MNU)
    p.copy(1, 0)
    p.stencil_t(1, "CD")
    p.store(1, "bW2")
    p.scale(0, par=P_ISX)
    p.diff_t(0)
    p.stencil_t(0, "CD")
    p.store(0, "bW1")
    Q.append(p)

    # Q4 (y, N-2 lines): F* = A_y^-1 (B_y Q1 + (B S)_y Q2); W1 = S_y U*; W2 = D_y S_y V* / sz
    p = Prog("Q4", 1, L_NG, 4)
    p.load(0, "bUS", L_MG)
    p.load(3, "bW1", L_M)
    p.stencil_t(3, "CD")
    p.axpy(0, 3)
    p.load(1, "bVS", L_MG)
    p.load(3, "bW2", L_M)
    p.scale(3, par=P_ISZ)
    p.diff_t(3)
    p.stencil_t(3, "CD")
    p.axpy(1, 3)
    p.load(2, "bTG", L_MG)
    p.fdma_t(0, ["Ay_U", "Ay_U", "Ay_T"])
    for i, F in enumerate("UVT"):
        p.copy(3, i)
        p.banded(3, "BSyT", -4, 4, L_MG)
        p.store(3, "bQ2_" + F)
        p.banded(i, "ByT", -4, 3, L_M)
        p.store(i, "bQ1_" + F)
    Q.append(p)

    # Q3s (x, M lines): Q1 = A_x^-1 B_x RHS; Q2 = A_x^-1 (B S)_x F (starts the state gradient); then,
    # per-field form, from the RHS gradient in slots 0-2 the transposed right-hand-side terms (the
    # same axis and lines: one pass); fused form: those terms and the x-transform in Q3
    p = Prog("Q3s", 0, L_M, 6)
    for i, F in enumerate("UVT"):
        p.load(i, "bQ1_" + F, L_NG)
        p.load(3 + i, "bQ2_" + F, L_NG)
    p.fdma_t(0, [ax[F] for F in "UVT"] * 2)
    for i, F in enumerate("UVT"):
        p.banded(i, "BxT", -4, 3, L_N)
        p.store(i, "bRHS_" + F)               # read by Q3
        p.banded(3 + i, "BSx_TT" if F == "T" else "BSx_UT", -4, 4, L_NG)
        p.store(3 + i, "b" + F + "G")
    if not split:  # Q3 (x, M lines): the terms and the forward x-transform, as the forward P3 / P3s
        Q.append(p)
        p = Prog("Q3", 0, L_M, 4)
        for i, F in enumerate("UVT"):
            p.load(i, "bRHS_" + F, L_N)
    for i, F in enumerate("UVT"):
        if beta:
            _explicit_diffusion_x_t(p, 3, F, kinds[F], i)
        if F == "U":
            p.copy(3, i)
            p.scale(3, par=P_MDTSX)
            p.diff_t(3)
            p.store_add(3, "bPRES")
        elif F == "V":
            p.copy(3, i)
            p.scale(3, par=P_MDTSZ)
            p.store(3, "bDPZ")
            p.copy(3, i)
            p.scale(3, par=P_DT)
            p.stencil_t(3, tkind)
            p.store(3, "bTSY")
        if not split:
            p.scale(i, par=P_MDT)
            p.setlen(i, L_ND)
    if not split:
        p.dct(0, FWD_T, fft, count=3)
        for i, F in enumerate("UVT"):
            p.store(i, "bC_" + F)
    Q.append(p)

    if split:  # Q3 (x, M lines), per field (three descriptors): RHS = -dt Fwd_x C
        p = Prog("Q3", 0, L_M, 1)
        p.load(0, "bRHS_F", L_N, par=P_MDT)
        p.setlen(0, L_ND)
        p.dct(0, FWD_T, fft)
        p.store(0, "bC_F")
        p.variants = [{"arrays": {"bRHS_F": "bRHS_" + F, "bC_F": "bC_" + F}} for F in "UVT"]
        Q.append(p)

    if beta:
        Q.append(_explicit_diffusion_y_t())

    # Q2u / Q2f / Q2z (y, Nd lines): C = Fwd_y(dF/dx ux + dF/dz uz [+ DTB1 uz]), linearised.
    # Q2f runs once per field (three descriptors of one program, "variants"), so one instance
    # gives three times the CTAs; the fields' contributions to ux bar, uz bar meet in Q2z.
    p = Prog("Q2u", 1, L_ND, 2)
    for s, F in ((0, "U"), (1, "V")):
        p.load(s, "A_" + F + "0", L_MG)
        p.stencil(s, "CD")
        p.setlen(s, L_MD)
    p.dct(0, BWD, fft, count=2)
    if rk3:
        for s_, O in ((0, "UXO"), (1, "UZO")):
            p.scale(s_, par=P_B)
            p.load_add(s_, O, par=P_C)
    p.store(0, "UXP")
    p.store(1, "UZP")
    p.load(0, "bDPZ", L_M)
    p.diff_t(0)
    p.store_add(0, "bPRES")
    p.load(0, "bTSY", L_M)
    p.stencil_t(0, "CD")
    p.store_add(0, "bTG")
    Q.append(p)

    p = Prog("Q2f", 1, L_ND, 5)
    p.load(0, "UXP", L_MD)
    p.load(1, "UZP", L_MD)
    p.load(2, "bC_F", L_M)
    p.setlen(2, L_MD)
    p.dct(2, FWD_T, fft)                          # conv bar
    p.load(3, "A_Fx", L_MG)
    p.stencil(3, "CD")
    p.setlen(3, L_MD)
    p.load(4, "A_F0", L_MG)
    p.stencil(4, "CD")
    p.diff(4)
    p.scale(4, par=P_ISZ)
    p.setlen(4, L_MD)
    p.dct(3, BWD, fft, count=2)                   # dF/dx, dF/dz (physical)
    p.mul(3, 2)
    p.store(3, "bUX_F")                           # ux bar, this field's part
    p.load_add(4, "DTB1", par=P_TF)               # + DTB1 (temperature: the lift term)
    p.mul(4, 2)
    p.store(4, "bUZ_F")                           # uz bar, this field's part
    p.copy(3, 2)
    p.mul(3, 0)                                   # dF/dx bar = conv bar * ux
    p.mul(2, 1)                                   # dF/dz bar = conv bar * uz
    p.dct(2, BWD_T, fft, count=2)
    p.setlen(3, L_M)
    p.stencil_t(3, "CD")
    p.store(3, "bA_Fx")
    p.setlen(2, L_M)
    p.scale(2, par=P_ISZ)
    p.diff_t(2)
    p.stencil_t(2, "CD")
    p.store(2, "bA_F0")
    p.variants = [{"arrays": {"bC_F": "bC_" + F, "A_Fx": "A_" + F + "x", "A_F0": "A_" + F + "0",
                              "bA_Fx": "bA_" + F + "x", "bA_F0": "bA_" + F + "0", "bUX_F": "bUX_" + F,
                              "bUZ_F": "bUZ_" + F},
                   "par": {P_TF: 1.0 if F == "T" else 0.0}} for F in "UVT"]
    Q.append(p)

    p = Prog("Q2z", 1, L_ND, 1)   # per velocity component: ux bar -> A_U0 bar, uz bar -> A_V0 bar
    p.load(0, "bX_U", L_MD)
    p.load_add(0, "bX_V")
    p.load_add(0, "bX_T")
    if rk3:
        p.add("STORE", 0, arr="bXO", par=P_C)     # c_k part: the previous stage's velocity
        p.scale(0, par=P_B)
        p.load_add(0, "bXC")                      # + the next stage's c_(k+1) part on this velocity
    p.dct(0, BWD_T, fft)
    p.setlen(0, L_M)
    p.stencil_t(0, "CD")
    p.store_add(0, "bA_X0")
    p.variants = [{"arrays": {"bX_U": X + "U", "bX_V": X + "V", "bX_T": X + "T", "bA_X0": "bA_" + F + "0",
                              "bXO": X[:-1] + "O", "bXC": X[:-1] + "C"}}
                  for X, F in (("bUX_", "U"), ("bUZ_", "V"))]
    Q.append(p)

    # Q1 (x, M-2 lines), once per field: A_F0 = Bwd_x S_x F; A_Fx = Bwd_x D_x S_x F / sx
    p = Prog("Q1", 0, L_MG, 2)
    p.load(0, "bA_F0", L_ND)
    p.load(1, "bA_Fx", L_ND)
    p.dct(0, BWD_T, fft, count=2)
    p.setlen(0, L_N)
    p.setlen(1, L_N)
    p.scale(1, par=P_ISX)
    p.diff_t(1)
    p.axpy(0, 1)
    p.stencil_t(0, "F")
    p.store_add(0, "bFG")
    p.variants = [{"arrays": {"bA_F0": "bA_" + F + "0", "bA_Fx": "bA_" + F + "x", "bFG": "b" + F + "G"},
                   "tables": {"sten_F": "sten_" + kinds[F]}} for F in "UVT"]
    Q.append(p)
    return Q


def adjoint_shapes(N, M, Nd, Md, beta=False, rk3=False):
    """Intermediate arrays of the adjoint passes (name -> shape); ``rk3``: with the velocity
    gradients carried between stages (bUX_0 / bUX_1 for u_0 / u_1, a sink for stage 0's zero
    part and a zero input for stage 2)."""
    sh = {}
    if rk3:
        for X in ("bUX_", "bUZ_"):
            for k in ("0", "1", "S", "Z"):
                sh[X + k] = (Nd, Md)
    if beta:
        for F in "UVT":
            sh["bEY0_" + F] = (N - 2, M)
            sh["bEYY_" + F] = (N - 2, M)
    for k in ("bUS", "bVS", "bX", "bR2"):
        sh[k] = (N - 2, M - 2)
    for k in ("bG1", "bG2", "bY1", "bY2", "bW1", "bW2", "bR1", "bTSY"):
        sh[k] = (N - 2, M)
    for F in "UVT":
        sh["bQ1_" + F] = (N - 2, M)
        sh["bQ2_" + F] = (N - 2, M - 2)
        sh["bRHS_" + F] = (N, M)
        sh["bC_" + F] = (Nd, M)
        sh["bA_" + F + "0"] = (Nd, M - 2)
        sh["bA_" + F + "x"] = (Nd, M - 2)
    sh["bDPZ"] = (N, M)
    for k in ("bUX_U", "bUX_V", "bUX_T", "bUZ_U", "bUZ_V", "bUZ_T"):
        sh[k] = (Nd, Md)
    return sh


# stage k of the reverse RK3 step: carried gradient on its own velocity (C) and on the previous one (O)
RK3_CARRY = ({"bUXC": "bUX_0", "bUZC": "bUZ_0", "bUXO": "bUX_S", "bUZO": "bUZ_S"},
             {"bUXC": "bUX_1", "bUZC": "bUZ_1", "bUXO": "bUX_0", "bUZO": "bUZ_0"},
             {"bUXC": "bUX_Z", "bUZC": "bUZ_Z", "bUXO": "bUX_1", "bUZO": "bUZ_1"})


def add_adjoint_buffers(I, bar_views, beta=False):
    """Gradient arrays, scratch and transposed operator tables of one instance."""
    ns = I.ns
    N, M, Nd, Md = I.N, I.M, I.Nd, I.Md
    dev = device()
    a = I.arrays
    for k in BAR_STATE:
        a[k] = bar_views[k]
    rk3 = I.nstage == 3
    for k, shp in adjoint_shapes(N, M, Nd, Md, beta, rk3).items():
        a[k] = torch.zeros(shp, dtype=DTYPE, device=dev)
    if rk3:
        for st, carry in zip(I.stage_arrays, RK3_CARRY):
            st.update(carry)
    host = host_tables(N, M, ns.T.xs[0].id, ns.dt * float(ns.beta), ns.nu, ns.kappa, ns.scale, ns.solver_P._fd,
                       adjoint=True)
    for k in ("BxT", "ByT", "BSx_UT", "BSx_TT", "BSyT", "HyT", "QyT"):
        I.tables[k] = to_dev(host[k])


class FusedAdjoint(FusedBatch):
    """Forward and reverse fused steps for a batch of instances.

    ``state_arena`` holds the forward state of every instance (U, V, T, P,
    pres), ``bar_arena`` the gradient with respect to it, in the same layout.
    ``adjoint_step()`` replaces the gradient w.r.t. the state after one step
    taken from the current ``state_arena`` by the gradient w.r.t. that state.
    """

    def __init__(self, solvers, split=None):
        FusedBatch.__init__(self, solvers, split=split)
        self.bar_arena = torch.zeros_like(self.state_arena)
        for I, d in zip(self.insts, self.views(self.bar_arena, keys=_Instance.STATE)):
            add_adjoint_buffers(I, {"b" + key: v for key, v in d.items()}, self.beta)
        tkind = self.solvers[0].T.xs[0].id
        self.aprogs = build_adjoint_programs(tkind, self.fft, self.split, self.beta, rk3=self.nstage == 3)
        # per stage (RK3: its parameters, ADI tables and carried velocity gradients)
        self.alaunches_st = [[self._pass_launches(p, stage=k) for p in self.aprogs] for k in range(self.nstage)]
        self.alaunches = self.alaunches_st[0]
        self._snap = torch.zeros((2, self.state_arena.numel()), dtype=DTYPE, device=self.state_arena.device) \
            if self.nstage == 3 else None
        self.agraph = None

    def run_adjoint_pass(self, i, stage=0):
        for L in self.alaunches_st[stage][i]:
            self._run_launch(L)

    def adjoint_step_eager(self, recompute=True):
        """The reverse-mode passes; ``recompute=False`` skips R1 when the caller has put the
        step's P1 outputs (``a_arena``) in place itself (IMEX Euler)."""
        if self.nstage == 3:
            self._adjoint_step_rk3()
            return
        for i in range(0 if recompute else 1, len(self.alaunches)):
            self.run_adjoint_pass(i)

    def _adjoint_step_rk3(self):
        """Reverse of one three-stage step from its input X0 (state_arena, restored at the end):
        stages 0 and 1 run forward again (their outputs X1, X2; UX_A / UZ_A keep u_0 and UX_B / UZ_B
        u_1, since stage 2 is not rerun), then stages 2, 1, 0 run backward, each from its own input
        state (R1 recomputes the stage's P1 outputs)."""
        npass = len(self.progs)
        self._snap[0].copy_(self.state_arena)
        for i in range(npass):
            self.run_pass(i)
        self._snap[1].copy_(self.state_arena)
        for i in range(npass, 2 * npass):
            self.run_pass(i)
        for k in (2, 1, 0):
            if k < 2:
                self.state_arena.copy_(self._snap[k])
            for i in range(len(self.aprogs)):
                self.run_adjoint_pass(i, k)

    def adjoint_step(self):
        if self.agraph is not None and self._agraph_gen == self.launch_generation:
            self.agraph.replay()
        else:
            self.adjoint_step_eager()

    @property
    def adjoint_launches_per_step(self):
        n = sum(len(g) for st in self.alaunches_st for g in st)
        if self.nstage == 3:  # the forward recomputation of stages 0 and 1
            n += sum(len(g) for g in self.launches[:2 * len(self.progs)])
        return n

    def autotune_adjoint(self, reps=3, verbose=False):
        """Tile choice for every launch of the adjoint passes (state and gradients restored after)."""
        saved_s, saved_b = self.state_arena.clone(), self.bar_arena.clone()
        chosen = self._tune([g for st in self.alaunches_st for g in st], reps, verbose)
        self.state_arena.copy_(saved_s)
        self.bar_arena.copy_(saved_b)
        torch.cuda.synchronize()
        self.agraph = None
        self.atuned = chosen
        return chosen

    def capture_adjoint(self):
        """Record one adjoint step in a CUDA graph (``adjoint_step()`` then replays it)."""
        saved_s, saved_b = self.state_arena.clone(), self.bar_arena.clone()
        self.adjoint_step_eager()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.adjoint_step_eager()
        torch.cuda.synchronize()
        self.state_arena.copy_(saved_s)
        self.bar_arena.copy_(saved_b)
        self.agraph, self._agraph_gen = g, self.launch_generation

    # -- views of the per-instance state in the arenas
    def views(self, arena, keys=("UG", "VG", "TG")):
        """Per instance, views of ``keys`` into ``arena``, a tensor with the layout of ``state_arena``."""
        base, out = self.state_arena.data_ptr(), []
        for I in self.insts:
            d = {}
            for key in keys:
                r, c = I.arrays[key].shape
                off = (I.arrays[key].data_ptr() - base) // 8
                d[key] = arena[off:off + r * c].view(r, c)
            out.append(d)
        return out


class HorizonGradient:
    """Value and gradient of J_i(X_i) = ||Phi^H(X_i) - X_i||_2 for every instance of a batch,
    X = (U, V, T) with the pressure (and P) starting from zero, by the fused adjoint.

    Forward states are checkpointed every ``every`` steps during the forward
    sweep.  The reverse sweep recomputes each segment from its checkpoint
    (``every`` fused steps; what the adjoint passes read of each step, the P1
    outputs, is kept in a trajectory buffer) and steps it back with the
    adjoint passes.  With ``overlap`` the recomputation of
    segment s-1 runs on a second stream, on a private working copy of the
    batch, while the adjoint passes of segment s run on the main stream (two
    trajectory buffers alternate); a single small instance leaves most SMs
    idle in either sweep, so the two fill the GPU together.  With ``graph``
    the whole evaluation (forward sweep, objective, reverse sweep, both
    streams) is one CUDA graph: one replay per call.
    """

    def __init__(self, fa, nsteps, every=20, overlap=True, graph=True):
        self.fa, self.H, self.every = fa, nsteps, every
        self.overlap, self.use_graph = overlap, graph
        n = fa.state_arena.numel()
        self.nseg = -(-nsteps // every)
        dev = fa.state_arena.device
        z = lambda *shape: torch.zeros(shape, dtype=DTYPE, device=dev)  # noqa: E731
        self.ckpt = z(self.nseg, n)
        # per step of a segment: the P1 outputs (physical-space operands of the convection terms),
        # which is all the reverse-mode passes of an Euler step read of the forward state; for RK3
        # the step's input state (its reverse recomputes the stages from it)
        self.rk3 = fa.nstage == 3
        self.traj = z(2 if overlap else 1, every, n if self.rk3 else fa.a_arena.numel())
        self.x0, self.x_in, self.g_out, self.y_out, self.g_in = z(n), z(n), z(n), z(n), z(n)
        self.J_out = z(len(fa.insts))
        self._mask = z(n)
        for d in fa.views(self._mask):
            for v in d.values():
                v.fill_(1.0)
        self._state_mask = z(n)      # every input of a step: U, V, T, pres (not P)
        for d in fa.views(self._state_mask, keys=("UG", "VG", "TG", "PRES")):
            for v in d.values():
                v.fill_(1.0)
        self.rec = None
        if overlap:
            self.rec = FusedBatch(fa.solvers, bind=False, split=fa.split)
            self.rec._build_launches(fa.tiles())
            self.side = torch.cuda.Stream(device=dev)
        self.graphs = {}

    def _seg_len(self, s):
        return min(self.every, self.H - s * self.every)

    # ---------------------------------------------------------------- pieces
    def _forward_sweep(self, keep):
        fa = self.fa
        fa.state_arena.copy_(self.x0)
        for s in range(self.nseg):
            if keep:
                self.ckpt[s].copy_(fa.state_arena)
            for _ in range(self._seg_len(s)):
                fa.step_eager()

    def _objective(self):
        """r = (Phi^H(X) - X) on U, V, T; J per instance; returns (J, seed = r / J)."""
        fa = self.fa
        r = (fa.state_arena - self.x0) * self._mask
        J = torch.stack([torch.sqrt(sum((v * v).sum() for v in d.values())) for d in fa.views(r)])
        scale = torch.zeros_like(r)
        for d, j in zip(fa.views(scale), J):
            for v in d.values():
                v.copy_((1.0 / j).expand_as(v))
        return J, r * scale

    def _recompute(self, batch, s, buf):
        """P1 outputs (RK3: input states) of every step of segment s into traj[buf] (batch: a
        working set)."""
        k = self._seg_len(s)
        batch.state_arena.copy_(self.ckpt[s])
        for j in range(k):
            if self.rk3:
                self.traj[buf, j].copy_(batch.state_arena)
                if j + 1 < k:
                    batch.step_eager()
                continue
            if j + 1 < k:
                batch.step_eager()
            else:
                batch.run_pass(0)           # the last step only needs its P1
            self.traj[buf, j].copy_(batch.a_arena)

    def _reverse(self, s, buf):
        fa = self.fa
        for j in reversed(range(self._seg_len(s))):
            if self.rk3:
                fa.state_arena.copy_(self.traj[buf, j])
                fa.adjoint_step_eager()
            else:
                fa.a_arena.copy_(self.traj[buf, j])
                fa.adjoint_step_eager(recompute=False)

    def _reverse_sweep(self):
        if not self.overlap:
            for s in reversed(range(self.nseg)):
                self._recompute(self.fa, s, 0)
                self._reverse(s, 0)
            return
        main = torch.cuda.current_stream()
        ready = [torch.cuda.Event() for _ in range(self.nseg)]
        used = [torch.cuda.Event() for _ in range(self.nseg)]
        fork = torch.cuda.Event()
        fork.record(main)
        self.side.wait_event(fork)

        def issue_recompute(s):
            with torch.cuda.stream(self.side):
                if s + 2 < self.nseg:                  # traj[s % 2] was last read by segment s + 2
                    self.side.wait_event(used[s + 2])
                self._recompute(self.rec, s, s % 2)
                ready[s].record(self.side)

        last = self.nseg - 1
        issue_recompute(last)
        for s in reversed(range(self.nseg)):
            if s - 1 >= 0:
                issue_recompute(s - 1)
            main.wait_event(ready[s])
            self._reverse(s, s % 2)
            used[s].record(main)
        join = torch.cuda.Event()
        join.record(self.side)
        main.wait_event(join)

    def _run(self, what):
        """'value': objective; 'grad': objective and gradient; 'map': Phi^H(x0) into y_out (keeping
        the checkpoints); 'vjp': the reverse sweep of the last 'map' from the seed in g_in."""
        if what in ("value", "grad", "map"):
            self._forward_sweep(keep=what != "value")
        if what == "map":
            self.y_out.copy_(self.fa.state_arena)
            return
        if what == "vjp":
            self.fa.bar_arena.copy_(self.g_in)
            self._reverse_sweep()
            self.g_out.copy_(self.fa.bar_arena * self._state_mask)
            return
        J, seed = self._objective()
        self.J_out.copy_(J)
        if what == "grad":
            self.fa.bar_arena.copy_(seed)
            self._reverse_sweep()
            self.g_out.copy_((self.fa.bar_arena - seed) * self._mask)

    def _replay(self, what):
        if not self.use_graph:
            self._run(what)
            return
        gen = self.fa.launch_generation
        g, g_gen = self.graphs.get(what, (None, None))
        if g is not None and g_gen != gen:   # the batch's launches were rebuilt since: record again
            g = None
        if g is None:
            saved = (self.ckpt.clone(), self.y_out.clone()) if what == "vjp" else None
            self._run(what)                 # warm-up outside the capture
            torch.cuda.synchronize()
            if saved is not None:           # the warm-up sweep must not disturb the checkpoints
                self.ckpt.copy_(saved[0])
                self.y_out.copy_(saved[1])
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self._run(what)
            self.graphs[what] = (g, gen)
        g.replay()

    # ------------------------------------------------------------------- API
    def value(self, X):
        """J per instance for the initial states X (arena-shaped; only U, V, T entries are used)."""
        self.x_in.copy_(X)
        self.x0.copy_(self.x_in * self._mask)
        self._replay("value")
        return self.J_out.clone()

    def value_and_grad(self, X):
        """(J per instance, dJ/dX arena-shaped: U, V, T entries; zero elsewhere)."""
        self.x_in.copy_(X)
        self.x0.copy_(self.x_in * self._mask)
        self._replay("grad")
        return self.J_out.clone(), self.g_out.clone()

    # -- the horizon map and its vector-Jacobian product (for FusedHorizon)
    def forward_map(self, X):
        """Phi^H(X) over the whole state (U, V, T, P, pres in the arena layout); keeps the checkpoints
        for ``vjp``."""
        self.x0.copy_(X)
        self._replay("map")
        return self.y_out.clone()

    def vjp(self, gY):
        """d<gY, Phi^H(X)>/dX for the X of the last ``forward_map`` (P is not an input of a step:
        its entries of the result are zero, and a gradient on the final P is not propagated)."""
        self.g_in.copy_(gY)
        self._replay("vjp")
        return self.g_out.clone()



class HorizonGradientGroups:
    """Horizon gradients of many instances as ``groups`` independent FusedAdjoint / HorizonGradient
    pairs (contiguous instance groups), each replayed on its own stream: the groups' sequential
    sweeps overlap, filling the SMs that one group's small launches leave idle."""

    def __init__(self, solvers, nsteps, every=20, groups=4, tune=True):
        bounds = [round(len(solvers) * g / groups) for g in range(groups + 1)]
        self.parts = []
        for a, b in zip(bounds[:-1], bounds[1:]):
            if b <= a:
                continue
            fa = FusedAdjoint(solvers[a:b])
            if tune:
                fa.autotune(reps=2)
                fa.autotune_adjoint(reps=2)
            self.parts.append((fa, HorizonGradient(fa, nsteps, every), torch.cuda.Stream()))

    def states(self):
        """Copies of every group's state arena (the layout value_and_grad takes)."""
        return [fa.state_arena.clone() for fa, _, _ in self.parts]

    def value_and_grad(self, Xs):
        """[(J, dJ/dX)] per group for the group states ``Xs``; the current stream waits for all."""
        main = torch.cuda.current_stream()
        out = []
        for (_, hg, st), X in zip(self.parts, Xs):
            st.wait_stream(main)
            with torch.cuda.stream(st):
                J, g = hg.value_and_grad(X)
            J.record_stream(main)
            g.record_stream(main)
            out.append((J, g))
        for _, _, st in self.parts:
            main.wait_stream(st)
        return out


class FusedHorizon(torch.autograd.Function):
    """Y = Phi^H(X) on the fused passes, differentiable: backward runs the fused reverse-mode
    passes over the checkpointed horizon.  X and Y are whole-batch state arenas (``fa.views``
    gives the per-instance U, V, T, P, pres); the gradient flows to U, V, T and pres.

        hg = HorizonGradient(FusedAdjoint(solvers), nsteps=200, every=20)
        Y = FusedHorizon.apply(X, hg)       # X.requires_grad_()
        loss = any_function_of(Y, X); loss.backward()
    """

    @staticmethod
    def forward(ctx, X, hg):
        ctx.hg = hg
        return hg.forward_map(X.detach())

    @staticmethod
    def backward(ctx, gY):
        return ctx.hg.vjp(gY.contiguous()), None
