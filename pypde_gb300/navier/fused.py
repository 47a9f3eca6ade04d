"""Fused Rayleigh-Benard step: eleven line-program passes per IMEX Euler step.

The plain path (``NavierStokes.update``) launches one kernel per pypde
operation (~150 launches per step).  Here the same step is regrouped into
passes that each stream every array once through shared memory and chain all
1-D operators along that axis: stencil, derivative recurrence, pad, DCT-I,
pointwise products, forward DCT, unpad, pseudo-inverse B, four-diagonal LU
sweep, ...  Operators acting along different axes commute, so x- and y-parts of
the reference's sequence (rbc2d.py:396-434) are grouped per axis:

  P1  x  S_x, D_x, pad, DCT^-1 of U, V, T          -> A_F0, A_Fx   (Nd x M-2)
  P2  y  S_y, D_y, pad, DCT^-1; ux, uz; products;  -> C_F          (Nd x M)
         forward DCT_y + unpad; D_y pres; S_y T
  P3  x  forward DCT_x + unpad; rhs (pressure, buoyancy, BC terms) -> RHS_F
  P3s x  B_x; A_x^-1 (ADI x-sweep); old terms B_x S_x F    -> Q1_F, Q2_F
  P4  y  B_y Q1 + B_y S_y Q2; A_y^-1 -> U*, V*, T^{n+1}; S_y U*, D_y S_y V*
  P5  x  divergence; pres -= nu div; B_x div              -> R1
  P6  y  H_y (fast-diagonalisation rhs)                   -> R2
  P7  x  per-eigenvalue Poisson sweep                     -> X
  P8  y  Q_y, P[0,0] = 0; S_y P, D_y S_y P
  P9  x  pres += S P / dt; grad P; (S^T S)^-1 S^T (x)     -> G1, G2
  P10 y  (S^T S)^-1 S^T (y); U = U* - G1, V = V* - G2

A batch of independent instances (any sizes, any Rayleigh numbers) runs the
same eleven launches: every CTA picks (instance, tile) from a work list, so one
launch per pass covers all instances.  ``capture()`` records the passes of a
step in a CUDA graph.
"""
import ctypes

import numpy as np
import torch

from .. import _lib
from .._dev import DTYPE, device, stream, to_dev
from ..host import fdma_lu, pseudoinverse_d2, stencil_matrix, stencil_sub

# fixed len[] indices
L_LINES, L_N, L_M, L_NG, L_MG, L_ND, L_MD = range(7)
# fixed par[] indices
P_ISX, P_ISZ, P_MDT, P_DT, P_DTK, P_MDTSX, P_MDTSZ, P_MNU, P_IDT, P_B, P_C, P_TF, P_EDU, P_EDT = range(14)

FFT_RADICES = (2, 3)


def fft_ok(n):
    L = 2 * (n - 1)
    for r in FFT_RADICES:
        while L % r == 0 and L > 1:
            L //= r
    return L == 1


class Prog:
    """Builder of one line program with symbolic arrays and tables."""

    def __init__(self, name, axis, lines, nslots):
        self.name, self.axis, self.lines, self.nslots = name, axis, lines, nslots
        self.ops, self.arrs, self.mats = [], {}, {}
        self.has_dct = False
        # variants: the same program run as several descriptors per instance, each renaming
        # arrays / tables and overriding parameters ({"arrays": {}, "tables": {}, "par": {}})
        self.variants = [{}]

    def _a(self, name):
        return self.arrs.setdefault(name, len(self.arrs))

    def _m(self, name):
        return self.mats.setdefault(name, len(self.mats))

    def add(self, code, a=0, b=-1, arr=None, mat=None, len=-1, k=0, alpha=1.0, par=-1):  # noqa: A002
        self.ops.append(_lib.op(code, a=a, b=b, arr=-1 if arr is None else self._a(arr),
                                mat=-1 if mat is None else self._m(mat), len=len, k=k, alpha=alpha, par=par))

    # convenience
    def load(self, s, arr, n, alpha=1.0, par=-1):
        self.add("LOAD", s, arr=arr, len=n, alpha=alpha, par=par)

    def load_add(self, s, arr, alpha=1.0, par=-1):
        self.add("LOAD_ADD", s, arr=arr, alpha=alpha, par=par)

    def store(self, s, arr):
        self.add("STORE", s, arr=arr)

    def stencil(self, s, kind):
        self.add("STENCIL", s, mat="sten_" + kind)

    def stencil_t(self, s, kind):
        self.add("STENCIL_T", s, mat="sten_" + kind)

    def tdma(self, s, kind):
        self.add("TDMA2", s, mat="tdma_" + kind)

    def diff(self, s, count=1):
        self.add("DIFF", s, k=count)

    def scale(self, s, alpha=1.0, par=-1):
        self.add("SCALE", s, alpha=alpha, par=par)

    def axpy(self, s, src, alpha=1.0, par=-1):
        self.add("AXPY", s, b=src, alpha=alpha, par=par)

    def mul(self, s, src):
        self.add("MUL", s, b=src)

    def copy(self, s, src):
        self.add("COPY", s, b=src)

    def setlen(self, s, n):
        self.add("SETLEN", s, len=n)

    _DENSE_DCT = {_lib.DCT_FWD: "dct_fwd", _lib.DCT_BWD: "dct_bwd", _lib.DCT_FWD_T: "dct_fwd_t",
                  _lib.DCT_BWD_T: "dct_bwd_t"}

    def dct(self, s, mode, fft, count=1):
        """DCT-I (``mode``) of slots s .. s+count-1, which hold lines of one length: one DCT
        op for all of them (each phase of the transform runs over every slot's lines at once),
        or ``count`` dense-matrix ops."""
        self.has_dct = True
        if fft:
            self._m(self._DENSE_DCT[mode])  # the dense form, for launches that contract on tensor cores
            self.add("DCT", s, b=count, mat="dct", k=mode)
        else:
            for i in range(count):
                self.add("DENSE", s + i, mat=self._DENSE_DCT[mode], len=L_ND + self.axis)

    def banded(self, s, name, off0, ndiag, rows):
        self.add("BANDED", s, b=off0, mat=name, len=rows, k=ndiag)

    def dense(self, s, name, rows):
        self.add("DENSE", s, mat=name, len=rows)

    def fdma(self, s, names, code="FDMA"):
        """One FDMA op over consecutive slots s, s+1, ... with factor tables ``names``
        (``code`` FDMA_T: the transposed solve with the same factors)."""
        if isinstance(names, str):
            names = [names]
        first = None
        for i, nm in enumerate(names):
            key = "%s#%d.%d" % (nm, len(self.ops), i)  # fresh keys -> consecutive table indices
            idx = self._m(key)
            first = idx if first is None else first
            assert idx == first + i
        self.ops.append(_lib.op(code, a=s, b=len(names), mat=first))

    def fdma_t(self, s, names):
        self.fdma(s, names, code="FDMA_T")

    def diff_t(self, s, count=1):
        self.add("DIFF_T", s, k=count)

    def store_add(self, s, arr, alpha=1.0, par=-1):
        self.add("STORE_ADD", s, arr=arr, alpha=alpha, par=par)

    def tdma_multi(self, s, count, kind):
        self.add("TDMA2", s, b=count, mat="tdma_" + kind)


def _split_convection_programs(tkind, fft, rk3, beta=False):
    """P1, P2u, P2, P3, P3rs with P1 / P2 / P3 written once for a generic field F (variants)."""
    BWD, FWD = _lib.DCT_BWD, _lib.DCT_FWD
    kinds = {"U": "CD", "V": "CD", "T": tkind}
    P = []
    p = Prog("P1", 0, L_MG, 2)
    p.load(0, "FG", L_NG)
    p.stencil(0, "F")
    p.copy(1, 0)
    p.diff(1)
    p.scale(1, par=P_ISX)
    p.setlen(0, L_ND)
    p.setlen(1, L_ND)
    p.dct(0, BWD, fft, count=2)
    p.store(0, "A_F0")
    p.store(1, "A_Fx")
    p.variants = [{"arrays": {"FG": F + "G", "A_F0": "A_" + F + "0", "A_Fx": "A_" + F + "x"},
                   "tables": {"sten_F": "sten_" + kinds[F]}} for F in "UVT"]
    P.append(p)

    p = Prog("P2u", 1, L_ND, 2)
    for s, F in ((0, "U"), (1, "V")):
        p.load(s, "A_" + F + "0", L_MG)
        p.stencil(s, "CD")
        p.setlen(s, L_MD)
    p.dct(0, BWD, fft, count=2)
    if rk3:
        for s, C, O in ((0, "UXC", "UXO"), (1, "UZC", "UZO")):
            p.store(s, C)
            p.scale(s, par=P_B)
            p.load_add(s, O, par=P_C)
    p.store(0, "UXP")
    p.store(1, "UZP")
    p.load(0, "PRES", L_M)
    p.diff(0)
    p.store(0, "DPZ")
    p.load(0, "TG", L_MG)
    p.stencil(0, "CD")
    p.store(0, "TSY")
    P.append(p)

    p = Prog("P2", 1, L_ND, 4)
    p.load(0, "UXP", L_MD)
    p.load(1, "UZP", L_MD)
    p.load(2, "A_Fx", L_MG)
    p.stencil(2, "CD")
    p.setlen(2, L_MD)
    p.load(3, "A_F0", L_MG)
    p.stencil(3, "CD")
    p.diff(3)
    p.scale(3, par=P_ISZ)
    p.setlen(3, L_MD)
    p.dct(2, BWD, fft, count=2)
    p.mul(2, 0)
    p.load_add(3, "DTB1", par=P_TF)         # temperature: + the lift's dT/dz
    p.mul(3, 1)
    p.axpy(2, 3)
    p.dct(2, FWD, fft)
    p.setlen(2, L_M)
    p.store(2, "C_F")
    p.variants = [{"arrays": {"A_Fx": "A_" + F + "x", "A_F0": "A_" + F + "0", "C_F": "C_" + F},
                   "par": {P_TF: 1.0 if F == "T" else 0.0}} for F in "UVT"]
    P.append(p)

    p = Prog("P3", 0, L_M, 1)
    p.load(0, "C_F", L_ND)
    p.dct(0, FWD, fft)
    p.setlen(0, L_N)
    p.scale(0, par=P_MDT)
    p.store(0, "RHS_F")
    p.variants = [{"arrays": {"C_F": "C_" + F, "RHS_F": "RHS_" + F}} for F in "UVT"]
    P.append(p)

    # P3rs (x, lines M): the non-convective right-hand-side terms, then B_x and the ADI x-sweeps
    # (the same axis and lines: one pass)
    p = Prog("P3rs", 0, L_M, 6)
    for i, F in enumerate("UVT"):
        p.load(i, "RHS_" + F, L_N)
    p.load(3, "PRES", L_N)
    p.diff(3)
    p.axpy(0, 3, par=P_MDTSX)
    p.load_add(1, "DPZ", par=P_MDTSZ)
    p.load_add(1, "TBCC", par=P_DT)
    p.load(3, "TSY", L_NG)
    p.stencil(3, tkind)
    p.axpy(1, 3, par=P_DT)
    p.load_add(2, "DTB2", par=P_DTK)
    if beta:
        for i, F in enumerate("UVT"):
            _explicit_diffusion_x(p, 3, F, kinds[F])
            p.axpy(i, 3, par=P_EDT if F == "T" else P_EDU)
    _adi_x(p, kinds)
    P.append(p)
    return P


def _adi_x(p, kinds):
    """B_x on the right-hand sides in slots 0-2 and the ADI x-sweep of them and of the old-time
    terms B_x S_x F (slots 3-5): the six independent sweeps as one multi-slot chain op; stores
    Q1_F, Q2_F."""
    ax = {"U": "Ax_U", "V": "Ax_U", "T": "Ax_T"}
    for i, F in enumerate("UVT"):
        p.banded(i, "Bx", 0, 3, L_NG)
        p.load(3 + i, F + "G", L_NG)
        p.banded(3 + i, "BSx_T" if F == "T" else "BSx_U", -2, 4, L_NG)
    p.fdma(0, [ax[F] for F in "UVT"] + [ax[F] for F in "UVT"])
    for i, F in enumerate("UVT"):
        p.store(i, "Q1_" + F)
        p.store(3 + i, "Q2_" + F)


def _explicit_diffusion_y():
    """P2e (y, lines N-2): S_y F and D_y^2 S_y F / sz^2 of the state, the y-halves of the explicit
    diffusion (1 - beta) dt a nu (d_xx + d_zz) F of rbc2d.py:268-283 (x-halves in P3)."""
    p = Prog("P2e", 1, L_NG, 1)
    for F in "UVT":
        p.load(0, F + "G", L_MG)
        p.stencil(0, "CD")
        p.store(0, "EY0_" + F)
        p.diff(0, count=2)
        p.scale(0, par=P_ISZ)
        p.scale(0, par=P_ISZ)
        p.store(0, "EYY_" + F)
    return p


def _explicit_diffusion_x(p, s, F, kind):
    """Slot s = D_x^2 S_x EY0_F / sx^2 + S_x EYY_F (Chebyshev x Chebyshev); uses slot s + 1."""
    p.load(s, "EY0_" + F, L_NG)
    p.stencil(s, kind)
    p.diff(s, count=2)
    p.scale(s, par=P_ISX)
    p.scale(s, par=P_ISX)
    p.load(s + 1, "EYY_" + F, L_NG)
    p.stencil(s + 1, kind)
    p.axpy(s, s + 1)


def build_programs(tkind, fft, rk3=False, split=False, beta=False):
    """The eleven passes of one IMEX Euler step.  ``tkind`` is the x-basis of T
    ("CD" for the linear / zero cases, "CN" for rbc).

    ``rk3``: the passes of one stage of the three-stage IMEX Runge-Kutta step
    (rbc2d_base.py:86-102).  The stage coefficients arrive as per-stage parameters
    (dt a, 1/(dt a), b, c) and per-stage ADI tables; the convection of the stage,
    b conv(u) + c conv(u_old) (rbc2d.py:252-378), is the product with the
    combined velocity b u + c u_old, since conv is linear in the velocity.  P2
    keeps the stage's physical velocities for the next stage (UXC, UZC) and reads
    the previous stage's (UXO, UZO).

    ``split``: P1 - P3 as per-field programs run as three descriptors of one launch
    (U, V, T), plus P2u (velocities, D_y pres, S_y T) and P3rs (the non-convective
    right-hand-side terms and the ADI x-sweeps): the same transforms in twelve passes, with three
    times the CTAs in the transform-heavy ones - for batches of few instances.

    ``beta``: diffusion beta-implicit (beta != 1, rbc2d.py:268-283, 390-391): the ADI tables and the
    pressure update carry beta (per-instance tables and parameters), and an extra pass P2e with
    additions to P3 (P3rs in the per-field form) put the explicit part into the right-hand sides."""
    P = []
    BWD, FWD = _lib.DCT_BWD, _lib.DCT_FWD
    kinds = {"U": "CD", "V": "CD", "T": tkind}

    if split:
        P += _split_convection_programs(tkind, fft, rk3, beta)
        if beta:
            P.insert(3, _explicit_diffusion_y())   # P1, P2u, P2, P2e, P3, P3rs
    else:
        # P1 (x, lines M-2): physical-in-x parts of F and dF/dx
        p = Prog("P1", 0, L_MG, 2)
        for F in "UVT":
            p.load(0, F + "G", L_NG)
            p.stencil(0, kinds[F])
            p.copy(1, 0)
            p.diff(1)
            p.scale(1, par=P_ISX)
            p.setlen(0, L_ND)
            p.setlen(1, L_ND)
            p.dct(0, BWD, fft, count=2)
            p.store(0, "A_" + F + "0")
            p.store(1, "A_" + F + "x")
        P.append(p)

        # P2 (y, lines Nd): velocities, products, forward y-transform; D_y pres; S_y T
        p = Prog("P2", 1, L_ND, 4)
        for s, F in ((0, "U"), (1, "V")):
            p.load(s, "A_" + F + "0", L_MG)
            p.stencil(s, "CD")
            p.setlen(s, L_MD)
        p.dct(0, BWD, fft, count=2)
        if rk3:
            for s, C, O in ((0, "UXC", "UXO"), (1, "UZC", "UZO")):
                p.store(s, C)
                p.scale(s, par=P_B)
                p.load_add(s, O, par=P_C)
        for F in "UVT":
            p.load(2, "A_" + F + "x", L_MG)
            p.stencil(2, "CD")
            p.setlen(2, L_MD)
            p.load(3, "A_" + F + "0", L_MG)
            p.stencil(3, "CD")
            p.diff(3)
            p.scale(3, par=P_ISZ)
            p.setlen(3, L_MD)
            p.dct(2, BWD, fft, count=2)
            p.mul(2, 0)
            p.mul(3, 1)
            p.axpy(2, 3)
            if F == "T":
                p.load(3, "DTB1", L_MD)
                p.mul(3, 1)
                p.axpy(2, 3)
            p.dct(2, FWD, fft)
            p.setlen(2, L_M)
            p.store(2, "C_" + F)
        p.load(2, "PRES", L_M)
        p.diff(2)
        p.store(2, "DPZ")
        p.load(2, "TG", L_MG)
        p.stencil(2, "CD")
        p.store(2, "TSY")
        P.append(p)

        if beta:
            P.append(_explicit_diffusion_y())
        # P3 (x, lines M): forward x-transform, right-hand sides; P3s: B_x and the ADI x-sweeps (as
        # one pass with P3 the batch ran 2 % slower: more shared memory, fewer CTAs per SM)
        p = Prog("P3", 0, L_M, 5 if beta else 4)
        for i, F in enumerate("UVT"):
            p.load(i, "C_" + F, L_ND)
        p.dct(0, FWD, fft, count=3)
        for i, F in enumerate("UVT"):
            p.setlen(i, L_N)
            p.scale(i, par=P_MDT)
            if F == "U":
                p.load(3, "PRES", L_N)
                p.diff(3)
                p.axpy(i, 3, par=P_MDTSX)
            elif F == "V":
                p.load_add(i, "DPZ", par=P_MDTSZ)
                p.load_add(i, "TBCC", par=P_DT)
                p.load(3, "TSY", L_NG)
                p.stencil(3, tkind)
                p.axpy(i, 3, par=P_DT)
            else:
                p.load_add(i, "DTB2", par=P_DTK)
            if beta:
                _explicit_diffusion_x(p, 3, F, kinds[F])
                p.axpy(i, 3, par=P_EDT if F == "T" else P_EDU)
            p.store(i, "RHS_" + F)
        P.append(p)
        p = Prog("P3s", 0, L_M, 6)
        for i, F in enumerate("UVT"):
            p.load(i, "RHS_" + F, L_N)
        _adi_x(p, kinds)
        P.append(p)

    # P4 (y, lines N-2): B_y, ADI y-sweep -> U*, V*, T; divergence pieces
    p = Prog("P4", 1, L_NG, 4)
    for i, F in enumerate("UVT"):
        p.load(i, "Q1_" + F, L_M)
        p.banded(i, "By", 0, 3, L_MG)
        p.load(3, "Q2_" + F, L_MG)
        p.banded(3, "BSy", -2, 4, L_MG)
        p.axpy(i, 3)
    p.fdma(0, ["Ay_U", "Ay_U", "Ay_T"])
    for i, F in enumerate("UVT"):
        p.store(i, F + "G")
    p.stencil(0, "CD")
    p.store(0, "W1")
    p.stencil(1, "CD")
    p.diff(1)
    p.scale(1, par=P_ISZ)
    p.store(1, "W2")
    P.append(p)

    # P5 (x, lines M): divergence, pres -= nu div, B_x div
    p = Prog("P5", 0, L_M, 2)
    p.load(0, "W1", L_NG)
    p.stencil(0, "CD")
    p.diff(0)
    p.scale(0, par=P_ISX)
    p.load(1, "W2", L_NG)
    p.stencil(1, "CD")
    p.axpy(0, 1)
    p.load(1, "PRES", L_N)
    p.axpy(1, 0, par=P_MNU)
    p.store(1, "PRES")
    p.banded(0, "Bx", 0, 3, L_NG)
    p.store(0, "R1")
    P.append(p)

    # P6 (y, lines N-2): H_y
    p = Prog("P6", 1, L_NG, 1)
    p.load(0, "R1", L_M)
    p.dense(0, "Hy", L_MG)
    p.store(0, "R2")
    P.append(p)

    # P7 (x, lines M-2): per-eigenvalue four-diagonal sweep
    p = Prog("P7", 0, L_MG, 1)
    p.load(0, "R2", L_NG)
    p.add("POISSON", 0, mat="Pois")
    p.store(0, "X")
    P.append(p)

    # P8 (y, lines N-2): Q_y, P[0,0] = 0, S_y P, D_y S_y P
    p = Prog("P8", 1, L_NG, 1)
    p.load(0, "X", L_MG)
    p.dense(0, "Qy", L_MG)
    p.add("ZERO00", 0)
    p.store(0, "PG")
    p.stencil(0, "CN")
    p.store(0, "Y1")
    p.diff(0)
    p.scale(0, par=P_ISZ)
    p.store(0, "Y2")
    P.append(p)

    # P9 (x, lines M): pres += S_x S_y P / dt; grad P -> from_chebyshev along x
    p = Prog("P9", 0, L_M, 3)
    p.load(0, "Y1", L_NG)
    p.stencil(0, "CN")
    p.load(2, "PRES", L_N)
    p.axpy(2, 0, par=P_IDT)
    p.store(2, "PRES")
    p.diff(0)
    p.scale(0, par=P_ISX)
    p.stencil_t(0, "CD")
    p.load(1, "Y2", L_NG)
    p.stencil(1, "CN")
    p.stencil_t(1, "CD")
    p.tdma_multi(0, 2, "CD")
    p.store(0, "G1")
    p.store(1, "G2")
    P.append(p)

    # P10 (y, lines N-2): from_chebyshev along y, velocity correction
    p = Prog("P10", 1, L_NG, 3)
    p.load(0, "G1", L_M)
    p.stencil_t(0, "CD")
    p.load(1, "G2", L_M)
    p.stencil_t(1, "CD")
    p.tdma_multi(0, 2, "CD")
    for i, F in enumerate("UV"):
        p.load(2, F + "G", L_MG)
        p.axpy(2, i, alpha=-1.0)
        p.store(2, F + "G")
    P.append(p)
    return P


_GLOBAL = {}


def global_tables_host():
    """Length-independent tables: stencil sub-diagonals and offset-2 TDMA factors.

    For the Shen CD / CN stencils S[i+2, i] depends on i only, and so do the
    forward factors of the TDMA on S^T S (the last two w_i of a shorter system
    are never used by the sweep), so one long table serves every size.
    """
    n = _lib.LMAX - 8
    t = {}
    for kind in ("CD", "CN"):
        sub = stencil_sub(kind, n + 2)
        t["sten_" + kind] = np.concatenate([sub, np.zeros(2)])
        b = 1.0 + sub * sub
        a = sub.copy()
        c = sub.copy()
        w = np.zeros(n)
        rden = np.zeros(n)
        aa = np.zeros(n)
        for i in range(n):
            den = b[i] if i < 2 else b[i] - a[i - 2] * w[i - 2]
            w[i] = c[i] / den
            rden[i] = 1.0 / den
            aa[i] = 0.0 if i < 2 else a[i - 2] / den
        # interleaved (a r, r, w): the forward sweep g_i = r_i x_i - (a r)_i g_{i-2}
        t["tdma_" + kind] = np.stack([aa, rden, w], axis=1).ravel()
    return t


def _global_tables():
    """global_tables_host() on the current device (built once per device)."""
    dev = torch.cuda.current_device()
    if dev not in _GLOBAL:
        _GLOBAL[dev] = {k: to_dev(v) for k, v in global_tables_host().items()}
    return _GLOBAL[dev]


def _banded_table(A, off0, ndiag):
    rows, cols = A.shape
    tab = np.zeros((ndiag, rows))
    for d in range(ndiag):
        for r in range(rows):
            c = r + off0 + 2 * d
            if 0 <= c < cols:
                tab[d, r] = A[r, c]
    # every nonzero of A must be on the stored diagonals
    R = np.zeros_like(A)
    for d in range(ndiag):
        for r in range(rows):
            c = r + off0 + 2 * d
            if 0 <= c < cols:
                R[r, c] = tab[d, r]
    assert np.array_equal(R, A), "matrix is not banded on the expected diagonals"
    return tab.ravel()


def _fdma_table(A):
    """[l | 1/d | u1/d | u2/d]: the upper factor pre-scaled so each back-substitution step is
    one FMA on the dependency chain."""
    l, d, u1, u2 = fdma_lu(A)
    n = d.size
    tab = np.zeros((4, n))
    tab[0, 2:] = l
    tab[1] = 1.0 / d
    tab[2, :n - 2] = u1 / d[:n - 2]
    tab[3, :n - 4] = u2 / d[:n - 4]
    return tab.ravel()


def _poisson_table(Ax, Cx, lam):
    """Per-eigenvalue LU factors of A + lam_j C with the singular rule (fdma.f90:146-185),
    laid out [l | 1/d | u1/d | u2/d] per line; a singular line solves rows 1: and has 1/d_0 = 0."""
    n = Ax.shape[0]
    m = lam.size
    tab = np.zeros((m, 4, n))
    for j in range(m):
        o = 1 if abs(lam[j]) < 1e-10 else 0
        A = (Ax + Cx * lam[j])[o:, o:]
        l, d, u1, u2 = fdma_lu(A)
        ns = n - o
        tab[j, 0, o + 2:] = l
        tab[j, 1, o:] = 1.0 / d
        tab[j, 2, o:o + ns - 2] = u1 / d[:ns - 2]
        tab[j, 3, o:o + ns - 4] = u2 / d[:ns - 4]
    return tab.ravel()


def dense_dct_host(n):
    """Dense DCT matrices (n x n, row-major) with the Chebyshev scalings folded in, and their transposes."""
    N = n - 1
    k = np.arange(n)[:, None]
    j = np.arange(n)[None, :]
    C = 2.0 * np.cos(np.pi * ((j * k) % (2 * N)) / N)
    C[:, 0] = 1.0
    C[:, -1] = (-1.0) ** np.arange(n)
    pre = np.where((j == 0) | (j == N), 1.0, 0.5) * (-1.0) ** j
    post = np.where((k == 0) | (k == N), 0.5 / N, 1.0 / N) * (-1.0) ** k
    bwd, fwd = C * pre, C * post
    return {"dct_bwd": bwd, "dct_fwd": fwd, "dct_bwd_t": np.ascontiguousarray(bwd.T),
            "dct_fwd_t": np.ascontiguousarray(fwd.T)}


_DENSE_DCT_CACHE = {}


def _dense_dct_tables(n):
    """Dense DCT matrices of length n on the current device, shared by every instance."""
    key = (torch.cuda.current_device(), n)
    if key not in _DENSE_DCT_CACHE:
        _DENSE_DCT_CACHE[key] = {k: to_dev(v) for k, v in dense_dct_host(n).items()}
    return _DENSE_DCT_CACHE[key]


def _dct_tables(n, fft):
    """Twiddles of the FFT-based DCT op (``fft``) and the dense matrices of the DENSE form."""
    t = dict(_dense_dct_tables(n))
    if fft:
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().pgx_dct_table(n, ctypes.byref(h)), "dct table")
        t["dct"] = h.value
    return t


def host_tables(N, M, tk, dt, nu, kappa, scale, fd, adjoint=False):
    """Operator tables of one instance (host, device layout): banded B / B S, the
    pre-factored ADI sweeps, the Poisson per-eigenvalue factors, H_y, Q_y and, with
    ``adjoint``, the transposed tables of the reverse-mode passes.  ``fd`` holds the
    fast-diagonalisation matrices Ax, Cx, wy, Qy, Hy of the pressure plan."""
    sx, sz = scale
    t = {}
    Bx, By = pseudoinverse_d2(N)[2:, :], pseudoinverse_d2(M)[2:, :]
    Sx_U, Sx_T, Sy = stencil_matrix("CD", N), stencil_matrix(tk, N), stencil_matrix("CD", M)
    t["Bx"] = _banded_table(Bx, 0, 3)
    t["By"] = _banded_table(By, 0, 3)
    t["BSx_U"] = _banded_table(Bx @ Sx_U, -2, 4)
    t["BSx_T"] = _banded_table(Bx @ Sx_T, -2, 4)
    t["BSy"] = _banded_table(By @ Sy, -2, 4)
    Ix, Iy = np.eye(N)[2:, :], np.eye(M)[2:, :]
    lu, lt = dt * nu, dt * kappa
    t["Ax_U"] = _fdma_table(Bx @ Sx_U - lu / sx ** 2 * Ix @ Sx_U)
    t["Ax_T"] = _fdma_table(Bx @ Sx_T - lt / sx ** 2 * Ix @ Sx_T)
    t["Ay_U"] = _fdma_table(By @ Sy - lu / sz ** 2 * Iy @ Sy)
    t["Ay_T"] = _fdma_table(By @ Sy - lt / sz ** 2 * Iy @ Sy)
    t["Pois"] = _poisson_table(np.asarray(fd["Ax"]), np.asarray(fd["Cx"]), np.real(fd["wy"]))
    Hy, Qy = np.real(np.asarray(fd["Hy"])), np.real(np.asarray(fd["Qy"]))
    t["Hy"] = np.ascontiguousarray(Hy)
    t["Qy"] = np.ascontiguousarray(Qy)
    if adjoint:
        T = lambda A: np.ascontiguousarray(A.T)  # noqa: E731
        t["BxT"] = _banded_table(T(Bx), -4, 3)
        t["ByT"] = _banded_table(T(By), -4, 3)
        t["BSx_UT"] = _banded_table(T(Bx @ Sx_U), -4, 4)
        t["BSx_TT"] = _banded_table(T(Bx @ Sx_T), -4, 4)
        t["BSyT"] = _banded_table(T(By @ Sy), -4, 4)
        t["HyT"] = T(Hy)
        t["QyT"] = T(Qy)
    return t


def instance_params(N, M, dealias, dt, nu, kappa, scale, a=1.0, b=1.0, c=0.0, beta=1.0):
    """len[] and par[] of one instance (indices L_* and P_*) for the stage coefficients a, b, c
    (IMEX Euler: 1, 1, 0) and the implicit fraction ``beta`` of the diffusion."""
    Nd, Md = (int(1.5 * N), int(1.5 * M)) if dealias else (N, M)
    sx, sz = scale
    lens = [0, N, M, N - 2, M - 2, Nd, Md]
    da = dt * a
    par = [1.0 / sx, 1.0 / sz, -dt, da, da * kappa, -da / sx, -da / sz, -nu * beta, 1.0 / da, b, c, 0.0,
           da * (1.0 - beta) * nu, da * (1.0 - beta) * kappa]
    return lens, par


A_KEYS = ("A_U0", "A_Ux", "A_V0", "A_Vx", "A_T0", "A_Tx")


def scratch_shapes(N, M, Nd, Md, beta=False):
    """Intermediate arrays of the forward passes (name -> shape); ``beta``: with those of the
    explicit diffusion (beta != 1)."""
    sh = {}
    if beta:
        for F in "UVT":
            sh["EY0_" + F] = (N - 2, M)
            sh["EYY_" + F] = (N - 2, M)
    for F in "UVT":
        sh["A_" + F + "0"] = (Nd, M - 2)
        sh["A_" + F + "x"] = (Nd, M - 2)
        sh["C_" + F] = (Nd, M)
        sh["RHS_" + F] = (N, M)
        sh["Q1_" + F] = (N - 2, M)
        sh["Q2_" + F] = (N - 2, M - 2)
    sh["DPZ"] = (N, M)
    sh["TSY"] = (N - 2, M)
    sh["UXP"] = (Nd, Md)
    sh["UZP"] = (Nd, Md)
    for k in ("W1", "W2", "R1", "Y1", "Y2", "G1", "G2"):
        sh[k] = (N - 2, M)
    sh["R2"] = (N - 2, M - 2)
    sh["X"] = (N - 2, M - 2)
    return sh


class _Instance:
    """Device state, scratch and operator tables of one RBC instance."""

    STATE = ("UG", "VG", "TG", "PG", "PRES")

    @staticmethod
    def state_shapes(ns):
        N, M = ns.shape
        return {"UG": (N - 2, M - 2), "VG": (N - 2, M - 2), "TG": (N - 2, M - 2), "PG": (N - 2, M - 2),
                "PRES": (N, M)}

    def __init__(self, ns, fft, views=None, bind=True, beta=False):
        if ns.nstage not in (1, 3):
            raise NotImplementedError("the fused step covers IMEX Euler and RK3; use update() otherwise")
        self.ns = ns
        N, M = ns.shape
        Nd, Md = (int(1.5 * N), int(1.5 * M)) if ns.dealias else (N, M)
        self.N, self.M, self.Nd, self.Md = N, M, Nd, Md
        dev = device()
        z = lambda r, c: torch.zeros((r, c), dtype=DTYPE, device=dev)  # noqa: E731
        a = {}
        # state (shared with the NavierStokes object's fields)
        # (bind=False: a private copy, e.g. a second working set of the same instance)
        for key, fld in (("UG", ns.U), ("VG", ns.V), ("TG", ns.T), ("PG", ns.P), ("PRES", ns.pres)):
            if views is not None:
                views[key].copy_(fld.vhat)
                a[key] = views[key]
            else:
                a[key] = fld.vhat.contiguous() if bind else fld.vhat.clone()
            if bind:
                fld.vhat = a[key]
        a["TBCC"] = ns.Tbc_cheby.contiguous()
        a["DTB1"] = ns.dTbcdz1.contiguous()
        a["DTB2"] = ns.dTbcdz2.contiguous()
        for k, shp in scratch_shapes(N, M, Nd, Md, beta).items():
            a[k] = views[k] if (views is not None and k in views) else z(*shp)
        self.arrays = a
        bt = float(ns.beta)
        self.lens, self.par = instance_params(N, M, ns.dealias, ns.dt, ns.nu, ns.kappa, ns.scale, beta=bt)
        # operator tables
        g = _global_tables()
        t = {"sten_CD": g["sten_CD"], "sten_CN": g["sten_CN"], "tdma_CD": g["tdma_CD"]}
        host = host_tables(N, M, ns.T.xs[0].id, ns.dt * bt, ns.nu, ns.kappa, ns.scale, ns.solver_P._fd)
        t.update({k: to_dev(v) for k, v in host.items()})
        self.tables = t
        # per stage: parameters, ADI tables (lambda = dt a nu or dt a kappa) and the velocity arrays
        # of the stage and of the previous one (RK3)
        self.nstage = ns.nstage
        self.stage_par, self.stage_tables, self.stage_arrays = [self.par], [{}], [{}]
        if self.nstage == 3:
            for k in ("UX_A", "UX_B", "UZ_A", "UZ_B"):
                a[k] = z(Nd, Md)
            self.stage_par, self.stage_tables, self.stage_arrays = [], [], []
            for st in range(3):
                ak, bk, ck = float(ns.a[st]), float(ns.b[st]), float(ns.c[st])
                self.stage_par.append(instance_params(N, M, ns.dealias, ns.dt, ns.nu, ns.kappa, ns.scale,
                                                      ak, bk, ck, bt)[1])
                hs = host_tables(N, M, ns.T.xs[0].id, ns.dt * ak * bt, ns.nu, ns.kappa, ns.scale,
                                 ns.solver_P._fd)
                self.stage_tables.append({k: to_dev(hs[k]) for k in ("Ax_U", "Ax_T", "Ay_U", "Ay_T")})
                cur, old = ("A", "A") if st == 0 else (("B", "A") if st == 1 else ("A", "B"))
                self.stage_arrays.append({"UXC": "UX_" + cur, "UZC": "UZ_" + cur, "UXO": "UX_" + old,
                                          "UZO": "UZ_" + old})
        self.dct_x = _dct_tables(Nd, fft)
        self.dct_y = _dct_tables(Md, fft)

    def sync_in(self):
        """Point the solver's fields back at the fused state tensors (copying any newer values)."""
        ns = self.ns
        for key, fld in (("UG", ns.U), ("VG", ns.V), ("TG", ns.T), ("PG", ns.P), ("PRES", ns.pres)):
            t = self.arrays[key]
            if fld.vhat is not t:
                t.copy_(fld.vhat)
                fld.vhat = t

    def lines(self, prog):
        return self.lens[prog.lines] if prog.lines else 0

    def fill(self, prog, inst, stage=0, variant=None):
        """Resolve ``prog``'s symbolic arrays / tables for this instance (time-step stage ``stage``,
        program variant ``variant``) into a PgxInstance."""
        variant = variant or {}
        vmap, vtab, vpar = variant.get("arrays", {}), variant.get("tables", {}), variant.get("par", {})
        amap, tmap = self.stage_arrays[stage], self.stage_tables[stage]
        for name, idx in prog.arrs.items():
            name = vmap.get(name, name)
            t = self.arrays[amap.get(name, name)]
            A = inst.arr[idx]
            A.ptr, A.s0, A.s1, A.n0, A.n1 = t.data_ptr(), t.stride(0), t.stride(1), t.shape[0], t.shape[1]
        dct = self.dct_x if prog.axis == 0 else self.dct_y
        for name, idx in prog.mats.items():
            base = name.split("#")[0]
            base = vtab.get(base, base)
            v = dct[base] if base.startswith("dct") else tmap.get(base, self.tables.get(base))
            inst.mat[idx] = v if isinstance(v, int) else v.data_ptr()
        for i, n in enumerate(self.lens):
            inst.len[i] = n
        inst.len[L_LINES] = self.lens[prog.lines]
        for i, v in enumerate(self.stage_par[stage]):
            inst.par[i] = vpar.get(i, v)


def program_maxlen(prog, lens):
    """Longest line a slot of ``prog`` holds for an instance with lengths ``lens``."""
    slen = [0] * 8
    m = 0
    for o in prog.ops:
        c = o.code
        if c in (_lib.OP["LOAD"], _lib.OP["SETLEN"], _lib.OP["BANDED"], _lib.OP["DENSE"]):
            slen[o.a] = lens[o.len]
        elif c == _lib.OP["STENCIL"]:
            slen[o.a] += 2
        elif c == _lib.OP["STENCIL_T"]:
            slen[o.a] -= 2
        elif c in (_lib.OP["AXPY"], _lib.OP["MUL"]):
            slen[o.a] = max(slen[o.a], slen[o.b])
        elif c == _lib.OP["COPY"]:
            slen[o.a] = slen[o.b]
        m = max(m, slen[o.a])
    return m


CHAIN_OPS = ("FDMA", "POISSON", "TDMA2", "FDMA_T", "POISSON_T")
_CHAIN_CODES = tuple(_lib.OP[k] for k in CHAIN_OPS)


def dct_in_slot_ok(fft_n):
    """Whether a DCT of length ``fft_n`` can run in its slot's own lines and the spare slot
    (PGX_DCT_SLOT): n - 1 even, with an FFT stage count that can be made odd (n - 1 = 2^p 3^b
    with p >= 2, or p = 1 and b even)."""
    N = fft_n - 1
    if N < 2 or N % 2:
        return False
    p = b = 0
    while N % 2 == 0:
        N //= 2
        p += 1
    while N % 3 == 0:
        N //= 3
        b += 1
    return N == 1 and (p >= 2 or b % 2 == 0)


def fft_bytes_per_line(fft_n, one_slot=False):
    """Shared memory of the DCT-I work buffers per line: two buffers of n-1 (folded algorithm,
    even n-1) or 2(n-1) (paired lines) complex values per pair of lines, plus one scalar.  With
    ``one_slot`` (every DCT op transforms one slot) and the folded algorithm the transforms run in
    the slots' own lines and the spare slot (lengths ``dct_in_slot_ok``) or the second buffer is
    the spare slot (for an even number of lines per tile)."""
    if fft_n <= 1:
        return 0
    even = (fft_n - 1) % 2 == 0
    if one_slot and dct_in_slot_ok(fft_n):
        return 8
    stride = fft_n - 1 if even else 2 * (fft_n - 1)
    return (8 if (one_slot and even) else 16) * stride + 8
SMEM_PER_SM = 227 * 1024


def _fft_slots(prog, sd=False):
    """Slots of the widest DCT op: the FFT buffers hold that many slots' lines (one with
    ``sd``, the DCT ops split into one op per slot)."""
    if sd:
        return 1
    return max([max(o.b, 1) for o in prog.ops if o.code == _lib.OP["DCT"]] or [1])


# A multi-slot DCT op saves barriers, but its FFT buffers take shared memory from the
# tile: past this transform length each slot's lines alone fill the CTA's threads.
JOINT_DCT_MAX_N = 257


def _pick(prog, lines_total, lcap, fft_n, max_lines):
    """Lines per CTA and threads for one pass over ``lines_total`` lines (all instances).

    FFT passes: at most ~113 KB of shared memory per CTA so two CTAs share an SM
    (one computes while the other waits at a barrier).  Passes dominated by
    sequential banded sweeps: many lines per CTA, because each (line, parity)
    chain is one thread and the FP64 pipe of every SM sub-partition needs a
    warp of chains.
    """
    nbuf = prog.nslots + 1
    sd = _fft_slots(prog) > 1 and fft_n > JOINT_DCT_MAX_N
    fs = _fft_slots(prog, sd)
    per_line = 8 * nbuf * lcap + fs * fft_bytes_per_line(fft_n, fs == 1)
    chains = any(o.code in [_lib.OP[k] for k in CHAIN_OPS] for o in prog.ops)
    if fft_n > 1:
        budget = SMEM_PER_SM // 2 - 2048
        cap = 16
    elif chains:
        budget = SMEM_PER_SM - 4096
        cap = 64
    else:
        budget = SMEM_PER_SM // 2 - 2048
        cap = 32
    tbmax = max(1, budget // per_line)
    want = max(1, -(-lines_total // (2 * 152)))  # at least two CTAs per SM when there is work
    tb = max(1, min(cap, tbmax, want, max(max_lines, 1)))
    if fft_n > 1:
        tb = min(max(tb, 2), max(2, tbmax - tbmax % 2))
        tb -= tb % 2
    # one thread per (slot, line, parity) chain of the widest chain op
    width = 1
    for o in prog.ops:
        if o.code in _CHAIN_CODES:
            width = max(width, 2 * max(o.b, 1))
        elif o.code in (_lib.OP["DIFF"], _lib.OP["DIFF_T"]):
            width = max(width, max(o.b, 1))
    nt = max(256, 32 * -(-width * tb // 32))
    # few chains in the whole launch: one warp per chain (scanned) instead of one thread
    wc = chains and width * lines_total < 152 * 64
    ntmax = _max_threads(prog, fft_n, False)
    if wc:
        nt = max(256, min(ntmax, 32 * width * tb))
    return tb, min(nt, ntmax), bool(wc), sd, False


def _max_threads(prog, fft_n, dm):
    """CTA size limit of a launch: programs that keep DCT ops run the FFT build of the kernel."""
    fft = fft_n > 1 and not dm and any(o.code == _lib.OP["DCT"] for o in prog.ops)
    return _lib.MAX_THREADS_FFT if fft else _lib.MAX_THREADS


def _candidates(prog, lines_total, lcap, fft_n, max_lines):
    """Tile shapes the autotuner tries for one pass: lines per CTA chosen so that 1, 2, 3
    or 4 CTAs fit an SM's shared memory, plus small tiles for short passes; programs with
    multi-slot DCT ops also with the DCTs one slot at a time (smaller FFT buffers)."""
    out = []
    for sd in ((False, True) if _fft_slots(prog) > 1 and fft_n > 1 else (False,)):
        out += _candidates_sd(prog, lines_total, lcap, fft_n, max_lines, sd, False)
    if _has_dense(prog, fft_n):  # transforms / dense operators as tensor-core contractions
        out += _candidates_sd(prog, lines_total, lcap, 0, max_lines, False, True)
    return out


def _has_dense(prog, fft_n):
    """Whether a launch of ``prog`` has contractions the tensor cores can run (DENSE ops, or
    DCT ops whose dense matrices the program carries)."""
    return any(o.code == _lib.OP["DENSE"] or (o.code == _lib.OP["DCT"] and fft_n > 1) for o in prog.ops)


def _candidates_sd(prog, lines_total, lcap, fft_n, max_lines, sd, dm):
    ntmax = _max_threads(prog, fft_n, dm)
    nbuf = prog.nslots + 1
    fs = _fft_slots(prog, sd)
    per_line = 8 * nbuf * lcap + fs * fft_bytes_per_line(fft_n, fs == 1)
    width = 1
    for o in prog.ops:
        if o.code in _CHAIN_CODES:
            width = max(width, 2 * max(o.b, 1))
        elif o.code in (_lib.OP["DIFF"], _lib.OP["DIFF_T"]):
            width = max(width, max(o.b, 1))
    tbs = set()
    for ctas in (1, 2, 3, 4):
        tb = (SMEM_PER_SM // ctas - 2048) // per_line
        tbs.add(int(tb) - int(tb) % 8 if dm and tb >= 8 else int(tb))
    tbs.update({8, 16, 32} if dm else {1, 2, 4, 8, 16})  # tensor-core tiles are 8 lines wide
    chains = any(o.code in _CHAIN_CODES for o in prog.ops)
    out = []
    for tb in sorted(tbs):
        tb = min(tb, 64, max(max_lines, 1))
        if fft_n > 1 and tb > 1:  # FFT lines go in pairs; a single line (paired with zeros) gives
            tb -= tb % 2          # twice the CTAs when an instance has few lines
        if tb < 1 or tb * per_line > SMEM_PER_SM - 2048:
            continue
        for nt in (64, 128, 256, 512):
            nt = max(nt, 32 * -(-width * tb // 32))
            if nt <= ntmax and (tb, nt, False, sd, dm) not in out:
                out.append((tb, nt, False, sd, dm))
        if chains:  # warp-per-chain variants: a warp for each of the CTA's chains, up to ntmax
            for nt in (256, min(ntmax, 32 * width * tb)):
                nt = max(nt, 256)
                if nt <= ntmax and (tb, nt, True, sd, dm) not in out:
                    out.append((tb, nt, True, sd, dm))
    return out


def launch_ops(prog, sd=False, dm=False):
    """The ops of one launch of ``prog``: with ``sd`` each multi-slot DCT op becomes one op per
    slot; with ``dm`` each DCT op becomes dense-matrix ops (the program carries the matrices)
    and every DENSE op runs on the FP64 tensor cores."""
    ops = []
    for o in prog.ops:
        if dm and o.code == _lib.OP["DCT"]:
            mat = prog.mats[Prog._DENSE_DCT[o.k]]
            ops += [_lib.op("DENSE", a=o.a + i, mat=mat, len=L_ND + prog.axis, k=_lib.DENSE_MMA)
                    for i in range(max(o.b, 1))]
        elif dm and o.code == _lib.OP["DENSE"]:
            ops.append(_lib.op("DENSE", a=o.a, b=o.b, arr=o.arr, mat=o.mat, len=o.len,
                               k=o.k | _lib.DENSE_MMA, alpha=o.alpha, par=o.par))
        elif sd and o.code == _lib.OP["DCT"] and o.b > 1:
            ops += [_lib.op("DCT", a=o.a + i, b=1, mat=o.mat, k=o.k) for i in range(o.b)]
        else:
            ops.append(o)
    return ops


def launch_program(prog, key, tb, nt, wc=False, sd=False, dm=False):
    """The PgxProgram of one launch of ``prog`` for the size class ``key`` = (lcap, fft_n) with
    ``tb`` lines and ``nt`` threads a CTA (``wc``, ``sd``, ``dm`` as in ``FusedBatch._group_launch``).
    One-slot transforms of the pass's (dealiased) length on even tiles run in the slots' own lines
    (PGX_DCT_SLOT): no FFT buffers of shared memory."""
    lcap, fft_n = key
    ops = launch_ops(prog, sd, dm)
    if dm:
        fft_n = 0
    P = _lib.PgxProgram()
    P.axis, P.lines_len, P.tb, P.lcap = prog.axis, L_LINES, tb, lcap
    P.nslots, P.nops, P.fft_n, P.nthreads = prog.nslots, len(ops), fft_n, nt
    assert len(ops) <= _lib.MAX_OPS, (prog.name, len(ops))
    dct = [o for o in ops if o.code == _lib.OP["DCT"]]
    in_slot = bool(dct) and tb % 2 == 0 and all(o.b <= 1 for o in dct) and dct_in_slot_ok(fft_n)
    for i, o in enumerate(ops):
        P.ops[i] = o
        if wc and o.code in _CHAIN_CODES:
            P.ops[i].k = o.k | _lib.CHAIN_WARP
        if in_slot and o.code == _lib.OP["DCT"]:
            P.ops[i].k = o.k | _lib.DCT_SLOT
    return P


class FusedBatch:
    """Fused Euler step for a batch of NavierStokes instances (any sizes / Ra)."""

    SPLIT_MAX = 4

    def __init__(self, solvers, bind=True, split=None):
        """``bind``: the solvers' fields become views of this batch's state arena (the default);
        with bind=False the batch works on its own copy of the states.  ``split``: per-field
        convection passes (more CTAs per instance; default for batches of up to SPLIT_MAX
        instances)."""
        self.solvers = list(solvers)
        tkinds = {ns.T.xs[0].id for ns in self.solvers}
        if len(tkinds) != 1:
            raise ValueError("all instances of a batch need the same temperature basis")
        sizes = [(int(1.5 * ns.shape[0]), int(1.5 * ns.shape[1])) if ns.dealias else ns.shape for ns in self.solvers]
        self.fft = all(fft_ok(n) for s in sizes for n in s)
        # all instance states live in one arena: one H2D / D2H copy moves the whole batch
        shapes = [_Instance.state_shapes(ns) for ns in self.solvers]
        total = sum(r * c for sh in shapes for (r, c) in sh.values())
        self.state_arena = torch.zeros(total, dtype=DTYPE, device=device())
        # the physical-space operands of the convection terms (pass P1's outputs) of all instances
        # share a second arena: the reverse sweep keeps them per step with one copy per batch
        ashapes = [{k: v for k, v in scratch_shapes(*ns.shape, *nd).items() if k in A_KEYS}
                   for ns, nd in zip(self.solvers, sizes)]
        self.a_arena = torch.zeros(sum(r * c for sh in ashapes for (r, c) in sh.values()), dtype=DTYPE,
                                   device=device())
        # explicit diffusion (beta != 1) in any instance: the batch runs the passes that carry it
        # (instances with beta = 1 add zero)
        self.beta = any(float(ns.beta) != 1.0 for ns in self.solvers)
        # the states lie in the arena grouped by instance shape (the instances keep the caller's order):
        # a host-memory pipeline group of one shape is one contiguous copy each way and launches one
        # size class per pass
        order = sorted(range(len(self.solvers)), key=lambda k: tuple(self.solvers[k].shape))
        soff, off = [0] * len(self.solvers), 0
        for k in order:
            soff[k] = off
            off += sum(r * c for (r, c) in shapes[k].values())
        self.insts, aoff = [], 0
        for ns, sh, ash, off in zip(self.solvers, shapes, ashapes, soff):
            views = {}
            for key in _Instance.STATE:
                r, c = sh[key]
                views[key] = self.state_arena[off:off + r * c].view(r, c)
                off += r * c
            for key, (r, c) in ash.items():
                views[key] = self.a_arena[aoff:aoff + r * c].view(r, c)
                aoff += r * c
            self.insts.append(_Instance(ns, self.fft, views, bind, self.beta))
        nst = {ns.nstage for ns in self.solvers}
        if len(nst) != 1:
            raise ValueError("all instances of a batch need the same integrator")
        self.nstage = nst.pop()
        self.tkind = tkinds.pop()
        self.split = len(self.solvers) <= self.SPLIT_MAX if split is None else bool(split)
        self.progs = build_programs(self.tkind, self.fft, rk3=self.nstage == 3, split=self.split, beta=self.beta)
        self._build_launches()
        self.graph = None

    # ------------------------------------------------------------- launches
    # A pass over a heterogeneous batch is split into one launch per class of
    # instances with the same slot capacity (longest line) and FFT length: the
    # shared-memory tile of a launch is sized for its own class, so a launch of
    # small instances holds proportionally more lines per CTA instead of
    # padding every line to the largest instance's length.
    def _groups(self, prog):
        """[((lcap, fft_n), [instance indices])] for one pass, largest class first."""
        g = {}
        for k, I in enumerate(self.insts):
            lcap = (program_maxlen(prog, I.lens) + 1) | 1
            fft_n = I.lens[L_ND + prog.axis] if (prog.has_dct and self.fft) else 0
            g.setdefault((lcap, fft_n), []).append(k)
        return sorted(g.items(), reverse=True)

    def _d_insts(self, prog, stage=0):
        """Descriptors of every instance (x every program variant: instance k, variant v at
        k * len(variants) + v)."""
        nv = len(prog.variants)
        insts = (_lib.PgxInstance * (len(self.insts) * nv))()
        for k, I in enumerate(self.insts):
            for v, var in enumerate(prog.variants):
                I.fill(prog, insts[k * nv + v], stage, var)
        d = torch.frombuffer(bytearray(bytes(insts)), dtype=torch.uint8).to(device())
        # the host copy travels with the device descriptors: _group_launch checks every
        # launch against it (the batched kernel reads its descriptors on the device only)
        d.pgx_host = insts
        return d

    def _group_launch(self, prog, d_insts, key, members, tb, nt, wc=False, name=None, sd=False, dm=False):
        """One launch of ``prog`` over ``members``; ``wc``: chain ops in warp-per-chain mode;
        ``sd``: multi-slot DCT ops as one op per slot; ``dm``: DCT ops as dense matrices and every
        DENSE op on the FP64 tensor cores (no FFT buffers)."""
        P = launch_program(prog, key, tb, nt, wc, sd, dm)
        nv = len(prog.variants)
        # the batched launch cannot read its descriptors on the host: check every member's host copy
        host = getattr(d_insts, "pgx_host", None)
        if host is None:
            raise RuntimeError("%s: launch descriptors without their host copy (not made by _d_insts)"
                               % (name or prog.name))
        check = _lib.lib().pgx_check_instance
        for k in members:
            for v in range(nv):
                _lib.check(check(ctypes.byref(P), ctypes.byref(host[k * nv + v])),
                           "%s: instance %d, variant %d" % (name or prog.name, k, v))
        work = [(k * nv + v, t) for k in members for v in range(nv)
                for t in range(-(-self.insts[k].lines(prog) // tb))]
        d_work = torch.as_tensor(np.asarray(work, dtype=np.int32).ravel(), device=device())
        return {"name": name or prog.name, "P": P, "d_insts": d_insts, "d_work": d_work, "nwork": len(work),
                "key": key, "members": members, "prog": prog, "wc": bool(wc), "sd": bool(sd), "dm": bool(dm)}

    def _pass_launches(self, prog, tiles=None, stage=0, key_tiles=None):
        d_insts = self._d_insts(prog, stage)
        name = prog.name if stage == 0 else "%s@%d" % (prog.name, stage)
        out = []
        for gi, (key, members) in enumerate(self._groups(prog)):
            lines = [self.insts[k].lines(prog) for k in members]
            tag = "%s#%d" % (name, gi)
            if key_tiles and (name, key) in key_tiles:
                tb, nt, wc, sd, dm = key_tiles[(name, key)]
            elif tiles and tag in tiles:
                tb, nt, wc, sd, dm = (tuple(tiles[tag][:5]) + (False,) * 3)[:5]
            else:
                tb, nt, wc, sd, dm = _pick(prog, sum(lines) * len(prog.variants), key[0], key[1], max(lines))
            out.append(self._group_launch(prog, d_insts, key, members, tb, nt, bool(wc), name, bool(sd), bool(dm)))
        return out

    def _build_launches(self, tiles=None):
        """Launch descriptors of the forward passes; ``tiles`` = {"pass#group": (lines per CTA,
        threads)} overrides the default choice (e.g. another batch's autotuned tiles)."""
        self.launches = [self._pass_launches(p, tiles, st) for st in range(self.nstage) for p in self.progs]
        # a graph recorded before reads the old launches' descriptors and work lists: drop it with them
        self.graph, self.graph_branches = None, []
        self.launch_generation = getattr(self, "launch_generation", 0) + 1

    @staticmethod
    def _tiles_of(launch_sets):
        return {"%s#%d" % (L["name"], gi): (L["P"].tb, L["P"].nthreads, L["wc"], L["sd"], L["dm"])
                for group in launch_sets for gi, L in enumerate(group)}

    def tiles(self):
        """{"pass#group": (lines per CTA, threads)} of the current forward launches."""
        return self._tiles_of(self.launches)

    def _run_launch(self, L):
        _lib.check(_lib.lib().pgx_run_batched(ctypes.byref(L["P"]), L["d_insts"].data_ptr(), L["d_work"].data_ptr(),
                                              L["nwork"], stream()), L["name"])

    def run_pass(self, i):
        for L in self.launches[i]:
            self._run_launch(L)

    def _tune(self, launch_sets, reps, verbose):
        """Time every candidate tile of every launch (each alone) and keep the fastest.
        The caller saves and restores whatever state the launches modify.  Graphs recorded over
        the old launches (here or by a HorizonGradient) see the new ``launch_generation``."""
        self.launch_generation = getattr(self, "launch_generation", 0) + 1
        if not hasattr(self, "tune_log"):
            self.tune_log = {}
        stream = torch.cuda.current_stream()
        chosen = {}
        for group in launch_sets:
            for gi, L0 in enumerate(group):
                prog, key, members = L0["prog"], L0["key"], L0["members"]
                lines = [self.insts[k].lines(prog) for k in members]
                best, tried = None, []
                for tb, nt, wc, sd, dm in _candidates(prog, sum(lines) * len(prog.variants), key[0], key[1],
                                                      max(lines)):
                    L = self._group_launch(prog, L0["d_insts"], key, members, tb, nt, wc, L0["name"], sd, dm)
                    self._run_launch(L)
                    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    for _ in range(reps):
                        self._run_launch(L)
                    b.record(stream)
                    torch.cuda.synchronize()
                    ms = a.elapsed_time(b) / reps
                    if verbose:
                        print(prog.name, gi, tb, nt, wc, sd, dm, round(ms, 4))
                    tried.append((ms, (tb, nt, wc, sd, dm)))
                    if best is None or ms < best[0]:
                        best = (ms, L, tb, nt, wc, sd, dm)
                group[gi] = best[1]
                chosen["%s#%d" % (L0["name"], gi)] = best[2:] + (round(best[0], 4),)
                self.tune_log["%s#%d" % (L0["name"], gi)] = sorted(tried)
        return chosen

    def tune_in_graph(self, names=("P2",), within=0.15, reps=20, most=6):
        """Second look at the tiles of the passes ``names`` inside the step's graph: the candidates
        within ``within`` of a launch's best time alone are timed as part of the whole step (with
        its parallel branches, as captured last), where other branches share the SMs; the fastest
        step keeps its tile.  The state is restored after every trial.  Returns {tag: (tile, ms)}."""
        groups = getattr(self, "graph_groups_arg", 1)
        saved = self.state_arena.clone()

        def step_ms():
            self.capture(1, groups=groups)
            for _ in range(3):
                self.step()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
            for a, b in ev:
                a.record()
                self.step()
                b.record()
            torch.cuda.synchronize()
            self.state_arena.copy_(saved)
            return sum(a.elapsed_time(b) for a, b in ev) / reps

        base = step_ms()
        out = {}
        for group in self.launches:
            for gi, L0 in enumerate(group):
                if L0["name"] not in names:
                    continue
                tag = "%s#%d" % (L0["name"], gi)
                log = getattr(self, "tune_log", {}).get(tag, [])
                cur = (L0["P"].tb, L0["P"].nthreads, L0["wc"], L0["sd"], L0["dm"])
                cands = [t for ms, t in log if log and ms <= log[0][0] * (1.0 + within) and t != cur][:most]
                best, best_ms = L0, base
                for tb, nt, wc, sd, dm in cands:
                    group[gi] = self._group_launch(L0["prog"], L0["d_insts"], L0["key"], L0["members"], tb, nt,
                                                   wc, L0["name"], sd, dm)
                    ms = step_ms()
                    if ms < best_ms:
                        best, best_ms = group[gi], ms
                group[gi] = best
                base = best_ms
                out[tag] = ((best["P"].tb, best["P"].nthreads, best["wc"], best["sd"], best["dm"]), round(best_ms, 4))
        self.launch_generation = getattr(self, "launch_generation", 0) + 1
        self.capture(1, groups=groups)
        torch.cuda.synchronize()
        return out

    def autotune(self, reps=3, verbose=False):
        """Time every candidate tile shape of every launch of every pass on this batch and keep
        the fastest.  The passes update the state in place, so the state is saved before and
        restored after tuning.  Returns {"pass#group": (lines per CTA, threads, ms)}."""
        saved = [{k: I.arrays[k].clone() for k in _Instance.STATE} for I in self.insts]
        chosen = self._tune(self.launches, reps, verbose)
        for I, s in zip(self.insts, saved):
            for k, v in s.items():
                I.arrays[k].copy_(v)
        torch.cuda.synchronize()
        self.graph = None
        self.tuned = chosen
        return chosen

    def step_eager(self):
        for i in range(len(self.launches)):
            self.run_pass(i)

    def capture(self, nsteps=1, groups=1):
        """Record ``nsteps`` fused steps in a CUDA graph; ``step()`` then replays it.  ``groups`` > 1:
        the instances in that many groups (``_split_groups``), each group's launches a parallel
        branch of the graph, so one group's next pass starts while another's drains."""
        # the passes update the state in place: keep a copy, warm up once outside the
        # capture (kernel attributes, lazy tables), restore, then record
        saved = [{k: I.arrays[k].clone() for k in ("UG", "VG", "TG", "PG", "PRES")} for I in self.insts]
        self.step_eager()
        torch.cuda.synchronize()
        for I, s in zip(self.insts, saved):
            for k, v in s.items():
                I.arrays[k].copy_(v)
        branches = []
        if isinstance(groups, str) and groups.startswith("shape"):
            # one branch per instance shape (every launch of a branch is one size class); "shapeK":
            # each shape's instances in K branches
            per = int(groups[5:] or 1)
            shapes = {}
            for k, I in enumerate(self.insts):
                shapes.setdefault((I.N, I.M), []).append(k)
            parts = [idx[j::per] for idx in shapes.values() for j in range(per) if idx[j::per]]
            branches = [(self._subset(idx), torch.cuda.Stream()) for idx in parts]
        elif groups > 1:
            if self.state_arena is None:   # a launch subset: groups of about equal instance counts
                parts = [p for p in np.array_split(np.arange(len(self.insts)), groups) if len(p)]
            else:
                parts = [idx for idx, _, _ in self._split_groups(groups)]
            branches = [(self._subset(list(idx)), torch.cuda.Stream()) for idx in parts]
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            cur = torch.cuda.current_stream()
            for _ in range(nsteps):
                if len(branches) > 1:
                    for sub, st in branches:
                        st.wait_stream(cur)
                        with torch.cuda.stream(st):
                            sub.step_eager()
                    for _, st in branches:
                        cur.wait_stream(st)
                else:
                    self.step_eager()
        torch.cuda.synchronize()
        for I, s in zip(self.insts, saved):
            for k, v in s.items():
                I.arrays[k].copy_(v)
        self.graph, self.graph_steps, self.graph_groups_arg = g, nsteps, groups
        # the graph reads the branches' instance descriptors and work lists: they live as long as it
        self.graph_branches = branches
        self.graph_groups = max(1, len(branches))
        self.graph_launches = sum(sub.launches_per_step for sub, _ in branches) if len(branches) > 1 \
            else self.launches_per_step

    def capture_best(self, tries=4, reps=10):
        """Record the step's graph ``tries`` times (same launches and branches as the last ``capture``)
        and keep the recording whose replays run fastest: replays of graphs with several parallel
        branches differ by a few percent from one recording to the next.  The state is restored
        after every trial.  Returns the ms per step of every recording."""
        groups = getattr(self, "graph_groups_arg", 1)
        saved = self.state_arena.clone()
        best, times = None, []
        for _ in range(tries):
            self.capture(1, groups=groups)
            for _ in range(3):
                self.step()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
            for a, b in ev:
                a.record()
                self.step()
                b.record()
            torch.cuda.synchronize()
            times.append(sum(a.elapsed_time(b) for a, b in ev) / reps)
            self.state_arena.copy_(saved)
            if best is None or times[-1] < best[0]:
                best = (times[-1], self.graph, self.graph_branches, self.graph_groups, self.graph_launches)
        _, self.graph, self.graph_branches, self.graph_groups, self.graph_launches = best
        self.graph_steps = 1
        torch.cuda.synchronize()
        return times

    def step(self):
        """One fused step (graph replay when captured with nsteps == 1)."""
        if self.graph is not None and self.graph_steps == 1:
            self.graph.replay()
        else:
            self.step_eager()

    @property
    def launches_per_step(self):
        return sum(len(g) for g in self.launches)

    # ------------------------------------------------- host-resident state
    def _subset(self, idx):
        """Launch set of the instances ``idx`` (same state, scratch and tables), each launch with
        the tile this batch uses for the same pass and size class."""
        key_tiles = {(L["name"], L["key"]): (L["P"].tb, L["P"].nthreads, L["wc"], L["sd"], L["dm"])
                     for group in self.launches for L in group}
        sub = FusedBatch.__new__(FusedBatch)
        sub.solvers, sub.insts = [self.solvers[i] for i in idx], [self.insts[i] for i in idx]
        sub.fft, sub.nstage, sub.tkind, sub.split, sub.beta = self.fft, self.nstage, self.tkind, self.split, self.beta
        sub.progs, sub.state_arena, sub.graph = self.progs, None, None
        sub.launches = [sub._pass_launches(p, None, st, key_tiles) for st in range(sub.nstage) for p in sub.progs]
        return sub

    def tune_groups(self, candidates=(1, 2, 4, 8, "shape"), reps=20):
        """Capture the step with each number of instance groups (parallel graph branches), time
        ``reps`` replays of each and keep the fastest ("shape": one branch per instance shape); the
        state is restored after every trial.  Returns {groups: ms per step}.  (Graphs of 16 or more
        branches ran slower, and from one capture to the next their time varied by 10 %.)"""
        saved = self.state_arena.clone()
        times = {}
        for G in candidates:
            if not isinstance(G, str) and G > len(self.insts):
                continue
            self.capture(1, groups=G)
            for _ in range(3):
                self.step()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
            for a, b in ev:   # an event pair around every replay, as a timed loop records them
                a.record()
                self.step()
                b.record()
            torch.cuda.synchronize()
            times[G] = sum(a.elapsed_time(b) for a, b in ev) / reps
            self.state_arena.copy_(saved)
        best = min(times, key=times.get)
        self.capture(1, groups=best)
        torch.cuda.synchronize()
        return times

    def _arena_order(self):
        """(instance indices in the order their states lie in ``state_arena``, their start offsets
        in that order followed by the arena's end)."""
        base = self.state_arena.data_ptr()
        starts = [(I.arrays["UG"].data_ptr() - base) // 8 for I in self.insts]
        order = sorted(range(len(self.insts)), key=lambda k: starts[k])
        return order, [starts[k] for k in order] + [self.state_arena.numel()]

    def _split_groups(self, groups):
        """[(instance indices, first, end offset in state_arena)]: up to ``groups`` groups of
        instances contiguous in the arena and of about equal state size; ``groups`` = "shape": one
        group per instance shape (contiguous: the arena is laid out by shape), "shapeK": K per shape."""
        order, starts = self._arena_order()
        if isinstance(groups, str) and groups.startswith("shape"):
            # runs of one shape ("shapeK": each run in K contiguous parts of about equal counts)
            per = int(groups[5:] or 1)
            runs = [0] + [j for j in range(1, len(order))
                          if (self.insts[order[j]].N, self.insts[order[j]].M)
                          != (self.insts[order[j - 1]].N, self.insts[order[j - 1]].M)] + [len(order)]
            cuts = sorted({a + (b - a) * q // per for a, b in zip(runs[:-1], runs[1:]) for q in range(per)} | {len(order)})
        else:
            cum = np.cumsum(np.diff(starts))
            cuts = [0] + [int(np.searchsorted(cum, cum[-1] * g / groups)) + 1 for g in range(1, groups)] + [len(cum)]
            cuts = sorted(set(min(max(c, 0), len(cum)) for c in cuts))
        return [(order[a:b], starts[a], starts[b]) for a, b in zip(cuts[:-1], cuts[1:]) if b > a]

    def host_pipeline(self, groups="shape", branches=1):
        """Prepare ``step_host``: the instances in ``groups`` groups contiguous in the state arena, of
        about equal state size (``groups`` = "shape": one group per instance shape), each with its
        own launch set, CUDA graph (``branches``: its graph branches, as in ``capture``) and
        stream."""
        self._pipe = []
        for idx, o0, o1 in self._split_groups(groups):
            sub = self._subset(idx)
            sub.capture(1, groups=branches)
            self._pipe.append((sub, o0, o1, torch.cuda.Stream()))
        self._pipe_fresh = True
        return len(self._pipe)

    def step_host(self, host, wait=False):
        """One step of every instance with the state in host memory: ``host`` (pinned, the layout of
        ``state_arena``) is copied in, stepped and copied back.  The instance groups of
        ``host_pipeline`` run on their own streams, so one group's copies overlap another's
        passes and the next step's upload of a group follows its own download; the current
        stream waits for all groups before the call returns (asynchronously).

        Between two calls the groups do not wait for the current stream, so that consecutive
        steps overlap.  Work enqueued on the current stream since the last call that reads or
        writes ``host`` or ``state_arena`` needs ``wait=True`` (the groups then start after it;
        the first call always does)."""
        if getattr(self, "_pipe", None) is None:
            self.host_pipeline()
        main = torch.cuda.current_stream()
        for sub, o0, o1, st in self._pipe:
            if self._pipe_fresh or wait:
                st.wait_stream(main)
            with torch.cuda.stream(st):
                self.state_arena[o0:o1].copy_(host[o0:o1], non_blocking=True)
                sub.step()
                host[o0:o1].copy_(self.state_arena[o0:o1], non_blocking=True)
        self._pipe_fresh = False
        for *_, st in self._pipe:
            main.wait_stream(st)

    # ------------------------------------------------- persistent launch
    def persistent(self, nsteps=1, threads=0, ctas=0, spin_seconds=1.0):
        """Prepare ``nsteps`` steps of every instance as ONE launch (``pgx_run_persistent``).

        The launches of the step become work items -- (program, descriptor, tile) of every pass,
        size class and instance, step after step, pass after pass -- that the CTAs of one resident
        grid take from a queue.  An item of pass p of instance k waits for instance k's pass p - 1
        (pass 0 of a step for the previous step's last pass), so every instance runs through its
        passes and steps at its own pace while others are still in earlier passes.  The programs
        keep this batch's tiles; every one runs with the launch's CTA size (``threads``: 0 = the
        largest of the programs').  ``ctas`` = 0: every CTA the device holds at once.  A wait that
        lasts longer than ``spin_seconds`` ends the launch with an error (``persistent_error``)."""
        lib = _lib.lib()
        progs, desc_host, desc_base, per_pass = [], [], [], []
        npass, ninst = len(self.launches), len(self.insts)
        need = np.zeros((ninst, npass), dtype=np.int64)
        ndesc = 0
        for p, group in enumerate(self.launches):
            host = getattr(group[0]["d_insts"], "pgx_host", None)
            if host is None:
                raise RuntimeError("%s: launch descriptors without their host copy" % group[0]["name"])
            desc_host.append(host)
            desc_base.append(ndesc)
            ndesc += len(host)
            its = []
            for L in group:
                if L["d_insts"] is not group[0]["d_insts"]:
                    raise RuntimeError("%s: the size classes of a pass must share its descriptors" % L["name"])
                nv = len(L["prog"].variants)
                for d, t in L["d_work"].cpu().numpy().reshape(-1, 2):
                    k = int(d) // nv
                    its.append((len(progs), desc_base[p] + int(d), int(t), k))
                    need[k, p] += 1
                progs.append(L["P"])
            per_pass.append(its)
        items = persistent_items(per_pass, need, nsteps)
        h_progs = (_lib.PgxProgram * len(progs))(*progs)
        descs = (_lib.PgxInstance * ndesc)()
        for host, base in zip(desc_host, desc_base):
            ctypes.memmove(ctypes.addressof(descs) + base * ctypes.sizeof(_lib.PgxInstance), ctypes.addressof(host),
                           ctypes.sizeof(host))
        dev = device()
        shape = (ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64())
        _lib.check(lib.pgx_persistent_shape(ctypes.byref(h_progs), len(progs), int(threads),
                                            *[ctypes.byref(x) for x in shape]), "persistent shape")
        self._persist = {
            "h_progs": h_progs, "nprogs": len(progs),
            "d_progs": torch.frombuffer(bytearray(bytes(h_progs)), dtype=torch.uint8).to(dev),
            "d_descs": torch.frombuffer(bytearray(bytes(descs)), dtype=torch.uint8).to(dev), "ndescs": ndesc,
            "d_items": torch.as_tensor(np.asarray(items, dtype=np.int32).reshape(-1), device=dev),
            "nitems": len(items), "ncounters": ninst * npass,
            "d_counters": torch.zeros(ninst * npass, dtype=torch.int32, device=dev),
            "d_state": torch.zeros(3, dtype=torch.int32, device=dev),
            "ctas": int(ctas), "threads": int(shape[0].value), "ctas_per_sm": int(shape[1].value),
            "smem": int(shape[2].value), "spin": int(spin_seconds * 2.1e9), "nsteps": nsteps,
            "launch_generation": getattr(self, "launch_generation", 0), "graph": None}
        return {k: self._persist[k] for k in ("nitems", "nprogs", "threads", "ctas_per_sm", "smem", "nsteps")}

    def persistent_tiles(self, threads, ctas_per_sm):
        """Re-pick every launch's tile for the persistent form: among the tiles the last ``autotune``
        timed (alone), the fastest that runs with ``threads`` threads and leaves room for
        ``ctas_per_sm`` CTAs of the persistent kernel on an SM (its descriptor and program head
        included).  Launches without such a tile keep theirs.  Returns {"pass#group": tile}."""
        lib = _lib.lib()
        log = getattr(self, "tune_log", {})
        cap = SMEM_PER_SM // ctas_per_sm - 1024 - PERSIST_HEAD
        tiles = {}
        for group in self.launches:
            for gi, L in enumerate(group):
                tag = "%s#%d" % (L["name"], gi)
                for ms, tile in log.get(tag, []):
                    if tile[1] != threads:
                        continue
                    P = self._group_launch(L["prog"], L["d_insts"], L["key"], L["members"], *tile[:3], L["name"],
                                           *tile[3:5])["P"]
                    if lib.pgx_program_smem(ctypes.byref(P)) <= cap:
                        tiles[tag] = tuple(tile)
                        break
                else:
                    tiles[tag] = (L["P"].tb, L["P"].nthreads, L["wc"], L["sd"], L["dm"])
        self._build_launches(tiles)
        return tiles

    def run_persistent(self):
        """Launch the persistent form prepared by ``persistent`` (``nsteps`` steps of every instance)."""
        q = getattr(self, "_persist", None)
        if q is None or q["launch_generation"] != getattr(self, "launch_generation", 0):
            raise RuntimeError("persistent(): not prepared for the current launches")
        _lib.check(_lib.lib().pgx_run_persistent(
            ctypes.byref(q["h_progs"]), q["d_progs"].data_ptr(), q["nprogs"], q["d_descs"].data_ptr(), q["ndescs"],
            q["d_items"].data_ptr(), q["nitems"], q["d_counters"].data_ptr(), q["ncounters"], q["d_state"].data_ptr(),
            q["ctas"], q["threads"], q["spin"], stream()), "persistent step")

    def capture_persistent(self):
        """Record ``run_persistent`` (its counter resets and the one kernel) in a CUDA graph;
        ``step_persistent`` replays it."""
        q = self._persist
        self.run_persistent()   # first launch outside the capture (kernel attributes)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run_persistent()
        torch.cuda.synchronize()
        q["graph"] = g

    def step_persistent(self):
        """``nsteps`` steps of every instance in one launch (graph replay once captured)."""
        q = self._persist
        if q["graph"] is not None:
            q["graph"].replay()
        else:
            self.run_persistent()

    def persistent_error(self):
        """(error, item) of the last persistent launch: error 0 = every item ran (synchronises)."""
        err, where = ctypes.c_int32(), ctypes.c_int32()
        _lib.check(_lib.lib().pgx_persist_error(self._persist["d_state"].data_ptr(), ctypes.byref(err),
                                                ctypes.byref(where), stream()), "persistent error")
        return err.value, where.value

    def single(self, i):
        """Launch set of instance ``i`` alone (same tables and state): the one-by-one form."""
        one = FusedBatch.__new__(FusedBatch)
        one.solvers, one.insts, one.fft = [self.solvers[i]], [self.insts[i]], self.fft
        one.nstage, one.tkind, one.split, one.beta = self.nstage, self.tkind, True, self.beta
        one.progs = build_programs(self.tkind, self.fft, rk3=self.nstage == 3, split=True, beta=self.beta)
        one.state_arena = None
        one._build_launches()
        one.graph = None
        return one

    def scratch_bytes(self):
        return sum(t.numel() * 8 for I in self.insts for k, t in I.arrays.items())

    def pass_work(self):
        """Algorithmic FP64 flops and HBM bytes per launch of every pass (all instances)."""
        out = []
        for prog in self.progs * self.nstage:
            fl = by = 0.0
            for I in self.insts:
                f, b = program_work(prog, I)
                fl += f * len(prog.variants)
                by += b * len(prog.variants)
            out.append((prog.name, fl, by))
        return out


def _log2(x):
    return float(np.log2(x))


def program_work(prog, I):
    """Algorithmic work of ``prog`` on instance ``I``: (flops, bytes).

    Counts per line of n elements: DCT-I 2.5 n log2(2(n-1)) (the FFT count) per slot;
    stencil / transpose 2 per output; derivative 2 per element and pass;
    offset-2 TDMA 5; four-diagonal sweep 7; Poisson sweep 9; banded 2 per
    diagonal and row; dense 2 per column and row; scale / mul 1, axpy /
    load-add 2.  Bytes: 8 per element loaded or stored.
    """
    lines = I.lens[prog.lines]
    slen = [0] * 8
    fl = by = 0.0
    for o in prog.ops:
        code = o.code
        if code == _lib.OP["LOAD"]:
            slen[o.a] = I.lens[o.len]
            by += 8.0 * I.lens[o.len] * lines
            if o.par >= 0 or o.alpha != 1.0:
                fl += slen[o.a] * lines
        elif code in (_lib.OP["LOAD_ADD"], _lib.OP["LOAD_MUL"]):
            by += 8.0 * slen[o.a] * lines
            fl += 2.0 * slen[o.a] * lines
        elif code in (_lib.OP["STORE"], _lib.OP["STORE_ADD"]):
            by += 8.0 * slen[o.a] * lines
        elif code == _lib.OP["SCALE"]:
            fl += slen[o.a] * lines
        elif code in (_lib.OP["AXPY"], _lib.OP["MUL"], _lib.OP["COPY"]):
            slen[o.a] = slen[o.b] if code == _lib.OP["COPY"] else max(slen[o.a], slen[o.b])
            fl += (2.0 if code == _lib.OP["AXPY"] else (1.0 if code == _lib.OP["MUL"] else 0.0)) * slen[o.a] * lines
        elif code == _lib.OP["SETLEN"]:
            slen[o.a] = I.lens[o.len]
        elif code == _lib.OP["STENCIL"]:
            slen[o.a] += 2
            fl += 2.0 * slen[o.a] * lines
        elif code == _lib.OP["STENCIL_T"]:
            slen[o.a] -= 2
            fl += 2.0 * slen[o.a] * lines
        elif code == _lib.OP["TDMA2"]:
            fl += 5.0 * sum(slen[o.a:o.a + max(o.b, 1)]) * lines
        elif code in (_lib.OP["DIFF"], _lib.OP["DIFF_T"]):
            fl += 2.0 * o.k * sum(slen[o.a:o.a + max(o.b, 1)]) * lines
        elif code == _lib.OP["DCT"]:   # every slot of a multi-slot op is one transform
            n = slen[o.a]
            fl += 2.5 * n * _log2(2 * (n - 1)) * lines * max(o.b, 1)
        elif code == _lib.OP["BANDED"]:
            slen[o.a] = I.lens[o.len]
            fl += 2.0 * o.k * slen[o.a] * lines
        elif code == _lib.OP["DENSE"]:
            cols = slen[o.a]
            slen[o.a] = I.lens[o.len]
            fl += 2.0 * cols * slen[o.a] * lines
        elif code in (_lib.OP["FDMA"], _lib.OP["FDMA_T"]):
            fl += 7.0 * sum(slen[o.a:o.a + max(o.b, 1)]) * lines
        elif code in (_lib.OP["POISSON"], _lib.OP["POISSON_T"]):
            fl += 9.0 * slen[o.a] * lines
    return fl, by


# bytes of a persistent CTA's shared memory before its slots: the descriptor and the program
PERSIST_HEAD = 16 * (-(-ctypes.sizeof(_lib.PgxInstance) // 16) + -(-ctypes.sizeof(_lib.PgxProgram) // 16))


def persistent_items(per_pass, need, nsteps):
    """Work items of ``nsteps`` steps for ``pgx_run_persistent``: (prog, desc, tile, wait, need, done).

    ``per_pass[p]`` lists the (prog, desc, tile, instance) items of pass p of one step and
    ``need[k, p]`` how many of them belong to instance k.  Counter k * npass + p counts the completed
    items of instance k's pass p over all steps of the launch.  The list runs step after step and
    pass after pass, so an item always comes after every item it waits for: pass p of step s waits
    for (s + 1) need[k, p - 1] completions of pass p - 1, pass 0 for s need[k, npass - 1] of the
    last pass."""
    npass = len(per_pass)
    items = []
    for st in range(nsteps):
        for p in range(npass):
            for prog, desc, tile, k in per_pass[p]:
                if p > 0:
                    wait, nd = k * npass + p - 1, (st + 1) * int(need[k, p - 1])
                elif st > 0:
                    wait, nd = k * npass + npass - 1, st * int(need[k, npass - 1])
                else:
                    wait, nd = -1, 0
                items.append((prog, desc, tile, wait, nd, k * npass + p))
    return items


class FusedStep(FusedBatch):
    """Fused step of a single NavierStokes instance."""

    def __init__(self, ns):
        FusedBatch.__init__(self, [ns])
