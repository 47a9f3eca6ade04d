"""The oracle calls the reference's native kernels as often, and on the same sizes, as pypde does.

``tests/golden/call_counts.json`` (made by ``tests/golden/make_call_counts.py`` from the
reference itself) lists, for one Rayleigh-Benard step of six configurations, every call of
the reference's native kernels -- scipy's DCT-I and the f2py modules differentiate_cheby,
tdma, twodma, fdma -- by family, transform length and number of lines.  The oracle's
counterparts are counted on the same step here and must match call for call.  The fused step's programs are held
to the same counts: the same transform lengths and never more line transforms.
"""
import collections
import json
import os

import numpy as np
import pytest

from oracle import linalg as ol
from oracle import rbc2d as orb
from oracle import spectral as osp

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "call_counts.json")
CASES = json.load(open(GOLDEN))


def _lines(shape, n):
    return int(np.prod(shape)) // n


@pytest.fixture
def counted(monkeypatch):
    counts = collections.Counter()

    def wrap(mod, name, shape_of):
        f0 = getattr(mod, name)

        def f(*a, **k):
            key = shape_of(*a, **k)
            if key is not None:
                counts[key] += 1
            return f0(*a, **k)
        monkeypatch.setattr(mod, name, f)

    def along(f, axis=0):
        s = np.shape(f)
        return s[axis], _lines(s, s[axis])

    wrap(osp, "dct1", lambda f, axis=0: ("dct",) + along(f, axis))
    wrap(osp, "cheb_diff1", lambda c, axis=0: ("diff",) + along(c, axis))
    wrap(ol, "tdma_offset", lambda a, b, c, d, k: ("tdma", len(b), _lines(np.shape(d), len(b))))
    wrap(ol, "twodma_solve", lambda d, u, x: ("twodma", len(d), _lines(np.shape(x), len(d))))
    # shared-coefficient solves only: the stacked per-eigenvalue solves belong to fdma_type2
    wrap(ol, "fdma_solve", lambda l, d, u1, u2, x: ("fdma", len(d), _lines(np.shape(x), len(d)))
         if np.ndim(d) == 1 else None)
    wrap(ol, "fdma_type2", lambda A, C, lam, x, singular=False: ("type2", np.shape(x)[0], np.shape(x)[1]))
    return counts


@pytest.mark.parametrize("tag", sorted(CASES))
def test_oracle_kernel_calls_match_reference(counted, tag):
    cfg = dict(CASES[tag])
    case, shape, calls = cfg.pop("case"), tuple(cfg.pop("shape")), cfg.pop("calls")
    ns = orb.NavierStokes(case=case, shape=shape, pr=1.0, beta=cfg.pop("beta", 1.0), aspect=cfg.pop("aspect", 1.0),
                          tsave=None, **cfg)
    orb.seeded_temperature(ns, 0, 1e-3)
    ns.update()
    counted.clear()
    ns.update()
    got = sorted([list(k) + [v] for k, v in counted.items()])
    assert got == calls


def _fused_dct_lines(tag):
    """{transform length: line transforms} of the fused step's programs for the configuration ``tag``."""
    from pypde_gb300 import _lib
    from pypde_gb300.navier.fused import build_programs, instance_params
    cfg = CASES[tag]
    N, M = cfg["shape"]
    lens, _ = instance_params(N, M, cfg.get("dealias", True), 0.01, 1e-3, 1e-3, (0.5, 0.5))
    rk3 = cfg.get("integrator") == "rk3"
    progs = build_programs("CN" if cfg["case"] == "rbc" else "CD", True, rk3=rk3, split=False,
                           beta=cfg.get("beta", 1.0) != 1.0)
    op = _lib.OP
    got = collections.Counter()
    for p in progs * (3 if rk3 else 1):
        slen = [0] * 8
        for o in p.ops:
            if o.code in (op["LOAD"], op["SETLEN"], op["BANDED"], op["DENSE"]):
                slen[o.a] = lens[o.len]
            elif o.code == op["COPY"]:
                slen[o.a] = slen[o.b]
            elif o.code in (op["AXPY"], op["MUL"]):
                slen[o.a] = max(slen[o.a], slen[o.b])
            elif o.code in (op["STENCIL"], op["STENCIL_T"]):
                slen[o.a] += 2 if o.code == op["STENCIL"] else -2
            elif o.code == op["DCT"]:
                got[slen[o.a]] += lens[p.lines] * max(o.b, 1) * len(p.variants)
    return got


@pytest.mark.parametrize("tag", sorted(CASES))
def test_fused_step_transforms_no_more_lines_than_the_reference(tag):
    """The fused step's DCT-I line transforms, by length, against the reference's (same lengths,
    never more lines: the fused passes skip the zero-padded lines of the 3/2 grid and RK3 reuses
    the previous stage's velocities)."""
    ref = collections.Counter()
    for fam, n, lines, k in CASES[tag]["calls"]:
        if fam == "dct":
            ref[n] += lines * k
    got = _fused_dct_lines(tag)
    assert set(got) == set(ref)
    for n in ref:
        assert 0.55 * ref[n] <= got[n] <= ref[n], (n, got[n], ref[n])
