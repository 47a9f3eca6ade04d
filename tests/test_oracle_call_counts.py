"""The oracle calls the reference's native kernels as often, and on the same sizes, as pypde does.

``tests/golden/call_counts.json`` (made by ``tests/golden/make_call_counts.py`` from the
reference itself) lists, for one Rayleigh-Benard step of six configurations, every call of
the reference's native kernels -- scipy's DCT-I and the f2py modules differentiate_cheby,
tdma, twodma, fdma -- by family, transform length and number of lines.  The oracle's
counterparts are counted on the same step here and must match call for call.
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
