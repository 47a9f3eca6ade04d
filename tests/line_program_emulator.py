"""NumPy emulator of the pgx line-program interpreter (test infrastructure).

Runs a ``pypde_gb300.navier.fused.Prog`` (symbolic arrays and tables) on host
arrays with the op semantics of the CUDA interpreter (pgx_kernels.cu):
slots with a logical length and a zero tail, LOAD / STORE that clip to the
array's extent and skip lines beyond it, chain sweeps with the device table
layouts.  DCT-type ops use dense matrices.  It checks the construction of the
programs (which arrays, which tables, which order) on the CPU; the kernels
themselves are checked on the GPU.
"""
import numpy as np

from pypde_gb300 import _lib
from pypde_gb300.navier.fused import dense_dct_host

OPN = {v: k for k, v in _lib.OP.items()}
DCT_NAME = {_lib.DCT_FWD: "dct_fwd", _lib.DCT_BWD: "dct_bwd", _lib.DCT_FWD_T: "dct_fwd_t",
            _lib.DCT_BWD_T: "dct_bwd_t"}


def cheb_diff_matrix(n):
    """Chebyshev-coefficient derivative (recurrence dc_{n-1} = 0, dc_{n-2} = 2(n-1) c_{n-1},
    dc_i = dc_{i+2} + 2(i+1) c_{i+1}, dc_0 halved) as an n x n matrix."""
    D = np.zeros((n, n))
    for j in range(n):
        c = np.zeros(n)
        c[j] = 1.0
        dc = np.zeros(n)
        if n >= 2:
            dc[n - 2] = 2.0 * (n - 1) * c[n - 1]
        for i in range(n - 3, -1, -1):
            dc[i] = dc[i + 2] + 2.0 * (i + 1) * c[i + 1]
        dc[0] *= 0.5
        D[:, j] = dc
    return D


def _fdma(x, tab, n, transpose):
    """Banded LU sweep with the device table [l | 1/d | u1/d | u2/d] (per parity chain)."""
    l, dinv, u1d, u2d = tab[:n], tab[n:2 * n], tab[2 * n:3 * n], tab[3 * n:4 * n]
    for p in (0, 1):
        idx = list(range(p, n, 2))
        if not transpose:
            for i in idx[1:]:
                x[i] -= l[i] * x[i - 2]
            x2 = x4 = 0.0
            for i in reversed(idx):
                v = x[i] * dinv[i] - u2d[i] * x4 - u1d[i] * x2
                x[i] = v
                x4, x2 = x2, v
        else:
            z2 = z4 = 0.0   # zeta = z / dinv
            for i in idx:
                v = x[i]
                if i >= 4:
                    v -= u2d[i - 4] * z4
                if i >= 2:
                    v -= u1d[i - 2] * z2
                x[i] = v * dinv[i]
                z4, z2 = z2, v
            xn = 0.0
            for i in reversed(idx):
                li = l[i + 2] if i + 2 < n else 0.0
                xn = x[i] - li * xn
                x[i] = xn


class Machine:
    """One instance: ``arrays`` (name -> 2-D float64 array, updated in place), ``tables``
    (name -> 1-D or 2-D host table in device layout), ``lens`` and ``par`` as on the device."""

    def __init__(self, arrays, tables, lens, par):
        self.arrays, self.tables, self.lens, self.par = arrays, tables, lens, par

    def run(self, prog):
        """Run every variant of ``prog`` (one descriptor per variant on the device)."""
        for var in prog.variants:
            self._run(prog, var)

    def _run(self, prog, var):
        vmap, vtab, vpar = var.get("arrays", {}), var.get("tables", {}), var.get("par", {})
        L = self.lens[prog.lines]
        lcap = 8 + max(self.lens) * 2
        arr_name = {i: vmap.get(k, k) for k, i in prog.arrs.items()}
        mat_name = {i: vtab.get(k.split("#")[0], k.split("#")[0]) for k, i in prog.mats.items()}
        par = list(self.par)
        for i, v in vpar.items():
            par[i] = v
        axis = prog.axis
        nd = self.lens[5 + axis]
        dense = dense_dct_host(nd)
        slot = np.zeros((prog.nslots + 1, L, lcap))
        slen = [0] * (prog.nslots + 1)

        def alpha(o):
            return o.alpha * (par[o.par] if o.par >= 0 else 1.0)

        def view(name):
            A = self.arrays[name]
            return A if axis == 0 else A.T     # (elements, lines)

        for o in prog.ops:
            op = OPN[o.code]
            a = o.a
            if op in ("LOAD", "LOAD_ADD", "LOAD_MUL"):
                V = view(arr_name[o.arr])
                n = self.lens[o.len] if op == "LOAD" else slen[a]
                vals = np.zeros((L, n))
                ne, nl = min(n, V.shape[0]), min(L, V.shape[1])
                vals[:nl, :ne] = V[:ne, :nl].T
                vals *= alpha(o)
                if op == "LOAD":
                    slot[a] = 0.0
                    slot[a, :, :n] = vals
                    slen[a] = n
                elif op == "LOAD_ADD":
                    slot[a, :, :n] += vals
                else:
                    slot[a, :, :n] *= vals
            elif op in ("STORE", "STORE_ADD"):
                V = view(arr_name[o.arr])
                ne, nl = V.shape[0], min(L, V.shape[1])
                vals = alpha(o) * slot[a, :nl, :ne].T
                if op == "STORE":
                    V[:ne, :nl] = vals
                else:
                    V[:ne, :nl] += vals
            elif op == "SCALE":
                slot[a, :, :slen[a]] *= alpha(o)
            elif op in ("AXPY", "MUL", "COPY"):
                b = o.b
                n = slen[b] if op == "COPY" else max(slen[a], slen[b])
                if op == "AXPY":
                    slot[a, :, :n] += alpha(o) * slot[b, :, :n]
                elif op == "MUL":
                    slot[a, :, :n] *= alpha(o) * slot[b, :, :n]
                else:
                    slot[a] = 0.0
                    slot[a, :, :n] = alpha(o) * slot[b, :, :n]
                slen[a] = n
            elif op == "SETLEN":
                n = self.lens[o.len]
                if n < slen[a]:
                    slot[a, :, n:] = 0.0
                slen[a] = n
            elif op in ("STENCIL", "STENCIL_T"):
                sub = self.tables[mat_name[o.mat]]
                x = slot[a].copy()
                slot[a] = 0.0
                if op == "STENCIL":
                    M = slen[a]
                    slot[a, :, :M] = x[:, :M]
                    slot[a, :, 2:M + 2] += sub[:M] * x[:, :M]
                    slen[a] = M + 2
                else:
                    M = slen[a] - 2
                    slot[a, :, :M] = x[:, :M] + sub[:M] * x[:, 2:M + 2]
                    slen[a] = M
            elif op == "TDMA2":
                sub = self.tables["sten_" + mat_name[o.mat].split("_")[1]]
                for s in range(max(o.b, 1)):
                    n = slen[a + s]
                    K = np.diag(1.0 + sub[:n] ** 2) + np.diag(sub[:n - 2], 2) + np.diag(sub[:n - 2], -2)
                    slot[a + s, :, :n] = np.linalg.solve(K, slot[a + s, :, :n].T).T
            elif op in ("DIFF", "DIFF_T"):
                for s in range(max(o.b, 1)):
                    n = slen[a + s]
                    D = cheb_diff_matrix(n)
                    if op == "DIFF_T":
                        D = D.T
                    for _ in range(o.k):
                        slot[a + s, :, :n] = slot[a + s, :, :n] @ D.T
            elif op == "DCT":
                n = slen[a]
                C = dense_dct_host(n)[DCT_NAME[o.k]]
                for s in range(max(o.b, 1)):    # one length for all slots of the op
                    assert slen[a + s] == n, (prog.name, a + s, slen[a + s], n)
                    slot[a + s, :, :n] = slot[a + s, :, :n] @ C.T
            elif op == "DENSE":
                name = mat_name[o.mat]
                A = dense[name] if name.startswith("dct") else self.tables[name]
                rows, cols = self.lens[o.len], slen[a]
                A = np.asarray(A).reshape(rows, cols)
                y = slot[a, :, :cols] @ A.T
                slot[a] = 0.0
                slot[a, :, :rows] = y
                slen[a] = rows
            elif op == "BANDED":
                tab = self.tables[mat_name[o.mat]]
                rows, cols, off0 = self.lens[o.len], slen[a], o.b
                tab = tab.reshape(o.k, rows)
                x = slot[a].copy()
                slot[a] = 0.0
                for r in range(rows):
                    for d in range(o.k):
                        c = r + off0 + 2 * d
                        if 0 <= c < cols:
                            slot[a, :, r] += tab[d, r] * x[:, c]
                slen[a] = rows
            elif op in ("FDMA", "FDMA_T"):
                for s in range(max(o.b, 1)):
                    tab = self.tables[mat_name[o.mat + s]]
                    n = slen[a + s]
                    for t in range(L):
                        _fdma(slot[a + s, t], tab, n, op == "FDMA_T")
            elif op in ("POISSON", "POISSON_T"):
                tab = self.tables[mat_name[o.mat]]
                n = slen[a]
                for t in range(L):
                    _fdma(slot[a, t], tab[t * 4 * n:(t + 1) * 4 * n], n, op == "POISSON_T")
            elif op == "ZERO00":
                slot[a, 0, 0] = 0.0
            else:
                raise NotImplementedError(op)
