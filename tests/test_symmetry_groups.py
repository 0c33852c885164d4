"""Host logic (no GPU): libfdga's init_sym_grp! class maps equal the oracle's restatement of
MatsubaraFunctions' SymmetryGroup (same classes, same representative, same Operation)."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O


def _cfg(local, nG, nK1, nK2, nK3, L, f):
    from fdgasolver import _lib
    c = _lib.fdga_config()
    c.nG, c.nK1 = nG, nK1
    c.nK2[0], c.nK2[1] = nK2
    c.nK3[0], c.nK3[1] = nK3
    c.L = c.LG = L
    c.mPi_factor = f
    c.local = int(local)
    c.T, c.U = 0.5, 1.0
    c.nR[0], c.nR[1] = 1, 1
    return c


def _ref_to_dev(kind, shape, L):
    """Permutation: reference column-major index -> libfdga device index."""
    if kind in ("Sigma", "K1"):
        n = int(np.prod(shape))
        return np.arange(n)
    idx = np.arange(int(np.prod(shape)))
    coords = np.unravel_index(idx, shape, order="F")  # (Ω, ν, [ν'], P)
    # device row-major over (P, Ω, ν, [ν'])
    order = (coords[-1],) + coords[:-1]
    dshape = (shape[-1],) + shape[:-1]
    return np.ravel_multi_index(order, dshape, order="C")


GROUPS = [("Sigma", 0), ("pp1", 1), ("pp2", 2), ("ph2", 3), ("pp3", 4), ("ph3", 5), ("ppL3", 6), ("phL3", 7)]


@pytest.mark.parametrize("local,L", [(True, 1), (False, 3), (False, 4)])
def test_group_maps_match_oracle(local, L):
    from fdgasolver import _lib
    lib = _lib.load()
    nG, nK1, nK2, nK3, f = 6, 6, (3, 3), (2, 3), 2
    cfg = _cfg(local, nG, nK1, nK2, nK3, L, f)
    orc = O.OracleSolver(nG=nG, nK1=nK1, nK2=nK2, nK3=nK3, T=0.5, U=1.0, L=L, local=local, mPi_factor=f)
    orc.finalize()
    orc.init_sym_grp()
    Nq = L * L
    shapes = {"Sigma": (2 * nG, Nq), "K1": (2 * nK1 - 1, Nq), "K2": (2 * nK2[0] - 1, 2 * nK2[1], Nq),
              "K3": (2 * nK3[0] - 1, 2 * nK3[1], 2 * nK3[1], Nq)}
    for name, which in GROUPS:
        kind = "Sigma" if name == "Sigma" else "K" + name[-1]
        shape = shapes[kind]
        n = int(np.prod(shape))
        m = np.zeros(n, dtype=np.uint32)
        ncl = ctypes.c_int()
        assert lib.fdga_group_map(ctypes.byref(cfg), which, m.ctypes.data, n, ctypes.byref(ncl)) == 0
        perm = _ref_to_dev(kind, shape, L)          # ref j -> dev
        inv = np.empty(n, dtype=np.int64)
        inv[perm] = np.arange(n)                    # dev -> ref
        rep_ref = inv[(m[perm] >> 2).astype(np.int64)]
        op = (m[perm] & 3).astype(np.int64)
        cs, mem, ops = orc.group(name)
        o_rep = np.empty(n, dtype=np.int64)
        o_op = np.empty(n, dtype=np.int64)
        for c in range(len(cs) - 1):
            members = mem[cs[c]:cs[c + 1]]
            o_rep[members] = members[0]
            o_op[members] = ops[cs[c]:cs[c + 1]]
        assert ncl.value == len(cs) - 1, name
        assert np.array_equal(rep_ref, o_rep), name
        assert np.array_equal(op, o_op), name
