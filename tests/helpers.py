"""Shared builders: the same seeded problem as an oracle solver and as a libfdga solver."""
import numpy as np

from oracle import oracle as O

REF_NAMES = ["Fp_p", "Fp_x", "Ft_p", "Ft_x"]


def make_inputs(cfg):
    from fdgasolver.workloads import make_inputs as mi
    return mi(cfg)


def make_oracle(cfg, sym):
    Gb, G0, S0, rv = make_inputs(cfg)
    local = cfg["kind"] == "siam"
    s = O.OracleSolver(nG=cfg["nG"], nK1=cfg["nK1"], nK2=cfg["nK2"], nK3=cfg["nK3"], T=cfg["T"], U=cfg["U"],
                       L=1 if local else cfg["L"], local=local, mPi_factor=cfg["mPi_factor"], nR=rv.nR)
    s.set("Gbare", Gb)
    s.set("G0", G0)
    s.set("Sigma0", S0)
    for n, a in zip(REF_NAMES, rv.arrays):
        s.set(n, a)
    s.finalize()
    if sym:
        s.init_sym_grp()
    return s


def make_gpu(cfg, sym):
    from fdgasolver.workloads import make_solver
    return make_solver(cfg, sym)


def blocks(cfg):
    """(name, start, stop) of the flatten(S) blocks: γp(K1,K2,K3), γt, γa, Σ."""
    local = cfg["kind"] == "siam"
    Nq = 1 if local else cfg["L"] ** 2
    n1 = (2 * cfg["nK1"] - 1) * Nq
    n2 = (2 * cfg["nK2"][0] - 1) * 2 * cfg["nK2"][1] * Nq
    n3 = (2 * cfg["nK3"][0] - 1) * (2 * cfg["nK3"][1]) ** 2 * Nq
    out, o = [], 0
    for ch in "pta":
        for nm, n in (("K1", n1), ("K2", n2), ("K3", n3)):
            out.append((f"{ch}.{nm}", o, o + n))
            o += n
    nS = 2 * cfg["nG"] * Nq
    out.append(("Sigma", o, o + nS))
    return out


def blockwise_rel_err(cfg, a, b):
    """max over blocks of max|a-b| / max|b| (block max norm)."""
    worst = 0.0
    for name, s, e in blocks(cfg):
        ref = np.abs(b[s:e]).max()
        if ref == 0:
            err = np.abs(a[s:e]).max()
        else:
            err = np.abs(a[s:e] - b[s:e]).max() / ref
        worst = max(worst, err)
    return worst
