"""Susceptibilities χ_m, χ_d, χ_s of a converged state (K1_r = -U² χ_r; the reference's TRIQS
import src/utility/load_triqs.jl:67-75,106-114 and spin algebra src/types.jl:34-66).

The device χ (fdga_susceptibility) is compared with the same definition applied to the oracle's
K1 arrays after both solvers ran the same number of Anderson iterations, to 1e-10 relative, for
the momentum-resolved χ(Ω, q) and the momentum average χ_loc(Ω).
"""
import numpy as np
import pytest

from helpers import make_gpu, make_oracle

TOL = 1e-10

SMALL_NL = dict(kind="hubbard", T=0.5, U=2.0, mu=0.3, t1=1.0, t2=-0.2, L=4, nG=8, nK1=8, nK2=(3, 3), nK3=(2, 3),
                mPi_factor=4, refvertex_noise=0.05, seed=7)
SMALL_LOCAL = dict(kind="siam", T=0.1, U=1.0, e=0.2, Delta=0.5, D=10.0, nG=16, nK1=16, nK2=(5, 4), nK3=(4, 4),
                   mPi_factor=6)


def chi_from_k1(K1p, K1t, K1a, U, channel):
    """The definition restated on host arrays (test-side check)."""
    if channel == "m":
        return K1a / U ** 2
    if channel == "d":
        return (K1a - 2 * K1t) / U ** 2
    return -2 * K1p / U ** 2


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [SMALL_NL, SMALL_LOCAL], ids=["nl4", "local"])
def test_susceptibility_matches_oracle(cfg):
    orc = make_oracle(cfg, True)
    gpu = make_gpu(cfg, True)
    r_o = orc.solve("fdPA", maxiter=12, tol=1e-14, beta=0.5, mem=8)
    r_g = gpu.solve("fdPA", maxiter=12, tol=1e-14, delta=0.5, mem=8)
    assert r_o["iterations"] == r_g["iterations"] == 12
    NO = 2 * cfg["nK1"] - 1
    Nq = 1 if cfg["kind"] == "siam" else cfg["L"] ** 2
    K1 = {c: orc.get(f"F.{c}.K1") for c in "pta"}
    for ch in "mds":
        ref = chi_from_k1(K1["p"], K1["t"], K1["a"], cfg["U"], ch)
        got = gpu.susceptibility(ch)
        assert got.shape == (NO * Nq,)
        assert np.abs(got - ref).max() <= TOL * np.abs(ref).max(), ch
        loc_ref = ref.reshape(Nq, NO).mean(axis=0)  # [Ω, q] column-major: Ω fastest
        loc = gpu.susceptibility(ch, local=True)
        assert np.abs(loc - loc_ref).max() <= TOL * np.abs(loc_ref).max(), ch


def test_susceptibility_rejects_bad_length():
    """Argument validation happens before any device work."""
    import ctypes
    from fdgasolver import _lib
    lib = _lib.load()
    assert "fdga_susceptibility" in _lib.EXPORTS
    buf = (ctypes.c_double * 2)()
    assert lib.fdga_susceptibility(None, 0, buf, 1) != 0
