"""Mixed-precision path: FP32 K3 contractions inside the map, FP64 iterative refinement outside.

(1) One map application in FDGA_MIXED agrees with FDGA_FP64 to FP32 accuracy (1e-5 relative per
    flatten block) and differs from it (the FP32 kernels ran).
(2) fdga_solve_mixed reaches the FP64 fixed point: converged at tol 1e-10 on the FP64 residual,
    the state and χ_m / χ_d agree with the CPU oracle's Anderson solution (tol 1e-10) to 1e-8
    relative.
"""
import numpy as np
import pytest

from helpers import blockwise_rel_err, make_gpu, make_oracle

SMALL_LOCAL = dict(kind="siam", T=0.1, U=1.0, e=0.2, Delta=0.5, D=10.0, nG=16, nK1=16, nK2=(5, 4), nK3=(4, 4),
                   mPi_factor=6)
SMALL_NL = dict(kind="hubbard", T=0.5, U=2.0, mu=0.3, t1=1.0, t2=-0.2, L=4, nG=8, nK1=8, nK2=(3, 3), nK3=(2, 3),
                mPi_factor=4, refvertex_noise=0.05, seed=7)
# an odd lattice: the mixed map's FP32 bubble takes the DFT path
ODD_NL = dict(kind="hubbard", T=0.4, U=1.5, mu=0.1, t1=1.0, L=3, nG=6, nK1=6, nK2=(3, 2), nK3=(2, 2), mPi_factor=3,
              refvertex_noise=0.05, seed=3)


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [SMALL_LOCAL, SMALL_NL, ODD_NL], ids=["local", "nl4", "nl3odd"])
def test_mixed_map_close_to_fp64(cfg):
    rng = np.random.default_rng(4)
    gpu = make_gpu(cfg, True)
    x = gpu.flatten()
    x = x + 0.05 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
    y = gpu.fixed_point(x, "fdPA") + x  # FP64, also makes FL and Σ nonzero for the next call
    y64 = gpu.fixed_point(y, "fdPA") + y
    gpu.set_precision("mixed")
    y32 = gpu.fixed_point(y, "fdPA") + y
    gpu.set_precision("fp64")
    err = blockwise_rel_err(cfg, y32, y64)
    assert err < 1e-5
    assert err > 1e-12  # the FP32 contractions were used


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [SMALL_LOCAL, SMALL_NL], ids=["local", "nl4"])
def test_solve_mixed_reaches_fp64_fixed_point(cfg):
    orc = make_oracle(cfg, True)
    gpu = make_gpu(cfg, True)
    r_o = orc.solve("fdPA", maxiter=200, tol=1e-10, beta=0.5, mem=8)
    r_g = gpu.solve_mixed("fdPA", maxiter=400, tol=1e-10, delta=0.5, mem=8)
    assert r_o["converged"] and r_g["converged"]
    assert r_g["residual"] < 1e-10
    assert r_g["evals_mixed"] > r_g["evals_fp64"]
    assert blockwise_rel_err(cfg, gpu.flatten(), orc.flatten()) < 1e-8
    U = cfg["U"]
    K1 = {c: orc.get(f"F.{c}.K1") for c in "ta"}
    for ch, ref in (("m", K1["a"] / U ** 2), ("d", (K1["a"] - 2 * K1["t"]) / U ** 2)):
        got = gpu.susceptibility(ch)
        assert np.abs(got - ref).max() <= 1e-8 * np.abs(ref).max(), ch


def test_mixed_entry_points_exported():
    from fdgasolver import _lib
    lib = _lib.load()
    for name in ("fdga_set_precision", "fdga_solve_mixed"):
        assert hasattr(lib, name) and name in _lib.EXPORTS
    assert lib.fdga_set_precision(None, 1) != 0
