"""The strategy variants of iterate_solver! (src/solve.jl:26-82) against the oracle.

:fdPA_new / :scPA_new (local solver): K1 and K2 in the form (F Π - F0 Π0) U
(src/BSEa/BSEa_K1.jl:57-100, src/BSEa/BSEa_K2.jl:104-150), K3 and (fdPA_new) FL.K3 as in fdPA.
:fdPA_1loop (nonlocal solver): the one-loop BSEs F (Π - Π0) F0 (src/nonlocal/BSEa/BSE_1loop.jl).
Two map applications per case agree with the oracle to 1e-10 per flatten block; the
combinations without a reference method are refused; the mixed map of a variant agrees with its
FP64 map to 1e-5.
"""
import numpy as np
import pytest

from helpers import blockwise_rel_err, make_gpu, make_oracle

LOCAL = dict(kind="siam", T=0.1, U=1.0, e=0.2, Delta=0.5, D=10.0, nG=16, nK1=16, nK2=(5, 4), nK3=(4, 4),
             mPi_factor=6)
LOCAL_RV = dict(LOCAL, refvertex_noise=0.05, seed=5)
NL4 = dict(kind="hubbard", T=0.5, U=2.0, mu=0.3, t1=1.0, t2=-0.2, L=4, nG=8, nK1=8, nK2=(3, 3), nK3=(2, 3),
           mPi_factor=4, refvertex_noise=0.05, seed=7)
NL3 = dict(kind="hubbard", T=0.4, U=1.5, mu=0.1, t1=1.0, L=3, nG=6, nK1=6, nK2=(3, 2), nK3=(2, 2), mPi_factor=3,
           refvertex_noise=0.05, seed=3)

CASES = [(LOCAL, "fdPA_new"), (LOCAL, "scPA_new"), (LOCAL_RV, "fdPA_new"), (LOCAL_RV, "scPA_new"),
         (NL4, "fdPA_1loop"), (NL3, "fdPA_1loop")]
IDS = ["local-fdPA_new", "local-scPA_new", "localrv-fdPA_new", "localrv-scPA_new", "nl4-fdPA_1loop",
       "nl3-fdPA_1loop"]


@pytest.mark.gpu
@pytest.mark.parametrize("cfg,strategy", CASES, ids=IDS)
@pytest.mark.parametrize("sym", [False, True], ids=["trivial", "sym"])
def test_variant_map_parity(cfg, strategy, sym):
    rng = np.random.default_rng(17)
    orc = make_oracle(cfg, sym)
    gpu = make_gpu(cfg, sym)
    x = orc.flatten()
    x = x + 0.05 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
    for _ in range(2):
        y_orc = orc.residual(x, strategy) + x
        y_gpu = gpu.fixed_point(x, strategy) + x
        assert blockwise_rel_err(cfg, y_gpu, y_orc) < 1e-10
        x = y_orc + 0.01 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))


@pytest.mark.gpu
@pytest.mark.parametrize("cfg,strategy", [(LOCAL_RV, "fdPA_new"), (NL4, "fdPA_1loop")], ids=["local", "nl4"])
def test_variant_mixed_map(cfg, strategy):
    rng = np.random.default_rng(4)
    gpu = make_gpu(cfg, True)
    x = gpu.flatten()
    x = x + 0.05 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
    y64 = gpu.fixed_point(x, strategy) + x
    gpu.set_precision("mixed")
    y32 = gpu.fixed_point(x, strategy) + x
    assert blockwise_rel_err(cfg, y32, y64) < 1e-5


@pytest.mark.gpu
def test_variants_without_reference_method_are_refused():
    from fdgasolver import _lib
    for cfg, strategy in ((LOCAL, "fdPA_1loop"), (NL4, "fdPA_new"), (NL4, "scPA_new")):
        gpu = make_gpu(cfg, False)
        with pytest.raises(_lib.FdgaError) as e:
            gpu.fixed_point(gpu.flatten(), strategy)
        assert e.value.code == 2  # FDGA_ERR_UNSUPPORTED


def test_oracle_variants_solve_local():
    """CPU: the _new forms converge to a fixed point near the fdPA one (a different truncation)."""
    orc = make_oracle(LOCAL, True)
    r = orc.solve("fdPA", maxiter=300, tol=1e-10, beta=0.5, mem=8)
    x = orc.flatten()
    assert r["converged"]
    r2 = orc.solve("fdPA_new", maxiter=300, tol=1e-10, beta=0.5, mem=8)
    assert r2["converged"]
    x2 = orc.flatten()
    assert 0 < np.abs(x2 - x).max() < 0.1 * np.abs(x).max()
