"""GPU (libfdga, FP64 plain path) vs the CPU oracle: one application of the parquet map
Φ(x) = flatten(iterate_solver!(unflatten!(S, x))) on identical seeded inputs.

Tolerance: every flatten block (K1/K2/K3 of γp, γt, γa and Σ) agrees to 1e-10 relative to the
block's max norm.  Cases cover the local and nonlocal solvers, fdPA and scPA, trivial and
init_sym_grp! symmetry groups, a RefVertex with K3-shaped corrections, the bubble mesh with
1/ν tails, and the full config-2 (Hubbard 8x8) shapes.
"""
import numpy as np
import pytest

from helpers import blockwise_rel_err, make_gpu, make_oracle

pytestmark = pytest.mark.gpu
TOL = 1e-10

SMALL_LOCAL = dict(kind="siam", T=0.1, U=1.0, e=0.2, Delta=0.5, D=10.0, nG=16, nK1=16, nK2=(5, 4), nK3=(4, 4),
                   mPi_factor=6)
SMALL_NL = dict(kind="hubbard", T=0.5, U=2.0, mu=0.3, t1=1.0, t2=-0.2, L=4, nG=8, nK1=8, nK2=(3, 3), nK3=(2, 3),
                mPi_factor=4, refvertex_noise=0.05, seed=7)
ODD_NL = dict(kind="hubbard", T=0.4, U=1.5, mu=0.1, t1=1.0, L=3, nG=6, nK1=6, nK2=(3, 2), nK3=(2, 2), mPi_factor=3,
              refvertex_noise=0.05, seed=3)


# the lattice sizes of the precision (16x16, radix-2 FFT) and differentiation (24x24, 3·2^a FFT)
# configurations, with small frequency boxes so that the oracle finishes in seconds
NL16 = dict(kind="hubbard", T=0.5, U=3.0, mu=-0.3, t1=1.0, t2=-0.2, L=16, nG=4, nK1=4, nK2=(2, 2), nK3=(2, 2),
            mPi_factor=3)
NL24 = dict(kind="hubbard", T=0.5, U=2.5, mu=0.0, t1=1.0, L=24, nG=4, nK1=4, nK2=(2, 2), nK3=(2, 2), mPi_factor=3)
# the other lattices of the mixed-radix (3·2^a) register FFT
NL6 = dict(kind="hubbard", T=0.5, U=2.0, mu=0.2, t1=1.0, t2=-0.1, L=6, nG=6, nK1=6, nK2=(3, 3), nK3=(2, 3),
           mPi_factor=3, refvertex_noise=0.05, seed=5)
NL12 = dict(kind="hubbard", T=0.5, U=2.5, mu=-0.1, t1=1.0, t2=-0.2, L=12, nG=4, nK1=4, nK2=(2, 2), nK3=(2, 2),
            mPi_factor=3)


def _state(S_or, rng, scale=0.05):
    x = S_or.flatten()
    return x + scale * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))


@pytest.mark.parametrize("cfg", [SMALL_LOCAL, SMALL_NL, ODD_NL], ids=["local", "nl4", "nl3odd"])
@pytest.mark.parametrize("sym", [False, True], ids=["trivial", "sym"])
@pytest.mark.parametrize("strategy", ["fdPA", "scPA"])
def test_map_parity(cfg, sym, strategy):
    rng = np.random.default_rng(11)
    orc = make_oracle(cfg, sym)
    gpu = make_gpu(cfg, sym)
    x = _state(orc, rng)
    for _ in range(2):  # two applications: the second exercises a nonzero FL and Σ
        R_orc = orc.residual(x, strategy)
        R_gpu = gpu.fixed_point(x, strategy)
        y_orc = R_orc + x
        y_gpu = R_gpu + x
        assert blockwise_rel_err(cfg, y_gpu, y_orc) < TOL
        x = y_orc + 0.01 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))


@pytest.mark.parametrize("cfg", [NL16, NL24, NL6, NL12], ids=["nl16", "nl24", "nl6", "nl12"])
def test_map_parity_large_lattice(cfg):
    """One map application from the PA start and one from a perturbed state, init_sym_grp! groups."""
    rng = np.random.default_rng(2)
    orc = make_oracle(cfg, True)
    gpu = make_gpu(cfg, True)
    x = orc.flatten()
    for _ in range(2):
        y_orc = orc.residual(x, "fdPA") + x
        y_gpu = gpu.fixed_point(x, "fdPA") + x
        assert blockwise_rel_err(cfg, y_gpu, y_orc) < TOL
        x = y_orc + 0.01 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))


@pytest.mark.parametrize("cfg", [SMALL_LOCAL, SMALL_NL], ids=["local", "nl4"])
def test_intermediates(cfg):
    """Bubbles, K3 caches and the left vertex FL after one fdPA iteration."""
    rng = np.random.default_rng(5)
    # trivial groups: with init_sym_grp! only the (P, Ω) blocks holding class representatives of
    # the caches are computed
    orc = make_oracle(cfg, False)
    gpu = make_gpu(cfg, False)
    for name in ("Pi0pp", "Pi0ph", "Pipp", "Piph", "G"):
        a, b = gpu.get(name), orc.get(name)
        assert np.abs(a - b).max() <= TOL * max(np.abs(b).max(), 1e-300), name
    x = _state(orc, rng)
    orc.unflatten(x); orc.iterate("fdPA")
    gpu.unflatten(x); gpu.iterate_solver("fdPA")
    names = ["cache_Gpx", "cache_F0p", "cache_F0a", "cache_F0t", "cache_Gpp", "cache_Ga", "cache_Gt", "cache_Fp",
             "cache_Fa", "cache_Ft"] + [f"FL.{c}.K{k}" for c in "pta" for k in (2, 3)]
    for name in names:
        a, b = gpu.get(name), orc.get(name)
        assert np.abs(a - b).max() <= TOL * max(np.abs(b).max(), 1e-300), name


def test_flatten_roundtrip_and_layout():
    cfg = SMALL_NL
    gpu = make_gpu(cfg, False)
    rng = np.random.default_rng(2)
    x = rng.standard_normal(gpu.state_len) + 1j * rng.standard_normal(gpu.state_len)
    gpu.unflatten(x)
    assert np.array_equal(gpu.flatten(), x)
    # named blocks come back in the reference's column-major layout
    n1 = (2 * cfg["nK1"] - 1) * cfg["L"] ** 2
    assert np.array_equal(gpu.get("F.p.K1"), x[:n1])


def test_hubbard8x8_map_parity():
    """Full config-2 shapes (Hubbard 8x8, nK3=(8,12), mΠν_factor=32, synthetic RefVertex), sym groups."""
    from fdgasolver.workloads import CONFIGS
    cfg = dict(CONFIGS["hubbard8x8_b5_nk3_8x12"])
    orc = make_oracle(cfg, True)
    gpu = make_gpu(cfg, True)
    rng = np.random.default_rng(3)
    x = _state(orc, rng, 0.02)
    y_orc = orc.residual(x, "fdPA") + x
    y_gpu = gpu.fixed_point(x, "fdPA") + x
    assert blockwise_rel_err(cfg, y_gpu, y_orc) < TOL


def test_solve_matches_oracle_trajectory():
    """solve! (Anderson m=8, β=0.5) on the device follows the oracle's trajectory."""
    cfg = SMALL_NL
    orc = make_oracle(cfg, True)
    gpu = make_gpu(cfg, True)
    r_o = orc.solve("fdPA", maxiter=40, tol=1e-10, beta=0.5, mem=8)
    r_g = gpu.solve("fdPA", maxiter=40, tol=1e-10, delta=0.5, mem=8)
    assert r_o["converged"] and r_g["converged"]
    assert r_o["iterations"] == r_g["iterations"]
    assert blockwise_rel_err(cfg, gpu.flatten(), orc.flatten()) < 1e-9


@pytest.mark.parametrize("case,e,nK2", [("half_filling", 0.0, (6, 6)), ("doped", 0.5, (7, 6))])
def test_siam_scpa_reference_golden_on_gpu(case, e, nK2):
    """The reference's own golden values (test/test_siam_scPA.jl, bubble mesh factor 1) from the
    device solve! (Anderson m = 8, β = 0.85, tol 1e-4 as the reference), to the 5e-4 that the
    stopping tolerance allows."""
    import json
    import os

    from fdgasolver.solver import parquet_solver_siam_parquet_approximation
    from test_oracle_golden import _c, _k1_at
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_golden.json")))
    g = gold[f"siam_scPA_{case}"]
    T, U, nG, nK1 = 0.1, 1.0, 36, 24
    S = parquet_solver_siam_parquet_approximation(nG, nK1, nK2, nK2, e=e, Delta=np.pi / 5, D=10.0, T=T, U=U,
                                                  mPi_factor=1)
    S.init_sym_grp()
    r = S.solve("scPA", maxiter=100, tol=1e-4, delta=0.85, mem=8)
    assert r["converged"]
    sig = S.get("Sigma")[np.array([-2, -1, 0, 1]) + nG]
    assert np.max(np.abs(sig - _c(g["Sigma"])) / np.abs(_c(g["Sigma"]))) < 5e-4
    xs = 2 * np.pi * T * -2 + np.arange(4) * 1.0
    for ch in "apt":
        k1 = S.get(f"F.{ch}.K1")
        v = np.array([_k1_at(k1, x, T, nK1) for x in xs])
        assert np.max(np.abs(v - _c(g[ch])) / np.abs(_c(g[ch]))) < 5e-4, ch
    S.close()
