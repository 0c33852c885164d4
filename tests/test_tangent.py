"""Tangent map (fdga_frule): the hand-written forward-mode derivative of one iteration.

(1) With Σ, G and Π held fixed (update_sigma = false) the map is quadratic in the vertex, so the
    central difference (Φ(x + hv) − Φ(x − hv))/(2h) of the oracle is its exact derivative up to
    rounding: fdga_frule agrees with it to 1e-10 relative per flatten block.
(2) The full map (Dyson, bubbles, SDE included): fdga_frule agrees with Richardson-extrapolated
    central differences of the oracle (steps h and h/2, truncation O(h⁴)) to 1e-8 relative.
(3) The value y = Φ(x) returned beside the derivative is the plain map (1e-10 against the oracle).
(4) The tangent of the mixed-precision map agrees with the FP64 tangent to 2e-5 relative.
"""
import numpy as np
import pytest

from helpers import blockwise_rel_err, make_gpu, make_oracle

pytestmark = pytest.mark.gpu

LOCAL = dict(kind="siam", T=0.1, U=1.0, e=0.2, Delta=0.5, D=10.0, nG=16, nK1=16, nK2=(5, 4), nK3=(4, 4),
             mPi_factor=6)
NL4 = dict(kind="hubbard", T=0.5, U=2.0, mu=0.3, t1=1.0, t2=-0.2, L=4, nG=8, nK1=8, nK2=(3, 3), nK3=(2, 3),
           mPi_factor=4, refvertex_noise=0.05, seed=7)
NL3 = dict(kind="hubbard", T=0.4, U=1.5, mu=0.1, t1=1.0, L=3, nG=6, nK1=6, nK2=(3, 2), nK3=(2, 2), mPi_factor=3,
           refvertex_noise=0.05, seed=3)
CFGS = [LOCAL, NL4, NL3]
IDS = ["local", "nl4", "nl3odd"]


def _base(orc, rng, strategy):
    """A state near the PA start with nonzero FL and Σ (two damped map applications, then noise)."""
    x = orc.flatten()
    for _ in range(2):
        x = x + 0.5 * orc.residual(x, strategy)
    return x + 0.02 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))


def _dir(rng, n):
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


def _orc_map(orc, x, strategy, update_sigma):
    orc.unflatten(x)
    orc.iterate(strategy, update_sigma=update_sigma)
    return orc.flatten()


@pytest.mark.parametrize("cfg", CFGS, ids=IDS)
@pytest.mark.parametrize("sym", [False, True], ids=["trivial", "sym"])
@pytest.mark.parametrize("strategy", ["fdPA", "scPA"])
def test_frule_exact_on_fixed_bubble(cfg, sym, strategy):
    rng = np.random.default_rng(21)
    orc = make_oracle(cfg, sym)
    gpu = make_gpu(cfg, sym)
    x = _base(orc, rng, strategy)
    # the same G and Π in both: one full application at x
    orc.residual(x, strategy)
    gpu.fixed_point(x, strategy)
    v = _dir(rng, x.size)
    h = 1e-3
    ref = (_orc_map(orc, x + h * v, strategy, False) - _orc_map(orc, x - h * v, strategy, False)) / (2 * h)
    gpu.unflatten(x)
    y, jv = gpu.frule(v, strategy, update_sigma=False)
    assert blockwise_rel_err(cfg, jv, ref) < 1e-10
    assert blockwise_rel_err(cfg, y, _orc_map(orc, x, strategy, False)) < 1e-10


@pytest.mark.parametrize("cfg", CFGS, ids=IDS)
@pytest.mark.parametrize("sym", [False, True], ids=["trivial", "sym"])
@pytest.mark.parametrize("strategy", ["fdPA", "scPA"])
def test_frule_full_map(cfg, sym, strategy):
    rng = np.random.default_rng(5)
    orc = make_oracle(cfg, sym)
    gpu = make_gpu(cfg, sym)
    x = _base(orc, rng, strategy)
    v = _dir(rng, x.size)
    h = 2e-3

    def phi(z):
        return orc.residual(z, strategy) + z

    d1 = (phi(x + h * v) - phi(x - h * v)) / (2 * h)
    d2 = (phi(x + 0.5 * h * v) - phi(x - 0.5 * h * v)) / h
    ref = (4 * d2 - d1) / 3
    gpu.unflatten(x)
    y, jv = gpu.frule(v, strategy)
    assert blockwise_rel_err(cfg, jv, ref) < 1e-8
    assert blockwise_rel_err(cfg, y, phi(x)) < 1e-10
    # the state is left at x
    assert np.abs(gpu.flatten() - x).max() == 0.0


@pytest.mark.parametrize("cfg", [LOCAL, NL4, NL3], ids=["local", "nl4", "nl3odd"])
def test_frule_mixed_precision(cfg):
    rng = np.random.default_rng(9)
    orc = make_oracle(cfg, True)
    gpu = make_gpu(cfg, True)
    x = _base(orc, rng, "fdPA")
    v = _dir(rng, x.size)
    gpu.unflatten(x)
    _, j64 = gpu.frule(v)
    gpu.set_precision("mixed")
    _, j32 = gpu.frule(v)
    gpu.set_precision("fp64")
    err = blockwise_rel_err(cfg, j32, j64)
    assert 0 < err < 2e-5


def test_frule_hubbard8x8_shapes():
    """Full config-2 shapes (Hubbard 8x8, sym groups): enough (P, Ω) rows that the K2 kernels run
    their 4-warp CTAs.  FP64 tangent vs Richardson central differences of the oracle (1e-8); the
    mixed tangent vs the FP64 tangent (2e-5)."""
    from fdgasolver.workloads import CONFIGS
    cfg = dict(CONFIGS["hubbard8x8_b5_nk3_8x12"])
    rng = np.random.default_rng(13)
    orc = make_oracle(cfg, True)
    gpu = make_gpu(cfg, True)
    x = orc.flatten()
    x = x + 0.5 * orc.residual(x, "fdPA")
    v = _dir(rng, x.size)
    h = 2e-3

    def phi(z):
        return orc.residual(z, "fdPA") + z

    d1 = (phi(x + h * v) - phi(x - h * v)) / (2 * h)
    d2 = (phi(x + 0.5 * h * v) - phi(x - 0.5 * h * v)) / h
    ref = (4 * d2 - d1) / 3
    gpu.unflatten(x)
    _, j64 = gpu.frule(v)
    assert blockwise_rel_err(cfg, j64, ref) < 1e-8
    gpu.set_precision("mixed")
    gpu.unflatten(x)
    _, j32 = gpu.frule(v)
    assert 0 < blockwise_rel_err(cfg, j32, j64) < 2e-5
    gpu.close()


def test_tangent_refuses_strategies_without_a_tangent_map():
    """The tangent graphs exist for :fdPA and :scPA; other strategies are refused, not indexed."""
    from fdgasolver import _lib
    gpu = make_gpu(NL4, True)
    x = gpu.flatten()
    gpu.frule(_dir(np.random.default_rng(1), x.size))
    with pytest.raises(_lib.FdgaError) as e:
        gpu.tangent_repeat(1, "fdPA_1loop")
    assert e.value.code == 2  # FDGA_ERR_UNSUPPORTED
    gpu.tangent_repeat(1, "fdPA")  # still usable
    gpu.close()
