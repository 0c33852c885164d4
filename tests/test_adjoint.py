"""Adjoint map (fdga_rrule): the hand-written reverse-mode derivative of one iteration.

The transpose identity <ȳ, Φ'(x) v> = <Φ'(x)ᵀ ȳ, v> (real inner product Re Σ conj(a) b) holds
between fdga_rrule and the tangent map fdga_frule, itself pinned to the oracle's central
differences, for random v and ȳ: relative to ‖ȳ‖‖Φ'(x) v‖ the two sides agree to 1e-12.  Cases:
the local and nonlocal solvers (radix-2 and DFT lattices), trivial and init_sym_grp! groups, fdPA
and scPA, with and without the Σ update.  y = Φ(x) returned beside the cotangent is the map.
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


def _rdot(a, b):
    return float(np.real(np.vdot(a, b)))


@pytest.mark.parametrize("cfg", [LOCAL, NL4, NL3], ids=["local", "nl4", "nl3odd"])
@pytest.mark.parametrize("sym", [False, True], ids=["trivial", "sym"])
@pytest.mark.parametrize("strategy", ["fdPA", "scPA"])
@pytest.mark.parametrize("update_sigma", [True, False], ids=["full", "fixed_bubble"])
def test_rrule_is_transpose_of_frule(cfg, sym, strategy, update_sigma):
    rng = np.random.default_rng(31)
    orc = make_oracle(cfg, sym)
    gpu = make_gpu(cfg, sym)
    x = orc.flatten()
    for _ in range(2):
        x = x + 0.5 * orc.residual(x, strategy)
    x = x + 0.02 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
    gpu.fixed_point(x, strategy)  # G and Π of x for the fixed-bubble map
    for _ in range(2):
        v = rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size)
        yb = rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size)
        gpu.unflatten(x)
        y1, jv = gpu.frule(v, strategy, update_sigma=update_sigma)
        gpu.unflatten(x)
        y2, xb = gpu.rrule(yb, strategy, update_sigma=update_sigma)
        lhs, rhs = _rdot(yb, jv), _rdot(xb, v)
        scale = np.linalg.norm(yb) * np.linalg.norm(jv)
        assert abs(lhs - rhs) <= 1e-12 * scale, (lhs, rhs, scale)
        assert blockwise_rel_err(cfg, y2, y1) < 1e-12
