"""Newton–Krylov solve, Jacobian-vector products and the linear response dχ/dU.

(1) fdga_jvp agrees with central differences of the oracle's map (step 1e-6) to 1e-6 relative.
(2) fdga_solve_newton reaches the FP64 fixed point (FP64 and mixed JVPs, by the tangent kernels
    and by differences): converged at 1e-10 on the FP64 residual, state within 1e-8 of the
    oracle's Anderson solution.
(3) dχ_m/dU and dχ_d/dU at the fixed point (GMRES on (I − J) dx/dU = ∂Φ/∂U) agree with central
    differences h = 1e-4 of the oracle's converged χ at U ± h to 1e-6 relative.  The RefVertex
    is the bare U here, so that the reference vertex depends on U only through U itself.
"""
import numpy as np
import pytest

from helpers import blockwise_rel_err, make_gpu, make_oracle

NL4 = dict(kind="hubbard", T=0.5, U=2.0, mu=0.3, t1=1.0, t2=-0.2, L=4, nG=8, nK1=8, nK2=(3, 3), nK3=(2, 3),
           mPi_factor=4)
NL4_NOISE = dict(NL4, refvertex_noise=0.05, seed=7)
LOCAL = dict(kind="siam", T=0.1, U=1.0, e=0.2, Delta=0.5, D=10.0, nG=16, nK1=16, nK2=(5, 4), nK3=(4, 4),
             mPi_factor=6)


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [NL4_NOISE, LOCAL], ids=["nl4", "local"])
def test_jvp_matches_oracle_differences(cfg):
    rng = np.random.default_rng(8)
    orc = make_oracle(cfg, True)
    gpu = make_gpu(cfg, True)
    x = orc.flatten()
    for _ in range(3):
        x = x + 0.5 * orc.residual(x)
    v = rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size)
    h = 1e-6
    ref = ((orc.residual(x + h * v) + x + h * v) - (orc.residual(x - h * v) + x - h * v)) / (2 * h)
    gpu.unflatten(x)
    got = gpu.jvp(v)
    assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max()


@pytest.mark.gpu
@pytest.mark.parametrize("tangent", [1, 0], ids=["tangent", "differences"])
@pytest.mark.parametrize("jvp", ["fp64", "mixed"])
@pytest.mark.parametrize("cfg", [NL4_NOISE, LOCAL], ids=["nl4", "local"])
def test_newton_reaches_fixed_point(cfg, jvp, tangent):
    orc = make_oracle(cfg, True)
    gpu = make_gpu(cfg, True)
    gpu.set_option("jvp_tangent", tangent)
    r_o = orc.solve("fdPA", maxiter=300, tol=1e-11, beta=0.5, mem=8)
    r_g = gpu.solve_newton("fdPA", maxiter=400, tol=1e-10, restart=30, jvp=jvp)
    assert r_o["converged"] and r_g["converged"], (r_g["trace"], r_g["evals_fp64"], r_g["evals_mixed"])
    assert blockwise_rel_err(cfg, gpu.flatten(), orc.flatten()) < 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize("tangent", [1, 0], ids=["tangent", "differences"])
@pytest.mark.parametrize("cfg", [NL4, LOCAL], ids=["nl4", "local"])
def test_dchi_dU_matches_oracle_differences(cfg, tangent):
    h = 1e-4
    chi = {}
    for sgn in (+1, -1):
        c = dict(cfg, U=cfg["U"] + sgn * h)
        o = make_oracle(c, True)
        r = o.solve("fdPA", maxiter=400, tol=1e-13, beta=0.5, mem=8)
        assert r["converged"]
        K1a, K1t = o.get("F.a.K1"), o.get("F.t.K1")
        chi[sgn] = {"m": K1a / c["U"] ** 2, "d": (K1a - 2 * K1t) / c["U"] ** 2}
    gpu = make_gpu(cfg, True)
    gpu.set_option("jvp_tangent", tangent)
    r = gpu.solve("fdPA", maxiter=400, tol=1e-13, delta=0.5, mem=8)
    assert r["converged"]
    for ch in ("m", "d"):
        ref = (chi[+1][ch] - chi[-1][ch]) / (2 * h)
        got, info = gpu.dchi_dU(ch, hU=1e-4, restart=40, cycles=4, rtol=1e-10)
        assert np.abs(got - ref).max() <= 1e-6 * np.abs(ref).max(), (ch, info)


def test_newton_entry_points_exported():
    from fdgasolver import _lib
    lib = _lib.load()
    for name in ("fdga_solve_newton", "fdga_jvp", "fdga_set_U", "fdga_dchi_dU"):
        assert hasattr(lib, name) and name in _lib.EXPORTS
    assert lib.fdga_set_U(None, 1.0) != 0
