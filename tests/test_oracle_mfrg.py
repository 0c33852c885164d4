"""The oracle's restatement of the mfRG linear map (src/mfRG.jl:20-89, caches of
src/nonlocal_2/build_K3_cache.jl:97-165) checked against properties of the reference's algorithm (CPU).

* In the parquet approximation (G0 = 0, so Π0 = 0) every BSE of the map vanishes: A x = x.
* With a bare-U reference vertex the map is real-linear (to 1e-13).
* With RefVertex corrections whose crossed p component is independent of the parallel one, the crossed
  p cache F(γp = false) - F.F0(γp = false) keeps the x-independent term -F0p(Ω,ω,Ω-ν') - F0x(Ω,ω,ν'):
  A is affine, A(0) ≠ 0, as in the reference.
* fixed_point_preconditioned! iterated as x <- x + R converges faster than the plain fixed point.
"""
import numpy as np
import pytest

from helpers import make_oracle

BASE = dict(kind="hubbard", T=0.5, U=2.0, mu=0.3, t1=1.0, t2=-0.2, L=4, nG=8, nK1=8, nK2=(3, 3), nK3=(2, 3),
            mPi_factor=4)


def _cfg(g0=True, noise=False):
    from fdgasolver.models import hubbard_bare_Green
    c = dict(BASE)
    if g0:
        c["G0"] = hubbard_bare_Green(c["T"], c["nG"], c["L"], mu=c["mu"] - 0.2, t1=c["t1"], t2=c["t2"] + 0.1)
        c["Sigma0"] = 0.03 * c["G0"]
    if noise:
        c["refvertex_noise"], c["seed"] = 0.1, 7
    return c


def _vectors(orc):
    x0 = orc.flatten()
    nF = orc.vertex_len()
    orc.iterate("fdPA")
    x1 = orc.flatten()
    orc.iterate("fdPA")
    x2 = orc.flatten()
    orc.unflatten(x0)
    return x1[:nF].copy(), (x2 - x1)[:nF].copy()


def test_mfrg_identity_in_parquet_approximation():
    orc = make_oracle(_cfg(g0=False), True)
    a, b = _vectors(orc)
    assert np.array_equal(orc.mfrg_apply(a), a)


def test_mfrg_linear_with_bare_reference_vertex():
    orc = make_oracle(_cfg(), True)
    a, b = _vectors(orc)
    ya, yb = orc.mfrg_apply(a), orc.mfrg_apply(b)
    y = orc.mfrg_apply(0.3 * a - 1.7 * b)
    assert np.abs(y - (0.3 * ya - 1.7 * yb)).max() <= 1e-13 * np.abs(ya).max()
    assert np.abs(ya - a).max() > 1e-3 * np.abs(a).max()  # the map is not the identity here
    assert np.abs(orc.mfrg_apply(np.zeros_like(a))).max() == 0.0


def test_mfrg_affine_with_crossing_breaking_refvertex():
    orc = make_oracle(_cfg(noise=True), False)
    a, _ = _vectors(orc)
    assert np.abs(orc.mfrg_apply(np.zeros_like(a))).max() > 1e-6


def test_mfrg_preconditioned_iteration_converges():
    pytest.importorskip("scipy")
    orc = make_oracle(_cfg(), True)
    nF = orc.vertex_len()
    x = orc.flatten()[:nF].copy()
    res = []
    for _ in range(4):
        R = orc.fixed_point_preconditioned(x, "fdPA", update_sigma=False, rtol=1e-10, maxiter=50)
        res.append(np.abs(R).max())
        x = x + R
    assert res[-1] < 2e-3 * res[0]
