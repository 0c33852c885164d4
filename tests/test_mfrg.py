"""mfRG / Krylov-preconditioned solver on the GPU: mfRGLinearMap (src/mfRG.jl:20-89) with the caches of
the two-argument build_K3_cache_mfRG! that the map dispatches to on the nonlocal solver
(src/nonlocal_2/build_K3_cache.jl:97-165), the is_mfRG BSE branches (src/nonlocal/BSEa/BSEa_K1.jl:29-37,
BSEa_K2.jl:70-77, BSEa_K3.jl:83-97), fixed_point_preconditioned! (src/mfRG.jl:93-173) and the Anderson
driver solve_using_mfRG_without_mixing! (src/mfRG.jl:686-776).

Tolerances: one application of the FP64 map agrees with the oracle's restatement to 1e-10 relative per
flatten block; the mixed map to 1e-5.  The preconditioned residual, whose Krylov solve runs to
rtol 1e-7 on the GPU (FP32 Krylov basis with FP64 residuals: its floor is near 1e-7; the reference asks
1e-6) and to 1e-12 in the oracle (scipy GMRES on the real-linear map), agrees to 1e-5.  The preconditioned Anderson solve reaches the same fixed point as the
plain solve to 1e-7.

The reference map is linear in x only when F(γr = false) - F.F0(γr = false) has no x-independent part:
a bare-U or crossing-symmetric RefVertex.  A Vertex-valued F0 (its own γr survives that difference,
since the nonlocal vertex evaluates its F0 without the channel flags) and RefVertex data that break
crossing symmetry make it affine; the parity cases cover both, the linearity and solve cases use
linear maps.
"""
import numpy as np
import pytest

from helpers import blockwise_rel_err, make_gpu, make_oracle

pytestmark = pytest.mark.gpu
TOL = 1e-10

BASE = dict(kind="hubbard", T=0.5, U=2.0, mu=0.3, t1=1.0, t2=-0.2, L=4, nG=8, nK1=8, nK2=(3, 3), nK3=(2, 3),
            mPi_factor=4)
ODD = dict(kind="hubbard", T=0.4, U=1.5, mu=0.1, t1=1.0, t2=0.0, L=3, nG=6, nK1=6, nK2=(3, 2), nK3=(2, 2),
           mPi_factor=3)


def _with_reference_system(cfg, refvertex=None):
    """The target system with a nonzero reference Green function G0 (a shifted model) and Σ0, so that
    Π0 ≠ 0 (in the parquet approximation G0 = 0 and the map is the identity)."""
    import fdgasolver as F
    c = dict(cfg)
    c["G0"] = F.hubbard_bare_Green(c["T"], c["nG"], c["L"], mu=c["mu"] - 0.2, t1=c["t1"], t2=c["t2"] + 0.1)
    c["Sigma0"] = 0.03 * c["G0"]
    if refvertex == "noise":  # independent Fp_p/Fp_x/Ft_p/Ft_x: the crossed p cache keeps a constant term
        c["refvertex_noise"], c["seed"] = 0.1, 7
    return c


def _crossing_refvertex(cfg, nR, sigma=0.1, seed=11):
    """RefVertex corrections with Fp_x(Ω,ν,ν') = -Fp_p(Ω,ν,Ω-ν') (Fp_p supported where both ν' and
    Ω-ν' lie in the box): the crossed p cache of the map then has no constant term."""
    import fdgasolver as F
    rng = np.random.default_rng(seed)
    nO, nn = nR
    NO, Nn = 2 * nO - 1, 2 * nn
    z = lambda: (rng.standard_normal((NO, Nn, Nn)) + 1j * rng.standard_normal((NO, Nn, Nn))) * sigma * cfg["U"]
    pp, tp, tx = z(), z(), z()
    px = np.zeros_like(pp)
    for iO in range(NO):
        m = iO - (nO - 1)
        for ib in range(Nn):
            jb = (m - (ib - nn) - 1) + nn  # index of Ω - ν' (fermionic index m - b - 1)
            if 0 <= jb < Nn:
                px[iO, :, ib] = -pp[iO, :, jb]
            else:  # crossing partner outside the box: no correction (crossing is an involution)
                pp[iO, :, ib] = 0.0
    return F.RefVertex(cfg["T"], cfg["U"], pp, px, tp, tx)


def _pair(cfg, sym, refvertex=None):
    import fdgasolver as F
    from oracle import oracle as O
    c = _with_reference_system(cfg, refvertex if refvertex == "noise" else None)
    if refvertex == "crossing":
        rv = _crossing_refvertex(c, (2, 3))
        Gb, G0, S0 = F.hubbard_bare_Green(c["T"], c["nG"], c["L"], mu=c["mu"], t1=c["t1"], t2=c["t2"]), c["G0"], c["Sigma0"]
        orc = O.OracleSolver(nG=c["nG"], nK1=c["nK1"], nK2=c["nK2"], nK3=c["nK3"], T=c["T"], U=c["U"], L=c["L"],
                             local=False, mPi_factor=c["mPi_factor"], nR=rv.nR)
        orc.set("Gbare", Gb)
        orc.set("G0", G0)
        orc.set("Sigma0", S0)
        for n, a in zip(["Fp_p", "Fp_x", "Ft_p", "Ft_x"], rv.arrays):
            orc.set(n, a)
        orc.finalize()
        gpu = F.NL_ParquetSolver(c["nK1"], c["nK2"], c["nK3"], c["L"], Gb, G0, S0, rv, mPi_factor=c["mPi_factor"])
        if sym:
            orc.init_sym_grp()
            gpu.init_sym_grp()
        return c, orc, gpu
    return c, make_oracle(c, sym), make_gpu(c, sym)


def _states(orc, n=3):
    """Symmetric vertex vectors: the vertex part of successive iterates (and their differences)."""
    out = []
    x = orc.flatten()
    nF = orc.vertex_len()
    for _ in range(n):
        orc.iterate("fdPA")
        y = orc.flatten()
        out.append(y[:nF].copy())
        out.append((y - x)[:nF].copy())
        x = y
    orc.unflatten(x)
    return out


def _vertex_err(cfg, a, b):
    nS = 2 * cfg["nG"] * cfg["L"] ** 2
    pad = np.zeros(nS, dtype=np.complex128)
    return blockwise_rel_err(cfg, np.concatenate([a, pad]), np.concatenate([b, pad]))


CASES = [(BASE, False, "noise"), (BASE, True, None), (BASE, False, "crossing"), (ODD, True, None)]
IDS = ["nl4-trivial-noisy-refvertex", "nl4-sym-U", "nl4-trivial-crossing-refvertex", "nl3odd-sym-U"]


@pytest.mark.parametrize("cfg,sym,rv", CASES, ids=IDS)
def test_mfrg_map_parity(cfg, sym, rv):
    c, orc, gpu = _pair(cfg, sym, rv)
    for strategy in ("fdPA", "fdPA_1loop"):
        for x in _states(orc, 2):
            y_orc = orc.mfrg_apply(x)
            y_gpu = gpu.mfrg_apply(x, strategy)
            assert _vertex_err(c, y_gpu, y_orc) < TOL, strategy
    gpu.close()


def test_mfrg_map_vertex_reference():
    """A Vertex-valued F0 (fdDΓA from a solved reference system): its own γr enters the Γ caches."""
    import test_vertex_reference as V
    cfg, box = V.NL4, V.F0_BOX["nl4"][0]
    for sym in (False, True):
        orc, gpu = V._pair(cfg, box, sym)
        x = orc.flatten()
        nF = orc.vertex_len()
        for _ in range(2):
            orc.iterate("fdPA")
            v = orc.flatten()[:nF].copy()
            assert blockwise_rel_err(V._bcfg(cfg), np.concatenate([gpu.mfrg_apply(v), x[nF:]]),
                                     np.concatenate([orc.mfrg_apply(v), x[nF:]])) < TOL
        gpu.close()


def test_mfrg_map_mixed_and_linear():
    c, orc, gpu = _pair(BASE, True, None)
    xs = _states(orc, 2)
    for x in xs:
        y64 = gpu.mfrg_apply(x)
        assert _vertex_err(c, y64, orc.mfrg_apply(x)) < TOL
    # real-linear (the symmetry operations conjugate): A(a x1 + b x2) = a A x1 + b A x2 for real a, b
    a, b = 0.7, -1.3
    lhs = gpu.mfrg_apply(a * xs[0] + b * xs[1])
    rhs = a * gpu.mfrg_apply(xs[0]) + b * gpu.mfrg_apply(xs[1])
    assert np.abs(lhs - rhs).max() <= 1e-12 * np.abs(rhs).max()
    gpu.set_precision("mixed")
    for x in xs[:2]:
        assert _vertex_err(c, gpu.mfrg_apply(x), orc.mfrg_apply(x)) < 1e-5
    gpu.close()


def test_mfrg_rejections():
    from fdgasolver import FdgaError, mfRGLinearMap
    c, orc, gpu = _pair(BASE, False, None)
    n = orc.vertex_len()
    with pytest.raises(FdgaError):
        gpu.mfrg_apply(np.zeros(n), "fdPA_new")  # the _new BSEs are a local-solver strategy here
    with pytest.raises(FdgaError):
        gpu.mfrg_apply(np.zeros(n + 1))
    with pytest.raises(ValueError):
        mfRGLinearMap(gpu, "scPA")
    A = mfRGLinearMap(gpu, "fdPA")
    assert A.shape == (n, n)
    x = _states(orc, 1)[0]
    assert np.array_equal(A * x, gpu.mfrg_apply(x))
    gpu.close()


@pytest.mark.parametrize("update_sigma", [False, True], ids=["vertex", "vertex+sigma"])
@pytest.mark.parametrize("rv", [None, "crossing"], ids=["U", "crossing-refvertex"])
def test_fixed_point_preconditioned(update_sigma, rv):
    c, orc, gpu = _pair(BASE, rv is None, rv)
    x = orc.flatten()
    nF = orc.vertex_len()
    orc.iterate("fdPA")
    x = orc.flatten() + 0.01 * (x - orc.flatten())  # a symmetric state off the fixed point
    xin = x if update_sigma else x[:nF]
    gpu.unflatten(x)
    R_gpu, info = gpu.fixed_point_preconditioned(xin, "fdPA", update_sigma=update_sigma, krylov_maxiter=400,
                                                 krylov_rtol=1e-7, krylov_atol=0.0)
    orc.unflatten(x)
    R_orc = orc.fixed_point_preconditioned(xin, "fdPA", update_sigma=update_sigma, rtol=1e-12)
    assert info["krylov_iterations"] > 0 and info["krylov_residual"] < 1e-6
    assert np.abs(R_gpu[:nF] - R_orc[:nF]).max() <= 1e-5 * np.abs(R_orc[:nF]).max()
    if update_sigma:
        assert np.abs(R_gpu[nF:] - R_orc[nF:]).max() <= 1e-10 * max(np.abs(R_orc[nF:]).max(), 1e-300)
    gpu.close()


def test_solve_mfrg_converges_to_plain_fixed_point():
    c, orc, gpu = _pair(BASE, True, None)
    x0 = gpu.flatten()
    ref = gpu.solve("fdPA", maxiter=300, tol=1e-10, delta=0.5, mem=8)
    assert ref["converged"]
    x_plain = gpu.flatten()
    gpu.unflatten(x0)
    out = gpu.solve_mfrg("fdPA", maxiter=40, tol=1e-9, delta=0.85, mem=50, update_sigma=True, krylov_maxiter=400)
    assert out["converged"], out
    assert out["iterations"] < ref["iterations"]
    assert out["krylov_iterations"] > 0
    assert np.abs(gpu.flatten() - x_plain).max() <= 1e-7 * np.abs(x_plain).max()
    gpu.close()
