"""fdDΓA from a Vertex-valued reference vertex on the GPU: ParquetSolver{Q, VT, RefVT} with RefVT a
Vertex (src/ParquetSolver.jl:5-157), the construction ParquetSolver(nK1, nK2, nK3, Gbare, S0.G, S0.Σ,
S0.F) of test/test_siam_fdPA.jl:79-84, and its nonlocal counterpart (test/test_nonlocal_fdPA.jl:50-54).

The reference vertex F0 = RefVertex(U) + γ0p + γ0t + γ0a has boxes of its own, larger or smaller than
the solver's.  It enters every vertex evaluation (the caches F0p/F0a/F0t, the factor F0(Ω, ω̃, ∞) of
the K1/K2 BSEs, the reduced vertex difference of the K2 BSE) and the SDE recursion through F.F0
(src/SDE.jl:35-48: its Vertex level without U² and Hartree, its RefVertex level divided by 3).

Tolerances: one application of the FP64 map agrees with the oracle's restatement to 1e-10 relative
per flatten block; the mixed map to 1e-5; the tangent map agrees with central differences of the
GPU's FP64 map to 1e-7.  The reference's own golden value Σ(πT) of the fdPA solve from a Vertex
reference (test/test_siam_fdPA.jl:179) is reproduced to 2e-4 (the solve stops at the reference's
default tolerance 1e-4; the golden value matches the fdPA SDE with the reference system's Hartree
term subtracted once, option "fdpa_single_hartree").
"""
import json
import os

import numpy as np
import pytest

from helpers import blockwise_rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-10

LOCAL = dict(local=True, T=0.1, U=1.0, nG=16, nK1=16, nK2=(5, 4), nK3=(4, 4), mPi_factor=6,
             model=dict(e=0.2, Delta=0.5, D=10.0))
NL4 = dict(local=False, T=0.5, U=2.0, L=4, nG=8, nK1=8, nK2=(3, 3), nK3=(2, 3), mPi_factor=4,
           model=dict(mu=0.3, t1=1.0, t2=-0.2))
NL3 = dict(local=False, T=0.4, U=1.5, L=3, nG=6, nK1=6, nK2=(3, 2), nK3=(2, 2), mPi_factor=3,
           model=dict(mu=0.1, t1=1.0))
# boxes of the reference vertex F0: larger than the solver's, and smaller
F0_BOX = {"local": [(20, (6, 6), (5, 5)), (12, (4, 3), (3, 3))],
          "nl4": [(10, (4, 4), (3, 3)), (6, (2, 2), (2, 2))],
          "nl3odd": [(8, (4, 3), (3, 2))]}
CASES = [(LOCAL, "local", b) for b in F0_BOX["local"]] + [(NL4, "nl4", b) for b in F0_BOX["nl4"]] + \
        [(NL3, "nl3odd", b) for b in F0_BOX["nl3odd"]]
CASE_IDS = [f"{n}-F0K1_{b[0]}" for _, n, b in CASES]


def _oracle_reference_solver(cfg, box, iters=8):
    """The reference system S0: a scPA solver with F0's boxes, iterated a few times from the PA start
    (its F has the structure of a solved vertex; convergence is not needed for parity)."""
    from oracle import oracle as O
    T, U = cfg["T"], cfg["U"]
    kw = dict(nG=cfg["nG"], nK1=box[0], nK2=box[1], nK3=box[2], T=T, U=U, mPi_factor=cfg["mPi_factor"])
    if cfg["local"]:
        s = O.OracleSolver(local=True, **kw)
        s.siam_bare_green("Gbare", **cfg["model"])
    else:
        s = O.OracleSolver(local=False, L=cfg["L"], **kw)
        s.hubbard_bare_green("Gbare", **cfg["model"])
    s.finalize()
    s.init_sym_grp()
    x = s.flatten()
    for _ in range(iters):
        x = x + 0.5 * s.residual(x, "scPA")
    s.unflatten(x)
    s.iterate("scPA")
    return s


def _target_gbare(cfg):
    """The target system's bare G: a shifted model (as the reference's fdPA tests do)."""
    import fdgasolver as F
    m = dict(cfg["model"])
    if cfg["local"]:
        return F.siam_bare_Green(cfg["T"], cfg["nG"], Delta=m["Delta"] * 1.2, e=m["e"] + 0.3, D=m["D"])
    return F.hubbard_bare_Green(cfg["T"], cfg["nG"], cfg["L"], mu=m["mu"] + 0.2, t1=m["t1"], t2=m.get("t2", 0.0) - 0.1)


def _pair(cfg, box, sym):
    """The same fdDΓA problem on the oracle and on the GPU: G0 = S0.G, Σ0 = S0.Σ, F0 = S0.F."""
    import fdgasolver as F
    from oracle import oracle as O
    s0 = _oracle_reference_solver(cfg, box)
    flat0 = s0.flatten()
    nS = 2 * cfg["nG"] * (1 if cfg["local"] else cfg["L"] ** 2)
    f0_flat = flat0[:-nS]
    G0, Sig0 = s0.get("G"), s0.get("Sigma")
    Gb = _target_gbare(cfg)
    T, U = cfg["T"], cfg["U"]
    kw = dict(nG=cfg["nG"], nK1=cfg["nK1"], nK2=cfg["nK2"], nK3=cfg["nK3"], T=T, U=U, mPi_factor=cfg["mPi_factor"],
              f0_vertex_box=box)
    orc = O.OracleSolver(local=True, **kw) if cfg["local"] else O.OracleSolver(local=False, L=cfg["L"], **kw)
    orc.set("Gbare", Gb)
    orc.set("G0", G0)
    orc.set("Sigma0", Sig0)
    for ch in "pta":
        for k in ("K1", "K2", "K3"):
            orc.set(f"F0.{ch}.{k}", s0.get(f"F.{ch}.{k}"))
    orc.finalize()
    L = 1 if cfg["local"] else cfg["L"]
    F0 = F.Vertex(F.RefVertex(T, U), box[0], box[1], box[2], f0_flat, L=L)
    if cfg["local"]:
        gpu = F.ParquetSolver(cfg["nK1"], cfg["nK2"], cfg["nK3"], Gb, G0, Sig0, F0, mPi_factor=cfg["mPi_factor"])
    else:
        gpu = F.NL_ParquetSolver(cfg["nK1"], cfg["nK2"], cfg["nK3"], L, Gb, G0, Sig0, F0,
                                 mPi_factor=cfg["mPi_factor"])
    if sym:
        orc.init_sym_grp()
        gpu.init_sym_grp()
    return orc, gpu


def _bcfg(cfg):
    """Block layout of flatten(S) for helpers.blockwise_rel_err."""
    return dict(kind="siam" if cfg["local"] else "hubbard", L=cfg.get("L", 1), nG=cfg["nG"], nK1=cfg["nK1"],
                nK2=cfg["nK2"], nK3=cfg["nK3"])


def _state(x, rng, scale=0.02):
    return x + scale * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))


@pytest.mark.parametrize("cfg,name,box", CASES, ids=CASE_IDS)
@pytest.mark.parametrize("sym", [False, True], ids=["trivial", "sym"])
@pytest.mark.parametrize("strategy", ["fdPA", "scPA"])
def test_vertex_reference_map_parity(cfg, name, box, sym, strategy):
    rng = np.random.default_rng(31)
    orc, gpu = _pair(cfg, box, sym)
    x = _state(orc.flatten(), rng)
    for _ in range(2):  # the second application has a nonzero FL and Σ
        y_orc = orc.residual(x, strategy) + x
        y_gpu = gpu.fixed_point(x, strategy) + x
        assert blockwise_rel_err(_bcfg(cfg), y_gpu, y_orc) < TOL
        x = _state(y_orc, rng, 0.005)
    gpu.close()


@pytest.mark.parametrize("cfg,name,box,strategy",
                         [(LOCAL, "local", F0_BOX["local"][0], "fdPA_new"),
                          (LOCAL, "local", F0_BOX["local"][1], "scPA_new"),
                          (NL4, "nl4", F0_BOX["nl4"][0], "fdPA_1loop")],
                         ids=["local-fdPA_new", "local-scPA_new", "nl4-fdPA_1loop"])
def test_vertex_reference_strategy_variants(cfg, name, box, strategy):
    rng = np.random.default_rng(32)
    orc, gpu = _pair(cfg, box, True)
    x = _state(orc.flatten(), rng)
    for _ in range(2):
        y_orc = orc.residual(x, strategy) + x
        y_gpu = gpu.fixed_point(x, strategy) + x
        assert blockwise_rel_err(_bcfg(cfg), y_gpu, y_orc) < TOL
        x = _state(y_orc, rng, 0.005)
    gpu.close()


@pytest.mark.parametrize("cfg,name,box", [CASES[0], CASES[2]], ids=["local", "nl4"])
def test_vertex_reference_mixed_map(cfg, name, box):
    """The mixed map (FP32 vertex mirrors, including F0's channels) against the oracle."""
    rng = np.random.default_rng(33)
    orc, gpu = _pair(cfg, box, True)
    x = _state(orc.flatten(), rng)
    y_orc = orc.residual(x, "fdPA") + x
    gpu.set_precision("mixed")
    y32 = gpu.fixed_point(x, "fdPA") + x
    err = blockwise_rel_err(_bcfg(cfg), y32, y_orc)
    assert 0 < err < 1e-5
    gpu.close()


@pytest.mark.parametrize("cfg,name,box", [CASES[0], CASES[2]], ids=["local", "nl4"])
def test_vertex_reference_tangent(cfg, name, box):
    """fdga_frule with a Vertex F0 (constant) against central differences of the GPU's FP64 map."""
    rng = np.random.default_rng(34)
    orc, gpu = _pair(cfg, box, True)
    x = _state(orc.flatten(), rng)
    v = rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size)
    h = 1e-4

    def phi(z):
        return gpu.fixed_point(z, "fdPA") + z

    d1 = (phi(x + h * v) - phi(x - h * v)) / (2 * h)
    d2 = (phi(x + 0.5 * h * v) - phi(x - 0.5 * h * v)) / h
    ref = (4 * d2 - d1) / 3  # Richardson: O(h⁴)
    gpu.unflatten(x)
    y, jv = gpu.frule(v, "fdPA")
    assert blockwise_rel_err(_bcfg(cfg), jv, ref) < 1e-7
    assert blockwise_rel_err(_bcfg(cfg), y, phi(x)) < 1e-13
    with pytest.raises(Exception):
        gpu.rrule(v, "fdPA")  # the adjoint map covers a RefVertex reference only
    gpu.close()


def test_siam_fdpa_golden_from_vertex_reference():
    """test/test_siam_fdPA.jl:79-84,179 on the GPU: S0 = scPA SIAM (nmax 12, e = -0.3, Δ = π/3, D = 10),
    then fdPA to the target (nmax 8, e = 0.5, Δ = π/5, D = 20) with F0 = S0.F; Σ(πT) against the golden
    value.  Bubble mesh factor 1, as the reference's golden values were generated."""
    import fdgasolver as F
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_golden.json")))
    g = gold["siam_fdPA_sigma_piT"]
    T, U, nG, nK1 = 0.1, 1.0, 96, 96
    S0 = F.parquet_solver_siam_parquet_approximation(nG, nK1, (12, 12), (12, 12), e=-0.3, Delta=np.pi / 3, D=10.0,
                                                     T=T, U=U, mPi_factor=1)
    S0.init_sym_grp()
    assert S0.solve("scPA", maxiter=100, tol=1e-4)["converged"]
    Gbare = F.siam_bare_Green(T, nG, Delta=np.pi / 5, e=0.5, D=20.0)
    S = F.ParquetSolver(64, (8, 8), (8, 8), Gbare, S0.get("G"), S0.get("Sigma"), S0.F, mPi_factor=1)
    S.init_sym_grp()
    S.set_option("fdpa_single_hartree", 1)
    assert S.solve("fdPA", maxiter=100, tol=1e-4)["converged"]
    v = S.get("Sigma")[nG]
    gv = complex(*g["value"])
    assert abs(v - gv) / abs(gv) < 2e-4
    S.close()
    S0.close()


def test_vertex_reference_rejections():
    """A Vertex F0 upload needs f0_vertex = 1 and its exact size."""
    import ctypes

    import fdgasolver as F
    from fdgasolver import _lib
    cfg = LOCAL
    S = F.parquet_solver_siam_parquet_approximation(cfg["nG"], cfg["nK1"], cfg["nK2"], cfg["nK3"], T=cfg["T"],
                                                    U=cfg["U"], **cfg["model"])
    buf = np.zeros(8, dtype=np.complex128)
    rc = S._lib.fdga_set_input(S._h, _lib.IN_F0_VERTEX, buf.ctypes.data, buf.size)
    assert rc == 1 and b"RefVertex" in S._lib.fdga_last_error(S._h)
    S.close()
    with pytest.raises(ValueError):
        F.Vertex(F.RefVertex(0.1, 1.0), 4, (2, 2), (1, 2), np.zeros(5, complex))
    del ctypes
