"""Seeded synthetic workloads of the benchmark configurations (host-side input generation).

The reference names no dataset; these reproduce the configuration text: model, parameters, box
sizes (read as the reference constructor arguments) and, for the nonlocal plain-method case, a
seeded synthetic RefVertex.

siam_b10_nk3_16: SIAM, local fdPA, β=10, U=1, flat band Δ(iν) = -iΓ sign ν, Γ = 0.5 (D = ∞), e = 0,
         nK1=64, nK2=(32,32), nK3=(16,16), nG=64, mΠν_factor=6.
hubbard8x8_b5_nk3_8x12: Hubbard 8x8, nonlocal fdPA, t=1, t'=0, μ=0, U=2, β=5, nK1=32, nK2=(16,16), nK3=(8,12),
         nG=32, mΠν_factor=32; F0 = RefVertex(U) with corrections on the K3 box drawn as
         complex Gaussian noise σ = 0.05 U, symmetrised ν<->ν', scaled 1/sqrt((1+|ν|)(1+|ν'|)).
hubbard16x16_n09_nk3_20x40: Hubbard 16x16, nonlocal fdPA, t=1, t'=-0.2, U=3, β=10, nK1=80, nK2=(40,40), nK3=(20,40), nG=80,
         mΠν_factor=32; μ tuned once on Gbare (Σ = 0) to density n = 0.9 (per-spin occupation 0.45).
siam_batch48: 48 SIAM instances, local fdPA, flat band (D = ∞), e = 0, seeded U ~ U[0.5, 3], β ∈ {5, 10, 20, 40},
         Γ ~ U[0.3, 1]; boxes scale with β: nK3 = (nν/2, nν) with nν = 16, 32, 48, 64 for β = 5, 10, 20,
         40, nK2 = (nν, nν), nK1 = nG = 2nν, mΠν_factor = 6 (batch_instances).
hubbard24x24_b8_nk3_24x48: Hubbard 24x24, nonlocal fdPA, t=1, t'=0, μ=0, U=2.5, β=8, nK1=96, nK2=(48,48), nK3=(24,48), nG=96,
         mΠν_factor=32.
"""
import numpy as np

from .models import fermionic_values
from .solver import RefVertex

CONFIGS = {
    "siam_b10_nk3_16": dict(kind="siam", T=0.1, U=1.0, e=0.0, Delta=0.5, D=float("inf"), nG=64, nK1=64, nK2=(32, 32),
                    nK3=(16, 16), mPi_factor=6),
    "hubbard8x8_b5_nk3_8x12": dict(kind="hubbard", T=0.2, U=2.0, mu=0.0, t1=1.0, t2=0.0, L=8, nG=32, nK1=32, nK2=(16, 16),
                    nK3=(8, 12), mPi_factor=32, refvertex_noise=0.05, seed=20261203),
    "hubbard16x16_n09_nk3_20x40": dict(kind="hubbard", T=0.1, U=3.0, mu=None, filling=0.9, t1=1.0, t2=-0.2, L=16, nG=80, nK1=80,
                    nK2=(40, 40), nK3=(20, 40), mPi_factor=32),
    # the 16x16 workload's frequency boxes on a 4x4 lattice: the size the K3 tensor-core kernel is profiled at
    "hubbard4x4_n09_nk3_20x40": dict(kind="hubbard", T=0.1, U=3.0, mu=None, filling=0.9, t1=1.0, t2=-0.2, L=4, nG=80, nK1=80,
                     nK2=(40, 40), nK3=(20, 40), mPi_factor=32),
    "hubbard24x24_b8_nk3_24x48": dict(kind="hubbard", T=0.125, U=2.5, mu=0.0, t1=1.0, t2=0.0, L=24, nG=96, nK1=96, nK2=(48, 48),
                    nK3=(24, 48), mPi_factor=32),
}


def synthetic_refvertex(T, U, nK3, sigma, seed):
    """Seeded RefVertex corrections on the K3 box (see module docstring)."""
    rng = np.random.default_rng(seed)
    nO, nn = nK3
    NO, Nn = 2 * nO - 1, 2 * nn
    nu = np.abs(fermionic_values(T, nn))
    w = 1.0 / np.sqrt((1 + nu[:, None]) * (1 + nu[None, :]))
    out = []
    for _ in range(4):
        z = (rng.standard_normal((NO, Nn, Nn)) + 1j * rng.standard_normal((NO, Nn, Nn))) * (sigma * U / np.sqrt(2))
        z = 0.5 * (z + np.transpose(z, (0, 2, 1)))
        out.append(z * w[None, :, :])
    return RefVertex(T, U, *out)


def make_inputs(cfg):
    """(Gbare, G0, Σ0, RefVertex) of a workload dict: kind 'siam' (local) or 'hubbard' (nonlocal)."""
    from .models import hubbard_bare_Green, siam_bare_Green
    T, U = cfg["T"], cfg["U"]
    if cfg["kind"] == "siam":
        Gb = siam_bare_Green(T, cfg["nG"], Delta=cfg["Delta"], e=cfg["e"], D=cfg["D"])
    else:
        mu = cfg["mu"]
        if mu is None:  # tuned once on Gbare (Σ = 0) to the target filling
            from .models import compute_hubbard_chemical_potential
            # compute_occupation is per spin (1/2 at half filling): density n <-> occupation n/2
            mu = compute_hubbard_chemical_potential(cfg["filling"] / 2, np.zeros((2 * cfg["nG"], cfg["L"] ** 2), complex),
                                                    T, cfg["nG"], cfg["L"], t1=cfg["t1"], t2=cfg.get("t2", 0.0))
        Gb = hubbard_bare_Green(T, cfg["nG"], cfg["L"], mu=mu, t1=cfg["t1"], t2=cfg.get("t2", 0.0))
    G0 = cfg.get("G0")
    S0 = cfg.get("Sigma0")
    G0 = np.zeros_like(Gb) if G0 is None else G0
    S0 = np.zeros_like(Gb) if S0 is None else S0
    if cfg.get("refvertex_noise"):
        rv = synthetic_refvertex(T, U, cfg.get("nR", cfg["nK3"]), cfg["refvertex_noise"], cfg.get("seed", 1))
    else:
        rv = RefVertex(T, U)
    return Gb, G0, S0, rv


def make_solver(cfg, sym=True):
    """libfdga solver of a workload dict, with init_sym_grp! applied when sym."""
    from .solver import NL_ParquetSolver, ParquetSolver
    Gb, G0, S0, rv = make_inputs(cfg)
    if cfg["kind"] == "siam":
        S = ParquetSolver(cfg["nK1"], cfg["nK2"], cfg["nK3"], Gb, G0, S0, rv, mPi_factor=cfg["mPi_factor"])
    else:
        S = NL_ParquetSolver(cfg["nK1"], cfg["nK2"], cfg["nK3"], cfg["L"], Gb, G0, S0, rv,
                             mPi_factor=cfg["mPi_factor"])
    if sym:
        S.init_sym_grp()
    return S


def batch_instances(n=48, seed=20261204):
    """The config-4 instance list (see the module docstring)."""
    rng = np.random.default_rng(seed)
    nnu_of = {5: 16, 10: 32, 20: 48, 40: 64}
    out = []
    for _ in range(n):
        U = float(rng.uniform(0.5, 3.0))
        beta = int(rng.choice([5, 10, 20, 40]))
        gamma = float(rng.uniform(0.3, 1.0))
        nnu = nnu_of[beta]
        out.append(dict(kind="siam", T=1.0 / beta, U=U, e=0.0, Delta=gamma, D=float("inf"), nG=2 * nnu, nK1=2 * nnu,
                        nK2=(nnu, nnu), nK3=(nnu // 2, nnu), mPi_factor=6))
    return out
