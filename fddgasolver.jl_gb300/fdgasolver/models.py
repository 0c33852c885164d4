"""Model inputs (host side, numpy): bare Green functions stored as i*G.

siam_bare_Green     src/models/siam.jl:9-29
hubbard_bare_Green  src/models/hubbard.jl:8-44   (k index x + L*y, k = 2π(x, y)/L)
compute_hubbard_chemical_potential  src/dyson.jl:45-58
"""
import numpy as np


def fermionic_values(T: float, nG: int) -> np.ndarray:
    n = np.arange(-nG, nG)
    return (2 * n + 1) * np.pi * T


def siam_bare_Green(T: float, nG: int, *, Delta: float, e: float, D: float) -> np.ndarray:
    """iG0(ν) = 1/(ν + i e + Δ sign ν) for D = ∞, else 1/(ν + i e + 2Δ/π atan(D/ν)); shape (2nG,)."""
    nu = fermionic_values(T, nG)
    if np.isinf(D):
        return 1.0 / (nu + 1j * e + Delta * np.sign(nu))
    return 1.0 / (nu + 1j * e + 2 * Delta / np.pi * np.arctan(D / nu))


def hubbard_band(k1, k2, *, t1, t2=0.0, t3=0.0):
    ek = -2 * t1 * (np.cos(k1) + np.cos(k2))
    ek = ek + -4 * t2 * np.cos(k1) * np.cos(k2)
    ek = ek + -2 * t3 * (np.cos(2 * k1) + np.cos(2 * k2))
    return ek


def hubbard_bare_Green(T: float, nG: int, L: int, *, mu: float, t1: float, t2: float = 0.0, t3: float = 0.0):
    """iG0(ν, k) = i/(iν + μ - ε_k); column-major [ν, k] returned as shape (2nG, L*L)."""
    nu = fermionic_values(T, nG)
    idx = np.arange(L * L)
    k1 = 2 * np.pi * (idx % L) / L
    k2 = 2 * np.pi * (idx // L) / L
    ek = hubbard_band(k1, k2, t1=t1, t2=t2, t3=t3)
    return 1.0 / (1j * nu[:, None] + mu - ek[None, :]) * 1j


def compute_occupation(G: np.ndarray, T: float) -> float:
    """n = 1/2 + T Im ΣG / Nk (src/dyson.jl:33-41); G of shape (2nG,) or (2nG, Nk)."""
    G = np.asarray(G)
    nk = 1 if G.ndim == 1 else G.shape[1]
    return 0.5 + np.imag(G.sum()) * T / nk


def compute_hubbard_chemical_potential(occ_target: float, Sigma: np.ndarray, T: float, nG: int, L: int, *, t1: float,
                                       t2: float = 0.0, t3: float = 0.0) -> float:
    """μ with compute_occupation(Dyson(Σ, Gbare(μ))) = occ_target, bracketed in [-4|t1|, 4|t1|]
    (src/dyson.jl:45-58; the reference uses Roots.find_zero on the same bracket, here Brent's
    method to full double precision).  Σ and G are stored as i*Σ, i*G like the solver inputs, so
    Dyson reads G = 1/(1/Gbare + Σ) (src/dyson.jl:5-31)."""
    from scipy.optimize import brentq

    def occ(mu):
        Gb = hubbard_bare_Green(T, nG, L, mu=mu, t1=t1, t2=t2, t3=t3)
        G = 1.0 / (1.0 / Gb + Sigma)
        return compute_occupation(G, T) - occ_target

    return brentq(occ, -4 * abs(t1), 4 * abs(t1), xtol=1e-15, rtol=4 * np.finfo(float).eps, maxiter=500)
