"""Model inputs (host side, numpy): bare Green functions stored as i*G.

siam_bare_Green     src/models/siam.jl:9-29
hubbard_bare_Green  src/models/hubbard.jl:8-44   (k index x + L*y, k = 2π(x, y)/L)
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
