"""interpolate_solver! (src/interpolate.jl:1-191) on the GPU against a numpy restatement.

The source solver is iterated a few times (a symmetric state with structure in every block), then
interpolated onto solvers with other lattices (L = 4 -> 8, 3 -> 4 odd source, 8 -> 4 down-sampling)
and other frequency boxes (larger: zero rows; smaller: truncation).  Σ, K1/K2/K3 of the three
channels agree with the restatement to 1e-12 (relative to each block's max), including
symmetrize_solver! with the target's groups, and G of the target is the Dyson G of its Σ.
"""
import numpy as np
import pytest

from helpers import blocks, make_gpu

pytestmark = pytest.mark.gpu


def fourier_interpolate(yi, Lo, Li):
    """_fourier_interpolate! (src/interpolate.jl:1-27): momentum index column-major over (Li, Li)."""
    yiR = np.fft.fft2(yi.reshape(Li, Li, order="F")) / Li**2
    yoR = np.zeros((Lo, Lo), complex)
    h = Li // 2
    for R1 in range(-h, h + 1):
        for R2 in range(-h, h + 1):
            w = 1.0
            if Li % 2 == 0:
                if abs(R1) == h:
                    w /= 2
                if abs(R2) == h:
                    w /= 2
            yoR[R1 % Lo, R2 % Lo] += yiR[R1 % Li, R2 % Li] * w
    return (np.fft.ifft2(yoR) * Lo**2).reshape(-1, order="F")


def interpolate_state(xi, ci, co):
    """interpolate_vertex! per block and the clamped Σ evaluation of interpolate_solver!."""
    Li, Lo = ci["L"], co["L"]
    bi, bo = {b[0]: b for b in blocks(ci)}, {b[0]: b for b in blocks(co)}
    xo = np.zeros(bo["Sigma"][2], complex)
    for ch in "pta":
        for cls in ("K1", "K2", "K3"):
            _, si, ei = bi[f"{ch}.{cls}"]
            _, so, eo = bo[f"{ch}.{cls}"]
            if cls == "K1":
                fi, fo = [2 * ci["nK1"] - 1], [2 * co["nK1"] - 1]
                off_i, off_o = [ci["nK1"] - 1], [co["nK1"] - 1]
            elif cls == "K2":
                fi = [2 * ci["nK2"][0] - 1, 2 * ci["nK2"][1]]
                fo = [2 * co["nK2"][0] - 1, 2 * co["nK2"][1]]
                off_i, off_o = [ci["nK2"][0] - 1, ci["nK2"][1]], [co["nK2"][0] - 1, co["nK2"][1]]
            else:
                fi = [2 * ci["nK3"][0] - 1, 2 * ci["nK3"][1], 2 * ci["nK3"][1]]
                fo = [2 * co["nK3"][0] - 1, 2 * co["nK3"][1], 2 * co["nK3"][1]]
                off_i = [ci["nK3"][0] - 1, ci["nK3"][1], ci["nK3"][1]]
                off_o = [co["nK3"][0] - 1, co["nK3"][1], co["nK3"][1]]
            A = xi[si:ei].reshape(*fi, Li * Li, order="F")
            B = np.zeros((*fo, Lo * Lo), complex)
            for idx in np.ndindex(*fo):
                vals = [j - o for j, o in zip(idx, off_o)]
                src = [v + o for v, o in zip(vals, off_i)]
                if all(0 <= s_ < n for s_, n in zip(src, fi)):
                    B[idx] = fourier_interpolate(A[tuple(src)], Lo, Li)
            xo[so:eo] = B.reshape(-1, order="F")
    _, si, ei = bi["Sigma"]
    _, so, eo = bo["Sigma"]
    S = xi[si:ei].reshape(2 * ci["nG"], Li * Li, order="F")
    T = np.zeros((2 * co["nG"], Lo * Lo), complex)
    for j in range(2 * co["nG"]):
        n = min(max(j - co["nG"], -ci["nG"]), ci["nG"] - 1)
        T[j] = fourier_interpolate(S[n + ci["nG"]], Lo, Li)
    xo[so:eo] = T.reshape(-1, order="F")
    return xo


def _group_map(cfg, which, n):
    import ctypes
    from fdgasolver import _lib
    lib = _lib.load()
    c = _lib.fdga_config()
    c.nG, c.nK1 = cfg["nG"], cfg["nK1"]
    c.nK2[0], c.nK2[1] = cfg["nK2"]
    c.nK3[0], c.nK3[1] = cfg["nK3"]
    c.L = c.LG = cfg["L"]
    c.mPi_factor = cfg["mPi_factor"]
    c.local = 0
    c.T, c.U = cfg["T"], cfg["U"]
    c.nR[0], c.nR[1] = 1, 1
    m = np.zeros(n, np.uint32)
    assert lib.fdga_group_map(ctypes.byref(c), which, m.ctypes.data, n, None) == 0
    return m


def symmetrize_state(v, cfg):
    """symmetrize_solver! (src/ParquetSolver.jl:246-259) with the solver's init_sym_grp! groups: each
    element takes its class representative's value under the class operation (bit 0 sign, bit 1
    conjugation); the group maps index the (momentum-outermost) device layout."""
    v = v.copy()
    Nq = cfg["L"] ** 2
    shapes = {"K1": [2 * cfg["nK1"] - 1], "K2": [2 * cfg["nK2"][0] - 1, 2 * cfg["nK2"][1]],
              "K3": [2 * cfg["nK3"][0] - 1, 2 * cfg["nK3"][1], 2 * cfg["nK3"][1]]}
    for name, s, e in blocks(cfg):
        if name == "Sigma":
            fshape, which = [2 * cfg["nG"]], 0
        else:
            ch, cls = name.split(".")
            fshape = shapes[cls]
            which = {"K1": 1, "K2": 2 if ch == "p" else 3, "K3": 4 if ch == "p" else 5}[cls]
        A = v[s:e].reshape(*fshape, Nq, order="F")
        D = np.moveaxis(A, -1, 0).reshape(-1)  # device order: momentum, then the frequencies (last fastest)
        mp = _group_map(cfg, which, D.size)
        val = D[mp >> 2]
        val = np.where(mp & 2, np.conj(val), val)
        val = np.where(mp & 1, -val, val)
        v[s:e] = np.moveaxis(val.reshape(Nq, *fshape), 0, -1).reshape(-1, order="F")
    return v


BASE = dict(kind="hubbard", T=0.5, U=2.0, mu=0.3, t1=1.0, t2=-0.2, nG=8, nK1=8, nK2=(3, 3), nK3=(2, 3), mPi_factor=4)
CASES = [
    (dict(BASE, L=4), dict(BASE, L=8)),
    (dict(BASE, L=4), dict(BASE, L=8, nG=10, nK1=10, nK2=(4, 4), nK3=(3, 4))),
    (dict(BASE, L=4), dict(BASE, L=8, nG=6, nK1=6, nK2=(2, 2), nK3=(2, 2))),
    (dict(BASE, L=3), dict(BASE, L=4)),
    (dict(BASE, L=8), dict(BASE, L=4)),
]
IDS = ["4to8", "4to8-larger-boxes", "4to8-smaller-boxes", "3to4", "8to4"]


def _rel(a, b):
    s = np.abs(b).max()
    return np.abs(a - b).max() / (s if s > 0 else 1.0)


@pytest.mark.parametrize("ci,co", CASES, ids=IDS)
@pytest.mark.parametrize("sym", [False, True], ids=["trivial", "sym"])
def test_interpolate_solver(ci, co, sym):
    from fdgasolver.solver import interpolate_solver
    Si = make_gpu(ci, sym)
    x = Si.flatten()
    for _ in range(3):
        x = x + 0.5 * Si.fixed_point(x)
    Si.unflatten(x)
    So = make_gpu(co, sym)
    interpolate_solver(So, Si)
    got = So.flatten()
    ref = interpolate_state(x, ci, co)
    if sym:
        ref = symmetrize_state(ref, co)
    for name, s, e in blocks(co):
        assert _rel(got[s:e], ref[s:e]) < 1e-12, name
    # G of the target: Dyson of the interpolated Σ with the target's Gbare (iG = 1/(1/iGbare + iΣ))
    from fdgasolver.workloads import make_inputs
    Gb = make_inputs(co)[0].reshape(-1, order="F")
    _, s, e = blocks(co)[-1]
    G = 1.0 / (1.0 / Gb + got[s:e])
    assert _rel(So.get("G"), G) < 1e-13
    Si.close()
    So.close()


def test_interpolate_solver_refuses_in_place():
    """Source and target must be different solvers (the kernels read one and write the other)."""
    from fdgasolver import _lib
    from fdgasolver.solver import interpolate_solver
    S = make_gpu(dict(BASE, L=4), False)
    with pytest.raises(_lib.FdgaError) as e:
        interpolate_solver(S, S)
    assert e.value.code == 1  # FDGA_ERR_ARG
    S.close()
