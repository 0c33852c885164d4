"""fdga_bubble_noalloc: the bubble entry point for callers that cannot call cudaMalloc.

A host whose pool allocator owns the device memory (Julia CUDA.jl, PyTorch) passes its own device
buffers for G and the two bubbles; the library's only work array, G(R), is a fixed file-scope
device buffer instead of an allocation.  These tests call the entry point through the C ABI with
caller-owned device buffers (torch tensors) and compare it with the bubbles that the existing
entry point fdga_finalize computes for G0, to the 1e-10 tolerance of the other parity tests, on
two calls in a row with different problem shapes (the second call reuses the buffer the first
one wrote).
"""
import ctypes

import numpy as np
import pytest

TOL = 1e-10


def _config(local, nG, nK1, L, f, T):
    from fdgasolver import _lib
    c = _lib.fdga_config()
    c.nG, c.nK1 = nG, nK1
    c.nK2[0], c.nK2[1] = 2, 2
    c.nK3[0], c.nK3[1] = 1, 2
    c.L = c.LG = L
    c.mPi_factor = f
    c.local = int(local)
    c.T, c.U = T, 1.0
    c.nR[0], c.nR[1] = 1, 1
    return c


def _reference_bubbles(local, G, nK1, L, f, T):
    """Π0 of G0 = G through the existing entry point (fdga_create + fdga_finalize)."""
    import fdgasolver as F
    z = np.zeros_like(G)
    rv = F.RefVertex(T, 1.0)
    if local:
        S = F.ParquetSolver(nK1, (2, 2), (1, 2), G, G, z, rv, mPi_factor=f)
    else:
        S = F.NL_ParquetSolver(nK1, (2, 2), (1, 2), L, G, G, z, rv, mPi_factor=f)
    pp, ph = S.get("Pi0pp"), S.get("Pi0ph")
    S.close()
    return pp, ph


def _noalloc(lib, cfg, G):
    import torch
    g = torch.from_numpy(np.ascontiguousarray(G.reshape(-1, order="F")).view(np.float64).copy()).cuda()
    n = (2 * cfg.nK1 - 1) * (2 * cfg.nK1 * cfg.mPi_factor) * cfg.L * cfg.L
    pp = torch.full((2 * n,), float("nan"), dtype=torch.float64, device="cuda")
    ph = torch.full((2 * n,), float("nan"), dtype=torch.float64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.fdga_bubble_noalloc(ctypes.byref(cfg), ctypes.c_void_p(g.data_ptr()), ctypes.c_void_p(pp.data_ptr()),
                                 ctypes.c_void_p(ph.data_ptr()), stream)
    torch.cuda.synchronize()
    assert rc == 0, lib.fdga_last_error(None)
    return pp.cpu().numpy().view(np.complex128), ph.cpu().numpy().view(np.complex128)


@pytest.mark.gpu
def test_noalloc_bubble_matches_finalize_two_calls():
    import fdgasolver as F
    from fdgasolver import _lib
    lib = _lib.load()
    cases = [
        # nonlocal 4x4 lattice, t' != 0, bubble mesh with 1/ν tails
        dict(local=False, nG=8, nK1=8, L=4, f=4, T=0.5,
             G=lambda: F.hubbard_bare_Green(0.5, 8, 4, mu=0.3, t1=1.0, t2=-0.2)),
        # local solver (L = 1): a different shape reusing the same work array
        dict(local=True, nG=16, nK1=12, L=1, f=3, T=0.1,
             G=lambda: F.siam_bare_Green(0.1, 16, Delta=0.5, e=0.2, D=10.0)),
    ]
    for case in cases:
        G = case["G"]()
        cfg = _config(case["local"], case["nG"], case["nK1"], case["L"], case["f"], case["T"])
        pp_ref, ph_ref = _reference_bubbles(case["local"], G, case["nK1"], case["L"], case["f"], case["T"])
        pp, ph = _noalloc(lib, cfg, G)
        assert np.abs(pp - pp_ref).max() <= TOL * np.abs(pp_ref).max()
        assert np.abs(ph - ph_ref).max() <= TOL * np.abs(ph_ref).max()


def _oracle_bubbles(local, G, nK1, L, f, T):
    """Π0 of G0 = G from the CPU oracle (the restatement of src/nonlocal/bubble.jl / src/bubble.jl)."""
    from oracle import oracle as O
    orc = O.OracleSolver(nG=G.shape[0] // 2, nK1=nK1, nK2=(2, 2), nK3=(1, 2), T=T, U=1.0, L=L, local=bool(local),
                         mPi_factor=f)
    orc.set("Gbare", G)
    orc.set("G0", G)
    orc.finalize()
    return orc.get("Pi0pp"), orc.get("Pi0ph")


@pytest.mark.gpu
def test_noalloc_bubble_matches_oracle():
    """The same two calls against the oracle's bubbles directly."""
    import fdgasolver as F
    from fdgasolver import _lib
    lib = _lib.load()
    cases = [
        dict(local=False, nG=8, nK1=8, L=4, f=4, T=0.5,
             G=lambda: F.hubbard_bare_Green(0.5, 8, 4, mu=0.3, t1=1.0, t2=-0.2)),
        dict(local=True, nG=16, nK1=12, L=1, f=3, T=0.1,
             G=lambda: F.siam_bare_Green(0.1, 16, Delta=0.5, e=0.2, D=10.0)),
    ]
    for case in cases:
        G = case["G"]()
        cfg = _config(case["local"], case["nG"], case["nK1"], case["L"], case["f"], case["T"])
        pp_ref, ph_ref = _oracle_bubbles(case["local"], G, case["nK1"], case["L"], case["f"], case["T"])
        pp, ph = _noalloc(lib, cfg, G)
        assert np.abs(pp - pp_ref).max() <= TOL * np.abs(pp_ref).max()
        assert np.abs(ph - ph_ref).max() <= TOL * np.abs(ph_ref).max()


def _check_rejections():
    """Both limits are checked on the host before any device work, so host buffers are safe here."""
    from fdgasolver import _lib
    lib = _lib.load()
    buf = (ctypes.c_double * 2)()
    cfg = _config(False, 2048, 8, 8, 4, 0.5)  # 2nG*L*L = 262144 > 131072
    rc = lib.fdga_bubble_noalloc(ctypes.byref(cfg), buf, buf, buf, None)
    assert rc == 1  # FDGA_ERR_ARG
    assert b"exceeds the work-array maximum" in lib.fdga_last_error(None)
    cfg = _config(False, 2, 8, 57, 4, 0.5)  # 2nG*L*L = 12996 fits, but L = 57 > 56
    rc = lib.fdga_bubble_noalloc(ctypes.byref(cfg), buf, buf, buf, None)
    assert rc == 1
    assert b"exceeds the maximum lattice size 56" in lib.fdga_last_error(None)


def test_noalloc_rejects_sizes_beyond_the_work_array():
    """Size validation on a host without a GPU (the library loads without one)."""
    _check_rejections()


@pytest.mark.gpu
def test_noalloc_rejects_sizes_beyond_the_work_array_gpu():
    """The same rejections in the GPU process that uses the entry point."""
    _check_rejections()
