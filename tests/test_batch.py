"""Batches of independent solvers (one graph launch iterates every member) and the K3 tile autotuner.

(1) One batch iteration leaves every member in exactly the state that its own iterate_solver!
    produces (same kernels, same order: bitwise equal), in FP64 and in mixed precision, for a
    batch that mixes local and nonlocal members of different sizes.
(2) The autotuner only changes which thread computes which output tile of the K3 GEMMs; each
    element's ω-sum keeps its order, so the FP64 map is bitwise unchanged.
"""
import numpy as np
import pytest

from helpers import make_gpu

MEMBERS = [
    dict(kind="siam", T=0.1, U=1.0, e=0.2, Delta=0.5, D=10.0, nG=16, nK1=16, nK2=(5, 4), nK3=(4, 4), mPi_factor=6),
    dict(kind="siam", T=0.2, U=2.0, e=0.0, Delta=0.7, D=float("inf"), nG=12, nK1=12, nK2=(6, 6), nK3=(3, 6),
         mPi_factor=6),
    dict(kind="hubbard", T=0.5, U=2.0, mu=0.3, t1=1.0, t2=-0.2, L=4, nG=8, nK1=8, nK2=(3, 3), nK3=(2, 3),
         mPi_factor=4, refvertex_noise=0.05, seed=7),
    dict(kind="siam", T=0.05, U=0.8, e=0.0, Delta=0.4, D=float("inf"), nG=20, nK1=20, nK2=(10, 10), nK3=(5, 10),
         mPi_factor=6),
]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_iteration_equals_individual(precision):
    from fdgasolver.solver import Batch
    rng = np.random.default_rng(3)
    A = [make_gpu(c, True) for c in MEMBERS]
    B = [make_gpu(c, True) for c in MEMBERS]
    for a, b in zip(A, B):
        x = a.flatten()
        x = x + 0.05 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
        a.unflatten(x)
        b.unflatten(x)
    batch = Batch(A)
    for _ in range(2):
        batch.iterate("fdPA", precision)
    batch.synchronize()
    for b in B:
        b.set_precision(precision)
        b.iterate_solver("fdPA")
        b.iterate_solver("fdPA")
    for a, b in zip(A, B):
        assert np.array_equal(a.flatten(), b.flatten())
    ms, kernels = batch.time(2, "fdPA", precision)
    assert ms > 0 and kernels >= len(MEMBERS)
    batch.close()


@pytest.mark.gpu
def test_autotune_keeps_fp64_map_bitwise():
    cfg = MEMBERS[3]
    rng = np.random.default_rng(5)
    a, b = make_gpu(cfg, True), make_gpu(cfg, True)
    x = a.flatten()
    x = x + 0.05 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
    y0 = a.fixed_point(x)
    tiles = b.autotune()
    assert all(t in (16, 24, 32, 116, 124, 132) for pair in tiles.values() for t in pair)
    y1 = b.fixed_point(x)
    assert np.array_equal(y0, y1)


def test_batch_rejects_bad_arguments():
    import ctypes
    from fdgasolver import _lib
    lib = _lib.load()
    out = ctypes.c_void_p()
    assert lib.fdga_batch_create(None, 0, ctypes.byref(out)) != 0
    assert lib.fdga_batch_iterate(None, 0, 0) != 0


@pytest.mark.gpu
def test_batch_rejects_a_handle_twice():
    """Each member's state is written by its own branch of the batch graph."""
    from fdgasolver import _lib
    from fdgasolver.solver import Batch
    a = make_gpu(MEMBERS[0], True)
    with pytest.raises(_lib.FdgaError) as e:
        Batch([a, a])
    assert e.value.code == 1  # FDGA_ERR_ARG
    a.close()
