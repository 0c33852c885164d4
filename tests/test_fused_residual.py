"""fixed_point!(R, x, S) (src/solve.jl:119-157) on page-locked host buffers: fdga_residual then runs
as one graph whose host copies overlap the iteration (Σ first, the vertex part of R copied back
while the SDE runs).

The fused call returns the same R as the sequential copy-iterate-copy path (the same kernels on the
same data: agreement to 1e-14 per flatten block), agrees with the oracle's residual to 1e-10, and
leaves the state at Φ(x).  The cached graph follows changes of the buffers, the strategy and the
precision.
"""
import numpy as np
import pytest

from helpers import blockwise_rel_err, make_gpu, make_oracle

pytestmark = pytest.mark.gpu

LOCAL = dict(kind="siam", T=0.1, U=1.0, e=0.2, Delta=0.5, D=10.0, nG=16, nK1=16, nK2=(5, 4), nK3=(4, 4),
             mPi_factor=6)
NL4 = dict(kind="hubbard", T=0.5, U=2.0, mu=0.3, t1=1.0, t2=-0.2, L=4, nG=8, nK1=8, nK2=(3, 3), nK3=(2, 3),
           mPi_factor=4, refvertex_noise=0.05, seed=7)


def _state(gpu, seed):
    rng = np.random.default_rng(seed)
    x = gpu.flatten()
    return x + 0.05 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))


def _fused(gpu, xb, Rb, x, strategy):
    xb.array[:] = x
    gpu.fixed_point_ptr(xb.ptr, Rb.ptr, strategy)
    return Rb.array.copy()


@pytest.mark.parametrize("cfg", [LOCAL, NL4], ids=["local", "nl4"])
@pytest.mark.parametrize("sym", [False, True], ids=["trivial", "sym"])
def test_fused_residual_matches_sequential_and_oracle(cfg, sym):
    from fdgasolver.solver import PinnedBuffer
    gpu = make_gpu(cfg, sym)
    orc = make_oracle(cfg, sym)
    xb, Rb = PinnedBuffer(gpu.state_len), PinnedBuffer(gpu.state_len)
    xb2, Rb2 = PinnedBuffer(gpu.state_len), PinnedBuffer(gpu.state_len)
    try:
        for k, (strategy, precision) in enumerate([("fdPA", "fp64"), ("scPA", "fp64"), ("fdPA", "mixed"),
                                                   ("fdPA", "fp64")]):
            gpu.set_precision(precision)
            x = _state(gpu, 3 + k)
            gpu.set_option("fused_residual", 0)
            R_seq = gpu.fixed_point(x, strategy)
            gpu.set_option("fused_residual", 1)
            R = _fused(gpu, xb, Rb, x, strategy)
            assert blockwise_rel_err(cfg, R, R_seq) < 1e-14, (strategy, precision)
            # the state is Φ(x)
            assert blockwise_rel_err(cfg, gpu.flatten(), x + R_seq) < 1e-14
            if precision == "fp64":
                assert blockwise_rel_err(cfg, R, orc.residual(x, strategy)) < 1e-10
            # another pair of buffers (a new graph), then the first pair again
            R2 = _fused(gpu, xb2, Rb2, x, strategy)
            assert blockwise_rel_err(cfg, R2, R_seq) < 1e-14
            R3 = _fused(gpu, xb, Rb, x, strategy)
            assert blockwise_rel_err(cfg, R3, R_seq) < 1e-14
    finally:
        for b in (xb, Rb, xb2, Rb2):
            b.free()
        gpu.close()


def test_fused_residual_pageable_buffers_take_the_sequential_path():
    """numpy (pageable) arrays: the same residual through the copy-iterate-copy sequence."""
    gpu = make_gpu(NL4, True)
    x = _state(gpu, 11)
    R1 = gpu.fixed_point(x)
    gpu.set_option("fused_residual", 0)
    R0 = gpu.fixed_point(x)
    assert np.array_equal(R0, R1)
    gpu.close()
