"""The mixed map's K3 contractions on the tensor cores (tcgen05, TF32 hi/lo split, FP32 accumulation).

For boxes with 2·Nν3 ≤ 256 and Nν3 a multiple of 8, FDGA_MIXED runs the two K3 GEMMs as tcgen05
MMAs.  One map application must agree with the FP64 map to FP32 accuracy (1e-5 relative per
flatten block), and with the FP32 CUDA-core form of the same contraction to 1e-5; both fdPA (L_K3
and K3 GEMMs) and scPA (K3 GEMM only) run.
"""
import numpy as np
import pytest

from helpers import blockwise_rel_err, make_gpu

LOCAL32 = dict(kind="siam", T=0.1, U=1.0, e=0.2, Delta=0.5, D=10.0, nG=24, nK1=24, nK2=(8, 16), nK3=(4, 16),
               mPi_factor=4)
NL32 = dict(kind="hubbard", T=0.5, U=2.0, mu=0.3, t1=1.0, t2=-0.2, L=4, nG=16, nK1=16, nK2=(4, 16), nK3=(2, 16),
            mPi_factor=2, refvertex_noise=0.05, seed=7)
LOCAL80 = dict(kind="siam", T=0.05, U=1.5, e=0.0, Delta=0.6, D=float("inf"), nG=40, nK1=40, nK2=(8, 40),
               nK3=(3, 40), mPi_factor=3)


@pytest.mark.gpu
@pytest.mark.parametrize("strategy", ["fdPA", "scPA"])
@pytest.mark.parametrize("cfg", [LOCAL32, NL32, LOCAL80], ids=["local32", "nl32", "local80"])
def test_tensor_core_k3_matches_fp64_and_cuda_cores(cfg, strategy):
    rng = np.random.default_rng(9)
    gpu = make_gpu(cfg, True)
    x = gpu.flatten()
    x = x + 0.05 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
    y = gpu.fixed_point(x, strategy) + x  # nonzero FL and Σ for the compared application
    y64 = gpu.fixed_point(y, strategy) + y
    gpu.set_precision("mixed")
    gpu.set_option("k3_tensor_cores", 1)
    y_tc = gpu.fixed_point(y, strategy) + y
    gpu.set_option("k3_tensor_cores", 0)
    y_cc = gpu.fixed_point(y, strategy) + y
    gpu.set_precision("fp64")
    assert blockwise_rel_err(cfg, y_tc, y64) < 1e-5
    assert blockwise_rel_err(cfg, y_cc, y64) < 1e-5
    assert blockwise_rel_err(cfg, y_tc, y_cc) < 1e-5
    assert blockwise_rel_err(cfg, y_tc, y_cc) > 0.0  # two different contraction paths ran
