"""The mixed map's K3 contractions on the tensor cores (tcgen05, TF32 hi/lo split, FP32 accumulation).

For boxes with 2·Nν3 ≤ 256 and Nν3 a multiple of 8, FDGA_MIXED runs the two K3 GEMMs as tcgen05
MMAs: by default in the TMA-fed warp-specialised kernel (fdga_k3_tma.cu), with option k3_tma = 0 in
the staging kernel (fdga_k3_tc.cu), with k3_tensor_cores = 0 as FP32 CUDA-core GEMMs.  One map
application must agree with the FP64 map to FP32 accuracy (1e-5 relative per flatten block) on every
path; the two tensor-core kernels issue the same MMAs on the same operands and agree to 1e-6.  The
tangent map (mode 2 of the contraction: dA·M + A·dM over the concatenated inner index) is compared
the same way.  Cases: Nν3 = 32 (local and 4x4 lattice), 80, 96 and 128 (where the tangent's operand
stages exceed the shared memory and the staging kernel takes mode 2).
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
LOCAL96 = dict(kind="siam", T=0.05, U=1.2, e=0.1, Delta=0.6, D=10.0, nG=48, nK1=48, nK2=(6, 48), nK3=(3, 48),
               mPi_factor=2)
LOCAL128 = dict(kind="siam", T=0.04, U=1.0, e=0.0, Delta=0.5, D=float("inf"), nG=64, nK1=64, nK2=(4, 64),
                nK3=(2, 64), mPi_factor=2)
CASES = [LOCAL32, NL32, LOCAL80, LOCAL96, LOCAL128]
IDS = ["local32", "nl32", "local80", "local96", "local128"]


def _state(gpu, rng, strategy):
    x = gpu.flatten()
    x = x + 0.05 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
    return gpu.fixed_point(x, strategy) + x  # nonzero FL and Σ for the compared application


@pytest.mark.gpu
@pytest.mark.parametrize("strategy", ["fdPA", "scPA"])
@pytest.mark.parametrize("cfg", CASES, ids=IDS)
def test_tensor_core_k3_matches_fp64_and_cuda_cores(cfg, strategy):
    rng = np.random.default_rng(9)
    gpu = make_gpu(cfg, True)
    y = _state(gpu, rng, strategy)
    y64 = gpu.fixed_point(y, strategy) + y
    gpu.set_precision("mixed")
    gpu.set_option("k3_tensor_cores", 1)
    gpu.set_option("k3_tma", 1)
    y_tma = gpu.fixed_point(y, strategy) + y
    gpu.set_option("k3_tma", 0)
    y_tc = gpu.fixed_point(y, strategy) + y
    gpu.set_option("k3_tensor_cores", 0)
    y_cc = gpu.fixed_point(y, strategy) + y
    gpu.set_precision("fp64")
    assert blockwise_rel_err(cfg, y_tma, y64) < 1e-5
    assert blockwise_rel_err(cfg, y_tc, y64) < 1e-5
    assert blockwise_rel_err(cfg, y_cc, y64) < 1e-5
    assert blockwise_rel_err(cfg, y_tma, y_tc) < 1e-6
    assert blockwise_rel_err(cfg, y_tc, y_cc) > 0.0  # the tensor-core and CUDA-core paths both ran
    gpu.close()


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", CASES, ids=IDS)
def test_tensor_core_k3_tangent(cfg):
    rng = np.random.default_rng(10)
    gpu = make_gpu(cfg, True)
    y = _state(gpu, rng, "fdPA")
    v = rng.standard_normal(y.size) + 1j * rng.standard_normal(y.size)
    gpu.unflatten(y)
    _, j64 = gpu.frule(v)
    gpu.set_precision("mixed")
    gpu.set_option("k3_tma", 1)
    gpu.unflatten(y)
    _, j_tma = gpu.frule(v)
    gpu.set_option("k3_tma", 0)
    gpu.unflatten(y)
    _, j_tc = gpu.frule(v)
    assert blockwise_rel_err(cfg, j_tma, j64) < 2e-5
    assert blockwise_rel_err(cfg, j_tma, j_tc) < 1e-6
    gpu.close()


@pytest.mark.gpu
def test_fp64_to_fp32_rounding_matches_hardware():
    """The integer-path FP64 -> FP32 rounding used by every narrowing of the mixed map (d2f_rn)
    gives the hardware conversion's bits on 2^26 hashed inputs (ties of both parities, values next
    to ties, the FP32 range edges, zeros, subnormals, infinities, NaNs)."""
    from fdgasolver.solver import _lib_query
    assert _lib_query("selftest_d2f") == 0
