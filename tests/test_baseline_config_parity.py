"""GPU vs the CPU oracle at the shapes of the benchmark workloads that the other parity tests do
not reach: the local SIAM workload (nK1=64, nK2=(32,32), nK3=(16,16), mΠν_factor=6) and the boxes of
the Hubbard 16x16 precision workload (nK3=(20,40), Nν3 = 80) on a 4x4 lattice.

Tolerances: the FP64 map agrees with the oracle to 1e-10 relative per flatten block (the plain path's
parity bar; at both shapes, Nν3 = 32 and 80, its K3 contractions run on the tensor cores by digit
slicing, the default from Nν3 = 32 on); the mixed map, whose K3 contractions run on the tensor cores (tcgen05, TF32 hi/lo split,
FP32 accumulation) at Nν3 = 80, agrees with the oracle's FP64 map to 1e-5 per block.  solve! on the
device (Anderson m = 8, δ = 0.5, tol 1e-8, maxiter 50) follows the oracle's trajectory: the same
iteration count and the same fixed point to 1e-9.
"""
import numpy as np
import pytest

from helpers import blockwise_rel_err, make_gpu, make_oracle

pytestmark = pytest.mark.gpu
TOL = 1e-10
TOL_MIXED = 1e-5


def _cfg(name):
    from fdgasolver.workloads import CONFIGS
    return dict(CONFIGS[name])


def _perturbed(x, rng, scale):
    return x + scale * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))


def test_siam_local_workload_map_parity():
    """Two map applications at the full local-workload shapes, init_sym_grp! groups, fdPA."""
    cfg = _cfg("siam_b10_nk3_16")
    orc = make_oracle(cfg, True)
    gpu = make_gpu(cfg, True)
    rng = np.random.default_rng(21)
    x = _perturbed(orc.flatten(), rng, 0.02)
    for _ in range(2):
        y_orc = orc.residual(x, "fdPA") + x
        y_gpu = gpu.fixed_point(x, "fdPA") + x
        assert blockwise_rel_err(cfg, y_gpu, y_orc) < TOL
        x = _perturbed(y_orc, rng, 0.005)
    gpu.close()


def test_siam_local_workload_solve_trajectory():
    """solve!(S; δ = 0.5, maxiter = 50, tol = 1e-8) from the PA start on the device and on the oracle."""
    cfg = _cfg("siam_b10_nk3_16")
    orc = make_oracle(cfg, True)
    gpu = make_gpu(cfg, True)
    r_o = orc.solve("fdPA", maxiter=50, tol=1e-8, beta=0.5, mem=8)
    r_g = gpu.solve("fdPA", maxiter=50, tol=1e-8, delta=0.5, mem=8)
    assert r_o["converged"] and r_g["converged"]
    assert r_o["iterations"] == r_g["iterations"]
    assert blockwise_rel_err(cfg, gpu.flatten(), orc.flatten()) < 1e-9
    gpu.close()


def test_precision_workload_boxes_fp64_and_tensor_core_maps():
    """nK3 = (20, 40) boxes (Nν3 = 80) on 4x4: the FP64 map at 1e-10 and the mixed map (tcgen05 K3
    contractions) at 1e-5 against the oracle, from the same perturbed state."""
    cfg = _cfg("hubbard4x4_n09_nk3_20x40")
    orc = make_oracle(cfg, True)
    gpu = make_gpu(cfg, True)
    assert gpu.query("k3_block_dim") == 80
    rng = np.random.default_rng(22)
    x = _perturbed(orc.flatten(), rng, 0.01)
    y_orc = orc.residual(x, "fdPA") + x
    y64 = gpu.fixed_point(x, "fdPA") + x
    assert blockwise_rel_err(cfg, y64, y_orc) < TOL
    gpu.set_precision("mixed")
    gpu.set_option("k3_tensor_cores", 1)
    y32 = gpu.fixed_point(x, "fdPA") + x
    err = blockwise_rel_err(cfg, y32, y_orc)
    assert 0 < err < TOL_MIXED
    gpu.close()
