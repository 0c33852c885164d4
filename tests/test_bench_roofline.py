"""bench.py's roofline entry for the fused K3 contraction, on a stand-in solver (no GPU): the FP64
CUDA-core kernel is reported against the FP64 FMA rate, the digit-sliced tensor-core kernel by its
BF16 MMA work against the measured bf16 peak, with its FP64-equivalent rate beside it."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


class FakeSolver:
    def __init__(self, blocks, dim, tensor_cores):
        self.v = {"k3_blocks": blocks, "k3_block_dim": dim, "fp64_gflops": 1000.0,
                  "k3_fp64_tensor_cores": 1.0 if tensor_cores else 0.0}

    def query(self, key):
        return self.v[key]


STAGES = {"bse_K3_gemm": 0.5, "sde": 0.5}


def test_fp64_cuda_core_roofline():
    r = bench.k3_gemm_roofline(FakeSolver(100, 24, False), STAGES, "nonexistent_workload")
    assert r["bound"] == "fp64" and r["unit"] == "TFLOP/s"
    flops = 3 * 100 * 8 * 24 ** 3
    assert r["achieved"] == pytest.approx(flops / 0.5e-3 / 1e12)
    assert r["frac"] == pytest.approx(r["achieved"] / 1.0)
    assert r["share_of_iteration"] == pytest.approx(0.5)


def test_digit_sliced_roofline():
    r = bench.k3_gemm_roofline(FakeSolver(234, 80, True), STAGES, "nonexistent_workload")
    assert r["bound"] == "tensor" and "k_bse_K3_oz" in r["kernel"]
    mma = 3 * 234 * 36 * 2 * 128 * 160 * 160
    assert r["flops_per_launch"] == mma
    assert r["achieved"] == pytest.approx(mma / 0.5e-3 / 1e12)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    fp64_equiv = 3 * 234 * 8 * 80 ** 3 / 0.5e-3 / 1e12
    assert r["fp64_equivalent_tflops"] == pytest.approx(fp64_equiv)
    assert r["fp64_equivalent_frac"] == pytest.approx(fp64_equiv / 1.0)
    assert r["traffic"] is None  # no committed profile under that workload name
