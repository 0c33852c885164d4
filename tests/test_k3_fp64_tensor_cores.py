"""The FP64 map's K3 contractions on the tensor cores by exact digit slicing (fdga_k3_oz.cu).

Option k3_fp64_tensor_cores: 2 (default) from Nν3 = 32 on, 1 at every supported Nν3 (a multiple of 8
between 8 and 128), 0 never (FP64 CUDA-core GEMMs).  One FP64 map application with the digit-sliced
kernel agrees with the FP64 CUDA-core GEMMs to 1e-12 per flatten block (about 1e-14 is seen) and with
the oracle to the plain path's 1e-10; the tangent map, whose K3 contractions (modes 0 and 1, and
mode 2 as a dA·M launch and an A·dM launch) run the same kernel, agrees with its CUDA-core form
likewise.  A NaN in the state reaches every K3 entry that the
CUDA-core path turns into NaN.  Cases: Nν3 = 8, 24 (the Hubbard 8x8 workload's box), 32 (local and
4x4 lattice), 80, 96 and 128.
"""
import numpy as np
import pytest

from helpers import blockwise_rel_err, blocks, make_gpu, make_oracle

pytestmark = pytest.mark.gpu

LOCAL8 = dict(kind="siam", T=0.1, U=1.0, e=0.2, Delta=0.5, D=10.0, nG=16, nK1=16, nK2=(5, 4), nK3=(4, 4),
              mPi_factor=6)
NL24 = dict(kind="hubbard", T=0.2, U=2.0, mu=0.0, t1=1.0, L=4, nG=16, nK1=16, nK2=(6, 16), nK3=(3, 12),
            mPi_factor=3, refvertex_noise=0.05, seed=2)
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
NL8 = dict(kind="hubbard", T=0.5, U=2.0, mu=0.3, t1=1.0, t2=-0.2, L=4, nG=8, nK1=8, nK2=(3, 4), nK3=(2, 4),
           mPi_factor=4, refvertex_noise=0.05, seed=7)
CASES = [LOCAL8, NL24, LOCAL32, NL32, LOCAL80, LOCAL96, LOCAL128]
IDS = ["local8", "nl24", "local32", "nl32", "local80", "local96", "local128"]


def _state(gpu, rng, strategy):
    x = gpu.flatten()
    x = x + 0.05 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
    return gpu.fixed_point(x, strategy) + x  # nonzero FL and Σ for the compared application


@pytest.mark.parametrize("strategy", ["fdPA", "scPA"])
@pytest.mark.parametrize("cfg", CASES, ids=IDS)
def test_digit_sliced_k3_matches_cuda_cores(cfg, strategy):
    rng = np.random.default_rng(21)
    gpu = make_gpu(cfg, True)
    y = _state(gpu, rng, strategy)
    gpu.set_option("k3_fp64_tensor_cores", 0)
    assert gpu.query("k3_fp64_tensor_cores") == 0
    y_cc = gpu.fixed_point(y, strategy) + y
    gpu.set_option("k3_fp64_tensor_cores", 1)
    assert gpu.query("k3_fp64_tensor_cores") == 1
    y_tc = gpu.fixed_point(y, strategy) + y
    assert blockwise_rel_err(cfg, y_tc, y_cc) < 1e-12
    assert blockwise_rel_err(cfg, y_tc, y_cc) > 0.0  # the two paths both ran
    gpu.close()


@pytest.mark.parametrize("cfg", [LOCAL8, NL24, LOCAL32, NL32], ids=["local8", "nl24", "local32", "nl32"])
def test_digit_sliced_k3_oracle_parity(cfg):
    rng = np.random.default_rng(22)
    orc = make_oracle(cfg, True)
    gpu = make_gpu(cfg, True)
    gpu.set_option("k3_fp64_tensor_cores", 1)
    x = orc.flatten()
    x = x + 0.05 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
    for _ in range(2):
        y_orc = orc.residual(x, "fdPA") + x
        y_gpu = gpu.fixed_point(x, "fdPA") + x
        assert blockwise_rel_err(cfg, y_gpu, y_orc) < 1e-10
        x = y_orc + 0.01 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
    gpu.close()


def test_default_follows_the_box():
    gpu = make_gpu(NL24, True)  # Nν3 = 24: CUDA cores by default
    assert gpu.query("k3_fp64_tensor_cores") == 0
    gpu.close()
    gpu = make_gpu(NL32, True)  # Nν3 = 32: tensor cores by default
    assert gpu.query("k3_fp64_tensor_cores") == 1
    gpu.set_option("k3_fp64_tensor_cores", 0)
    assert gpu.query("k3_fp64_tensor_cores") == 0
    with pytest.raises(Exception):
        gpu.set_option("k3_fp64_tensor_cores", 4)
    gpu.close()


@pytest.mark.parametrize("cfg", [NL24, NL32, LOCAL80], ids=["nl24", "nl32", "local80"])
def test_digit_sliced_k3_exponent_bound(cfg):
    """The bound of M from the FP64 exponents of its factors (a few bits looser than the FP32 bound,
    taken when that bound overflows) keeps the map within 1e-12 of the CUDA-core GEMMs; the
    tangent's two launches take it as well."""
    rng = np.random.default_rng(25)
    gpu = make_gpu(cfg, True)
    y = _state(gpu, rng, "fdPA")
    v = rng.standard_normal(y.size) + 1j * rng.standard_normal(y.size)
    gpu.set_option("k3_fp64_tensor_cores", 0)
    y_cc = gpu.fixed_point(y, "fdPA") + y
    gpu.unflatten(y)
    _, j_cc = gpu.frule(v)
    gpu.set_option("k3_fp64_tensor_cores", 3)
    assert gpu.query("k3_fp64_tensor_cores") == 1
    y_eb = gpu.fixed_point(y, "fdPA") + y
    gpu.unflatten(y)
    _, j_eb = gpu.frule(v)
    assert blockwise_rel_err(cfg, y_eb, y_cc) < 1e-12
    assert blockwise_rel_err(cfg, j_eb, j_cc) < 1e-12
    gpu.close()


@pytest.mark.parametrize("cfg", [NL32, LOCAL80], ids=["nl32", "local80"])
def test_digit_sliced_k3_tangent(cfg):
    rng = np.random.default_rng(23)
    gpu = make_gpu(cfg, True)
    y = _state(gpu, rng, "fdPA")
    v = rng.standard_normal(y.size) + 1j * rng.standard_normal(y.size)
    gpu.set_option("k3_fp64_tensor_cores", 0)
    gpu.unflatten(y)
    _, j_cc = gpu.frule(v)
    gpu.set_option("k3_fp64_tensor_cores", 1)
    gpu.unflatten(y)
    _, j_tc = gpu.frule(v)
    assert blockwise_rel_err(cfg, j_tc, j_cc) < 1e-12
    gpu.close()


def test_digit_sliced_k3_propagates_nan():
    rng = np.random.default_rng(24)
    gpu = make_gpu(NL32, True)
    y = _state(gpu, rng, "fdPA")
    _, s, e = [b for b in blocks(NL32) if b[0] == "t.K3"][0]
    y[s + (e - s) // 3] = np.nan
    gpu.set_option("k3_fp64_tensor_cores", 0)
    r_cc = gpu.fixed_point(y, "fdPA")
    gpu.set_option("k3_fp64_tensor_cores", 1)
    r_tc = gpu.fixed_point(y, "fdPA")
    nan_cc = np.isnan(r_cc)
    assert nan_cc.any()
    assert np.isnan(r_tc[nan_cc]).all()
    gpu.close()


@pytest.mark.parametrize("cfg,what", [(NL8, "fdPA_1loop"), (LOCAL8, "fdPA_new"), (LOCAL8, "scPA_new"), (NL8, "mfrg")],
                         ids=["nl8-fdPA_1loop", "local8-fdPA_new", "local8-scPA_new", "nl8-mfrg"])
def test_digit_sliced_k3_other_maps(cfg, what):
    """The strategy variants (the one-loop K3 form among them) and the mfRG map run the same K3
    contractions; at Nν3 = 8 with option 1 they agree with their CUDA-core form to 1e-12."""
    rng = np.random.default_rng(26)
    gpu = make_gpu(cfg, True)
    x = gpu.flatten()
    x = x + 0.05 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
    nF = blocks(cfg)[-1][1]  # the vertex part of the state

    def run():
        if what == "mfrg":
            return np.concatenate([gpu.mfrg_apply(x[:nF]), x[nF:]])
        return gpu.fixed_point(x, what) + x

    gpu.set_option("k3_fp64_tensor_cores", 0)
    y_cc = run()
    gpu.set_option("k3_fp64_tensor_cores", 1)
    assert gpu.query("k3_fp64_tensor_cores") == 1
    y_tc = run()
    assert blockwise_rel_err(cfg, y_tc, y_cc) < 1e-12
    gpu.close()
