"""Host-side check of the arithmetic behind the FP64 K3 contraction on the tensor cores (the digit
slicing of fdga_k3_oz.cu), emulated exactly in numpy integers: 56-bit fixed point relative to the
block bounds, 8 digits of 7 bits, the 36 digit-pair products summed by diagonal with each diagonal
rounded to FP32 as the tensor-memory accumulator holds it, the diagonals joined in two 64-bit
integers, and the FP32 magnitude bound of the M tile.  The emulated product must match A·M in FP64
to 2e-14 of max|A·M| on blocks whose entries spread over e^6, for the forms of M of BSE_L_K3, BSE_K3
and the tangent's A·dM launch, and the bound of M must lie within 2 binary orders of max|M|.  The
CUDA kernel itself is compared on the GPU (test_k3_fp64_tensor_cores.py).
"""
import numpy as np
import pytest

S, DB = 8, 7


def _expo(v):
    return ((np.ascontiguousarray(v, dtype=np.float64).view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)).astype(
        np.int64)


def _cexpo(c):
    return np.maximum(_expo(c.real), _expo(c.imag))


def _mag_up(x):
    """FP32 upper bound of |x| from the top 23 significand bits + 1 ulp (2^-126 below the range)."""
    b = np.abs(np.ascontiguousarray(x, dtype=np.float64)).view(np.uint64)
    e = (b >> np.uint64(52)).astype(np.int64) - 896
    assert (e < 255).all()
    bits = ((np.clip(e, 0, 255).astype(np.uint64) << np.uint64(23)) | ((b >> np.uint64(29)) & np.uint64(0x7FFFFF)))
    f = (bits.astype(np.uint32) + np.uint32(1)).view(np.float32)
    return np.where(e <= 0, np.where(b != 0, np.float32(2.0 ** -126), np.float32(0)), f).astype(np.float32)


def _fixed56(v, F):
    b = np.ascontiguousarray(v, dtype=np.float64).view(np.uint64)
    ev = ((b >> np.uint64(52)) & np.uint64(0x7FF)).astype(np.int64)
    mant = (b & np.uint64(0xFFFFFFFFFFFFF)) | np.uint64(1 << 52)
    rs = F - ev - 3
    assert (rs[ev != 0] >= -3).all()  # every entry lies below the bound
    Y = np.where(rs < 0, mant << np.clip(-rs, 0, 3).astype(np.uint64), mant >> np.clip(rs, 0, 63).astype(np.uint64))
    Y = np.where((ev != 0) & (rs < 64), Y, np.uint64(0)).astype(np.int64)
    return [np.where(v < 0, -1, 1) * ((Y >> (DB * (S - 1 - s))) & 127) for s in range(S)]


def _digit_sliced_product(A, M, FM):
    N = A.shape[0]
    Ar = np.zeros((N, 2 * N))
    Ar[:, 0::2], Ar[:, 1::2] = A.real, A.imag
    Br = np.zeros((2 * N, 2 * N))  # rows n = 2ν' + p, columns k = 2ω + q
    Br[0::2, 0::2], Br[0::2, 1::2] = M.real.T, -M.imag.T
    Br[1::2, 0::2], Br[1::2, 1::2] = M.imag.T, M.real.T
    FA = int(_cexpo(A).max())
    da, db = _fixed56(Ar, FA), _fixed56(Br, FM)
    hi = np.zeros((N, 2 * N), dtype=np.int64)
    lo = np.zeros_like(hi)
    for g in range(S):
        acc = sum(da[s] @ db[g - s].T for s in range(S) if 0 <= g - s < S)
        acc = acc.astype(np.float32).astype(np.int64)  # the FP32 accumulator
        assert np.abs(acc).max() < 2 ** 26
        if g < 4:
            hi = hi * 128 + acc
        else:
            lo = lo * 128 + acc
    assert np.abs(hi).max() < 2 ** 53 and np.abs(lo).max() < 2 ** 53
    E = FA + FM - 2044
    D = hi.astype(np.float64) * 2.0 ** (E - 35) + lo.astype(np.float64) * 2.0 ** (E - 63)
    return D[:, 0::2] + 1j * D[:, 1::2]


def _bound_exponent(terms):
    """F_M from the FP32 bound of |M| = |Σ q_i(ω) Σ_j X_ij(ω, ν')| (the kernel's pass 1): the parts of
    a sum of X's are bounded by the sums of their parts' bounds."""
    bx = by = np.float32(0)
    for q, Xs in terms:
        qx, qy = _mag_up(q.real)[:, None], _mag_up(q.imag)[:, None]
        xx = sum(_mag_up(X.real) for X in Xs)
        xy = sum(_mag_up(X.imag) for X in Xs)
        bx = bx + qx * xx + qy * xy
        by = by + qx * xy + qy * xx
    B = np.float32(max(bx.max(), by.max()))
    Bp = np.float32(B + B * np.float32(2.0 ** -16))
    return int(np.array([Bp], dtype=np.float32).view(np.uint32)[0] >> 23) + 896


@pytest.mark.parametrize("N", [8, 24, 96])
@pytest.mark.parametrize("form", ["one", "three", "tangent"])
def test_digit_sliced_product_matches_fp64(N, form):
    """one: Π0 F0 (BSE_L_K3); three: s1 (Π - Π0) F0 + s1 Π (Γ ± γL) (BSE_K3); tangent:
    s1 dΠ (F0 + Γ ± γL) + s1 Π (dΓ ± dγL) (the A·dM launch of the tangent)."""
    rng = np.random.default_rng(N + {"one": 0, "three": 1000, "tangent": 2000}[form])

    def crand(*sh, spread=6.0):
        return (rng.standard_normal(sh) + 1j * rng.standard_normal(sh)) * np.exp(-rng.uniform(0, spread, sh))

    A = crand(N, N)
    if form == "one":
        terms = [(crand(N, spread=10.0), [crand(N, N)])]
    elif form == "three":
        p = crand(N, spread=10.0)
        terms = [(crand(N, spread=10.0), [crand(N, N)]), (p, [crand(N, N), -crand(N, N)])]
    else:
        terms = [(crand(N, spread=10.0), [crand(N, N), crand(N, N), -crand(N, N)]),
                 (crand(N, spread=10.0), [crand(N, N), -crand(N, N)])]
    M = sum(q[:, None] * sum(Xs) for q, Xs in terms)
    FM = _bound_exponent(terms)
    assert _cexpo(M).max() <= FM <= _cexpo(M).max() + 2
    C = _digit_sliced_product(A, M, FM)
    ref = A @ M
    assert np.abs(C - ref).max() / np.abs(ref).max() < 2e-14
