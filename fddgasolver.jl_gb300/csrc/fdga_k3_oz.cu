// fdga_k3_oz.cu -- the K3 Bethe-Salpeter contractions of the FP64 map on the tcgen05 tensor cores,
// by exact digit slicing (the Ozaki scheme): FP64 results from BF16 products.
//
// Per (channel, representative (P, Ω) block) the BSE is one complex product C = A·M of Nν3 x Nν3
// matrices (src/BSEa/BSEa_K3.jl:1-128; M formed elementwise in FP64 from the caches, Π, Π0 and FL,
// exactly as the FP64 CUDA-core kernel forms it).  It runs as the real GEMM
// D[ν][n] = Σ_k A_r[ν][k] B_r[k][n] in the 2x2 real form of the tcgen05 TF32 kernel (k = 2ω + q,
// n = 2ν' + p), split in column tiles of NT = 32 real columns.
//
// Exact slicing.  Every entry v of the block of A, and of the tile of M, is written in fixed point
// relative to a bound 2^(F-1022) > |v| with 56 fractional bits, Y = ⌊|v| 2^(56+1022-F)⌋ < 2^56, taken
// straight from the FP64 significand by an integer shift, and Y is cut into S = 8 digits of 7 bits:
//   v ≈ sign(v) Σ_s d_s 2^(F-1022-7(s+1)),  0 ≤ d_s ≤ 127  (truncation error < 2^-56 of the bound).
// F_A is the largest exponent field over the block of A; F_M comes from an FP32 upper bound of |M|
// over the tile formed from the magnitudes of M's factors (within a factor 2 of max|M| short of
// cancellation), so that pass 1 spends no FP64 operation.  A digit times a sign is a BF16 number
// exactly (8 significant bits).  The products of digit pairs (s, t) with s + t = g share one FP32
// accumulator in tensor memory (g = 0..S-1, 8 x 32 columns): each product is an integer below 2^14,
// so for K ≤ 2·128 the diagonals g ≤ 3 (at most 4 pairs) sum below 2^24 and are exact; the longer
// diagonals pass 2^24 only when most digits of a row and a column are near 127 with equal signs,
// and then round at 2^-24 of the accumulator (below 2^-41 of max|A| max|M| for g = 4, less for the
// later ones).  The pairs with s + t ≥ S are dropped: with the truncation this leaves below ~2^-52
// of max|A| max|M| per product term, the size of an FP64 rounding (a CPU emulation of these sums,
// bounds included, on random blocks with entries spread over e^6 gives max|C - A·M| / max|A·M| ≤
// 7e-15 at Nν = 96).  The epilogue joins the integer diagonals exactly in two 64-bit integers and
// applies the block scales with one FP64 addition,
//   D = 2^(F_A + F_M - 2044) Σ_g 2^(-7(g+2)) acc_g,
// then the BSE's epilogue (T C and γL), as the FP64 kernel does.  A block of A or tile of M that
// holds an infinity or NaN writes NaN, as the FP64 sum would.
//
// Per launch and group of blocks: k_oz_adigits finds F_A of every A block and writes its digit
// operands to a global buffer, once per block, in the shared-memory operand layout; then the
// contraction runs one CTA of 256 threads per (channel slot, block, column tile), K in chunks of 16
// (8 ω) with two shared-memory stages of 8 + 8 digit operands.  Per chunk one thread bulk-copies the
// 8 A digit operands (cp.async.bulk, completing on an mbarrier) while warps 4-7 form the tile of M
// in FP64 and digitise it; then the same thread issues the 36 MMAs (kind::f16, BF16 inputs, FP32
// accumulation) and commits them to the stage's mbarrier.  Every wait is bounded (a timeout sets
// *err; the kernel still waits, bounded, for its copies and MMAs in flight and releases its tensor
// memory).
#include <algorithm>

#include "fdga_kernels.h"

namespace fdga {

namespace {

constexpr int OZ_THREADS = 256;
constexpr int S = 8;                      // digits per operand
constexpr int DB = 7;                     // bits per digit
constexpr int KC = 16;                    // real K per chunk (one BF16 MMA)
constexpr int CW = KC / 2;                // ω per chunk
constexpr int NT = 32;                    // real columns per tile
constexpr int A_DIG = 128 * KC * 2;       // one A digit operand: 128 rows x 16 BF16 = 4 KB
constexpr int B_DIG = NT * KC * 2;        // one B digit operand: 32 rows x 16 BF16 = 1 KB
constexpr int STAGE = S * (A_DIG + B_DIG);
constexpr uint32_t SPIN_LIMIT = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
// byte offset of element (row r, k) in a K-major no-swizzle operand of 16-bit elements, KC columns:
// 8-row x 16-byte core matrices, K-adjacent ones 128 B apart, 8-row groups KC·16 = 256 B apart
__device__ __forceinline__ uint32_t op16(int r, int k) {
    return (uint32_t)((((r >> 3) * (KC / 8) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}
__device__ __forceinline__ uint64_t sdesc16(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)((KC * 16) >> 4) << 32) |
           (1ull << 46);
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t i = 0; i < SPIN_LIMIT; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// global -> shared bulk copy (16-byte aligned addresses, a multiple of 16 bytes), completing on bar
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ void mma_bf16(uint32_t dt, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        :
        : "r"(dt), "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
// the exponent field of an FP64 value
__device__ __forceinline__ int efield(double v) {
    return (int)(((unsigned long long)__double_as_longlong(v) >> 52) & 0x7ffull);
}
// |v| in fixed point relative to the bound 2^(F-1022), 56 fractional bits: ⌊|v| 2^(56+1022-F)⌋
// (0 for zero and subnormal v).  |v| < 2^(F-1022) gives ev ≤ F, so the shift F - ev - 3 is ≥ -3.
__device__ __forceinline__ unsigned long long fixed56(double v, int F) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int ev = (int)((b >> 52) & 0x7ffull);
    if (ev == 0 || F == 0) return 0ull;
    const int rs = F - ev + (53 - S * DB);
    const unsigned long long mant = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    return rs < 0 ? (mant << (-rs)) : (rs < 64 ? (mant >> rs) : 0ull);
}
__device__ __forceinline__ uint32_t digit(unsigned long long Y, int s) {
    return (uint32_t)(Y >> (DB * (S - 1 - s))) & 127u;
}
// two digits d < 128 as a pair of signed BF16 numbers (low half first), sgn holding the sign bits
// (bits 15 and 31): the pattern 0x4300 | d is the BF16 number 128 + d (0xC300 | d: -(128 + d)), and
// one packed BF16 subtraction of ±128 leaves ±d exactly
__device__ __forceinline__ uint32_t bf_pair(uint32_t dlo, uint32_t dhi, uint32_t sgn) {
    const uint32_t b = 0x43004300u | sgn;
    uint32_t r;
    asm("sub.rn.bf16x2 %0, %1, %2;" : "=r"(r) : "r"(b | dlo | (dhi << 16)), "r"(b));
    return r;
}
__device__ __forceinline__ uint32_t sbit(double v) {
    return (uint32_t)((unsigned long long)__double_as_longlong(v) >> 63);
}
// the larger exponent field of the two parts of a complex number: both |x|, |y| < 2^(E - 1022)
// (zero and subnormal parts included, with E = 0)
__device__ __forceinline__ int cexpo(cplx v) { return max(efield(v.x), efield(v.y)); }
// an FP32 upper bound of |x| from its top 23 significand bits (+1 ulp); 2^-126 below the FP32
// normal range, +inf above it and for an infinity or NaN
__device__ __forceinline__ float mag_up(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
    const int e = (int)(b >> 52) - 896;  // the FP32 exponent field of |x|
    if (e <= 0) return b ? __uint_as_float(0x00800000u) : 0.0f;
    if (e >= 255) return __uint_as_float(0x7F800000u);
    return __uint_as_float((((uint32_t)e << 23) | ((uint32_t)(b >> 29) & 0x7FFFFFu)) + 1u);
}
__device__ __forceinline__ float2 mag_up(cplx v) { return make_float2(mag_up(v.x), mag_up(v.y)); }
// bounds of |Re(a b)| and |Im(a b)| from part bounds of a and b, added to acc
__device__ __forceinline__ void prod_bound(float2 a, float2 b, float2& acc) {
    acc.x = fmaf(a.x, b.x, fmaf(a.y, b.y, acc.x));
    acc.y = fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y));
}
// x · 2^e for an integer |x| < 2^53 (exact), built from its bits on the integer pipes; 0 below the
// normal range
__device__ __forceinline__ double i2d_scaled(long long x, int e) {
    if (x == 0) return 0.0;
    const unsigned long long sg = x < 0 ? (1ull << 63) : 0ull;
    const unsigned long long u = x < 0 ? (unsigned long long)(-x) : (unsigned long long)x;
    const int p = 63 - __clzll((long long)u);  // 2^p ≤ u < 2^(p+1), p ≤ 52
    const int ef = p + e + 1023;
    if (ef <= 0) return 0.0;
    if (ef >= 2047) return __longlong_as_double((long long)(sg | 0x7FF0000000000000ull));
    const unsigned long long mant = (u << (52 - p)) & 0xFFFFFFFFFFFFFull;
    return __longlong_as_double((long long)(sg | ((unsigned long long)ef << 52) | mant));
}

// The A digit operands of the blocks r0, r0 + 1, ..: one CTA per block finds F_A, the largest
// exponent field of the block's entries (both parts; stored in fa_blk for the contraction), then
// writes, per chunk of 8 ω, S digit operands of the block's N rows in the K-major no-swizzle layout
// of op16 (N·32 bytes each, rows ≥ N left out).  Each A block is so read and digitised once, not once
// per column tile; the contraction copies the operands into shared memory.  Item e = (chunk, row,
// quad) holds row `row` and the four ω 4·quad.. of the chunk.
__global__ void __launch_bounds__(256) k_oz_adigits(K3Args3 args, Dims d, int* __restrict__ fa_blk, uint8_t* adig,
                                                    int r0) {
    __shared__ int wmax[8];
    const int N = d.N3n, nchunks = N / CW;
    const int rr = blockIdx.x, rest = r0 + rr, nb = args.nblocks;
    const int slot = rest / nb, bi = rest % nb;
    const int blk = args.blocks ? args.blocks[bi] : bi;
    const cplx* A = (slot == 0 ? args.a[0].A : slot == 1 ? args.a[1].A : args.a[2].A) + (size_t)blk * N * N;
    int mx = 0;
    for (int e = threadIdx.x; e < N * N; e += 256) mx = max(mx, cexpo(ldg(A + e)));
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = mx;
    __syncthreads();
    int FA = wmax[0];
    for (int w = 1; w < 8; ++w) FA = max(FA, wmax[w]);
    if (threadIdx.x == 0) fa_blk[rest] = FA;
    const size_t arow = (size_t)N * 32;
    for (int e = threadIdx.x; e < 2 * N * nchunks; e += 256) {
        const int c = e / (2 * N), rq = e % (2 * N), row = rq >> 1, quad = rq & 1;
        const cplx* src = A + (size_t)row * N + CW * c + 4 * quad;
        uint32_t wd[S][4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const cplx v = ldg(src + i);
            const unsigned long long yr = fixed56(v.x, FA), yi = fixed56(v.y, FA);
            const uint32_t sg = (sbit(v.x) << 15) | (sbit(v.y) << 31);
#pragma unroll
            for (int s = 0; s < S; ++s) wd[s][i] = bf_pair(digit(yr, s), digit(yi, s), sg);
        }
        uint8_t* dst = adig + ((size_t)rr * nchunks + c) * S * arow + op16(row, 8 * quad);
#pragma unroll
        for (int s = 0; s < S; ++s)
            *reinterpret_cast<uint4*>(dst + (size_t)s * arow) = make_uint4(wd[s][0], wd[s][1], wd[s][2], wd[s][3]);
    }
}

template <int MODE>
__global__ void __launch_bounds__(OZ_THREADS, 2)
    k_bse_K3_oz(K3Args3 args, Dims d, int ntile, const int* __restrict__ fa_blk, const uint8_t* __restrict__ adig,
                int r0, int ebound, int* err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ uint64_t mbar[2];   // per stage: the chunk's MMAs are done (tcgen05.commit)
    __shared__ uint64_t afull[2];  // per stage: the chunk's A digit operands have arrived
    __shared__ uint32_t tmem_base;
    // the ω factors of M with their signs: [0] Π0 (mode 0), s1 (Π - Π0) (mode 1) or s1 dΠ (mode 3),
    // [1] s1 Π, and the exponent bounds of [0] and of Π
    __shared__ cplx qf[128][2];
    __shared__ int qe[128][2];
    __shared__ float2 qm[128][2];  // part bounds of [0] and of Π
    // bounds of the tile of M: [0] the FP32 bound of |M| (as bits), [1] the exponent-sum bound (when
    // the FP32 bound is not finite), [2] non-finite operands
    __shared__ int mbnd[3];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = d.N3n;
    const int nchunks = N / CW;  // N is a multiple of 8
    const int nb = args.nblocks;
    const int tile = blockIdx.x % ntile;
    const int rest = r0 + (int)(blockIdx.x / ntile);
    const int slot = rest / nb;
    const int blk = args.blocks ? args.blocks[rest % nb] : (int)(rest % nb);
    const K3Args& a = args.a[slot];
    const int CH = args.ch[slot];
    const int m = blk % d.N3O - (d.n3O - 1), P = blk / d.N3O;
    const size_t base = (size_t)blk * N * N;
    const int col0 = tile * NT;                      // first real column of the tile
    const int ncol = min(NT, 2 * N - col0);          // 16 or 32
    const int cc0 = col0 / 2, ncc = ncol / 2;        // complex columns ν'
    const double s1 = (CH == CH_A) ? 1.0 : -1.0, s2 = (CH == CH_T) ? -1.0 : 1.0;
    // M has the Γ and γL terms (mode 1 but the one-loop form; mode 3 always)
    const bool full = MODE == 3 || (MODE == 1 && (a.flags & K3F_1LOOP) == 0);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(&tmem_base))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid < N) {
        const size_t ip = ixPi(d, P, m, tid - d.n3n);
        const cplx pi0 = (MODE != 3 && a.Pi0) ? ldg(a.Pi0 + ip) : mk(0.0, 0.0);
        cplx q0 = pi0, q1 = mk(0.0, 0.0);
        if (MODE >= 1) {
            const cplx pi = ldg(a.Pi + ip);
            q1 = pi * s1;
            q0 = (MODE == 3) ? ldg(a.tPi + ip) * s1 : (pi - pi0) * s1;
        }
        qf[tid][0] = q0;
        qf[tid][1] = q1;
        qe[tid][0] = cexpo(q0);
        qe[tid][1] = cexpo(q1);
        qm[tid][0] = mag_up(q0);
        qm[tid][1] = mag_up(q1);
    }
    if (tid < 3) mbnd[tid] = 0;
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[i])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&afull[i])) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    // γL at a K3 index in the channel's spin combination (t: 2 FL.γt - FL.γa), of FL or of the
    // tangent's dFL
    auto gl_of = [&](const cplx* FLc, const cplx* FLt, const cplx* FLa, size_t i) -> cplx {
        if (CH == CH_T) {
            const cplx t = ldg(FLt + i), u = ldg(FLa + i);
            return cplx{fma(t.x, 2.0, -u.x), fma(t.y, 2.0, -u.y)};
        }
        return ldg(FLc + i);
    };
    auto gl_at = [&](size_t i) -> cplx { return gl_of(a.FLc, a.FLt, a.FLa, i); };
    auto glt_at = [&](size_t i) -> cplx { return gl_of(a.tFLc, a.tFLt, a.tFLa, i); };
    // part bounds of γL (t: |2t - u| ≤ 2|t| + |u|)
    auto gl_bound = [&](const cplx* FLc, const cplx* FLt, const cplx* FLa, size_t i) -> float2 {
        if (CH == CH_T) {
            const float2 tb = mag_up(ldg(FLt + i)), ub = mag_up(ldg(FLa + i));
            return make_float2(fmaf(2.0f, tb.x, ub.x), fmaf(2.0f, tb.y, ub.y));
        }
        return mag_up(ldg(FLc + i));
    };
    // exponent bound of γL (t: |2t - u| < 2^(max(Et+1, Eu)+1-1022)) and whether it is finite
    auto gl_expo = [&](const cplx* FLc, const cplx* FLt, const cplx* FLa, size_t i, int& nf) -> int {
        if (CH == CH_T) {
            const int et = cexpo(ldg(FLt + i)), eu = cexpo(ldg(FLa + i));
            nf |= (et == 0x7ff) | (eu == 0x7ff);
            return max(et + 1, eu) + 1;
        }
        const int e = cexpo(ldg(FLc + i));
        nf |= (e == 0x7ff);
        return e;
    };
    // pass 1: F_A, the exponent field bound of A over the block (its largest exponent field), comes
    // from k_oz_adigits, which reads every A block once for all its column tiles; here, a bound of |M|
    // over the tile from FP32 upper bounds of the parts of its factors (one product in
    // mode 0 and one-loop, s1[(Π-Π0)F0 + Π Γ] + s2 Π γL otherwise; |Re(ab)| ≤ |a.x||b.x| + |a.y||b.y|,
    // |Im(ab)| ≤ |a.x||b.y| + |a.y||b.x|), raised by 2^-16 for the FP32 roundings:
    // |M| ≤ B < 2^(F_M - 1022) with F_M = (FP32 exponent field of B) + 896.  Where B is not finite
    // (operands beyond the FP32 range, an infinity or a NaN), a second pass bounds M from the FP64
    // exponent fields of its factors instead (a complex product of parts below 2^(Ea-1022) and
    // 2^(Eb-1022) has parts below 2^(Ea+Eb-2043); at most three products: F_M = max(Ea + Eb) - 1019).
    {
        float bm = 0.0f;
        for (int e = tid; e < N * ncc; e += OZ_THREADS) {
            const int w = e / ncc, col = cc0 + e % ncc;
            float2 mb = make_float2(0.0f, 0.0f);
            const float2 f0b = mag_up(ldg(a.B0 + base + (size_t)w * N + col));
            if (MODE == 3) {
                // dM = s1 [dΠ (F0 + Γ) + Π dΓ] + s2 [dΠ γL + Π dγL]
                const size_t ig = (CH == CH_P) ? base + (size_t)w * N + col : base + (size_t)col * N + w;
                const float2 gb = mag_up(ldg(a.G + ig));
                prod_bound(qm[w][0], make_float2(f0b.x + gb.x, f0b.y + gb.y), mb);
                prod_bound(qm[w][1], mag_up(ldg(a.tG + ig)), mb);
                const int ot = cross(CH, m, w - d.n3n);
                if (fin(ot, d.n3n)) {
                    const size_t il = base + (size_t)(ot + d.n3n) * N + col;
                    prod_bound(qm[w][0], gl_bound(a.FLc, a.FLt, a.FLa, il), mb);
                    prod_bound(qm[w][1], gl_bound(a.tFLc, a.tFLt, a.tFLa, il), mb);
                }
            } else {
                prod_bound(qm[w][0], f0b, mb);
                if (full) {
                    const size_t ig = (CH == CH_P) ? base + (size_t)w * N + col : base + (size_t)col * N + w;
                    prod_bound(qm[w][1], mag_up(ldg(a.G + ig)), mb);
                    const int ot = cross(CH, m, w - d.n3n);
                    if (fin(ot, d.n3n))
                        prod_bound(qm[w][1], gl_bound(a.FLc, a.FLt, a.FLa, (size_t)(base + (size_t)(ot + d.n3n) * N + col)), mb);
                }
            }
            bm = fmaxf(bm, fmaxf(mb.x, mb.y));  // the parts are ≥ 0, so no NaN arises
        }
        for (int o = 16; o > 0; o >>= 1) bm = fmaxf(bm, __shfl_xor_sync(0xffffffffu, bm, o));
        if (lane == 0) atomicMax(&mbnd[0], (int)__float_as_uint(bm));  // non-negative floats order as integers
    }
    if (ebound && tid == 0) atomicMax(&mbnd[0], 0x7F800000);  // the exponent bound on request (tests)
    __syncthreads();
    if (mbnd[0] >= 0x7F800000) {  // the FP32 bound overflowed: FP64 exponent bound (block-uniform branch)
        int fs = 0, nf = 0;
        for (int e = tid; e < N * ncc; e += OZ_THREADS) {
            const int w = e / ncc, col = cc0 + e % ncc;
            const int e0 = qe[w][0], ep = qe[w][1];
            const int ef0 = cexpo(ldg(a.B0 + base + (size_t)w * N + col));
            int sv = e0 + ef0;
            nf |= (e0 == 0x7ff) | (ef0 == 0x7ff) | (ep == 0x7ff);
            if (full) {
                const size_t ig = (CH == CH_P) ? base + (size_t)w * N + col : base + (size_t)col * N + w;
                const int egs = cexpo(ldg(a.G + ig));
                nf |= (egs == 0x7ff);
                if (MODE == 3) {  // dΠ (F0 + Γ) + Π dΓ: |F0 + Γ| < 2^(max(E0, EΓ)+1-1022)
                    const int etg = cexpo(ldg(a.tG + ig));
                    nf |= (etg == 0x7ff);
                    sv = max(e0 + max(ef0, egs) + 1, ep + etg);
                } else {
                    sv = max(sv, ep + egs);
                }
                const int ot = cross(CH, m, w - d.n3n);
                if (fin(ot, d.n3n)) {
                    const size_t il = base + (size_t)(ot + d.n3n) * N + col;
                    if (MODE == 3) {
                        sv = max(sv, e0 + gl_expo(a.FLc, a.FLt, a.FLa, il, nf));
                        sv = max(sv, ep + gl_expo(a.tFLc, a.tFLt, a.tFLa, il, nf));
                    } else {
                        sv = max(sv, ep + gl_expo(a.FLc, a.FLt, a.FLa, il, nf));
                    }
                }
            }
            fs = max(fs, sv);
        }
        for (int o = 16; o > 0; o >>= 1) {
            fs = max(fs, __shfl_xor_sync(0xffffffffu, fs, o));
            nf |= __shfl_xor_sync(0xffffffffu, nf, o);
        }
        if (lane == 0) {
            atomicMax(&mbnd[1], fs);
            if (nf) atomicOr(&mbnd[2], 1);
        }
        __syncthreads();
    }
    const int FA = fa_blk[rest];
    int FM;
    if (mbnd[0] >= 0x7F800000) {
        FM = max(mbnd[1] - 1019, 0);
    } else {
        const float B = __uint_as_float((uint32_t)mbnd[0]);
        const uint32_t eb = __float_as_uint(fmaf(B, 1.52587890625e-05f, B)) >> 23;  // B (1 + 2^-16)
        FM = (B == 0.0f) ? 0 : (eb >= 255u ? 1152 : (int)eb + 896);
    }
    const bool nonfinite = FA == 0x7ff || mbnd[2] != 0;
    // instruction descriptor: D FP32, A and B BF16, both K-major, N = ncol, M = 128
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(ncol >> 3) << 17) | ((128u >> 4) << 24);
    // shared-memory descriptors of the first A and B digit operands of stage 0 (the start address
    // field, bits 0-13, takes the byte offsets of the other operands >> 4 without carry: all of the
    // shared memory lies below 2^18 bytes)
    const uint64_t dA0 = sdesc16(smem_u32(sm)), dB0 = sdesc16(smem_u32(sm) + S * A_DIG);
    // A digit operands (k_oz_adigits) arrive by bulk copies of the N rows of each digit; rows N..127
    // of both stages are zero, written once here (the tail of each operand from byte N·32 on)
    const uint32_t arow = (uint32_t)N * 32u;
    const uint8_t* asrc = adig + (size_t)(rest - r0) * nchunks * S * arow;
    {
        const int per = (A_DIG - (int)arow) / 16;  // 16-byte words per digit operand tail
        for (int e = tid; e < 2 * S * per; e += OZ_THREADS) {
            const int op = e / per, wdx = e % per;
            uint8_t* stg = sm + (size_t)(op / S) * STAGE + (size_t)(op % S) * A_DIG;
            *reinterpret_cast<uint4*>(stg + arow + 16 * wdx) = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    bool ok = true;
    for (int c = 0; c < nchunks; ++c) {
        const int st = c & 1;
        if (c >= 2 && !mbar_wait(smem_u32(&mbar[st]), ((c - 2) >> 1) & 1)) ok = false;
        uint8_t* Ad = sm + (size_t)st * STAGE;  // S A digit operands, then S B digit operands
        uint8_t* Bd = Ad + S * A_DIG;
        const int w0 = CW * c;
        if (tid == 0) {  // A: row ν, k = 2ω_l holds Re A, 2ω_l + 1 holds Im A
            const uint32_t bar = smem_u32(&afull[st]);
            mbar_expect_tx(bar, (uint32_t)S * arow);
            const uint8_t* src = asrc + (size_t)c * S * arow;
#pragma unroll
            for (int s = 0; s < S; ++s) bulk_g2s(smem_u32(Ad + (size_t)s * A_DIG), src + (size_t)s * arow, arow, bar);
        }
        // B (rows n = 2ν'_l + p of the tile, k = 2ω_l + q): row 2ν'_l holds [Re M, -Im M], row
        // 2ν'_l + 1 holds [Im M, Re M]; M formed in FP64 as the CUDA-core kernel forms it.  Warps 4-7
        // stage B (warp 0 also issues the MMAs).
        for (int e = tid - OZ_THREADS / 2; e >= 0 && e < CW * ncc; e += OZ_THREADS / 2) {
            const int cl = e % ncc, wl = e / ncc, w = w0 + wl, col = cc0 + cl;
            const cplx f0 = ldg(a.B0 + base + (size_t)w * N + col);
            cplx v;
            // s2 Π = ±s1 Π and s2 dΠ = ±s1 dΠ (sign s1 s2), so the γL terms join the Γ terms before
            // the products: two complex products per element instead of three (four for dM)
            if (MODE == 3) {  // dM = s1 dΠ (F0 + Γ ± γL) + s1 Π (dΓ ± dγL)
                const size_t ig = (CH == CH_P) ? base + (size_t)w * N + col : base + (size_t)col * N + w;
                cplx x0 = f0 + ldg(a.G + ig), x1 = ldg(a.tG + ig);
                const int ot = cross(CH, m, w - d.n3n);
                if (fin(ot, d.n3n)) {
                    const size_t il = base + (size_t)(ot + d.n3n) * N + col;
                    const cplx g = gl_at(il), gt = glt_at(il);
                    x0 = (s1 == s2) ? x0 + g : x0 - g;
                    x1 = (s1 == s2) ? x1 + gt : x1 - gt;
                }
                v = cfma(qf[w][0], x0, qf[w][1] * x1);
            } else if (full) {  // M = s1 (Π - Π0) F0 + s1 Π (Γ ± γL)
                const size_t ig = (CH == CH_P) ? base + (size_t)w * N + col : base + (size_t)col * N + w;
                cplx x1 = ldg(a.G + ig);
                const int ot = cross(CH, m, w - d.n3n);
                if (fin(ot, d.n3n)) {
                    const cplx g = gl_at(base + (size_t)(ot + d.n3n) * N + col);
                    x1 = (s1 == s2) ? x1 + g : x1 - g;
                }
                v = cfma(qf[w][0], f0, qf[w][1] * x1);
            } else {
                v = qf[w][0] * f0;
            }
            const unsigned long long yr = fixed56(v.x, FM), yi = fixed56(v.y, FM);
            const uint32_t sr = sbit(v.x), si = sbit(v.y);
            const uint32_t o0 = op16(2 * cl, 2 * wl), o1 = op16(2 * cl + 1, 2 * wl);
            const uint32_t sg0 = (sr << 15) | ((si ^ 1u) << 31), sg1 = (si << 15) | (sr << 31);
#pragma unroll
            for (int s = 0; s < S; ++s) {
                uint8_t* b = Bd + (size_t)s * B_DIG;
                const uint32_t dr = digit(yr, s), di = digit(yi, s);
                *reinterpret_cast<uint32_t*>(b + o0) = bf_pair(dr, di, sg0);
                *reinterpret_cast<uint32_t*>(b + o1) = bf_pair(di, dr, sg1);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            if (!mbar_wait(smem_u32(&afull[st]), (c >> 1) & 1)) ok = false;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint64_t so = (uint64_t)((st * STAGE) >> 4);
#pragma unroll
            for (int s = 0; s < S; ++s)
#pragma unroll
                for (int t = 0; t + s < S; ++t)
                    mma_bf16(tmem + (uint32_t)((s + t) * NT), dA0 + so + (uint64_t)((s * A_DIG) >> 4),
                             dB0 + so + (uint64_t)((t * B_DIG) >> 4), idesc, (c > 0 || s > 0) ? 1u : 0u);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&mbar[st]))
                         : "memory");
        }
    }
    if (nchunks >= 2 && !mbar_wait(smem_u32(&mbar[nchunks & 1]), ((nchunks - 2) >> 1) & 1)) ok = false;
    const uint32_t last_bar = smem_u32(&mbar[(nchunks - 1) & 1]), last_par = ((nchunks - 1) >> 1) & 1;
    if (!mbar_wait(last_bar, last_par)) ok = false;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int q = warp & 3, h = warp >> 2;
    const int nu = 32 * q + lane;
    if (!ok) {
        // a wait gave up: report it, and give the MMAs in flight one more bounded wait before the
        // tensor memory is released
        if (tid == 0) {
            atomicExch(err, 1);
            // and for the A copies in flight (issued by this thread), likewise bounded
            mbar_wait(smem_u32(&afull[(nchunks - 1) & 1]), ((nchunks - 1) >> 1) & 1);
            if (nchunks >= 2) mbar_wait(smem_u32(&afull[nchunks & 1]), ((nchunks - 2) >> 1) & 1);
        }
        mbar_wait(last_bar, last_par);
    } else if (32 * q < N && 16 * h < ncol) {
        // epilogue: warp w reads TMEM lanes 32(w%4).. (rows ν) and the 16-column half w/4 of the
        // tile, 8 columns at a time.  The diagonals are integers (|acc_g| < 2^26); they are joined
        // exactly in two 64-bit integers, hi = Σ_{g<4} acc_g 2^(7(3-g)) < 2^44 and
        // lo = Σ_{g≥4} acc_g 2^(7(7-g)) < 2^46, so D = 2^(E-35) hi + 2^(E-63) lo (E = F_A + F_M - 2044)
        // costs one FP64 addition.
        const int E = FA + FM - 2044;
        const bool zero = FA == 0 || FM == 0;
#pragma unroll 1
        for (int hh = 0; hh < 2; ++hh) {
            long long hi[8], lo[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) hi[j] = lo[j] = 0;
#pragma unroll
            for (int g = 0; g < S; ++g) {
                uint32_t r[8];
                const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(g * NT + 16 * h + 8 * hh);
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                               "=r"(r[7])
                             : "r"(taddr)
                             : "memory");
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const long long v = (long long)__float2int_rn(__uint_as_float(r[j]));
                    if (g < 4) hi[j] = hi[j] * 128 + v;
                    else lo[j] = lo[j] * 128 + v;
                }
            }
            if (nu < N) {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int col = cc0 + 8 * h + 4 * hh + j;
                    const size_t io = base + (size_t)nu * N + col;
                    cplx o;
                    if (nonfinite) {
                        const double qn = __longlong_as_double(0x7ff8000000000000ll);
                        o = mk(qn, qn);
                    } else {
                        const cplx cv = zero ? mk(0.0, 0.0)
                                             : cplx{i2d_scaled(hi[2 * j], E - 35) + i2d_scaled(lo[2 * j], E - 63),
                                                    i2d_scaled(hi[2 * j + 1], E - 35) + i2d_scaled(lo[2 * j + 1], E - 63)};
                        if (MODE == 0) {
                            o = cv * (d.T * ((CH == CH_A) ? 1.0 : -1.0));
                        } else if (a.flags & K3F_NOEPI) {
                            o = cv * d.T;
                        } else {
                            const cplx g = (MODE == 3) ? glt_at(io) : gl_at(io);
                            o = cplx{fma(cv.x, d.T, g.x), fma(cv.y, d.T, g.y)};
                        }
                        if (a.flags & K3F_ACC) o = a.out[io] + o;
                    }
                    a.out[io] = o;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem) : "memory");
}

}  // namespace

bool k3_oz_supported(const Dims& d) {
    // rows ν < N of the 128-lane accumulator; column tiles of 32 or a last one of 16 (MMA N % 16)
    return d.N3n >= 8 && d.N3n <= 128 && (d.N3n % 8) == 0;
}

static size_t k3_oz_smem() { return 2 * (size_t)STAGE; }

cudaError_t prepare_bse_K3_oz() {
    static SmemRecord set0, set1, set3;
    cudaError_t e = raise_smem_limit(k_bse_K3_oz<0>, set0, k3_oz_smem(), 0);
    if (e == cudaSuccess) e = raise_smem_limit(k_bse_K3_oz<1>, set1, k3_oz_smem(), 0);
    if (e == cudaSuccess) e = raise_smem_limit(k_bse_K3_oz<3>, set3, k3_oz_smem(), 0);
    return e;
}

// mode 0 (BSE_L_K3), 1 (BSE_K3), 2 (the tangent dK3 = T (dA·M + A·dM) + dγL): mode 2 runs as two
// launches, each with its own block scales (dA and A need not share a magnitude): the mode-1 kernel
// on dA with the epilogue term left out, then the A·dM kernel adding T C + dγL into the output
cudaError_t launch_bse_K3_oz(cudaStream_t s, int mode, const K3Args3& a, int nslots, const Dims& d, int* err,
                             int* fa_scratch, uint8_t* adig, int adig_blocks, int ebound) {
    if (!k3_oz_supported(d) || mode < 0 || mode > 2 || !fa_scratch || !adig || adig_blocks < 1)
        return cudaErrorInvalidValue;
    const int ntile = (2 * d.N3n + NT - 1) / NT;
    const int nblk = nslots * a.nblocks;
    // per launch: groups of at most adig_blocks blocks (the size of the digit buffer), each
    // digitised (with its exponent bounds) and contracted in stream order
    auto run = [&](auto kernel, const K3Args3& ka) -> cudaError_t {
        cudaError_t e = cudaSuccess;
        for (int r0 = 0; e == cudaSuccess && r0 < nblk; r0 += adig_blocks) {
            const int cnt = std::min(adig_blocks, nblk - r0);
            k_oz_adigits<<<(unsigned)cnt, 256, 0, s>>>(ka, d, fa_scratch, adig, r0);
            e = cudaGetLastError();
            if (e != cudaSuccess) break;
            kernel<<<(unsigned)(cnt * ntile), OZ_THREADS, k3_oz_smem(), s>>>(ka, d, ntile, fa_scratch, adig, r0, ebound,
                                                                            err);
            e = cudaGetLastError();
        }
        return e;
    };
    if (mode == 2) {
        K3Args3 a1 = a, a3 = a;
        for (int i = 0; i < nslots; ++i) {
            if (a.a[i].flags & K3F_1LOOP) return cudaErrorInvalidValue;  // no tangent of the one-loop form
            a1.a[i].A = a.a[i].tA;
            a1.a[i].flags |= K3F_NOEPI;
            a3.a[i].flags |= K3F_ACC;
        }
        // stream order: the second launch's pre-pass overwrites the scratch after the first
        // contraction has read it
        const cudaError_t e = run(k_bse_K3_oz<1>, a1);
        if (e != cudaSuccess) return e;
        return run(k_bse_K3_oz<3>, a3);
    }
    return mode == 1 ? run(k_bse_K3_oz<1>, a) : run(k_bse_K3_oz<0>, a);
}

size_t k3_oz_digit_bytes(const Dims& d) { return (size_t)32 * d.N3n * d.N3n; }

}  // namespace fdga
