// fdga_k3_tma.cu -- the K3 Bethe-Salpeter contractions of the mixed map on the tcgen05 tensor cores,
// fed by TMA (cp.async.bulk.tensor) and warp-specialised.
//
// The contraction (src/BSEa/BSEa_K3.jl:1-128): per (channel, representative (P, Ω) block) one complex
// product C = A·M of Nν3 x Nν3 matrices, M formed elementwise from the caches, Π, Π0 and FL.  As in
// fdga_k3_tc.cu it runs as one real GEMM D[128 x 2N] = A_r[128 x 2N'] · B_r[2N' x 2N] with the complex
// product in 2x2 real form (k = 2ω + q, n = 2ν' + p) and TF32 hi/lo operands accumulated as
// hi·hi + hi·lo + lo·hi in FP32 tensor memory.
//
// Structure: a persistent CTA (one per SM) loops over the (channel, block) work items; warp roles:
//   warp 0        producer: per chunk of CW = 8 ω, 2-8 TMA tile loads (A columns, the rows of cacheF0,
//                 the Γ cache in rows (p) or columns (a, t), FL rows and the tangent operands) and 1D
//                 bulk copies of the chunk's Π, Π0, dΠ into one of 2-8 input stages, signalled on the
//                 stage's mbarrier by the transaction count;
//   last warp     converter: the chunk's Π, Π0, dΠ to FP32 once per stage use (the conversion runs on
//                 GB300's FP64 pipe, so it is not repeated per operand element);
//   formers       (8 or 16 warps from warp 2) split A into TF32 hi/lo and form M (and dM) from the
//                 staged tiles into one of two operand buffers in the no-swizzle K-major canonical layout;
//   warp 1        allocates the tensor memory and issues the MMAs (one thread), 6 per chunk, then
//                 tcgen05.commit frees the operand buffer; the last commit of an item hands its
//                 accumulator (one of two TMEM buffers of 256 columns) to the epilogue;
//   epilogue      (8 or 12 warps, two or three per 32-lane TMEM quadrant) tcgen05.ld of the accumulator,
//                 transposed through shared memory, T·D plus the γL(ν,ν') term, widened to FP64 by bit
//                 operations (exact) and stored as contiguous row segments; then the TMEM buffer is freed.
// The loads of the next chunks, the forming, the MMAs and the previous item's epilogue overlap.
// Every mbarrier wait is bounded: a timeout sets *err and the shared abort flag, every role leaves its
// loop, outstanding TMA loads and MMAs are waited for (bounded), and the tensor memory is released.
// No role waits on a barrier without a bound (no named barriers), so an abort cannot leave a warp behind.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "fdga_kernels.h"

namespace fdga {

namespace {

constexpr int KC = 16;          // real K per chunk (CW complex ω)
constexpr int CW = KC / 2;      // ω per chunk
constexpr int MAX_IN = 8;       // input stages (TMA destinations): as many as the shared memory holds, 2..8
constexpr int NS_OP = 2;        // operand buffers (MMA sources)
constexpr int W_PROD = 0, W_MMA = 1, W_FORM0 = 2;
// role split per mode (measured): the left contraction (mode 0, no γL epilogue term) is bound by the
// forming and takes 16 former and 8 epilogue warps; the others, whose epilogue reads γL, 8 and 12
template <int MODE>
struct Roles {
    static constexpr int N_FORM = MODE == 0 ? 16 : 8;
    static constexpr int N_EPI = MODE == 0 ? 8 : 12;
    static constexpr int W_EPI0 = W_FORM0 + N_FORM;
    static constexpr int W_CONV = W_EPI0 + N_EPI;
    static constexpr int THREADS = 32 * (W_CONV + 1);
    static constexpr int EPI_PER_Q = N_EPI / 4;  // epilogue warps per TMEM lane quadrant
    static constexpr int FORMERS = 32 * N_FORM;
};
constexpr int MAX_EPI = 12;
constexpr int TP = 18;                      // row pitch (floats) of an epilogue warp's transpose tile

constexpr int A_OP = 128 * KC * 4;           // one A operand (hi or lo) of a chunk: 8 KB
constexpr uint32_t SPIN_LIMIT = 1u << 22;    // bounded mbarrier polling
constexpr size_t MIN_SMEM = 116 * 1024;      // one CTA per SM: it owns all 512 TMEM columns
constexpr size_t SMEM_BUDGET = 192 * 1024;   // dynamic shared memory for the stages and operand buffers

// input tile slots of a stage (each 64·N bytes: an N x KC column box or a CW x 2N row box)
enum { T_A = 0, T_B0 = 1, T_G = 2, T_TG = 3, T_FL0 = 4, T_FL1 = 5, T_TFL0 = 6, T_TFL1 = 7 };

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t op_off(int r, int k) {
    return (uint32_t)((((r >> 3) * (KC / 4) + (k >> 2)) << 7) + ((r & 7) << 4) + ((k & 3) << 2));
}
// shared-memory matrix descriptor: start, LBO = 128 B, SBO = KC·32 B, fixed 0b001 at bits 46-48, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)((KC * 32) >> 4) << 32) |
           (1ull << 46);
}
__device__ __forceinline__ void split_tf32(float v, float& hi, float& lo) {
    hi = __uint_as_float(__float_as_uint(v) & 0xFFFFE000u);
    lo = v - hi;
}
__device__ __forceinline__ void st_quad(uint8_t* base_hi, uint8_t* base_lo, uint32_t off, float4 v) {
    float4 hi, lo;
    split_tf32(v.x, hi.x, lo.x);
    split_tf32(v.y, hi.y, lo.y);
    split_tf32(v.z, hi.z, lo.z);
    split_tf32(v.w, hi.w, lo.w);
    *reinterpret_cast<float4*>(base_hi + off) = hi;
    *reinterpret_cast<float4*>(base_lo + off) = lo;
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n" ::"r"(smem_u32(b)),
                 "r"(bytes)
                 : "memory");
}
// bounded wait for the completion of the phase with the given parity; false on timeout or abort
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* abort_flag) {
    const uint32_t a = smem_u32(b);
    for (uint32_t i = 0; i < SPIN_LIMIT; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((i & 255u) == 255u && *abort_flag) return false;
    }
    return false;
}
// 2D tiled TMA load (x: innermost coordinate, a multiple of 4 floats = 16 bytes)
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}
// 1D bulk copy (16-byte aligned addresses, size a multiple of 16) completing on an mbarrier
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void mma_tf32(uint32_t dt, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
        :
        : "r"(dt), "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* b) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(b))
                 : "memory");
}
__device__ __forceinline__ cplxf ld2(const uint8_t* p) {
    const float2 v = *reinterpret_cast<const float2*>(p);
    return cplxf{v.x, v.y};
}
// FP32 -> FP64 by bit operations (exact; FP32 subnormals become signed zeros): the conversion
// instruction runs on GB300's FP64 pipe at 1/64 of the FP32 rate, integer operations do not
__device__ __forceinline__ double f2d_bits(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint64_t sgn = (uint64_t)(u & 0x80000000u) << 32;
    const uint32_t e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
    uint64_t r = sgn;
    if (e == 255u) r |= (0x7FFull << 52) | ((uint64_t)m << 29);
    else if (e != 0u) r |= ((uint64_t)(e + 896u) << 52) | ((uint64_t)m << 29);
    return __longlong_as_double((long long)r);
}
__device__ __forceinline__ cplx c2d_bits(cplxf v) { return cplx{f2d_bits(v.x), f2d_bits(v.y)}; }
// γL at a K3 index in the channel's spin combination (t: 2 FL.γt - FL.γa), FP32 copies
__device__ __forceinline__ cplxf fl_box(const cplxf* FLc, const cplxf* FLt, const cplxf* FLa, int ch, size_t i) {
    if (ch == CH_T) {
        const float2 qt = __ldg(reinterpret_cast<const float2*>(FLt + i));
        const float2 qa = __ldg(reinterpret_cast<const float2*>(FLa + i));
        return cplxf{2.f * qt.x - qa.x, 2.f * qt.y - qa.y};
    }
    const float2 qc = __ldg(reinterpret_cast<const float2*>(FLc + i));
    return cplxf{qc.x, qc.y};
}

}  // namespace

// one operand array in a TMA-mapped buffer: the buffer (map pair 2·buf, 2·buf + 1) and its first row
struct TmaOperand {
    int buf;
    int row0;
};
struct TmaSlot {
    TmaOperand A, B0, G, tA, tG, FL[2], tFL[2];
    const cplx* Pi;
    const cplx* Pi0;
    const cplx* tPi;
    const cplxf* FLc;  // epilogue γL terms (FP32 FL.K3 copies)
    const cplxf* FLt;
    const cplxf* FLa;
    const cplxf* tFLc;
    const cplxf* tFLt;
    const cplxf* tFLa;
    cplx* out;
    int flags;
    int ch;
};
// maps[2·b + 0]: N x KC column boxes, maps[2·b + 1]: CW x 2N row boxes of buffer b
struct TmaParams {
    CUtensorMap maps[8];
    TmaSlot slot[3];
    const int* blocks;
    int nblocks;
    int nslots;
    int nsin;  // input stages
};

namespace {

__host__ __device__ inline int stage_tiles(int mode) { return mode == 0 ? 2 : (mode == 1 ? 6 : 8); }
// a stage: the tiles, then the chunk's Π, Π0, dΠ (CW FP64 complex each, 128 B apart), then their FP32
// forms written by the converter warp (3 CW FP32 complex); 640 B reserved
constexpr int PI_F32 = 3 * CW * 16;  // offset of the FP32 forms in the Π area
__host__ __device__ inline size_t stage_bytes(int mode, int N) { return (size_t)stage_tiles(mode) * 64 * N + 640; }
__host__ __device__ inline size_t opbuf_bytes(int N) { return 2 * (size_t)A_OP + 2 * (size_t)(2 * N) * KC * 4; }

template <int MODE>
__global__ void __launch_bounds__(Roles<MODE>::THREADS, 1) k_bse_K3_tma(const __grid_constant__ TmaParams p, Dims d, int* err) {
    constexpr int N_FORM = Roles<MODE>::N_FORM, N_EPI = Roles<MODE>::N_EPI, W_EPI0 = Roles<MODE>::W_EPI0;
    constexpr int W_CONV = Roles<MODE>::W_CONV, EPI_PER_Q = Roles<MODE>::EPI_PER_Q, FORMERS = Roles<MODE>::FORMERS;
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ __align__(8) uint64_t full[MAX_IN], empty[MAX_IN], ready[MAX_IN], opready[NS_OP], opfree[NS_OP], tfull[2],
        tfree[2], finbar;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_flag;
    __shared__ __align__(16) float epi_tile[MAX_EPI * 32 * TP];  // the epilogue warps' transpose tiles
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = d.N3n, NN = 2 * N;
    const int nchunks = N / CW;
    const int nck = (MODE == 2 ? 2 : 1) * nchunks;
    const int TILE = 64 * N;
    const size_t STG = stage_bytes(MODE, N);
    const int NS_IN = p.nsin;
    uint8_t* in_base = sm;
    uint8_t* op_base = sm + NS_IN * STG;
    const int OPB = 2 * N * KC * 4;
    const int nitems = p.nslots * p.nblocks;

    if (tid == 0) {
        abort_flag = 0;
        for (int i = 0; i < NS_IN; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], N_FORM); mbar_init(&ready[i], 1); }
        for (int i = 0; i < NS_OP; ++i) { mbar_init(&opready[i], N_FORM); mbar_init(&opfree[i], 1); }
        for (int i = 0; i < 2; ++i) { mbar_init(&tfull[i], 1); mbar_init(&tfree[i], N_EPI); }
        mbar_init(&finbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == W_MMA) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&tmem_base))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    auto fail = [&]() {
        if (!abort_flag) {
            abort_flag = 1;
            atomicExch(err, 1);
        }
    };

    if (warp == W_PROD) {
        // ---------------- producer ----------------
        if (lane == 0) {
            uint32_t g = 0;
            int last_parity[MAX_IN];
            for (int s = 0; s < MAX_IN; ++s) last_parity[s] = -1;
            for (int item = blockIdx.x; item < nitems && !abort_flag; item += gridDim.x) {
                const TmaSlot& sl = p.slot[item / p.nblocks];
                const int bi = item % p.nblocks;
                const int blk = p.blocks ? p.blocks[bi] : bi;
                const int m = blk % d.N3O - (d.n3O - 1), P = blk / d.N3O;
                const int rb = blk * N;  // the block's first row in every operand array
                const int ch = sl.ch;
                const bool oneloop = (sl.flags & K3F_1LOOP) != 0;
                const int nfl = (ch == CH_T) ? 2 : 1;
                bool ok = true;
                for (int ck = 0; ck < nck; ++ck) {
                    const bool h1 = (MODE == 2 && ck >= nchunks);
                    const int w0 = CW * (h1 ? ck - nchunks : ck);
                    const int s = g % NS_IN;
                    if (g >= NS_IN && !mbar_wait(&empty[s], ((g / NS_IN) - 1) & 1, &abort_flag)) { ok = false; break; }
                    int ntiles = 2;
                    if (MODE >= 1 && !oneloop) ntiles += 1 + nfl + (h1 ? 1 + nfl : 0);
                    // the chunk's bubble factors: CW consecutive ω of the (P, Ω) row, 128 B each
                    const size_t ip = ixPi(d, P, m, w0 - d.n3n);
                    const int npi = (MODE >= 1 ? 1 : 0) + (sl.Pi0 ? 1 : 0) + (MODE == 2 ? 1 : 0);
                    mbar_expect_tx(&full[s], (uint32_t)(ntiles * TILE + npi * CW * 16));
                    last_parity[s] = (int)((g / NS_IN) & 1);
                    uint8_t* st = in_base + (size_t)s * STG;
                    uint8_t* pa = st + (size_t)stage_tiles(MODE) * TILE;
                    if (MODE >= 1) bulk_load(pa, sl.Pi + ip, CW * 16, &full[s]);
                    if (sl.Pi0) bulk_load(pa + CW * 16, sl.Pi0 + ip, CW * 16, &full[s]);
                    if (MODE == 2) bulk_load(pa + 2 * CW * 16, sl.tPi + ip, CW * 16, &full[s]);
                    const TmaOperand& A = (MODE == 2 && !h1) ? sl.tA : sl.A;
                    tma_load_2d(st + T_A * TILE, &p.maps[2 * A.buf], 2 * w0, A.row0 + rb, &full[s]);
                    tma_load_2d(st + T_B0 * TILE, &p.maps[2 * sl.B0.buf + 1], 0, sl.B0.row0 + rb + w0, &full[s]);
                    if (MODE >= 1 && !oneloop) {
                        if (ch == CH_P) tma_load_2d(st + T_G * TILE, &p.maps[2 * sl.G.buf + 1], 0, sl.G.row0 + rb + w0, &full[s]);
                        else tma_load_2d(st + T_G * TILE, &p.maps[2 * sl.G.buf], 2 * w0, sl.G.row0 + rb, &full[s]);
                        // FL at the crossed frequency ω̃ (p: rows m-ω-1 + n3n, descending; a, t: rows ω)
                        const int r0 = (ch == CH_P) ? m - (w0 + CW - 1) + N - 1 : w0;
                        for (int f = 0; f < nfl; ++f)
                            tma_load_2d(st + (T_FL0 + f) * TILE, &p.maps[2 * sl.FL[f].buf + 1], 0, sl.FL[f].row0 + rb + r0,
                                        &full[s]);
                        if (h1) {
                            if (ch == CH_P)
                                tma_load_2d(st + T_TG * TILE, &p.maps[2 * sl.tG.buf + 1], 0, sl.tG.row0 + rb + w0, &full[s]);
                            else tma_load_2d(st + T_TG * TILE, &p.maps[2 * sl.tG.buf], 2 * w0, sl.tG.row0 + rb, &full[s]);
                            for (int f = 0; f < nfl; ++f)
                                tma_load_2d(st + (T_TFL0 + f) * TILE, &p.maps[2 * sl.tFL[f].buf + 1], 0,
                                            sl.tFL[f].row0 + rb + r0, &full[s]);
                        }
                    }
                    ++g;
                }
                if (!ok) { fail(); break; }
            }
            // loads still in flight after an abort land before the CTA exits
            if (abort_flag)
                for (int s = 0; s < NS_IN; ++s)
                    if (last_parity[s] >= 0) {
                        volatile int never = 0;
                        mbar_wait(&full[s], (uint32_t)last_parity[s], &never);
                    }
        }
    } else if (warp == W_MMA) {
        // ---------------- MMA issue ----------------
        if (lane == 0) {
            const uint32_t idesc =
                (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NN >> 3) << 17) | ((128u >> 4) << 24);
            uint32_t g = 0;
            int li = 0;
            for (int item = blockIdx.x; item < nitems && !abort_flag; item += gridDim.x, ++li) {
                const int t = li & 1;
                if (li >= 2 && !mbar_wait(&tfree[t], ((li >> 1) - 1) & 1, &abort_flag)) { fail(); break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t dt = tmem + (uint32_t)(t * 256);
                bool ok = true;
                for (int ck = 0; ck < nck; ++ck) {
                    const int o = g % NS_OP;
                    if (!mbar_wait(&opready[o], (g / NS_OP) & 1, &abort_flag)) { ok = false; break; }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    uint8_t* ob = op_base + (size_t)o * opbuf_bytes(N);
                    const uint32_t ah = smem_u32(ob), al = ah + A_OP, bh = al + A_OP, bl = bh + OPB;
                    for (int ks = 0; ks < KC / 8; ++ks) {
                        const uint32_t off = (uint32_t)ks * 256u;  // 8 tf32 of K = two core matrices
                        mma_tf32(dt, sdesc(ah + off), sdesc(bh + off), idesc, (ck > 0 || ks > 0) ? 1u : 0u);
                        mma_tf32(dt, sdesc(ah + off), sdesc(bl + off), idesc, 1u);
                        mma_tf32(dt, sdesc(al + off), sdesc(bh + off), idesc, 1u);
                    }
                    mma_commit(&opfree[o]);
                    ++g;
                }
                if (!ok) { fail(); break; }
                mma_commit(&tfull[t]);
            }
            // every MMA issued here has completed before the tensor memory is released
            mma_commit(&finbar);
            volatile int never = 0;
            if (!mbar_wait(&finbar, 0, &never)) fail();
        }
    } else if (warp < W_EPI0) {
        // ---------------- formers ----------------
        const int ft = tid - 32 * W_FORM0;
        uint32_t g = 0;
        for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
            if (abort_flag) break;
            const TmaSlot& sl = p.slot[item / p.nblocks];
            const int bi = item % p.nblocks;
            const int blk = p.blocks ? p.blocks[bi] : bi;
            const int m = blk % d.N3O - (d.n3O - 1);
            const int ch = sl.ch;
            const float s1 = (ch == CH_A) ? 1.f : -1.f, s2 = (ch == CH_T) ? -1.f : 1.f;
            const bool has_pi0 = sl.Pi0 != nullptr;
            const bool oneloop = (sl.flags & K3F_1LOOP) != 0;
            bool ok = true;
            for (int ck = 0; ck < nck; ++ck) {
                const bool h1 = (MODE == 2 && ck >= nchunks);
                const int w0 = CW * (h1 ? ck - nchunks : ck);
                const int s = g % NS_IN, o = g % NS_OP;
                if (!mbar_wait(&full[s], (g / NS_IN) & 1, &abort_flag)) { ok = false; break; }
                if (!mbar_wait(&ready[s], (g / NS_IN) & 1, &abort_flag)) { ok = false; break; }
                if (g >= NS_OP && !mbar_wait(&opfree[o], ((g / NS_OP) - 1) & 1, &abort_flag)) { ok = false; break; }
                const uint8_t* st = in_base + (size_t)s * STG;
                const cplxf* pf = reinterpret_cast<const cplxf*>(st + (size_t)stage_tiles(MODE) * TILE + PI_F32);
                uint8_t* ob = op_base + (size_t)o * opbuf_bytes(N);
                uint8_t* Ahi = ob;
                uint8_t* Alo = ob + A_OP;
                uint8_t* Bhi = ob + 2 * A_OP;
                uint8_t* Blo = Bhi + OPB;
                // A: rows ν < N (rows ≥ N of the 128-lane operand are never read back), K = [Re, Im] pairs
                for (int e = ft; e < 4 * N; e += FORMERS) {  // A items (row r, K quad j), rows fastest
                    const int r = e % N, j = e / N;
                    const float4 v = *reinterpret_cast<const float4*>(st + T_A * TILE + (size_t)(r * KC + 4 * j) * 4);
                    st_quad(Ahi, Alo, op_off(r, 4 * j), v);
                }
                // B: (ω pair j, ν') items, ν' fastest; rows 2ν' and 2ν'+1 of the real form, k = 4j..4j+3:
                // [Re M(ω), −Im M(ω), Re M(ω+1), −Im M(ω+1)] and [Im M(ω), Re M(ω), Im M(ω+1), Re M(ω+1)]
                for (int e = ft; e < 4 * N; e += FORMERS) {  // B items (column ν', ω pair j), columns fastest
                    const int col = e % N, j = e / N;
                    cplxf M2[2];
#pragma unroll
                    for (int h2 = 0; h2 < 2; ++h2) {
                        const int wl = 2 * j + h2, w = w0 + wl;
                        const cplxf pi0 = has_pi0 ? pf[CW + wl] : cplxf{0.f, 0.f};
                        const cplxf f0 = ld2(st + T_B0 * TILE + (size_t)(wl * NN + 2 * col) * 4);
                        cplxf M{0.f, 0.f};
                        if (MODE == 0) {
                            M = pi0 * f0;
                        } else {
                            const cplxf pi = pf[wl];
                            if (oneloop) {
                                M = ((pi - pi0) * f0) * s1;
                            } else {
                                // Γ at (ω, ν') (p: row tile) or (ν', ω) (a, t: column tile)
                                const size_t og = (ch == CH_P) ? (size_t)(wl * NN + 2 * col) * 4 : (size_t)(col * KC + 2 * wl) * 4;
                                const cplxf gs = ld2(st + T_G * TILE + og);
                                const int ot = cross(ch, m, w - d.n3n);
                                const bool inb = fin(ot, d.n3n);
                                const int rl = (ch == CH_P) ? (CW - 1 - wl) : wl;  // row of FL(ω̃, ·) in the tile
                                const size_t ofl = (size_t)(rl * NN + 2 * col) * 4;
                                cplxf fl{0.f, 0.f};
                                if (inb) {
                                    if (ch == CH_T) {
                                        const cplxf a0 = ld2(st + T_FL0 * TILE + ofl), a1 = ld2(st + T_FL1 * TILE + ofl);
                                        fl = cplxf{2.f * a0.x - a1.x, 2.f * a0.y - a1.y};
                                    } else {
                                        fl = ld2(st + T_FL0 * TILE + ofl);
                                    }
                                }
                                if (!h1) {  // s1 [(Π-Π0) F0 + Π Γ] + s2 Π γL
                                    M = ((pi - pi0) * f0 + pi * gs) * s1;
                                    if (inb) M += pi * fl * s2;
                                } else {  // dM = s1 [dΠ (F0 + Γ) + Π dΓ] + s2 [dΠ γL + Π dγL]
                                    const cplxf tpi = pf[2 * CW + wl];
                                    const cplxf tg = ld2(st + T_TG * TILE + og);
                                    M = (tpi * (f0 + gs) + pi * tg) * s1;
                                    if (inb) {
                                        cplxf tfl;
                                        if (ch == CH_T) {
                                            const cplxf a0 = ld2(st + T_TFL0 * TILE + ofl), a1 = ld2(st + T_TFL1 * TILE + ofl);
                                            tfl = cplxf{2.f * a0.x - a1.x, 2.f * a0.y - a1.y};
                                        } else {
                                            tfl = ld2(st + T_TFL0 * TILE + ofl);
                                        }
                                        M += (tpi * fl + pi * tfl) * s2;
                                    }
                                }
                            }
                        }
                        M2[h2] = M;
                    }
                    st_quad(Bhi, Blo, op_off(2 * col, 4 * j), make_float4(M2[0].x, -M2[0].y, M2[1].x, -M2[1].y));
                    st_quad(Bhi, Blo, op_off(2 * col + 1, 4 * j), make_float4(M2[0].y, M2[0].x, M2[1].y, M2[1].x));
                }
                // generic-proxy writes -> visible to the tensor core (async proxy)
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) {
                    mbar_arrive(&opready[o]);
                    mbar_arrive(&empty[s]);
                }
                ++g;
            }
            if (!ok) { fail(); break; }
        }
    } else if (warp < W_CONV) {
        // ---------------- epilogue ----------------
        // TMEM lane quadrant q holds rows 32q..32q+31; its EPI_PER_Q warps take alternate groups of 16
        // accumulator columns (8 complex outputs).  Each group is transposed through the warp's tile so
        // that a warp reads FL and writes the FP64 outputs as 4 contiguous row segments per instruction.
        const int q = warp & 3, sub = (warp - W_EPI0) >> 2;
        float* tile = epi_tile + (warp - W_EPI0) * 32 * TP;
        const float Tf = (float)d.T;
        int li = 0;
        for (int item = blockIdx.x; item < nitems; item += gridDim.x, ++li) {
            if (abort_flag) break;
            const TmaSlot& sl = p.slot[item / p.nblocks];
            const int bi = item % p.nblocks;
            const int blk = p.blocks ? p.blocks[bi] : bi;
            const size_t base = (size_t)blk * N * N;
            const int ch = sl.ch;
            const float sgn = (ch == CH_A) ? 1.f : -1.f;
            const bool epi = MODE >= 1 && !(sl.flags & K3F_NOEPI);
            const bool acc = (sl.flags & K3F_ACC) != 0;
            const int t = li & 1;
            if (!mbar_wait(&tfull[t], (li >> 1) & 1, &abort_flag)) { fail(); break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (32 * q < N) {  // (a quadrant beyond the block's rows has nothing to store)
                for (int c0 = 16 * sub; c0 < NN; c0 += 16 * EPI_PER_Q) {
                    uint32_t r[16];
                    const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(t * 256 + c0);
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                        "[%16];"
                        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                          "=r"(r[14]), "=r"(r[15])
                        : "r"(taddr)
                        : "memory");
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                    for (int k = 0; k < 16; ++k) tile[lane * TP + k] = __uint_as_float(r[k]);
                    __syncwarp();
                    const int cc = lane & 7;  // complex column within the group
                    // the γL terms of all 8 passes are loaded before any is used (one load latency per group)
                    cplxf gl[8];
#pragma unroll
                    for (int pass = 0; pass < 8; ++pass) {
                        const int row = 32 * q + pass * 4 + (lane >> 3);
                        const size_t io = base + (size_t)row * N + c0 / 2 + cc;
                        gl[pass] = cplxf{0.f, 0.f};
                        if (epi && row < N)
                            gl[pass] = MODE == 1 ? fl_box(sl.FLc, sl.FLt, sl.FLa, ch, io)
                                                 : fl_box(sl.tFLc, sl.tFLt, sl.tFLa, ch, io);
                    }
                    // the accumulating form (an FP64 read-modify-write) is a separate loop, so that the
                    // plain stores carry no FP64 add the compiler might evaluate ahead of the select
                    if (!acc) {
                        // independent batches (tile loads, arithmetic, stores) keep the 8 passes in flight together
                        float2 dv[8];
#pragma unroll
                        for (int pass = 0; pass < 8; ++pass)
                            dv[pass] = *reinterpret_cast<const float2*>(tile + (pass * 4 + (lane >> 3)) * TP + 2 * cc);
                        double2 o[8];
#pragma unroll
                        for (int pass = 0; pass < 8; ++pass) {
                            const cplxf v{dv[pass].x, dv[pass].y};
                            const cplxf f = (MODE == 0) ? v * (Tf * sgn) : v * Tf + gl[pass];
                            o[pass] = make_double2(f2d_bits(f.x), f2d_bits(f.y));
                        }
                        double2* dst = reinterpret_cast<double2*>(sl.out + base) + (size_t)(32 * q + (lane >> 3)) * N + c0 / 2 + cc;
#pragma unroll
                        for (int pass = 0; pass < 8; ++pass)
                            if (32 * q + pass * 4 + (lane >> 3) < N) dst[(size_t)pass * 4 * N] = o[pass];
                    } else {
                        for (int pass = 0; pass < 8; ++pass) {
                            const int rr = pass * 4 + (lane >> 3);
                            const int row = 32 * q + rr;
                            if (row < N) {
                                const float2 dv = *reinterpret_cast<const float2*>(tile + rr * TP + 2 * cc);
                                const cplxf v{dv.x, dv.y};
                                const cplxf f = (MODE == 0) ? v * (Tf * sgn) : v * Tf + gl[pass];
                                const size_t io = base + (size_t)row * N + c0 / 2 + cc;
                                sl.out[io] = sl.out[io] + c2d_bits(f);
                            }
                        }
                    }
                    __syncwarp();
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&tfree[t]);
        }
    } else {
        // ---------------- converter: the chunk's Π, Π0, dΠ to FP32, once per stage use ----------------
        uint32_t g = 0;
        for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
            if (abort_flag) break;
            bool ok = true;
            for (int ck = 0; ck < nck; ++ck) {
                const int s = g % NS_IN;
                if (!mbar_wait(&full[s], (g / NS_IN) & 1, &abort_flag)) { ok = false; break; }
                uint8_t* pbase = in_base + (size_t)s * STG + (size_t)stage_tiles(MODE) * TILE;
                if (lane < 3 * CW) {
                    const cplx v = reinterpret_cast<const cplx*>(pbase)[lane];
                    reinterpret_cast<cplxf*>(pbase + PI_F32)[lane] = to_f32(v);
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(&ready[s]);
                ++g;
            }
            if (!ok) { fail(); break; }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == W_MMA)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

// shared-memory limit records of the three instantiations (per device)
SmemRecord g_raised[3];

// input stages that fit beside the operand buffers (0: the box does not fit)
int tma_stages(int mode, int N) {
    const size_t ops = NS_OP * opbuf_bytes(N);
    if (ops >= SMEM_BUDGET) return 0;
    size_t n = (SMEM_BUDGET - ops) / stage_bytes(mode, N);
    if (n > (size_t)MAX_IN) n = MAX_IN;
    return n >= 2 ? (int)n : 0;
}
size_t tma_smem(int mode, int N) {
    const size_t need = tma_stages(mode, N) * stage_bytes(mode, N) + NS_OP * opbuf_bytes(N);
    return need < MIN_SMEM ? MIN_SMEM : need;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    });
    return fn;
}

// the two box shapes over buffer b (rows of 2N floats): N rows x KC floats, and CW rows x 2N floats
bool encode_pair(CUtensorMap* m, const void* base, size_t ncplx, int N) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t rows = ncplx / N;
    const cuuint64_t dims[2] = {(cuuint64_t)(2 * N), rows};
    const cuuint64_t strides[1] = {(cuuint64_t)(8 * N)};
    const cuuint32_t es[2] = {1, 1};
    const cuuint32_t boxc[2] = {(cuuint32_t)KC, (cuuint32_t)N};
    const cuuint32_t boxr[2] = {(cuuint32_t)(2 * N), (cuuint32_t)CW};
    void* g = const_cast<void*>(base);
    if (fn(&m[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, g, dims, strides, boxc, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
        CUDA_SUCCESS)
        return false;
    return fn(&m[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, g, dims, strides, boxr, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

}  // namespace

bool k3_tma_supported(const Dims& d, int mode) {
    if (!(d.N3n >= 32 && d.N3n <= 128 && (d.N3n % 8) == 0)) return false;
    if (!encode_fn()) return false;
    return tma_stages(mode, d.N3n) >= 2;
}

cudaError_t launch_bse_K3_tma(cudaStream_t s, int mode, const K3Args3F& a, int nslots, const Dims& d, int* err,
                              const TmaBuffers& bufs) {
    const int N = d.N3n;
    if (!k3_tma_supported(d, mode) || nslots < 1 || nslots > 3 || a.nblocks < 1) return cudaErrorInvalidValue;
    TmaParams p;
    std::memset(&p, 0, sizeof(p));
    for (int b = 0; b < 4; ++b)
        if (bufs.base[b] && !encode_pair(&p.maps[2 * b], bufs.base[b], bufs.ncplx[b], N)) return cudaErrorInvalidValue;
    // an operand pointer -> (buffer, first row); every operand array starts at a whole row
    bool bad = false;
    auto locate = [&](const cplxf* ptr) -> TmaOperand {
        TmaOperand o{0, 0};
        if (!ptr) { bad = true; return o; }
        for (int b = 0; b < 4; ++b) {
            const cplxf* base = static_cast<const cplxf*>(bufs.base[b]);
            if (base && ptr >= base && ptr < base + bufs.ncplx[b]) {
                const size_t off = (size_t)(ptr - base);
                if (off % N) bad = true;
                o.buf = b;
                o.row0 = (int)(off / N);
                return o;
            }
        }
        bad = true;
        return o;
    };
    for (int i = 0; i < nslots; ++i) {
        const K3ArgsF& x = a.a[i];
        TmaSlot& sl = p.slot[i];
        sl.ch = a.ch[i];
        sl.flags = x.flags;
        sl.A = locate(x.A);
        sl.B0 = locate(x.B0);
        sl.Pi = x.Pi; sl.Pi0 = x.Pi0; sl.tPi = x.tPi;
        sl.out = x.out;
        sl.FLc = x.FLc; sl.FLt = x.FLt; sl.FLa = x.FLa;
        sl.tFLc = x.tFLc; sl.tFLt = x.tFLt; sl.tFLa = x.tFLa;
        if (mode >= 1 && !(x.flags & K3F_1LOOP)) {
            sl.G = locate(x.G);
            if (sl.ch == CH_T) { sl.FL[0] = locate(x.FLt); sl.FL[1] = locate(x.FLa); }
            else sl.FL[0] = locate(x.FLc);
        }
        if (mode == 2) {
            sl.tA = locate(x.tA);
            sl.tG = locate(x.tG);
            if (sl.ch == CH_T) { sl.tFL[0] = locate(x.tFLt); sl.tFL[1] = locate(x.tFLa); }
            else sl.tFL[0] = locate(x.tFLc);
        }
        if ((mode >= 1 && !x.Pi) || (mode == 2 && !x.tPi) || !x.out) bad = true;
    }
    if (bad) return cudaErrorInvalidValue;
    p.blocks = a.blocks;
    p.nblocks = a.nblocks;
    p.nslots = nslots;
    p.nsin = tma_stages(mode, N);
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const size_t smem = tma_smem(mode, N);
    e = mode == 0 ? raise_smem_limit(k_bse_K3_tma<0>, g_raised[0], smem, 0)
                  : (mode == 1 ? raise_smem_limit(k_bse_K3_tma<1>, g_raised[1], smem, 0)
                               : raise_smem_limit(k_bse_K3_tma<2>, g_raised[2], smem, 0));
    if (e != cudaSuccess) return e;
    const int nitems = nslots * a.nblocks;
    const unsigned grid = (unsigned)(nitems < nsm ? nitems : nsm);
    if (mode == 0) k_bse_K3_tma<0><<<grid, Roles<0>::THREADS, smem, s>>>(p, d, err);
    else if (mode == 1) k_bse_K3_tma<1><<<grid, Roles<1>::THREADS, smem, s>>>(p, d, err);
    else k_bse_K3_tma<2><<<grid, Roles<2>::THREADS, smem, s>>>(p, d, err);
    return cudaGetLastError();
}

cudaError_t prepare_bse_K3_tma(const Dims& d) {
    // the shared-memory limits are raised before any graph capture (the launch then finds them raised)
    cudaError_t e = cudaSuccess;
    if (k3_tma_supported(d, 0)) e = raise_smem_limit(k_bse_K3_tma<0>, g_raised[0], tma_smem(0, d.N3n), 0);
    if (e == cudaSuccess && k3_tma_supported(d, 1)) e = raise_smem_limit(k_bse_K3_tma<1>, g_raised[1], tma_smem(1, d.N3n), 0);
    if (e == cudaSuccess && k3_tma_supported(d, 2)) e = raise_smem_limit(k_bse_K3_tma<2>, g_raised[2], tma_smem(2, d.N3n), 0);
    return e;
}

}  // namespace fdga
