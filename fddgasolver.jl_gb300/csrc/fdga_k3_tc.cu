// fdga_k3_tc.cu -- the K3 Bethe-Salpeter contractions of the mixed map on the 5th-generation
// tensor cores (tcgen05, sm_103a).
//
// Per (channel, representative (P, Ω) block) the BSE is one complex product C = A·M of Nν3 x Nν3
// matrices (src/BSEa/BSEa_K3.jl:1-128; M formed elementwise from the caches, Π, Π0 and FL).  It
// runs as one real GEMM D[128 x 2N] += A_r[128 x 2N'] · B_r[2N' x 2N] with the complex product in
// 2x2 real form (k = 2ω + q, n = 2ν' + p):
//   A_r[ν][2ω] = Re A(ν,ω), A_r[ν][2ω+1] = Im A(ν,ω)
//   B_r[2ω][2ν'] = Re M, B_r[2ω][2ν'+1] = Im M, B_r[2ω+1][2ν'] = −Im M, B_r[2ω+1][2ν'+1] = Re M
// so that D[ν][2ν'] = Re C(ν,ν') and D[ν][2ν'+1] = Im C(ν,ν').  Operands are FP32 (the mixed map's
// FP32 caches); each is split into TF32 hi + lo and the product accumulates hi·hi + hi·lo + lo·hi
// (kind::tf32, FP32 accumulation in tensor memory), which keeps FP32-level accuracy.
//
// Mode 2 (the tangent of the K3 BSE, dC = dA·M + A·dM) is one GEMM over the concatenated inner
// index: the chunks first stage (dA, M), then (A, dM), into the same accumulator.
//
// One CTA of 512 threads per block: rows ν < N of the 128-lane accumulator, 2N ≤ 256 columns.
// K runs in chunks of CW ω (2·CW real k); two shared-memory stages; the threads stage chunk c+1
// while the tensor core works on chunk c (tcgen05.commit -> mbarrier).  Shared-memory operands use
// the no-swizzle K-major canonical layout: 8-row x 16-byte core matrices, K-adjacent core
// matrices 128 B apart (LBO), 8-row groups KC·32 = 512 B apart (SBO).  Every wait is bounded; a timeout
// sets *err and the kernel still releases its tensor memory.
#include "fdga_kernels.h"

namespace fdga {

namespace {

constexpr int TC_THREADS = 512;  // 16 warps stage the operands; warps 4q..4q+3 read TMEM lanes 32q..
constexpr int KC = 16;                      // real K per chunk
constexpr int CW = KC / 2;                  // ω per chunk
constexpr int A_BYTES = 128 * KC * 4;       // one A operand (hi or lo) of a chunk: 8 KB
// (a chunk of 8 ω keeps a CTA under 113 KB of shared memory, so two CTAs share an SM and hide
// each other's operand-staging latency; two CTAs use all 512 TMEM columns)
constexpr uint32_t SPIN_LIMIT = 1u << 22;   // bounded mbarrier polling

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
// byte offset of element (row r, k) in a K-major no-swizzle operand with KC columns of K
__device__ __forceinline__ uint32_t op_off(int r, int k) {
    return (uint32_t)((((r >> 3) * (KC / 4) + (k >> 2)) << 7) + ((r & 7) << 4) + ((k & 3) << 2));
}
// shared-memory matrix descriptor: start, LBO = 128 B, SBO = KC·32 B, fixed 0b001 at bits 46-48,
// no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)((KC * 32) >> 4) << 32) |
           (1ull << 46);
}
__device__ __forceinline__ void split_tf32(float v, float& hi, float& lo) {
    hi = __uint_as_float(__float_as_uint(v) & 0xFFFFE000u);
    lo = v - hi;
}
// four consecutive k of one row (16 bytes, 16-byte aligned): TF32 hi and lo parts
__device__ __forceinline__ void st_quad(uint8_t* base_hi, uint8_t* base_lo, uint32_t off, float4 v) {
    float4 hi, lo;
    split_tf32(v.x, hi.x, lo.x);
    split_tf32(v.y, hi.y, lo.y);
    split_tf32(v.z, hi.z, lo.z);
    split_tf32(v.w, hi.w, lo.w);
    *reinterpret_cast<float4*>(base_hi + off) = hi;
    *reinterpret_cast<float4*>(base_lo + off) = lo;
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
// γL at a K3 index: FL.γ_ch (a, p) or 2 FL.γt − FL.γa (t, density component)
__device__ __forceinline__ cplxf fl_box(const cplxf* FLc, const cplxf* FLt, const cplxf* FLa, int ch, size_t i) {
    if (ch == CH_T) {
        const float2 qt = __ldg(reinterpret_cast<const float2*>(FLt + i));
        const float2 qa = __ldg(reinterpret_cast<const float2*>(FLa + i));
        return cplxf{2.f * qt.x - qa.x, 2.f * qt.y - qa.y};
    }
    const float2 qc = __ldg(reinterpret_cast<const float2*>(FLc + i));
    return cplxf{qc.x, qc.y};
}
__device__ __forceinline__ void mma_tf32(uint32_t dt, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
        :
        : "r"(dt), "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

template <int MODE>
__global__ void __launch_bounds__(TC_THREADS, 2) k_bse_K3_tc(K3Args3F args, Dims d, int* err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ uint64_t mbar[2];
    __shared__ uint32_t tmem_base;
    __shared__ float pis[128][6];  // Π(ω), Π0(ω), dΠ(ω) of the block (re, im pairs), loaded once
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int N = d.N3n, NN = 2 * N;
    const int nchunks = (N + CW - 1) / CW;
    const int nck = (MODE == 2 ? 2 : 1) * nchunks;  // mode 2: (dA, M) chunks, then (A, dM) chunks
    const int nb = args.nblocks;
    const int slot = blockIdx.x / nb;
    const int blk = args.blocks ? args.blocks[blockIdx.x % nb] : (int)(blockIdx.x % nb);
    const K3ArgsF& a = args.a[slot];
    const int CH = args.ch[slot];
    const int m = blk % d.N3O - (d.n3O - 1), P = blk / d.N3O;
    const size_t base = (size_t)blk * N * N;
    const float s1 = (CH == CH_A) ? 1.f : -1.f, s2 = (CH == CH_T) ? -1.f : 1.f;
    const int B_BYTES = NN * KC * 4;
    const int STAGE = 2 * A_BYTES + 2 * B_BYTES;
    // tensor memory: 256 columns (2N ≤ 256)
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(&tmem_base))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid < N) {
        float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const size_t ip = ixPi(d, P, m, tid - d.n3n);
        const cplx p0 = a.Pi0 ? ldg(a.Pi0 + ip) : mk(0.0, 0.0);
        v[2] = d2f_rn(p0.x); v[3] = d2f_rn(p0.y);
        if (MODE >= 1) { const cplx p = ldg(a.Pi + ip); v[0] = d2f_rn(p.x); v[1] = d2f_rn(p.y); }
        if (MODE == 2) { const cplx p = ldg(a.tPi + ip); v[4] = d2f_rn(p.x); v[5] = d2f_rn(p.y); }
        for (int j = 0; j < 6; ++j) pis[tid][j] = v[j];
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NN >> 3) << 17) | ((128u >> 4) << 24);
    bool ok = true;
    for (int c = 0; c < nck; ++c) {
        const int st = c & 1;
        const bool tM = (MODE == 2 && c >= nchunks);
        const cplxf* Ap = (MODE == 2 && !tM) ? a.tA : a.A;
        if (c >= 2 && !mbar_wait(smem_u32(&mbar[st]), ((c - 2) >> 1) & 1)) ok = false;
        uint8_t* Ahi = sm + (size_t)st * STAGE;
        uint8_t* Alo = Ahi + A_BYTES;
        uint8_t* Bhi = Alo + A_BYTES;
        uint8_t* Blo = Bhi + B_BYTES;
        const int w0 = CW * (tM ? c - nchunks : c);
        // A: (ω pair j, row ν) items, rows fastest so that a quarter warp's 16-byte stores fall in
        // distinct banks; k = 4j..4j+3 holds [Re A(ω), Im A(ω), Re A(ω+1), Im A(ω+1)]
        for (int e = tid; e < 128 * (KC / 4); e += TC_THREADS) {
            const int nu = e & 127, j = e >> 7, w = w0 + 2 * j;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (nu < N && w < N) {
                const float2 q0 = __ldg(reinterpret_cast<const float2*>(Ap + base + (size_t)nu * N + w));
                v.x = q0.x; v.y = q0.y;
                if (w + 1 < N) {
                    const float2 q1 = __ldg(reinterpret_cast<const float2*>(Ap + base + (size_t)nu * N + w + 1));
                    v.z = q1.x; v.w = q1.y;
                }
            }
            st_quad(Ahi, Alo, op_off(nu, 4 * j), v);
        }
        // B: (ω pair j, ν') items, ν' fastest (coalesced loads of the cache rows); rows 2ν' and
        // 2ν'+1 of the real form, k = 4j..4j+3: [Re M(ω), −Im M(ω), Re M(ω+1), −Im M(ω+1)] and
        // [Im M(ω), Re M(ω), Im M(ω+1), Re M(ω+1)]
        for (int e = tid; e < (KC / 4) * N; e += TC_THREADS) {
            const int j = e / N, col = e % N;
            cplxf M2[2];
            for (int h2 = 0; h2 < 2; ++h2) {
                const int t = 2 * j + h2, w = w0 + t;
                cplxf M{0.f, 0.f};
                if (w < N) {
                    const cplxf pi0{pis[w][2], pis[w][3]};
                    const float2 q0 = __ldg(reinterpret_cast<const float2*>(a.B0 + base + (size_t)w * N + col));
                    const cplxf f0{q0.x, q0.y};
                    if (MODE == 0) {
                        M = pi0 * f0;
                    } else {
                        const cplxf pi{pis[w][0], pis[w][1]};
                        const size_t ig = (CH == CH_P) ? base + (size_t)w * N + col : base + (size_t)col * N + w;
                        const int ot = cross(CH, m, w - d.n3n);
                        const size_t il = base + (size_t)(ot + d.n3n) * N + col;
                        cplxf gs{0.f, 0.f};
                        if (!(a.flags & K3F_1LOOP)) {
                            const float2 qg = __ldg(reinterpret_cast<const float2*>(a.G + ig));
                            gs = cplxf{qg.x, qg.y};
                        }
                        if (a.flags & K3F_1LOOP) {
                            M = ((pi - pi0) * f0) * s1;
                        } else if (!tM) {
                            M = ((pi - pi0) * f0 + pi * gs) * s1;
                            if (fin(ot, d.n3n)) M += pi * fl_box(a.FLc, a.FLt, a.FLa, CH, il) * s2;
                        } else {  // dM = s1 [dΠ (F0 + Γ) + Π dΓ] + s2 [dΠ γL + Π dγL]
                            const cplxf tpi{pis[w][4], pis[w][5]};
                            const float2 qt = __ldg(reinterpret_cast<const float2*>(a.tG + ig));
                            M = (tpi * (f0 + gs) + pi * cplxf{qt.x, qt.y}) * s1;
                            if (fin(ot, d.n3n))
                                M += (tpi * fl_box(a.FLc, a.FLt, a.FLa, CH, il) +
                                      pi * fl_box(a.tFLc, a.tFLt, a.tFLa, CH, il)) * s2;
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
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t ah = smem_u32(Ahi), al = smem_u32(Alo), bh = smem_u32(Bhi), bl = smem_u32(Blo);
            for (int ks = 0; ks < KC / 8; ++ks) {
                const uint32_t o = (uint32_t)ks * 256u;  // 8 tf32 of K = two core matrices
                mma_tf32(tmem, sdesc(ah + o), sdesc(bh + o), idesc, (c > 0 || ks > 0) ? 1u : 0u);
                mma_tf32(tmem, sdesc(ah + o), sdesc(bl + o), idesc, 1u);
                mma_tf32(tmem, sdesc(al + o), sdesc(bh + o), idesc, 1u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&mbar[st]))
                         : "memory");
        }
        // no barrier here: the next chunk writes the other stage, and a stage is rewritten only after
        // the mbarrier reports the MMAs that read it complete
    }
    // the last chunk of each stage
    if (nck >= 2 && !mbar_wait(smem_u32(&mbar[nck & 1]), ((nck - 2) >> 1) & 1)) ok = false;
    if (!mbar_wait(smem_u32(&mbar[(nck - 1) & 1]), ((nck - 1) >> 1) & 1)) ok = false;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok) {
        // a wait gave up: report it, and give the MMAs in flight one more bounded wait before the
        // tensor memory is released (the loop went on staging, so every thread still reaches the
        // CTA barriers; the results are discarded with the error)
        if (tid == 0) atomicExch(err, 1);
        mbar_wait(smem_u32(&mbar[(nck - 1) & 1]), ((nck - 1) >> 1) & 1);
    } else {
        // epilogue: warp w reads lanes 32(w%4).. (rows ν), every 4th group of 16 columns from 16(w/4)
        const int q = warp & 3, grp = warp >> 2;
        const int nu = 32 * q + lane;
        const double T = d.T;
        for (int c0 = 16 * grp; c0 < NN; c0 += 64) {
            uint32_t r[16];
            const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(taddr)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (nu < N) {
                // epilogue in FP32 (one conversion per value at the store)
                const float Tf = (float)T, sgn = (CH == CH_A) ? 1.f : -1.f;
                for (int j = 0; j < 8; ++j) {
                    const int col = c0 / 2 + j;
                    if (col >= N) break;
                    const cplxf v{__uint_as_float(r[2 * j]), __uint_as_float(r[2 * j + 1])};
                    const size_t io = base + (size_t)nu * N + col;
                    cplx o;
                    if (MODE == 0) {
                        o = to_d(v * (Tf * sgn));
                    } else if (a.flags & K3F_NOEPI) {
                        o = to_d(v * Tf);
                    } else if (MODE == 1) {
                        o = to_d(v * Tf + fl_box(a.FLc, a.FLt, a.FLa, CH, io));
                    } else {
                        o = to_d(v * Tf + fl_box(a.tFLc, a.tFLt, a.tFLa, CH, io));
                    }
                    a.out[io] = (a.flags & K3F_ACC) ? a.out[io] + o : o;
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

bool k3_tc_supported(const Dims& d) {
    // 2N MMA columns: a multiple of 16, at most 256; the 128-lane accumulator holds N ≤ 128 rows
    return d.N3n >= 32 && d.N3n <= 128 && (d.N3n % 8) == 0;
}

static size_t k3_tc_smem(const Dims& d) { return 2 * ((size_t)2 * A_BYTES + (size_t)2 * (2 * d.N3n) * KC * 4); }

cudaError_t prepare_bse_K3_tc(const Dims& d) {
    // the dynamic shared-memory limit is raised once per size, before any graph capture
    static SmemRecord set0, set1, set2;
    const size_t smem = k3_tc_smem(d);
    cudaError_t e = raise_smem_limit(k_bse_K3_tc<0>, set0, smem, 0);  // (static shared memory too)
    if (e == cudaSuccess) e = raise_smem_limit(k_bse_K3_tc<1>, set1, smem, 0);
    if (e == cudaSuccess) e = raise_smem_limit(k_bse_K3_tc<2>, set2, smem, 0);
    return e;
}

cudaError_t launch_bse_K3_tc(cudaStream_t s, int mode, const K3Args3F& a, int nslots, const Dims& d, int* err) {
    if (!k3_tc_supported(d)) return cudaErrorInvalidValue;
    const size_t smem = k3_tc_smem(d);
    const unsigned grid = (unsigned)(nslots * a.nblocks);
    if (mode == 2) k_bse_K3_tc<2><<<grid, TC_THREADS, smem, s>>>(a, d, err);
    else if (mode) k_bse_K3_tc<1><<<grid, TC_THREADS, smem, s>>>(a, d, err);
    else k_bse_K3_tc<0><<<grid, TC_THREADS, smem, s>>>(a, d, err);
    return cudaGetLastError();
}

}  // namespace fdga
