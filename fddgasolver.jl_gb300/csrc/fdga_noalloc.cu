// fdga_noalloc.cu -- fdga_bubble_noalloc: the particle-particle / particle-hole bubbles of a Green
// function for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: a host whose own pool allocator already owns the device
// memory (a Julia CUDA.jl or PyTorch process with its memory pool in control of the HBM), or code
// on a path where cudaMalloc's implicit device synchronisation is not allowed.  Such a caller owns
// the input G and the output bubbles; the only extra device memory the bubble needs is its work
// array G(R) (the Green function on the real-space lattice), and here that work array is a
// file-scope __device__ buffer of fixed size instead of an allocation.
//
// The computation is the nonlocal real-space bubble of fdDGAsolver.jl
// (src/nonlocal/bubble.jl:87-158; for L = 1 it equals the local src/bubble.jl:9-36):
//   G(R) = (1/N) Σ_k G(k) e^{-2πi k·R/L};  Πpp(R) = G(R,Ω-ν) G(R,ν), Πph(R) = G(R,Ω+ν) G(-R,ν),
//   the R = 0 term with the 1/ν tail;  Π(P) = Σ_R Π(R) e^{+2πi P·R/L}.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/fdga.h"
#include "fdga_kernels.h"

namespace fdga_internal {
void set_create_error(const std::string& msg);  // fdga_create_error() text, fdga_runtime.cu
}

namespace {

using fdga::cplx;
using fdga::Dims;
using fdga::fin;
using fdga::mk;

// The shared work array: one instance per device; every call on that device uses (and overwrites) it.
__device__ __align__(256) cplx g_bubble_scratch[FDGA_BUBBLE_NOALLOC_MAX_ELEMS];

constexpr int kMaxL = 64;        // twiddle table size
constexpr int kMaxLattice = 56;  // largest L whose bubble tile (one frequency) fits the shared memory
struct Twiddles {
    cplx m[kMaxL];  // e^{-2πi j/L}
    cplx p[kMaxL];  // e^{+2πi j/L}
};

__device__ __forceinline__ cplx tail_or(const cplx* GR, const Dims& d, int n) {
    if (fin(n, d.nG)) return GR[n + d.nG];
    return mk(1.0 / ((2.0 * n + 1.0) * M_PI * d.T), 0.0);
}

__global__ void k_noalloc_greal(const cplx* G, cplx* GR, Twiddles tw, Dims d) {
    const int NR = d.L * d.L;
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= (size_t)NR * d.NG) return;
    const int nu = (int)(i % d.NG), R = (int)(i / d.NG);
    const int Rx = R % d.L, Ry = R / d.L;
    cplx s = mk(0, 0);
    for (int k = 0; k < NR; ++k) {
        const int kx = k % d.L, ky = k / d.L;
        s += G[(size_t)k * d.NG + nu] * tw.m[(kx * Rx + ky * Ry) % d.L];
    }
    GR[i] = s * (1.0 / NR);
}

// One CTA = one Ω and TV fermionic frequencies; output in the reference's column-major [Ω, ν, P].
__global__ void k_noalloc_bubble(const cplx* GR, cplx* pp, cplx* ph, Twiddles tw, Dims d, int TV) {
    extern __shared__ cplx sh[];
    const int L = d.L, NR = L * L;
    cplx* A = sh;
    cplx* B = sh + 2 * (size_t)TV * NR;
    const int m = blockIdx.y - (d.nPO - 1);
    const int n0 = blockIdx.x * TV - d.nPn;
    for (int e = threadIdx.x; e < TV * NR; e += blockDim.x) {
        const int v = e / NR, R = e % NR;
        const int n = n0 + v;
        cplx vpp = mk(0, 0), vph = mk(0, 0);
        if (n < d.nPn) {
            const int Rx = R % L, Ry = R / L;
            const int mR = ((L - Rx) % L) + L * ((L - Ry) % L);
            if (R == 0) {
                vpp = tail_or(GR, d, m - n - 1) * tail_or(GR, d, n);
                vph = tail_or(GR, d, m + n) * tail_or(GR, d, n);
            } else {
                const int a = m - n - 1, b = m + n;
                if (fin(a, d.nG) && fin(n, d.nG)) vpp = GR[(size_t)R * d.NG + a + d.nG] * GR[(size_t)R * d.NG + n + d.nG];
                if (fin(b, d.nG) && fin(n, d.nG)) vph = GR[(size_t)R * d.NG + b + d.nG] * GR[(size_t)mR * d.NG + n + d.nG];
            }
        }
        A[(size_t)v * NR + R] = vpp;
        A[(size_t)(TV + v) * NR + R] = vph;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 2 * TV * NR; e += blockDim.x) {
        const int row = e / NR, r = e % NR;
        const int Px = r % L, y = r / L;
        const cplx* a = A + (size_t)row * NR + (size_t)y * L;
        cplx s = mk(0, 0);
        for (int x = 0; x < L; ++x) s += a[x] * tw.p[(Px * x) % L];
        B[(size_t)row * NR + r] = s;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 2 * TV * NR; e += blockDim.x) {
        const int v = e % TV;
        const int rest = e / TV;
        const int P = rest % NR, which = rest / NR;
        const int Px = P % L, Py = P / L;
        const int n = n0 + v;
        if (n >= d.nPn) continue;
        const cplx* b = B + (size_t)(which * TV + v) * NR;
        cplx s = mk(0, 0);
        for (int y = 0; y < L; ++y) s += b[(size_t)y * L + Px] * tw.p[(Py * y) % L];
        const size_t io = (size_t)(m + d.nPO - 1) + (size_t)d.NPO * ((size_t)(n + d.nPn) + (size_t)d.NPn * P);
        (which ? ph : pp)[io] = s;
    }
}

// Device address of g_bubble_scratch, looked up once per device with that device current.
std::mutex g_mu;
void* g_addr[256] = {};

int scratch_address(cplx** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        fdga_internal::set_create_error(std::string("fdga_bubble_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return FDGA_ERR_CUDA;
    }
    if (dev < 0 || dev >= 256) {
        fdga_internal::set_create_error("fdga_bubble_noalloc: device ordinal out of range");
        return FDGA_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_bubble_scratch);
        if (e != cudaSuccess || !p) {
            fdga_internal::set_create_error(std::string("fdga_bubble_noalloc: cudaGetSymbolAddress: ") +
                                            cudaGetErrorString(e));
            return FDGA_ERR_CUDA;
        }
        g_addr[dev] = p;
    }
    *out = static_cast<cplx*>(g_addr[dev]);
    return FDGA_OK;
}

}  // namespace

extern "C" int fdga_bubble_noalloc(const fdga_config* c, const double* G, double* Pipp, double* Piph, void* stream) {
    auto bad = [](int code, const std::string& m) { fdga_internal::set_create_error("fdga_bubble_noalloc: " + m); return code; };
    if (!c || !G || !Pipp || !Piph) return bad(FDGA_ERR_ARG, "null argument");
    if (c->nG < 1 || c->nK1 < 1 || c->mPi_factor < 1 || c->L < 1 || !(c->T > 0)) return bad(FDGA_ERR_ARG, "invalid sizes");
    if (c->LG != c->L) return bad(FDGA_ERR_UNSUPPORTED, "L_G != L");
    if (c->local && c->L != 1) return bad(FDGA_ERR_ARG, "the local solver has L = 1");
    if (c->L > kMaxLattice) return bad(FDGA_ERR_ARG, "L = " + std::to_string(c->L) + " exceeds the maximum lattice size 56");
    const size_t NG = 2 * (size_t)c->nG, NR = (size_t)c->L * c->L;
    if (NG * NR > (size_t)FDGA_BUBBLE_NOALLOC_MAX_ELEMS)
        return bad(FDGA_ERR_ARG, "2nG*L*L = " + std::to_string(NG * NR) + " exceeds the work-array maximum of " +
                                     std::to_string((size_t)FDGA_BUBBLE_NOALLOC_MAX_ELEMS) + " complex values");
    Dims d{};
    d.nG = c->nG; d.NG = 2 * c->nG; d.L = c->L; d.Nq = (int)NR; d.Nk = (int)NR;
    d.nPO = c->nK1; d.NPO = 2 * c->nK1 - 1; d.nPn = c->nK1 * c->mPi_factor; d.NPn = 2 * d.nPn;
    d.T = c->T; d.U = c->U; d.local = c->local ? 1 : 0;
    int tv = 32;
    while (tv > 1 && (size_t)4 * tv * NR * sizeof(cplx) > 160 * 1024) tv >>= 1;
    const size_t shm = (size_t)4 * tv * NR * sizeof(cplx);
    if (shm > 200 * 1024) return bad(FDGA_ERR_ARG, "momentum mesh too large for the shared-memory tile");  // (L <= 56 fits)
    cplx* GR = nullptr;
    int r = scratch_address(&GR);
    if (r) return r;
    Twiddles tw;
    for (int j = 0; j < c->L; ++j) {
        const double a = 2.0 * M_PI * j / c->L;
        tw.m[j] = mk(std::cos(a), -std::sin(a));
        tw.p[j] = mk(std::cos(a), std::sin(a));
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    static fdga::SmemRecord smem_raised;  // per device, under the library's shared-memory lock
    cudaError_t e = fdga::raise_smem_limit(k_noalloc_bubble, smem_raised, shm);
    if (e != cudaSuccess) return bad(FDGA_ERR_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
    const size_t ng = NR * NG;
    k_noalloc_greal<<<(unsigned)((ng + 127) / 128), 128, 0, s>>>(reinterpret_cast<const cplx*>(G), GR, tw, d);
    e = cudaGetLastError();
    if (e != cudaSuccess) return bad(FDGA_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    dim3 grid((d.NPn + tv - 1) / tv, d.NPO);
    k_noalloc_bubble<<<grid, 256, shm, s>>>(GR, reinterpret_cast<cplx*>(Pipp), reinterpret_cast<cplx*>(Piph), tw, d, tv);
    e = cudaGetLastError();
    if (e != cudaSuccess) return bad(FDGA_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return FDGA_OK;
}
