// fdga_kernels.cu -- sm_103a kernels of one parquet iteration (FP64 plain path).
//
// Each kernel restates one reference function (cited per kernel).  Work items of the
// symmetry-grouped sums are class representatives (device indices); the remaining elements
// are filled by k_finalize3 with the class operation, as MatsubaraFunctions' SymmetryGroup does.
#include "fdga_device.cuh"
#include "fdga_kernels.h"

#include <algorithm>
#include <cmath>
#include <type_traits>

namespace fdga {

// ---------------------------------------------------------------------------------------------
// Elementwise: Dyson G = 1/(1/Gbare + Σ)  (src/dyson.jl:5-31; G, Σ store iG, iΣ)
// ---------------------------------------------------------------------------------------------
__global__ void k_dyson(cplx* G, const cplx* Sig, const cplx* Gb, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const cplx one = mk(1.0, 0.0);
    G[i] = cdiv(one, cdiv(one, Gb[i]) + Sig[i]);
}

// Tangent of the Dyson update G = 1/(1/Gb + Σ) (in the stored iG, iΣ convention): dG = -G² dΣ.
__global__ void k_dyson_tan(cplx* tG, const cplx* G, const cplx* tSig, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const cplx g = G[i];
    tG[i] = (g * g) * (tSig[i] * -1.0);
}

// n = 1/2 + T Im(Σ G) / Nk  (src/dyson.jl:33-41); single block, deterministic order.
__global__ void k_occupation(const cplx* G, size_t n, double T, int Nk, double* out) {
    __shared__ double red[1024];
    double s = 0.0;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) s += G[i].y;
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = 0.5 + red[0] * T / (double)Nk;
}

// ---------------------------------------------------------------------------------------------
// G(R) = (1/N) Σ_k G(k) e^{-2πi k·R/L}  (fft(...)/L² of src/nonlocal/bubble.jl:110-111)
// tw[j] = e^{-2πi j/L}, j < L.   GR layout [R][ν]
// ---------------------------------------------------------------------------------------------
__global__ void k_g_realspace(const cplx* G, cplx* GR, const cplx* tw, Dims d) {
    const int NR = d.L * d.L;
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= (size_t)NR * d.NG) return;
    const int nu = (int)(i % d.NG), R = (int)(i / d.NG);
    const int Rx = R % d.L, Ry = R / d.L;
    cplx s = mk(0, 0);
    for (int k = 0; k < NR; ++k) {
        const int kx = k % d.L, ky = k / d.L;
        const int ph = (kx * Rx + ky * Ry) % d.L;
        s = cfma(G[(size_t)k * d.NG + nu], tw[ph], s);
    }
    GR[i] = s * (1.0 / NR);
}

// ---------------------------------------------------------------------------------------------
// Local bubbles Πpp(Ω,ν) = G(ν) G(Ω-ν), Πph(Ω,ν) = G(ν) G(Ω+ν), G -> 1/ν outside its box
// (src/bubble.jl:9-36).
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ cplx g_tail(const cplx* G, const Dims& d, int k, int n) {
    if (fin(n, d.nG)) return G[ixG(d, k, n)];
    return mk(1.0 / ((2.0 * n + 1.0) * M_PI * d.T), 0.0);
}
// the same in arithmetic type C from storage G (cplx or the mixed map's FP32 copy)
template <class C, class G>
__device__ __forceinline__ C g_tail_t(const G* Gp, const Dims& d, int k, int n) {
    using R = decltype(C::x);
    if (fin(n, d.nG)) return to_c<C>(Gp[ixG(d, k, n)]);
    return C{(R)1 / (((R)2 * n + (R)1) * (R)M_PI * (R)d.T), (R)0};
}

// tangent of g_tail_t: the 1/ν tail is constant, so the derivative is zero outside the box
template <class C, class G>
__device__ __forceinline__ C g_box_t(const G* Gp, const Dims& d, int k, int n) {
    if (fin(n, d.nG)) return to_c<C>(Gp[ixG(d, k, n)]);
    return C{0, 0};
}
// a·b, or for the tangent map (TAN) the product rule da·b + a·db
template <bool TAN, class C>
__device__ __forceinline__ C prod2(C a, C da, C b, C db) {
    if (TAN) return cfma(da, b, a * db);
    return a * b;
}

// TAN: the tangent bubbles dΠ from G and its tangent tG (product rule, the tails are constant)
template <bool TAN>
__global__ void k_bubble_local(const cplx* G, const cplx* tG, cplx* pp, cplx* ph, Dims d) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= (size_t)d.NPO * d.NPw) return;
    const int n = (int)(i % d.NPw) - d.nPw, m = (int)(i / d.NPw) - (d.nPO - 1);
    const cplx Gn = g_tail(G, d, 0, n);
    if (!TAN) {
        pp[i] = Gn * g_tail(G, d, 0, m - n - 1);
        ph[i] = Gn * g_tail(G, d, 0, m + n);
        return;
    }
    const cplx tn = g_box_t<cplx>(tG, d, 0, n);
    pp[i] = prod2<true>(Gn, tn, g_tail(G, d, 0, m - n - 1), g_box_t<cplx>(tG, d, 0, m - n - 1));
    ph[i] = prod2<true>(Gn, tn, g_tail(G, d, 0, m + n), g_box_t<cplx>(tG, d, 0, m + n));
}

// Nonlocal bubbles in real space (src/nonlocal/bubble.jl:87-158) for L_G = L:
//   Πpp(R) = G(R, Ω-ν) G(R, ν),  Πph(R) = G(R, Ω+ν) G(-R, ν),  R = 0 with the 1/ν tail,
//   Π(P) = Σ_R Π(R) e^{+2πi P·R/L}  (bfft).  For L_G = L the ±L/2 half weights of the reference's
//   R scan sum to one per lattice site, so the scan is one pass over the L x L sites.
// One CTA = one Ω and a tile of TV fermionic frequencies; shared: Π(R) then the P transform.
// C: arithmetic type (FP64, or FP32 for the mixed map's bubble from the FP32 copy of G(R)); G:
// storage of G(R).  The twiddles are staged in shared memory in C.
template <bool TAN, class C, class G>
__global__ void k_bubble_nl(const G* GR, const G* tGR, cplx* pp, cplx* ph, const cplx* twp, Dims d, int TV) {
    extern __shared__ __align__(16) unsigned char sh_raw[];
    const int L = d.L, NR = L * L;
    C* A = reinterpret_cast<C*>(sh_raw);  // [2][TV][NR]   (pp, ph) in R
    C* B = A + 2 * (size_t)TV * NR;       // [2][TV][NR]  after the x transform
    C* tw = B + 2 * (size_t)TV * NR;      // [L]
    for (int j = threadIdx.x; j < L; j += blockDim.x) tw[j] = to_c<C>(twp[j]);
    const int m = blockIdx.y - (d.nPO - 1);
    const int n0 = blockIdx.x * TV - d.nPw;
    for (int e = threadIdx.x; e < TV * NR; e += blockDim.x) {
        const int v = e / NR, R = e % NR;
        const int n = n0 + v;
        C vpp{0, 0}, vph{0, 0};
        if (n < d.nPw) {
            const int Rx = R % L, Ry = R / L;
            const int mR = ((L - Rx) % L) + L * ((L - Ry) % L);
            if (R == 0) {
                const C gn = g_tail_t<C>(GR, d, 0, n), tn = TAN ? g_box_t<C>(tGR, d, 0, n) : gn;
                vpp = prod2<TAN>(g_tail_t<C>(GR, d, 0, m - n - 1), TAN ? g_box_t<C>(tGR, d, 0, m - n - 1) : gn, gn, tn);
                vph = prod2<TAN>(g_tail_t<C>(GR, d, 0, m + n), TAN ? g_box_t<C>(tGR, d, 0, m + n) : gn, gn, tn);
            } else {
                const int a = m - n - 1, b = m + n;
                if (fin(a, d.nG) && fin(n, d.nG)) {
                    const size_t i1 = ixG(d, R, a), i2 = ixG(d, R, n);
                    const C g1 = to_c<C>(GR[i1]), g2 = to_c<C>(GR[i2]);
                    vpp = prod2<TAN>(g1, TAN ? to_c<C>(tGR[i1]) : g1, g2, TAN ? to_c<C>(tGR[i2]) : g2);
                }
                if (fin(b, d.nG) && fin(n, d.nG)) {
                    const size_t i1 = ixG(d, R, b), i2 = ixG(d, mR, n);
                    const C g1 = to_c<C>(GR[i1]), g2 = to_c<C>(GR[i2]);
                    vph = prod2<TAN>(g1, TAN ? to_c<C>(tGR[i1]) : g1, g2, TAN ? to_c<C>(tGR[i2]) : g2);
                }
            }
        }
        A[(size_t)v * NR + R] = vpp;
        A[(size_t)(TV + v) * NR + R] = vph;
    }
    __syncthreads();
    // transform along x: B[v][Py*L + Px] = Σ_x A[v][y*L + x] w^{Px x}, stored as (Px, y)
    for (int e = threadIdx.x; e < 2 * TV * NR; e += blockDim.x) {
        const int row = e / NR, r = e % NR;
        const int Px = r % L, y = r / L;
        const C* a = A + (size_t)row * NR + (size_t)y * L;
        C s{0, 0};
        for (int x = 0; x < L; ++x) s = cfma(a[x], tw[(Px * x) % L], s);
        B[(size_t)row * NR + r] = s;
    }
    __syncthreads();
    // transform along y and write Π[P][Ω][ν]
    for (int e = threadIdx.x; e < 2 * TV * NR; e += blockDim.x) {
        const int v = e % TV;               // ν fastest across threads for coalesced stores
        const int rest = e / TV;
        const int P = rest % NR, which = rest / NR;
        const int Px = P % L, Py = P / L;
        const int n = n0 + v;
        if (n >= d.nPw) continue;
        const C* b = B + (size_t)(which * TV + v) * NR;
        C s{0, 0};
        for (int y = 0; y < L; ++y) s = cfma(b[(size_t)y * L + Px], tw[(Py * y) % L], s);
        (which ? ph : pp)[ixPi(d, P, m, n)] = to_d(s);
    }
}

// Radix-2 FFT variant of k_bubble_nl for power-of-two L (same mathematics; the R->P transform
// costs O(L log L) per row instead of O(L²)).  c_twp32[j] = e^{+2πi j/32}.
__constant__ cplx c_twp32[32];

template <int L>
__host__ __device__ constexpr int bitrev(int i) {
    int r = 0;
    for (int b = 1; b < L; b <<= 1) { r = (r << 1) | (i & 1); i >>= 1; }
    return r;
}

__constant__ cplxf c_twp32f[32];
template <class C> __device__ __forceinline__ C twp32(int j);
template <> __device__ __forceinline__ cplx twp32<cplx>(int j) { return c_twp32[j]; }
template <> __device__ __forceinline__ cplxf twp32<cplxf>(int j) { return c_twp32f[j]; }
// e^{+2πi j/96}: the twiddles of the lattices L = 3·2^a (3 ≤ L ≤ 96)
__constant__ cplx c_twp96[96];
__constant__ cplxf c_twp96f[96];
template <class C> __device__ __forceinline__ C twp96(int j);
template <> __device__ __forceinline__ cplx twp96<cplx>(int j) { return c_twp96[j]; }
template <> __device__ __forceinline__ cplxf twp96<cplxf>(int j) { return c_twp96f[j]; }

// in-place backward DFT (e^{+2πi jk/L}) of v[0..L) held in registers
template <int L, class C>
__device__ __forceinline__ void fft_bwd(C (&v)[L]) {
#pragma unroll
    for (int i = 0; i < L; ++i) {
        const int j = bitrev<L>(i);
        if (j > i) { const C t = v[i]; v[i] = v[j]; v[j] = t; }
    }
#pragma unroll
    for (int len = 2; len <= L; len <<= 1) {
        const int half = len / 2;
#pragma unroll
        for (int i = 0; i < L; i += len) {
#pragma unroll
            for (int k = 0; k < half; ++k) {
                const C b = v[i + k + half];
                C t;
                if (k == 0) t = b;
                else if (4 * k == len) t = C{-b.y, b.x};  // multiply by i
                else t = b * twp32<C>(k * (32 / len));
                const C u = v[i + k];
                v[i + k] = u + t;
                v[i + k + half] = u - t;
            }
        }
    }
}

// in-place backward DFT of length L = 3M (M a power of two), by one mixed-radix step
// (Cooley–Tukey, n = 3 n1 + n2, k = k1 + M k2): three length-M transforms of the residues n2, the
// twiddles e^{2πi n2 k1 / L}, then M length-3 transforms, Z0 = u0 + s, Z1,2 = u0 - s/2 ± i(√3/2) d
// with s = u1 + u2, d = u1 - u2.
template <int L, class C>
__device__ __forceinline__ void fft_bwd_3m(C (&v)[L]) {
    using R = decltype(C::x);
    constexpr int M = L / 3;
    static_assert(3 * M == L && (M & (M - 1)) == 0 && L <= 96, "L = 3 * 2^a, L <= 96");
    C y0[M], y1[M], y2[M];
#pragma unroll
    for (int n1 = 0; n1 < M; ++n1) { y0[n1] = v[3 * n1]; y1[n1] = v[3 * n1 + 1]; y2[n1] = v[3 * n1 + 2]; }
    if constexpr (M > 1) {
        fft_bwd<M>(y0);
        fft_bwd<M>(y1);
        fft_bwd<M>(y2);
    }
    const R h3 = (R)0.86602540378443864676;  // √3 / 2
#pragma unroll
    for (int k1 = 0; k1 < M; ++k1) {
        const C a = y0[k1];
        const C b = k1 == 0 ? y1[k1] : y1[k1] * twp96<C>(k1 * (96 / L));
        const C c = k1 == 0 ? y2[k1] : y2[k1] * twp96<C>(2 * k1 * (96 / L));
        const C sm = b + c, df = b - c;
        const C hh = C{a.x - (R)0.5 * sm.x, a.y - (R)0.5 * sm.y};
        const C rot = C{-h3 * df.y, h3 * df.x};
        v[k1] = a + sm;
        v[k1 + M] = hh + rot;
        v[k1 + 2 * M] = hh - rot;
    }
}
// backward DFT for the lattices with a register FFT: powers of two up to 32, and 3·2^a up to 24
template <int L, class C>
__device__ __forceinline__ void fft_bwd_any(C (&v)[L]) {
    if constexpr ((L & (L - 1)) == 0) fft_bwd<L>(v);
    else fft_bwd_3m<L>(v);
}

template <int L, class C, class G, bool TAN>
__global__ void k_bubble_fft(const G* GR, const G* tGR, cplx* pp, cplx* ph, Dims d, int TV) {
    extern __shared__ __align__(16) unsigned char sh_raw[];
    C* sh = reinterpret_cast<C*>(sh_raw);
    constexpr int NR = L * L, RS = L + 1, BS = L * (L + 1) + 1;
    const int m = blockIdx.y - (d.nPO - 1);
    const int n0 = blockIdx.x * TV - d.nPw;
    for (int e = threadIdx.x; e < TV * NR; e += blockDim.x) {
        const int v = e / NR, R = e % NR;
        const int n = n0 + v;
        const int Rx = R % L, Ry = R / L;
        C vpp{0, 0}, vph{0, 0};
        if (n < d.nPw) {
            const int mR = ((L - Rx) % L) + L * ((L - Ry) % L);
            if (R == 0) {
                const C gn = g_tail_t<C>(GR, d, 0, n), tn = TAN ? g_box_t<C>(tGR, d, 0, n) : gn;
                vpp = prod2<TAN>(g_tail_t<C>(GR, d, 0, m - n - 1), TAN ? g_box_t<C>(tGR, d, 0, m - n - 1) : gn, gn, tn);
                vph = prod2<TAN>(g_tail_t<C>(GR, d, 0, m + n), TAN ? g_box_t<C>(tGR, d, 0, m + n) : gn, gn, tn);
            } else {
                const int a = m - n - 1, b = m + n;
                if (fin(a, d.nG) && fin(n, d.nG)) {
                    const size_t i1 = ixG(d, R, a), i2 = ixG(d, R, n);
                    const C g1 = to_c<C>(GR[i1]), g2 = to_c<C>(GR[i2]);
                    vpp = prod2<TAN>(g1, TAN ? to_c<C>(tGR[i1]) : g1, g2, TAN ? to_c<C>(tGR[i2]) : g2);
                }
                if (fin(b, d.nG) && fin(n, d.nG)) {
                    const size_t i1 = ixG(d, R, b), i2 = ixG(d, mR, n);
                    const C g1 = to_c<C>(GR[i1]), g2 = to_c<C>(GR[i2]);
                    vph = prod2<TAN>(g1, TAN ? to_c<C>(tGR[i1]) : g1, g2, TAN ? to_c<C>(tGR[i2]) : g2);
                }
            }
        }
        sh[(size_t)v * BS + Ry * RS + Rx] = vpp;
        sh[(size_t)(TV + v) * BS + Ry * RS + Rx] = vph;
    }
    __syncthreads();
    for (int r = threadIdx.x; r < 2 * TV * L; r += blockDim.x) {  // along x
        C* row = sh + (size_t)(r / L) * BS + (r % L) * RS;
        C v[L];
#pragma unroll
        for (int x = 0; x < L; ++x) v[x] = row[x];
        fft_bwd_any<L>(v);
#pragma unroll
        for (int x = 0; x < L; ++x) row[x] = v[x];
    }
    __syncthreads();
    for (int c = threadIdx.x; c < 2 * TV * L; c += blockDim.x) {  // along y
        C* col = sh + (size_t)(c / L) * BS + (c % L);
        C v[L];
#pragma unroll
        for (int y = 0; y < L; ++y) v[y] = col[y * RS];
        fft_bwd_any<L>(v);
#pragma unroll
        for (int y = 0; y < L; ++y) col[y * RS] = v[y];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 2 * TV * NR; e += blockDim.x) {
        const int v = e % TV;
        const int rest = e / TV;
        const int P = rest % NR, which = rest / NR;
        const int n = n0 + v;
        if (n >= d.nPw) continue;
        const C val = sh[(size_t)(which * TV + v) * BS + (P / L) * RS + (P % L)];
        (which ? ph : pp)[ixPi(d, P, m, n)] = to_d(val);
    }
}

// Batched 2D transform over the L x L momentum grid: out[R][row] = scale Σ_P e^{sign 2πi P·R/L} in[P][row]
// (momentum index x + L y outermost, `rows` contiguous values per momentum).  One CTA transforms TR
// consecutive rows through shared memory (coalesced loads and stores along the rows).
template <int L>
__global__ void k_fft2_rows(const cplx* in, cplx* out, int rows, int sign, double scale, int TR) {
    extern __shared__ cplx sh[];
    constexpr int NR = L * L, RS = L + 1, BS = L * (L + 1) + 1;
    const int r0 = blockIdx.x * TR;
    for (int e = threadIdx.x; e < TR * NR; e += blockDim.x) {
        const int r = e % TR, P = e / TR;
        cplx v = (r0 + r < rows) ? in[(size_t)P * rows + r0 + r] : mk(0, 0);
        if (sign < 0) v.y = -v.y;  // forward transform = conj(backward(conj))
        sh[(size_t)r * BS + (P / L) * RS + (P % L)] = v;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < TR * L; q += blockDim.x) {
        cplx* row = sh + (size_t)(q / L) * BS + (q % L) * RS;
        cplx v[L];
#pragma unroll
        for (int x = 0; x < L; ++x) v[x] = row[x];
        fft_bwd_any<L>(v);
#pragma unroll
        for (int x = 0; x < L; ++x) row[x] = v[x];
    }
    __syncthreads();
    for (int q = threadIdx.x; q < TR * L; q += blockDim.x) {
        cplx* col = sh + (size_t)(q / L) * BS + (q % L);
        cplx v[L];
#pragma unroll
        for (int y = 0; y < L; ++y) v[y] = col[y * RS];
        fft_bwd_any<L>(v);
#pragma unroll
        for (int y = 0; y < L; ++y) col[y * RS] = v[y];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < TR * NR; e += blockDim.x) {
        const int r = e % TR, R = e / TR;
        if (r0 + r >= rows) continue;
        cplx v = sh[(size_t)r * BS + (R / L) * RS + (R % L)];
        if (sign < 0) v.y = -v.y;
        out[(size_t)R * rows + r0 + r] = v * scale;
    }
}
// Separable DFT variant of k_fft2_rows for L that is not a power of two: the TR rows of a CTA are
// staged in shared memory and transformed along x then y, one output element per thread and pass
// (2L products per output instead of L² for the direct 2D sum).  tw[j] = e^{sign 2πi j/L}.
__global__ void k_dft2_sep(const cplx* in, cplx* out, int rows, int L, const cplx* tw, double scale, int TR) {
    extern __shared__ cplx sh[];
    const int NR = L * L, RS = L + 1, BS = L * (L + 1) + 1;
    cplx* twS = sh + (size_t)2 * TR * BS;
    for (int j = threadIdx.x; j < L; j += blockDim.x) twS[j] = tw[j];
    const int r0 = blockIdx.x * TR;
    cplx* A = sh;                         // [TR][L][L+1]
    cplx* B = sh + (size_t)TR * BS;       // [TR][L][L+1]
    for (int e = threadIdx.x; e < TR * NR; e += blockDim.x) {
        const int r = e % TR, P = e / TR;
        A[(size_t)r * BS + (P / L) * RS + (P % L)] = (r0 + r < rows) ? in[(size_t)P * rows + r0 + r] : mk(0, 0);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < TR * NR; e += blockDim.x) {  // along x: B[r][y][kx] = Σ_x A[r][y][x] w^{kx x}
        const int r = e / NR, q = e % NR, y = q / L, kx = q % L;
        const cplx* a = A + (size_t)r * BS + y * RS;
        cplx s = mk(0, 0);
        int ph = 0;
        for (int x = 0; x < L; ++x) {
            s = cfma(a[x], twS[ph], s);
            ph += kx;
            if (ph >= L) ph -= L;
        }
        B[(size_t)r * BS + y * RS + kx] = s;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < TR * NR; e += blockDim.x) {  // along y, written as out[R][row]
        const int r = e % TR, R = e / TR, ky = R / L, kx = R % L;
        if (r0 + r >= rows) continue;
        const cplx* b = B + (size_t)r * BS + kx;
        cplx s = mk(0, 0);
        int ph = 0;
        for (int y = 0; y < L; ++y) {
            s = cfma(b[y * RS], twS[ph], s);
            ph += ky;
            if (ph >= L) ph -= L;
        }
        out[(size_t)R * rows + r0 + r] = s * scale;
    }
}
// Direct-DFT fallback of k_fft2_rows for L that is not a power of two; one thread per output.
__global__ void k_dft2_rows(const cplx* in, cplx* out, int rows, int L, const cplx* tw, double scale) {
    const int NR = L * L;
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= (size_t)NR * rows) return;
    const int r = (int)(i % rows), R = (int)(i / rows);
    const int Rx = R % L, Ry = R / L;
    cplx acc = mk(0, 0);
    for (int P = 0; P < NR; ++P) acc = cfma(in[(size_t)P * rows + r], tw[((P % L) * Rx + (P / L) * Ry) % L], acc);
    out[i] = acc * scale;
}

// ---------------------------------------------------------------------------------------------
// Momentum averages A = Σ_P K[P] / Nq (s-wave evaluation, src/nonlocal/swave.jl:32-72)
// blockIdx.y = channel*3 + class
// ---------------------------------------------------------------------------------------------
__global__ void k_qavg(const ChanArrays in, ChanArraysW out, Dims d) {
    const int ch = blockIdx.y / 3, cl = blockIdx.y % 3;
    const size_t per = cl == 0 ? (size_t)d.N1 : (cl == 1 ? (size_t)d.N2O * d.N2n : (size_t)d.N3O * d.N3n * d.N3n);
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= per) return;
    const cplx* src = cl == 0 ? in.K1[ch] : (cl == 1 ? in.K2[ch] : in.K3[ch]);
    cplx* dst = cl == 0 ? out.K1[ch] : (cl == 1 ? out.K2[ch] : out.K3[ch]);
    cplx s = mk(0, 0);
    int P = 0;
    for (; P + 4 <= d.Nq; P += 4) {  // four independent loads in flight, summed in order
        const cplx a0 = src[(size_t)P * per + i], a1 = src[(size_t)(P + 1) * per + i];
        const cplx a2 = src[(size_t)(P + 2) * per + i], a3 = src[(size_t)(P + 3) * per + i];
        s += a0; s += a1; s += a2; s += a3;
    }
    for (; P < d.Nq; ++P) s += src[(size_t)P * per + i];
    dst[i] = s * (1.0 / d.Nq);
}

// ---------------------------------------------------------------------------------------------
// K3 caches (src/build_K3_cache.jl:20-95, src/nonlocal/build_K3_cache.jl:18-94).
// One thread per K3 mesh point (P, Ω, a, b) of the listed (P, Ω) blocks (the blocks holding
// symmetry-class representatives; all blocks without groups); "left" caches use (Ω, ω=a, ν'=b),
// "right" caches (Ω, ν=a, ω=b).  Output order: Γpx F0p F0a F0t Γpp Γa Γt Fp Fa Ft.
// ---------------------------------------------------------------------------------------------
// V0 (every vertex-evaluating kernel): compiled with the evaluation of a Vertex-valued reference
// vertex F0.  The plain instantiation clears has0 in a local copy of the view, so the compiler drops
// those paths and the RefVertex kernels keep their registers.
template <bool V0, class S>
__device__ __forceinline__ VertPT<S> vert_spec(const VertPT<S>& F) {
    VertPT<S> G = F;
    if constexpr (!V0) G.has0 = 0;
    return G;
}
template <bool V0, class S>
__device__ __forceinline__ TanArgsT<S> tan_spec(const TanArgsT<S>& T) {
    TanArgsT<S> U = T;
    if constexpr (!V0) U.F.has0 = 0;
    return U;
}
// S: vertex storage and arithmetic (cplx; cplxf reads the FP32 mirror of the mixed map).
template <class S, bool V0>
__global__ void k_build_cache(VertPT<S> Fin, Caches C, const int* blocks, int nblocks, Dims d) {
    const VertPT<S> F = vert_spec<V0>(Fin);
    using R = decltype(S::x);
    const size_t bs = (size_t)d.N3n * d.N3n;
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)nblocks * bs) return;
    const int bl = blocks ? blocks[t / bs] : (int)(t / bs);  // block = P * NΩ3 + iΩ
    const size_t e = t % bs;
    const size_t i = (size_t)bl * bs + e;
    const int b = (int)(e % d.N3n) - d.n3n;
    const int a = (int)(e / d.N3n) - d.n3n;
    const int m = bl % d.N3O - (d.n3O - 1);
    const int P = bl / d.N3O;
    // left
    S v[10];
    v[0] = vert_eval(F, d, CH_P, SP_X, m, a, b, P, FL_GT | FL_GA);
    v[1] = f0_xSp(F, d, CH_P, m, a, b, P) - f0_xSp(F, d, CH_P, m, a, FINF, P);
    const S f0a = f0_pSp(F, d, CH_A, m, a, b, P) - f0_pSp(F, d, CH_A, m, a, FINF, P);
    const S f0t = f0_pSp(F, d, CH_T, m, a, b, P) - f0_pSp(F, d, CH_T, m, a, FINF, P);
    v[2] = f0a;
    v[3] = f0t * (R)2 - f0a;
    // right
    const S gpp = vert_pSp(F, d, CH_P, m, a, b, P, FL_GT | FL_GA);
    const S ga = vert_pSp(F, d, CH_A, m, a, b, P, FL_GP | FL_GT);
    const S gt = vert_pSp(F, d, CH_T, m, a, b, P, FL_GP | FL_GA);
    const S fp = vert_pSp(F, d, CH_P, m, a, b, P, FL_F0 | FL_GP) - vert_pSp(F, d, CH_P, m, FINF, b, P, FL_F0 | FL_GP) + gpp;
    const S fa = vert_pSp(F, d, CH_A, m, a, b, P, FL_F0 | FL_GA) - vert_pSp(F, d, CH_A, m, FINF, b, P, FL_F0 | FL_GA) + ga;
    const S ft = vert_pSp(F, d, CH_T, m, a, b, P, FL_F0 | FL_GT) - vert_pSp(F, d, CH_T, m, FINF, b, P, FL_F0 | FL_GT) + gt;
    v[4] = gpp;
    v[5] = ga;
    v[6] = gt * (R)2 - ga;
    v[7] = fp;
    v[8] = fa;
    v[9] = ft * (R)2 - fa;
    // an absent cache (nullptr) is not written: the RefVertex caches of a tangent vertex are zero
    if (C.f[0]) {
#pragma unroll
        for (int k = 0; k < 10; ++k)
            if (C.f[k]) C.f[k][i] = to_f32(v[k]);
    } else {
#pragma unroll
        for (int k = 0; k < 10; ++k)
            if (C.c[k]) C.c[k][i] = to_d(v[k]);
    }
}

// ---------------------------------------------------------------------------------------------
// Bubble row sums SΠ(P, Ω) = Σ_ν Π(P, Ω, ν) over the whole bubble mesh; blockIdx.y = array.
// ---------------------------------------------------------------------------------------------
__global__ void k_rowsum(const cplx* A0, const cplx* A1, cplx* S0, cplx* S1, int rowlen) {
    __shared__ double rx[256], ry[256];
    const cplx* A = blockIdx.y ? A1 : A0;
    cplx* S = blockIdx.y ? S1 : S0;
    const size_t row = blockIdx.x;
    double sx = 0.0, sy = 0.0;
    for (int i = threadIdx.x; i < rowlen; i += blockDim.x) {
        const cplx v = A[row * rowlen + i];
        sx += v.x;
        sy += v.y;
    }
    rx[threadIdx.x] = sx;
    ry[threadIdx.x] = sy;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) { rx[threadIdx.x] += rx[threadIdx.x + o]; ry[threadIdx.x] += ry[threadIdx.x + o]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) S[row] = mk(rx[0], ry[0]);
}

// Full-mesh bubble row sums in real space, for a stored window narrower than the mesh:
//   SR[w][Ω][R] = Σ_{ν ∈ bubble mesh} Π_R^w(Ω, ν, R),   S^w(P, Ω) = Σ_R e^{+2πi P·R/L} SR[w][Ω][R],
// with Π_R as in k_bubble_nl (R = 0 carries the 1/ν tail; R ≠ 0 needs both G in their box).
// T0[w][Ω] = Σ over the bubble mesh of the tail·tail products (both G outside their box); depends
// only on T and the meshes.  One warp per (w, Ω).
__global__ void k_tail_const(cplx* T0, Dims d) {
    const size_t w = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (size_t)2 * d.NPO) return;
    const int which = (int)(w / d.NPO), m = (int)(w % d.NPO) - (d.nPO - 1);
    cplx acc = mk(0, 0);
    for (int n = -d.nPn + lane; n < d.nPn; n += 32) {
        const int a = which ? m + n : m - n - 1;
        if (fin(n, d.nG) || fin(a, d.nG)) continue;
        acc = cfma(g_tail(nullptr, d, 0, a), g_tail(nullptr, d, 0, n), acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) T0[w] = acc;
}
// TAN: row sums of the tangent bubbles (product rule with tGR; the tails and T0 are constant)
template <class C, class G, bool TAN>
__global__ void k_pisum_R(const G* GR, const G* tGR, const cplx* T0, cplx* SR, Dims d) {
    const int NR = d.L * d.L;
    const size_t w = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (size_t)2 * d.NPO * NR) return;
    const int which = (int)(w / ((size_t)d.NPO * NR));
    const int rest = (int)(w % ((size_t)d.NPO * NR));
    const int R = rest / d.NPO, m = rest % d.NPO - (d.nPO - 1);  // SR[w][R][Ω]
    const int L = d.L, Rx = R % L, Ry = R / L;
    const int mR = ((L - Rx) % L) + L * ((L - Ry) % L);
    C acc{0, 0};
    if (R == 0) {
        // terms with at least one factor inside the G box; the tail·tail remainder is the
        // iteration-independent T0 (k_tail_const), added below
        for (int n = -d.nG + lane; n < d.nG; n += 32) {  // n inside the box
            if (!fin(n, d.nPn)) continue;
            const int p = which ? m + n : m - n - 1;
            if (TAN)
                acc += prod2<true>(g_tail_t<C>(GR, d, 0, p), g_box_t<C>(tGR, d, 0, p), g_tail_t<C>(GR, d, 0, n),
                                   g_box_t<C>(tGR, d, 0, n));
            else
                acc = cfma(g_tail_t<C>(GR, d, 0, p), g_tail_t<C>(GR, d, 0, n), acc);
        }
        for (int a = -d.nG + lane; a < d.nG; a += 32) {  // partner inside the box, n outside
            const int n = which ? a - m : m - 1 - a;
            if (fin(n, d.nG) || !fin(n, d.nPn)) continue;
            acc = cfma(TAN ? g_box_t<C>(tGR, d, 0, a) : g_tail_t<C>(GR, d, 0, a), g_tail_t<C>(GR, d, 0, n), acc);
        }
        if (lane == 0 && T0 && !TAN) acc += to_c<C>(T0[(size_t)which * d.NPO + (m + d.nPO - 1)]);
    } else {
        for (int n = -d.nG + lane; n < d.nG; n += 32) {
            if (!fin(n, d.nPn)) continue;
            const int p = which ? m + n : m - n - 1;
            if (!fin(p, d.nG)) continue;
            const size_t i1 = ixG(d, R, p), i2 = ixG(d, which ? mR : R, n);
            const C g1 = to_c<C>(GR[i1]), g2 = to_c<C>(GR[i2]);
            if (TAN) acc += prod2<true>(g1, to_c<C>(tGR[i1]), g2, to_c<C>(tGR[i2]));
            else acc = cfma(g1, g2, acc);
        }
    }
    acc = warp_sum(acc);
    if (lane == 0) SR[w] = to_d(acc);
}
// S_X(ch, P, Ω) = Σ_ω [(Π-Π0)(Ω,ω,P) U + Π(Ω,ω,P) FL(Ω,ω̃,∞)]: the ω-sum of the BSE's right factor
// (src/BSEa/BSEa_K1.jl:43, BSEa_K2.jl:185), from the row sums and the K2 window of FL.
// Layout SX[ch][P][Ω] with Ω over the K1 box; SPi/SPi0 [w][P][Ω] with w = 0 pp, 1 ph.
// A Vertex-valued F0 adds (Π-Π0)(Ω,ω) [F0(Ω,ω̃,∞) - U] = (SΠ - SΠ0) k0 + Σ_{ω̃ ∈ F0's K2 box}
// (Π-Π0)(ω) [f0_right(ω̃) - k0], k0 = its own channel's K1 (f0_right at ω̃ = ∞).
__global__ void k_sx(const cplx* Pipp, const cplx* Piph, const cplx* Pi0pp, const cplx* Pi0ph, const cplx* SPi,
                     const cplx* SPi0, FLP FL, VertP F0v, cplx* SX, Dims d) {
    const size_t per = (size_t)d.Nq * d.NPO;
    const size_t i = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;  // warp per output
    const int lane = threadIdx.x & 31;
    if (i >= 3 * per) return;
    const int ch = (int)(i / per);
    const size_t r = i % per;
    const int m = (int)(r % d.NPO) - (d.nPO - 1), P = (int)(r / d.NPO);
    const int w = (ch == CH_P) ? 0 : 1;
    const cplx* Pi = w ? Piph : Pipp;
    cplx v = mk(0, 0);
    if (bin(m, d.n2O)) {
        for (int t = lane; t < d.N2n; t += 32) {
            const int nt = t - d.n2n;
            const int n = (ch == CH_P) ? m - nt - 1 : nt;
            if (!fin(n, d.nPw)) continue;
            v += Pi[ixPi(d, P, m, n)] * fl_right(FL.K2[CH_P], FL.K2[CH_T], FL.K2[CH_A], d, ch, m, nt, P);
        }
    }
    cplx k0 = mk(0, 0);
    if (F0v.has0 && bin(m, F0v.b0.n1)) {
        const cplx* Pi0 = w ? Pi0ph : Pi0pp;
        k0 = f0_right(F0v, ch, m, FINF, P);
        if (bin(m, F0v.b0.n2O)) {
            for (int t = lane; t < F0v.b0.N2n; t += 32) {
                const int nt = t - F0v.b0.n2n;
                const int n = (ch == CH_P) ? m - nt - 1 : nt;
                if (!fin(n, d.nPw)) continue;
                const size_t ip = ixPi(d, P, m, n);
                v += (Pi[ip] - Pi0[ip]) * (f0_right(F0v, ch, m, nt, P) - k0);
            }
        }
    }
    v = warp_sum(v);
    if (lane == 0) {
        const cplx ds = SPi[w * per + r] - SPi0[w * per + r];
        SX[i] = F0v.has0 ? ds * (mk(d.U, 0) + k0) + v : ds * d.U + v;
    }
}

// Tangent of S_X: dS_X = dSΠ U + Σ_ω [dΠ FL(Ω,ω̃,∞) + Π dFL(Ω,ω̃,∞)]  (SΠ0 is constant).
__global__ void k_sx_tan(const cplx* Pipp, const cplx* Piph, const cplx* tPipp, const cplx* tPiph, const cplx* tSPi,
                         FLP FL, FLP tFL, VertP F0v, cplx* tSX, Dims d) {
    const size_t per = (size_t)d.Nq * d.NPO;
    const size_t i = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= 3 * per) return;
    const int ch = (int)(i / per);
    const size_t r = i % per;
    const int m = (int)(r % d.NPO) - (d.nPO - 1), P = (int)(r / d.NPO);
    const int w = (ch == CH_P) ? 0 : 1;
    const cplx* Pi = w ? Piph : Pipp;
    const cplx* tPi = w ? tPiph : tPipp;
    cplx v = mk(0, 0);
    if (bin(m, d.n2O)) {
        for (int t = lane; t < d.N2n; t += 32) {
            const int nt = t - d.n2n;
            const int n = (ch == CH_P) ? m - nt - 1 : nt;
            if (!fin(n, d.nPw)) continue;
            const size_t ip = ixPi(d, P, m, n);
            v += tPi[ip] * fl_right(FL.K2[CH_P], FL.K2[CH_T], FL.K2[CH_A], d, ch, m, nt, P);
            v += Pi[ip] * fl_right(tFL.K2[CH_P], tFL.K2[CH_T], tFL.K2[CH_A], d, ch, m, nt, P);
        }
    }
    cplx k0 = mk(0, 0);  // a Vertex-valued F0 (constant): dΠ times its F0(Ω,ω̃,∞) - U, as in k_sx
    if (F0v.has0 && bin(m, F0v.b0.n1)) {
        k0 = f0_right(F0v, ch, m, FINF, P);
        if (bin(m, F0v.b0.n2O)) {
            for (int t = lane; t < F0v.b0.N2n; t += 32) {
                const int nt = t - F0v.b0.n2n;
                const int n = (ch == CH_P) ? m - nt - 1 : nt;
                if (!fin(n, d.nPw)) continue;
                v += tPi[ixPi(d, P, m, n)] * (f0_right(F0v, ch, m, nt, P) - k0);
            }
        }
    }
    v = warp_sum(v);
    if (lane == 0) tSX[i] = F0v.has0 ? tSPi[w * per + r] * (mk(d.U, 0) + k0) + v : tSPi[w * per + r] * d.U + v;
}

// ---------------------------------------------------------------------------------------------
// K1 BSE (src/BSEa/BSEa_K1.jl:2-54, src/nonlocal/BSEa/BSEa_K1.jl:2-57), warp per item:
//   K1(Ω,P) = T s Σ_ω F(Ω,∞,ω) X(ω),  X(ω) = (Π-Π0)(Ω,ω) U + Π(Ω,ω) FL(Ω,ω̃,∞).
// F(Ω,∞,ω) depends on ω only through the same channel's K2(Ω, ω) (ω in the K2 box), so the sum is
// evaluated exactly as c·S_X + Σ_{ω ∈ K2 box} (F(Ω,∞,ω) - c) X(ω), c = F(Ω,∞,∞).
// ---------------------------------------------------------------------------------------------
// TAN: the tangent dK1 = K1(dF; Π, FL, S_X) + K1(F; dΠ, dFL, dS_X) in one pass (T: the tangent
// factors; dX = dΠ (FL + U) + Π dFL).
template <int CH, class S, bool TAN>
__device__ __forceinline__ void bse_K1_body(const VertPT<S>& F, const FLPT<S>& FL, const cplx* Pi, const cplx* Pi0,
                                            const cplx* SX, cplx* out, const int* items, int nitems, int accum,
                                            const Dims& d, const TanArgsT<S>& T) {
    using R = decltype(S::x);
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nitems) return;
    const int idx = items ? items[w] : w;
    const int m = idx % d.N1 - (d.n1 - 1), P = idx / d.N1;
    constexpr int SP = (CH == CH_T) ? SP_D : SP_P;
    const S c = vert_eval(F, d, CH, SP, m, FINF, FINF, P);
    S tc{0, 0};
    if constexpr (TAN) tc = vert_eval(T.F, d, CH, SP, m, FINF, FINF, P);
    const cplx* tPi = (CH == CH_P) ? T.pp : T.ph;
    S acc{0, 0};
    // F(Ω,∞,ω) varies in the K2 boxes of F and (a Vertex-valued) F0: the extents xn2O, xn2n
    if (bin(m, d.xn2O)) {
        for (int n = -d.xn2n + lane; n < d.xn2n; n += 32) {
            if (!fin(n, d.nPw)) continue;
            const int wt = cross(CH, m, n);
            const S Fl = vert_eval(F, d, CH, SP, m, FINF, n, P) - c;
            const S FLr = fl_right(FL.K2[CH_P], FL.K2[CH_T], FL.K2[CH_A], d, CH, m, wt, P);
            const size_t ip = ixPi(d, P, m, n);
            const S pi = to_c<S>(ldg(Pi + ip)), pi0 = Pi0 ? to_c<S>(ldg(Pi0 + ip)) : S{0, 0};
            // F0r = F0(Ω, ω̃, ∞) = U_sp (RefVertex), plus the own channel of a Vertex-valued F0
            const S U0 = F.has0 ? cre<S>(d.U) + f0_right(F, CH, m, wt, P) : cre<S>(d.U);
            if constexpr (!TAN) {
                if (F.has0) acc = cfma(Fl, cfma(pi, FLr, (pi - pi0) * U0), acc);
                else acc = cfma(Fl, cfma(pi, FLr, (pi - pi0) * (R)d.U), acc);
            } else {
                const S X = F.has0 ? cfma(pi, FLr, (pi - pi0) * U0) : cfma(pi, FLr, (pi - pi0) * (R)d.U);
                const S tFl = vert_eval(T.F, d, CH, SP, m, FINF, n, P) - tc;
                const S tFLr = fl_right(T.FL.K2[CH_P], T.FL.K2[CH_T], T.FL.K2[CH_A], d, CH, m, wt, P);
                const S tpi = to_c<S>(ldg(tPi + ip));
                const S tX = cfma(tpi, FLr + U0, pi * tFLr);
                acc = cfma(tFl, X, cfma(Fl, tX, acc));
            }
        }
    }
    acc = warp_sum(acc);
    if (lane == 0) {
        const size_t is = (size_t)CH * d.Nq * d.NPO + (size_t)P * d.NPO + (m + d.nPO - 1);
        const S sx = SX ? to_c<S>(SX[is]) : S{0, 0};
        S r = c * sx + acc;
        if constexpr (TAN) r = cfma(tc, sx, c * to_c<S>(T.SX[is])) + acc;
        const cplx v = to_d(r * (R)(d.T * (CH == CH_T ? -1.0 : 1.0)));
        out[idx] = accum ? out[idx] + v : v;
    }
}

// ---------------------------------------------------------------------------------------------
// Left K2 BSE (fdPA), warp per item:
//   local (src/BSEa/BSEa_K2.jl:1-40):        Σ_{ω∈Π mesh} Γ_irr(Ω,ν,ω) Π0(Ω,ω) U
//   nonlocal (src/nonlocal/BSEa/BSEa_K2.jl:1-39): Σ_{ω∈K2 mesh} Γ_irr(Ω,ν,ω̃) Π0(Ω,ω) U
// ---------------------------------------------------------------------------------------------
template <int CH, class S>
__device__ __forceinline__ void bse_L_K2_body(const VertPT<S>& F, const cplx* Pi0, cplx* out, const int* items,
                                              int nitems, const Dims& d) {
    using R = decltype(S::x);
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nitems) return;
    const int idx = items ? items[w] : w;
    const int nu = idx % d.N2n - d.n2n;
    const int m = (idx / d.N2n) % d.N2O - (d.n2O - 1);
    const int P = idx / (d.N2n * d.N2O);
    constexpr int SP = (CH == CH_T) ? SP_D : SP_P;
    constexpr int IRR = (CH == CH_P) ? (FL_GT | FL_GA) : (CH == CH_T ? (FL_GP | FL_GA) : (FL_GP | FL_GT));
    S acc{0, 0};
    if (F.has0) {
        // a Vertex-valued F0: the factor F0r = F0(Ω, ω̃, ∞) (local) or F0(Ω, ω, ∞) (nonlocal) depends on ω
        if (d.local) {
            for (int n = -d.nPw + lane; n < d.nPw; n += 32) {
                const S Gp = vert_eval(F, d, CH, SP, m, nu, n, P, IRR);
                const S f0r = cre<S>(d.U) + f0_right(F, CH, m, cross(CH, m, n), P);
                acc = cfma(Gp, to_c<S>(ldg(Pi0 + ixPi(d, P, m, n))) * f0r, acc);
            }
        } else {
            for (int n = -d.n2n + lane; n < d.n2n; n += 32) {
                const S Gl = vert_eval(F, d, CH, SP, m, nu, cross(CH, m, n), P, IRR);
                const S f0r = cre<S>(d.U) + f0_right(F, CH, m, n, P);
                acc = cfma(Gl, to_c<S>(ldg(Pi0 + ixPi(d, P, m, n))) * f0r, acc);
            }
        }
        acc = warp_sum(acc);
        if (lane == 0) out[idx] = to_d(acc * (R)(d.T * (CH == CH_T ? -1.0 : 1.0)));
        return;
    }
    if (d.local) {
        for (int n = -d.nPw + lane; n < d.nPw; n += 32) {  // local solver: nPw = nPn
            const S Gp = vert_eval(F, d, CH, SP, m, nu, n, P, IRR);
            acc = cfma(Gp, to_c<S>(ldg(Pi0 + ixPi(d, P, m, n))), acc);
        }
    } else {
        for (int n = -d.n2n + lane; n < d.n2n; n += 32) {
            const S Gl = vert_eval(F, d, CH, SP, m, nu, cross(CH, m, n), P, IRR);
            acc = cfma(Gl, to_c<S>(ldg(Pi0 + ixPi(d, P, m, n))), acc);
        }
    }
    acc = warp_sum(acc);
    if (lane == 0) out[idx] = to_d(acc * (R)(d.U * d.T * (CH == CH_T ? -1.0 : 1.0)));
}

// ---------------------------------------------------------------------------------------------
// K2 BSE (src/BSEa/BSEa_K2.jl:43-103, src/nonlocal/BSEa/BSEa_K2.jl:43-105), warp per item:
//   T s Σ_ω [F(Ω,ν,ω) - F(Ω,∞,ω)] X(ω).
// Outside the union of (i) the K2 and RefVertex fermionic boxes and (ii) the ω for which a
// converted bosonic frequency of another channel lies in the K1 box (centres ν, -(Ω+ν+1) and,
// for the p channel, Ω-ν-1; src/convention.jl:4-36), F(Ω,ν,ω) - F(Ω,∞,ω) equals its
// ω-independent value c = F(Ω,ν,∞) - F(Ω,∞,∞); the sum is evaluated exactly as
// c·S_X + Σ_{ω ∈ union} (F(Ω,ν,ω) - F(Ω,∞,ω) - c) X(ω).
// ---------------------------------------------------------------------------------------------
// One CTA per (channel, P, Ω) row of representatives (the items of a row differ only in ν).  The
// ν-independent factor of the ω-sum, X(ω) = Π(ω) FL(Ω,ω,∞) + (Π - Π0)(ω) U, is tabulated once per
// row in shared memory over the ω range any window can reach, [-W, W) with
// W = n2O + n2n + n1 + nRn + 2 (clipped to the stored bubble window); each warp then sums one
// item's window terms.  The vertex factor F(Ω,ν,ω) - F(Ω,∞,ω) - c is evaluated in its reduced form
// (pSp_k2diff; the t channel's 2 pSp + xSp by crossing, xSp = -pSp in the a representation).
// GB300's FP64 pipe bounds this kernel: both take FP64 work out of the per-term loop.
// TAN: the tangent in one pass, as for K1 (tables X and dX).
__host__ __device__ __forceinline__ int k2_table_half(const Dims& d) {
    const int W = d.xn2O + d.xn2n + d.xn1 + d.nRn + 2;  // (extents over F and a Vertex-valued F0)
    return W < d.nPw ? W : d.nPw;
}
template <int CH, class S, bool TAN>
__device__ __forceinline__ void bse_K2_row(const VertPT<S>& F, const FLPT<S>& FL, const cplx* Pi, const cplx* Pi0,
                                           const cplx* SX, cplx* out, const int* items, const int* gstart,
                                           int ngroups, int accum, const Dims& d, const TanArgsT<S>& T, S* tab) {
    using R = decltype(S::x);
    const int g = blockIdx.x;
    if (g >= ngroups) return;
    const int i0 = gstart ? gstart[g] : g * d.N2n, i1 = gstart ? gstart[g + 1] : (g + 1) * d.N2n;
    const int first = items ? items[i0] : i0;
    const int m = (first / d.N2n) % d.N2O - (d.n2O - 1);
    const int P = first / (d.N2n * d.N2O);
    const int half = k2_table_half(d), NT = 2 * half;
    S* Xt = tab;
    S* tXt = tab + NT;
    const cplx* tPi = (CH == CH_P) ? T.pp : T.ph;
    for (int j = threadIdx.x; j < NT; j += blockDim.x) {
        const int n = j - half;
        const int wt = cross(CH, m, n);
        const S FLr = fl_right(FL.K2[CH_P], FL.K2[CH_T], FL.K2[CH_A], d, CH, m, wt, P);
        const size_t ip = ixPi(d, P, m, n);
        const S pi = to_c<S>(ldg(Pi + ip)), pi0 = Pi0 ? to_c<S>(ldg(Pi0 + ip)) : S{0, 0};
        // F0r = U_sp, plus the own channel of a Vertex-valued F0 (f0_right)
        const S U0 = F.has0 ? cre<S>(d.U) + f0_right(F, CH, m, wt, P) : cre<S>(d.U);
        Xt[j] = F.has0 ? cfma(pi, FLr, (pi - pi0) * U0) : cfma(pi, FLr, (pi - pi0) * (R)d.U);
        if constexpr (TAN) {
            const S tFLr = fl_right(T.FL.K2[CH_P], T.FL.K2[CH_T], T.FL.K2[CH_A], d, CH, m, wt, P);
            const S tpi = to_c<S>(ldg(tPi + ip));
            tXt[j] = cfma(tpi, FLr + U0, pi * tFLr);
        }
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const int lo = -d.nPw, hi = d.nPw - 1, h1 = d.xn1 - 1;
    const size_t is = (size_t)CH * d.Nq * d.NPO + (size_t)P * d.NPO + (m + d.nPO - 1);
    for (int it = i0 + warp; it < i1; it += nwarps) {
        const int idx = items ? items[it] : it;
        const int nu = idx % d.N2n - d.n2n;
        const S c = k2_c<CH>(F, d, m, nu, P);
        S tc{0, 0};
        if constexpr (TAN) tc = k2_c<CH>(T.F, d, m, nu, P);
        Windows win;
        win.add(-d.xn2n, d.xn2n - 1, lo, hi);
        win.add(-d.nRn, d.nRn - 1, lo, hi);
        win.add(nu - h1, nu + h1, lo, hi);
        win.add(-(m + nu + 1) - h1, -(m + nu + 1) + h1, lo, hi);
        if (CH == CH_P) win.add(m - nu - 1 - h1, m - nu - 1 + h1, lo, hi);
        win.merge();
        S acc{0, 0};
        for (int t = lane; t < win.total; t += 32) {
            const int n = win.at(t);
            const int j = n + half;
            if constexpr (!TAN) {
                const S Fl = k2_vertex_diff<CH>(F, d, m, nu, n, P);
                acc = cfma(Fl, Xt[j], acc);
            } else {
                S Fl, tFl;
                k2_vertex_diff2<CH>(F, T.F, d, m, nu, n, P, Fl, tFl);
                acc = cfma(tFl, Xt[j], cfma(Fl, tXt[j], acc));
            }
        }
        acc = warp_sum(acc);
        if (lane == 0) {
            const S sx = SX ? to_c<S>(SX[is]) : S{0, 0};
            S r = c * sx + acc;
            if constexpr (TAN) r = cfma(tc, sx, c * to_c<S>(T.SX[is])) + acc;
            const cplx v = to_d(r * (R)(d.T * (CH == CH_T ? -1.0 : 1.0)));
            out[idx] = accum ? out[idx] + v : v;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// K3 BSE as one complex GEMM per (ch, P, Ω) block, C = A·M (src/BSEa/BSEa_K3.jl:1-128,
// src/nonlocal/BSEa/BSEa_K3.jl:1-128):
//   MODE 0 (BSE_L_K3):  A = cacheΓ(ν,ω),  M(ω,ν') = Π0(ω) cacheF0(ω,ν');          out = T s C
//   MODE 1 (BSE_K3):    A = cacheF(ν,ω),  M(ω,ν') = s1[(Π-Π0)(ω) cacheF0(ω,ν') + Π(ω) Γs(ω,ν')]
//                                                    + s2 Π(ω) γL(ω̃,ν')[ω̃ in box]; out = T C + γL(ν,ν')
// TILE x TILE output tile per CTA (TILE = 16, 24 or 32 chosen to fit Nν), (TILE/2)^2 threads with
// 2x2 outputs each, K chunks of 8.  blockIdx.x = channel-slot * (Nq·NΩ3) + (P·NΩ3 + iΩ), blockIdx.y /
// blockIdx.z = row / column tile; the three channels of one mode share a launch.
// ---------------------------------------------------------------------------------------------
// Operand loads of the K3 GEMM: FP64 storage converted to the arithmetic type, or FP32 storage
// (the mixed map's caches and FL.K3 copy) read as is.
template <class C> __device__ __forceinline__ C ldk(const cplx* p) { return to_c<C>(ldg(p)); }
template <class C> __device__ __forceinline__ C ldk(const cplxf* p) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    return C{v.x, v.y};
}

// ARGS = K3Args3 (FP64 operands) or K3Args3F (FP32 operands).  C = cplx: FP64 arithmetic (the plain
// path).  C = cplxf: FP32 products and accumulation, FP64 epilogue (the mixed path; FP64 operands
// are converted when they are staged into shared memory).
// FP64 arithmetic (the plain path, bound by GB300's FP64 pipe) forms each complex product with three
// real multiplications (Gauss): t1 = Σ ar br, t2 = Σ ai bi, t3 = Σ (ar + ai)(br + bi), then
// C = (t1 - t2) + i (t3 - t1 - t2).  The sums ar + ai and br + bi are formed once, when an element
// is staged, so the inner loop issues 3 FMAs per complex multiply-add instead of 4.
template <int MODE, int TILE, int TCOL, class C, class ARGS>
__global__ void __launch_bounds__((TILE / 2) * (TCOL / 2)) k_bse_K3_gemm(ARGS args, Dims d) {
    using R = decltype(C::x);
    constexpr int TK = 8, H = TILE / 2, HC = TCOL / 2, NT = H * HC;
    constexpr bool G3 = std::is_same<C, cplx>::value;  // three-multiplication form in FP64
    __shared__ C As[TILE][TK + 1];
    __shared__ C Ms[TK][TCOL + 1];
    __shared__ R Asum[G3 ? TILE : 1][TK + 1];  // ar + ai of the staged A (FP64 form)
    __shared__ R Msum[G3 ? TK : 1][TCOL + 1];  // br + bi of the staged M
    // the ω-only factors of M, signs folded in, for the current and the next K chunk:
    // [0] s1(Π-Π0) (mode 0: Π0)  [1] s1 Π  [2] s2 Π  [3] s1 dΠ  [4] s2 dΠ
    __shared__ C Pk[2][TK][5];
    const int tid = threadIdx.x;
    const int tx = tid % HC, ty = tid / HC;
    const int col0 = blockIdx.z * TCOL, row0 = blockIdx.y * TILE;
    const int nb = args.nblocks;
    const int slot = blockIdx.x / nb;
    const int blk = args.blocks ? args.blocks[blockIdx.x % nb] : (int)(blockIdx.x % nb);
    const auto& a = args.a[slot];
    const int CH = args.ch[slot];
    const int m = blk % d.N3O - (d.n3O - 1), P = blk / d.N3O;
    const int N = d.N3n;
    const size_t base = (size_t)blk * N * N;
    const R s1 = (CH == CH_A) ? (R)1 : (R)-1, s2 = (CH == CH_T) ? (R)-1 : (R)1;
    const bool oneloop = (a.flags & K3F_1LOOP) != 0;
    auto fill_pk = [&](int buf, int k0) {
        if (tid < TK) {
            C* q = Pk[buf][tid];
            const int k = k0 + tid;
            for (int j = 0; j < 5; ++j) q[j] = czero<C>();
            if (k < N) {
                const size_t ip = ixPi(d, P, m, k - d.n3n);
                const C pi0 = a.Pi0 ? to_c<C>(ldg(a.Pi0 + ip)) : czero<C>();
                if (MODE == 0) {
                    q[0] = pi0;
                } else {
                    const C pi = to_c<C>(ldg(a.Pi + ip));
                    q[0] = (pi - pi0) * s1;
                    q[1] = pi * s1;
                    q[2] = pi * s2;
                    if (MODE == 2) {
                        const C tpi = to_c<C>(ldg(a.tPi + ip));
                        q[3] = tpi * s1;
                        q[4] = tpi * s2;
                    }
                }
            }
        }
    };
    // γL at a K3 index in the channel's spin combination (t: 2 FL.γt - FL.γa)
    auto gl_at = [&](const auto* FLc, const auto* FLt, const auto* FLa, size_t i) -> C {
        if (CH == CH_T) {
            const C t = ldk<C>(FLt + i), u = ldk<C>(FLa + i);
            return C{fma(t.x, (R)2, -u.x), fma(t.y, (R)2, -u.y)};
        }
        return ldk<C>(FLc + i);
    };
    C acc[2][2] = {{czero<C>(), czero<C>()}, {czero<C>(), czero<C>()}};  // G3: (t1, t2)
    R acc3[2][2] = {{(R)0, (R)0}, {(R)0, (R)0}};                           // G3: t3
    fill_pk(0, 0);
    __syncthreads();
    int cur = 0;
    // MODE 2 (tangent): the inner index runs twice, first over (dA, M), then over (A, dM)
    constexpr int NH = (MODE == 2) ? 2 : 1;
    for (int half = 0; half < NH; ++half) {
        const auto* Ap = (MODE == 2 && half == 0) ? a.tA : a.A;
        const bool tM = (MODE == 2 && half == 1);
        for (int k0 = 0; k0 < N; k0 += TK) {
            for (int e = tid; e < TILE * TK; e += NT) {
                const int r = e / TK, kk = e % TK;
                const int row = row0 + r, k = k0 + kk;
                const C v = (row < N && k < N) ? ldk<C>(Ap + base + (size_t)row * N + k) : czero<C>();
                As[r][kk] = v;
                if constexpr (G3) Asum[r][kk] = v.x + v.y;
            }
            for (int e = tid; e < TK * TCOL; e += NT) {
                const int kk = e / TCOL, c = e % TCOL;
                const int k = k0 + kk, col = col0 + c;
                const C* q = Pk[cur][kk];
                C v = czero<C>();
                if (k < N && col < N) {
                    const C f0 = ldk<C>(a.B0 + base + (size_t)k * N + col);
                    if (MODE == 0) {
                        v = q[0] * f0;
                    } else if (oneloop) {
                        v = q[0] * f0;
                    } else {
                        const size_t ig = (CH == CH_P) ? base + (size_t)k * N + col : base + (size_t)col * N + k;
                        const C gs = ldk<C>(a.G + ig);
                        const int ot = cross(CH, m, k - d.n3n);
                        const size_t il = base + (size_t)(ot + d.n3n) * N + col;
                        if (!tM) {  // s1 [(Π-Π0) F0 + Π Γ] + s2 Π γL
                            v = cfma(q[0], f0, q[1] * gs);
                            if (fin(ot, d.n3n)) v = cfma(q[2], gl_at(a.FLc, a.FLt, a.FLa, il), v);
                        } else {  // dM = s1 [dΠ (F0 + Γ) + Π dΓ] + s2 [dΠ γL + Π dγL]
                            v = cfma(q[3], f0 + gs, q[1] * ldk<C>(a.tG + ig));
                            if (fin(ot, d.n3n))
                                v = cfma(q[4], gl_at(a.FLc, a.FLt, a.FLa, il),
                                         cfma(q[2], gl_at(a.tFLc, a.tFLt, a.tFLa, il), v));
                        }
                    }
                }
                Ms[kk][c] = v;
                if constexpr (G3) Msum[kk][c] = v.x + v.y;
            }
            // the next chunk's factors (the next K chunk, or the first chunk of the next half)
            const int nk0 = (k0 + TK < N) ? k0 + TK : 0;
            if (k0 + TK < N || half + 1 < NH) fill_pk(cur ^ 1, nk0);
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < TK; ++kk) {
                const C a0 = As[ty][kk], a1 = As[ty + H][kk];
                const C b0 = Ms[kk][tx], b1 = Ms[kk][tx + HC];
                if constexpr (G3) {
                    const R sa[2] = {Asum[ty][kk], Asum[ty + H][kk]}, sb[2] = {Msum[kk][tx], Msum[kk][tx + HC]};
                    const C aa[2] = {a0, a1}, bb[2] = {b0, b1};
#pragma unroll
                    for (int i = 0; i < 2; ++i)
#pragma unroll
                        for (int j = 0; j < 2; ++j) {
                            acc[i][j].x = fma(aa[i].x, bb[j].x, acc[i][j].x);
                            acc[i][j].y = fma(aa[i].y, bb[j].y, acc[i][j].y);
                            acc3[i][j] = fma(sa[i], sb[j], acc3[i][j]);
                        }
                } else {
                    acc[0][0] = cfma(a0, b0, acc[0][0]);
                    acc[0][1] = cfma(a0, b1, acc[0][1]);
                    acc[1][0] = cfma(a1, b0, acc[1][0]);
                    acc[1][1] = cfma(a1, b1, acc[1][1]);
                }
            }
            __syncthreads();
            cur ^= 1;
        }
    }
    const R Tr = (R)d.T;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int row = row0 + ty + H * i, col = col0 + tx + HC * j;
            if (row >= N || col >= N) continue;
            const size_t io = base + (size_t)row * N + col;
            // epilogue in the arithmetic type C (FP64 ops cost 64 FP32 ops on this part)
            C c = acc[i][j];
            if constexpr (G3) c = C{acc[i][j].x - acc[i][j].y, acc3[i][j] - (acc[i][j].x + acc[i][j].y)};
            cplx v;
            if (MODE == 0) {
                v = to_d(c * (R)(d.T * ((CH == CH_A) ? 1.0 : -1.0)));
            } else if (a.flags & K3F_NOEPI) {
                v = to_d(c * Tr);
            } else {
                const C g = (MODE == 1) ? gl_at(a.FLc, a.FLt, a.FLa, io) : gl_at(a.tFLc, a.tFLt, a.tFLa, io);
                v = to_d(C{fma(c.x, Tr, g.x), fma(c.y, Tr, g.y)});
            }
            a.out[io] = (a.flags & K3F_ACC) ? a.out[io] + v : v;
        }
}



// ---------------------------------------------------------------------------------------------
// SDE: L_pp, L_ph (src/SDE.jl:79-217, src/nonlocal/SDE.jl:3-143), warp per item.
//   vertex part:    L_pp = T U Σ_ω Πpp(Ω,ω) γp(Ω,Ω-ω,ν),  L_ph = T U Σ_ω Πph(Ω,ω) (γt+γa)(Ω,ν,ω)
//   RefVertex part: L_pp = T U Σ_ω Πpp (F0_p(Ω,Ω-ω,ν) - U),  L_ph = T U Σ_ω Πph (F0_a + F0_t - 2U)
// The channel factor depends on ω only where the ω-argument lies in the K2 (vertex) or RefVertex
// box; elsewhere it equals c = γ(…, ν, ∞), so the vertex sum is c·SΠ + Σ_{window} Π (γ - c).
// out = T [vertex part] + T ref_scale [RefVertex part].
// ---------------------------------------------------------------------------------------------
// TAN: dL = L(dF; Π, SΠ) + L(F; dΠ, dSΠ) + ref_scale·RefVertex part with dΠ, in one pass.
template <int WHICH, class S, bool TAN>
__device__ __forceinline__ void sde_L_body(const VertPT<S>& F, const cplx* Pi, const cplx* SPi, cplx* out,
                                           const int* items, int nitems, int use_vertex, double ref_scale, int accum,
                                           const Dims& d, const TanArgsT<S>& T) {
    using R = decltype(S::x);
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nitems) return;
    const int idx = items ? items[w] : w;
    const int nu = idx % d.N2n - d.n2n;
    const int m = (idx / d.N2n) % d.N2O - (d.n2O - 1);
    const int P = idx / (d.N2n * d.N2O);
    const cplx* tPi = WHICH == 0 ? T.pp : T.ph;
    S acc{0, 0}, accr{0, 0}, c{0, 0}, tc{0, 0};
    if (use_vertex & 1) {
        if (WHICH == 0) {
            c = chan_eval(F.g[CH_P], d, m, FINF, nu, P);
            if constexpr (TAN) tc = chan_eval(T.F.g[CH_P], d, m, FINF, nu, P);
            for (int t = lane; t < d.N2n; t += 32) {
                const int n = m - (t - d.n2n) - 1;  // Ω-ω runs over the K2 box
                if (!fin(n, d.nPw)) continue;
                const S g = chan_eval(F.g[CH_P], d, m, m - n - 1, nu, P) - c;
                const size_t ip = ixPi(d, P, m, n);
                if constexpr (!TAN) {
                    acc = cfma(to_c<S>(ldg(Pi + ip)), g, acc);
                } else {
                    const S tg = chan_eval(T.F.g[CH_P], d, m, m - n - 1, nu, P) - tc;
                    acc = cfma(to_c<S>(ldg(tPi + ip)), g, cfma(to_c<S>(ldg(Pi + ip)), tg, acc));
                }
            }
        } else {
            c = chan_eval(F.g[CH_T], d, m, nu, FINF, P) + chan_eval(F.g[CH_A], d, m, nu, FINF, P);
            if constexpr (TAN) tc = chan_eval(T.F.g[CH_T], d, m, nu, FINF, P) + chan_eval(T.F.g[CH_A], d, m, nu, FINF, P);
            for (int n = -d.n2n + lane; n < d.n2n; n += 32) {
                if (!fin(n, d.nPw)) continue;
                const S g = chan_eval(F.g[CH_T], d, m, nu, n, P) + chan_eval(F.g[CH_A], d, m, nu, n, P) - c;
                const size_t ip = ixPi(d, P, m, n);
                if constexpr (!TAN) {
                    acc = cfma(to_c<S>(ldg(Pi + ip)), g, acc);
                } else {
                    const S tg = chan_eval(T.F.g[CH_T], d, m, nu, n, P) + chan_eval(T.F.g[CH_A], d, m, nu, n, P) - tc;
                    acc = cfma(to_c<S>(ldg(tPi + ip)), g, cfma(to_c<S>(ldg(Pi + ip)), tg, acc));
                }
            }
        }
    }
    // the Vertex level of a Vertex-valued F0 (use_vertex bit 2): the same sums over its channels g0
    // (box b0), SDE!(Σ, …, F.F0, …) of the reference's recursion; constant in the tangent map
    S acc0{0, 0}, c0{0, 0};
    if ((use_vertex & 2) && F.has0) {
        const Box& b = F.b0;
        if (WHICH == 0) {
            c0 = chan_eval(F.g0[CH_P], b, m, FINF, nu, P);
            for (int t = lane; t < b.N2n; t += 32) {
                const int n = m - (t - b.n2n) - 1;
                if (!fin(n, d.nPw)) continue;
                const S g = chan_eval(F.g0[CH_P], b, m, m - n - 1, nu, P) - c0;
                acc0 = cfma(to_c<S>(ldg((TAN ? tPi : Pi) + ixPi(d, P, m, n))), g, acc0);
            }
        } else {
            c0 = chan_eval(F.g0[CH_T], b, m, nu, FINF, P) + chan_eval(F.g0[CH_A], b, m, nu, FINF, P);
            for (int n = -b.n2n + lane; n < b.n2n; n += 32) {
                if (!fin(n, d.nPw)) continue;
                const S g = chan_eval(F.g0[CH_T], b, m, nu, n, P) + chan_eval(F.g0[CH_A], b, m, nu, n, P) - c0;
                acc0 = cfma(to_c<S>(ldg((TAN ? tPi : Pi) + ixPi(d, P, m, n))), g, acc0);
            }
        }
    }
    if (ref_scale != 0.0) {
        for (int t = lane; t < d.NRn; t += 32) {
            const int r = t - d.nRn;
            const int n = (WHICH == 0) ? m - r - 1 : r;
            if (!fin(n, d.nPw)) continue;
            S g;
            if (WHICH == 0) g = ref_pSp(F, d, CH_P, m, m - n - 1, nu) - cre<S>(d.U);
            else g = ref_pSp(F, d, CH_A, m, nu, n) + ref_pSp(F, d, CH_T, m, nu, n) - cre<S>(d.U) - cre<S>(d.U);
            accr = cfma(to_c<S>(ldg((TAN ? tPi : Pi) + ixPi(d, P, m, n))), g, accr);
        }
    }
    acc = warp_sum(acc) * (R)d.U;
    accr = warp_sum(accr) * (R)d.U;
    if ((use_vertex & 2) && F.has0) {
        acc0 = warp_sum(acc0);
        if (lane == 0) {
            const size_t is0 = (size_t)P * d.NPO + (m + d.nPO - 1);
            const cplx* sp0 = TAN ? (WHICH == 0 ? T.SPpp : T.SPph) : SPi;
            acc += cfma(c0, to_c<S>(ldg(sp0 + is0)), acc0) * (R)d.U;
        }
    }
    if (lane == 0) {
        const size_t is = (size_t)P * d.NPO + (m + d.nPO - 1);
        if (use_vertex & 1) {
            if constexpr (!TAN) {
                acc += c * (to_c<S>(ldg(SPi + is)) * (R)d.U);
            } else {
                const S tsp = to_c<S>(ldg((WHICH == 0 ? T.SPpp : T.SPph) + is));
                acc += cfma(tc, to_c<S>(ldg(SPi + is)), c * tsp) * (R)d.U;
            }
        }
        const cplx v = to_d(acc * (R)d.T + accr * (R)(d.T * ref_scale));
        out[idx] = accum ? out[idx] + v : v;
    }
}

// ---------------------------------------------------------------------------------------------
// K1 and K2 of the :fdPA_new / :scPA_new strategies, local solver (src/BSEa/BSEa_K1.jl:57-100,
// src/BSEa/BSEa_K2.jl:104-150), warp per item:
//   K1(Ω)   = T s U Σ_ω [F(Ω,∞,ω) Π(Ω,ω) - F0(Ω,∞,ω) Π0(Ω,ω)]
//   K2(Ω,ν) = T s U Σ_ω [(F(Ω,ν,ω) - F(Ω,∞,ω)) Π - (F0(Ω,ν,ω) - F0(Ω,∞,ω)) Π0],  ω over the bubble mesh.
// F0(Ω,∞,ω) is U_sp for every ω.  For K1, F(Ω,∞,ω) = F(Ω,∞,∞) = c outside the K2 box, so the sum is
// c SΠ + Σ_{K2 box} (F - c) Π - U_sp SΠ0.  For K2 the F difference is ω-independent outside the
// windows of bse_K2_row and the F0 difference vanishes outside the RefVertex box.
// ---------------------------------------------------------------------------------------------
// A Vertex-valued F0 varies in its own K2 box: F0(Ω,∞,ω) = u0 + (F0(Ω,∞,ω) - u0) there, and its
// difference F0(Ω,ν,ω) - F0(Ω,∞,ω) has the ω-independent part c0 = F0(Ω,ν,∞) - F0(Ω,∞,∞) (its K2(ν))
// outside the windows, which enlarge to the boxes of F0 (the extents xn1, xn2O, xn2n).
template <int CH, class S>
__device__ __forceinline__ void bse_K1_new_body(const VertPT<S>& F, const cplx* Pi, const cplx* Pi0, const cplx* SPi,
                                                const cplx* SPi0, cplx* out, const int* items, int nitems,
                                                const Dims& d) {
    using R = decltype(S::x);
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nitems) return;
    const int idx = items ? items[w] : w;
    const int m = idx % d.N1 - (d.n1 - 1), P = idx / d.N1;
    constexpr int SP = (CH == CH_T) ? SP_D : SP_P;
    const S c = vert_eval(F, d, CH, SP, m, FINF, FINF, P);
    const S u0 = f0_eval(F, d, CH, SP, m, FINF, FINF, P);
    S acc{0, 0};
    if (bin(m, d.xn2O)) {
        for (int n = -d.xn2n + lane; n < d.xn2n; n += 32) {
            if (!fin(n, d.nPw)) continue;
            const size_t ip = ixPi(d, P, m, n);
            acc = cfma(vert_eval(F, d, CH, SP, m, FINF, n, P) - c, to_c<S>(ldg(Pi + ip)), acc);
            if (F.has0) acc = acc - (f0_eval(F, d, CH, SP, m, FINF, n, P) - u0) * to_c<S>(ldg(Pi0 + ip));
        }
    }
    acc = warp_sum(acc);
    if (lane == 0) {
        const size_t is = (size_t)P * d.NPO + (m + d.nPO - 1);
        const S v = cfma(c, to_c<S>(SPi[is]), acc) - u0 * to_c<S>(SPi0[is]);
        out[idx] = to_d(v * (R)(d.U * d.T * (CH == CH_T ? -1.0 : 1.0)));
    }
}
template <int CH, class S>
__device__ __forceinline__ void bse_K2_new_body(const VertPT<S>& F, const cplx* Pi, const cplx* Pi0, const cplx* SPi,
                                                const cplx* SPi0, cplx* out, const int* items, int nitems,
                                                const Dims& d) {
    using R = decltype(S::x);
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nitems) return;
    const int idx = items ? items[w] : w;
    const int nu = idx % d.N2n - d.n2n;
    const int m = (idx / d.N2n) % d.N2O - (d.n2O - 1);
    const int P = idx / (d.N2n * d.N2O);
    constexpr int SP = (CH == CH_T) ? SP_D : SP_P;
    const S cinf = vert_eval(F, d, CH, SP, m, FINF, FINF, P);
    const S c = vert_eval(F, d, CH, SP, m, nu, FINF, P) - cinf;
    const S u0 = f0_eval(F, d, CH, SP, m, FINF, FINF, P);
    const S c0 = F.has0 ? f0_eval(F, d, CH, SP, m, nu, FINF, P) - u0 : S{0, 0};  // (zero for a RefVertex)
    Windows win;
    const int lo = -d.nPw, hi = d.nPw - 1, h1 = d.xn1 - 1;
    win.add(-d.xn2n, d.xn2n - 1, lo, hi);
    win.add(-d.nRn, d.nRn - 1, lo, hi);
    win.add(nu - h1, nu + h1, lo, hi);
    win.add(-(m + nu + 1) - h1, -(m + nu + 1) + h1, lo, hi);
    if (CH == CH_P) win.add(m - nu - 1 - h1, m - nu - 1 + h1, lo, hi);
    win.merge();
    S acc{0, 0};
    for (int t = lane; t < win.total; t += 32) {
        const int n = win.at(t);
        const S Finf = fin(n, d.xn2n) ? vert_eval(F, d, CH, SP, m, FINF, n, P) : cinf;
        const S Fl = vert_eval(F, d, CH, SP, m, nu, n, P) - Finf - c;
        const S F0l = F.has0 ? f0_eval(F, d, CH, SP, m, nu, n, P) - f0_eval(F, d, CH, SP, m, FINF, n, P) - c0
                             : ref_eval(F, d, CH, SP, m, nu, n) - u0;
        const size_t ip = ixPi(d, P, m, n);
        acc = cfma(Fl, to_c<S>(ldg(Pi + ip)), acc);
        acc = acc - F0l * to_c<S>(ldg(Pi0 + ip));
    }
    acc = warp_sum(acc);
    if (lane == 0) {
        const size_t is = (size_t)P * d.NPO + (m + d.nPO - 1);
        S v = cfma(c, to_c<S>(SPi[is]), acc);
        if (F.has0) v = v - c0 * to_c<S>(SPi0[is]);
        out[idx] = to_d(v * (R)(d.U * d.T * (CH == CH_T ? -1.0 : 1.0)));
    }
}
template <class S, bool V0>
__global__ void k_bse_K1_new_all(VertPT<S> Fin, BubbleP B, const cplx* SPi, const cplx* SPi0, ChanWork cw, Dims d) {
    const VertPT<S> F = vert_spec<V0>(Fin);
    const size_t nS = (size_t)d.Nq * d.NPO;
    switch (blockIdx.y) {
        case CH_P: bse_K1_new_body<CH_P>(F, B.pp, B.pp0, SPi, SPi0, cw.out[CH_P], cw.items[CH_P], cw.nitems[CH_P], d); break;
        case CH_T: bse_K1_new_body<CH_T>(F, B.ph, B.ph0, SPi + nS, SPi0 + nS, cw.out[CH_T], cw.items[CH_T], cw.nitems[CH_T], d); break;
        default:   bse_K1_new_body<CH_A>(F, B.ph, B.ph0, SPi + nS, SPi0 + nS, cw.out[CH_A], cw.items[CH_A], cw.nitems[CH_A], d); break;
    }
}
template <class S, bool V0>
__global__ void k_bse_K2_new_all(VertPT<S> Fin, BubbleP B, const cplx* SPi, const cplx* SPi0, ChanWork cw, Dims d) {
    const VertPT<S> F = vert_spec<V0>(Fin);
    const size_t nS = (size_t)d.Nq * d.NPO;
    switch (blockIdx.y) {
        case CH_P: bse_K2_new_body<CH_P>(F, B.pp, B.pp0, SPi, SPi0, cw.out[CH_P], cw.items[CH_P], cw.nitems[CH_P], d); break;
        case CH_T: bse_K2_new_body<CH_T>(F, B.ph, B.ph0, SPi + nS, SPi0 + nS, cw.out[CH_T], cw.items[CH_T], cw.nitems[CH_T], d); break;
        default:   bse_K2_new_body<CH_A>(F, B.ph, B.ph0, SPi + nS, SPi0 + nS, cw.out[CH_A], cw.items[CH_A], cw.nitems[CH_A], d); break;
    }
}

// ---------------------------------------------------------------------------------------------
// All-channel launches: blockIdx.y selects the channel (0 = p, 1 = t, 2 = a; SDE: 0 = pp, 1 = ph).
// ---------------------------------------------------------------------------------------------
template <class S, bool TAN, bool V0>
__global__ void k_bse_K1_all(VertPT<S> Fin, FLPT<S> FL, BubbleP B, const cplx* SX, ChanWork cw, Dims d,
                             TanArgsT<S> Tin) {
    const VertPT<S> F = vert_spec<V0>(Fin);
    const TanArgsT<S> T = tan_spec<V0>(Tin);
    switch (blockIdx.y) {
        case CH_P: bse_K1_body<CH_P, S, TAN>(F, FL, B.pp, B.pp0, SX, cw.out[CH_P], cw.items[CH_P], cw.nitems[CH_P], cw.acc, d, T); break;
        case CH_T: bse_K1_body<CH_T, S, TAN>(F, FL, B.ph, B.ph0, SX, cw.out[CH_T], cw.items[CH_T], cw.nitems[CH_T], cw.acc, d, T); break;
        default:   bse_K1_body<CH_A, S, TAN>(F, FL, B.ph, B.ph0, SX, cw.out[CH_A], cw.items[CH_A], cw.nitems[CH_A], cw.acc, d, T); break;
    }
}
template <class S, bool V0>
__global__ void k_bse_L_K2_all(VertPT<S> Fin, BubbleP B, ChanWork cw, Dims d) {
    const VertPT<S> F = vert_spec<V0>(Fin);
    switch (blockIdx.y) {
        case CH_P: bse_L_K2_body<CH_P>(F, B.pp0, cw.out[CH_P], cw.items[CH_P], cw.nitems[CH_P], d); break;
        case CH_T: bse_L_K2_body<CH_T>(F, B.ph0, cw.out[CH_T], cw.items[CH_T], cw.nitems[CH_T], d); break;
        default:   bse_L_K2_body<CH_A>(F, B.ph0, cw.out[CH_A], cw.items[CH_A], cw.nitems[CH_A], d); break;
    }
}
template <class S, bool TAN, bool V0>
__global__ void __launch_bounds__(512) k_bse_K2_all(VertPT<S> Fin, FLPT<S> FL, BubbleP B, const cplx* SX, ChanWork cw,
                                                    Dims d, TanArgsT<S> Tin) {
    const VertPT<S> F = vert_spec<V0>(Fin);
    const TanArgsT<S> T = tan_spec<V0>(Tin);
    extern __shared__ __align__(16) unsigned char k2_smem[];
    S* tab = reinterpret_cast<S*>(k2_smem);
    switch (blockIdx.y) {
        case CH_P: bse_K2_row<CH_P, S, TAN>(F, FL, B.pp, B.pp0, SX, cw.out[CH_P], cw.items[CH_P], cw.gstart[CH_P], cw.ngroups[CH_P], cw.acc, d, T, tab); break;
        case CH_T: bse_K2_row<CH_T, S, TAN>(F, FL, B.ph, B.ph0, SX, cw.out[CH_T], cw.items[CH_T], cw.gstart[CH_T], cw.ngroups[CH_T], cw.acc, d, T, tab); break;
        default:   bse_K2_row<CH_A, S, TAN>(F, FL, B.ph, B.ph0, SX, cw.out[CH_A], cw.items[CH_A], cw.gstart[CH_A], cw.ngroups[CH_A], cw.acc, d, T, tab); break;
    }
}
template <class S, bool TAN, bool V0>
__global__ void k_sde_L_all(VertPT<S> Fin, BubbleP B, const cplx* SPpp, const cplx* SPph, ChanWork cw, int use_vertex,
                            double ref_scale, Dims d, TanArgsT<S> Tin) {
    const VertPT<S> F = vert_spec<V0>(Fin);
    const TanArgsT<S> T = tan_spec<V0>(Tin);
    if (blockIdx.y == 0)
        sde_L_body<0, S, TAN>(F, B.pp, SPpp, cw.out[0], cw.items[0], cw.nitems[0], use_vertex, ref_scale, cw.acc, d, T);
    else sde_L_body<1, S, TAN>(F, B.ph, SPph, cw.out[1], cw.items[1], cw.nitems[1], use_vertex, ref_scale, cw.acc, d, T);
}

// Finalize of one vertex class for the three channels (out-of-place from the representative
// values): out_c[i] = op_c(raw_c[rep_c(i)]) (SymmetryGroup broadcast), then for K2 the FL terms of
// BSE_K2! (src/BSEa/BSEa_K2.jl:95-101), then the t-channel pSp recombination (γtd + γa)/2
// (src/BSE_templates.jl:35-38).  Slots are indexed by channel; an absent slot has out = nullptr.
__global__ void k_finalize3(Finalize3 f, int k2_epilogue, int t_recombine, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    cplx v[3];
    uint32_t e_prev = 0;
    const uint32_t* map_prev = nullptr;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        v[c] = mk(0, 0);
        if (!f.out[c]) continue;
        if (f.map[c]) {
            // the t and a channels share the ph group: its map entry is read once
            const uint32_t e = (f.map[c] == map_prev) ? e_prev : f.map[c][i];
            map_prev = f.map[c];
            e_prev = e;
            v[c] = apply_op((int)(e & 3u), ld16(f.raw[c] + (e >> 2)));
        } else {
            v[c] = ld16(f.raw[c] + i);
        }
    }
    if (k2_epilogue) {
        const cplx flt = ld16(f.FL[CH_T] + i), fla = ld16(f.FL[CH_A] + i);
        v[CH_P] += ld16(f.FL[CH_P] + i);
        v[CH_A] += fla;
        v[CH_T] += cplx{twice_exact(flt.x), twice_exact(flt.y)};
        v[CH_T] -= fla;
    }
    if (t_recombine) {  // (γtd + γa)/2
        const cplx s = v[CH_T] + v[CH_A];
        v[CH_T] = cplx{half_exact(s.x), half_exact(s.y)};
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (f.out[c]) st16(f.out[c] + i, v[c]);
        if (f.outf[c]) f.outf[c][i] = to_c<cplxf>(v[c]);
    }
}

// Σ_inner in real space (src/nonlocal/SDE.jl:208-280; local src/SDE.jl:241-263 is the L = 1 case):
//   Σ_R(ν, R) = Σ_Ω [G(-R, Ω-ν) Lpp(R, Ω, ν) + G(R, Ω+ν) Lph(-R, Ω, ν)],  L(R) = (1/N) Σ_P L(P) e^{-iP·R},
//   Σ(ν, k) = T Σ_R e^{+ik·R} Σ_R(ν, R)   (the k transform is launch_fft2).  For L_G = L the ±L/2
//   half weights of the reference's R scan sum to one per site.  Warp per (R, ν), lanes over Ω.
// TAN: the tangent dΣ_R = Σ_Ω [dG L + G dL] from tGR and the transformed tangent tLppR, tLphR.
template <bool TAN>
__global__ void k_sde_sigma_R(const cplx* GR, const cplx* LppR, const cplx* LphR, const cplx* tGR, const cplx* tLppR,
                              const cplx* tLphR, cplx* SR, Dims d) {
    const size_t w = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int NR = d.L * d.L;
    if (w >= (size_t)NR * d.NG) return;
    const int nu = (int)(w % d.NG) - d.nG, R = (int)(w / d.NG);
    const int L = d.L, Rx = R % L, Ry = R / L;
    const int mR = ((L - Rx) % L) + L * ((L - Ry) % L);
    cplx acc = mk(0, 0);
    if (fin(nu, d.n2n)) {
        for (int t = lane; t < d.N2O; t += 32) {
            const int m = t - (d.n2O - 1);
            const int a = m - nu - 1, b = m + nu;
            if (fin(a, d.nG)) {
                const size_t ig = ixG(d, mR, a), il = ix2(d, R, m, nu);
                acc = TAN ? cfma(tGR[ig], LppR[il], cfma(GR[ig], tLppR[il], acc)) : cfma(GR[ig], LppR[il], acc);
            }
            if (fin(b, d.nG)) {
                const size_t ig = ixG(d, R, b), il = ix2(d, mR, m, nu);
                acc = TAN ? cfma(tGR[ig], LphR[il], cfma(GR[ig], tLphR[il], acc)) : cfma(GR[ig], LphR[il], acc);
            }
        }
    }
    acc = warp_sum(acc);
    if (lane == 0) SR[w] = acc;
}

// U² term (src/SDE.jl:328-364, src/nonlocal/SDE.jl:400-447), factorised:
//   C_R(s) = Σ_{n1} G(-R, n1) G(R, n1 + s);   Σ_U²(ν, R) = U² T² Σ_{n2} G(R, n2) C_R(ν - n2)
// GR layout [R][ν] (G(R)); s in [-(2nG-1), 2nG-1].
// TAN: tangents dC from tGR (product rule), then dΣ_U² = U² T² Σ [dG C + G dC].
template <bool TAN>
__global__ void k_u2_corr(const cplx* GR, const cplx* tGR, cplx* C, Dims d) {
    const int NS = 2 * d.NG - 1;
    const size_t w = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int NR = d.L * d.L;
    if (w >= (size_t)NR * NS) return;
    const int s = (int)(w % NS) - (d.NG - 1), R = (int)(w / NS);
    const int L = d.L, Rx = R % L, Ry = R / L;
    const int mR = ((L - Rx) % L) + L * ((L - Ry) % L);
    cplx acc = mk(0, 0);
    for (int n1 = -d.nG + lane; n1 < d.nG; n1 += 32) {
        const int n3 = n1 + s;
        if (!fin(n3, d.nG)) continue;
        const size_t i1 = ixG(d, mR, n1), i3 = ixG(d, R, n3);
        acc = TAN ? cfma(tGR[i1], GR[i3], cfma(GR[i1], tGR[i3], acc)) : cfma(GR[i1], GR[i3], acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) C[w] = acc;
}
template <bool TAN>
__global__ void k_u2_sum(const cplx* GR, const cplx* C, const cplx* tGR, const cplx* tC, cplx* out, Dims d) {
    const int NS = 2 * d.NG - 1;
    const size_t w = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int NR = d.L * d.L;
    if (w >= (size_t)NR * d.NG) return;
    const int nu = (int)(w % d.NG) - d.nG, R = (int)(w / d.NG);
    cplx acc = mk(0, 0);
    for (int n2 = -d.nG + lane; n2 < d.nG; n2 += 32) {
        const int s = nu - n2;  // in [-(2nG-1), 2nG-1]
        const size_t ig = ixG(d, R, n2), ic = (size_t)R * NS + (s + d.NG - 1);
        acc = TAN ? cfma(tGR[ig], C[ic], cfma(GR[ig], tC[ic], acc)) : cfma(GR[ig], C[ic], acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) out[w] = acc * (d.U * d.U * d.T * d.T);
}
// Σ assembly (src/SDE.jl:3-33, 219-283): Σ = op(Σin + Σ_U²)[rep] + H  (+ fdPA: - C0 + Σ0 - H0)
__global__ void k_sigma_assemble(const cplx* Sin, const cplx* SU2, const uint32_t* map, const double* occ,
                                 const cplx* C0, const cplx* Sig0, cplx* Sig, double U, int hartree, int fdpa,
                                 double n0, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    size_t r = i;
    int op = 0;
    if (map) { const uint32_t e = map[i]; r = e >> 2; op = (int)(e & 3u); }
    cplx v = apply_op(op, Sin[r] + SU2[r]);
    if (hartree) v += mk(0.0, (*occ - 0.5) * U);
    if (fdpa) {  // 1: the reference system's Hartree term subtracted twice (src/SDE.jl:9-24); 2: once
        v = v + (C0[i] * -1.0);
        v += Sig0[i];
        if (hartree) {
            v = v + mk(0.0, -(n0 - 0.5) * U);
            if (fdpa == 1) v = v + mk(0.0, -(n0 - 0.5) * U);
        }
    }
    Sig[i] = v;
}

// ---------------------------------------------------------------------------------------------
// State-vector helpers
// ---------------------------------------------------------------------------------------------
__global__ void k_gather(cplx* dst, const cplx* src, const uint32_t* perm, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[perm[i]];
}
__global__ void k_scatter(cplx* dst, const cplx* src, const uint32_t* perm, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) dst[perm[i]] = src[i];
}
// fx = y - x ; g = x + beta fx ; partial max|fx|² per block (the host takes the square root of the
// maximum, which equals the maximum of |fx| since the square root is monotone).  x == nullptr
// reads as zero; fx and g may be nullptr (not written).
__global__ void k_residual(const cplx* y, const cplx* x, cplx* fx, cplx* g, double beta, double* pmax, size_t n) {
    __shared__ double red[256];
    double mx = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const cplx f = x ? y[i] - x[i] : y[i];
        if (fx) fx[i] = f;
        if (g && x) g[i] = x[i] + f * beta;
        mx = fmax(mx, f.x * f.x + f.y * f.y);
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) pmax[blockIdx.x] = red[0];
}
// out[i] = y[perm[i]] - x[perm[i]]: the residual of the device-layout states in reference order
__global__ void k_gather_sub(cplx* out, const cplx* y, const cplx* x, const uint32_t* perm, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) {
        const uint32_t j = perm[i];
        out[i] = y[j] - x[j];
    }
}
__global__ void k_sub(cplx* out, const cplx* a, const cplx* b, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] - b[i];
}
// χ_r from the K1 arrays ([P][Ω], identical to the reference's column-major [Ω, P]):
// m: γa.K1/U², d: (γa.K1 - 2γt.K1)/U², s: -2γp.K1/U²; local != 0 averages over P (fixed order).
__global__ void k_chi(const cplx* K1p, const cplx* K1t, const cplx* K1a, int which, double invU2, int NO, int Nq,
                      int local, cplx* out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    auto chi = [&](size_t i) -> cplx {
        if (which == 0) return K1a[i] * invU2;
        if (which == 1) return (K1a[i] - K1t[i] * 2.0) * invU2;
        return K1p[i] * (-2.0 * invU2);
    };
    if (local) {
        if (j >= NO) return;
        cplx s = mk(0.0, 0.0);
        for (int P = 0; P < Nq; ++P) s += chi((size_t)P * NO + j);
        out[j] = s * (1.0 / Nq);
    } else if ((size_t)j < (size_t)NO * Nq) {
        out[j] = chi(j);
    }
}
// FP64 FMA throughput calibration: four independent FMA chains per thread
__global__ void k_fp64_rate(double* out, double a, double b, int iters) {
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    for (int i = 0; i < iters; ++i) { x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b); }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}
// count of non-finite values
__global__ void k_nonfinite(const cplx* a, size_t n, unsigned int* count) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n && !(isfinite(a[i].x) && isfinite(a[i].y))) atomicAdd(count, 1u);
}

// =============================================================================================
// Launchers
// =============================================================================================
static inline unsigned blocks_for(size_t n, int t) { return (unsigned)((n + t - 1) / t); }
cudaError_t launch_fft2(cudaStream_t s, const cplx* in, cplx* out, int rows, int sign, double scale,
                        const cplx* tw_sign, const Dims& d);
#define LAUNCH_CHECK() do { cudaError_t e_ = cudaGetLastError(); if (e_ != cudaSuccess) return e_; } while (0)

cudaError_t launch_dyson(cudaStream_t s, cplx* G, const cplx* Sig, const cplx* Gb, size_t n) {
    k_dyson<<<blocks_for(n, 256), 256, 0, s>>>(G, Sig, Gb, n);
    LAUNCH_CHECK(); return cudaSuccess;
}
cudaError_t launch_occupation(cudaStream_t s, const cplx* G, size_t n, double T, int Nk, double* out) {
    k_occupation<<<1, 1024, 0, s>>>(G, n, T, Nk, out);
    LAUNCH_CHECK(); return cudaSuccess;
}
cudaError_t launch_g_realspace(cudaStream_t s, const cplx* G, cplx* GR, const cplx* tw, const Dims& d) {
    return launch_fft2(s, G, GR, d.NG, -1, 1.0 / (d.L * d.L), tw, d);
}
// DFT bubble (any L): TV fermion frequencies per CTA, (4 TV L² + L) values of shared memory
template <bool TAN, class C, class G>
static cudaError_t launch_bubble_dft(cudaStream_t s, const G* GR, const G* tGR, cplx* pp, cplx* ph, const cplx* twp,
                                     const Dims& d) {
    const int NR = d.L * d.L;
    int tv = 32;
    while (tv > 1 && (size_t)(4 * tv * NR + d.L) * sizeof(C) > 160 * 1024) tv >>= 1;
    const size_t shm = (size_t)(4 * tv * NR + d.L) * sizeof(C);
    static SmemRecord shm_set;  // raised once, outside graph capture (first call is from fdga_finalize)
    cudaError_t e = raise_smem_limit(k_bubble_nl<TAN, C, G>, shm_set, shm);
    if (e != cudaSuccess) return e;
    dim3 grid((d.NPw + tv - 1) / tv, d.NPO);
    k_bubble_nl<TAN, C, G><<<grid, 256, shm, s>>>(GR, tGR, pp, ph, twp, d, tv);
    LAUNCH_CHECK(); return cudaSuccess;
}
int bubble_tile(const Dims& d) {
    const int NR = d.L * d.L;
    int tv = 32;
    while (tv > 1 && (size_t)4 * tv * NR * sizeof(cplx) > 160 * 1024) tv >>= 1;
    return tv;
}
template <int L, bool TAN>
static cudaError_t launch_bubble_fft(cudaStream_t s, const cplx* GR, const cplx* tGR, cplx* pp, cplx* ph,
                                     const Dims& d) {
    constexpr int BS = L * (L + 1) + 1;
    int tv = 32;
    while (tv > 1 && (size_t)2 * tv * BS * sizeof(cplx) > 80 * 1024) tv >>= 1;
    const size_t shm = (size_t)2 * tv * BS * sizeof(cplx);
    static SmemRecord shm_set;  // raised once, outside graph capture (first call is from fdga_finalize)
    cudaError_t e = raise_smem_limit(k_bubble_fft<L, cplx, cplx, TAN>, shm_set, shm);
    if (e != cudaSuccess) return e;
    dim3 grid((d.NPw + tv - 1) / tv, d.NPO);
    k_bubble_fft<L, cplx, cplx, TAN><<<grid, 256, shm, s>>>(GR, tGR, pp, ph, d, tv);
    return cudaGetLastError();
}
// FP32 form (mixed map) from the FP32 copy of G(R); its tile fits the default 48 KB of shared memory
template <int L, bool TAN>
static cudaError_t launch_bubble_fft_f32(cudaStream_t s, const cplxf* GR, const cplxf* tGR, cplx* pp, cplx* ph,
                                         const Dims& d) {
    constexpr int BS = L * (L + 1) + 1;
    int tv = 32;
    while (tv > 1 && (size_t)2 * tv * BS * sizeof(cplxf) > 48 * 1024) tv >>= 1;
    const size_t shm = (size_t)2 * tv * BS * sizeof(cplxf);
    dim3 grid((d.NPw + tv - 1) / tv, d.NPO);
    k_bubble_fft<L, cplxf, cplxf, TAN><<<grid, 256, shm, s>>>(GR, tGR, pp, ph, d, tv);
    return cudaGetLastError();
}
bool bubble_f32_supported(const Dims& d) { return !d.local; }
template <bool TAN>
static cudaError_t bubble_f32_t(cudaStream_t s, const cplxf* GRf, const cplxf* tGRf, cplx* pp, cplx* ph,
                                const cplx* twp, const Dims& d) {
    switch (d.L) {
        case 2: return launch_bubble_fft_f32<2, TAN>(s, GRf, tGRf, pp, ph, d);
        case 4: return launch_bubble_fft_f32<4, TAN>(s, GRf, tGRf, pp, ph, d);
        case 8: return launch_bubble_fft_f32<8, TAN>(s, GRf, tGRf, pp, ph, d);
        case 16: return launch_bubble_fft_f32<16, TAN>(s, GRf, tGRf, pp, ph, d);
        case 32: return launch_bubble_fft_f32<32, TAN>(s, GRf, tGRf, pp, ph, d);
        case 3: return launch_bubble_fft_f32<3, TAN>(s, GRf, tGRf, pp, ph, d);
        case 6: return launch_bubble_fft_f32<6, TAN>(s, GRf, tGRf, pp, ph, d);
        case 12: return launch_bubble_fft_f32<12, TAN>(s, GRf, tGRf, pp, ph, d);
        case 24: return launch_bubble_fft_f32<24, TAN>(s, GRf, tGRf, pp, ph, d);
        default: return launch_bubble_dft<TAN, cplxf, cplxf>(s, GRf, tGRf, pp, ph, twp, d);
    }
}
cudaError_t launch_bubble_f32(cudaStream_t s, const cplxf* GRf, cplx* pp, cplx* ph, const cplx* twp, const Dims& d) {
    return bubble_f32_t<false>(s, GRf, nullptr, pp, ph, twp, d);
}
cudaError_t launch_bubble_f32_tan(cudaStream_t s, const cplxf* GRf, const cplxf* tGRf, cplx* tpp, cplx* tph,
                                  const cplx* twp, const Dims& d) {
    return bubble_f32_t<true>(s, GRf, tGRf, tpp, tph, twp, d);
}

cudaError_t set_fft_twiddles() {
    cplx tw[32];
    cplxf twf[32];
    for (int j = 0; j < 32; ++j) {
        tw[j] = mk(std::cos(2.0 * M_PI * j / 32.0), std::sin(2.0 * M_PI * j / 32.0));
        twf[j] = cplxf{(float)tw[j].x, (float)tw[j].y};
    }
    cudaError_t e = cudaMemcpyToSymbol(c_twp32, tw, sizeof(tw));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_twp32f, twf, sizeof(twf));
    cplx t96[96];
    cplxf t96f[96];
    for (int j = 0; j < 96; ++j) {
        t96[j] = mk(std::cos(2.0 * M_PI * j / 96.0), std::sin(2.0 * M_PI * j / 96.0));
        t96f[j] = cplxf{(float)t96[j].x, (float)t96[j].y};
    }
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_twp96, t96, sizeof(t96));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_twp96f, t96f, sizeof(t96f));
    return e;
}

template <bool TAN>
static cudaError_t bubble_t(cudaStream_t s, const cplx* G, const cplx* tG, const cplx* GR, const cplx* tGR, cplx* pp,
                            cplx* ph, const cplx* twp, const Dims& d) {
    if (d.local) {
        const size_t n = (size_t)d.NPO * d.NPw;
        k_bubble_local<TAN><<<blocks_for(n, 256), 256, 0, s>>>(G, tG, pp, ph, d);
        LAUNCH_CHECK(); return cudaSuccess;
    }
    switch (d.L) {
        case 2: return launch_bubble_fft<2, TAN>(s, GR, tGR, pp, ph, d);
        case 4: return launch_bubble_fft<4, TAN>(s, GR, tGR, pp, ph, d);
        case 8: return launch_bubble_fft<8, TAN>(s, GR, tGR, pp, ph, d);
        case 16: return launch_bubble_fft<16, TAN>(s, GR, tGR, pp, ph, d);
        case 32: return launch_bubble_fft<32, TAN>(s, GR, tGR, pp, ph, d);
        case 3: return launch_bubble_fft<3, TAN>(s, GR, tGR, pp, ph, d);
        case 6: return launch_bubble_fft<6, TAN>(s, GR, tGR, pp, ph, d);
        case 12: return launch_bubble_fft<12, TAN>(s, GR, tGR, pp, ph, d);
        case 24: return launch_bubble_fft<24, TAN>(s, GR, tGR, pp, ph, d);
        default: break;
    }
    return launch_bubble_dft<TAN, cplx, cplx>(s, GR, tGR, pp, ph, twp, d);
}
cudaError_t launch_bubble(cudaStream_t s, const cplx* G, const cplx* GR, cplx* pp, cplx* ph, const cplx* twp,
                          const Dims& d) {
    return bubble_t<false>(s, G, nullptr, GR, nullptr, pp, ph, twp, d);
}
cudaError_t launch_bubble_tan(cudaStream_t s, const cplx* G, const cplx* tG, const cplx* GR, const cplx* tGR,
                              cplx* tpp, cplx* tph, const cplx* twp, const Dims& d) {
    return bubble_t<true>(s, G, tG, GR, tGR, tpp, tph, twp, d);
}

template <int L>
static cudaError_t launch_fft2_tpl(cudaStream_t s, const cplx* in, cplx* out, int rows, int sign, double scale) {
    constexpr int BS = L * (L + 1) + 1, NR = L * L;
    // rows per CTA: enough CTAs to cover the GPU (two per SM for 152 SMs), within 48 KB of tile
    int tr = 1;
    while (tr < 32 && (size_t)(2 * tr) * BS * sizeof(cplx) <= 48 * 1024 && (rows + 2 * tr - 1) / (2 * tr) >= 304) tr *= 2;
    const size_t shm = (size_t)tr * BS * sizeof(cplx);
    const int threads = std::min(256, std::max(32, ((tr * NR + 31) / 32) * 32));
    k_fft2_rows<L><<<(unsigned)((rows + tr - 1) / tr), threads, shm, s>>>(in, out, rows, sign, scale, tr);
    return cudaGetLastError();
}
cudaError_t launch_fft2(cudaStream_t s, const cplx* in, cplx* out, int rows, int sign, double scale,
                        const cplx* tw_sign, const Dims& d) {
    switch (d.L) {
        case 1: return launch_fft2_tpl<1>(s, in, out, rows, sign, scale);
        case 2: return launch_fft2_tpl<2>(s, in, out, rows, sign, scale);
        case 4: return launch_fft2_tpl<4>(s, in, out, rows, sign, scale);
        case 8: return launch_fft2_tpl<8>(s, in, out, rows, sign, scale);
        case 16: return launch_fft2_tpl<16>(s, in, out, rows, sign, scale);
        case 3: return launch_fft2_tpl<3>(s, in, out, rows, sign, scale);
        case 6: return launch_fft2_tpl<6>(s, in, out, rows, sign, scale);
        case 12: return launch_fft2_tpl<12>(s, in, out, rows, sign, scale);
        case 24: return launch_fft2_tpl<24>(s, in, out, rows, sign, scale);
        default: break;
    }
    const int L = d.L, BS = L * (L + 1) + 1;
    int tr = 16;
    while (tr > 1 && (size_t)(2 * tr * BS + L) * sizeof(cplx) > 48 * 1024) tr >>= 1;
    if ((size_t)(2 * tr * BS + L) * sizeof(cplx) <= 48 * 1024) {
        const size_t shm = (size_t)(2 * tr * BS + L) * sizeof(cplx);
        k_dft2_sep<<<(unsigned)((rows + tr - 1) / tr), 256, shm, s>>>(in, out, rows, L, tw_sign, scale, tr);
        LAUNCH_CHECK(); return cudaSuccess;
    }
    const size_t n = (size_t)L * L * rows;
    k_dft2_rows<<<blocks_for(n, 128), 128, 0, s>>>(in, out, rows, L, tw_sign, scale);
    LAUNCH_CHECK(); return cudaSuccess;
}

cudaError_t launch_tail_const(cudaStream_t s, cplx* T0, const Dims& d) {
    k_tail_const<<<blocks_for((size_t)2 * d.NPO * 32, 128), 128, 0, s>>>(T0, d);
    LAUNCH_CHECK(); return cudaSuccess;
}
cudaError_t launch_rowsum(cudaStream_t s, const cplx* A0, const cplx* A1, const cplx* GR, cplx* SRtmp, const cplx* twp,
                          cplx* S0, cplx* S1, const Dims& d, const cplx* T0, const cplxf* GRf) {
    if (d.nPw == d.nPn) {  // the full mesh is stored: sum the rows
        dim3 grid((unsigned)(d.Nq * d.NPO), 2);
        k_rowsum<<<grid, 256, 0, s>>>(A0, A1, S0, S1, d.NPw);
        LAUNCH_CHECK(); return cudaSuccess;
    }
    const int NR = d.L * d.L;
    const unsigned nb = blocks_for((size_t)2 * d.NPO * NR * 32, 128);
    if (GRf) k_pisum_R<cplxf, cplxf, false><<<nb, 128, 0, s>>>(GRf, nullptr, T0, SRtmp, d);
    else k_pisum_R<cplx, cplx, false><<<nb, 128, 0, s>>>(GR, nullptr, T0, SRtmp, d);
    LAUNCH_CHECK();
    // S^w[P][Ω] = Σ_R e^{+2πi P·R/L} SR[w][R][Ω]
    cudaError_t e = launch_fft2(s, SRtmp, S0, d.NPO, +1, 1.0, twp, d);
    if (e != cudaSuccess) return e;
    e = launch_fft2(s, SRtmp + (size_t)NR * d.NPO, S1, d.NPO, +1, 1.0, twp, d);
    if (e != cudaSuccess) return e;
    return cudaSuccess;
}
cudaError_t launch_sx(cudaStream_t s, const BubbleP& B, const cplx* SPi, const cplx* SPi0, const FLP& FL,
                      const VertP& F0v, cplx* SX, const Dims& d) {
    const size_t n = (size_t)3 * d.Nq * d.NPO * 32;
    k_sx<<<blocks_for(n, 128), 128, 0, s>>>(B.pp, B.ph, B.pp0, B.ph0, SPi, SPi0, FL, F0v, SX, d);
    LAUNCH_CHECK(); return cudaSuccess;
}

cudaError_t launch_qavg(cudaStream_t s, const ChanArrays& in, const ChanArraysW& out, const Dims& d) {
    const size_t per = std::max((size_t)d.N1, std::max((size_t)d.N2O * d.N2n, (size_t)d.N3O * d.N3n * d.N3n));
    dim3 grid(blocks_for(per, 256), 9);
    k_qavg<<<grid, 256, 0, s>>>(in, out, d);
    LAUNCH_CHECK(); return cudaSuccess;
}
template <class S>
static cudaError_t build_cache_t(cudaStream_t s, const VertPT<S>& F, const Caches& C, const int* blocks, int nblocks,
                                 const Dims& d) {
    const size_t n = (size_t)nblocks * d.N3n * d.N3n;
    if (F.has0) k_build_cache<S, true><<<blocks_for(n, 128), 128, 0, s>>>(F, C, blocks, nblocks, d);
    else k_build_cache<S, false><<<blocks_for(n, 128), 128, 0, s>>>(F, C, blocks, nblocks, d);
    LAUNCH_CHECK(); return cudaSuccess;
}
cudaError_t launch_build_cache(cudaStream_t s, const VertP& F, const Caches& C, const int* blocks, int nblocks,
                               const Dims& d) {
    return build_cache_t(s, F, C, blocks, nblocks, d);
}
cudaError_t launch_build_cache(cudaStream_t s, const VertPF& F, const Caches& C, const int* blocks, int nblocks,
                               const Dims& d) {
    return build_cache_t(s, F, C, blocks, nblocks, d);
}
// K2 rows: one CTA per (channel, P, Ω) row of representatives
static unsigned row_grid(const ChanWork& cw, int nch) {
    int mx = 0;
    for (int c = 0; c < nch; ++c) mx = std::max(mx, cw.ngroups[c]);
    return (unsigned)std::max(mx, 1);
}
// 4 warps per row; 16 when the launch has fewer than four rows per SM of GB300 (the local solver,
// whose rows are only the NΩ2 bosonic frequencies)
static unsigned row_threads(const ChanWork& cw, int nch) { return row_grid(cw, nch) * nch < 4 * 152 ? 512 : 128; }
template <class S, bool TAN>
static size_t k2_row_smem(const Dims& d) {
    return (size_t)(TAN ? 2 : 1) * 2 * k2_table_half(d) * sizeof(S);
}
template <class K>
static cudaError_t k2_smem_attr(K kernel, size_t smem) {
    if (smem > 227 * 1024) return cudaErrorInvalidValue;
    static SmemRecord raised;  // one record per kernel instantiation
    return raise_smem_limit(kernel, raised, smem);
}
static unsigned warp_grid(const ChanWork& cw, int nch) {
    int mx = 0;
    for (int c = 0; c < nch; ++c) mx = std::max(mx, cw.nitems[c]);
    return blocks_for((size_t)mx * 32, 128);
}
// each vertex-evaluating kernel is launched in its V0 = F.has0 instantiation (see vert_spec)
template <class K>
static cudaError_t k2_launch_attr(K k_plain, K k_v0, bool v0, size_t smem) {
    return k2_smem_attr(v0 ? k_v0 : k_plain, smem);
}
#define FDGA_VERTEX_LAUNCHERS(VT, FT, TT, ST)                                                                       \
    cudaError_t launch_bse_K1_all(cudaStream_t s, const VT& F, const FT& FL, const BubbleP& B, const cplx* SX,    \
                                  const ChanWork& cw, const Dims& d) {                                             \
        const dim3 g(warp_grid(cw, 3), 3);                                                                          \
        if (F.has0) k_bse_K1_all<ST, false, true><<<g, 128, 0, s>>>(F, FL, B, SX, cw, d, TT{});                     \
        else k_bse_K1_all<ST, false, false><<<g, 128, 0, s>>>(F, FL, B, SX, cw, d, TT{});                           \
        LAUNCH_CHECK(); return cudaSuccess;                                                                         \
    }                                                                                                               \
    cudaError_t launch_bse_L_K2_all(cudaStream_t s, const VT& F, const BubbleP& B, const ChanWork& cw,             \
                                    const Dims& d) {                                                                \
        const dim3 g(warp_grid(cw, 3), 3);                                                                          \
        if (F.has0) k_bse_L_K2_all<ST, true><<<g, 128, 0, s>>>(F, B, cw, d);                                        \
        else k_bse_L_K2_all<ST, false><<<g, 128, 0, s>>>(F, B, cw, d);                                              \
        LAUNCH_CHECK(); return cudaSuccess;                                                                         \
    }                                                                                                               \
    cudaError_t launch_bse_K2_all(cudaStream_t s, const VT& F, const FT& FL, const BubbleP& B, const cplx* SX,    \
                                  const ChanWork& cw, const Dims& d) {                                             \
        const size_t smem = k2_row_smem<ST, false>(d);                                                             \
        cudaError_t e = k2_launch_attr(k_bse_K2_all<ST, false, false>, k_bse_K2_all<ST, false, true>, F.has0, smem); \
        if (e != cudaSuccess) return e;                                                                             \
        const dim3 g(row_grid(cw, 3), 3);                                                                           \
        if (F.has0) k_bse_K2_all<ST, false, true><<<g, row_threads(cw, 3), smem, s>>>(F, FL, B, SX, cw, d, TT{});   \
        else k_bse_K2_all<ST, false, false><<<g, row_threads(cw, 3), smem, s>>>(F, FL, B, SX, cw, d, TT{});         \
        LAUNCH_CHECK(); return cudaSuccess;                                                                         \
    }                                                                                                               \
    cudaError_t launch_sde_L_all(cudaStream_t s, const VT& F, const BubbleP& B, const cplx* SPpp, const cplx* SPph, \
                                 const ChanWork& cw, int use_vertex, double ref_scale, const Dims& d) {             \
        const dim3 g(warp_grid(cw, 2), 2);                                                                          \
        if (F.has0) k_sde_L_all<ST, false, true><<<g, 128, 0, s>>>(F, B, SPpp, SPph, cw, use_vertex, ref_scale, d, TT{}); \
        else k_sde_L_all<ST, false, false><<<g, 128, 0, s>>>(F, B, SPpp, SPph, cw, use_vertex, ref_scale, d, TT{});  \
        LAUNCH_CHECK(); return cudaSuccess;                                                                         \
    }                                                                                                               \
    cudaError_t launch_bse_K1_tan(cudaStream_t s, const VT& F, const FT& FL, const BubbleP& B, const cplx* SX,    \
                                  const TT& T, const ChanWork& cw, const Dims& d) {                                \
        const dim3 g(warp_grid(cw, 3), 3);                                                                          \
        if (F.has0) k_bse_K1_all<ST, true, true><<<g, 128, 0, s>>>(F, FL, B, SX, cw, d, T);                         \
        else k_bse_K1_all<ST, true, false><<<g, 128, 0, s>>>(F, FL, B, SX, cw, d, T);                               \
        LAUNCH_CHECK(); return cudaSuccess;                                                                         \
    }                                                                                                               \
    cudaError_t launch_bse_K2_tan(cudaStream_t s, const VT& F, const FT& FL, const BubbleP& B, const cplx* SX,    \
                                  const TT& T, const ChanWork& cw, const Dims& d) {                                \
        const size_t smem = k2_row_smem<ST, true>(d);                                                              \
        cudaError_t e = k2_launch_attr(k_bse_K2_all<ST, true, false>, k_bse_K2_all<ST, true, true>, F.has0, smem);  \
        if (e != cudaSuccess) return e;                                                                             \
        const dim3 g(row_grid(cw, 3), 3);                                                                           \
        if (F.has0) k_bse_K2_all<ST, true, true><<<g, row_threads(cw, 3), smem, s>>>(F, FL, B, SX, cw, d, T);       \
        else k_bse_K2_all<ST, true, false><<<g, row_threads(cw, 3), smem, s>>>(F, FL, B, SX, cw, d, T);             \
        LAUNCH_CHECK(); return cudaSuccess;                                                                         \
    }                                                                                                               \
    cudaError_t launch_sde_L_tan(cudaStream_t s, const VT& F, const BubbleP& B, const cplx* SPpp, const cplx* SPph, \
                                 const TT& T, const ChanWork& cw, double ref_scale, const Dims& d) {                \
        const dim3 g(warp_grid(cw, 2), 2);                                                                          \
        if (F.has0) k_sde_L_all<ST, true, true><<<g, 128, 0, s>>>(F, B, SPpp, SPph, cw, 3, ref_scale, d, T);       \
        else k_sde_L_all<ST, true, false><<<g, 128, 0, s>>>(F, B, SPpp, SPph, cw, 1, ref_scale, d, T);             \
        LAUNCH_CHECK(); return cudaSuccess;                                                                         \
    }
#define FDGA_NEW_LAUNCHERS(VT, ST)                                                                                 \
    cudaError_t launch_bse_K1_new(cudaStream_t s, const VT& F, const BubbleP& B, const cplx* SPi, const cplx* SPi0,  \
                                  const ChanWork& cw, const Dims& d) {                                             \
        const dim3 g(warp_grid(cw, 3), 3);                                                                          \
        if (F.has0) k_bse_K1_new_all<ST, true><<<g, 128, 0, s>>>(F, B, SPi, SPi0, cw, d);                           \
        else k_bse_K1_new_all<ST, false><<<g, 128, 0, s>>>(F, B, SPi, SPi0, cw, d);                                 \
        LAUNCH_CHECK(); return cudaSuccess;                                                                         \
    }                                                                                                               \
    cudaError_t launch_bse_K2_new(cudaStream_t s, const VT& F, const BubbleP& B, const cplx* SPi, const cplx* SPi0,  \
                                  const ChanWork& cw, const Dims& d) {                                             \
        const dim3 g(warp_grid(cw, 3), 3);                                                                          \
        if (F.has0) k_bse_K2_new_all<ST, true><<<g, 128, 0, s>>>(F, B, SPi, SPi0, cw, d);                           \
        else k_bse_K2_new_all<ST, false><<<g, 128, 0, s>>>(F, B, SPi, SPi0, cw, d);                                 \
        LAUNCH_CHECK(); return cudaSuccess;                                                                         \
    }
FDGA_NEW_LAUNCHERS(VertP, cplx)
FDGA_NEW_LAUNCHERS(VertPF, cplxf)
#undef FDGA_NEW_LAUNCHERS
FDGA_VERTEX_LAUNCHERS(VertP, FLP, TanArgs, cplx)
FDGA_VERTEX_LAUNCHERS(VertPF, FLPF, TanArgsF, cplxf)
#undef FDGA_VERTEX_LAUNCHERS
cudaError_t launch_finalize3(cudaStream_t s, const Finalize3& f, int k2_epilogue, int t_recombine, size_t n) {
    k_finalize3<<<blocks_for(n, 256), 256, 0, s>>>(f, k2_epilogue, t_recombine, n);
    LAUNCH_CHECK(); return cudaSuccess;
}
template <int MODE, int TILE, int TCOL, class C, class ARGS>
static cudaError_t launch_k3_tile(cudaStream_t s, const ARGS& a, int nslots, const Dims& d) {
    const unsigned rt = (unsigned)((d.N3n + TILE - 1) / TILE), ct = (unsigned)((d.N3n + TCOL - 1) / TCOL);
    dim3 grid((unsigned)(nslots * a.nblocks), rt, ct);
    k_bse_K3_gemm<MODE, TILE, TCOL, C, ARGS><<<grid, (TILE / 2) * (TCOL / 2), 0, s>>>(a, d);
    return cudaGetLastError();
}
// Tile codes: 16, 24, 32 = square TILE x TILE output tiles; 100 + TILE = TILE rows x TILE/2
// columns (twice the CTAs, each forming only its own columns of M: better balance over the SMs
// for launches with few CTAs per SM, at twice the operand staging per flop; the autotuner decides,
// the default is square: measured on GB300 at Nν3 = 24, 675 blocks, the split is 7 % slower).
bool k3_tile_valid(int tile) { return tile == 16 || tile == 24 || tile == 32 || tile == 116 || tile == 124 || tile == 132; }
static int k3_default_tile(int N) { return N <= 16 ? 16 : (N <= 24 ? 24 : 32); }
template <int MODE, class C, class ARGS>
static cudaError_t launch_k3_mode(cudaStream_t s, const ARGS& a, int nslots, const Dims& d, int tile) {
    switch (tile) {
        case 16: return launch_k3_tile<MODE, 16, 16, C>(s, a, nslots, d);
        case 24: return launch_k3_tile<MODE, 24, 24, C>(s, a, nslots, d);
        case 116: return launch_k3_tile<MODE, 16, 8, C>(s, a, nslots, d);
        case 124: return launch_k3_tile<MODE, 24, 12, C>(s, a, nslots, d);
        case 132: return launch_k3_tile<MODE, 32, 16, C>(s, a, nslots, d);
        default: return launch_k3_tile<MODE, 32, 32, C>(s, a, nslots, d);
    }
}
template <class C, class ARGS>
static cudaError_t launch_bse_K3_t(cudaStream_t s, int mode, const ARGS& a, int nslots, const Dims& d, int tile) {
    if (!k3_tile_valid(tile)) tile = k3_default_tile(d.N3n);
    if (mode == 0) return launch_k3_mode<0, C>(s, a, nslots, d, tile);
    if (mode == 2) return launch_k3_mode<2, C>(s, a, nslots, d, tile);
    return launch_k3_mode<1, C>(s, a, nslots, d, tile);
}
cudaError_t launch_bse_K3(cudaStream_t s, int mode, const K3Args3& a, int nslots, const Dims& d, int mixed, int tile) {
    return mixed ? launch_bse_K3_t<cplxf>(s, mode, a, nslots, d, tile)
                 : launch_bse_K3_t<cplx>(s, mode, a, nslots, d, tile);
}
cudaError_t launch_bse_K3_f32(cudaStream_t s, int mode, const K3Args3F& a, int nslots, const Dims& d, int tile) {
    return launch_bse_K3_t<cplxf>(s, mode, a, nslots, d, tile);
}
__global__ void k_to_f32(const cplx* in, cplxf* out, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = to_c<cplxf>(in[i]);
}
cudaError_t launch_to_f32(cudaStream_t s, const cplx* in, cplxf* out, size_t n) {
    k_to_f32<<<blocks_for(n, 256), 256, 0, s>>>(in, out, n);
    LAUNCH_CHECK(); return cudaSuccess;
}
cudaError_t launch_sde_sigma(cudaStream_t s, const cplx* GR, const cplx* Lpp, const cplx* Lph, cplx* LR, cplx* SR,
                             cplx* S, const cplx* twm, const cplx* twp, const Dims& d) {
    const int rows = d.N2O * d.N2n, NR = d.L * d.L;
    const double invN = 1.0 / NR;
    cudaError_t e = launch_fft2(s, Lpp, LR, rows, -1, invN, twm, d);
    if (e == cudaSuccess) e = launch_fft2(s, Lph, LR + (size_t)NR * rows, rows, -1, invN, twm, d);
    if (e != cudaSuccess) return e;
    k_sde_sigma_R<false><<<blocks_for((size_t)NR * d.NG * 32, 128), 128, 0, s>>>(GR, LR, LR + (size_t)NR * rows, nullptr,
                                                                                 nullptr, nullptr, SR, d);
    LAUNCH_CHECK();
    return launch_fft2(s, SR, S, d.NG, +1, d.T, twp, d);
}
cudaError_t launch_sde_sigma_tan(cudaStream_t s, const cplx* GR, const cplx* LR, const cplx* tGR, const cplx* tLpp,
                                 const cplx* tLph, cplx* tLR, cplx* tSR, cplx* tS, const cplx* twm, const cplx* twp,
                                 const Dims& d) {
    const int rows = d.N2O * d.N2n, NR = d.L * d.L;
    const double invN = 1.0 / NR;
    cudaError_t e = launch_fft2(s, tLpp, tLR, rows, -1, invN, twm, d);
    if (e == cudaSuccess) e = launch_fft2(s, tLph, tLR + (size_t)NR * rows, rows, -1, invN, twm, d);
    if (e != cudaSuccess) return e;
    k_sde_sigma_R<true><<<blocks_for((size_t)NR * d.NG * 32, 128), 128, 0, s>>>(
        GR, LR, LR + (size_t)NR * rows, tGR, tLR, tLR + (size_t)NR * rows, tSR, d);
    LAUNCH_CHECK();
    return launch_fft2(s, tSR, tS, d.NG, +1, d.T, twp, d);
}
cudaError_t launch_u2(cudaStream_t s, const cplx* GR, cplx* C, cplx* SR, cplx* out, const cplx* twc, const Dims& d) {
    const int NR = d.L * d.L, NS = 2 * d.NG - 1;
    k_u2_corr<false><<<blocks_for((size_t)NR * NS * 32, 128), 128, 0, s>>>(GR, nullptr, C, d);
    LAUNCH_CHECK();
    k_u2_sum<false><<<blocks_for((size_t)NR * d.NG * 32, 128), 128, 0, s>>>(GR, C, nullptr, nullptr, SR, d);
    LAUNCH_CHECK();
    return launch_fft2(s, SR, out, d.NG, +1, 1.0, twc, d);
}
cudaError_t launch_u2_tan(cudaStream_t s, const cplx* GR, const cplx* C, const cplx* tGR, cplx* tC, cplx* tSR,
                          cplx* tout, const cplx* twc, const Dims& d) {
    const int NR = d.L * d.L, NS = 2 * d.NG - 1;
    k_u2_corr<true><<<blocks_for((size_t)NR * NS * 32, 128), 128, 0, s>>>(GR, tGR, tC, d);
    LAUNCH_CHECK();
    k_u2_sum<true><<<blocks_for((size_t)NR * d.NG * 32, 128), 128, 0, s>>>(GR, C, tGR, tC, tSR, d);
    LAUNCH_CHECK();
    return launch_fft2(s, tSR, tout, d.NG, +1, 1.0, twc, d);
}
cudaError_t launch_dyson_tan(cudaStream_t s, cplx* tG, const cplx* G, const cplx* tSig, size_t n) {
    k_dyson_tan<<<blocks_for(n, 256), 256, 0, s>>>(tG, G, tSig, n);
    LAUNCH_CHECK(); return cudaSuccess;
}
cudaError_t launch_sx_tan(cudaStream_t s, const cplx* Pipp, const cplx* Piph, const cplx* tPipp, const cplx* tPiph,
                          const cplx* tSPi, const FLP& FL, const FLP& tFL, const VertP& F0v, cplx* tSX,
                          const Dims& d) {
    const size_t n = (size_t)3 * d.Nq * d.NPO * 32;
    k_sx_tan<<<blocks_for(n, 128), 128, 0, s>>>(Pipp, Piph, tPipp, tPiph, tSPi, FL, tFL, F0v, tSX, d);
    LAUNCH_CHECK(); return cudaSuccess;
}
cudaError_t launch_rowsum_tan(cudaStream_t s, const cplx* tA0, const cplx* tA1, const cplx* GR, const cplx* tGR,
                              cplx* SRtmp, const cplx* twp, cplx* tS0, cplx* tS1, const Dims& d, const cplxf* GRf,
                              const cplxf* tGRf) {
    if (d.nPw == d.nPn) {  // the full mesh is stored: the row sums are linear in Π
        dim3 grid((unsigned)(d.Nq * d.NPO), 2);
        k_rowsum<<<grid, 256, 0, s>>>(tA0, tA1, tS0, tS1, d.NPw);
        LAUNCH_CHECK(); return cudaSuccess;
    }
    const int NR = d.L * d.L;
    const unsigned nb = blocks_for((size_t)2 * d.NPO * NR * 32, 128);
    if (GRf) k_pisum_R<cplxf, cplxf, true><<<nb, 128, 0, s>>>(GRf, tGRf, nullptr, SRtmp, d);
    else k_pisum_R<cplx, cplx, true><<<nb, 128, 0, s>>>(GR, tGR, nullptr, SRtmp, d);
    LAUNCH_CHECK();
    cudaError_t e = launch_fft2(s, SRtmp, tS0, d.NPO, +1, 1.0, twp, d);
    if (e != cudaSuccess) return e;
    return launch_fft2(s, SRtmp + (size_t)NR * d.NPO, tS1, d.NPO, +1, 1.0, twp, d);
}
cudaError_t launch_sigma_assemble(cudaStream_t s, const cplx* Sin, const cplx* SU2, const uint32_t* map,
                                  const double* occ, const cplx* C0, const cplx* Sig0, cplx* Sig, double U, int hartree,
                                  int fdpa, double n0, size_t n) {
    k_sigma_assemble<<<blocks_for(n, 256), 256, 0, s>>>(Sin, SU2, map, occ, C0, Sig0, Sig, U, hartree, fdpa, n0, n);
    LAUNCH_CHECK(); return cudaSuccess;
}
cudaError_t launch_gather(cudaStream_t s, cplx* dst, const cplx* src, const uint32_t* perm, size_t n) {
    k_gather<<<blocks_for(n, 256), 256, 0, s>>>(dst, src, perm, n);
    LAUNCH_CHECK(); return cudaSuccess;
}
cudaError_t launch_scatter(cudaStream_t s, cplx* dst, const cplx* src, const uint32_t* perm, size_t n) {
    k_scatter<<<blocks_for(n, 256), 256, 0, s>>>(dst, src, perm, n);
    LAUNCH_CHECK(); return cudaSuccess;
}
cudaError_t launch_residual(cudaStream_t s, const cplx* y, const cplx* x, cplx* fx, cplx* g, double beta, double* pmax,
                            int nblk, size_t n) {
    k_residual<<<nblk, 256, 0, s>>>(y, x, fx, g, beta, pmax, n);
    LAUNCH_CHECK(); return cudaSuccess;
}
cudaError_t launch_gather_sub(cudaStream_t s, cplx* out, const cplx* y, const cplx* x, const uint32_t* perm, size_t n) {
    k_gather_sub<<<blocks_for(n, 256), 256, 0, s>>>(out, y, x, perm, n);
    LAUNCH_CHECK(); return cudaSuccess;
}
cudaError_t launch_sub(cudaStream_t s, cplx* out, const cplx* a, const cplx* b, size_t n) {
    k_sub<<<blocks_for(n, 256), 256, 0, s>>>(out, a, b, n);
    LAUNCH_CHECK(); return cudaSuccess;
}
cudaError_t launch_chi(cudaStream_t s, const cplx* K1p, const cplx* K1t, const cplx* K1a, int which, double U,
                       int NO, int Nq, int local, cplx* out) {
    const size_t n = local ? (size_t)NO : (size_t)NO * Nq;
    k_chi<<<blocks_for(n, 256), 256, 0, s>>>(K1p, K1t, K1a, which, 1.0 / (U * U), NO, Nq, local, out);
    LAUNCH_CHECK(); return cudaSuccess;
}
// Self-check of d2f_rn against the hardware conversion: n inputs from a hash of the index --
// random bit patterns over all exponents, exact ties (the 29 dropped bits 1000...0) of both
// parities, values just below and above a tie, and the zero/subnormal/overflow/infinity/NaN edges.
__global__ void k_selftest_d2f(unsigned long long seed, size_t n, unsigned int* mismatches) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        unsigned long long z = (i + 1) * 0x9E3779B97F4A7C15ull + seed;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        unsigned long long b = z;
        switch (i % 8) {
            case 1: b = (z & ~0x1FFFFFFFull) | 0x10000000ull; break;          // tie
            case 2: b = (z & ~0x1FFFFFFFull) | 0x0FFFFFFFull; break;          // just below a tie
            case 3: b = (z & ~0x1FFFFFFFull) | 0x10000001ull; break;          // just above a tie
            case 4: b = (z & 0x800FFFFFFFFFFFFFull) | ((unsigned long long)(870 + (z >> 52) % 291) << 52); break;  // FP32 range edges
            case 5: b = (z & 0x800FFFFFFFFFFFFFull) | (((z >> 40) % 3 == 0 ? 0x7ffull : (z >> 40) % 3 == 1 ? 0ull : 0x47full) << 52); break;
            default: break;
        }
        const double x = __longlong_as_double((long long)b);
        const unsigned int a = __float_as_uint(d2f_rn(x)), h = __float_as_uint(__double2float_rn(x));
        const bool both_nan = isnan(x);
        if (a != h && !both_nan) atomicAdd(mismatches, 1u);
    }
}
cudaError_t selftest_d2f(size_t n, unsigned int* mismatches_host) {
    unsigned int* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(unsigned int));
    if (e != cudaSuccess) return e;
    e = cudaMemset(d, 0, sizeof(unsigned int));
    if (e == cudaSuccess) {
        k_selftest_d2f<<<1024, 256>>>(0x5DEECE66Dull, n, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(mismatches_host, d, sizeof(unsigned int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e;
}

cudaError_t measure_fp64_rate(float* ms, double* gflops) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int blocks = sms * 8, threads = 256, iters = 4096;
    double* buf = nullptr;
    e = cudaMalloc(&buf, (size_t)blocks * threads * sizeof(double));
    if (e != cudaSuccess) return e;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0);
        k_fp64_rate<<<blocks, threads>>>(buf, 0.999, 1e-3, iters);
        cudaEventRecord(e1);
        e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) break;
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        best = std::min(best, t);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    *ms = best;
    *gflops = 2.0 * 4.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e9;
    return e;
}
cudaError_t launch_nonfinite(cudaStream_t s, const cplx* a, size_t n, unsigned int* count) {
    k_nonfinite<<<blocks_for(n, 256), 256, 0, s>>>(a, n, count);
    LAUNCH_CHECK(); return cudaSuccess;
}

}  // namespace fdga
