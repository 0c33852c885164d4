// fdga_device.cuh -- device-side types, layouts and vertex evaluators of libfdga.
//
// Device layout (row-major, last index fastest; chosen so that each (P, Ω) block of a K3-shaped
// array is one contiguous Nν x Nν matrix and every ω-sum streams contiguous memory):
//   G-like  [k][ν]          (identical to the reference's column-major [ν, k])
//   Π       [P][Ω][ν]       ν over the stored window [-nPw, nPw) of the bubble mesh (every ω at
//                           which a BSE/SDE sum reads Π lies in it; full-mesh sums use row sums)
//   K1      [P][Ω]          K2 [P][Ω][ν]          K3 [P][Ω][ν][ν']
// The reference stores the same data column-major with Ω fastest; flatten/unflatten permute.
//
// Mesh-index arithmetic follows the reference conventions (src/types.jl, src/convention.jl):
// fermion n <-> (2n+1)πT on [-N, N-1]; boson m <-> 2mπT on [-(N-1), N-1];
// Ω_m - ν_n -> fermion m-n-1, Ω_m + ν_n -> m+n, ν_n - ν_n' -> boson n-n', ν_n + ν_n' -> n+n'+1.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fdga {

struct cplx {
    double x, y;
};
__host__ __device__ __forceinline__ cplx mk(double a, double b) { return cplx{a, b}; }
__host__ __device__ __forceinline__ cplx operator+(cplx a, cplx b) { return cplx{a.x + b.x, a.y + b.y}; }
__host__ __device__ __forceinline__ cplx operator-(cplx a, cplx b) { return cplx{a.x - b.x, a.y - b.y}; }
__host__ __device__ __forceinline__ cplx operator-(cplx a) { return cplx{-a.x, -a.y}; }
__host__ __device__ __forceinline__ cplx operator*(cplx a, cplx b) {
    return cplx{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
__host__ __device__ __forceinline__ cplx operator*(cplx a, double s) { return cplx{a.x * s, a.y * s}; }
__host__ __device__ __forceinline__ cplx operator*(double s, cplx a) { return cplx{a.x * s, a.y * s}; }
__host__ __device__ __forceinline__ cplx& operator+=(cplx& a, cplx b) { a.x += b.x; a.y += b.y; return a; }
__host__ __device__ __forceinline__ cplx& operator-=(cplx& a, cplx b) { a.x -= b.x; a.y -= b.y; return a; }
__host__ __device__ __forceinline__ cplx conjg(cplx a) { return cplx{a.x, -a.y}; }
__device__ __forceinline__ cplx cdiv(cplx a, cplx b) {
    // a / b with Smith's scaling
    if (fabs(b.x) >= fabs(b.y)) {
        double r = b.y / b.x, den = b.x + b.y * r;
        return cplx{(a.x + a.y * r) / den, (a.y - a.x * r) / den};
    }
    double r = b.x / b.y, den = b.x * r + b.y;
    return cplx{(a.x * r + a.y) / den, (a.y * r - a.x) / den};
}
__device__ __forceinline__ cplx ldg(const cplx* p) {
    double2 v = __ldg(reinterpret_cast<const double2*>(p));
    return cplx{v.x, v.y};
}
// 16-byte load and store of a device array element (cudaMalloc'd arrays indexed in cplx units are
// 16-byte aligned; the struct itself is 8-byte aligned, which would split every access in two)
__device__ __forceinline__ cplx ld16(const cplx* p) {
    const double2 v = *reinterpret_cast<const double2*>(p);
    return cplx{v.x, v.y};
}
__device__ __forceinline__ void st16(cplx* p, cplx v) { *reinterpret_cast<double2*>(p) = make_double2(v.x, v.y); }
// FP32 complex for the mixed-precision contractions (storage stays cplx)
struct cplxf {
    float x, y;
};
__host__ __device__ __forceinline__ cplxf operator+(cplxf a, cplxf b) { return cplxf{a.x + b.x, a.y + b.y}; }
__host__ __device__ __forceinline__ cplxf operator-(cplxf a, cplxf b) { return cplxf{a.x - b.x, a.y - b.y}; }
__host__ __device__ __forceinline__ cplxf operator*(cplxf a, cplxf b) {
    return cplxf{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
__host__ __device__ __forceinline__ cplxf operator*(cplxf a, float s) { return cplxf{a.x * s, a.y * s}; }
__host__ __device__ __forceinline__ cplxf& operator+=(cplxf& a, cplxf b) { a.x += b.x; a.y += b.y; return a; }
__host__ __device__ __forceinline__ cplxf& operator-=(cplxf& a, cplxf b) { a.x -= b.x; a.y -= b.y; return a; }
__host__ __device__ __forceinline__ cplxf operator-(cplxf a) { return cplxf{-a.x, -a.y}; }
__host__ __device__ __forceinline__ cplxf conjg(cplxf a) { return cplxf{a.x, -a.y}; }
// c + a·b with four fused multiply-adds (a complex product followed by an add costs six)
__device__ __forceinline__ cplx cfma(cplx a, cplx b, cplx c) {
    return cplx{fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y))};
}
__device__ __forceinline__ cplxf cfma(cplxf a, cplxf b, cplxf c) {
    return cplxf{fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y))};
}
// conversions between the storage type and the arithmetic type C of a templated kernel
template <class C> __device__ __forceinline__ C to_c(cplx v);
template <> __device__ __forceinline__ cplx to_c<cplx>(cplx v) { return v; }
// FP64 -> FP32 with IEEE 754 round-to-nearest-even, done on the integer pipes: GB300 issues the
// F2F conversion on its FP64 pipe (1/64 rate), where it costs as much as the FP64 arithmetic the
// mixed map removes.  The 52-bit significand is rounded to 23 bits on the 29 dropped bits (ties
// to even); a carry out of the significand steps the exponent, up to infinity.  FP64 zeros and
// subnormals give a signed zero (exact: they lie below half the smallest FP32 subnormal); results
// that would be FP32 subnormal, and infinities and NaNs, take the hardware conversion (same value).
__device__ __forceinline__ float d2f_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned int hi = (unsigned int)(b >> 32);
    const unsigned int sign = hi & 0x80000000u;
    const int ef = (int)((hi >> 20) & 0x7ffu);
    if (ef == 0) return __uint_as_float(sign);
    const int e = ef - 1023 + 127;
    if (e <= 0 || e >= 255) return __double2float_rn(x);
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    unsigned int r = (unsigned int)(m >> 29);
    const unsigned int rem = (unsigned int)(m & 0x1FFFFFFFull);
    if (rem > 0x10000000u || (rem == 0x10000000u && (r & 1u))) r += 1u;
    return __uint_as_float((sign | ((unsigned int)e << 23)) + r);
}
template <> __device__ __forceinline__ cplxf to_c<cplxf>(cplx v) { return cplxf{d2f_rn(v.x), d2f_rn(v.y)}; }
template <class C> __device__ __forceinline__ C to_c(cplxf v) { return C{v.x, v.y}; }
__device__ __forceinline__ cplx to_d(cplx v) { return v; }
__device__ __forceinline__ cplx to_d(cplxf v) { return cplx{(double)v.x, (double)v.y}; }
__device__ __forceinline__ cplxf to_f32(cplx v) { return cplxf{d2f_rn(v.x), d2f_rn(v.y)}; }
__device__ __forceinline__ cplxf to_f32(cplxf v) { return v; }
template <class C> __device__ __forceinline__ C czero() { return C{0, 0}; }

// symmetry operation bits: 1 = negate, 2 = conjugate (MatsubaraFunctions Operation(sgn, con))
template <class S>
__device__ __forceinline__ S apply_op(int op, S v) {
    if (op & 2) v.y = -v.y;
    if (op & 1) { v.x = -v.x; v.y = -v.y; }
    return v;
}
// Exact FP64 sign flips and power-of-two scalings on the integer pipes (GB300's FP64 pipe is the
// bound of the class expansions): -x flips the sign bit; x/2 and 2x step the exponent field when x
// and the result are normal, and take the FP64 multiply otherwise (same value in every case).
__device__ __forceinline__ double neg_exact(double x) {
    return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}
__device__ __forceinline__ double half_exact(double x) {
    const long long b = __double_as_longlong(x);
    const unsigned int ef = (unsigned int)((unsigned long long)b >> 52) & 0x7ffu;
    return (ef >= 2u && ef < 0x7ffu) ? __longlong_as_double(b - (1ll << 52)) : x * 0.5;
}
__device__ __forceinline__ double twice_exact(double x) {
    const long long b = __double_as_longlong(x);
    const unsigned int ef = (unsigned int)((unsigned long long)b >> 52) & 0x7ffu;
    return (ef >= 1u && ef < 0x7feu) ? __longlong_as_double(b + (1ll << 52)) : x * 2.0;
}
template <>
__device__ __forceinline__ cplx apply_op<cplx>(int op, cplx v) {
    if (op & 2) v.y = neg_exact(v.y);
    if (op & 1) { v.x = neg_exact(v.x); v.y = neg_exact(v.y); }
    return v;
}

static constexpr int FINF = -(1 << 30);  // νInf
static constexpr int KAVG = -1;          // kSW: momentum average
enum { CH_P = 0, CH_T = 1, CH_A = 2 };
enum { SP_P = 0, SP_X = 1, SP_D = 2 };

__host__ __device__ __forceinline__ bool bin(int m, int N) { return m > -N && m < N; }
__host__ __device__ __forceinline__ bool fin(int n, int N) { return n >= -N && n < N; }

// Problem dimensions, passed by value to every kernel.
struct Dims {
    int nG, NG, Nk, L, Nq;
    int n1, N1, n2O, N2O, n2n, N2n, n3O, N3O, n3n, N3n;
    int nPO, NPO, nPn, NPn;
    int nPw, NPw;  // stored bubble window: fermion indices [-nPw, nPw) of the mesh [-nPn, nPn)
    int nRO, NRO, nRn, NRn;
    int local;
    double T, U;
    // extents of the union of the vertex boxes of F and of a Vertex-valued reference vertex F0 (equal
    // to n1, n2O, n2n, n3n when F0 is a RefVertex): the ω windows of the BSE and SDE sums use them
    int xn1, xn2O, xn2n, xn3n;
};

// Box of a channel's K1/K2/K3 (the member names of Dims, so that the channel evaluators take either):
// the reference vertex F0 of fdDΓA is a Vertex with boxes of its own (src/ParquetSolver.jl:5,88).
struct Box {
    int n1, N1, n2O, N2O, n2n, N2n, n3O, N3O, n3n, N3n;
};

// One channel's K1/K2/K3 and their momentum averages (A* alias K* for the local solver), stored
// as S (cplx; cplxf for the FP32 mirror of the mixed map).  Evaluators compute in S.
template <class S>
struct ChanPT {
    const S* K1;
    const S* K2;
    const S* K3;
    const S* A1;
    const S* A2;
    const S* A3;
};
// Target vertex F = F0 + γp + γt + γa.  The reference vertex F0 is RefVertex(U, Fp_p, Fp_x, Ft_p, Ft_x),
// or (has0) a Vertex F0 = RefVertex + γ0p + γ0t + γ0a whose channels g0 have their own box b0
// (fdDΓA from a solved vertex: ParquetSolver{Q, VT, RefVT} with RefVT a Vertex, src/ParquetSolver.jl:5-88).
template <class S>
struct VertPT {
    ChanPT<S> g[3];
    const S* Fp_p;
    const S* Fp_x;
    const S* Ft_p;
    const S* Ft_x;
    int noref;  // 1: the reference-vertex terms (U, its corrections and F0's channels) read as zero (a tangent vertex)
    int has0;   // 1: F0 is a Vertex with the channels g0 (box b0) on top of the RefVertex terms
    ChanPT<S> g0[3];
    Box b0;
};
using ChanP = ChanPT<cplx>;
using VertP = VertPT<cplx>;
using VertPF = VertPT<cplxf>;

__device__ __forceinline__ cplx ldv(const cplx* p) { return ldg(p); }
__device__ __forceinline__ cplxf ldv(const cplxf* p) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    return cplxf{v.x, v.y};
}
template <class S> __device__ __forceinline__ S cre(double x) { return S{(decltype(S::x))x, 0}; }

// index of a channel element in its box; D = Dims (the solver's own boxes) or Box (the boxes of F0)
template <class D>
__host__ __device__ __forceinline__ size_t ix1(const D& d, int P, int m) { return (size_t)P * d.N1 + (m + d.n1 - 1); }
template <class D>
__host__ __device__ __forceinline__ size_t ix2(const D& d, int P, int m, int n) {
    return ((size_t)P * d.N2O + (m + d.n2O - 1)) * d.N2n + (n + d.n2n);
}
template <class D>
__host__ __device__ __forceinline__ size_t ix3(const D& d, int P, int m, int n, int np) {
    return (((size_t)P * d.N3O + (m + d.n3O - 1)) * d.N3n + (n + d.n3n)) * d.N3n + (np + d.n3n);
}
__device__ __forceinline__ size_t ixPi(const Dims& d, int P, int m, int n) {
    return ((size_t)P * d.NPO + (m + d.nPO - 1)) * d.NPw + (n + d.nPw);
}
__device__ __forceinline__ size_t ixG(const Dims& d, int k, int n) { return (size_t)k * d.NG + (n + d.nG); }

template <class S, class D>
__device__ __forceinline__ S k1v(const ChanPT<S>& c, const D& d, int m, int P) {
    return P == KAVG ? ldv(c.A1 + (m + d.n1 - 1)) : ldv(c.K1 + ix1(d, P, m));
}
template <class S, class D>
__device__ __forceinline__ S k2v(const ChanPT<S>& c, const D& d, int m, int n, int P) {
    return P == KAVG ? ldv(c.A2 + ix2(d, 0, m, n)) : ldv(c.K2 + ix2(d, P, m, n));
}
template <class S, class D>
__device__ __forceinline__ S k3v(const ChanPT<S>& c, const D& d, int m, int n, int np, int P) {
    return P == KAVG ? ldv(c.A3 + ix3(d, 0, m, n, np)) : ldv(c.K3 + ix3(d, P, m, n, np));
}

// Channel evaluator γ(Ω, ν, ν', P): src/channel.jl:220-339, src/nonlocal/channel.jl:246-382.
// chan_val writes the value into t and returns true, or returns false (t untouched) where the
// channel vanishes (Ω outside the K1 box).  The sums start from their first term: GB300's FP64
// pipe is the bound of every evaluator-heavy kernel, and an addition of zero costs as much as any.
template <class S, class D>
__device__ __forceinline__ bool chan_val(S& t, const ChanPT<S>& c, const D& d, int m, int n, int np, int P) {
    if (!bin(m, d.n1)) return false;
    t = k1v(c, d, m, P);
    if (!bin(m, d.n2O)) return true;
    const bool ninf = (n == FINF), npinf = (np == FINF);
    if (!ninf && !npinf) {
        const bool a = fin(n, d.n2n), b = fin(np, d.n2n);
        if (a && b) {
            t += k2v(c, d, m, n, P) + k2v(c, d, m, np, P);
            if (bin(m, d.n3O) && fin(n, d.n3n) && fin(np, d.n3n)) t += k3v(c, d, m, n, np, P);
        } else if (a) {
            t += k2v(c, d, m, n, P);
        } else if (b) {
            t += k2v(c, d, m, np, P);
        }
    } else if (ninf && !npinf) {
        if (fin(np, d.n2n)) t += k2v(c, d, m, np, P);
    } else if (!ninf && npinf) {
        if (fin(n, d.n2n)) t += k2v(c, d, m, n, P);
    }
    return true;
}
template <class S, class D>
__device__ __forceinline__ S chan_eval(const ChanPT<S>& c, const D& d, int m, int n, int np, int P) {
    S t;
    return chan_val(t, c, d, m, n, np, P) ? t : S{0, 0};
}

// Frequency conversion between channel representations (src/convention.jl:4-36).
__device__ __forceinline__ void conv(int from, int to, int m, int n, int np, int& mo, int& no, int& npo) {
    if (from == to) { mo = m; no = n; npo = np; return; }
    if (from == CH_P) {
        if (to == CH_T) { mo = m - n - np - 1; no = np; npo = n; }
        else            { mo = n - np; no = m - n - 1; npo = np; }
    } else if (from == CH_T) {
        if (to == CH_P) { mo = m + n + np + 1; no = np; npo = n; }
        else            { mo = np - n; no = m + n; npo = n; }
    } else {
        if (to == CH_P) { mo = m + np + n + 1; no = m + np; npo = np; }
        else            { mo = n - np; no = np; npo = m + np; }
    }
}

// RefVertex corrections: MeshFunction call; false (r untouched) outside the box, where they vanish.
template <class S>
__device__ __forceinline__ bool ref_val(S& r, const S* f, const Dims& d, int m, int n, int np) {
    if (!bin(m, d.nRO) || !fin(n, d.nRn) || !fin(np, d.nRn)) return false;
    r = ldv(f + (size_t)(m + d.nRO - 1) + (size_t)d.NRO * ((size_t)(n + d.nRn) + (size_t)d.NRn * (np + d.nRn)));
    return true;
}
template <class S>
__device__ __forceinline__ S ref_call(const S* f, const Dims& d, int m, int n, int np) {
    S r;
    return ref_val(r, f, d, m, n, np) ? r : S{0, 0};
}
// RefVertex in the parallel spin component (src/refvertex.jl:90-125, 178-216): U + correction
// (only the real part carries U).
template <class S>
__device__ __forceinline__ S ref_pSp(const VertPT<S>& F, const Dims& d, int ch, int m, int n, int np) {
    using R = decltype(S::x);
    if (F.noref) return S{0, 0};
    const R U = (R)d.U;
    if (n == FINF || np == FINF) return S{U, 0};
    S r;
    if (ch == CH_A) return ref_val(r, F.Ft_x, d, m, np, n) ? S{U - r.x, -r.y} : S{U, 0};
    return ref_val(r, ch == CH_P ? F.Fp_p : F.Ft_p, d, m, n, np) ? S{r.x + U, r.y} : S{U, 0};
}
// RefVertex in the crossed spin component (src/refvertex.jl:127-164): -U + correction.
template <class S>
__device__ __forceinline__ S ref_xSp(const VertPT<S>& F, const Dims& d, int ch, int m, int n, int np) {
    using R = decltype(S::x);
    if (F.noref) return S{0, 0};
    const R U = (R)d.U;
    if (n == FINF || np == FINF) return S{-U, 0};
    S r;
    if (ch == CH_A) return ref_val(r, F.Ft_p, d, m, np, n) ? S{-r.x - U, -r.y} : S{-U, 0};
    return ref_val(r, ch == CH_P ? F.Fp_x : F.Ft_x, d, m, n, np) ? S{r.x - U, r.y} : S{-U, 0};
}
template <class S>
__device__ __forceinline__ S ref_eval(const VertPT<S>& F, const Dims& d, int ch, int sp, int m, int n, int np) {
    using R = decltype(S::x);
    if (sp == SP_P) return ref_pSp(F, d, ch, m, n, np);
    if (sp == SP_X) return ref_xSp(F, d, ch, m, n, np);
    const S p = ref_pSp(F, d, ch, m, n, np), x = ref_xSp(F, d, ch, m, n, np);
    return S{fma(p.x, (R)2, x.x), fma(p.y, (R)2, x.y)};  // 2p is exact: one rounding, as 2p + x
}

// Channels of a Vertex-valued reference vertex F0 in representation ch, parallel spin, at (Ω,ν,ν')
// with momentum P: the own channel at P, the other two (frequencies converted) at their momentum
// average; with ν or ν' at infinity only the own channel (src/vertex.jl:209-284 and
// src/nonlocal/vertex.jl:69-153, 216-379 applied to F0).  False (t untouched): no channel term.
template <class S>
__device__ __forceinline__ bool f0chan_val(S& t, const VertPT<S>& F, const Dims& d, int ch, int m, int n, int np,
                                           int P) {
    if (n == FINF || np == FINF) return chan_val(t, F.g0[ch], F.b0, m, n, np, P);
    const int Pc = (d.Nq == 1) ? 0 : KAVG;
    bool has = false;
    S u;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        int a, b, c;
        conv(ch, r, m, n, np, a, b, c);
        if (chan_val(u, F.g0[r], F.b0, a, b, c, r == ch ? P : Pc)) {
            if (has) t += u;
            else { t = u; has = true; }
        }
    }
    return has;
}
// The reference vertex F0 in the parallel spin component: the RefVertex, plus its channels when F0
// is a Vertex (the RefVertex terms come first, as in the reference's recursion F.F0.F0).
template <class S>
__device__ __forceinline__ S f0_pSp(const VertPT<S>& F, const Dims& d, int ch, int m, int n, int np, int P) {
    S v = ref_pSp(F, d, ch, m, n, np);
    if (F.has0 && !F.noref) {
        S t;
        if (f0chan_val(t, F, d, ch, m, n, np, P)) v += t;
    }
    return v;
}
// F0 in the crossed spin component.  A RefVertex stores it (Fp_x, Ft_x); a Vertex F0 has it by
// crossing symmetry, xSp = -pSp at the crossed arguments, for its RefVertex part too
// (src/vertex.jl:288-313).
template <class S>
__device__ __forceinline__ S f0_xSp(const VertPT<S>& F, const Dims& d, int ch, int m, int n, int np, int P) {
    if (!F.has0) return ref_xSp(F, d, ch, m, n, np);
    if (ch == CH_P) return -f0_pSp(F, d, CH_P, m, n, (np == FINF) ? FINF : m - np - 1, P);
    if (ch == CH_T) return -f0_pSp(F, d, CH_A, m, n, np, P);
    return -f0_pSp(F, d, CH_T, m, n, np, P);
}
template <class S>
__device__ __forceinline__ S f0_eval(const VertPT<S>& F, const Dims& d, int ch, int sp, int m, int n, int np, int P) {
    using R = decltype(S::x);
    if (!F.has0) return ref_eval(F, d, ch, sp, m, n, np);
    if (sp == SP_P) return f0_pSp(F, d, ch, m, n, np, P);
    if (sp == SP_X) return f0_xSp(F, d, ch, m, n, np, P);
    const S p = f0_pSp(F, d, ch, m, n, np, P), x = f0_xSp(F, d, ch, m, n, np, P);
    return S{fma(p.x, (R)2, x.x), fma(p.y, (R)2, x.y)};
}
// F0(Ω, ω, ∞) - U in the spin combination of channel ch's BSE (pSp for p and a, dSp = 2 pSp + xSp for
// t): zero for a RefVertex; for a Vertex F0 its own channel's K1 + K2(ω) (t: 2 γ0t - γ0a, since
// xSp(t) = -pSp(a) at these arguments).  The factor F0r of the K1/K2 BSEs is U_sp plus this.
template <class S>
__device__ __forceinline__ S f0_right(const VertPT<S>& F, int ch, int m, int n, int P) {
    using R = decltype(S::x);
    if (!F.has0) return S{0, 0};
    if (ch != CH_T) return chan_eval(F.g0[ch], F.b0, m, n, FINF, P);
    const S t = chan_eval(F.g0[CH_T], F.b0, m, n, FINF, P), a = chan_eval(F.g0[CH_A], F.b0, m, n, FINF, P);
    return S{fma(t.x, (R)2, -a.x), fma(t.y, (R)2, -a.y)};
}

// Flags of the vertex evaluator: bit 0 F0, bit 1 γp, bit 2 γt, bit 3 γa.
enum { FL_F0 = 1, FL_GP = 2, FL_GT = 4, FL_GA = 8, FL_ALL = 15 };
__device__ __forceinline__ int swap_ta(int fl) {
    return (fl & (FL_F0 | FL_GP)) | ((fl & FL_GA) ? FL_GT : 0) | ((fl & FL_GT) ? FL_GA : 0);
}

// Vertex in the parallel spin component with momenta (P, kSW, kSW):
// src/vertex.jl:209-284, src/nonlocal/vertex.jl:69-153, 216-379.  Terms are summed in the order
// F0, γp, γt, γa; the first present term is assigned, not added to zero.
template <class S>
__device__ __forceinline__ S vert_pSp(const VertPT<S>& F, const Dims& d, int ch, int m, int n, int np, int P, int fl) {
    S v{0, 0}, t;
    bool has = false;
    auto put = [&](const S& x) {
        if (has) v += x;
        else { v = x; has = true; }
    };
    if (fl & FL_F0) {  // (zero for a tangent vertex; kept so that `has` is known at compile time)
        v = f0_pSp(F, d, ch, m, n, np, P);
        has = true;
    }
    if (n == FINF || np == FINF) {
        const int bit = (ch == CH_P) ? FL_GP : (ch == CH_T ? FL_GT : FL_GA);
        if ((fl & bit) && chan_val(t, F.g[ch], d, m, n, np, P)) put(t);
        return v;
    }
    const int Pc = (d.Nq == 1) ? 0 : KAVG;
    if (fl & FL_GP) { int a, b, c; conv(ch, CH_P, m, n, np, a, b, c); if (chan_val(t, F.g[CH_P], d, a, b, c, ch == CH_P ? P : Pc)) put(t); }
    if (fl & FL_GT) { int a, b, c; conv(ch, CH_T, m, n, np, a, b, c); if (chan_val(t, F.g[CH_T], d, a, b, c, ch == CH_T ? P : Pc)) put(t); }
    if (fl & FL_GA) { int a, b, c; conv(ch, CH_A, m, n, np, a, b, c); if (chan_val(t, F.g[CH_A], d, a, b, c, ch == CH_A ? P : Pc)) put(t); }
    return v;
}
// Crossed component via crossing symmetry (src/vertex.jl:288-313): xSp = -xneg.
template <class S>
__device__ __forceinline__ S vert_xneg(const VertPT<S>& F, const Dims& d, int ch, int m, int n, int np, int P, int fl) {
    const int sw = swap_ta(fl);
    if (ch == CH_P) return vert_pSp(F, d, CH_P, m, n, (np == FINF) ? FINF : m - np - 1, P, sw);
    if (ch == CH_T) return vert_pSp(F, d, CH_A, m, n, np, P, sw);
    return vert_pSp(F, d, CH_T, m, n, np, P, sw);
}
template <class S>
__device__ __forceinline__ S vert_xSp(const VertPT<S>& F, const Dims& d, int ch, int m, int n, int np, int P, int fl) {
    return -vert_xneg(F, d, ch, m, n, np, P, fl);
}
template <class S>
__device__ __forceinline__ S vert_eval(const VertPT<S>& F, const Dims& d, int ch, int sp, int m, int n, int np, int P,
                                       int fl = FL_ALL) {
    using R = decltype(S::x);
    if (sp == SP_P) return vert_pSp(F, d, ch, m, n, np, P, fl);
    if (sp == SP_X) return vert_xSp(F, d, ch, m, n, np, P, fl);
    const S p = vert_pSp(F, d, ch, m, n, np, P, fl), x = vert_xneg(F, d, ch, m, n, np, P, fl);
    return S{fma(p.x, (R)2, -x.x), fma(p.y, (R)2, -x.y)};  // 2 pSp + xSp, 2p exact: one rounding
}

// F(Ω,ν,ω) - F(Ω,∞,ω) - F(Ω,ν,∞) + F(Ω,∞,∞) of the spin-parallel vertex in representation ch
// (the vertex factor of the K2 BSE, src/BSEa/BSEa_K2.jl:43-103).  With ν or ω at infinity only the
// RefVertex's U and the own channel's K1 and K2 terms survive, and those cancel in the difference,
// which is therefore [F0(Ω,ν,ω) - U] + K3_ch(Ω,ν,ω) + Σ_{c ≠ ch} γ_c(conv(Ω,ν,ω)): the
// RefVertex correction, the own channel's K3 and the other two channels, each added only inside
// its box.  Same value as the four evaluations up to rounding, at a fraction of the FP64 work.
template <class S>
__device__ __forceinline__ S pSp_k2diff(const VertPT<S>& F, const Dims& d, int ch, int m, int n, int np, int P) {
    S v{0, 0}, t;
    bool has = false;
    auto put = [&](const S& x) {
        if (has) v += x;
        else { v = x; has = true; }
    };
    if (!F.noref) {
        if (ch == CH_A) {
            if (ref_val(t, F.Ft_x, d, m, np, n)) put(-t);
        } else if (ref_val(t, ch == CH_P ? F.Fp_p : F.Ft_p, d, m, n, np)) {
            put(t);
        }
    }
    if (F.has0 && !F.noref) {  // a Vertex F0 reduces the same way: its own K3 and its other two channels
        const Box& b = F.b0;
        if (bin(m, b.n1) && bin(m, b.n2O) && fin(n, b.n2n) && fin(np, b.n2n) && bin(m, b.n3O) && fin(n, b.n3n) &&
            fin(np, b.n3n))
            put(k3v(F.g0[ch], b, m, n, np, P));
        const int Pc0 = (d.Nq == 1) ? 0 : KAVG;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            if (r == ch) continue;
            int a, bb, c;
            conv(ch, r, m, n, np, a, bb, c);
            if (chan_val(t, F.g0[r], b, a, bb, c, Pc0)) put(t);
        }
    }
    if (bin(m, d.n1) && bin(m, d.n2O) && fin(n, d.n2n) && fin(np, d.n2n) && bin(m, d.n3O) && fin(n, d.n3n) &&
        fin(np, d.n3n))
        put(k3v(F.g[ch], d, m, n, np, P));
    const int Pc = (d.Nq == 1) ? 0 : KAVG;
    if (ch != CH_P) { int a, b, c; conv(ch, CH_P, m, n, np, a, b, c); if (chan_val(t, F.g[CH_P], d, a, b, c, Pc)) put(t); }
    if (ch != CH_T) { int a, b, c; conv(ch, CH_T, m, n, np, a, b, c); if (chan_val(t, F.g[CH_T], d, a, b, c, Pc)) put(t); }
    if (ch != CH_A) { int a, b, c; conv(ch, CH_A, m, n, np, a, b, c); if (chan_val(t, F.g[CH_A], d, a, b, c, Pc)) put(t); }
    return v;
}

// pSp_k2diff of a vertex F and of a tangent vertex dF (RefVertex terms off) in one pass: the
// frequency conversions, box tests and offsets are shared, only the loads are doubled.
template <class S>
__device__ __forceinline__ bool chan_val2(S& t, S& u, const ChanPT<S>& c, const ChanPT<S>& e, const Dims& d, int m,
                                          int n, int np, int P) {
    if (!bin(m, d.n1)) return false;
    t = k1v(c, d, m, P);
    u = k1v(e, d, m, P);
    if (!bin(m, d.n2O)) return true;
    const bool a = fin(n, d.n2n), b = fin(np, d.n2n);  // n, np finite here
    if (a && b) {
        t += k2v(c, d, m, n, P) + k2v(c, d, m, np, P);
        u += k2v(e, d, m, n, P) + k2v(e, d, m, np, P);
        if (bin(m, d.n3O) && fin(n, d.n3n) && fin(np, d.n3n)) {
            t += k3v(c, d, m, n, np, P);
            u += k3v(e, d, m, n, np, P);
        }
    } else if (a) {
        t += k2v(c, d, m, n, P);
        u += k2v(e, d, m, n, P);
    } else if (b) {
        t += k2v(c, d, m, np, P);
        u += k2v(e, d, m, np, P);
    }
    return true;
}
template <class S>
__device__ __forceinline__ void pSp_k2diff2(const VertPT<S>& F, const VertPT<S>& E, const Dims& d, int ch, int m, int n,
                                            int np, int P, S& v, S& w) {
    S t, u;
    bool has = false;
    auto put = [&](const S& x, const S& y) {
        if (has) { v += x; w += y; }
        else { v = x; w = y; has = true; }
    };
    v = S{0, 0};
    w = S{0, 0};
    if (!F.noref) {  // (the tangent vertex has no RefVertex terms)
        if (ch == CH_A) {
            if (ref_val(t, F.Ft_x, d, m, np, n)) put(-t, S{0, 0});
        } else if (ref_val(t, ch == CH_P ? F.Fp_p : F.Ft_p, d, m, n, np)) {
            put(t, S{0, 0});
        }
        if (F.has0) {  // the reduced difference of a Vertex F0 (constant: no tangent part)
            const Box& b = F.b0;
            if (bin(m, b.n1) && bin(m, b.n2O) && fin(n, b.n2n) && fin(np, b.n2n) && bin(m, b.n3O) && fin(n, b.n3n) &&
                fin(np, b.n3n))
                put(k3v(F.g0[ch], b, m, n, np, P), S{0, 0});
            const int Pc0 = (d.Nq == 1) ? 0 : KAVG;
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                if (r == ch) continue;
                int a, bb, c;
                conv(ch, r, m, n, np, a, bb, c);
                if (chan_val(t, F.g0[r], b, a, bb, c, Pc0)) put(t, S{0, 0});
            }
        }
    }
    if (bin(m, d.n1) && bin(m, d.n2O) && fin(n, d.n2n) && fin(np, d.n2n) && bin(m, d.n3O) && fin(n, d.n3n) &&
        fin(np, d.n3n))
        put(k3v(F.g[ch], d, m, n, np, P), k3v(E.g[ch], d, m, n, np, P));
    const int Pc = (d.Nq == 1) ? 0 : KAVG;
    if (ch != CH_P) { int a, b, c; conv(ch, CH_P, m, n, np, a, b, c); if (chan_val2(t, u, F.g[CH_P], E.g[CH_P], d, a, b, c, Pc)) put(t, u); }
    if (ch != CH_T) { int a, b, c; conv(ch, CH_T, m, n, np, a, b, c); if (chan_val2(t, u, F.g[CH_T], E.g[CH_T], d, a, b, c, Pc)) put(t, u); }
    if (ch != CH_A) { int a, b, c; conv(ch, CH_A, m, n, np, a, b, c); if (chan_val2(t, u, F.g[CH_A], E.g[CH_A], d, a, b, c, Pc)) put(t, u); }
}

// Vertex factors of the K2 BSE (bse_K2_row) and of its transpose.
// F(Ω,ν,ω) - F(Ω,∞,ω) - F(Ω,ν,∞) + F(Ω,∞,∞) in the spin combination of the K2 BSE of channel CH
template <int CH, class S>
__device__ __forceinline__ S k2_vertex_diff(const VertPT<S>& F, const Dims& d, int m, int nu, int n, int P) {
    using R = decltype(S::x);
    if constexpr (CH != CH_T) {
        return pSp_k2diff(F, d, CH, m, nu, n, P);
    } else {  // density: 2 pSp + xSp, xSp(t) = -pSp(a); 2p exact, one rounding
        const S p = pSp_k2diff(F, d, CH_T, m, nu, n, P), x = pSp_k2diff(F, d, CH_A, m, nu, n, P);
        return S{fma(p.x, (R)2, -x.x), fma(p.y, (R)2, -x.y)};
    }
}
// the same for F and a tangent vertex dF in one pass
template <int CH, class S>
__device__ __forceinline__ void k2_vertex_diff2(const VertPT<S>& F, const VertPT<S>& E, const Dims& d, int m, int nu,
                                                int n, int P, S& v, S& w) {
    using R = decltype(S::x);
    if constexpr (CH != CH_T) {
        pSp_k2diff2(F, E, d, CH, m, nu, n, P, v, w);
    } else {
        S p, q, x, y;
        pSp_k2diff2(F, E, d, CH_T, m, nu, n, P, p, q);
        pSp_k2diff2(F, E, d, CH_A, m, nu, n, P, x, y);
        v = S{fma(p.x, (R)2, -x.x), fma(p.y, (R)2, -x.y)};
        w = S{fma(q.x, (R)2, -y.x), fma(q.y, (R)2, -y.y)};
    }
}
// c = F(Ω,ν,∞) - F(Ω,∞,∞) in the same spin combination: only the own channel's K2(Ω,ν) survives
// (the t channel's crossed part is the a channel's, by crossing)
template <class S>
__device__ __forceinline__ S k2_own(const VertPT<S>& F, const Dims& d, int ch, int m, int nu, int P) {
    S v{0, 0};
    if (bin(m, d.n1) && bin(m, d.n2O) && fin(nu, d.n2n)) v = k2v(F.g[ch], d, m, nu, P);
    if (F.has0 && !F.noref) {  // the own channel of a Vertex-valued F0 contributes its K2(Ω, ν) too
        const Box& b = F.b0;
        if (bin(m, b.n1) && bin(m, b.n2O) && fin(nu, b.n2n)) v += k2v(F.g0[ch], b, m, nu, P);
    }
    return v;
}
template <int CH, class S>
__device__ __forceinline__ S k2_c(const VertPT<S>& F, const Dims& d, int m, int nu, int P) {
    using R = decltype(S::x);
    if constexpr (CH != CH_T) {
        return k2_own(F, d, CH, m, nu, P);
    } else {
        const S p = k2_own(F, d, CH_T, m, nu, P), x = k2_own(F, d, CH_A, m, nu, P);
        return S{fma(p.x, (R)2, -x.x), fma(p.y, (R)2, -x.y)};
    }
}
// FL(Ω, ω, νInf, Ch, Sp): FL has F0 = RefVertex(0) and K1 = 0, so only its K2 survives.
template <class S>
__device__ __forceinline__ S fl_right(const S* FLK2p, const S* FLK2t, const S* FLK2a, const Dims& d, int ch, int m,
                                      int n, int P) {
    using R = decltype(S::x);
    if (!bin(m, d.n2O) || !fin(n, d.n2n)) return S{0, 0};
    const size_t i = ix2(d, P, m, n);
    if (ch == CH_P) return ldv(FLK2p + i);
    if (ch == CH_A) return ldv(FLK2a + i);
    return ldv(FLK2t + i) * (R)2 - ldv(FLK2a + i);  // dSp = 2 pSp + xSp, xSp(t) = -pSp(a)
}

__device__ __forceinline__ int cross(int ch, int m, int n) { return ch == CH_P ? m - n - 1 : n; }

// A union of at most 6 closed ω intervals, merged and ordered; used to visit only the bubble
// frequencies at which a vertex factor differs from its ω-independent value.
struct Windows {
    int lo[6], hi[6];
    int n = 0, total = 0;
    __device__ __forceinline__ void add(int a, int b, int clo, int chi) {
        a = max(a, clo);
        b = min(b, chi);
        if (a <= b && n < 6) { lo[n] = a; hi[n] = b; ++n; }
    }
    __device__ __forceinline__ void merge() {
        for (int i = 1; i < n; ++i)  // insertion sort by lo
            for (int j = i; j > 0 && lo[j] < lo[j - 1]; --j) {
                int t = lo[j]; lo[j] = lo[j - 1]; lo[j - 1] = t;
                t = hi[j]; hi[j] = hi[j - 1]; hi[j - 1] = t;
            }
        int m = 0;
        for (int i = 0; i < n; ++i) {
            if (m > 0 && lo[i] <= hi[m - 1] + 1) { hi[m - 1] = max(hi[m - 1], hi[i]); }
            else { lo[m] = lo[i]; hi[m] = hi[i]; ++m; }
        }
        n = m;
        total = 0;
        for (int i = 0; i < n; ++i) total += hi[i] - lo[i] + 1;
    }
    // t-th frequency of the union, t < total
    __device__ __forceinline__ int at(int t) const {
        for (int i = 0; i < n; ++i) {
            const int len = hi[i] - lo[i] + 1;
            if (t < len) return lo[i] + t;
            t -= len;
        }
        return lo[0];
    }
};

__device__ __forceinline__ cplxf warp_sum(cplxf v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}
// warp reduction of a complex double
__device__ __forceinline__ cplx warp_sum(cplx v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

}  // namespace fdga
