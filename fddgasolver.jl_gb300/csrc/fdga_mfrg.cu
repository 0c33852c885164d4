// fdga_mfrg.cu -- stages of the mfRG linear map (src/mfRG.jl:20-89) that differ from the parquet
// iteration: the K3 caches of the map and its K1/K2 BSEs.  The left BSEs (FL.K2, FL.K3), the K3
// contraction (the plain kernel with Π = Π0, which drops its (Π - Π0) F0 term) and the class
// expansion are the iteration's own kernels.
//
// The map is called on the nonlocal solver, whose two-argument cache builder
// (src/nonlocal_2/build_K3_cache.jl:97-165) differs from the plain one in two ways:
//   * the irreducible caches are F(γr = false) - F.F0(γr = false): the plain Γ of the state vertex,
//     plus the reference vertex's own γr when F0 is a Vertex, and, in the crossed p cache of a
//     RefVertex F0, the RefVertex terms -F0p(Ω, ω, Ω-ν') - F0x(Ω, ω, ν') (zero for a RefVertex whose
//     crossed component obeys crossing symmetry, as the bare U does);
//   * the right "total vertex" caches come from F0 alone, F0(Ω, ν, ω) - F0(Ω, ∞, ω): constant over
//     the applications of one map, so they are written by a separate launch (part 1) once per solve;
//   * all seven are evaluated through the K3 symmetry groups (SG(cache, InitFunction(diagram))): the
//     representatives' values are broadcast to their classes.  F0(Ω, ν, ω) - F0(Ω, ∞, ω) is not
//     invariant under ν <-> ω, so the broadcast changes it; the launch after each cache stage
//     (launch_cache_broadcast) reproduces that.
#include "fdga_kernels.h"

namespace fdga {

namespace {

inline unsigned blocks_of(size_t n, int t) { return (unsigned)((n + t - 1) / t); }
#define MF_CHECK() do { cudaError_t e_ = cudaGetLastError(); if (e_ != cudaSuccess) return e_; } while (0)

// V0: compiled with the evaluation of a Vertex-valued reference vertex (has0 cleared otherwise, so
// the RefVertex instantiation drops those paths)
template <bool V0, class S>
__device__ __forceinline__ VertPT<S> spec(const VertPT<S>& F) {
    VertPT<S> G = F;
    if constexpr (!V0) G.has0 = 0;
    return G;
}

// part 0: Γpx, Γpp, Γa, Γt (slots 0, 4, 5, 6) of the state vertex F = x·factor.
// part 1: the F0-only caches, F0p/F0a/F0t (slots 1-3, as in the plain builder) and Fp/Fa/Ft (7-9).
template <class S, bool V0>
__global__ void k_build_cache_mfrg(VertPT<S> Fin, Caches C, const int* blocks, int nblocks, Dims d, int part) {
    const VertPT<S> F = spec<V0>(Fin);
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
    S v[10];
    if (part == 0) {
        S gpx = vert_eval(F, d, CH_P, SP_X, m, a, b, P, FL_GT | FL_GA);
        S gpp = vert_pSp(F, d, CH_P, m, a, b, P, FL_GT | FL_GA);
        S ga = vert_pSp(F, d, CH_A, m, a, b, P, FL_GP | FL_GT);
        S gt = vert_pSp(F, d, CH_T, m, a, b, P, FL_GP | FL_GA);
        if (F.has0) {
            // F0's own reducible vertex in the excluded channel, at momentum P (the crossed p cache
            // at ν' -> Ω - ν', with the sign of the crossed component)
            S u;
            if (chan_val(u, F.g0[CH_P], F.b0, m, a, m - b - 1, P)) gpx -= u;
            if (chan_val(u, F.g0[CH_P], F.b0, m, a, b, P)) gpp += u;
            if (chan_val(u, F.g0[CH_A], F.b0, m, a, b, P)) ga += u;
            if (chan_val(u, F.g0[CH_T], F.b0, m, a, b, P)) gt += u;
        } else {
            gpx -= ref_pSp(F, d, CH_P, m, a, m - b - 1) + ref_xSp(F, d, CH_P, m, a, b);
        }
        v[0] = gpx;
        v[4] = gpp;
        v[5] = ga;
        v[6] = gt * (R)2 - ga;
    } else {
        v[1] = f0_xSp(F, d, CH_P, m, a, b, P) - f0_xSp(F, d, CH_P, m, a, FINF, P);
        const S f0a = f0_pSp(F, d, CH_A, m, a, b, P) - f0_pSp(F, d, CH_A, m, a, FINF, P);
        const S f0t = f0_pSp(F, d, CH_T, m, a, b, P) - f0_pSp(F, d, CH_T, m, a, FINF, P);
        v[2] = f0a;
        v[3] = f0t * (R)2 - f0a;
        const S fp = f0_pSp(F, d, CH_P, m, a, b, P) - f0_pSp(F, d, CH_P, m, FINF, b, P);
        const S fa = f0_pSp(F, d, CH_A, m, a, b, P) - f0_pSp(F, d, CH_A, m, FINF, b, P);
        const S ft = f0_pSp(F, d, CH_T, m, a, b, P) - f0_pSp(F, d, CH_T, m, FINF, b, P);
        v[7] = fp;
        v[8] = fa;
        v[9] = ft * (R)2 - fa;
    }
    const int k0[4] = {0, 4, 5, 6}, k1[6] = {1, 2, 3, 7, 8, 9};
    const int nk = part == 0 ? 4 : 6;
    for (int j = 0; j < nk; ++j) {
        const int k = part == 0 ? k0[j] : k1[j];
        if (C.f[k]) C.f[k][i] = to_f32(v[k]);
        else if (C.c[k]) C.c[k][i] = to_d(v[k]);
    }
}

// K1 of the map (src/nonlocal/BSEa/BSEa_K1.jl:29-37), warp per representative:
//   K1(Ω, P) = T s Σ_ω F0(Ω, ∞, ω) Π0(Ω, ω) FL(Ω, ω̃, ∞).
// FL(Ω, ω̃, ∞) is FL's K2 (FL has no K1 and a zero reference vertex), so ω̃ runs over the K2 box.
template <int CH>
__device__ __forceinline__ void k1_body(const VertP& F, const FLP& FL, const cplx* Pi0, cplx* out, const int* items,
                                        int nitems, const Dims& d) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nitems) return;
    const int idx = items ? items[w] : w;
    const int m = idx % d.N1 - (d.n1 - 1), P = idx / d.N1;
    constexpr int SP = (CH == CH_T) ? SP_D : SP_P;
    cplx acc = mk(0, 0);
    if (bin(m, d.n2O)) {
        for (int nt = -d.n2n + lane; nt < d.n2n; nt += 32) {
            const int n = cross(CH, m, nt);
            if (!fin(n, d.nPw)) continue;
            const cplx Fl = f0_eval(F, d, CH, SP, m, FINF, n, P);
            const cplx FLr = fl_right(FL.K2[CH_P], FL.K2[CH_T], FL.K2[CH_A], d, CH, m, nt, P);
            acc = cfma(Fl * ldg(Pi0 + ixPi(d, P, m, n)), FLr, acc);
        }
    }
    acc = warp_sum(acc);
    if (lane == 0) out[idx] = acc * (d.T * (CH == CH_T ? -1.0 : 1.0));
}

// K2 of the map (src/nonlocal/BSEa/BSEa_K2.jl:70-77), warp per representative:
//   K2(Ω, ν, P) = T s Σ_ω [F0(Ω, ν, ω̃) - F0(Ω, ∞, ω̃)] Π0(Ω, ω) FL(Ω, ω, ∞),  ω over the K2 box;
// the FL.K2 epilogue of BSE_K2! is added by the class expansion.
template <int CH>
__device__ __forceinline__ void k2_body(const VertP& F, const FLP& FL, const cplx* Pi0, cplx* out, const int* items,
                                        int nitems, const Dims& d) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nitems) return;
    const int idx = items ? items[w] : w;
    const int nu = idx % d.N2n - d.n2n;
    const int m = (idx / d.N2n) % d.N2O - (d.n2O - 1);
    const int P = idx / (d.N2n * d.N2O);
    constexpr int SP = (CH == CH_T) ? SP_D : SP_P;
    cplx acc = mk(0, 0);
    for (int n = -d.n2n + lane; n < d.n2n; n += 32) {
        if (!fin(n, d.nPw)) continue;
        const int wt = cross(CH, m, n);
        const cplx Fl = f0_eval(F, d, CH, SP, m, nu, wt, P) - f0_eval(F, d, CH, SP, m, FINF, wt, P);
        const cplx FLr = fl_right(FL.K2[CH_P], FL.K2[CH_T], FL.K2[CH_A], d, CH, m, n, P);
        acc = cfma(Fl * ldg(Pi0 + ixPi(d, P, m, n)), FLr, acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) out[idx] = acc * (d.T * (CH == CH_T ? -1.0 : 1.0));
}

template <bool V0>
__global__ void k_bse_K1_mfrg(VertP Fin, FLP FL, BubbleP B, ChanWork cw, Dims d) {
    const VertP F = spec<V0>(Fin);
    switch (blockIdx.y) {
        case CH_P: k1_body<CH_P>(F, FL, B.pp0, cw.out[CH_P], cw.items[CH_P], cw.nitems[CH_P], d); break;
        case CH_T: k1_body<CH_T>(F, FL, B.ph0, cw.out[CH_T], cw.items[CH_T], cw.nitems[CH_T], d); break;
        default:   k1_body<CH_A>(F, FL, B.ph0, cw.out[CH_A], cw.items[CH_A], cw.nitems[CH_A], d); break;
    }
}
template <bool V0>
__global__ void k_bse_K2_mfrg(VertP Fin, FLP FL, BubbleP B, ChanWork cw, Dims d) {
    const VertP F = spec<V0>(Fin);
    switch (blockIdx.y) {
        case CH_P: k2_body<CH_P>(F, FL, B.pp0, cw.out[CH_P], cw.items[CH_P], cw.nitems[CH_P], d); break;
        case CH_T: k2_body<CH_T>(F, FL, B.ph0, cw.out[CH_T], cw.items[CH_T], cw.nitems[CH_T], d); break;
        default:   k2_body<CH_A>(F, FL, B.ph0, cw.out[CH_A], cw.items[CH_A], cw.nitems[CH_A], d); break;
    }
}

unsigned warp_blocks(const ChanWork& cw) {
    int mx = 0;
    for (int c = 0; c < 3; ++c) mx = mx > cw.nitems[c] ? mx : cw.nitems[c];
    return blocks_of((size_t)(mx > 0 ? mx : 1) * 32, 128);
}

// SymmetryGroup broadcast of up to three K3-shaped caches in place: c[i] = op_i(c[rep_i]).  A
// representative's own operation is the identity, so it is never rewritten and the in-place update
// has no read-after-write hazard.
template <class S>
__global__ void k_cache_broadcast(S* c0, S* c1, S* c2, const uint32_t* map, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t v = map[i];
        const size_t r = v >> 2;
        if (r == i) continue;
        const int op = (int)(v & 3u);
        c0[i] = apply_op(op, c0[r]);
        if (c1) c1[i] = apply_op(op, c1[r]);
        if (c2) c2[i] = apply_op(op, c2[r]);
    }
}

template <class S>
cudaError_t cache_mfrg_t(cudaStream_t s, const VertPT<S>& F, const Caches& C, const int* blocks, int nblocks,
                         const Dims& d, int part) {
    const size_t n = (size_t)nblocks * d.N3n * d.N3n;
    if (n == 0) return cudaSuccess;
    if (F.has0) k_build_cache_mfrg<S, true><<<blocks_of(n, 128), 128, 0, s>>>(F, C, blocks, nblocks, d, part);
    else k_build_cache_mfrg<S, false><<<blocks_of(n, 128), 128, 0, s>>>(F, C, blocks, nblocks, d, part);
    MF_CHECK();
    return cudaSuccess;
}

}  // namespace

cudaError_t launch_build_cache_mfrg(cudaStream_t s, const VertP& F, const Caches& C, const int* blocks, int nblocks,
                                    const Dims& d, int part) {
    return cache_mfrg_t(s, F, C, blocks, nblocks, d, part);
}
cudaError_t launch_build_cache_mfrg(cudaStream_t s, const VertPF& F, const Caches& C, const int* blocks, int nblocks,
                                    const Dims& d, int part) {
    return cache_mfrg_t(s, F, C, blocks, nblocks, d, part);
}
cudaError_t launch_cache_broadcast(cudaStream_t s, cplx* c0, cplx* c1, cplx* c2, const uint32_t* map, size_t n) {
    const unsigned g = blocks_of(n, 256) < 8192u ? blocks_of(n, 256) : 8192u;
    k_cache_broadcast<cplx><<<g, 256, 0, s>>>(c0, c1, c2, map, n);
    MF_CHECK();
    return cudaSuccess;
}
cudaError_t launch_cache_broadcast(cudaStream_t s, cplxf* c0, cplxf* c1, cplxf* c2, const uint32_t* map, size_t n) {
    const unsigned g = blocks_of(n, 256) < 8192u ? blocks_of(n, 256) : 8192u;
    k_cache_broadcast<cplxf><<<g, 256, 0, s>>>(c0, c1, c2, map, n);
    MF_CHECK();
    return cudaSuccess;
}
cudaError_t launch_bse_K1_mfrg(cudaStream_t s, const VertP& F, const FLP& FL, const BubbleP& B, const ChanWork& cw,
                               const Dims& d) {
    const dim3 g(warp_blocks(cw), 3);
    if (F.has0) k_bse_K1_mfrg<true><<<g, 128, 0, s>>>(F, FL, B, cw, d);
    else k_bse_K1_mfrg<false><<<g, 128, 0, s>>>(F, FL, B, cw, d);
    MF_CHECK();
    return cudaSuccess;
}
cudaError_t launch_bse_K2_mfrg(cudaStream_t s, const VertP& F, const FLP& FL, const BubbleP& B, const ChanWork& cw,
                               const Dims& d) {
    const dim3 g(warp_blocks(cw), 3);
    if (F.has0) k_bse_K2_mfrg<true><<<g, 128, 0, s>>>(F, FL, B, cw, d);
    else k_bse_K2_mfrg<false><<<g, 128, 0, s>>>(F, FL, B, cw, d);
    MF_CHECK();
    return cudaSuccess;
}

}  // namespace fdga

namespace fdga {
namespace {
__global__ void k_mfrg_scale(cplx* out, const cplx* in, double s, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = in[i] * s;
}
}  // namespace
// out = s · in
cudaError_t launch_scale(cudaStream_t s, cplx* out, const cplx* in, double sc, size_t n) {
    if (n == 0) return cudaSuccess;
    const unsigned g = blocks_of(n, 256) < 4096u ? blocks_of(n, 256) : 4096u;
    k_mfrg_scale<<<g, 256, 0, s>>>(out, in, sc, n);
    MF_CHECK();
    return cudaSuccess;
}
}  // namespace fdga
