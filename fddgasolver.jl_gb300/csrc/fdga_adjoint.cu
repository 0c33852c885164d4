// fdga_adjoint.cu -- reverse-mode derivative (the rrule) of one parquet iteration: x̄ = Φ'(x)ᵀ ȳ
// for the real inner product <a, b> = Re Σ conj(a) b, FP64.
//
// Every forward stage is transposed here.  The forward stages gather vertex values at transformed
// frequency arguments (channel and vertex evaluators, src/channel.jl:220-339, src/vertex.jl:209-336);
// their transposes scatter the cotangents back with atomic adds into the same array elements
// (*_adj evaluators below).  Products a·b transpose to ā += conj(b)·c̄, b̄ += conj(a)·c̄; the K3 BSE
// transposes into two batched GEMMs, Ā = T·C̄·Mᴴ and M̄ = T·Aᴴ·C̄; 2D momentum transforms transpose
// into the transform of opposite sign; the SymmetryGroup broadcast transposes into a scatter-add
// onto the representatives (its operations -, conj are self-adjoint).  The bubbles and G(R) are
// not stored for the backward pass: the cotangent kernels read G(R) of the base point, which the
// value pass recomputes.
#include <algorithm>

#include "fdga_kernels.h"

namespace fdga {

namespace {

__device__ __forceinline__ void aadd(cplx* p, cplx v) {
    atomicAdd(&p->x, v.x);
    atomicAdd(&p->y, v.y);
}
__device__ __forceinline__ cplx cj(cplx a) { return mk(a.x, -a.y); }
// conj(a)·b
__device__ __forceinline__ cplx cmulc(cplx a, cplx b) { return mk(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x); }
// acc + conj(a)·b
__device__ __forceinline__ cplx cfmac(cplx a, cplx b, cplx acc) {
    return mk(acc.x + a.x * b.x + a.y * b.y, acc.y + a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ int mirror(int R, int L) {
    const int Rx = R % L, Ry = R / L;
    return ((L - Rx) % L) + L * ((L - Ry) % L);
}

// ---- transposed evaluators: scatter g into every element the forward evaluator reads ----
__device__ __forceinline__ void k1a(const ChanBar& c, const Dims& d, int m, int P, cplx g) {
    aadd(P == KAVG ? c.A1 + (m + d.n1 - 1) : c.K1 + ix1(d, P, m), g);
}
__device__ __forceinline__ void k2a(const ChanBar& c, const Dims& d, int m, int n, int P, cplx g) {
    aadd(P == KAVG ? c.A2 + ix2(d, 0, m, n) : c.K2 + ix2(d, P, m, n), g);
}
__device__ __forceinline__ void k3a(const ChanBar& c, const Dims& d, int m, int n, int np, int P, cplx g) {
    aadd(P == KAVG ? c.A3 + ix3(d, 0, m, n, np) : c.K3 + ix3(d, P, m, n, np), g);
}
// transpose of chan_eval (fdga_device.cuh)
__device__ void chan_adj(const ChanBar& c, const Dims& d, int m, int n, int np, int P, cplx g) {
    const bool ninf = (n == FINF), npinf = (np == FINF);
    if (!bin(m, d.n1)) return;
    k1a(c, d, m, P, g);
    if (!bin(m, d.n2O)) return;
    if (!ninf && !npinf) {
        const bool a = fin(n, d.n2n), b = fin(np, d.n2n);
        if (a && b) {
            k2a(c, d, m, n, P, g);
            k2a(c, d, m, np, P, g);
            if (bin(m, d.n3O) && fin(n, d.n3n) && fin(np, d.n3n)) k3a(c, d, m, n, np, P, g);
        } else if (a) {
            k2a(c, d, m, n, P, g);
        } else if (b) {
            k2a(c, d, m, np, P, g);
        }
    } else if (ninf && !npinf) {
        if (fin(np, d.n2n)) k2a(c, d, m, np, P, g);
    } else if (!ninf && npinf) {
        if (fin(n, d.n2n)) k2a(c, d, m, n, P, g);
    }
}
// transpose of vert_pSp (the RefVertex terms are constant)
__device__ void pSp_adj(const VertBar& B, const Dims& d, int ch, int m, int n, int np, int P, int fl, cplx g) {
    if (n == FINF || np == FINF) {
        const int bit = (ch == CH_P) ? FL_GP : (ch == CH_T ? FL_GT : FL_GA);
        if (fl & bit) chan_adj(B.g[ch], d, m, n, np, P, g);
        return;
    }
    const int Pc = (d.Nq == 1) ? 0 : KAVG;
    if (fl & FL_GP) { int a, b, c; conv(ch, CH_P, m, n, np, a, b, c); chan_adj(B.g[CH_P], d, a, b, c, ch == CH_P ? P : Pc, g); }
    if (fl & FL_GT) { int a, b, c; conv(ch, CH_T, m, n, np, a, b, c); chan_adj(B.g[CH_T], d, a, b, c, ch == CH_T ? P : Pc, g); }
    if (fl & FL_GA) { int a, b, c; conv(ch, CH_A, m, n, np, a, b, c); chan_adj(B.g[CH_A], d, a, b, c, ch == CH_A ? P : Pc, g); }
}
__device__ void xSp_adj(const VertBar& B, const Dims& d, int ch, int m, int n, int np, int P, int fl, cplx g) {
    const int sw = swap_ta(fl);
    const cplx mg = g * -1.0;
    if (ch == CH_P) pSp_adj(B, d, CH_P, m, n, (np == FINF) ? FINF : m - np - 1, P, sw, mg);
    else if (ch == CH_T) pSp_adj(B, d, CH_A, m, n, np, P, sw, mg);
    else pSp_adj(B, d, CH_T, m, n, np, P, sw, mg);
}
__device__ void vert_adj(const VertBar& B, const Dims& d, int ch, int sp, int m, int n, int np, int P, int fl, cplx g) {
    if (sp == SP_P) { pSp_adj(B, d, ch, m, n, np, P, fl, g); return; }
    if (sp == SP_X) { xSp_adj(B, d, ch, m, n, np, P, fl, g); return; }
    pSp_adj(B, d, ch, m, n, np, P, fl, g * 2.0);
    xSp_adj(B, d, ch, m, n, np, P, fl, g);
}
// transpose of pSp_k2diff (fdga_device.cuh), the reduced K2 vertex difference: the own channel's
// K3 and the two other channels (the RefVertex correction is constant)
__device__ void pSp_k2diff_adj(const VertBar& B, const Dims& d, int ch, int m, int n, int np, int P, cplx g) {
    if (bin(m, d.n1) && bin(m, d.n2O) && fin(n, d.n2n) && fin(np, d.n2n) && bin(m, d.n3O) && fin(n, d.n3n) &&
        fin(np, d.n3n))
        k3a(B.g[ch], d, m, n, np, P, g);
    const int Pc = (d.Nq == 1) ? 0 : KAVG;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        if (r == ch) continue;
        int a, b, c;
        conv(ch, r, m, n, np, a, b, c);
        chan_adj(B.g[r], d, a, b, c, Pc, g);
    }
}
// transpose of fl_right
__device__ __forceinline__ void fl_right_adj(const FLBar& FL, const Dims& d, int ch, int m, int n, int P, cplx g) {
    if (!bin(m, d.n2O) || !fin(n, d.n2n)) return;
    const size_t i = ix2(d, P, m, n);
    if (ch == CH_P) aadd(FL.K2[CH_P] + i, g);
    else if (ch == CH_A) aadd(FL.K2[CH_A] + i, g);
    else { aadd(FL.K2[CH_T] + i, g * 2.0); aadd(FL.K2[CH_A] + i, g * -1.0); }
}

// ---- Σ assembly, occupation ----
// Σ = op(Σin + Σ_U²)[rep] + i (n - 1/2) U (+ constants): Σ̄in[rep] += op(Σ̄), Σ̄_U²[rep] += op(Σ̄)
__global__ void k_adj_assemble(const cplx* Sbar, const uint32_t* map, cplx* Sin_bar, cplx* SU2_bar, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    size_t r = i;
    int op = 0;
    if (map) { const uint32_t e = map[i]; r = e >> 2; op = (int)(e & 3u); }
    const cplx g = apply_op(op, Sbar[i]);
    aadd(Sin_bar + r, g);
    aadd(SU2_bar + r, g);
}
// n̄ = U Σ Im Σ̄ (Hartree term); single block, then Ḡ += i (T/Nk) n̄
__global__ void k_adj_occ_reduce(const cplx* Sbar, size_t n, double U, double* nbar) {
    __shared__ double red[1024];
    double s = 0.0;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) s += Sbar[i].y;
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *nbar = red[0] * U;
}
__global__ void k_adj_occ_apply(cplx* Gbar, const double* nbar, double T, int Nk, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    Gbar[i].y += *nbar * T / (double)Nk;
}
// Dyson: Σ̄ += conj(-G²) Ḡ
__global__ void k_adj_dyson(const cplx* G, const cplx* Gbar, cplx* Sbar, size_t n) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const cplx g = G[i];
    Sbar[i] += cmulc(g * g * -1.0, Gbar[i]);
}

// ---- U² term: out(R,ν) = U²T² Σ_n2 G(R,n2) C(R,ν-n2),  C(R,s) = Σ_n1 G(-R,n1) G(R,n1+s) ----
// ḠR(R,n2) += U²T² Σ_ν conj(C(R,ν-n2)) ō(R,ν);  C̄(R,s) = U²T² Σ_n2 conj(G(R,n2)) ō(R,s+n2)
__global__ void k_adj_u2_sum(const cplx* GR, const cplx* C, const cplx* obar, cplx* GRbar, cplx* Cbar, Dims d) {
    const int NS = 2 * d.NG - 1, NR = d.L * d.L;
    const size_t w = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const double s2 = d.U * d.U * d.T * d.T;
    const size_t nG = (size_t)NR * d.NG;
    if (w < nG) {  // ḠR(R, n2)
        const int n2 = (int)(w % d.NG) - d.nG, R = (int)(w / d.NG);
        cplx acc = mk(0, 0);
        for (int nu = -d.nG + lane; nu < d.nG; nu += 32)
            acc = cfmac(C[(size_t)R * NS + (nu - n2 + d.NG - 1)], obar[ixG(d, R, nu)], acc);
        acc = warp_sum(acc);
        if (lane == 0) GRbar[w] += acc * s2;
    } else if (w < nG + (size_t)NR * NS) {  // C̄(R, s)
        const size_t u = w - nG;
        const int s = (int)(u % NS) - (d.NG - 1), R = (int)(u / NS);
        cplx acc = mk(0, 0);
        for (int n2 = -d.nG + lane; n2 < d.nG; n2 += 32) {
            const int nu = s + n2;
            if (!fin(nu, d.nG)) continue;
            acc = cfmac(GR[ixG(d, R, n2)], obar[ixG(d, R, nu)], acc);
        }
        acc = warp_sum(acc);
        if (lane == 0) Cbar[u] = acc * s2;
    }
}
// C(R,s) = Σ_n1 G(mR,n1) G(R,n1+s):  ḠR(R',x) += Σ_s conj(G(m(R'),x+s)) C̄(m(R'),s) + Σ_s conj(G(m(R'),x-s)) C̄(R',s)
__global__ void k_adj_u2_corr(const cplx* GR, const cplx* Cbar, cplx* GRbar, Dims d) {
    const int NS = 2 * d.NG - 1, NR = d.L * d.L;
    const size_t w = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (size_t)NR * d.NG) return;
    const int x = (int)(w % d.NG) - d.nG, Rp = (int)(w / d.NG);
    const int R = mirror(Rp, d.L);
    cplx acc = mk(0, 0);
    for (int t = lane; t < NS; t += 32) {
        const int s = t - (d.NG - 1);
        if (fin(x + s, d.nG)) acc = cfmac(GR[ixG(d, R, x + s)], Cbar[(size_t)R * NS + t], acc);
        if (fin(x - s, d.nG)) acc = cfmac(GR[ixG(d, R, x - s)], Cbar[(size_t)Rp * NS + t], acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) GRbar[w] += acc;
}

// ---- Σ_R(R,ν) = Σ_Ω [G(mR,Ω-ν-1) LppR(R,Ω,ν) + G(R,Ω+ν) LphR(mR,Ω,ν)] for ν in the K2 box ----
// L̄R elementwise; ḠR by gathers over Ω
__global__ void k_adj_sigma_L(const cplx* GR, const cplx* SRbar, cplx* LRbar, Dims d) {
    const int NR = d.L * d.L, rows = d.N2O * d.N2n;
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= (size_t)2 * NR * rows) return;
    const int which = (int)(i / ((size_t)NR * rows));
    const size_t r = i % ((size_t)NR * rows);
    const int nu = (int)(r % d.N2n) - d.n2n;
    const int m = (int)((r / d.N2n) % d.N2O) - (d.n2O - 1);
    const int Rq = (int)(r / rows);  // the R index of LR
    cplx v = mk(0, 0);
    if (!fin(nu, d.nG)) {  // Σ_R exists on the G box only
    } else if (which == 0) {  // LppR(R,Ω,ν): conj(G(mR, Ω-ν-1)) S̄R(R,ν)
        const int a = m - nu - 1;
        if (fin(a, d.nG)) v = cmulc(GR[ixG(d, mirror(Rq, d.L), a)], SRbar[ixG(d, Rq, nu)]);
    } else {  // LphR(R',Ω,ν) with R' = mR: conj(G(R, Ω+ν)) S̄R(R,ν), R = m(R')
        const int b = m + nu, R = mirror(Rq, d.L);
        if (fin(b, d.nG)) v = cmulc(GR[ixG(d, R, b)], SRbar[ixG(d, R, nu)]);
    }
    LRbar[i] = v;
}
__global__ void k_adj_sigma_G(const cplx* LppR, const cplx* LphR, const cplx* SRbar, cplx* GRbar, Dims d) {
    const int NR = d.L * d.L;
    const size_t w = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (size_t)NR * d.NG) return;
    const int x = (int)(w % d.NG) - d.nG, Rp = (int)(w / d.NG);
    const int mRp = mirror(Rp, d.L);
    cplx acc = mk(0, 0);
    for (int t = lane; t < d.N2O; t += 32) {
        const int m = t - (d.n2O - 1);
        const int nu1 = m - x - 1;  // G(mR, a) with mR = R', a = x: R = m(R')
        if (fin(nu1, d.n2n) && fin(nu1, d.nG)) acc = cfmac(LppR[ix2(d, mRp, m, nu1)], SRbar[ixG(d, mRp, nu1)], acc);
        const int nu2 = x - m;  // G(R, b) with R = R', b = x
        if (fin(nu2, d.n2n) && fin(nu2, d.nG)) acc = cfmac(LphR[ix2(d, mRp, m, nu2)], SRbar[ixG(d, Rp, nu2)], acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) GRbar[w] += acc;
}

// ---- SymmetryGroup broadcast + FL epilogue + t-channel recombination (k_finalize3), transposed ----
__global__ void k_adj_finalize3(Finalize3 f, int k2_epilogue, int t_recombine, size_t n, cplx* FLbar0, cplx* FLbar1,
                                cplx* FLbar2) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    // f.raw[c]: the output cotangents ō_c (read), f.out[c]: the representatives' cotangents (scatter)
    cplx v[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] = f.raw[c] ? f.raw[c][i] : mk(0, 0);
    if (t_recombine) {
        const cplx h = v[CH_T] * 0.5;
        v[CH_T] = h;
        v[CH_A] += h;
    }
    if (k2_epilogue) {
        cplx* FLb[3] = {FLbar0, FLbar1, FLbar2};
        if (FLb[CH_P]) FLb[CH_P][i] += v[CH_P];
        if (FLb[CH_A]) FLb[CH_A][i] += v[CH_A] + v[CH_T] * -1.0;
        if (FLb[CH_T]) FLb[CH_T][i] += v[CH_T] * 2.0;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (!f.out[c]) continue;
        if (f.map[c]) {
            const uint32_t e = f.map[c][i];
            aadd(f.out[c] + (e >> 2), apply_op((int)(e & 3u), v[c]));
        } else {
            f.out[c][i] += v[c];
        }
    }
}

// ---- SDE L (sde_L_body), transposed: scatter into the new vertex's cotangent, Π̄, S̄Π ----
template <int WHICH>
__device__ void adj_sde_L_body(const VertP& F, const VertBar& Fb, const cplx* Pi, const cplx* SPi, cplx* Pibar,
                               cplx* SPibar, const cplx* rawbar, const int* items, int nitems, double rs,
                               const Dims& d) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nitems) return;
    const int idx = items ? items[w] : w;
    const int nu = idx % d.N2n - d.n2n;
    const int m = (idx / d.N2n) % d.N2O - (d.n2O - 1);
    const int P = idx / (d.N2n * d.N2O);
    const cplx s = rawbar[idx] * (d.T * d.U);
    cplx cbar = mk(0, 0);
    cplx c;
    if (WHICH == 0) c = chan_eval(F.g[CH_P], d, m, FINF, nu, P);
    else c = chan_eval(F.g[CH_T], d, m, nu, FINF, P) + chan_eval(F.g[CH_A], d, m, nu, FINF, P);
    if (WHICH == 0) {
        for (int t = lane; t < d.N2n; t += 32) {
            const int n = m - (t - d.n2n) - 1;
            if (!fin(n, d.nPw)) continue;
            const size_t ip = ixPi(d, P, m, n);
            const cplx g = chan_eval(F.g[CH_P], d, m, m - n - 1, nu, P) - c;
            const cplx pi = Pi[ip];
            aadd(Pibar + ip, cmulc(g, s));
            const cplx gb = cmulc(pi, s);
            chan_adj(Fb.g[CH_P], d, m, m - n - 1, nu, P, gb);
            cbar = cbar - gb;
        }
    } else {
        for (int n = -d.n2n + lane; n < d.n2n; n += 32) {
            if (!fin(n, d.nPw)) continue;
            const size_t ip = ixPi(d, P, m, n);
            const cplx g = chan_eval(F.g[CH_T], d, m, nu, n, P) + chan_eval(F.g[CH_A], d, m, nu, n, P) - c;
            const cplx pi = Pi[ip];
            aadd(Pibar + ip, cmulc(g, s));
            const cplx gb = cmulc(pi, s);
            chan_adj(Fb.g[CH_T], d, m, nu, n, P, gb);
            chan_adj(Fb.g[CH_A], d, m, nu, n, P, gb);
            cbar = cbar - gb;
        }
    }
    if (rs != 0.0) {  // RefVertex part: linear in Π
        const cplx sr = s * rs;
        for (int t = lane; t < d.NRn; t += 32) {
            const int r = t - d.nRn;
            const int n = (WHICH == 0) ? m - r - 1 : r;
            if (!fin(n, d.nPw)) continue;
            cplx g;
            if (WHICH == 0) g = ref_pSp(F, d, CH_P, m, m - n - 1, nu) - mk(d.U, 0);
            else g = ref_pSp(F, d, CH_A, m, nu, n) + ref_pSp(F, d, CH_T, m, nu, n) - mk(2.0 * d.U, 0);
            aadd(Pibar + ixPi(d, P, m, n), cmulc(g, sr));
        }
    }
    cbar = warp_sum(cbar);
    if (lane == 0) {
        const size_t is = (size_t)P * d.NPO + (m + d.nPO - 1);
        cbar += cmulc(SPi[is], s);
        aadd(SPibar + is, cmulc(c, s));
        if (WHICH == 0) chan_adj(Fb.g[CH_P], d, m, FINF, nu, P, cbar);
        else { chan_adj(Fb.g[CH_T], d, m, nu, FINF, P, cbar); chan_adj(Fb.g[CH_A], d, m, nu, FINF, P, cbar); }
    }
}
__global__ void k_adj_sde_L(VertP F, VertBar Fb, BubbleP B, const cplx* SPpp, const cplx* SPph, cplx* Pbpp, cplx* Pbph,
                            cplx* SPbpp, cplx* SPbph, const cplx* rawbar, ChanWork cw, double rs, Dims d) {
    if (blockIdx.y == 0)
        adj_sde_L_body<0>(F, Fb, B.pp, SPpp, Pbpp, SPbpp, rawbar, cw.items[0], cw.nitems[0], rs, d);
    else adj_sde_L_body<1>(F, Fb, B.ph, SPph, Pbph, SPbph, rawbar + cw.nitems[2], cw.items[1], cw.nitems[1], rs, d);
}

// ---- K1 / K2 BSE (bse_K1_body, bse_K2_row), transposed ----
template <int CH>
__device__ void adj_K1_body(const VertP& F, const FLP& FL, const cplx* Pi, const cplx* Pi0, const cplx* SX,
                            const VertBar& Fb, const FLBar& FLb, cplx* Pibar, cplx* SXbar, const cplx* rawbar,
                            const int* items, int nitems, const Dims& d) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nitems) return;
    const int idx = items ? items[w] : w;
    const int m = idx % d.N1 - (d.n1 - 1), P = idx / d.N1;
    constexpr int SP = (CH == CH_T) ? SP_D : SP_P;
    const cplx s = rawbar[idx] * (d.T * (CH == CH_T ? -1.0 : 1.0));
    const cplx c = vert_eval(F, d, CH, SP, m, FINF, FINF, P);
    cplx cbar = mk(0, 0);
    if (bin(m, d.n2O)) {
        for (int n = -d.n2n + lane; n < d.n2n; n += 32) {
            if (!fin(n, d.nPw)) continue;
            const int wt = cross(CH, m, n);
            const cplx Fl = vert_eval(F, d, CH, SP, m, FINF, n, P) - c;
            const cplx FLr = fl_right(FL.K2[CH_P], FL.K2[CH_T], FL.K2[CH_A], d, CH, m, wt, P);
            const size_t ip = ixPi(d, P, m, n);
            const cplx pi = Pi[ip], pi0 = Pi0[ip];
            const cplx X = cfma(pi, FLr, (pi - pi0) * d.U);
            const cplx Flb = cmulc(X, s);
            vert_adj(Fb, d, CH, SP, m, FINF, n, P, FL_ALL, Flb);
            cbar = cbar - Flb;
            const cplx Xb = cmulc(Fl, s);
            aadd(Pibar + ip, cmulc(FLr + mk(d.U, 0), Xb));
            fl_right_adj(FLb, d, CH, m, wt, P, cmulc(pi, Xb));
        }
    }
    cbar = warp_sum(cbar);
    if (lane == 0) {
        const size_t is = (size_t)CH * d.Nq * d.NPO + (size_t)P * d.NPO + (m + d.nPO - 1);
        cbar += cmulc(SX[is], s);
        aadd(SXbar + is, cmulc(c, s));
        vert_adj(Fb, d, CH, SP, m, FINF, FINF, P, FL_ALL, cbar);
    }
}
// K2 BSE, transposed in the form the forward kernel computes (bse_K2_row):
//   out = T s [c S_X + Σ_{ω ∈ window} D(ω) X(ω)],  c = own K2(Ω, ν) (t: 2 γt - γa),
//   D = the reduced vertex difference (k2_vertex_diff), X = Π FL(Ω, ω̃, ∞) + (Π - Π0) U.
// The own channel's K1 and K2 terms of F(Ω,ν,ω) - F(Ω,∞,ω) cancel exactly, so they receive no
// scatter; only the own K3, the other two channels, Π̄, FL̄ and S̄_X do.
template <int CH>
__device__ void adj_K2_body(const VertP& F, const FLP& FL, const cplx* Pi, const cplx* Pi0, const cplx* SX,
                            const VertBar& Fb, const FLBar& FLb, cplx* Pibar, cplx* SXbar, const cplx* rawbar,
                            const int* items, int nitems, const Dims& d) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nitems) return;
    const int idx = items ? items[w] : w;
    const int nu = idx % d.N2n - d.n2n;
    const int m = (idx / d.N2n) % d.N2O - (d.n2O - 1);
    const int P = idx / (d.N2n * d.N2O);
    const cplx s = rawbar[idx] * (d.T * (CH == CH_T ? -1.0 : 1.0));
    Windows win;
    const int lo = -d.nPw, hi = d.nPw - 1, h1 = d.xn1 - 1;
    win.add(-d.xn2n, d.xn2n - 1, lo, hi);
    win.add(-d.nRn, d.nRn - 1, lo, hi);
    win.add(nu - h1, nu + h1, lo, hi);
    win.add(-(m + nu + 1) - h1, -(m + nu + 1) + h1, lo, hi);
    if (CH == CH_P) win.add(m - nu - 1 - h1, m - nu - 1 + h1, lo, hi);
    win.merge();
    for (int t = lane; t < win.total; t += 32) {
        const int n = win.at(t);
        const int wt = cross(CH, m, n);
        const cplx D = k2_vertex_diff<CH>(F, d, m, nu, n, P);
        const cplx FLr = fl_right(FL.K2[CH_P], FL.K2[CH_T], FL.K2[CH_A], d, CH, m, wt, P);
        const size_t ip = ixPi(d, P, m, n);
        const cplx pi = Pi[ip], pi0 = Pi0[ip];
        const cplx X = cfma(pi, FLr, (pi - pi0) * d.U);
        const cplx Db = cmulc(X, s);
        if (CH != CH_T) {
            pSp_k2diff_adj(Fb, d, CH, m, nu, n, P, Db);
        } else {
            pSp_k2diff_adj(Fb, d, CH_T, m, nu, n, P, Db * 2.0);
            pSp_k2diff_adj(Fb, d, CH_A, m, nu, n, P, Db * -1.0);
        }
        const cplx Xb = cmulc(D, s);
        aadd(Pibar + ip, cmulc(FLr + mk(d.U, 0), Xb));
        fl_right_adj(FLb, d, CH, m, wt, P, cmulc(pi, Xb));
    }
    if (lane == 0) {
        const size_t is = (size_t)CH * d.Nq * d.NPO + (size_t)P * d.NPO + (m + d.nPO - 1);
        const cplx c = k2_c<CH>(F, d, m, nu, P);
        aadd(SXbar + is, cmulc(c, s));
        const cplx cb = cmulc(SX[is], s);
        if (bin(m, d.n1) && bin(m, d.n2O) && fin(nu, d.n2n)) {
            if (CH != CH_T) {
                k2a(Fb.g[CH], d, m, nu, P, cb);
            } else {
                k2a(Fb.g[CH_T], d, m, nu, P, cb * 2.0);
                k2a(Fb.g[CH_A], d, m, nu, P, cb * -1.0);
            }
        }
    }
}
__global__ void k_adj_K1(VertP F, FLP FL, BubbleP B, const cplx* SX, VertBar Fb, FLBar FLb, cplx* Pbpp, cplx* Pbph,
                         cplx* SXbar, const cplx* rawbar, ChanWork cw, size_t n1, Dims d) {
    switch (blockIdx.y) {
        case CH_P: adj_K1_body<CH_P>(F, FL, B.pp, B.pp0, SX, Fb, FLb, Pbpp, SXbar, rawbar, cw.items[CH_P], cw.nitems[CH_P], d); break;
        case CH_T: adj_K1_body<CH_T>(F, FL, B.ph, B.ph0, SX, Fb, FLb, Pbph, SXbar, rawbar + n1, cw.items[CH_T], cw.nitems[CH_T], d); break;
        default:   adj_K1_body<CH_A>(F, FL, B.ph, B.ph0, SX, Fb, FLb, Pbph, SXbar, rawbar + 2 * n1, cw.items[CH_A], cw.nitems[CH_A], d); break;
    }
}
__global__ void k_adj_K2(VertP F, FLP FL, BubbleP B, const cplx* SX, VertBar Fb, FLBar FLb, cplx* Pbpp, cplx* Pbph,
                         cplx* SXbar, const cplx* rawbar, ChanWork cw, size_t n2, Dims d) {
    switch (blockIdx.y) {
        case CH_P: adj_K2_body<CH_P>(F, FL, B.pp, B.pp0, SX, Fb, FLb, Pbpp, SXbar, rawbar, cw.items[CH_P], cw.nitems[CH_P], d); break;
        case CH_T: adj_K2_body<CH_T>(F, FL, B.ph, B.ph0, SX, Fb, FLb, Pbph, SXbar, rawbar + n2, cw.items[CH_T], cw.nitems[CH_T], d); break;
        default:   adj_K2_body<CH_A>(F, FL, B.ph, B.ph0, SX, Fb, FLb, Pbph, SXbar, rawbar + 2 * n2, cw.items[CH_A], cw.nitems[CH_A], d); break;
    }
}

// ---- S_X = (SΠ - SΠ0) U + Σ_t Π FL, transposed ----
__global__ void k_adj_sx(const cplx* Pipp, const cplx* Piph, FLP FL, const cplx* SXbar, cplx* Pbpp, cplx* Pbph,
                         cplx* SPibar, FLBar FLb, Dims d) {
    const size_t per = (size_t)d.Nq * d.NPO;
    const size_t i = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= 3 * per) return;
    const int ch = (int)(i / per);
    const size_t r = i % per;
    const int m = (int)(r % d.NPO) - (d.nPO - 1), P = (int)(r / d.NPO);
    const int w = (ch == CH_P) ? 0 : 1;
    const cplx* Pi = w ? Piph : Pipp;
    cplx* Pb = w ? Pbph : Pbpp;
    const cplx g = SXbar[i];
    if (lane == 0) aadd(SPibar + w * per + r, g * d.U);
    if (bin(m, d.n2O)) {
        for (int t = lane; t < d.N2n; t += 32) {
            const int nt = t - d.n2n;
            const int n = (ch == CH_P) ? m - nt - 1 : nt;
            if (!fin(n, d.nPw)) continue;
            const size_t ip = ixPi(d, P, m, n);
            const cplx flr = fl_right(FL.K2[CH_P], FL.K2[CH_T], FL.K2[CH_A], d, ch, m, nt, P);
            aadd(Pb + ip, cmulc(flr, g));
            fl_right_adj(FLb, d, ch, m, nt, P, cmulc(Pi[ip], g));
        }
    }
}

// ---- left K2 BSE (bse_L_K2_body), transposed ----
template <int CH>
__device__ void adj_L_K2_body(const cplx* Pi0, const VertBar& Fb, const cplx* rawbar, const int* items, int nitems,
                              const Dims& d) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nitems) return;
    const int idx = items ? items[w] : w;
    const int nu = idx % d.N2n - d.n2n;
    const int m = (idx / d.N2n) % d.N2O - (d.n2O - 1);
    const int P = idx / (d.N2n * d.N2O);
    constexpr int SP = (CH == CH_T) ? SP_D : SP_P;
    constexpr int IRR = (CH == CH_P) ? (FL_GT | FL_GA) : (CH == CH_T ? (FL_GP | FL_GA) : (FL_GP | FL_GT));
    const cplx s = rawbar[idx] * (d.U * d.T * (CH == CH_T ? -1.0 : 1.0));
    if (d.local) {
        for (int n = -d.nPw + lane; n < d.nPw; n += 32)
            vert_adj(Fb, d, CH, SP, m, nu, n, P, IRR, cmulc(Pi0[ixPi(d, P, m, n)], s));
    } else {
        for (int n = -d.n2n + lane; n < d.n2n; n += 32)
            vert_adj(Fb, d, CH, SP, m, nu, cross(CH, m, n), P, IRR, cmulc(Pi0[ixPi(d, P, m, n)], s));
    }
}
__global__ void k_adj_L_K2(BubbleP B, VertBar Fb, const cplx* rawbar, ChanWork cw, size_t n2, Dims d) {
    switch (blockIdx.y) {
        case CH_P: adj_L_K2_body<CH_P>(B.pp0, Fb, rawbar, cw.items[CH_P], cw.nitems[CH_P], d); break;
        case CH_T: adj_L_K2_body<CH_T>(B.ph0, Fb, rawbar + n2, cw.items[CH_T], cw.nitems[CH_T], d); break;
        default:   adj_L_K2_body<CH_A>(B.ph0, Fb, rawbar + 2 * n2, cw.items[CH_A], cw.nitems[CH_A], d); break;
    }
}

// ---- K3 caches (k_build_cache), transposed: one thread per cache element of the listed blocks ----
__global__ void k_adj_cache(VertBar Fb, Caches Cb, const int* blocks, int nblocks, Dims d) {
    const size_t bs = (size_t)d.N3n * d.N3n;
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)nblocks * bs) return;
    const int bl = blocks ? blocks[t / bs] : (int)(t / bs);
    const size_t e = t % bs;
    const size_t i = (size_t)bl * bs + e;
    const int b = (int)(e % d.N3n) - d.n3n;
    const int a = (int)(e / d.N3n) - d.n3n;
    const int m = bl % d.N3O - (d.n3O - 1);
    const int P = bl / d.N3O;
    const cplx c0 = Cb.c[0][i], c4 = Cb.c[4][i], c5 = Cb.c[5][i], c6 = Cb.c[6][i];
    const cplx c7 = Cb.c[7][i], c8 = Cb.c[8][i], c9 = Cb.c[9][i];
    // v6 = 2 gt - ga, v9 = 2 ft - fa, fx = [F0|Gx at (a,b)] - [F0|Gx at (∞,b)] + gx
    const cplx fpb = c7, fab = c8 - c9, ftb = c9 * 2.0;
    const cplx gppb = c4 + fpb, gab = c5 - c6 + fab, gtb = c6 * 2.0 + ftb;
    vert_adj(Fb, d, CH_P, SP_X, m, a, b, P, FL_GT | FL_GA, c0);
    pSp_adj(Fb, d, CH_P, m, a, b, P, FL_GT | FL_GA, gppb);
    pSp_adj(Fb, d, CH_A, m, a, b, P, FL_GP | FL_GT, gab);
    pSp_adj(Fb, d, CH_T, m, a, b, P, FL_GP | FL_GA, gtb);
    pSp_adj(Fb, d, CH_P, m, a, b, P, FL_GP, fpb);
    pSp_adj(Fb, d, CH_P, m, FINF, b, P, FL_GP, fpb * -1.0);
    pSp_adj(Fb, d, CH_A, m, a, b, P, FL_GA, fab);
    pSp_adj(Fb, d, CH_A, m, FINF, b, P, FL_GA, fab * -1.0);
    pSp_adj(Fb, d, CH_T, m, a, b, P, FL_GT, ftb);
    pSp_adj(Fb, d, CH_T, m, FINF, b, P, FL_GT, ftb * -1.0);
}

// ---- K3 BSE GEMM, transposed ----
// M of the forward contraction (mode 0: Π0·B0; mode 1: s1[(Π-Π0) B0 + Π Γs] + s2 Π γL) per listed block
__global__ void k_adj_build_M(K3Args3 args, int mode, Ptr3 Mout, Dims d) {
    const int N = d.N3n;
    const size_t bs = (size_t)N * N;
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const int slot = blockIdx.y;
    if (t >= (size_t)args.nblocks * bs) return;
    const int blk = args.blocks ? args.blocks[t / bs] : (int)(t / bs);
    const K3Args& a = args.a[slot];
    const int CH = args.ch[slot];
    const int m = blk % d.N3O - (d.n3O - 1), P = blk / d.N3O;
    const size_t base = (size_t)blk * bs;
    const int k = (int)((t % bs) / N), col = (int)(t % N);  // M(ω = k, ν' = col)
    const int o = k - d.n3n;
    const size_t ip = ixPi(d, P, m, o);
    const cplx pi0 = a.Pi0[ip];
    const cplx f0 = a.B0[base + (size_t)k * N + col];
    cplx v;
    if (mode == 0) {
        v = pi0 * f0;
    } else {
        const double s1 = (CH == CH_A) ? 1.0 : -1.0, s2 = (CH == CH_T) ? -1.0 : 1.0;
        const cplx pi = a.Pi[ip];
        const cplx gs = (CH == CH_P) ? a.G[base + (size_t)k * N + col] : a.G[base + (size_t)col * N + k];
        v = ((pi - pi0) * f0 + pi * gs) * s1;
        const int ot = cross(CH, m, o);
        if (fin(ot, d.n3n)) {
            const size_t il = base + (size_t)(ot + d.n3n) * N + col;
            const cplx gl = (CH == CH_T) ? a.FLt[il] * 2.0 - a.FLa[il] : a.FLc[il];
            v += pi * gl * s2;
        }
    }
    Mout.p[slot][base + (size_t)k * N + col] = v;
}
// batched C[b] = α op(A[b]) op(B[b]) (C += when accumulating) over the listed N x N blocks, op: 0 = as
// is, 1 = conjugate transpose; slot = blockIdx.z.  TILE x TILE output tiles (TILE = 16, 24 or 32 by N,
// as the forward K3 GEMM picks them, so that no block is padded beyond its size), 2 x 2 outputs per
// thread, K chunks of 8, and the forward GEMM's three-multiplication complex product:
// t1 = Σ ar br, t2 = Σ ai bi, t3 = Σ (ar + ai)(br + bi), C = (t1 - t2) + i (t3 - t1 - t2).
struct GemmBatch {
    const cplx* A[3];
    const cplx* B[3];
    cplx* C[3];
    double alpha[3];
    int accumulate;  // C += instead of C =
    const int* blocks;
    int nblocks;
};
template <int OPA, int OPB, int TILE>
__global__ void __launch_bounds__((TILE / 2) * (TILE / 2)) k_adj_gemm(GemmBatch g, Dims d) {
    constexpr int TK = 8, H = TILE / 2, NT = H * H;
    __shared__ cplx As[TILE][TK + 1];
    __shared__ cplx Bs[TK][TILE + 1];
    __shared__ double Asum[TILE][TK + 1], Bsum[TK][TILE + 1];
    const int N = d.N3n;
    const int slot = blockIdx.z;
    const int nt = (N + TILE - 1) / TILE;
    const int bidx = blockIdx.x / (nt * nt), tile = blockIdx.x % (nt * nt);
    const int blk = g.blocks ? g.blocks[bidx] : bidx;
    const size_t base = (size_t)blk * N * N;
    const int row0 = (tile / nt) * TILE, col0 = (tile % nt) * TILE;
    const int tid = threadIdx.x, tx = tid % H, ty = tid / H;
    // the slot's operands, chosen without indexing the parameter arrays by a run-time value (which
    // would copy the parameters to local memory)
    const cplx* A = (slot == 0 ? g.A[0] : slot == 1 ? g.A[1] : g.A[2]) + base;
    const cplx* B = (slot == 0 ? g.B[0] : slot == 1 ? g.B[1] : g.B[2]) + base;
    double t1[2][2] = {{0, 0}, {0, 0}}, t2[2][2] = {{0, 0}, {0, 0}}, t3[2][2] = {{0, 0}, {0, 0}};
    for (int k0 = 0; k0 < N; k0 += TK) {
        for (int e = tid; e < TILE * TK; e += NT) {
            // op(A)[r][k]: as is, k runs along memory; conjugate transpose, r does
            const int r = OPA ? e % TILE : e / TK, kk = OPA ? e / TILE : e % TK;
            const int gr = row0 + r, gk = k0 + kk;
            cplx v = mk(0, 0);
            if (gr < N && gk < N) v = OPA ? cj(A[(size_t)gk * N + gr]) : A[(size_t)gr * N + gk];
            As[r][kk] = v;
            Asum[r][kk] = v.x + v.y;
        }
        for (int e = tid; e < TK * TILE; e += NT) {
            // op(B)[k][c]: as is, c runs along memory; conjugate transpose, k does
            const int kk = OPB ? e % TK : e / TILE, c = OPB ? e / TK : e % TILE;
            const int gk = k0 + kk, gc = col0 + c;
            cplx v = mk(0, 0);
            if (gk < N && gc < N) v = OPB ? cj(B[(size_t)gc * N + gk]) : B[(size_t)gk * N + gc];
            Bs[kk][c] = v;
            Bsum[kk][c] = v.x + v.y;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; ++kk) {
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const cplx av = As[ty + H * i][kk];
                const double sa = Asum[ty + H * i][kk];
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const cplx bv = Bs[kk][tx + H * j];
                    t1[i][j] = fma(av.x, bv.x, t1[i][j]);
                    t2[i][j] = fma(av.y, bv.y, t2[i][j]);
                    t3[i][j] = fma(sa, Bsum[kk][tx + H * j], t3[i][j]);
                }
            }
        }
        __syncthreads();
    }
    const double alpha = slot == 0 ? g.alpha[0] : slot == 1 ? g.alpha[1] : g.alpha[2];
    cplx* Cb = (slot == 0 ? g.C[0] : slot == 1 ? g.C[1] : g.C[2]) + base;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int r = row0 + ty + H * i, c = col0 + tx + H * j;
            if (r < N && c < N) {
                cplx* C = Cb + (size_t)r * N + c;
                const cplx v = cplx{t1[i][j] - t2[i][j], t3[i][j] - (t1[i][j] + t2[i][j])} * alpha;
                *C = g.accumulate ? *C + v : v;
            }
        }
}
template <int OPA, int OPB, int TILE>
void launch_adj_gemm_tile(cudaStream_t s, const GemmBatch& g, const Dims& d) {
    const int nt = (d.N3n + TILE - 1) / TILE;
    const dim3 grid((unsigned)(g.nblocks * nt * nt), 1, 3);
    k_adj_gemm<OPA, OPB, TILE><<<grid, (TILE / 2) * (TILE / 2), 0, s>>>(g, d);
}
template <int OPA, int OPB>
void launch_adj_gemm(cudaStream_t s, const GemmBatch& g, const Dims& d) {
    if (d.N3n <= 16) launch_adj_gemm_tile<OPA, OPB, 16>(s, g, d);
    else if (d.N3n <= 24) launch_adj_gemm_tile<OPA, OPB, 24>(s, g, d);
    else launch_adj_gemm_tile<OPA, OPB, 32>(s, g, d);
}
// mode 1: M̄ -> Π̄ (row sums), Γ̄s, γ̄L (box) and the epilogue γ̄L(ν,ν') += ō; warp per (slot, block, ω)
__global__ void k_adj_distribute_M(K3Args3 args, Ptr3 Mbar, Ptr3 Obar, Ptr3 Gbar, cplx* Pbpp, cplx* Pbph, cplx* FLb0,
                                   cplx* FLb1, cplx* FLb2, Dims d) {
    const int N = d.N3n;
    const size_t wid = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int slot = blockIdx.y;
    if (wid >= (size_t)args.nblocks * N) return;
    const int blk = args.blocks ? args.blocks[wid / N] : (int)(wid / N);
    const int k = (int)(wid % N);
    const K3Args& a = args.a[slot];
    const int CH = args.ch[slot];
    cplx* FLb[3] = {FLb0, FLb1, FLb2};
    const int m = blk % d.N3O - (d.n3O - 1), P = blk / d.N3O;
    const size_t base = (size_t)blk * N * N;
    const double s1 = (CH == CH_A) ? 1.0 : -1.0, s2 = (CH == CH_T) ? -1.0 : 1.0;
    const int o = k - d.n3n;
    const size_t ip = ixPi(d, P, m, o);
    const cplx pi = a.Pi[ip];
    const int ot = cross(CH, m, o);
    const bool inb = fin(ot, d.n3n);
    cplx pib = mk(0, 0);
    for (int col = lane; col < N; col += 32) {
        const cplx mb = Mbar.p[slot][base + (size_t)k * N + col];
        const size_t ig = (CH == CH_P) ? base + (size_t)k * N + col : base + (size_t)col * N + k;
        const cplx f0 = a.B0[base + (size_t)k * N + col];
        cplx dMdpi = (f0 + a.G[ig]) * s1;
        aadd(Gbar.p[slot] + ig, cmulc(pi * s1, mb));
        if (inb) {
            const size_t il = base + (size_t)(ot + d.n3n) * N + col;
            const cplx gl = (CH == CH_T) ? a.FLt[il] * 2.0 - a.FLa[il] : a.FLc[il];
            dMdpi += gl * s2;
            const cplx glb = cmulc(pi * s2, mb);
            if (CH == CH_T) { aadd(FLb[CH_T] + il, glb * 2.0); aadd(FLb[CH_A] + il, glb * -1.0); }
            else aadd(FLb[CH] + il, glb);
        }
        pib = cfmac(dMdpi, mb, pib);
        // epilogue: out(ν = k, ν' = col) += γL(k, col)
        const size_t io = base + (size_t)k * N + col;
        const cplx ob = Obar.p[slot][io];
        if (CH == CH_T) { aadd(FLb[CH_T] + io, ob * 2.0); aadd(FLb[CH_A] + io, ob * -1.0); }
        else aadd(FLb[CH] + io, ob);
    }
    pib = warp_sum(pib);
    if (lane == 0) aadd((CH == CH_P ? Pbpp : Pbph) + ip, pib);
}

// ---- bubbles and their row sums, transposed (gathers over Ω; G(R) of the base point) ----
// ḠR(R',x) for x in the G box, from Π̄R[w][R][Ω][ν] (stored window) and S̄R[w][R][Ω] (full-mesh row
// sums, nullptr when the row sums are plain sums of the stored window)
__device__ __forceinline__ cplx gt_val(const cplx* GR, const Dims& d, int R, int n) {
    if (fin(n, d.nG)) return GR[ixG(d, R, n)];
    if (R != 0) return mk(0, 0);  // outside the box a product vanishes for R ≠ 0
    return mk(1.0 / ((2.0 * n + 1.0) * M_PI * d.T), 0.0);
}
__global__ void k_adj_bubble(const cplx* GR, const cplx* PbRpp, const cplx* PbRph, const cplx* SbRpp,
                             const cplx* SbRph, cplx* GRbar, Dims d) {
    const int NR = d.L * d.L;
    const size_t w = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= (size_t)NR * d.NG) return;
    const int x = (int)(w % d.NG) - d.nG, Rp = (int)(w / d.NG);
    const int mRp = mirror(Rp, d.L);
    cplx acc = mk(0, 0);
    for (int t = lane; t < d.NPO; t += 32) {
        const int m = t - (d.nPO - 1);
        // pp: Π(R,Ω,n) = G(R,Ω-n-1) G(R,n); partner of x in both roles: G(R', Ω-x-1)
        {
            const cplx p = gt_val(GR, d, Rp, m - x - 1);
            if (p.x != 0.0 || p.y != 0.0) {
                cplx s = mk(0, 0);
                const int n1 = m - x - 1;  // x as the first factor
                if (fin(n1, d.nPw)) s += PbRpp[ixPi(d, Rp, m, n1)];
                if (fin(x, d.nPw)) s += PbRpp[ixPi(d, Rp, m, x)];
                if (SbRpp) {
                    const cplx sr = SbRpp[(size_t)Rp * d.NPO + t];
                    if (fin(n1, d.nPn)) s += sr;
                    if (fin(x, d.nPn)) s += sr;
                }
                acc = cfmac(p, s, acc);
            }
        }
        // ph: Π(R,Ω,n) = G(R,Ω+n) G(mR,n)
        {
            const int n1 = x - m;  // x as the first factor: R = R', partner G(m(R'), x-Ω)
            const cplx p1 = gt_val(GR, d, mRp, n1);
            if (p1.x != 0.0 || p1.y != 0.0) {
                cplx s = mk(0, 0);
                if (fin(n1, d.nPw)) s += PbRph[ixPi(d, Rp, m, n1)];
                if (SbRph && fin(n1, d.nPn)) s += SbRph[(size_t)Rp * d.NPO + t];
                acc = cfmac(p1, s, acc);
            }
            const cplx p2 = gt_val(GR, d, mRp, m + x);  // x as the second factor: R = m(R'), partner G(m(R'), Ω+x)
            if (p2.x != 0.0 || p2.y != 0.0) {
                cplx s = mk(0, 0);
                if (fin(x, d.nPw)) s += PbRph[ixPi(d, mRp, m, x)];
                if (SbRph && fin(x, d.nPn)) s += SbRph[(size_t)mRp * d.NPO + t];
                acc = cfmac(p2, s, acc);
            }
        }
    }
    acc = warp_sum(acc);
    if (lane == 0) GRbar[w] += acc;
}
// row sums of the stored window (local, or a window equal to the mesh): Π̄ += S̄Π broadcast over ν
__global__ void k_adj_rowsum(const cplx* SPibar, cplx* Pbpp, cplx* Pbph, Dims d) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t per = (size_t)d.Nq * d.NPO * d.NPw;
    if (i >= 2 * per) return;
    const int w = (int)(i / per);
    const size_t r = i % per;
    const size_t row = r / d.NPw;  // P * NPO + iΩ
    (w ? Pbph : Pbpp)[r] += SPibar[(size_t)w * d.Nq * d.NPO + row];
}
// momentum averages A = Σ_P K[P] / Nq, transposed: K̄[P] += Ā / Nq
__global__ void k_adj_qavg(ChanBarArrays bar, Dims d) {
    const int ch = blockIdx.y / 3, cl = blockIdx.y % 3;
    const size_t per = cl == 0 ? (size_t)d.N1 : (cl == 1 ? (size_t)d.N2O * d.N2n : (size_t)d.N3O * d.N3n * d.N3n);
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= per) return;
    const cplx* A = cl == 0 ? bar.A1[ch] : (cl == 1 ? bar.A2[ch] : bar.A3[ch]);
    cplx* K = cl == 0 ? bar.K1[ch] : (cl == 1 ? bar.K2[ch] : bar.K3[ch]);
    const cplx v = A[i] * (1.0 / d.Nq);
    for (int P = 0; P < d.Nq; ++P) K[(size_t)P * per + i] += v;
}

inline unsigned nb(size_t n, int t) { return (unsigned)((n + t - 1) / t); }
#define LCHK() do { cudaError_t e_ = cudaGetLastError(); if (e_ != cudaSuccess) return e_; } while (0)

}  // namespace

// ---- launchers ----
cudaError_t launch_adj_assemble(cudaStream_t s, const cplx* Sbar, const uint32_t* map, cplx* Sin_bar, cplx* SU2_bar,
                                size_t n, int hartree, double U, double* nbar) {
    k_adj_assemble<<<nb(n, 256), 256, 0, s>>>(Sbar, map, Sin_bar, SU2_bar, n);
    LCHK();
    if (hartree) {
        k_adj_occ_reduce<<<1, 1024, 0, s>>>(Sbar, n, U, nbar);
        LCHK();
    }
    return cudaSuccess;
}
cudaError_t launch_adj_occupation(cudaStream_t s, cplx* Gbar, const double* nbar, double T, int Nk, size_t n) {
    k_adj_occ_apply<<<nb(n, 256), 256, 0, s>>>(Gbar, nbar, T, Nk, n);
    LCHK(); return cudaSuccess;
}
cudaError_t launch_adj_dyson(cudaStream_t s, const cplx* G, const cplx* Gbar, cplx* Sbar, size_t n) {
    k_adj_dyson<<<nb(n, 256), 256, 0, s>>>(G, Gbar, Sbar, n);
    LCHK(); return cudaSuccess;
}
cudaError_t launch_adj_u2(cudaStream_t s, const cplx* GR, const cplx* C, cplx* obar_k, cplx* obar_R, cplx* Cbar,
                          cplx* GRbar, const cplx* twm, const Dims& d) {
    // out = fft2(SR, +1, 1): S̄R = fft2(ō, -1, 1)
    const int NR = d.L * d.L, NS = 2 * d.NG - 1;
    cudaError_t e = launch_fft2(s, obar_k, obar_R, d.NG, -1, 1.0, twm, d);
    if (e != cudaSuccess) return e;
    k_adj_u2_sum<<<nb(((size_t)NR * d.NG + (size_t)NR * NS) * 32, 128), 128, 0, s>>>(GR, C, obar_R, GRbar, Cbar, d);
    LCHK();
    k_adj_u2_corr<<<nb((size_t)NR * d.NG * 32, 128), 128, 0, s>>>(GR, Cbar, GRbar, d);
    LCHK(); return cudaSuccess;
}
cudaError_t launch_adj_sigma(cudaStream_t s, const cplx* GR, const cplx* LR, const cplx* Sinbar, cplx* SRbar,
                             cplx* LRbar, cplx* Lbar, cplx* GRbar, const cplx* twm, const cplx* twp, const Dims& d) {
    // Σin = fft2(SR, +1, T): S̄R = fft2(Σ̄in, -1, T)
    const int NR = d.L * d.L, rows = d.N2O * d.N2n;
    cudaError_t e = launch_fft2(s, Sinbar, SRbar, d.NG, -1, d.T, twm, d);
    if (e != cudaSuccess) return e;
    k_adj_sigma_L<<<nb((size_t)2 * NR * rows, 256), 256, 0, s>>>(GR, SRbar, LRbar, d);
    LCHK();
    k_adj_sigma_G<<<nb((size_t)NR * d.NG * 32, 128), 128, 0, s>>>(LR, LR + (size_t)NR * rows, SRbar, GRbar, d);
    LCHK();
    // LR = fft2(L, -1, 1/NR): L̄ = fft2(L̄R, +1, 1/NR)
    e = launch_fft2(s, LRbar, Lbar, rows, +1, 1.0 / NR, twp, d);
    if (e == cudaSuccess) e = launch_fft2(s, LRbar + (size_t)NR * rows, Lbar + (size_t)NR * rows, rows, +1, 1.0 / NR, twp, d);
    return e;
}
cudaError_t launch_adj_finalize3(cudaStream_t s, const Finalize3& f, int k2_epilogue, int t_recombine, size_t n,
                                 cplx* const FLbar[3]) {
    k_adj_finalize3<<<nb(n, 256), 256, 0, s>>>(f, k2_epilogue, t_recombine, n, FLbar ? FLbar[0] : nullptr,
                                              FLbar ? FLbar[1] : nullptr, FLbar ? FLbar[2] : nullptr);
    LCHK(); return cudaSuccess;
}
static unsigned warp_grid3(const ChanWork& cw, int nch) {
    int mx = 0;
    for (int c = 0; c < nch; ++c) mx = std::max(mx, cw.nitems[c]);
    return nb((size_t)mx * 32, 128);
}
cudaError_t launch_adj_sde_L(cudaStream_t s, const VertP& F, const VertBar& Fb, const BubbleP& B, const cplx* SPpp,
                             const cplx* SPph, cplx* Pbpp, cplx* Pbph, cplx* SPbpp, cplx* SPbph, const cplx* rawbar,
                             const ChanWork& cw, size_t n2, double rs, const Dims& d) {
    ChanWork c = cw;
    c.nitems[2] = (int)n2;  // offset of the ph raw cotangents
    k_adj_sde_L<<<dim3(warp_grid3(cw, 2), 2), 128, 0, s>>>(F, Fb, B, SPpp, SPph, Pbpp, Pbph, SPbpp, SPbph, rawbar, c, rs, d);
    LCHK(); return cudaSuccess;
}
cudaError_t launch_adj_K1(cudaStream_t s, const VertP& F, const FLP& FL, const BubbleP& B, const cplx* SX,
                          const VertBar& Fb, const FLBar& FLb, cplx* Pbpp, cplx* Pbph, cplx* SXbar, const cplx* rawbar,
                          const ChanWork& cw, size_t n1, const Dims& d) {
    k_adj_K1<<<dim3(warp_grid3(cw, 3), 3), 128, 0, s>>>(F, FL, B, SX, Fb, FLb, Pbpp, Pbph, SXbar, rawbar, cw, n1, d);
    LCHK(); return cudaSuccess;
}
cudaError_t launch_adj_K2(cudaStream_t s, const VertP& F, const FLP& FL, const BubbleP& B, const cplx* SX,
                          const VertBar& Fb, const FLBar& FLb, cplx* Pbpp, cplx* Pbph, cplx* SXbar, const cplx* rawbar,
                          const ChanWork& cw, size_t n2, const Dims& d) {
    k_adj_K2<<<dim3(warp_grid3(cw, 3), 3), 128, 0, s>>>(F, FL, B, SX, Fb, FLb, Pbpp, Pbph, SXbar, rawbar, cw, n2, d);
    LCHK(); return cudaSuccess;
}
cudaError_t launch_adj_sx(cudaStream_t s, const cplx* Pipp, const cplx* Piph, const FLP& FL, const cplx* SXbar,
                          cplx* Pbpp, cplx* Pbph, cplx* SPibar, const FLBar& FLb, const Dims& d) {
    k_adj_sx<<<nb((size_t)3 * d.Nq * d.NPO * 32, 128), 128, 0, s>>>(Pipp, Piph, FL, SXbar, Pbpp, Pbph, SPibar, FLb, d);
    LCHK(); return cudaSuccess;
}
cudaError_t launch_adj_L_K2(cudaStream_t s, const BubbleP& B, const VertBar& Fb, const cplx* rawbar, const ChanWork& cw,
                            size_t n2, const Dims& d) {
    k_adj_L_K2<<<dim3(warp_grid3(cw, 3), 3), 128, 0, s>>>(B, Fb, rawbar, cw, n2, d);
    LCHK(); return cudaSuccess;
}
cudaError_t launch_adj_cache(cudaStream_t s, const VertBar& Fb, const Caches& Cb, const int* blocks, int nblocks,
                             const Dims& d) {
    const size_t n = (size_t)nblocks * d.N3n * d.N3n;
    k_adj_cache<<<nb(n, 128), 128, 0, s>>>(Fb, Cb, blocks, nblocks, d);
    LCHK(); return cudaSuccess;
}
// K3 contraction of mode 0 or 1, transposed: Ā += α ō Mᴴ into Abar[slot]; mode 1 also M̄ = α Aᴴ ō and its
// distribution into Γ̄s (Gbar[slot]), Π̄ and γ̄L (FLbar, including the epilogue term)
cudaError_t launch_adj_K3(cudaStream_t s, int mode, const K3Args3& a, const cplx* const Obar[3], cplx* const Abar[3],
                          cplx* const Gbar[3], cplx* const Mbuf[3], cplx* const Mbar[3], cplx* Pbpp, cplx* Pbph,
                          cplx* const FLbar[3], const Dims& d) {
    const int N = d.N3n;
    const size_t bs = (size_t)N * N;
    const Ptr3 mo{{Mbuf[0], Mbuf[1], Mbuf[2]}};  // slot pointers travel by value
    k_adj_build_M<<<dim3(nb((size_t)a.nblocks * bs, 256), 3), 256, 0, s>>>(a, mode, mo, d);
    LCHK();
    const double T = d.T;
    GemmBatch g{};
    g.blocks = a.blocks;
    g.nblocks = a.nblocks;
    for (int i = 0; i < 3; ++i) {
        const int ch = a.ch[i];
        g.A[i] = Obar[i];
        g.B[i] = Mbuf[i];
        g.C[i] = Abar[i];
        g.alpha[i] = mode == 0 ? T * ((ch == CH_A) ? 1.0 : -1.0) : T;
    }
    g.accumulate = 1;
    launch_adj_gemm<0, 1>(s, g, d);  // Ā += α ō Mᴴ
    LCHK();
    if (mode == 0) return cudaSuccess;
    GemmBatch h{};
    h.blocks = a.blocks;
    h.nblocks = a.nblocks;
    for (int i = 0; i < 3; ++i) {
        h.A[i] = a.a[i].A;
        h.B[i] = Obar[i];
        h.C[i] = Mbar[i];
        h.alpha[i] = T;
    }
    h.accumulate = 0;
    launch_adj_gemm<1, 0>(s, h, d);  // M̄ = T Aᴴ ō
    LCHK();
    const Ptr3 mb{{Mbar[0], Mbar[1], Mbar[2]}};
    const Ptr3 ob{{const_cast<cplx*>(Obar[0]), const_cast<cplx*>(Obar[1]), const_cast<cplx*>(Obar[2])}};
    const Ptr3 gb{{Gbar[0], Gbar[1], Gbar[2]}};
    k_adj_distribute_M<<<dim3(nb((size_t)a.nblocks * N * 32, 128), 3), 128, 0, s>>>(a, mb, ob, gb, Pbpp, Pbph, FLbar[0],
                                                                                   FLbar[1], FLbar[2], d);
    LCHK(); return cudaSuccess;
}
cudaError_t launch_adj_bubble(cudaStream_t s, const cplx* GR, cplx* Pbpp, cplx* Pbph, cplx* PbRpp, cplx* PbRph,
                              const cplx* SPibar, cplx* SRbar, cplx* GRbar, const cplx* twm, const Dims& d) {
    const int NR = d.L * d.L;
    const bool full = d.nPw == d.nPn;
    if (full) {  // row sums of the stored window: broadcast S̄Π into Π̄
        k_adj_rowsum<<<nb((size_t)2 * d.Nq * d.NPO * d.NPw, 256), 256, 0, s>>>(SPibar, Pbpp, Pbph, d);
        LCHK();
    } else {  // SΠ = fft2(SR, +1, 1): S̄R = fft2(S̄Π, -1, 1)
        const size_t nS = (size_t)d.Nq * d.NPO;
        cudaError_t e = launch_fft2(s, SPibar, SRbar, d.NPO, -1, 1.0, twm, d);
        if (e == cudaSuccess) e = launch_fft2(s, SPibar + nS, SRbar + (size_t)NR * d.NPO, d.NPO, -1, 1.0, twm, d);
        if (e != cudaSuccess) return e;
    }
    // Π(P) = Σ_R e^{+iP·R} Π(R): Π̄R = fft2(Π̄, -1, 1) (rows: the Ω x ν window)
    const int rows = d.NPO * d.NPw;
    cudaError_t e = launch_fft2(s, Pbpp, PbRpp, rows, -1, 1.0, twm, d);
    if (e == cudaSuccess) e = launch_fft2(s, Pbph, PbRph, rows, -1, 1.0, twm, d);
    if (e != cudaSuccess) return e;
    k_adj_bubble<<<nb((size_t)NR * d.NG * 32, 128), 128, 0, s>>>(GR, PbRpp, PbRph, full ? nullptr : SRbar,
                                                                full ? nullptr : SRbar + (size_t)NR * d.NPO, GRbar, d);
    LCHK(); return cudaSuccess;
}
cudaError_t launch_adj_qavg(cudaStream_t s, const ChanBarArrays& bar, const Dims& d) {
    const size_t per = std::max((size_t)d.N1, std::max((size_t)d.N2O * d.N2n, (size_t)d.N3O * d.N3n * d.N3n));
    k_adj_qavg<<<dim3(nb(per, 256), 9), 256, 0, s>>>(bar, d);
    LCHK(); return cudaSuccess;
}

}  // namespace fdga
