// fdga_anderson.cu -- device-resident Anderson acceleration (NLsolve method=:anderson).
//
// The update of one Anderson step (NLsolve 4.5.1 anderson.jl, Walker & Ni 2011; driven by
// src/solve.jl:179-188 of the reference) runs without a host round trip: the QR factor R, the
// Givens parameters of a column deletion, the Gram-Schmidt coefficients and γ = R⁻¹ Qᴴ f live in
// device memory, and each long-vector pass reduces its block partials into the coefficient it
// needs at the start of the next pass.  Every block reduces the same partials in the same fixed
// order, so all blocks use bit-identical coefficients.  Arithmetic order per element matches the
// serial restatement: modified Gram-Schmidt one column at a time, rotations i = 1..m-1 in order,
// x -= γ_i Δg_i for i = 0..m_eff-1 in order.
#include "fdga_kernels.h"

namespace fdga {

namespace {

constexpr int RT = 256;  // threads of every reduction block

// The long-vector passes are bound by GB300's FP64 pipe: complex products are written as FMAs.
// conj(a) b + c
__device__ __forceinline__ cplx cfma_conj(cplx a, cplx b, cplx c) {
    return mk(fma(a.x, b.x, fma(a.y, b.y, c.x)), fma(a.x, b.y, fma(-a.y, b.x, c.y)));
}
// c - a b
__device__ __forceinline__ cplx cfnma(cplx a, cplx b, cplx c) {
    return mk(fma(-a.x, b.x, fma(a.y, b.y, c.x)), fma(-a.x, b.y, fma(-a.y, b.x, c.y)));
}
__device__ __forceinline__ double norm2_acc(cplx v, double s) { return fma(v.x, v.x, fma(v.y, v.y, s)); }

// Sum of part[0..np) in a fixed order, identical in every block; the result is valid in all threads.
__device__ __forceinline__ cplx block_reduce_parts(const cplx* part, int np, cplx* sh) {
    cplx s = mk(0.0, 0.0);
    for (int i = threadIdx.x; i < np; i += RT) s += part[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = RT / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    const cplx r = sh[0];
    __syncthreads();
    return r;
}

// Block partial of a per-thread value, written to out[blockIdx.x].
__device__ __forceinline__ void block_store_partial(cplx v, cplx* sh, cplx* out) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = RT / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

// Δg = g - gold ; Δf = fx - fxold (in place in fxold) ; partial of <Qb, Δf> (or |Δf|² when Qb is null).
__global__ void __launch_bounds__(RT) k_aa_diff(cplx* dg, const cplx* g, const cplx* gold, cplx* df, const cplx* fx,
                                                const cplx* Qb, cplx* part_out, size_t n) {
    __shared__ cplx sh[RT];
    cplx s = mk(0.0, 0.0);
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) {
        dg[i] = g[i] - gold[i];
        const cplx v = fx[i] - df[i];
        df[i] = v;
        if (Qb) s = cfma_conj(Qb[i], v, s);
        else s.x = norm2_acc(v, s.x);
    }
    block_store_partial(s, sh, part_out);
}

// One modified Gram-Schmidt step: r = Σ part_in (= <Qa, Δf>), R entry = r, Δf -= r Qa; then the
// partial of the next projection <Qb, Δf> (or |Δf|² when Qb is null).
__global__ void __launch_bounds__(RT) k_aa_mgs(cplx* df, const cplx* Qa, const cplx* part_in, int np, cplx* Rentry,
                                               const cplx* Qb, cplx* part_out, size_t n) {
    __shared__ cplx sh[RT];
    const cplx r = block_reduce_parts(part_in, np, sh);
    if (blockIdx.x == 0 && threadIdx.x == 0) *Rentry = r;
    cplx s = mk(0.0, 0.0);
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) {
        const cplx v = cfnma(r, Qa[i], df[i]);
        df[i] = v;
        if (Qb) s = cfma_conj(Qb[i], v, s);
        else s.x = norm2_acc(v, s.x);
    }
    block_store_partial(s, sh, part_out);
}

// ‖Δf‖ = sqrt(Σ part_in), R(k,k) = ‖Δf‖, Q_k = Δf / ‖Δf‖.
__global__ void __launch_bounds__(RT) k_aa_qnew(cplx* Qk, const cplx* df, const cplx* part_in, int np, cplx* Rkk,
                                                size_t n) {
    __shared__ cplx sh[RT];
    const double nr = sqrt(fmax(0.0, block_reduce_parts(part_in, np, sh).x));
    if (blockIdx.x == 0 && threadIdx.x == 0) *Rkk = mk(nr, 0.0);
    const double inv = 1.0 / nr;  // one division per block, not two per element
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) {
        const cplx v = df[i];
        Qk[i] = mk(v.x * inv, v.y * inv);
    }
}

// Partials of <Q_i, fx> for the AA_CHUNK vectors of chunk blockIdx.y: part[(i) * np + blockIdx.x].
constexpr int AA_CHUNK = 8;
__global__ void __launch_bounds__(RT) k_aa_multidot(AAVecs Q, int nv, const cplx* fx, cplx* part, int np, size_t n) {
    __shared__ cplx sh[RT];
    const int i0 = blockIdx.y * AA_CHUNK;
    const int cnt = min(AA_CHUNK, nv - i0);
    cplx s[AA_CHUNK];
#pragma unroll
    for (int j = 0; j < AA_CHUNK; ++j) s[j] = mk(0.0, 0.0);
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) {
        const cplx f = fx[i];
#pragma unroll
        for (int j = 0; j < AA_CHUNK; ++j)
            if (j < cnt) s[j] = cfma_conj(Q.v[i0 + j][i], f, s[j]);
    }
    for (int j = 0; j < cnt; ++j) block_store_partial(s[j], sh, part + (size_t)(i0 + j) * np);
}

// γ = R⁻¹ (Σ_blocks part): one block; each column of partials is reduced exactly like the
// Gram-Schmidt coefficients, then thread 0 back-substitutes.  R is column-major m x m.
__global__ void __launch_bounds__(RT) k_aa_gamma(const cplx* part, int np, const cplx* R, int m, int meff, cplx* gam) {
    __shared__ cplx sh[RT];
    __shared__ cplx g[AA_MAX];
    for (int i = 0; i < meff; ++i) {
        const cplx s = block_reduce_parts(part + (size_t)i * np, np, sh);
        if (threadIdx.x == 0) g[i] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = meff - 1; i >= 0; --i) {
            cplx v = g[i];
            for (int j = i + 1; j < meff; ++j) v -= R[i + (size_t)m * j] * g[j];
            g[i] = cdiv(v, R[i + (size_t)m * i]);
        }
        for (int i = 0; i < meff; ++i) gam[i] = g[i];
    }
}

// x = g - Σ_i γ_i Δg_i (i in order) ; fxold = fx ; gold = g.
__global__ void __launch_bounds__(RT) k_aa_update(cplx* x, const cplx* g, AAVecs dG, const cplx* gam, int meff,
                                                  const cplx* fx, cplx* fxold, cplx* gold, size_t n) {
    __shared__ cplx gs[AA_MAX];
    for (int i = threadIdx.x; i < meff; i += RT) gs[i] = gam[i];
    __syncthreads();
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) {
        const cplx gi = g[i];
        cplx v = gi;
        for (int j = 0; j < meff; ++j) v = cfnma(gs[j], dG.v[j][i], v);
        x[i] = v;
        fxold[i] = fx[i];
        gold[i] = gi;
    }
}

// Deletion of the first column of the m x m QR factor by Givens rotations (NLsolve qrdelete!):
// rotation i = 1..m-1 acts on rows (i-1, i) of R; the parameters go to rot[i-1] = (c, s, -);
// then the columns shift left by one.  One thread: m² work on a handful of numbers.
__device__ __forceinline__ double cabs_(cplx a) { return hypot(a.x, a.y); }
__global__ void k_aa_givens(cplx* R, int m, cplx* rot) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    auto Rr = [&](int i, int j) -> cplx& { return R[i + (size_t)m * j]; };
    for (int i = 1; i < m; ++i) {
        const cplx f = Rr(i - 1, i), g = Rr(i, i);
        const double af = cabs_(f), ag = cabs_(g);
        double c;
        cplx sn;
        if (ag == 0.0) { c = 1.0; sn = mk(0.0, 0.0); }
        else if (af == 0.0) { c = 0.0; sn = mk(g.x / ag, -g.y / ag); }
        else {
            const double rr = hypot(af, ag);
            c = af / rr;
            const cplx fa = mk(f.x / af, f.y / af);
            sn = fa * conjg(g);
            sn = mk(sn.x / rr, sn.y / rr);
        }
        for (int j = 0; j < m; ++j) {
            const cplx a = Rr(i - 1, j), b = Rr(i, j);
            Rr(i - 1, j) = a * c + sn * b;
            Rr(i, j) = (-conjg(sn)) * a + b * c;
        }
        rot[2 * (i - 1)] = mk(c, 0.0);
        rot[2 * (i - 1) + 1] = sn;
    }
    for (int j = 0; j < m - 1; ++j)
        for (int i = 0; i < m - 1; ++i) Rr(i, j) = Rr(i, j + 1);
}

// The m-1 rotations applied to the columns of Q, in order, at each element.
__global__ void __launch_bounds__(RT) k_aa_qrot(AAVecsW Q, int m, const cplx* rot, size_t n) {
    __shared__ cplx rs[2 * AA_MAX];
    for (int i = threadIdx.x; i < 2 * (m - 1); i += RT) rs[i] = rot[i];
    __syncthreads();
    for (size_t t = blockIdx.x * (size_t)RT + threadIdx.x; t < n; t += (size_t)gridDim.x * RT) {
        cplx a = Q.v[0][t];
        for (int i = 1; i < m; ++i) {
            const double c = rs[2 * (i - 1)].x;
            const cplx sn = rs[2 * (i - 1) + 1];
            const cplx b = Q.v[i][t];
            // Q_{i-1} = c a + conj(s) b ; a = -s a + c b
            Q.v[i - 1][t] = mk(fma(a.x, c, fma(sn.x, b.x, sn.y * b.y)), fma(a.y, c, fma(sn.x, b.y, -sn.y * b.x)));
            a = mk(fma(b.x, c, fma(-sn.x, a.x, sn.y * a.y)), fma(b.y, c, fma(-sn.x, a.y, -sn.y * a.x)));
        }
        Q.v[m - 1][t] = a;
    }
}

}  // namespace

#define AA_CHECK()                                   \
    do {                                             \
        cudaError_t e__ = cudaGetLastError();        \
        if (e__ != cudaSuccess) return e__;          \
    } while (0)

cudaError_t launch_aa_diff(cudaStream_t s, int nblk, cplx* dg, const cplx* g, const cplx* gold, cplx* df,
                           const cplx* fx, const cplx* Qb, cplx* part_out, size_t n) {
    k_aa_diff<<<nblk, RT, 0, s>>>(dg, g, gold, df, fx, Qb, part_out, n);
    AA_CHECK(); return cudaSuccess;
}
cudaError_t launch_aa_mgs(cudaStream_t s, int nblk, cplx* df, const cplx* Qa, const cplx* part_in, cplx* Rentry,
                          const cplx* Qb, cplx* part_out, size_t n) {
    k_aa_mgs<<<nblk, RT, 0, s>>>(df, Qa, part_in, nblk, Rentry, Qb, part_out, n);
    AA_CHECK(); return cudaSuccess;
}
cudaError_t launch_aa_qnew(cudaStream_t s, int nblk, cplx* Qk, const cplx* df, const cplx* part_in, cplx* Rkk,
                           size_t n) {
    k_aa_qnew<<<nblk, RT, 0, s>>>(Qk, df, part_in, nblk, Rkk, n);
    AA_CHECK(); return cudaSuccess;
}
cudaError_t launch_aa_gamma(cudaStream_t s, int nblk, const AAVecs& Q, int meff, const cplx* fx, cplx* part,
                            const cplx* R, int m, cplx* gam, size_t n) {
    if (meff < 1 || meff > AA_MAX) return cudaErrorInvalidValue;
    k_aa_multidot<<<dim3(nblk, (meff + AA_CHUNK - 1) / AA_CHUNK), RT, 0, s>>>(Q, meff, fx, part, nblk, n);
    AA_CHECK();
    k_aa_gamma<<<1, RT, 0, s>>>(part, nblk, R, m, meff, gam);
    AA_CHECK(); return cudaSuccess;
}
cudaError_t launch_aa_update(cudaStream_t s, int nblk, cplx* x, const cplx* g, const AAVecs& dG, const cplx* gam,
                             int meff, const cplx* fx, cplx* fxold, cplx* gold, size_t n) {
    if (meff > AA_MAX) return cudaErrorInvalidValue;
    k_aa_update<<<nblk, RT, 0, s>>>(x, g, dG, gam, meff, fx, fxold, gold, n);
    AA_CHECK(); return cudaSuccess;
}
cudaError_t launch_aa_givens(cudaStream_t s, cplx* R, int m, cplx* rot) {
    if (m < 2 || m > AA_MAX) return cudaErrorInvalidValue;
    k_aa_givens<<<1, 32, 0, s>>>(R, m, rot);
    AA_CHECK(); return cudaSuccess;
}
cudaError_t launch_aa_gamma_solve(cudaStream_t s, const cplx* part, int np, const cplx* R, int m, int meff, cplx* gam) {
    if (meff < 1 || meff > AA_MAX) return cudaErrorInvalidValue;
    k_aa_gamma<<<1, RT, 0, s>>>(part, np, R, m, meff, gam);
    AA_CHECK(); return cudaSuccess;
}
cudaError_t launch_aa_delete(cudaStream_t s, int nblk, cplx* R, int m, cplx* rot, const AAVecsW& Q, size_t n) {
    if (m < 2 || m > AA_MAX) return cudaErrorInvalidValue;
    k_aa_givens<<<1, 32, 0, s>>>(R, m, rot);
    AA_CHECK();
    k_aa_qrot<<<nblk, RT, 0, s>>>(Q, m, rot, n);
    AA_CHECK(); return cudaSuccess;
}

}  // namespace fdga
