// fdga_anderson32.cu -- Anderson acceleration with an FP32 history, for the inner solves of the
// mixed-precision solver.
//
// Same algorithm as fdga_anderson.cu (NLsolve method=:anderson: modified Gram-Schmidt QR of the
// residual differences, Givens deletion of the oldest column, γ = R⁻¹ Qᴴ f), with the long
// vectors of the history -- f, Δf, the columns of Q and Δg -- stored and combined in FP32.  The
// iterate x, g = x + βf and g_old stay FP64 and the residual f = Φ(x) + c - x is formed in FP64,
// so the history only has to steer the step: its rounding changes the path of the inner
// iteration, never the equation it solves.  Dot products accumulate in FP32 over runs of 64
// elements and then in FP64; block partials, the QR factor R and γ are FP64 (shared with the
// FP64 solver's kernels).
#include "fdga_kernels.h"

namespace fdga {

namespace {

constexpr int RT = 256;
constexpr int FLUSH = 64;  // FP32 products summed per FP64 accumulation

__device__ __forceinline__ cplxf tof(cplx v) { return to_f32(v); }
__device__ __forceinline__ cplxf conjf_(cplxf a) { return cplxf{a.x, -a.y}; }

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
__device__ __forceinline__ void block_store_partial(cplx v, cplx* sh, cplx* out) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = RT / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

// FP32 accumulator flushed into FP64 every FLUSH terms
struct Acc {
    cplxf s32{0.f, 0.f};
    cplx s64{0.0, 0.0};
    int k = 0;
    __device__ __forceinline__ void add(cplxf v) {
        s32 += v;
        if (++k == FLUSH) { s64 += to_d(s32); s32 = cplxf{0.f, 0.f}; k = 0; }
    }
    __device__ __forceinline__ cplx total() const { return s64 + to_d(s32); }
};

// f = y (+ c) - x in FP64 ; f32 = f ; g = x + βf ; partial max|f|²
__global__ void __launch_bounds__(RT) k_ma_residual(const cplx* y, const cplx* c, const cplx* x, cplxf* f32, cplx* g,
                                                    double beta, double* pmax, size_t n) {
    __shared__ double red[RT];
    double mx = 0.0;
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) {
        cplx f = y[i] - x[i];
        if (c) f += c[i];
        f32[i] = tof(f);
        g[i] = x[i] + f * beta;
        mx = fmax(mx, f.x * f.x + f.y * f.y);
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int o = RT / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) pmax[blockIdx.x] = red[0];
}

// Δg = g - gold (FP64 difference, stored FP32) ; Δf = f - fold (FP32, in place) ; partial <Qb, Δf> or |Δf|²
__global__ void __launch_bounds__(RT) k_ma_diff(cplxf* dg, const cplx* g, const cplx* gold, cplxf* df, const cplxf* f,
                                                const cplxf* Qb, cplx* part_out, size_t n) {
    __shared__ cplx sh[RT];
    Acc a;
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) {
        dg[i] = tof(g[i] - gold[i]);
        const cplxf v = f[i] - df[i];
        df[i] = v;
        if (Qb) a.add(conjf_(Qb[i]) * v);
        else a.add(cplxf{v.x * v.x + v.y * v.y, 0.f});
    }
    block_store_partial(a.total(), sh, part_out);
}

// r = Σ part_in ; R entry = r ; Δf -= r Qa ; partial <Qb, Δf> or |Δf|²
__global__ void __launch_bounds__(RT) k_ma_mgs(cplxf* df, const cplxf* Qa, const cplx* part_in, int np, cplx* Rentry,
                                               const cplxf* Qb, cplx* part_out, size_t n) {
    __shared__ cplx sh[RT];
    const cplx r = block_reduce_parts(part_in, np, sh);
    if (blockIdx.x == 0 && threadIdx.x == 0) *Rentry = r;
    const cplxf rf = tof(r);
    Acc a;
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) {
        const cplxf v = df[i] - rf * Qa[i];
        df[i] = v;
        if (Qb) a.add(conjf_(Qb[i]) * v);
        else a.add(cplxf{v.x * v.x + v.y * v.y, 0.f});
    }
    block_store_partial(a.total(), sh, part_out);
}

// ‖Δf‖ = sqrt(Σ part_in) ; R(k,k) = ‖Δf‖ ; Q_k = Δf / ‖Δf‖
__global__ void __launch_bounds__(RT) k_ma_qnew(cplxf* Qk, const cplxf* df, const cplx* part_in, int np, cplx* Rkk,
                                                size_t n) {
    __shared__ cplx sh[RT];
    const double nr = sqrt(fmax(0.0, block_reduce_parts(part_in, np, sh).x));
    if (blockIdx.x == 0 && threadIdx.x == 0) *Rkk = mk(nr, 0.0);
    const float inv = (float)(1.0 / nr);
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) Qk[i] = df[i] * inv;
}

// partials of <Q_i, f> for the 8 vectors of chunk blockIdx.y
constexpr int CHUNK = 8;
__global__ void __launch_bounds__(RT) k_ma_multidot(AAVecs32 Q, int nv, const cplxf* f, cplx* part, int np, size_t n) {
    __shared__ cplx sh[RT];
    const int i0 = blockIdx.y * CHUNK;
    const int cnt = min(CHUNK, nv - i0);
    Acc a[CHUNK];
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) {
        const cplxf fi = f[i];
#pragma unroll
        for (int j = 0; j < CHUNK; ++j)
            if (j < cnt) a[j].add(conjf_(Q.v[i0 + j][i]) * fi);
    }
    for (int j = 0; j < cnt; ++j) block_store_partial(a[j].total(), sh, part + (size_t)(i0 + j) * np);
}

// x = g - Σ_i γ_i Δg_i (sum in FP32, subtraction in FP64) ; fold = f ; gold = g
__global__ void __launch_bounds__(RT) k_ma_update(cplx* x, const cplx* g, AAVecs32 dG, const cplx* gam, int meff,
                                                  const cplxf* f, cplxf* fold, cplx* gold, size_t n) {
    __shared__ cplxf gs[AA_MAX];
    for (int i = threadIdx.x; i < meff; i += RT) gs[i] = tof(gam[i]);
    __syncthreads();
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) {
        const cplx gi = g[i];
        cplxf s{0.f, 0.f};
        for (int j = 0; j < meff; ++j) s += gs[j] * dG.v[j][i];
        x[i] = gi - to_d(s);
        fold[i] = f[i];
        gold[i] = gi;
    }
}

// the m-1 Givens rotations (parameters from k_aa_givens, FP64) applied to the FP32 columns of Q
__global__ void __launch_bounds__(RT) k_ma_qrot(AAVecs32W Q, int m, const cplx* rot, size_t n) {
    __shared__ float rs[4 * AA_MAX];
    for (int i = threadIdx.x; i < m - 1; i += RT) {
        rs[4 * i] = (float)rot[2 * i].x;
        rs[4 * i + 1] = (float)rot[2 * i + 1].x;
        rs[4 * i + 2] = (float)rot[2 * i + 1].y;
    }
    __syncthreads();
    for (size_t t = blockIdx.x * (size_t)RT + threadIdx.x; t < n; t += (size_t)gridDim.x * RT) {
        cplxf a = Q.v[0][t];
        for (int i = 1; i < m; ++i) {
            const float c = rs[4 * (i - 1)];
            const cplxf sn{rs[4 * (i - 1) + 1], rs[4 * (i - 1) + 2]};
            const cplxf b = Q.v[i][t];
            Q.v[i - 1][t] = a * c + conjf_(sn) * b;
            a = cplxf{-sn.x, -sn.y} * a + b * c;
        }
        Q.v[m - 1][t] = a;
    }
}

}  // namespace

#define MA_CHECK()                                   \
    do {                                             \
        cudaError_t e__ = cudaGetLastError();        \
        if (e__ != cudaSuccess) return e__;          \
    } while (0)

cudaError_t launch_ma_residual(cudaStream_t s, int nblk, const cplx* y, const cplx* c, const cplx* x, cplxf* f32,
                               cplx* g, double beta, double* pmax, size_t n) {
    k_ma_residual<<<nblk, RT, 0, s>>>(y, c, x, f32, g, beta, pmax, n);
    MA_CHECK(); return cudaSuccess;
}
cudaError_t launch_ma_diff(cudaStream_t s, int nblk, cplxf* dg, const cplx* g, const cplx* gold, cplxf* df,
                           const cplxf* f, const cplxf* Qb, cplx* part_out, size_t n) {
    k_ma_diff<<<nblk, RT, 0, s>>>(dg, g, gold, df, f, Qb, part_out, n);
    MA_CHECK(); return cudaSuccess;
}
cudaError_t launch_ma_mgs(cudaStream_t s, int nblk, cplxf* df, const cplxf* Qa, const cplx* part_in, cplx* Rentry,
                          const cplxf* Qb, cplx* part_out, size_t n) {
    k_ma_mgs<<<nblk, RT, 0, s>>>(df, Qa, part_in, nblk, Rentry, Qb, part_out, n);
    MA_CHECK(); return cudaSuccess;
}
cudaError_t launch_ma_qnew(cudaStream_t s, int nblk, cplxf* Qk, const cplxf* df, const cplx* part_in, cplx* Rkk,
                           size_t n) {
    k_ma_qnew<<<nblk, RT, 0, s>>>(Qk, df, part_in, nblk, Rkk, n);
    MA_CHECK(); return cudaSuccess;
}
cudaError_t launch_ma_multidot(cudaStream_t s, int nblk, const AAVecs32& Q, int nv, const cplxf* f, cplx* part,
                               size_t n) {
    if (nv < 1 || nv > AA_MAX) return cudaErrorInvalidValue;
    k_ma_multidot<<<dim3(nblk, (nv + CHUNK - 1) / CHUNK), RT, 0, s>>>(Q, nv, f, part, nblk, n);
    MA_CHECK(); return cudaSuccess;
}
cudaError_t launch_ma_update(cudaStream_t s, int nblk, cplx* x, const cplx* g, const AAVecs32& dG, const cplx* gam,
                             int meff, const cplxf* f, cplxf* fold, cplx* gold, size_t n) {
    if (meff > AA_MAX) return cudaErrorInvalidValue;
    k_ma_update<<<nblk, RT, 0, s>>>(x, g, dG, gam, meff, f, fold, gold, n);
    MA_CHECK(); return cudaSuccess;
}
cudaError_t launch_ma_qrot(cudaStream_t s, int nblk, const AAVecs32W& Q, int m, const cplx* rot, size_t n) {
    if (m < 2 || m > AA_MAX) return cudaErrorInvalidValue;
    k_ma_qrot<<<nblk, RT, 0, s>>>(Q, m, rot, n);
    MA_CHECK(); return cudaSuccess;
}

}  // namespace fdga
