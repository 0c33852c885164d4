// fdga_krylov.cu -- GMRES building blocks for the Newton–Krylov solve of the parquet fixed point
// and for the linear response dx*/dU.
//
// The map Φ is real-linear but not complex-linear in the state (the symmetry operations
// conjugate), so the Jacobian acts on the state as a real vector of 2n components and GMRES runs
// in real arithmetic: inner products are Re<a, b> = Σ (a.x b.x + a.y b.y).  The Krylov basis is
// stored in FP32 (cplxf pairs); products accumulate in FP32 over runs of 64 terms and then in
// FP64; reductions, the Hessenberg matrix and the iterate are FP64.  Jacobian-vector products are
// forward differences of the map, (Φ(x + εv) − Φ(x)) / ε, evaluated by the same
// graph-captured iteration as the plain solver.
#include "fdga_kernels.h"

#include <algorithm>

namespace fdga {

namespace {

constexpr int RT = 256;
constexpr int FLUSH = 64;
constexpr int CHUNK = 8;

__device__ __forceinline__ cplxf tof(cplx v) { return to_f32(v); }

struct RAcc {  // real accumulator: FP32 runs flushed into FP64
    float s32 = 0.f;
    double s64 = 0.0;
    int k = 0;
    __device__ __forceinline__ void add(float v) {
        s32 += v;
        if (++k == FLUSH) { s64 += (double)s32; s32 = 0.f; k = 0; }
    }
    __device__ __forceinline__ double total() const { return s64 + (double)s32; }
};

__device__ __forceinline__ void store_partial(double v, double* sh, double* out) {
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = RT / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
    __syncthreads();
}
__device__ __forceinline__ float rdot(cplxf a, cplxf b) { return a.x * b.x + a.y * b.y; }

// xp = x + ε v
__global__ void __launch_bounds__(RT) k_kr_point(const cplx* x, const cplxf* v, double eps, cplx* xp, size_t n) {
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT)
        xp[i] = x[i] + to_d(v[i]) * eps;
}

// w = a·v + b·(y − y0)   (A v = v − J v: a = 1, b = −1/ε; the right-hand side ∂Φ: a = 0, b = 1/(2h))
__global__ void __launch_bounds__(RT) k_kr_apply(const cplx* y, const cplx* y0, const cplxf* v, double a, double b,
                                                 cplxf* w, size_t n) {
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) {
        cplx d = (y[i] - y0[i]) * b;
        if (v) d += to_d(v[i]) * a;
        w[i] = tof(d);
    }
}

// partials of Re<V_i, w> for the CHUNK vectors of chunk blockIdx.y: part[i * np + block]; when
// norm_slot >= 0 the chunk-0 blocks also write the partial of |w|² to part[norm_slot * np + block]
__global__ void __launch_bounds__(RT) k_kr_dots(KrVecs V, int nv, const cplxf* w, const float* wgt, double* part,
                                                int np, int norm_slot, size_t n) {
    __shared__ double sh[RT];
    const int i0 = blockIdx.y * CHUNK;
    const int cnt = max(0, min(CHUNK, nv - i0));
    const bool with_norm = norm_slot >= 0 && blockIdx.y == 0;
    RAcc a[CHUNK], an;
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) {
        cplxf wi = w[i];
        const cplxf wraw = wi;
        if (wgt) wi = wi * wgt[i];  // class-size weight of a compact (representative) entry
#pragma unroll
        for (int j = 0; j < CHUNK; ++j)
            if (j < cnt) a[j].add(rdot(V.v[i0 + j][i], wi));
        if (with_norm) an.add(rdot(wraw, wi));
    }
    for (int j = 0; j < cnt; ++j) store_partial(a[j].total(), sh, part + (size_t)(i0 + j) * np);
    if (with_norm) store_partial(an.total(), sh, part + (size_t)norm_slot * np);
}

// coef[i] = Σ_blocks part[i], i < ncoef (one block; a warp per coefficient, lanes over the
// partials in a fixed order, then a fixed shuffle tree: no block barriers)
__global__ void __launch_bounds__(RT) k_kr_reduce(const double* part, int np, int ncoef, double* coef) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = warp; i < ncoef; i += RT / 32) {
        double s = 0.0;
        for (int b = lane; b < np; b += 32) s += part[(size_t)i * np + b];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) coef[i] = s;
    }
}

// w -= Σ_{i<nv} c_i V_i (FP32)
__global__ void __launch_bounds__(RT) k_kr_sub(KrVecs V, int nv, const double* c, cplxf* w, size_t n) {
    __shared__ float cs[KR_MAX];
    for (int i = threadIdx.x; i < nv; i += RT) cs[i] = (float)c[i];
    __syncthreads();
    for (size_t t = blockIdx.x * (size_t)RT + threadIdx.x; t < n; t += (size_t)gridDim.x * RT) {
        cplxf s = w[t];
        for (int i = 0; i < nv; ++i) {
            const cplxf v = V.v[i][t];
            s.x -= cs[i] * v.x;
            s.y -= cs[i] * v.y;
        }
        w[t] = s;
    }
}

// out = w / nrm
__global__ void __launch_bounds__(RT) k_kr_scale(const cplxf* w, double nrm, cplxf* out, size_t n) {
    const float inv = (float)(1.0 / nrm);
    for (size_t t = blockIdx.x * (size_t)RT + threadIdx.x; t < n; t += (size_t)gridDim.x * RT) out[t] = w[t] * inv;
}

// x += Σ_{i<nv} y_i V_i (sum in FP32, added in FP64)
__global__ void __launch_bounds__(RT) k_kr_update(cplx* x, KrVecs V, int nv, const double* y, double scale, size_t n) {
    __shared__ float ys[KR_MAX];
    for (int i = threadIdx.x; i < nv; i += RT) ys[i] = (float)y[i];
    __syncthreads();
    for (size_t t = blockIdx.x * (size_t)RT + threadIdx.x; t < n; t += (size_t)gridDim.x * RT) {
        cplxf s{0.f, 0.f};
        for (int i = 0; i < nv; ++i) {
            const cplxf v = V.v[i][t];
            s.x += ys[i] * v.x;
            s.y += ys[i] * v.y;
        }
        x[t] = x[t] + to_d(s) * scale;
    }
}

// out = a (FP64 -> FP32 copy), partial of the (weighted) |a|²
__global__ void __launch_bounds__(RT) k_kr_load(const cplx* a, const float* wgt, cplxf* out, double* part, size_t n) {
    __shared__ double sh[RT];
    double s = 0.0;
    for (size_t t = blockIdx.x * (size_t)RT + threadIdx.x; t < n; t += (size_t)gridDim.x * RT) {
        const cplx v = a[t];
        out[t] = tof(v);
        s += (v.x * v.x + v.y * v.y) * (wgt ? (double)wgt[t] : 1.0);
    }
    store_partial(s, sh, part);
}

// Symmetric-subspace (representative) storage.  Every iterate, residual and Jacobian-vector
// product of the map is invariant under the solver's symmetry groups (the map expands its class
// representatives), so Krylov vectors are kept as one value per class: code[j] = compact index * 4
// + operation of full element j, pos[i] = full index of compact entry i.

// xp[j] = x[j] + ε op_j(v[code_j])   (v compact FP32)
__global__ void __launch_bounds__(RT) k_kc_point(const cplx* x, const cplxf* v, const uint32_t* code, double eps,
                                                 cplx* xp, size_t n) {
    for (size_t j = blockIdx.x * (size_t)RT + threadIdx.x; j < n; j += (size_t)gridDim.x * RT) {
        const uint32_t c = code[j];
        const cplx e = apply_op((int)(c & 3u), to_d(v[c >> 2])) * eps;
        xp[j] = x ? x[j] + e : e;
    }
}
// out[j] = x[j] + λ op_j(d[code_j])   (d compact FP64)
__global__ void __launch_bounds__(RT) k_kc_axpy(const cplx* x, const cplx* d, const uint32_t* code, double lam,
                                                cplx* out, size_t n) {
    for (size_t j = blockIdx.x * (size_t)RT + threadIdx.x; j < n; j += (size_t)gridDim.x * RT) {
        const uint32_t c = code[j];
        out[j] = x[j] + apply_op((int)(c & 3u), d[c >> 2]) * lam;
    }
}
// w[i] = a·v[i] + b·(y[pos_i] − y0[i])   (y full FP64, y0 compact FP64 or null, w compact FP32)
__global__ void __launch_bounds__(RT) k_kc_apply(const cplx* y, const cplx* y0, const uint32_t* pos, const cplxf* v,
                                                 double a, double b, cplxf* w, size_t nc) {
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < nc; i += (size_t)gridDim.x * RT) {
        cplx d = y[pos[i]];
        if (y0) d -= y0[i];
        d = d * b;
        if (v) d += to_d(v[i]) * a;
        w[i] = tof(d);
    }
}
// out[i] = (y[pos_i] − x[pos_i]) · s  (x may be null)   compact FP64 gather of a full difference
__global__ void __launch_bounds__(RT) k_kc_gather(const cplx* y, const cplx* x, const uint32_t* pos, double s,
                                                  cplx* out, size_t nc) {
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < nc; i += (size_t)gridDim.x * RT) {
        cplx d = y[pos[i]];
        if (x) d -= x[pos[i]];
        out[i] = d * s;
    }
}
// class sizes: w[code_j >> 2] += 1
__global__ void __launch_bounds__(RT) k_kc_count(const uint32_t* code, float* w, size_t n) {
    for (size_t j = blockIdx.x * (size_t)RT + threadIdx.x; j < n; j += (size_t)gridDim.x * RT)
        atomicAdd(&w[code[j] >> 2], 1.0f);
}
// compact codes of one state block from its group map (rep*4 + op; nullptr = identity) and its
// sorted representative list: code = (off + lower_bound(items, rep)) * 4 + op
__global__ void __launch_bounds__(RT) k_kc_codes(const uint32_t* map, const int* items, int nitems, size_t nblock,
                                                 size_t base, uint32_t off, uint32_t* code, uint32_t* pos) {
    for (size_t j = blockIdx.x * (size_t)RT + threadIdx.x; j < nblock; j += (size_t)gridDim.x * RT) {
        uint32_t rep = (uint32_t)j, op = 0;
        if (map) { rep = map[j] >> 2; op = map[j] & 3u; }
        uint32_t ci = rep;
        if (items) {
            int lo = 0, hi = nitems;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if ((uint32_t)items[mid] < rep) lo = mid + 1; else hi = mid;
            }
            ci = (uint32_t)lo;
        }
        code[base + j] = ((off + ci) << 2) | op;
        if (rep == (uint32_t)j) pos[off + ci] = (uint32_t)(base + j);
    }
}

// r = b + α v + β (y − yb)   (FP64; v FP32 or null)
__global__ void __launch_bounds__(RT) k_kr_resid(const cplx* b, const cplxf* v, double alpha, const cplx* y,
                                                 const cplx* yb, double beta, cplx* r, size_t n) {
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) {
        cplx t = b ? b[i] : mk(0.0, 0.0);
        if (v) t += to_d(v[i]) * alpha;
        if (y) t += (y[i] - yb[i]) * beta;
        r[i] = t;
    }
}
// out = a + λ b (FP64)
__global__ void __launch_bounds__(RT) k_kr_axpby(cplx* out, const cplx* a, double lam, const cplx* b, size_t n) {
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) out[i] = a[i] + b[i] * lam;
}

// ---------------------------------------------------------------------------------------------
// Device-resident Arnoldi column (the body of the WHILE node of a GMRES cycle).  j is read from
// the cycle state by every kernel; the basis pointers are the fixed V[0..m].
// ---------------------------------------------------------------------------------------------
__global__ void k_kr_init(KrDevState* st, int m, int budget, int cost, double thr, double beta) {
    if (threadIdx.x != 0) return;
    st->j = 0; st->k = 0; st->done = 0; st->nmaps = 0;
    st->budget = budget; st->cost = cost; st->m = m;
    st->thr = thr; st->est = beta; st->hn = 0.0;
    for (int i = 0; i <= KR_MAX; ++i) st->g[i] = 0.0;
    st->g[0] = beta;
}
__global__ void __launch_bounds__(RT) k_kc_point_j(const cplx* x, KrVecs V, const KrDevState* st,
                                                   const uint32_t* code, double eps, cplx* xp, size_t n) {
    const cplxf* v = V.v[st->j];
    for (size_t j = blockIdx.x * (size_t)RT + threadIdx.x; j < n; j += (size_t)gridDim.x * RT) {
        const uint32_t c = code[j];
        const cplx e = apply_op((int)(c & 3u), to_d(v[c >> 2])) * eps;
        xp[j] = x ? x[j] + e : e;
    }
}
__global__ void __launch_bounds__(RT) k_kc_apply_j(const cplx* y, const uint32_t* pos, KrVecs V, const KrDevState* st,
                                                   double a, double b, cplxf* w, size_t nc) {
    const cplxf* v = V.v[st->j];
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < nc; i += (size_t)gridDim.x * RT)
        w[i] = tof(y[pos[i]] * b + to_d(v[i]) * a);
}
// partials of Re<V_i, w>, i <= j, for the chunk of blockIdx.y (blocks past j only add the norm)
__global__ void __launch_bounds__(RT) k_kr_dots_j(KrVecs V, const KrDevState* st, const cplxf* w, const float* wgt,
                                                  double* part, int np, int norm_slot, size_t n) {
    __shared__ double sh[RT];
    const int nv = st->j + 1;
    const int i0 = blockIdx.y * CHUNK;
    const int cnt = max(0, min(CHUNK, nv - i0));
    const bool with_norm = norm_slot >= 0 && blockIdx.y == 0;
    if (cnt == 0 && !with_norm) return;
    RAcc a[CHUNK], an;
    for (size_t i = blockIdx.x * (size_t)RT + threadIdx.x; i < n; i += (size_t)gridDim.x * RT) {
        cplxf wi = w[i];
        const cplxf wraw = wi;
        if (wgt) wi = wi * wgt[i];
#pragma unroll
        for (int j = 0; j < CHUNK; ++j)
            if (j < cnt) a[j].add(rdot(V.v[i0 + j][i], wi));
        if (with_norm) an.add(rdot(wraw, wi));
    }
    for (int j = 0; j < cnt; ++j) store_partial(a[j].total(), sh, part + (size_t)(i0 + j) * np);
    if (with_norm) store_partial(an.total(), sh, part + (size_t)norm_slot * np);
}
// coef[i] = Σ part[i], i <= j; and coef[KR_MAX + 1] = Σ part[norm_slot] when norm_slot >= 0
__global__ void __launch_bounds__(RT) k_kr_reduce_j(const double* part, int np, const KrDevState* st, int norm_slot,
                                                    double* coef) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nrow = st->j + 1 + (norm_slot >= 0 ? 1 : 0);
    for (int r = warp; r < nrow; r += RT / 32) {
        const int i = r <= st->j ? r : norm_slot;
        double s = 0.0;
        for (int b = lane; b < np; b += 32) s += part[(size_t)i * np + b];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) coef[r <= st->j ? r : KR_MAX + 1] = s;
    }
}
// w -= Σ_{i<=j} c_i V_i; with hn (second pass): V[j+1] = w / H(j+1, j)
__global__ void __launch_bounds__(RT) k_kr_sub_j(KrVecs V, const KrDevState* st, const double* c, cplxf* w,
                                                 int scale_out, size_t n) {
    __shared__ float cs[KR_MAX];
    const int nv = st->j + 1;
    for (int i = threadIdx.x; i < nv; i += RT) cs[i] = (float)c[i];
    __syncthreads();
    const double hn = st->hn;
    cplxf* out = scale_out ? const_cast<cplxf*>(V.v[nv]) : w;
    const float inv = (scale_out && hn > 0.0) ? (float)(1.0 / hn) : 1.0f;
    for (size_t t = blockIdx.x * (size_t)RT + threadIdx.x; t < n; t += (size_t)gridDim.x * RT) {
        cplxf s = w[t];
        for (int i = 0; i < nv; ++i) {
            const cplxf v = V.v[i][t];
            s.x -= cs[i] * v.x;
            s.y -= cs[i] * v.y;
        }
        out[t] = s * inv;
    }
}
// Hessenberg column j from the two passes (h_ij = c1_i + c2_i; H(j+1, j)² = |w1|² - Σ c2_i², the
// norm after the second pass for the orthonormal basis), the previous rotations, the new one, and
// the residual estimate |g_{j+1}|.  One thread.
__global__ void k_kr_givens(KrDevState* st, const double* c1, const double* c2) {
    if (threadIdx.x != 0) return;
    const int j = st->j;
    constexpr int LD = KR_MAX + 1;
    double* Hj = st->H + (size_t)LD * j;
    double q = 0.0;
    for (int i = 0; i <= j; ++i) {
        Hj[i] = c1[i] + c2[i];
        q += c2[i] * c2[i];
    }
    const double hn = sqrt(fmax(0.0, c2[KR_MAX + 1] - q));
    Hj[j + 1] = hn;
    st->hn = hn;
    for (int i = 0; i < j; ++i) {
        const double a = Hj[i], b = Hj[i + 1];
        Hj[i] = st->cs[i] * a + st->sn[i] * b;
        Hj[i + 1] = -st->sn[i] * a + st->cs[i] * b;
    }
    const double a = Hj[j], b = Hj[j + 1], rho = hypot(a, b);
    st->cs[j] = rho > 0 ? a / rho : 1.0;
    st->sn[j] = rho > 0 ? b / rho : 0.0;
    Hj[j] = rho;
    Hj[j + 1] = 0.0;
    st->g[j + 1] = -st->sn[j] * st->g[j];
    st->g[j] = st->cs[j] * st->g[j];
    st->est = fabs(st->g[j + 1]);
    st->done = (!(st->est > st->thr) || !(hn > 0.0)) ? 1 : 0;  // (a NaN estimate or norm stops the cycle)
}
// column j complete: advance, and continue the WHILE node while not done, j < m and the budget
// allows one more application (j grows by one per pass, so the loop ends after at most m passes)
__global__ void k_kr_advance(KrDevState* st, cudaGraphConditionalHandle cond) {
    if (threadIdx.x != 0) return;
    st->nmaps += st->cost;
    st->k = st->j + 1;
    st->j = st->j + 1;
    const bool more = !st->done && st->j < st->m && st->nmaps + st->cost <= st->budget;
    cudaGraphSetConditional(cond, more ? 1u : 0u);
}

}  // namespace

#define KR_CHECK()                                   \
    do {                                             \
        cudaError_t e__ = cudaGetLastError();        \
        if (e__ != cudaSuccess) return e__;          \
    } while (0)

cudaError_t launch_kr_point(cudaStream_t s, int nblk, const cplx* x, const cplxf* v, double eps, cplx* xp, size_t n) {
    k_kr_point<<<nblk, RT, 0, s>>>(x, v, eps, xp, n);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kr_apply(cudaStream_t s, int nblk, const cplx* y, const cplx* y0, const cplxf* v, double a,
                            double b, cplxf* w, size_t n) {
    k_kr_apply<<<nblk, RT, 0, s>>>(y, y0, v, a, b, w, n);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kr_dots(cudaStream_t s, int nblk, const KrVecs& V, int nv, const cplxf* w, const float* wgt,
                           double* part, int norm_slot, size_t n) {
    if (nv > KR_MAX) return cudaErrorInvalidValue;
    const int chunks = std::max(1, (nv + CHUNK - 1) / CHUNK);
    k_kr_dots<<<dim3(nblk, chunks), RT, 0, s>>>(V, nv, w, wgt, part, nblk, norm_slot, n);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kr_reduce(cudaStream_t s, const double* part, int np, int ncoef, double* coef) {
    k_kr_reduce<<<1, RT, 0, s>>>(part, np, ncoef, coef);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kr_sub(cudaStream_t s, int nblk, const KrVecs& V, int nv, const double* c, cplxf* w, size_t n) {
    if (nv > KR_MAX) return cudaErrorInvalidValue;
    k_kr_sub<<<nblk, RT, 0, s>>>(V, nv, c, w, n);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kr_scale(cudaStream_t s, int nblk, const cplxf* w, double nrm, cplxf* out, size_t n) {
    k_kr_scale<<<nblk, RT, 0, s>>>(w, nrm, out, n);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kr_update(cudaStream_t s, int nblk, cplx* x, const KrVecs& V, int nv, const double* y, double scale,
                             size_t n) {
    if (nv > KR_MAX) return cudaErrorInvalidValue;
    k_kr_update<<<nblk, RT, 0, s>>>(x, V, nv, y, scale, n);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kr_load(cudaStream_t s, int nblk, const cplx* a, const float* wgt, cplxf* out, double* part,
                           size_t n) {
    k_kr_load<<<nblk, RT, 0, s>>>(a, wgt, out, part, n);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kc_point(cudaStream_t s, int nblk, const cplx* x, const cplxf* v, const uint32_t* code, double eps,
                            cplx* xp, size_t n) {
    k_kc_point<<<nblk, RT, 0, s>>>(x, v, code, eps, xp, n);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kc_axpy(cudaStream_t s, int nblk, const cplx* x, const cplx* d, const uint32_t* code, double lam,
                           cplx* out, size_t n) {
    k_kc_axpy<<<nblk, RT, 0, s>>>(x, d, code, lam, out, n);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kc_apply(cudaStream_t s, int nblk, const cplx* y, const cplx* y0, const uint32_t* pos,
                            const cplxf* v, double a, double b, cplxf* w, size_t nc) {
    k_kc_apply<<<nblk, RT, 0, s>>>(y, y0, pos, v, a, b, w, nc);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kc_gather(cudaStream_t s, int nblk, const cplx* y, const cplx* x, const uint32_t* pos, double sc,
                             cplx* out, size_t nc) {
    k_kc_gather<<<nblk, RT, 0, s>>>(y, x, pos, sc, out, nc);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kc_count(cudaStream_t s, int nblk, const uint32_t* code, float* w, size_t n) {
    k_kc_count<<<nblk, RT, 0, s>>>(code, w, n);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kc_codes(cudaStream_t s, const uint32_t* map, const int* items, int nitems, size_t nblock,
                            size_t base, uint32_t off, uint32_t* code, uint32_t* pos) {
    const unsigned g = (unsigned)std::min<size_t>((nblock + RT - 1) / RT, 65535u * 16u);
    k_kc_codes<<<g, RT, 0, s>>>(map, items, nitems, nblock, base, off, code, pos);
    KR_CHECK(); return cudaSuccess;
}

}  // namespace fdga

namespace fdga {
cudaError_t launch_kr_resid(cudaStream_t s, int nblk, const cplx* b, const cplxf* v, double alpha, const cplx* y,
                            const cplx* yb, double beta, cplx* r, size_t n) {
    k_kr_resid<<<nblk, RT, 0, s>>>(b, v, alpha, y, yb, beta, r, n);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kr_init(cudaStream_t s, KrDevState* st, int m, int budget, int cost, double thr, double beta) {
    if (m < 1 || m >= KR_MAX) return cudaErrorInvalidValue;
    k_kr_init<<<1, 32, 0, s>>>(st, m, budget, cost, thr, beta);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kc_point_j(cudaStream_t s, int nblk, const cplx* x, const KrVecs& V, const KrDevState* st,
                              const uint32_t* code, double eps, cplx* xp, size_t n) {
    k_kc_point_j<<<nblk, RT, 0, s>>>(x, V, st, code, eps, xp, n);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kc_apply_j(cudaStream_t s, int nblk, const cplx* y, const uint32_t* pos, const KrVecs& V,
                              const KrDevState* st, double a, double b, cplxf* w, size_t nc) {
    k_kc_apply_j<<<nblk, RT, 0, s>>>(y, pos, V, st, a, b, w, nc);
    KR_CHECK(); return cudaSuccess;
}
// both classical Gram-Schmidt passes of column j and its Hessenberg update (fixed grids: the
// launches are captured once and replayed for every j <= m - 1 of the cycle)
cudaError_t launch_kr_cgs_j(cudaStream_t s, int nblk, const KrVecs& V, KrDevState* st, cplxf* w, const float* wgt,
                            double* part, double* c1, double* c2, size_t n) {
    const int chunks = (KR_MAX + CHUNK - 1) / CHUNK;
    k_kr_dots_j<<<dim3(nblk, chunks), RT, 0, s>>>(V, st, w, wgt, part, nblk, -1, n);
    k_kr_reduce_j<<<1, RT, 0, s>>>(part, nblk, st, -1, c1);
    k_kr_sub_j<<<nblk, RT, 0, s>>>(V, st, c1, w, 0, n);
    k_kr_dots_j<<<dim3(nblk, chunks), RT, 0, s>>>(V, st, w, wgt, part, nblk, KR_MAX + 1, n);
    k_kr_reduce_j<<<1, RT, 0, s>>>(part, nblk, st, KR_MAX + 1, c2);
    k_kr_givens<<<1, 32, 0, s>>>(st, c1, c2);
    k_kr_sub_j<<<nblk, RT, 0, s>>>(V, st, c2, w, 1, n);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kr_advance(cudaStream_t s, KrDevState* st, cudaGraphConditionalHandle cond) {
    k_kr_advance<<<1, 32, 0, s>>>(st, cond);
    KR_CHECK(); return cudaSuccess;
}
cudaError_t launch_kr_axpby(cudaStream_t s, int nblk, cplx* out, const cplx* a, double lam, const cplx* b, size_t n) {
    k_kr_axpby<<<nblk, RT, 0, s>>>(out, a, lam, b, n);
    KR_CHECK(); return cudaSuccess;
}
}  // namespace fdga
