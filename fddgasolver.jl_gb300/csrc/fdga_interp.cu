// fdga_interp.cu -- Fourier interpolation of momentum-resolved arrays between lattice sizes
// (src/interpolate.jl:1-27 `_fourier_interpolate!`, :59-121 `interpolate_vertex!`, used by
// `interpolate_solver!` :147-191).
//
// For every frequency point of the target mesh that lies in the source mesh, the Li² momentum
// values y(k) are transformed to real space, y_R = fft(y)/Li² (sign -1), copied onto the Lo x Lo
// real-space grid for R in [-Li/2, Li/2]² with weight 1/2 per component |R_c| = Li/2 when Li is
// even (the two images of a boundary R share it), and transformed back unnormalised (sign +1).
// Frequency points outside the source mesh are zero; the self-energy takes the nearest source
// frequency (clamped at the mesh edges).  One CTA per target frequency point; the momentum index
// is outermost in every array, so a point's values are `rows` apart.
#include <cuda_runtime.h>

#include <algorithm>

#include "fdga_kernels.h"

namespace fdga {

namespace {

// separable 2D DFT of an L x L tile in shared memory (x fastest), sign ±1: out = Σ in e^{sign 2πi k·x/L}
__device__ void dft2_tile(const cplx* in, cplx* tmp, cplx* out, int L, int sign) {
    const int NN = L * L;
    for (int e = threadIdx.x; e < NN; e += blockDim.x) {  // along x
        const int kx = e % L, y = e / L;
        cplx s = mk(0, 0);
        for (int x = 0; x < L; ++x) {
            double sn, cs;
            sincospi(2.0 * sign * (double)((kx * x) % L) / L, &sn, &cs);
            s = cfma(in[x + L * y], mk(cs, sn), s);
        }
        tmp[kx + L * y] = s;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < NN; e += blockDim.x) {  // along y
        const int kx = e % L, ky = e / L;
        cplx s = mk(0, 0);
        for (int y = 0; y < L; ++y) {
            double sn, cs;
            sincospi(2.0 * sign * (double)((ky * y) % L) / L, &sn, &cs);
            s = cfma(tmp[kx + L * y], mk(cs, sn), s);
        }
        out[kx + L * ky] = s;
    }
    __syncthreads();
}

struct InterpRows {
    const cplx* in;
    cplx* out;
    int kind;  // 0 Σ (frequencies clamped), 1 K1, 2 K2, 3 K3
};

// source row of a target frequency point, or -1 when it lies outside the source mesh
__device__ int source_row(int kind, int r, const Dims& o, const Dims& i) {
    if (kind == 0) {
        int nu = r - o.nG;
        nu = max(-i.nG, min(i.nG - 1, nu));
        return nu + i.nG;
    }
    if (kind == 1) {
        const int m = r - (o.n1 - 1);
        return bin(m, i.n1) ? m + i.n1 - 1 : -1;
    }
    if (kind == 2) {
        const int n = r % o.N2n - o.n2n, m = r / o.N2n - (o.n2O - 1);
        if (!bin(m, i.n2O) || !fin(n, i.n2n)) return -1;
        return (m + i.n2O - 1) * i.N2n + (n + i.n2n);
    }
    const int np = r % o.N3n - o.n3n, n = (r / o.N3n) % o.N3n - o.n3n, m = r / (o.N3n * o.N3n) - (o.n3O - 1);
    if (!bin(m, i.n3O) || !fin(n, i.n3n) || !fin(np, i.n3n)) return -1;
    return ((m + i.n3O - 1) * i.N3n + (n + i.n3n)) * i.N3n + (np + i.n3n);
}

__global__ void k_fourier_interp(InterpRows a, int rows_o, int rows_i, Dims o, Dims i) {
    extern __shared__ cplx sm[];
    const int Li = i.L, Lo = o.L, Ni = Li * Li, No = Lo * Lo;
    cplx* A = sm;           // Li²: source values, then their real-space coefficients
    cplx* T = A + Ni;       // max(Li², Lo²): transform scratch
    cplx* B = T + max(Ni, No);  // Lo²: real-space target, then the target values
    const int r = blockIdx.x;
    const int ri = source_row(a.kind, r, o, i);
    if (ri < 0) {
        for (int e = threadIdx.x; e < No; e += blockDim.x) a.out[(size_t)e * rows_o + r] = mk(0, 0);
        return;
    }
    for (int e = threadIdx.x; e < Ni; e += blockDim.x) A[e] = a.in[(size_t)e * rows_i + ri];
    for (int e = threadIdx.x; e < No; e += blockDim.x) B[e] = mk(0, 0);
    __syncthreads();
    dft2_tile(A, T, A, Li, -1);  // in place through T: A <- fft(A) (unscaled)
    // R in [-Li/2, Li/2]², half weights on the boundary of an even Li; one thread per target cell
    const int h = Li / 2;
    const double scale = 1.0 / Ni;
    for (int e = threadIdx.x; e < No; e += blockDim.x) {
        const int ox = e % Lo, oy = e / Lo;
        cplx s = mk(0, 0);
        // the R ≡ (ox, oy) mod Lo of the source range (several when Lo ≤ Li: aliasing adds them)
        for (int R1 = -h + ((ox + h) % Lo + Lo) % Lo; R1 <= h; R1 += Lo)
            for (int R2 = -h + ((oy + h) % Lo + Lo) % Lo; R2 <= h; R2 += Lo) {
                double w = scale;
                if ((Li & 1) == 0) {
                    if (abs(R1) == h) w *= 0.5;
                    if (abs(R2) == h) w *= 0.5;
                }
                s += A[((R1 % Li) + Li) % Li + Li * (((R2 % Li) + Li) % Li)] * w;
            }
        B[e] = s;
    }
    __syncthreads();
    dft2_tile(B, T, B, Lo, +1);
    for (int e = threadIdx.x; e < No; e += blockDim.x) a.out[(size_t)e * rows_o + r] = B[e];
}

}  // namespace

size_t fourier_interp_smem(const Dims& o, const Dims& i) {
    const size_t Ni = (size_t)i.L * i.L, No = (size_t)o.L * o.L;
    return (Ni + std::max(Ni, No) + No) * sizeof(cplx);
}

// kind 0: Σ [k][ν]; 1..3: K1, K2, K3 of one channel [P][frequencies]
cudaError_t launch_fourier_interp(cudaStream_t s, int kind, const cplx* in, cplx* out, const Dims& o, const Dims& i) {
    int rows_o, rows_i;
    switch (kind) {
        case 0: rows_o = o.NG; rows_i = i.NG; break;
        case 1: rows_o = o.N1; rows_i = i.N1; break;
        case 2: rows_o = o.N2O * o.N2n; rows_i = i.N2O * i.N2n; break;
        default: rows_o = o.N3O * o.N3n * o.N3n; rows_i = i.N3O * i.N3n * i.N3n; break;
    }
    const size_t smem = fourier_interp_smem(o, i);
    static SmemRecord raised;
    cudaError_t e = raise_smem_limit(k_fourier_interp, raised, smem);
    if (e != cudaSuccess) return e;
    const int threads = std::min(256, std::max(32, ((std::max(i.L * i.L, o.L * o.L) + 31) / 32) * 32));
    InterpRows a{in, out, kind};
    k_fourier_interp<<<rows_o, threads, smem, s>>>(a, rows_o, rows_i, o, i);
    return cudaGetLastError();
}

}  // namespace fdga
