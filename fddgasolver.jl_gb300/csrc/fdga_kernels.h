// fdga_kernels.h -- kernel argument bundles and launchers (host-visible).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <mutex>

#include "fdga_device.cuh"

namespace fdga {

// Raises a kernel's dynamic shared-memory limit to at least `bytes` on the current device; `raised`
// is the caller's record of the largest limit set for that kernel, one entry per device ordinal
// (cudaFuncSetAttribute acts on the current device only).  One process-wide lock serialises the check
// and the update, so concurrent launchers never lower a limit another thread raised.  Sizes up to
// `floor` need no raise (48 KB for a kernel without static shared memory; the default limit counts
// both kinds, so a kernel with static shared memory passes 0 and raises before any graph capture).
struct SmemRecord {
    static constexpr int kMaxDevices = 64;
    size_t bytes[kMaxDevices] = {};
};
template <class K>
inline cudaError_t raise_smem_limit(K kernel, SmemRecord& raised, size_t bytes, size_t floor = 48 * 1024) {
    if (bytes <= floor) return cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= SmemRecord::kMaxDevices) return cudaErrorInvalidDevice;
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if (bytes <= raised.bytes[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) raised.bytes[dev] = bytes;
    return e;
}

struct ChanArrays {  // read-only K arrays of the three channels
    const cplx* K1[3];
    const cplx* K2[3];
    const cplx* K3[3];
};
struct ChanArraysW {  // written arrays of the three channels
    cplx* K1[3];
    cplx* K2[3];
    cplx* K3[3];
};
struct Caches {  // Γpx F0p F0a F0t Γpp Γa Γt Fp Fa Ft
    cplx* c[10];
    cplxf* f[10];  // FP32 copies written instead of c in the mixed map (nullptr: FP64 map)
};
template <class S>
struct FLPT {  // left vertex FL: only K2 enters the K1/K2 BSE through FL(Ω, ω, νInf)
    const S* K2[3];
};
using FLP = FLPT<cplx>;
using FLPF = FLPT<cplxf>;
struct K3Args {
    const cplx* A;    // cacheΓ (L_K3) or cacheF (K3)
    const cplx* B0;   // cacheF0
    const cplx* G;    // cacheΓ (K3, right part)
    const cplx* Pi;
    const cplx* Pi0;
    const cplx* FLc;  // FL.γ_ch.K3 (a, p)
    const cplx* FLt;  // FL.γt.K3
    const cplx* FLa;  // FL.γa.K3
    cplx* out;
    int flags;        // K3F_* (product-rule terms of the tangent map)
    // tangent contraction (mode 2): dA, dΓ, dΠ and dFL beside the values above
    const cplx* tA;
    const cplx* tG;
    const cplx* tPi;
    const cplx* tFLc;
    const cplx* tFLt;
    const cplx* tFLa;
};
// K3Args flags: accumulate into out; leave the γL(ν,ν') epilogue term out; Pi0 == nullptr reads zero
// K3F_1LOOP: the one-loop form of :fdPA_1loop, M = s1 (Π - Π0) F0 (no Γ and no FL terms)
enum { K3F_ACC = 1, K3F_NOEPI = 2, K3F_1LOOP = 4 };

struct K3ArgsF {  // FP32 operands of the mixed map (the FP32 caches and FL.K3 copy)
    const cplxf* A;
    const cplxf* B0;
    const cplxf* G;
    const cplx* Pi;
    const cplx* Pi0;
    const cplxf* FLc;
    const cplxf* FLt;
    const cplxf* FLa;
    cplx* out;
    int flags;
    const cplxf* tA;
    const cplxf* tG;
    const cplx* tPi;
    const cplxf* tFLc;
    const cplxf* tFLt;
    const cplxf* tFLa;
};
struct K3Args3F {
    K3ArgsF a[3];
    int ch[3];
    const int* blocks;
    int nblocks;
};
struct K3Args3 {  // the three channels of one K3 launch over a list of (P, Ω) blocks
    K3Args a[3];
    int ch[3];
    const int* blocks;  // block = P * NΩ3 + iΩ; nullptr = all blocks
    int nblocks;
};

struct ChanWork {  // per-channel work of an all-channel launch, indexed by channel (p, t, a) or (pp, ph)
    const int* items[3];  // representative device indices, ascending (nullptr: item = index)
    int nitems[3];
    // K2: rows of items that share (P, Ω); row r = items[gstart[r] .. gstart[r+1]) (nullptr: the
    // N2n consecutive indices of row r)
    const int* gstart[3];
    int ngroups[3];
    cplx* out[3];
    int acc;  // 1: out += value (product-rule terms of the tangent map)
};
struct BubbleP {
    const cplx* pp;
    const cplx* ph;
    const cplx* pp0;
    const cplx* ph0;
};
// Tangent factors of the K1/K2 BSE and SDE kernels (TAN form): the tangent vertex, dFL, dΠ, dS_X
// and dSΠ, beside the value arguments.
template <class S>
struct TanArgsT {
    VertPT<S> F;
    FLPT<S> FL;
    const cplx* pp;
    const cplx* ph;
    const cplx* SX;
    const cplx* SPpp;
    const cplx* SPph;
};
using TanArgs = TanArgsT<cplx>;
using TanArgsF = TanArgsT<cplxf>;
// cotangent (adjoint) views: writable K arrays and momentum averages of the three channels
struct ChanBar {
    cplx *K1, *K2, *K3, *A1, *A2, *A3;
};
struct VertBar {
    ChanBar g[3];
};
struct FLBar {
    cplx* K2[3];
};
struct ChanBarArrays {  // averages' cotangents (read) and the K arrays' cotangents (accumulated)
    const cplx* A1[3];
    const cplx* A2[3];
    const cplx* A3[3];
    cplx* K1[3];
    cplx* K2[3];
    cplx* K3[3];
};
struct Ptr3 {
    cplx* p[3];
};
struct Finalize3 {  // indexed by channel (p, t, a)
    const cplx* raw[3];
    cplx* out[3];
    const uint32_t* map[3];
    const cplx* FL[3];
    cplxf* outf[3];  // optional FP32 copies of out (FL.K3 of the mixed map)
};

constexpr int AA_MAX = 64;  // largest Anderson memory of the device solver
struct AAVecs {
    const cplx* v[AA_MAX];
};
struct AAVecsW {
    cplx* v[AA_MAX];
};
constexpr int KR_MAX = 64;  // largest Krylov basis of the GMRES solves
struct KrVecs {
    const cplxf* v[KR_MAX];
};
// Device-resident Arnoldi cycle (a GMRES restart cycle replayed as one graph with a WHILE node):
// the loop counters, the stopping data and the Hessenberg matrix with its Givens rotations.
struct KrDevState {
    int j;         // column being built
    int k;         // columns completed
    int done;      // converged (|g_{j+1}| <= thr) or breakdown (H(j+1, j) = 0)
    int nmaps;     // operator applications in this cycle
    int budget;    // applications allowed in this cycle
    int cost;      // applications per column
    int m;         // restart length
    int pad;
    double thr;    // absolute stopping threshold on the residual estimate
    double est;    // |g_{j+1}| after the last column
    double hn;     // H(j+1, j) of the last column
    double H[(KR_MAX + 1) * KR_MAX];  // column-major, leading dimension KR_MAX + 1
    double cs[KR_MAX], sn[KR_MAX], g[KR_MAX + 1];
};
struct AAVecs32 {
    const cplxf* v[AA_MAX];
};
struct AAVecs32W {
    cplxf* v[AA_MAX];
};

cudaError_t set_fft_twiddles();
// vertex-evaluating kernels: VertP/FLP (FP64 plain map) or VertPF/FLPF (FP32 mirror, mixed map)
cudaError_t launch_bse_K1_all(cudaStream_t s, const VertP& F, const FLP& FL, const BubbleP& B, const cplx* SX,
                              const ChanWork& cw, const Dims& d);
cudaError_t launch_bse_L_K2_all(cudaStream_t s, const VertP& F, const BubbleP& B, const ChanWork& cw, const Dims& d);
cudaError_t launch_bse_K2_all(cudaStream_t s, const VertP& F, const FLP& FL, const BubbleP& B, const cplx* SX,
                              const ChanWork& cw, const Dims& d);
cudaError_t launch_sde_L_all(cudaStream_t s, const VertP& F, const BubbleP& B, const cplx* SPpp, const cplx* SPph,
                             const ChanWork& cw, int use_vertex, double ref_scale, const Dims& d);
cudaError_t launch_bse_K1_all(cudaStream_t s, const VertPF& F, const FLPF& FL, const BubbleP& B, const cplx* SX,
                              const ChanWork& cw, const Dims& d);
cudaError_t launch_bse_L_K2_all(cudaStream_t s, const VertPF& F, const BubbleP& B, const ChanWork& cw, const Dims& d);
cudaError_t launch_bse_K2_all(cudaStream_t s, const VertPF& F, const FLPF& FL, const BubbleP& B, const cplx* SX,
                              const ChanWork& cw, const Dims& d);
cudaError_t launch_sde_L_all(cudaStream_t s, const VertPF& F, const BubbleP& B, const cplx* SPpp, const cplx* SPph,
                             const ChanWork& cw, int use_vertex, double ref_scale, const Dims& d);
cudaError_t launch_build_cache(cudaStream_t s, const VertPF& F, const Caches& C, const int* blocks, int nblocks,
                               const Dims& d);
// K1 and K2 of the :fdPA_new / :scPA_new strategies (local solver); SPi, SPi0: full-mesh row sums [2][Nq][NΠΩ]
cudaError_t launch_bse_K1_new(cudaStream_t s, const VertP& F, const BubbleP& B, const cplx* SPi, const cplx* SPi0,
                              const ChanWork& cw, const Dims& d);
cudaError_t launch_bse_K2_new(cudaStream_t s, const VertP& F, const BubbleP& B, const cplx* SPi, const cplx* SPi0,
                              const ChanWork& cw, const Dims& d);
cudaError_t launch_bse_K1_new(cudaStream_t s, const VertPF& F, const BubbleP& B, const cplx* SPi, const cplx* SPi0,
                              const ChanWork& cw, const Dims& d);
cudaError_t launch_bse_K2_new(cudaStream_t s, const VertPF& F, const BubbleP& B, const cplx* SPi, const cplx* SPi0,
                              const ChanWork& cw, const Dims& d);
// tangent forms: dK = K(dF; Π, FL, S_X) + K(F; dΠ, dFL, dS_X) in one pass (the T factors), and
// dL = L(dF; Π, SΠ) + L(F; dΠ, dSΠ) (+ the RefVertex part with dΠ)
cudaError_t launch_bse_K1_tan(cudaStream_t s, const VertP& F, const FLP& FL, const BubbleP& B, const cplx* SX,
                              const TanArgs& T, const ChanWork& cw, const Dims& d);
cudaError_t launch_bse_K2_tan(cudaStream_t s, const VertP& F, const FLP& FL, const BubbleP& B, const cplx* SX,
                              const TanArgs& T, const ChanWork& cw, const Dims& d);
cudaError_t launch_sde_L_tan(cudaStream_t s, const VertP& F, const BubbleP& B, const cplx* SPpp, const cplx* SPph,
                             const TanArgs& T, const ChanWork& cw, double ref_scale, const Dims& d);
cudaError_t launch_bse_K1_tan(cudaStream_t s, const VertPF& F, const FLPF& FL, const BubbleP& B, const cplx* SX,
                              const TanArgsF& T, const ChanWork& cw, const Dims& d);
cudaError_t launch_bse_K2_tan(cudaStream_t s, const VertPF& F, const FLPF& FL, const BubbleP& B, const cplx* SX,
                              const TanArgsF& T, const ChanWork& cw, const Dims& d);
cudaError_t launch_sde_L_tan(cudaStream_t s, const VertPF& F, const BubbleP& B, const cplx* SPpp, const cplx* SPph,
                             const TanArgsF& T, const ChanWork& cw, double ref_scale, const Dims& d);
cudaError_t launch_finalize3(cudaStream_t s, const Finalize3& f, int k2_epilogue, int t_recombine, size_t n);
// T0: the tail·tail part of the R = 0 row sums (launch_tail_const, once per solver);
// GRf (optional): FP32 copy of G(R) -> the real-space row sums run in FP32 (mixed map)
cudaError_t launch_rowsum(cudaStream_t s, const cplx* A0, const cplx* A1, const cplx* GR, cplx* SRtmp, const cplx* twp,
                          cplx* S0, cplx* S1, const Dims& d, const cplx* T0, const cplxf* GRf = nullptr);
cudaError_t launch_tail_const(cudaStream_t s, cplx* T0, const Dims& d);
bool bubble_f32_supported(const Dims& d);
cudaError_t launch_bubble_f32(cudaStream_t s, const cplxf* GRf, cplx* pp, cplx* ph, const cplx* twp, const Dims& d);
// F0v: the FP64 vertex view whose reference vertex enters F0(Ω, ω̃, ∞) (only has0/g0/b0 are read)
cudaError_t launch_sx(cudaStream_t s, const BubbleP& B, const cplx* SPi, const cplx* SPi0, const FLP& FL,
                      const VertP& F0v, cplx* SX, const Dims& d);
cudaError_t launch_dyson(cudaStream_t s, cplx* G, const cplx* Sig, const cplx* Gb, size_t n);
cudaError_t launch_occupation(cudaStream_t s, const cplx* G, size_t n, double T, int Nk, double* out);
cudaError_t launch_g_realspace(cudaStream_t s, const cplx* G, cplx* GR, const cplx* tw, const Dims& d);
int bubble_tile(const Dims& d);
cudaError_t launch_bubble(cudaStream_t s, const cplx* G, const cplx* GR, cplx* pp, cplx* ph, const cplx* twp,
                          const Dims& d);
cudaError_t launch_qavg(cudaStream_t s, const ChanArrays& in, const ChanArraysW& out, const Dims& d);
cudaError_t launch_build_cache(cudaStream_t s, const VertP& F, const Caches& C, const int* blocks, int nblocks,
                               const Dims& d);
// mode 0 (left K3), 1 (K3), 2 (tangent of K3: dA·M + A·dM + dγL as one GEMM over the concatenated
// inner index).  tile: 16, 24 or 32 (square output tiles of the GEMM kernel) or 116, 124, 132 (TILE
// rows x TILE/2 columns); any other value picks the default for Nν3 and the launch's CTA count
cudaError_t launch_bse_K3(cudaStream_t s, int mode, const K3Args3& a, int nslots, const Dims& d, int mixed, int tile);
bool k3_tile_valid(int tile);
cudaError_t launch_bse_K3_f32(cudaStream_t s, int mode, const K3Args3F& a, int nslots, const Dims& d, int tile);
cudaError_t launch_to_f32(cudaStream_t s, const cplx* in, cplxf* out, size_t n);
// TMA-fed, warp-specialised tcgen05 form (fdga_k3_tma.cu): the FP32 operand arrays live in up to four
// buffers (the caches, FL.K3, the tangent caches, the tangent FL.K3; base == nullptr: absent) over
// which the TMA tensor maps are built; every K3ArgsF operand pointer must lie in one of them
struct TmaBuffers {
    const void* base[4];
    size_t ncplx[4];
};
bool k3_tma_supported(const Dims& d, int mode);
cudaError_t prepare_bse_K3_tma(const Dims& d);
cudaError_t launch_bse_K3_tma(cudaStream_t s, int mode, const K3Args3F& a, int nslots, const Dims& d, int* err,
                              const TmaBuffers& bufs);
// tcgen05 form of the mixed K3 contractions (2Nν3 ≤ 256 MMA columns); *err set on a wait timeout
bool k3_tc_supported(const Dims& d);
cudaError_t prepare_bse_K3_tc(const Dims& d);
cudaError_t launch_bse_K3_tc(cudaStream_t s, int mode, const K3Args3F& a, int nslots, const Dims& d, int* err);
cudaError_t launch_sde_sigma(cudaStream_t s, const cplx* GR, const cplx* Lpp, const cplx* Lph, cplx* LR, cplx* SR,
                             cplx* S, const cplx* twm, const cplx* twp, const Dims& d);
cudaError_t launch_fft2(cudaStream_t s, const cplx* in, cplx* out, int rows, int sign, double scale,
                        const cplx* tw_sign, const Dims& d);
cudaError_t launch_u2(cudaStream_t s, const cplx* GR, cplx* C, cplx* SR, cplx* out, const cplx* twc, const Dims& d);
cudaError_t launch_sigma_assemble(cudaStream_t s, const cplx* Sin, const cplx* SU2, const uint32_t* map,
                                  const double* occ, const cplx* C0, const cplx* Sig0, cplx* Sig, double U, int hartree,
                                  int fdpa, double n0, size_t n);
cudaError_t launch_gather(cudaStream_t s, cplx* dst, const cplx* src, const uint32_t* perm, size_t n);
cudaError_t launch_scatter(cudaStream_t s, cplx* dst, const cplx* src, const uint32_t* perm, size_t n);
cudaError_t launch_residual(cudaStream_t s, const cplx* y, const cplx* x, cplx* fx, cplx* g, double beta, double* pmax,
                            int nblk, size_t n);
cudaError_t launch_sub(cudaStream_t s, cplx* out, const cplx* a, const cplx* b, size_t n);
cudaError_t launch_gather_sub(cudaStream_t s, cplx* out, const cplx* y, const cplx* x, const uint32_t* perm, size_t n);
cudaError_t launch_aa_diff(cudaStream_t s, int nblk, cplx* dg, const cplx* g, const cplx* gold, cplx* df,
                           const cplx* fx, const cplx* Qb, cplx* part_out, size_t n);
cudaError_t launch_aa_mgs(cudaStream_t s, int nblk, cplx* df, const cplx* Qa, const cplx* part_in, cplx* Rentry,
                          const cplx* Qb, cplx* part_out, size_t n);
cudaError_t launch_aa_qnew(cudaStream_t s, int nblk, cplx* Qk, const cplx* df, const cplx* part_in, cplx* Rkk,
                           size_t n);
cudaError_t launch_aa_gamma(cudaStream_t s, int nblk, const AAVecs& Q, int meff, const cplx* fx, cplx* part,
                            const cplx* R, int m, cplx* gam, size_t n);
cudaError_t launch_aa_update(cudaStream_t s, int nblk, cplx* x, const cplx* g, const AAVecs& dG, const cplx* gam,
                             int meff, const cplx* fx, cplx* fxold, cplx* gold, size_t n);
cudaError_t launch_aa_delete(cudaStream_t s, int nblk, cplx* R, int m, cplx* rot, const AAVecsW& Q, size_t n);
cudaError_t launch_aa_givens(cudaStream_t s, cplx* R, int m, cplx* rot);
cudaError_t launch_aa_gamma_solve(cudaStream_t s, const cplx* part, int np, const cplx* R, int m, int meff, cplx* gam);
// FP32-history Anderson (mixed-precision inner solves)
cudaError_t launch_ma_residual(cudaStream_t s, int nblk, const cplx* y, const cplx* c, const cplx* x, cplxf* f32,
                               cplx* g, double beta, double* pmax, size_t n);
cudaError_t launch_ma_diff(cudaStream_t s, int nblk, cplxf* dg, const cplx* g, const cplx* gold, cplxf* df,
                           const cplxf* f, const cplxf* Qb, cplx* part_out, size_t n);
cudaError_t launch_ma_mgs(cudaStream_t s, int nblk, cplxf* df, const cplxf* Qa, const cplx* part_in, cplx* Rentry,
                          const cplxf* Qb, cplx* part_out, size_t n);
cudaError_t launch_ma_qnew(cudaStream_t s, int nblk, cplxf* Qk, const cplxf* df, const cplx* part_in, cplx* Rkk,
                           size_t n);
cudaError_t launch_ma_multidot(cudaStream_t s, int nblk, const AAVecs32& Q, int nv, const cplxf* f, cplx* part,
                               size_t n);
cudaError_t launch_ma_update(cudaStream_t s, int nblk, cplx* x, const cplx* g, const AAVecs32& dG, const cplx* gam,
                             int meff, const cplxf* f, cplxf* fold, cplx* gold, size_t n);
cudaError_t launch_ma_qrot(cudaStream_t s, int nblk, const AAVecs32W& Q, int m, const cplx* rot, size_t n);
cudaError_t launch_chi(cudaStream_t s, const cplx* K1p, const cplx* K1t, const cplx* K1a, int which, double U,
                       int NO, int Nq, int local, cplx* out);
cudaError_t measure_fp64_rate(float* ms, double* gflops);
// number of mismatches between d2f_rn and the hardware FP64 -> FP32 conversion over n hashed inputs
cudaError_t selftest_d2f(size_t n, unsigned int* mismatches_host);
// mfRG linear map (fdga_mfrg.cu): part 0 the irreducible caches of the state vertex, part 1 the
// F0-only caches; the K1/K2 BSEs of the map (FP64, F0 and FL.K2 only)
cudaError_t launch_build_cache_mfrg(cudaStream_t s, const VertP& F, const Caches& C, const int* blocks, int nblocks,
                                    const Dims& d, int part);
cudaError_t launch_build_cache_mfrg(cudaStream_t s, const VertPF& F, const Caches& C, const int* blocks, int nblocks,
                                    const Dims& d, int part);
cudaError_t launch_bse_K1_mfrg(cudaStream_t s, const VertP& F, const FLP& FL, const BubbleP& B, const ChanWork& cw,
                               const Dims& d);
cudaError_t launch_bse_K2_mfrg(cudaStream_t s, const VertP& F, const FLP& FL, const BubbleP& B, const ChanWork& cw,
                               const Dims& d);
cudaError_t launch_scale(cudaStream_t s, cplx* out, const cplx* in, double sc, size_t n);
// FP64 K3 contractions on the tensor cores by exact BF16 digit slicing (fdga_k3_oz.cu), modes 0, 1
// and 2 (the tangent); fa_scratch holds nslots x nblocks ints (per-block exponent bounds), adig the
// A digit operands of adig_blocks blocks (k3_oz_digit_bytes each); ebound = 1 bounds every tile of
// M from the FP64 exponents of its factors (the path taken when the FP32 magnitude bound
// overflows), for tests
bool k3_oz_supported(const Dims& d);
size_t k3_oz_digit_bytes(const Dims& d);
cudaError_t prepare_bse_K3_oz();
cudaError_t launch_bse_K3_oz(cudaStream_t s, int mode, const K3Args3& a, int nslots, const Dims& d, int* err,
                             int* fa_scratch, uint8_t* adig, int adig_blocks, int ebound);
cudaError_t launch_cache_broadcast(cudaStream_t s, cplx* c0, cplx* c1, cplx* c2, const uint32_t* map, size_t n);
cudaError_t launch_cache_broadcast(cudaStream_t s, cplxf* c0, cplxf* c1, cplxf* c2, const uint32_t* map, size_t n);
// GMRES building blocks (real inner products on the FP32 Krylov basis)
cudaError_t launch_kr_point(cudaStream_t s, int nblk, const cplx* x, const cplxf* v, double eps, cplx* xp, size_t n);
cudaError_t launch_kr_apply(cudaStream_t s, int nblk, const cplx* y, const cplx* y0, const cplxf* v, double a,
                            double b, cplxf* w, size_t n);
cudaError_t launch_kr_dots(cudaStream_t s, int nblk, const KrVecs& V, int nv, const cplxf* w, const float* wgt,
                           double* part, int norm_slot, size_t n);
cudaError_t launch_kr_reduce(cudaStream_t s, const double* part, int np, int ncoef, double* coef);
cudaError_t launch_kr_sub(cudaStream_t s, int nblk, const KrVecs& V, int nv, const double* c, cplxf* w, size_t n);
cudaError_t launch_kr_scale(cudaStream_t s, int nblk, const cplxf* w, double nrm, cplxf* out, size_t n);
cudaError_t launch_kr_update(cudaStream_t s, int nblk, cplx* x, const KrVecs& V, int nv, const double* y, double scale,
                             size_t n);
cudaError_t launch_kr_load(cudaStream_t s, int nblk, const cplx* a, const float* wgt, cplxf* out, double* part,
                           size_t n);
// symmetric-subspace (one value per symmetry class) storage of Krylov vectors
cudaError_t launch_kc_point(cudaStream_t s, int nblk, const cplx* x, const cplxf* v, const uint32_t* code, double eps,
                            cplx* xp, size_t n);
cudaError_t launch_kc_axpy(cudaStream_t s, int nblk, const cplx* x, const cplx* d, const uint32_t* code, double lam,
                           cplx* out, size_t n);
cudaError_t launch_kc_apply(cudaStream_t s, int nblk, const cplx* y, const cplx* y0, const uint32_t* pos,
                            const cplxf* v, double a, double b, cplxf* w, size_t nc);
cudaError_t launch_kc_gather(cudaStream_t s, int nblk, const cplx* y, const cplx* x, const uint32_t* pos, double sc,
                             cplx* out, size_t nc);
cudaError_t launch_kc_count(cudaStream_t s, int nblk, const uint32_t* code, float* w, size_t n);
cudaError_t launch_kc_codes(cudaStream_t s, const uint32_t* map, const int* items, int nitems, size_t nblock,
                            size_t base, uint32_t off, uint32_t* code, uint32_t* pos);
cudaError_t launch_kr_resid(cudaStream_t s, int nblk, const cplx* b, const cplxf* v, double alpha, const cplx* y,
                            const cplx* yb, double beta, cplx* r, size_t n);
cudaError_t launch_kr_axpby(cudaStream_t s, int nblk, cplx* out, const cplx* a, double lam, const cplx* b, size_t n);
// the Arnoldi column j = st->j of the device-resident cycle (fdga_krylov.cu): the operator input
// V[j] expanded into xp (x + eps op(V[j])), its output gathered into w, the two classical
// Gram-Schmidt passes (the second with |w|²), the Hessenberg/Givens update, V[j+1] and the advance
// that sets the WHILE node's condition
cudaError_t launch_kr_init(cudaStream_t s, KrDevState* st, int m, int budget, int cost, double thr, double beta);
cudaError_t launch_kc_point_j(cudaStream_t s, int nblk, const cplx* x, const KrVecs& V, const KrDevState* st,
                              const uint32_t* code, double eps, cplx* xp, size_t n);
cudaError_t launch_kc_apply_j(cudaStream_t s, int nblk, const cplx* y, const uint32_t* pos, const KrVecs& V,
                              const KrDevState* st, double a, double b, cplxf* w, size_t nc);
cudaError_t launch_kr_cgs_j(cudaStream_t s, int nblk, const KrVecs& V, KrDevState* st, cplxf* w, const float* wgt,
                            double* part, double* c1, double* c2, size_t n);
cudaError_t launch_kr_advance(cudaStream_t s, KrDevState* st, cudaGraphConditionalHandle cond);
cudaError_t launch_nonfinite(cudaStream_t s, const cplx* a, size_t n, unsigned int* count);
// tangent (forward-mode derivative) stages of the iteration map; the value intermediates (G, G(R),
// Π, L(R), C of the U² term) of the same base point are inputs
cudaError_t launch_dyson_tan(cudaStream_t s, cplx* tG, const cplx* G, const cplx* tSig, size_t n);
cudaError_t launch_bubble_tan(cudaStream_t s, const cplx* G, const cplx* tG, const cplx* GR, const cplx* tGR,
                              cplx* tpp, cplx* tph, const cplx* twp, const Dims& d);
cudaError_t launch_bubble_f32_tan(cudaStream_t s, const cplxf* GRf, const cplxf* tGRf, cplx* tpp, cplx* tph,
                                  const cplx* twp, const Dims& d);
cudaError_t launch_rowsum_tan(cudaStream_t s, const cplx* tA0, const cplx* tA1, const cplx* GR, const cplx* tGR,
                              cplx* SRtmp, const cplx* twp, cplx* tS0, cplx* tS1, const Dims& d,
                              const cplxf* GRf = nullptr, const cplxf* tGRf = nullptr);
cudaError_t launch_sx_tan(cudaStream_t s, const cplx* Pipp, const cplx* Piph, const cplx* tPipp, const cplx* tPiph,
                          const cplx* tSPi, const FLP& FL, const FLP& tFL, const VertP& F0v, cplx* tSX,
                          const Dims& d);
cudaError_t launch_sde_sigma_tan(cudaStream_t s, const cplx* GR, const cplx* LR, const cplx* tGR, const cplx* tLpp,
                                 const cplx* tLph, cplx* tLR, cplx* tSR, cplx* tS, const cplx* twm, const cplx* twp,
                                 const Dims& d);
// Fourier interpolation between lattice sizes (fdga_interp.cu): kind 0 Σ [k][ν] (frequencies
// clamped to the source mesh), 1..3 K1, K2, K3 of one channel [P][frequencies] (zero outside it)
cudaError_t launch_fourier_interp(cudaStream_t s, int kind, const cplx* in, cplx* out, const Dims& o, const Dims& i);
// reverse-mode (adjoint) stages of the iteration map (fdga_adjoint.cu)
cudaError_t launch_adj_assemble(cudaStream_t s, const cplx* Sbar, const uint32_t* map, cplx* Sin_bar, cplx* SU2_bar,
                                size_t n, int hartree, double U, double* nbar);
cudaError_t launch_adj_occupation(cudaStream_t s, cplx* Gbar, const double* nbar, double T, int Nk, size_t n);
cudaError_t launch_adj_dyson(cudaStream_t s, const cplx* G, const cplx* Gbar, cplx* Sbar, size_t n);
cudaError_t launch_adj_u2(cudaStream_t s, const cplx* GR, const cplx* C, cplx* obar_k, cplx* obar_R, cplx* Cbar,
                          cplx* GRbar, const cplx* twm, const Dims& d);
cudaError_t launch_adj_sigma(cudaStream_t s, const cplx* GR, const cplx* LR, const cplx* Sinbar, cplx* SRbar,
                             cplx* LRbar, cplx* Lbar, cplx* GRbar, const cplx* twm, const cplx* twp, const Dims& d);
cudaError_t launch_adj_finalize3(cudaStream_t s, const Finalize3& f, int k2_epilogue, int t_recombine, size_t n,
                                 cplx* const FLbar[3]);
cudaError_t launch_adj_sde_L(cudaStream_t s, const VertP& F, const VertBar& Fb, const BubbleP& B, const cplx* SPpp,
                             const cplx* SPph, cplx* Pbpp, cplx* Pbph, cplx* SPbpp, cplx* SPbph, const cplx* rawbar,
                             const ChanWork& cw, size_t n2, double rs, const Dims& d);
cudaError_t launch_adj_K1(cudaStream_t s, const VertP& F, const FLP& FL, const BubbleP& B, const cplx* SX,
                          const VertBar& Fb, const FLBar& FLb, cplx* Pbpp, cplx* Pbph, cplx* SXbar, const cplx* rawbar,
                          const ChanWork& cw, size_t n1, const Dims& d);
cudaError_t launch_adj_K2(cudaStream_t s, const VertP& F, const FLP& FL, const BubbleP& B, const cplx* SX,
                          const VertBar& Fb, const FLBar& FLb, cplx* Pbpp, cplx* Pbph, cplx* SXbar, const cplx* rawbar,
                          const ChanWork& cw, size_t n2, const Dims& d);
cudaError_t launch_adj_sx(cudaStream_t s, const cplx* Pipp, const cplx* Piph, const FLP& FL, const cplx* SXbar,
                          cplx* Pbpp, cplx* Pbph, cplx* SPibar, const FLBar& FLb, const Dims& d);
cudaError_t launch_adj_L_K2(cudaStream_t s, const BubbleP& B, const VertBar& Fb, const cplx* rawbar, const ChanWork& cw,
                            size_t n2, const Dims& d);
cudaError_t launch_adj_cache(cudaStream_t s, const VertBar& Fb, const Caches& Cb, const int* blocks, int nblocks,
                             const Dims& d);
cudaError_t launch_adj_K3(cudaStream_t s, int mode, const K3Args3& a, const cplx* const Obar[3], cplx* const Abar[3],
                          cplx* const Gbar[3], cplx* const Mbuf[3], cplx* const Mbar[3], cplx* Pbpp, cplx* Pbph,
                          cplx* const FLbar[3], const Dims& d);
cudaError_t launch_adj_bubble(cudaStream_t s, const cplx* GR, cplx* Pbpp, cplx* Pbph, cplx* PbRpp, cplx* PbRph,
                              const cplx* SPibar, cplx* SRbar, cplx* GRbar, const cplx* twm, const Dims& d);
cudaError_t launch_adj_qavg(cudaStream_t s, const ChanBarArrays& bar, const Dims& d);
cudaError_t launch_u2_tan(cudaStream_t s, const cplx* GR, const cplx* C, const cplx* tGR, cplx* tC, cplx* tSR,
                          cplx* tout, const cplx* twc, const Dims& d);

}  // namespace fdga
