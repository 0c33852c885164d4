/* fdga.h -- C ABI of libfdga, the GB300 (sm_103a) implementation of the parquet-iteration hot
 * path of fdDGAsolver.jl.  Plain pointers and sizes only; complex arrays are interleaved
 * (re, im) doubles, i.e. Julia ComplexF64 / C double _Complex, in the reference's own
 * column-major layout (first mesh index fastest).  Every call returns 0 on success or a
 * nonzero FDGA_ERR_* status; fdga_last_error() gives the message.  No entry point aborts
 * or traps; there is no CPU fallback inside the library.
 *
 * One handle owns one solver's device state and one CUDA stream.  Calls on a handle must be
 * serialised by the caller; distinct handles may be used concurrently.
 */
#ifndef FDGA_H
#define FDGA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fdga_handle fdga_handle;

enum {
    FDGA_OK = 0,
    FDGA_ERR_ARG = 1,        /* invalid dimensions, names or sizes */
    FDGA_ERR_UNSUPPORTED = 2,/* a reference feature this build does not provide */
    FDGA_ERR_CUDA = 3,       /* CUDA runtime / launch error (message has the CUDA text) */
    FDGA_ERR_OOM = 4,        /* device allocation failed */
    FDGA_ERR_NONFINITE = 5,  /* NaN/Inf in an input or state vector */
    FDGA_ERR_STATE = 6       /* call order violated (e.g. iterate before finalize) */
};

/* iterate_solver! strategy (src/solve.jl:10-82): fdPA, scPA; the alternative K1/K2 form
 * (K = (F Π - F0 Π0) U) of :fdPA_new / :scPA_new, local solver only; the one-loop BSEs of
 * :fdPA_1loop, nonlocal solver only (FDGA_ERR_UNSUPPORTED elsewhere, where the reference has no
 * method).  The tangent and adjoint maps cover FDGA_FDPA and FDGA_SCPA. */
enum { FDGA_FDPA = 0, FDGA_SCPA = 1, FDGA_FDPA_NEW = 2, FDGA_SCPA_NEW = 3, FDGA_FDPA_1LOOP = 4 };
/* Arithmetic of the iteration map.  FDGA_FP64: every kernel in FP64 (the plain path, parity
 * with the reference).  FDGA_MIXED: the K3 Bethe-Salpeter contractions (the bulk of the work at
 * large boxes) in FP32 arithmetic with FP32 accumulation; storage, Dyson, bubbles, SDE, residual
 * and mixing stay FP64.  FDGA_MIXED maps are used inside fdga_solve_mixed, whose FP64 residual
 * (iterative refinement) recovers the FP64 fixed point. */
enum { FDGA_FP64 = 0, FDGA_MIXED = 1 };

/* Solver dimensions: the reference constructor arguments
 * ParquetSolver(nK1, nK2, nK3, Gbare, G0, Σ0, F0; mΠν_factor)         (src/ParquetSolver.jl:88-157)
 * NL_ParquetSolver(nK1, nK2, nK3, mK_Γ, Gbare, G0, Σ0, F0; mΠν_factor) (src/nonlocal/ParquetSolver.jl:77-152)
 * with the reference vertex F0 either the RefVertex F0 = RefVertex(U, Fp_p, Fp_x, Ft_p, Ft_x)
 * (src/refvertex.jl:1-35), or (f0_vertex = 1) a Vertex F0 = RefVertex + γp + γt + γa with its own
 * boxes nF0K1, nF0K2, nF0K3 (ParquetSolver{Q, VT, RefVT} with RefVT a Vertex: fdDΓA from a solved
 * vertex, e.g. ParquetSolver(nK1, nK2, nK3, Gbare, S0.G, S0.Σ, S0.F), test/test_siam_fdPA.jl:79-84).
 * The Vertex F0's own reference vertex is the RefVertex of U and nR above; its channels are uploaded
 * with FDGA_IN_F0_VERTEX.  A nonlocal solver's Vertex F0 has the solver's momentum mesh. */
typedef struct fdga_config {
    int32_t nG;          /* Green-function mesh: 2nG fermionic frequencies */
    int32_t nK1;         /* K1 box: 2nK1-1 bosonic frequencies */
    int32_t nK2[2];      /* K2 box (bosonic, fermionic) */
    int32_t nK3[2];      /* K3 box (bosonic, fermionic) */
    int32_t L;           /* vertex momentum mesh L x L (1 for the local solver) */
    int32_t LG;          /* Green-function momentum mesh; must equal L in this build */
    int32_t mPi_factor;  /* bubble fermionic mesh = nK1 * mPi_factor (reference default 6 local, 32 NL) */
    int32_t local;       /* 1: ParquetSolver (local BSE forms), 0: NL_ParquetSolver */
    double T;            /* temperature */
    double U;            /* bare interaction of the RefVertex */
    int32_t nR[2];       /* box of the RefVertex corrections Fp_p .. Ft_x; (1,1) = bare U */
    int32_t precision;   /* FDGA_FP64 or FDGA_MIXED: initial arithmetic of fdga_iterate / fdga_residual */
    int32_t f0_vertex;   /* 0: F0 is the RefVertex; 1: F0 is a Vertex with the boxes below */
    int32_t nF0K1;       /* K1 box of the Vertex F0 */
    int32_t nF0K2[2];    /* K2 box of the Vertex F0 (bosonic, fermionic) */
    int32_t nF0K3[2];    /* K3 box of the Vertex F0 (bosonic, fermionic) */
} fdga_config;

/* Inputs uploaded with fdga_set_input (reference column-major layout). */
enum {
    FDGA_IN_GBARE = 0,   /* [2nG, L*L]          Gbare (stores i*G)                      */
    FDGA_IN_G0 = 1,      /* [2nG, L*L]          G0                                       */
    FDGA_IN_SIGMA0 = 2,  /* [2nG, L*L]          Σ0 (stores i*Σ)                          */
    FDGA_IN_FP_P = 3,    /* [2nR0-1, 2nR1, 2nR1] RefVertex corrections                    */
    FDGA_IN_FP_X = 4,
    FDGA_IN_FT_P = 5,
    FDGA_IN_FT_X = 6,
    FDGA_IN_F0_VERTEX = 7 /* flatten(F0) = [γp(K1,K2,K3), γt, γa] of a Vertex F0 in its own boxes
                           * (flatten of a Vertex, src/vertex.jl:152-165)                      */
};

/* Creates a handle (replaces the reference constructors above; allocates all device state). */
int fdga_create(const fdga_config* cfg, fdga_handle** out);
void fdga_destroy(fdga_handle* h);
const char* fdga_last_error(const fdga_handle* h);
/* Library-level error text for failures that happen before a handle exists. */
const char* fdga_create_error(void);

/* Uploads one input array; n = number of complex elements. */
int fdga_set_input(fdga_handle* h, int which, const double* re_im, size_t n);

/* Constructor tail: Π0 = bubble(G0), Σ = Σ0, G = Dyson(Σ), Π = bubble(G), F = 0
 * (src/ParquetSolver.jl:291-310, src/nonlocal/ParquetSolver.jl:91-110). */
int fdga_finalize(fdga_handle* h);

/* init_sym_grp!(S) (src/ParquetSolver.jl:203-231, src/nonlocal/ParquetSolver.jl:198-300).
 * Without it every element is evaluated directly (the constructor's trivial groups). */
int fdga_init_sym_grp(fdga_handle* h);
/* Host-only (no device needed): the class map of one init_sym_grp! group for a configuration,
 * which = 0 Σ, 1 K1, 2 K2pp, 3 K2ph, 4 K3pp, 5 K3ph, 6 K3ppL, 7 K3phL; map[i] (device index i)
 * = representative*4 + op (bit 0 sign, bit 1 conjugation); n = number of mesh points. */
int fdga_group_map(const fdga_config* cfg, int which, uint32_t* map, size_t n, int* nclasses);

/* Length (complex elements) of flatten(S) = [γp(K1,K2,K3), γt, γa, Σ] (src/ParquetSolver.jl:277-306). */
int fdga_state_len(const fdga_handle* h, size_t* n);
int fdga_flatten(fdga_handle* h, double* x, size_t n);
int fdga_unflatten(fdga_handle* h, const double* x, size_t n);

/* iterate_solver!(S; strategy, update_Σ, compute_Hartree) (src/solve.jl:4-116): one parquet
 * iteration on the device state, replayed as one CUDA graph. */
int fdga_iterate(fdga_handle* h, int strategy, int update_sigma, int compute_hartree);

/* Arithmetic of subsequent fdga_iterate / fdga_residual / fdga_solve calls on this handle. */
int fdga_set_precision(fdga_handle* h, int precision);

/* Integer options: "k3_tensor_cores" (default 1): the mixed map's K3 contractions run on the
 * tensor cores (tcgen05, TF32 hi/lo split, FP32 accumulation) when 2·Nν3 ≤ 256 and Nν3 is a
 * multiple of 8, else as FP32 CUDA-core GEMMs.  "jvp_tangent" (default 1): the GMRES solves of
 * fdga_solve_newton and fdga_dchi_dU apply the Jacobian through the tangent kernels (as
 * fdga_frule); 0: by finite differences of the map.  "newton_gmres_cycles" (default 1): GMRES
 * restart cycles per Newton step of fdga_solve_newton (more for ill-conditioned fixed points).
 * "fused_residual" (default 1): fdga_residual on page-locked x and R runs as one CUDA graph whose
 * host copies overlap the iteration; 0: copy, iterate and copy back in sequence.
 * "k3_fp64_tensor_cores" (default 2): the FP64 map's K3 contractions (BSE_L_K3 and BSE_K3) run on
 * the tensor cores by exact digit slicing of the FP64 operands (8 BF16 digits of 7 bits, products
 * summed by diagonal in FP32 tensor memory, joined exactly; FP64-level results, ~1e-14 relative
 * to the CUDA-core FP64 GEMM) when Nν3 is a multiple of 8 between 8 and 128: 2 from Nν3 = 32 on,
 * 1 at every such Nν3, 0 never (FP64 CUDA-core GEMMs); 3 as 1 with every tile of M bounded from
 * the FP64 exponents of its factors, the path otherwise taken only when its FP32 bound overflows
 * (for tests). */
int fdga_set_option(fdga_handle* h, const char* key, int value);

/* fixed_point!(R, x, S) (src/solve.jl:119-157): unflatten x, iterate, R = flatten(S) - x.
 * x and R are host arrays of fdga_state_len elements.  When both are page-locked (cudaHostAlloc,
 * cudaHostRegister) the copies run inside the iteration's graph, overlapped with it; the graph is
 * kept for the last (x, R, precision, strategy) seen. */
int fdga_residual(fdga_handle* h, int strategy, const double* x, double* R, size_t n);

/* solve!(S; maxiter, tol, δ, mem) (src/solve.jl:160-196): Anderson acceleration (NLsolve
 * method=:anderson, m = mem, beta = δ, ftol = tol on max|R|) run on the device.
 * Returns the iteration count in *iters (negative when not converged), the last max|R| in
 * *res and, if trace != NULL, max|R| per iteration (maxiter doubles). */
int fdga_solve(fdga_handle* h, int strategy, int maxiter, double tol, double beta, int mem,
               int* iters, double* res, double* trace);

/* Mixed-precision solve of the same fixed point as fdga_solve, by iterative refinement (defect
 * correction).  Phase 1: at each outer iterate x the FP64 residual Φ64(x) - x is formed; the inner
 * equation z = Φ_mixed(z) + (Φ64(x) - Φ_mixed(x)) is solved from z = x by Anderson acceleration
 * (m = mem, beta) with an FP32 history until its residual falls below max(1e-3 max|Φ64(x) - x|,
 * tol/4) or stops improving (the rounding floor of the mixed map), and z becomes the next outer
 * iterate.  Phase 2 starts when an outer step reduced the FP64 residual by less than 10x: the
 * same FP32-history Anderson iteration then runs on the FP64 map until max|R| < tol.  The fixed
 * point is the FP64 one; convergence is declared on FP64 residuals only.  maxiter bounds the map
 * evaluations of both precisions together.  *iters = number of FP64 residuals formed (negative
 * when not converged); *res = the last one; trace (maxiter doubles, may be NULL) = the FP64
 * residuals in order; evals[0] = FP64 map evaluations, evals[1] = mixed map evaluations.  On
 * return S holds Φ64 of the last iterate. */
int fdga_solve_mixed(fdga_handle* h, int strategy, int maxiter, double tol, double beta, int mem,
                     int* iters, double* res, double* trace, int* evals);

/* Newton–Krylov solve of the fixed point x = Φ(x): Newton steps (I − J) dx = Φ(x) − x solved by
 * one GMRES(restart) cycle to an Eisenstat–Walker forcing tolerance, then a backtracking line
 * search on the FP64 residual.  J is applied as forward differences of the map in jvp_precision
 * (FDGA_FP64, or FDGA_MIXED for the FP32-contraction map, which gives way to FP64 JVPs once a
 * Newton step gains less than 2x: its rounding floor); the state is real-linear, so GMRES
 * runs on it as a real vector (Krylov basis in FP32, Hessenberg and iterate in FP64).
 * Convergence is tested on the FP64 residual.  Outputs as fdga_solve_mixed (*iters = Newton
 * residual evaluations). */
int fdga_solve_newton(fdga_handle* h, int strategy, int maxiter, double tol, int restart, int jvp_precision,
                      int* iters, double* res, double* trace, int* evals);

/* mfRGLinearMap(S, strategy) * x (src/mfRG.jl:20-89), nonlocal solver: y = x - Φ_mfRG(x f)/f with
 * f = 1e-2, where Φ_mfRG is the BSE sequence of the iteration on the vertex x f with the
 * reference system's bubble Π0 in every BSE and F0 in the right factors (the is_mfRG branches;
 * the caches of the two-argument build_K3_cache_mfRG!, src/nonlocal_2/build_K3_cache.jl:97-165).
 * x and y are host arrays of length(S.F) = the vertex part of flatten(S).  Strategies :fdPA and
 * :fdPA_1loop (the same map); :fdPA_new and the local solver return FDGA_ERR_UNSUPPORTED.  The
 * map depends on F0, Π0 and x only; it overwrites the handle's caches and FL (the next iteration
 * recomputes them) and leaves the state S unchanged. */
int fdga_mfrg_apply(fdga_handle* h, int strategy, const double* x, double* y, size_t n);

/* fixed_point_preconditioned!(R, x, S; strategy, update_Σ) (src/mfRG.jl:93-173): unflatten x
 * (flatten(S) when update_sigma, else flatten(S.F) with Σ kept), symmetrize, iterate, then
 * R_F = flatten(S.F) - x[1:length(S.F)] preconditioned by the mfRG map: R[1:length(S.F)] = z with
 * M z = R_F solved by restarted GMRES(min(64, krylov_maxiter)) on the device, real arithmetic on
 * the symmetry-class representatives, stopping at ‖M z - R_F‖ <= krylov_atol + krylov_rtol ‖R_F‖
 * or after krylov_maxiter map applications (the reference: Krylov.dqgmres with atol = rtol = 1e-6,
 * itmax = 400); R[length(S.F)+1:end] = flatten(S.Σ) - x_Σ when update_sigma.  *krylov_iters and
 * *krylov_res (may be NULL) receive the GMRES iterations and its final relative residual
 * estimate.  On return S holds Φ(x). */
int fdga_residual_mfrg(fdga_handle* h, int strategy, const double* x, double* R, size_t n, int update_sigma,
                       int krylov_maxiter, double krylov_rtol, double krylov_atol, int* krylov_iters,
                       double* krylov_res);

/* solve_using_mfRG_without_mixing!(S; tol, strategy, update_Σ, maxiter, memory, mixing,
 * krylov_maxiter) (src/mfRG.jl:686-776): nlsolve(fixed_point_preconditioned!, x0; method = :anderson,
 * beta = mixing, m = memory, ftol = tol) on the device: Anderson acceleration of
 * the preconditioned residual, starting from the current state S.  Outputs as fdga_solve;
 * *krylov_total (may be NULL) = GMRES iterations over the solve.  On return S holds the last
 * evaluated x, symmetrized (unflatten!(S, res.zero); symmetrize_solver!(S), src/mfRG.jl:764-771). */
int fdga_solve_mfrg(fdga_handle* h, int strategy, int maxiter, double tol, double beta, int mem, int update_sigma,
                    int krylov_maxiter, double krylov_rtol, double krylov_atol, int* iters, double* res,
                    double* trace, int* krylov_total);

/* Jacobian-vector product of the iteration map at the current state S: Jv = dΦ/dx · v, central
 * differences with step 1e-5 (1 + ‖x‖₂) along v/‖v‖₂, in the handle's precision.  v and Jv are
 * host arrays in the flatten(S) layout; J is real-linear (v and i·v give unrelated products). */
int fdga_jvp(fdga_handle* h, int strategy, const double* v, double* Jv, size_t n);

/* Forward-mode derivative of one iteration (the frule of fixed_point!, src/solve.jl:4-116 and
 * src/ParquetSolver.jl:277-306): at the current state S = x, y = Φ(x) and Jv = Φ'(x)·v, the
 * derivative computed by the hand-written tangent kernels (product rule through Dyson, the
 * bubbles, the caches, the K1/K2/K3 BSEs and the SDE; no finite differences), in the handle's
 * precision.  update_sigma and compute_hartree select the map as in fdga_iterate.  v, y and Jv
 * are host arrays in the flatten(S) layout (y may be NULL); S is left unchanged.  J is
 * real-linear. */
int fdga_frule(fdga_handle* h, int strategy, int update_sigma, int compute_hartree, const double* v, double* y,
               double* Jv, size_t n);

/* Reverse-mode derivative of one iteration (the rrule): at the current state S = x, y = Φ(x) and
 * x̄ = Φ'(x)ᵀ ȳ, the transpose for the real inner product <a, b> = Re Σ conj(a) b, so that
 * <ȳ, Φ'(x) v> = <x̄, v> for every v.  Computed by the hand-written adjoint kernels in FP64 (the
 * vertex gathers transposed into scatter-adds, the K3 BSE into two batched GEMMs, the bubbles from
 * G(R) recomputed by the value pass).  Arrays as in fdga_frule (y may be NULL). */
int fdga_rrule(fdga_handle* h, int strategy, int update_sigma, int compute_hartree, const double* ybar, double* y,
               double* xbar, size_t n);

/* Dyson!(S) and bubbles!(S) (src/dyson.jl:5-31, src/bubble.jl) of the current state: G from Σ
 * and Gbare, then the bubbles and their row sums. */
int fdga_dyson_bubbles(fdga_handle* h);

/* interpolate_solver!(So, Si) (src/interpolate.jl:147-191) for two nonlocal solvers of equal
 * temperature: Σ of Si Fourier-interpolated to So's lattice (frequencies clamped to Si's mesh),
 * Dyson and bubbles of So, K1/K2/K3 of the three channels interpolated per frequency point (zero
 * outside Si's boxes), then symmetrize_solver!(So).  The occ_target / μ update of the reference
 * is the caller's: set Gbare and call fdga_dyson_bubbles. */
int fdga_interpolate_solver(fdga_handle* so, fdga_handle* si);

/* Bare interaction U of the handle (the RefVertex's bare part, the SDE and Hartree terms); the
 * reference builds a new solver for another U.  Drops the captured graphs. */
int fdga_set_U(fdga_handle* h, double U);

/* Linear response of the susceptibility to U at a converged state S = x*: solves
 * (I − J) dx/dU = ∂Φ/∂U by restarted GMRES (central-difference Jacobian; ∂Φ/∂U by central
 * differences with step hU) and returns dχ/dU(Ω, q) = χ[dx/dU] − (2/U) χ[x*] (χ linear in K1 over
 * U²), n_out = NΩ1·Nq complex, column-major [Ω, q].  *gmres_iters and *relres report the solve. */
int fdga_dchi_dU(fdga_handle* h, int strategy, int channel, double hU, int restart, int cycles, double rtol,
                 double* out, size_t n_out, int* gmres_iters, double* relres);

/* K3 GEMM tile autotuner: times the output-tile variants of both K3 contractions (16/24/32
 * square tiles, and the same row heights with half-width column tiles: codes 116/124/132) on
 * this handle's data, in FP64 and mixed precision, and keeps the fastest.  Size classes
 * (Nν3, local/nonlocal, precision) are tuned once per process and shared by all handles.
 * tiles (4 ints, may be NULL) = {FP64 L_K3, FP64 K3, mixed L_K3, mixed K3}. */
int fdga_autotune(fdga_handle* h, int strategy, int* tiles);

/* Batches of independent solvers (e.g. many impurity models): one CUDA graph launch performs one
 * iteration (iterate_solver!, update_Σ, Hartree) of every member; the members' kernels run
 * concurrently as branches of the graph.  Members must be finalized handles; a handle may belong
 * to one batch at a time and must not be used on its own while a batch call is in flight. */
typedef struct fdga_batch fdga_batch;
int fdga_batch_create(fdga_handle* const* hs, int n, fdga_batch** out);
void fdga_batch_destroy(fdga_batch* b);
const char* fdga_batch_last_error(const fdga_batch* b);
int fdga_batch_iterate(fdga_batch* b, int strategy, int precision);
int fdga_batch_synchronize(fdga_batch* b);
/* Device milliseconds of `iters` batch iterations (CUDA events on the batch stream) and the
 * number of kernels one batch iteration launches. */
int fdga_batch_time(fdga_batch* b, int strategy, int precision, int iters, float* ms, int* kernels);

/* Named device arrays in the reference layout, for inspection and tests:
 * "G", "Sigma", "Gbare", "G0", "Sigma0", "Pipp", "Piph", "Pi0pp", "Pi0ph", "Lpp", "Lph",
 * "F.<p|t|a>.<K1|K2|K3>", "FL.<p|t|a>.<K2|K3>", "cache_<Gpx|F0p|F0a|F0t|Gpp|Ga|Gt|Fp|Fa|Ft>". */
int fdga_get_named(fdga_handle* h, const char* name, double* out, size_t n);
int fdga_named_len(const fdga_handle* h, const char* name, size_t* n);

/* Occupation n = 1/2 + T Im Σ G / Nk of the current G (src/dyson.jl:33-41). */
int fdga_occupation(fdga_handle* h, double* n);

/* Connected two-particle susceptibility of the current state, from the K1 class of the vertex:
 * K1_r = -U² χ_r in the physical spin channels (the reference's TRIQS import,
 * src/utility/load_triqs.jl:67-75,106-114, and the spin algebra src/types.jl:34-66), hence
 *   FDGA_CHI_M: χ_m(Ω,q) =  γa.K1(Ω,q) / U²
 *   FDGA_CHI_D: χ_d(Ω,q) = (γa.K1 - 2 γt.K1)(Ω,q) / U²
 *   FDGA_CHI_S: χ_s(Ω,q) = -2 γp.K1(Ω,q) / U²
 * (χ_d without the disconnected 2n²/T at Ω = 0.)  n = NΩ1·Nq gives χ(Ω,q) in the reference's
 * column-major [Ω, q] layout; n = NΩ1 gives the momentum average χ_loc(Ω) = (1/Nq) Σ_q χ(Ω,q).
 * Computed on the device in FP64. */
#define FDGA_CHI_M 0
#define FDGA_CHI_D 1
#define FDGA_CHI_S 2
int fdga_susceptibility(fdga_handle* h, int channel, double* out, size_t n);

/* Scalar facts of a handle, for benchmarks and tools: "k3_blocks" (the (P, Ω) blocks of the K3
 * mesh that hold class representatives), "k3_block_dim" (2·nK3ν), "state_len", "launches"
 * (kernels per iteration), "precision", "k3_fp64_tensor_cores" (1 when the FP64 map's K3
 * contractions run on the tensor cores); and, with h == NULL allowed, "fp64_gflops": a
 * calibration of the GPU's FP64 FMA throughput (GFLOP/s, one short kernel). */
int fdga_query(fdga_handle* h, const char* key, double* value);

/* Device timing on the handle's stream (CUDA events), for benchmarks. slot in [0, 8). */
int fdga_event_record(fdga_handle* h, int slot);
int fdga_event_elapsed_ms(fdga_handle* h, int slot_a, int slot_b, float* ms);
int fdga_synchronize(fdga_handle* h);
/* Per-stage device time of one eager (non-graph) iteration, averaged over nrep runs; the state
 * advances by nrep iterations.  names receives a comma-separated stage list. */
int fdga_stage_times(fdga_handle* h, int strategy, int nrep, char* names, size_t names_cap, double* ms,
                     int max_stages, int* nstages);
/* The same for the tangent map at the base point and direction of the last fdga_frule call. */
int fdga_tangent_stage_times(fdga_handle* h, int strategy, int nrep, char* names, size_t names_cap, double* ms,
                             int max_stages, int* nstages);
/* Applies the iteration map n times to the unchanged device state x (graph replays, no host
 * synchronisation): the device-resident timing loop of the benchmark. */
int fdga_map_repeat(fdga_handle* h, int strategy, int n);
/* Applies the tangent map n times (graph replays, no host synchronisation) at the base point and
 * direction of the last fdga_frule call (full map): the timing loop of the derivative. */
int fdga_tangent_repeat(fdga_handle* h, int strategy, int n);
/* Benchmark helper: replays the adjoint map's graph n times at the base point and cotangent of the
 * last fdga_rrule (update_sigma = compute_hartree = 1), without a host sync. */
int fdga_adjoint_repeat(fdga_handle* h, int strategy, int n);
/* Writes `bytes` of a device buffer on the handle's stream, evicting the L2 between timed
 * iterations of a benchmark (the buffer is allocated on first use). */
int fdga_flush_l2(fdga_handle* h, size_t bytes);
/* Page-locked host buffers for host<->device copies of state vectors. */
int fdga_host_alloc(size_t bytes, void** p);
int fdga_host_free(void* p);
/* Number of kernel launches made by the last fdga_iterate (graph nodes). */
int fdga_launches_per_iteration(const fdga_handle* h, int* n);

/* ---- Allocation-free bubble (no counterpart in the reference) ----------------------------
 * For callers that cannot call cudaMalloc: a host whose own pool allocator owns the device
 * memory (for example a Julia CUDA.jl or PyTorch process), or code on a path where cudaMalloc's
 * implicit device synchronisation is not allowed.  The caller passes DEVICE pointers:
 *   G     [2nG, L*L] complex (i*G, column-major [ν, k]),
 *   Pipp, Piph  [2nK1-1, 2nK1*mPi_factor, L*L] complex outputs (column-major [Ω, ν, P]),
 * and cfg supplies nG, nK1, mPi_factor, L (= LG), T, local.  The result equals the bubbles that
 * fdga_finalize computes for G0 (src/nonlocal/bubble.jl:87-158, src/bubble.jl:9-36).
 * No device or host memory is allocated: the work array G(R) lives in one file-scope __device__
 * buffer of FDGA_BUBBLE_NOALLOC_MAX_ELEMS complex values (2 MiB), which every GPU that loads the
 * library holds until the process exits.  Larger problems (2nG*L*L above the maximum, or L > 56,
 * the largest lattice whose bubble tile fits the shared memory) are rejected with FDGA_ERR_ARG and
 * a message in fdga_last_error(NULL), before any device work.
 * The first call on a device looks up the buffer's device address (cudaGetSymbolAddress with that
 * device current) and raises the kernel's shared-memory limit there; make that first call before
 * any stream capture.
 * Work is enqueued on `stream` (a cudaStream_t; NULL = default stream) and the call returns
 * without synchronising.  The buffer is per device: all calls on one device share it and it keeps
 * the last call's contents, so calls on the same device whose kernels overlap on the GPU (different
 * streams or threads without ordering) race on it: serialise them.  Calls on different devices do
 * not share it. */
#define FDGA_BUBBLE_NOALLOC_MAX_ELEMS 131072
int fdga_bubble_noalloc(const fdga_config* cfg, const double* G, double* Pipp, double* Piph, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FDGA_H */
