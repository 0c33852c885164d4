// fdga_runtime.cu -- host runtime of libfdga: handle, device state, symmetry groups, the
// per-iteration launch sequence (captured once into a CUDA graph), the Anderson driver and the
// C ABI declared in include/fdga.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <type_traits>
#include <vector>

#include "../../include/fdga.h"
#include "fdga_kernels.h"

using namespace fdga;

namespace {

thread_local std::string g_create_error;

enum ArrKind { AK_G = 0, AK_K1, AK_K2, AK_K3, AK_PI };

struct Group {
    bool trivial = true;
    int* d_items = nullptr;       // representative device indices, ascending
    int nitems = 0;
    int* d_gstart = nullptr;      // K2 groups: start of each (P, Ω) row of items, plus the end
    int ngroups = 0;
    uint32_t* d_map = nullptr;    // per device index: rep*4 + op
    size_t n = 0;
};

struct Graph {
    cudaGraphExec_t exec = nullptr;
    int nodes = 0;
};

}  // namespace

namespace fdga_internal {
void set_create_error(const std::string& msg) { g_create_error = msg; }
}  // namespace fdga_internal

struct fdga_handle {
    fdga_config cfg{};
    Dims d{};
    cudaStream_t st = nullptr;
    std::string err;
    bool finalized = false;
    bool c0_dirty = true;
    bool ref_nonzero = false;
    size_t nGk = 0, n1 = 0, n2 = 0, n3 = 0, nPi = 0, nRef = 0, nchan = 0, nstate = 0;
    // device state
    cplx *Gbare = nullptr, *G0 = nullptr, *Sig0 = nullptr, *G = nullptr;
    cplx *Pi0pp = nullptr, *Pi0ph = nullptr, *Pipp = nullptr, *Piph = nullptr;
    cplx *Fref[4] = {nullptr, nullptr, nullptr, nullptr};  // Fp_p Fp_x Ft_p Ft_x
    cplx *xS = nullptr, *yS = nullptr, *tmpS = nullptr;
    cplx *avg = nullptr, *cache = nullptr, *FLK2 = nullptr, *FLK3 = nullptr;
    cplxf *cachef = nullptr, *FLK3f = nullptr;  // FP32 caches and FL.K3 of the mixed map
    cplxf *xSf = nullptr, *ySf = nullptr, *avgf = nullptr, *FLK2f = nullptr;  // FP32 mirrors (mixed map)
    cplxf* Freff[4] = {nullptr, nullptr, nullptr, nullptr};
    cplxf* GRf = nullptr;  // FP32 copy of G(R) (mixed map)
    cplx* T0tail = nullptr;  // tail·tail part of the R = 0 bubble row sums [2][NΠΩ]
    // Vertex-valued reference vertex F0 (cfg.f0_vertex): its channels [p|t|a] x [K1|K2|K3] in the
    // device layout of its own boxes b0, their momentum averages, and FP32 copies for the mixed map
    bool has0 = false;
    Box b0{};
    size_t n0_1 = 0, n0_2 = 0, n0_3 = 0, n0chan = 0, n0avg = 0;
    cplx *F0v = nullptr, *F0avg = nullptr;
    cplxf *F0vf = nullptr, *F0avgf = nullptr;
    int fdpa_single_hartree = 0;  // option: subtract the reference system's Hartree term once
    size_t navg = 0;
    int* d_err = nullptr;                        // device error flag of bounded in-kernel waits
    int* oz_fa = nullptr;                        // per-block exponent bounds of the digit-sliced K3 (3 Nq NΩ3)
    uint8_t* oz_adig = nullptr;                  // A digit operands of oz_adig_blocks blocks (at most 512 MB)
    int oz_adig_blocks = 0;
    int k3_tc = 1;                               // mixed K3 contractions on the tensor cores when supported
    int k3_tma = 1;                              // ... in the TMA-fed warp-specialised kernel when it fits
    // FP64 K3 contractions on the tensor cores (exact digit slicing): 0 never, 1 where supported, 2 from
    // Nν3 = 32 on, 3 as 1 with the FP64 exponent bound of M in every tile (tests)
    int k3_oz = 2;
    int jvp_tangent = 1;                         // GMRES Jacobian products by the tangent kernels (else differences)
    int newton_cycles = 1;                       // GMRES restart cycles per Newton step
    cplx *Lpp = nullptr, *Lph = nullptr, *SigIn = nullptr, *SigU2 = nullptr, *C0 = nullptr;
    cplx *GR = nullptr, *u2C = nullptr, *u2R = nullptr, *twm = nullptr, *twp = nullptr;
    cplx *SPi = nullptr, *SPi0 = nullptr, *SX = nullptr;  // bubble row sums [2][Nq][NΠΩ]; S_X [3][Nq][NΠΩ]
    cplx* SRtmp = nullptr;                                 // real-space row sums [2][L*L][NΠΩ]
    cplx* LR = nullptr;                                    // L_pp, L_ph in real space [2][R][Ω][ν]
    cplx* SigR = nullptr;                                  // Σ in real space [R][ν]
    cplx *raw1 = nullptr, *raw2 = nullptr, *raw3 = nullptr;  // representative values [3 ch][K1|K2|K3]
    int* d_k3blocks = nullptr;                             // (P, Ω) blocks holding K3 class representatives
    void* flush_buf = nullptr;                             // L2 flush buffer (benchmarks)
    size_t flush_bytes = 0;
    unsigned char flush_val = 0;
    int nk3blocks = 0;
    double* occ = nullptr;
    double n0 = 0.5;
    uint32_t* perm = nullptr;  // reference flatten index -> device index
    Group gSig, gK1, gK2pp, gK2ph, gK3pp, gK3ph, gK3ppL, gK3phL;
    Graph graphs[2][5][2][2];  // [precision][strategy][update_sigma][hartree]
    // fdga_residual on page-locked host buffers: one graph with the copies inside (see residual_graph)
    struct {
        Graph g;
        const void* x = nullptr;
        void* R = nullptr;
        int precision = -1, strategy = -1;
    } rg;
    cplx* FLzero = nullptr;    // zero FL.K2 (the one-loop BSEs of :fdPA_1loop have no FL factor)
    cplxf* FLzerof = nullptr;
    int precision = FDGA_FP64;
    int fused_residual = 1;  // option "fused_residual": fdga_residual on page-locked buffers as one graph
    int k3_tile[2][2] = {{0, 0}, {0, 0}};  // [precision][mode]: K3 GEMM tile chosen by fdga_autotune (0: default)
    int last_launches = 0;
    cudaEvent_t ev[8] = {};
    cudaStream_t st2 = nullptr, st3 = nullptr;                         // branch streams of the iteration
    cudaEvent_t evfork = nullptr, evA = nullptr, evB = nullptr, evC = nullptr, evD = nullptr, evE = nullptr,
                evR = nullptr;
    // Anderson
    std::vector<cplx*> aa_buf;
    double* d_part = nullptr;
    cplx *aa_R = nullptr, *aa_rot = nullptr, *aa_gam = nullptr, *aa_part = nullptr;  // device QR state
    std::vector<cplx*> kr64;       // Newton-Krylov / linear response, compact (one value per class) FP64
    std::vector<cplxf*> kr32;      // Krylov basis V[0..m], w, scratch: compact FP32
    size_t kr_nc = 0;              // compact length the kr buffers were sized for
    cplx* kr_x = nullptr;          // full FP64 Newton iterate / fixed point
    std::vector<cplx*> jv;         // fdga_jvp work vectors (full FP64)
    double *kr_part = nullptr, *kr_coef = nullptr;
    // device-resident GMRES cycles: the cycle state (device, and a page-locked host copy read once per
    // cycle) and one instantiated WHILE-node graph per (operator, restart length)
    KrDevState* kr_st = nullptr;
    KrDevState* kr_st_host = nullptr;
    std::map<std::pair<int, int>, Graph> kr_graphs;
    int kr_device_loop = 1;  // option "gmres_device_loop"
    uint32_t *kc_code = nullptr, *kc_pos = nullptr;  // compact index of the state (symmetry classes)
    float* kc_w = nullptr;                           // class sizes
    size_t nc = 0;
    int groups_version = 0, kc_version = -1;
    std::vector<cplx*> ma_buf64;   // mixed solver: defect, g, g_old
    std::vector<cplxf*> ma_buf32;  // mixed solver: f, Δf, Q, Δg (FP32 history)
    // Tangent map (forward-mode derivative of one iteration): direction x, result y (state layout)
    // and the tangent intermediates; the value intermediates of the base point are the ones above.
    struct Tangent {
        cplx *x = nullptr, *y = nullptr, *avg = nullptr, *G = nullptr, *GR = nullptr;
        cplx *Pipp = nullptr, *Piph = nullptr, *SPi = nullptr, *SX = nullptr;
        cplx *cache = nullptr;  // 7 caches (Γpx Γpp Γa Γt Fp Fa Ft): the RefVertex caches have no tangent
        cplx *FLK2 = nullptr, *FLK3 = nullptr, *Lpp = nullptr, *Lph = nullptr, *LR = nullptr, *SR = nullptr;
        cplx *SigIn = nullptr, *u2C = nullptr, *u2R = nullptr, *SigU2 = nullptr;
        double* occ = nullptr;
        cplxf *cachef = nullptr, *FLK2f = nullptr, *FLK3f = nullptr, *xSf = nullptr, *ySf = nullptr;
        cplxf *avgf = nullptr, *GRf = nullptr;  // FP32 forms (tangent of the mixed map)
        Graph graphs[2][2][2][2];               // [precision][strategy][update_sigma][hartree]
    } tan;
    // Adjoint map (reverse-mode derivative of one FP64 iteration): cotangents x̄ (result) and ȳ (input,
    // plus the SDE's contributions to the new vertex), and the cotangent intermediates
    struct Adjoint {
        cplx *xb = nullptr, *yb = nullptr, *avgb = nullptr, *Gb = nullptr, *GRb = nullptr;
        cplx *Pbpp = nullptr, *Pbph = nullptr, *PbRpp = nullptr, *PbRph = nullptr, *SPib = nullptr, *SRb = nullptr;
        cplx *SXb = nullptr, *cacheb = nullptr, *FLK2b = nullptr, *FLK3b = nullptr;
        cplx *raw1 = nullptr, *raw2 = nullptr, *raw3 = nullptr, *M = nullptr, *Mb = nullptr;
        cplx *SigInb = nullptr, *SU2b = nullptr, *SigRb = nullptr, *u2Rb = nullptr, *u2Cb = nullptr;
        cplx *LRb = nullptr, *Lb = nullptr;
        double* nbar = nullptr;
        Graph graphs[2][2][2];  // [strategy][update_sigma][hartree] (FP64)
    } adj;
    // mfRG linear map (src/mfRG.jl:20-89): its scaled input vertex x·factor, its output Φ_mfRG and a
    // work vector (state layout; the Σ parts stay zero), one captured graph per precision
    struct Mfrg {
        cplx *x = nullptr, *y = nullptr, *u = nullptr;
        Graph graphs[2];
    } mf;
    size_t nc_sig = 0;  // offset of Σ's classes in the compact (one value per class) state
    std::vector<void*> allocs;
};

namespace {

const int NBLK_RED = 296;

int fail(fdga_handle* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    return code;
}
int cuda_fail(fdga_handle* h, cudaError_t e, const char* where) {
    return fail(h, FDGA_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
#define CK(call)                                                        \
    do {                                                                \
        cudaError_t e__ = (call);                                       \
        if (e__ != cudaSuccess) return cuda_fail(h, e__, #call);        \
    } while (0)

template <class T>
int dalloc(fdga_handle* h, T** p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) return fail(h, FDGA_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    h->allocs.push_back((void*)*p);
    return cudaMemsetAsync(*p, 0, n * sizeof(T), h->st) == cudaSuccess ? FDGA_OK : FDGA_ERR_CUDA;
}
#define AL(ptr, n)                                           \
    do {                                                     \
        int r__ = dalloc(h, &(ptr), (n));                    \
        if (r__) return r__;                                 \
    } while (0)

// the FP32 caches and FL.K3 copy of the mixed map (zero-filled), allocated on first use
int ensure_mixed(fdga_handle* h) {
    if (h->cachef) return FDGA_OK;
    AL(h->cachef, 10 * h->n3);
    AL(h->FLK3f, 3 * h->n3);
    AL(h->FLK2f, 3 * h->n2);
    AL(h->GRf, h->nGk);
    AL(h->xSf, 3 * h->nchan);
    AL(h->ySf, 3 * h->nchan);
    if (h->navg) AL(h->avgf, h->navg);
    for (auto& f : h->Freff) AL(f, h->nRef);
    if (h->has0) {
        AL(h->F0vf, 3 * h->n0chan);
        if (h->n0avg) AL(h->F0avgf, h->n0avg);
        CK(launch_to_f32(h->st, h->F0v, h->F0vf, 3 * h->n0chan));
        if (h->n0avg) CK(launch_to_f32(h->st, h->F0avg, h->F0avgf, h->n0avg));
    }
    AL(h->d_err, 1);
    if (k3_tc_supported(h->d)) CK(prepare_bse_K3_tc(h->d));
    CK(prepare_bse_K3_tma(h->d));
    CK(cudaStreamSynchronize(h->st));
    return FDGA_OK;
}
// a tensor-core wait that timed out inside a kernel (bounded polling) is reported here
// scratch of the digit-sliced K3: per-block exponent bounds and a digit buffer for up to 512 MB of
// blocks (larger launches run in groups)
int ensure_k3_oz(fdga_handle* h) {
    const Dims& d = h->d;
    const size_t nblk = 3 * (size_t)d.Nq * d.N3O;
    if (!h->d_err) AL(h->d_err, 1);
    if (!h->oz_fa) AL(h->oz_fa, nblk);
    if (!h->oz_adig) {
        const size_t per = k3_oz_digit_bytes(d);
        const size_t cap = std::max<size_t>(1, std::min(nblk, ((size_t)512 << 20) / per));
        AL(h->oz_adig, cap * per);
        h->oz_adig_blocks = (int)cap;
    }
    return FDGA_OK;
}
int check_device_error(fdga_handle* h) {
    if (!h->d_err) return FDGA_OK;
    int v = 0;
    CK(cudaMemcpyAsync(&v, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (v) {
        CK(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->st));
        return fail(h, FDGA_ERR_CUDA, "a tensor-core wait in the K3 contraction timed out");
    }
    return FDGA_OK;
}

// ---- channel views into a state vector ----
cplx* chanK(const fdga_handle* h, cplx* S, int ch, int cls) {
    cplx* base = S + (size_t)ch * h->nchan;
    return cls == 1 ? base : (cls == 2 ? base + h->n1 : base + h->n1 + h->n2);
}
cplx* sigmaOf(const fdga_handle* h, cplx* S) { return S + 3 * h->nchan; }
// the SDE of :fdPA_new and :fdPA_1loop is the fdPA one (src/SDE.jl:3-33)
bool strategy_fdpa_sde(int strategy) {
    return strategy == FDGA_FDPA || strategy == FDGA_FDPA_NEW || strategy == FDGA_FDPA_1LOOP;
}

// ---- reference column-major index <-> device index ----
size_t dev_index(const Dims& d, int kind, size_t j) {
    switch (kind) {
        case AK_G:
        case AK_K1:
            return j;
        case AK_K2: {
            size_t iO = j % d.N2O; j /= d.N2O;
            size_t in = j % d.N2n; size_t P = j / d.N2n;
            return (P * d.N2O + iO) * d.N2n + in;
        }
        case AK_K3: {
            size_t iO = j % d.N3O; j /= d.N3O;
            size_t a = j % d.N3n; j /= d.N3n;
            size_t b = j % d.N3n; size_t P = j / d.N3n;
            return ((P * d.N3O + iO) * d.N3n + a) * d.N3n + b;
        }
        default: {  // Π [Ω, ν, P]
            size_t iO = j % d.NPO; j /= d.NPO;
            size_t in = j % d.NPn; size_t P = j / d.NPn;
            return (P * d.NPO + iO) * d.NPn + in;
        }
    }
}

int make_dims(const fdga_config* c, Dims& d) {
    d.nG = c->nG; d.NG = 2 * c->nG; d.L = c->L; d.Nq = c->L * c->L; d.Nk = d.Nq;
    d.n1 = c->nK1; d.N1 = 2 * c->nK1 - 1;
    d.n2O = c->nK2[0]; d.N2O = 2 * c->nK2[0] - 1; d.n2n = c->nK2[1]; d.N2n = 2 * c->nK2[1];
    d.n3O = c->nK3[0]; d.N3O = 2 * c->nK3[0] - 1; d.n3n = c->nK3[1]; d.N3n = 2 * c->nK3[1];
    d.nPO = c->nK1; d.NPO = 2 * c->nK1 - 1; d.nPn = c->nK1 * c->mPi_factor; d.NPn = 2 * d.nPn;
    d.nRO = c->nR[0]; d.NRO = 2 * c->nR[0] - 1; d.nRn = c->nR[1]; d.NRn = 2 * c->nR[1];
    // Stored bubble window.  Every bubble frequency read by the nonlocal iteration satisfies
    // |ω| <= nK2Ω + nK2ν + nK1 (K2 windows around -(Ω+ν+1) and Ω-ν-1), <= nK2Ω + nRν (SDE RefVertex
    // window) or <= nK1 + nK2ν (S_X); the local solver's left K2 BSE sums the whole mesh.
    // A Vertex-valued F0 widens every window to the union of its boxes and the solver's.
    d.xn1 = d.n1; d.xn2O = d.n2O; d.xn2n = d.n2n; d.xn3n = d.n3n;
    if (c->f0_vertex) {
        d.xn1 = std::max(d.n1, c->nF0K1);
        d.xn2O = std::max(d.n2O, c->nF0K2[0]);
        d.xn2n = std::max(d.n2n, c->nF0K2[1]);
        d.xn3n = std::max(d.n3n, c->nF0K3[1]);
    }
    d.nPw = c->local ? d.nPn : std::min(d.nPn, d.xn2O + d.xn2n + d.xn1 + c->nR[1] + 2);
    d.NPw = 2 * d.nPw;
    d.local = c->local ? 1 : 0;
    d.T = c->T; d.U = c->U;
    return FDGA_OK;
}
// The solver's dims with the channel boxes of a Vertex-valued F0 (for its index maps and averages).
Dims f0_dims(const Dims& d, const Box& b) {
    Dims e = d;
    e.n1 = b.n1; e.N1 = b.N1; e.n2O = b.n2O; e.N2O = b.N2O; e.n2n = b.n2n; e.N2n = b.N2n;
    e.n3O = b.n3O; e.N3O = b.N3O; e.n3n = b.n3n; e.N3n = b.N3n;
    return e;
}

// ---------------------------------------------------------------------------------------------
// Symmetry classes (MatsubaraFunctions SymmetryGroup semantics): mesh points joined by the
// listed symmetries (images outside the box are dropped) form a class; classes are seeded in
// the reference's linear order, so the representative is the class's first point in that
// order; each member carries the composed Operation (1 = sign, 2 = conjugation).
// Symmetry maps: src/symmetries.jl:2-94 and src/nonlocal/symmetries.jl:4-133.
// ---------------------------------------------------------------------------------------------
struct Pt { int m, n, np, P; };
using SymF = std::function<int(const Pt&, Pt&)>;

struct ShapeDesc {
    int kind;             // AK_G (Σ), AK_K1, AK_K2, AK_K3
    int nO = 0, nf = 0;   // boson / fermion mesh parameters (Σ: nf = nG)
    int Nq = 1;
    size_t size() const {
        size_t s = (size_t)Nq;
        if (kind == AK_G) return s * 2 * nf;
        s *= (size_t)(2 * nO - 1);
        if (kind == AK_K2) s *= 2 * nf;
        if (kind == AK_K3) s *= (size_t)(2 * nf) * (2 * nf);
        return s;
    }
    Pt decode(size_t j) const {  // reference column-major
        Pt p{0, 0, 0, 0};
        if (kind == AK_G) { p.n = (int)(j % (2 * nf)) - nf; p.P = (int)(j / (2 * nf)); return p; }
        const int NO = 2 * nO - 1;
        p.m = (int)(j % NO) - (nO - 1); j /= NO;
        if (kind == AK_K1) { p.P = (int)j; return p; }
        p.n = (int)(j % (2 * nf)) - nf; j /= 2 * nf;
        if (kind == AK_K2) { p.P = (int)j; return p; }
        p.np = (int)(j % (2 * nf)) - nf; p.P = (int)(j / (2 * nf));
        return p;
    }
    bool inb(const Pt& p) const {
        if (kind == AK_G) return fin(p.n, nf);
        if (!bin(p.m, nO)) return false;
        if (kind == AK_K1) return true;
        if (!fin(p.n, nf)) return false;
        return kind == AK_K2 ? true : fin(p.np, nf);
    }
    size_t encode(const Pt& p) const {
        if (kind == AK_G) return (size_t)(p.n + nf) + (size_t)(2 * nf) * p.P;
        const int NO = 2 * nO - 1;
        size_t j = (size_t)(p.m + nO - 1);
        if (kind == AK_K1) return j + (size_t)NO * p.P;
        j += (size_t)NO * (p.n + nf);
        if (kind == AK_K2) return j + (size_t)NO * (2 * nf) * p.P;
        return j + (size_t)NO * (2 * nf) * ((p.np + nf) + (size_t)(2 * nf) * p.P);
    }
};

int pmod(int a, int L) { int r = a % L; return r < 0 ? r + L : r; }
int kneg(int P, int L) { return pmod(-(P % L), L) + L * pmod(-(P / L), L); }
int kref(int P, int L) { return (P / L) + L * (P % L); }
int krot(int P, int L) { return (P / L) + L * pmod(-(P % L), L); }

struct HostGroup {
    std::vector<uint32_t> map;  // device index -> rep*4 + op
    std::vector<int> items;     // representative device indices, sorted
};

void compute_group(const Dims& d, HostGroup& hg, const ShapeDesc& sh, int kind_dev, const std::vector<SymF>& syms) {
    const size_t n = sh.size();
    std::vector<int32_t> cls(n, -1);
    std::vector<uint8_t> op(n, 0);
    std::vector<size_t> rep_of_class;
    // Depth-first with a LIFO work list, symmetries applied in list order: where a cycle of
    // symmetries composes to a non-identity Operation the member's op depends on the traversal,
    // and this is the order of MatsubaraFunctions' class construction (pop! of the unprocessed list).
    std::vector<size_t> q;
    for (size_t s = 0; s < n; ++s) {
        if (cls[s] >= 0) continue;
        const int c = (int)rep_of_class.size();
        rep_of_class.push_back(s);
        cls[s] = c;
        op[s] = 0;
        q.clear();
        q.push_back(s);
        while (!q.empty()) {
            const size_t j = q.back();
            q.pop_back();
            const Pt p = sh.decode(j);
            for (const auto& f : syms) {
                Pt o = p;
                const int o_op = f(p, o);
                if (!sh.inb(o)) continue;
                const size_t k = sh.encode(o);
                if (cls[k] >= 0) continue;
                cls[k] = c;
                op[k] = (uint8_t)(op[j] ^ o_op);
                q.push_back(k);
            }
        }
    }
    hg.map.assign(n, 0);
    hg.items.clear();
    hg.items.reserve(rep_of_class.size());
    for (size_t j = 0; j < n; ++j) {
        const size_t dj = dev_index(d, kind_dev, j);
        const size_t dr = dev_index(d, kind_dev, rep_of_class[cls[j]]);
        hg.map[dj] = (uint32_t)(dr << 2) | op[j];
    }
    for (size_t r : rep_of_class) hg.items.push_back((int)dev_index(d, kind_dev, r));
    std::sort(hg.items.begin(), hg.items.end());
}

// The eight groups of init_sym_grp!, in the order Σ, K1, K2pp, K2ph, K3pp, K3ph, K3ppL, K3phL.
void compute_all_groups(const Dims& d, std::vector<HostGroup>& out) {
    const int L = d.L;
    const bool nl = !d.local;
    auto kn = [nl, L](int P) { return nl ? kneg(P, L) : P; };
    std::vector<SymF> sig = {[kn](const Pt& p, Pt& o) { o.n = -p.n - 1; o.P = kn(p.P); return 3; }};
    std::vector<SymF> k1 = {[kn](const Pt& p, Pt& o) { o.m = -p.m; o.P = kn(p.P); return 2; }};
    SymF k2pp1 = [kn](const Pt& p, Pt& o) { o.m = -p.m; o.n = -p.n - 1; o.P = kn(p.P); return 2; };
    SymF k2pp2 = [](const Pt& p, Pt& o) { o.n = p.m - p.n - 1; return 0; };
    SymF k2ph2 = [kn](const Pt& p, Pt& o) { o.m = -p.m; o.n = p.m + p.n; o.P = kn(p.P); return 0; };
    SymF k3pp1 = [kn](const Pt& p, Pt& o) { o.m = -p.m; o.n = -p.n - 1; o.np = -p.np - 1; o.P = kn(p.P); return 2; };
    SymF k3pp2 = [](const Pt& p, Pt& o) { o.n = p.np; o.np = p.n; return 0; };
    SymF k3pp3 = [](const Pt& p, Pt& o) { o.n = p.m - p.n - 1; o.np = p.m - p.np - 1; return 0; };
    SymF k3ph3 = [kn](const Pt& p, Pt& o) { o.m = -p.m; o.n = p.m + p.n; o.np = p.m + p.np; o.P = kn(p.P); return 0; };
    SymF ref = [L](const Pt& p, Pt& o) { o.P = kref(p.P, L); return 0; };
    SymF rot = [L](const Pt& p, Pt& o) { o.P = krot(p.P, L); return 0; };
    std::vector<SymF> k2pp = {k2pp1, k2pp2}, k2ph = {k2pp1, k2ph2};
    std::vector<SymF> k3pp = {k3pp1, k3pp2, k3pp3}, k3ppL = {k3pp1, k3pp3};
    std::vector<SymF> k3ph = {k3pp1, k3pp2, k3ph3}, k3phL = {k3pp1, k3ph3};
    if (nl) {
        for (auto* v : {&sig, &k1, &k2pp, &k2ph, &k3pp, &k3ppL, &k3ph, &k3phL}) { v->push_back(ref); v->push_back(rot); }
    }
    const ShapeDesc sS{AK_G, 0, d.nG, d.Nk}, s1{AK_K1, d.n1, 0, d.Nq}, s2{AK_K2, d.n2O, d.n2n, d.Nq},
        s3{AK_K3, d.n3O, d.n3n, d.Nq};
    out.assign(8, HostGroup());
    // the eight class constructions are independent: one host thread each
    const ShapeDesc* shp[8] = {&sS, &s1, &s2, &s2, &s3, &s3, &s3, &s3};
    const int kinds[8] = {AK_G, AK_K1, AK_K2, AK_K2, AK_K3, AK_K3, AK_K3, AK_K3};
    const std::vector<SymF>* sy[8] = {&sig, &k1, &k2pp, &k2ph, &k3pp, &k3ph, &k3ppL, &k3phL};
    std::vector<std::thread> th;
    for (int i = 0; i < 8; ++i)
        th.emplace_back([&, i]() { compute_group(d, out[i], *shp[i], kinds[i], *sy[i]); });
    for (auto& t : th) t.join();
}

// row: items with equal index / row form one row (the K2 groups' (P, Ω) rows); 0: no rows
int upload_group(fdga_handle* h, Group& g, const HostGroup& hg, int row = 0) {
    const size_t n = hg.map.size();
    if (!g.d_map) AL(g.d_map, n);
    if (!g.d_items) AL(g.d_items, n);
    CK(cudaMemcpyAsync(g.d_map, hg.map.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(g.d_items, hg.items.data(), hg.items.size() * sizeof(int), cudaMemcpyHostToDevice, h->st));
    std::vector<int> starts;
    if (row > 0) {
        for (size_t i = 0; i < hg.items.size(); ++i)
            if (i == 0 || hg.items[i] / row != hg.items[i - 1] / row) starts.push_back((int)i);
        starts.push_back((int)hg.items.size());
        if (!g.d_gstart) AL(g.d_gstart, n / row + 1);
        CK(cudaMemcpyAsync(g.d_gstart, starts.data(), starts.size() * sizeof(int), cudaMemcpyHostToDevice, h->st));
        g.ngroups = (int)starts.size() - 1;
    }
    CK(cudaStreamSynchronize(h->st));
    g.trivial = false;
    g.nitems = (int)hg.items.size();
    g.n = n;
    return FDGA_OK;
}

// ---------------------------------------------------------------------------------------------
// Launch sequence of one iteration: src/solve.jl:4-116
// ---------------------------------------------------------------------------------------------
// vertex view of a state-layout array (the FP64 state or its FP32 mirror) with its momentum
// averages and RefVertex corrections
template <class S>
VertPT<S> vertex_view_t(const fdga_handle* h, S* st, S* avg, S* const* fref) {
    VertPT<S> F{};
    for (int c = 0; c < 3; ++c) {
        S* base = st + (size_t)c * h->nchan;
        F.g[c].K1 = base;
        F.g[c].K2 = base + h->n1;
        F.g[c].K3 = base + h->n1 + h->n2;
        if (h->d.Nq == 1) {
            F.g[c].A1 = F.g[c].K1; F.g[c].A2 = F.g[c].K2; F.g[c].A3 = F.g[c].K3;
        } else {
            const size_t per1 = h->d.N1, per2 = (size_t)h->d.N2O * h->d.N2n, per3 = (size_t)h->d.N3O * h->d.N3n * h->d.N3n;
            S* a = avg + (size_t)c * (per1 + per2 + per3);
            F.g[c].A1 = a; F.g[c].A2 = a + per1; F.g[c].A3 = a + per1 + per2;
        }
    }
    F.Fp_p = fref[0]; F.Fp_x = fref[1]; F.Ft_p = fref[2]; F.Ft_x = fref[3];
    if (h->has0) {  // the channels of a Vertex-valued F0 (FP64, or their FP32 copies in the mixed map)
        S* f0 = nullptr;
        S* a0 = nullptr;
        if constexpr (std::is_same<S, cplx>::value) { f0 = h->F0v; a0 = h->F0avg; }
        else { f0 = h->F0vf; a0 = h->F0avgf; }
        const Box& b = h->b0;
        for (int c = 0; c < 3; ++c) {
            S* base = f0 + (size_t)c * h->n0chan;
            F.g0[c].K1 = base;
            F.g0[c].K2 = base + h->n0_1;
            F.g0[c].K3 = base + h->n0_1 + h->n0_2;
            if (h->d.Nq == 1) {
                F.g0[c].A1 = F.g0[c].K1; F.g0[c].A2 = F.g0[c].K2; F.g0[c].A3 = F.g0[c].K3;
            } else {
                const size_t per1 = b.N1, per2 = (size_t)b.N2O * b.N2n, per3 = (size_t)b.N3O * b.N3n * b.N3n;
                S* a = a0 + (size_t)c * (per1 + per2 + per3);
                F.g0[c].A1 = a; F.g0[c].A2 = a + per1; F.g0[c].A3 = a + per1 + per2;
            }
        }
        F.b0 = b;
        F.has0 = 1;
    }
    return F;
}
VertP vertex_view(fdga_handle* h, cplx* S) { return vertex_view_t<cplx>(h, S, h->avg, h->Fref); }

const Group& k2group(fdga_handle* h, int ch) { return ch == CH_P ? h->gK2pp : h->gK2ph; }
// the (P, Ω) rows of the K2 work of channel ch (the K2 BSE kernel runs one CTA per row)
void k2_rows(const fdga_handle* h, const Group& g, ChanWork& cw, int ch) {
    cw.gstart[ch] = g.trivial ? nullptr : g.d_gstart;
    cw.ngroups[ch] = g.trivial ? h->d.Nq * h->d.N2O : g.ngroups;
}

#define LC(call)                                                     \
    do {                                                             \
        cudaError_t e__ = (call);                                    \
        if (e__ != cudaSuccess) return cuda_fail(h, e__, #call);     \
        ++nl;                                                        \
    } while (0)

// L_pp and L_ph (vertex part and/or RefVertex part / 3) at the K2-group representatives, then the
// SymmetryGroup broadcast into h->Lpp, h->Lph.
template <class V>
cudaError_t sde_L_pair(fdga_handle* h, const V& F, const BubbleP& B, const cplx* SPi, int use_vertex, double rs,
                       int& nl) {
    const Dims& d = h->d;
    const size_t nS = (size_t)d.Nq * d.NPO;
    ChanWork cw{};
    const Group* g[2] = {&h->gK2pp, &h->gK2ph};
    for (int w = 0; w < 2; ++w) {
        cw.items[w] = g[w]->trivial ? nullptr : g[w]->d_items;
        cw.nitems[w] = g[w]->trivial ? (int)h->n2 : g[w]->nitems;
        cw.out[w] = h->raw2 + (size_t)w * h->n2;
    }
    cudaError_t e = launch_sde_L_all(h->st, F, B, SPi, SPi + nS, cw, use_vertex, rs, d);
    if (e != cudaSuccess) return e;
    ++nl;
    Finalize3 f{};
    f.raw[0] = h->raw2; f.out[0] = h->Lpp; f.map[0] = g[0]->trivial ? nullptr : g[0]->d_map;
    f.raw[2] = h->raw2 + h->n2; f.out[2] = h->Lph; f.map[2] = g[1]->trivial ? nullptr : g[1]->d_map;
    e = launch_finalize3(h->st, f, 0, 0, h->n2);
    if (e == cudaSuccess) ++nl;
    return e;
}

// The mixed map's K3 contraction on the tensor cores: the TMA-fed kernel when it fits the mode and
// the box, else the staging kernel of fdga_k3_tc.cu.  False: neither applies (FP32 CUDA-core GEMM).
bool k3_tensor_cores(const fdga_handle* h, int mode) {
    return h->k3_tc && ((h->k3_tma && k3_tma_supported(h->d, mode)) || k3_tc_supported(h->d));
}
cudaError_t launch_k3_tensor_cores(fdga_handle* h, cudaStream_t s, int mode, const K3Args3F& a3f) {
    if (h->k3_tma && k3_tma_supported(h->d, mode)) {
        TmaBuffers b{};
        b.base[0] = h->cachef; b.ncplx[0] = 10 * h->n3;
        b.base[1] = h->FLK3f; b.ncplx[1] = 3 * h->n3;
        b.base[2] = h->tan.cachef; b.ncplx[2] = h->tan.cachef ? 7 * h->n3 : 0;
        b.base[3] = h->tan.FLK3f; b.ncplx[3] = h->tan.FLK3f ? 3 * h->n3 : 0;
        return launch_bse_K3_tma(s, mode, a3f, 3, h->d, h->d_err, b);
    }
    return launch_bse_K3_tc(s, mode, a3f, 3, h->d, h->d_err);
}

// The FP64 map's K3 contraction: on the tensor cores by exact BF16 digit slicing when the option is
// on and the box fits (fdga_k3_oz.cu), else the FP64 CUDA-core GEMM.
// the FP64 K3 contractions (modes 0, 1 and the tangent's mode 2) on the tensor cores: where the
// digit-sliced kernel supports the box, and by default from Nν3 = 32 on (below, the CUDA-core
// kernel is as fast)
bool use_k3_oz(const fdga_handle* h) {
    if (!h->d_err || !h->oz_fa || !h->oz_adig || !k3_oz_supported(h->d)) return false;
    return h->k3_oz == 1 || h->k3_oz == 3 || (h->k3_oz == 2 && h->d.N3n >= 32);
}
cudaError_t launch_k3_fp64(fdga_handle* h, cudaStream_t s, int mode, const K3Args3& a3) {
    bool oneloop = false;
    for (int i = 0; i < 3; ++i) oneloop |= (a3.a[i].flags & K3F_1LOOP) != 0;
    if (use_k3_oz(h) && (mode <= 1 || !oneloop)) return launch_bse_K3_oz(s, mode, a3, 3, h->d, h->d_err, h->oz_fa, h->oz_adig, h->oz_adig_blocks,
                                                                h->k3_oz == 3);
    return launch_bse_K3(s, mode, a3, 3, h->d, 0, h->k3_tile[FDGA_FP64][mode < 2 ? mode : 1]);
}

using StageHook = std::function<void(const char*)>;
// enqueued on the main stream of a captured iteration: right after branch B (which needs only Σ)
// has forked, and right after the new vertex is complete (before the SDE)
struct IterHooks {
    std::function<int()> after_fork, vertex_done;
};

int enqueue_iteration(fdga_handle* h, int strategy, bool update_sigma, bool hartree, int& nl,
                      const StageHook& mark = StageHook(), const IterHooks* hooks = nullptr) {
    cudaStream_t s = h->st;
    auto stage = [&](const char* name) { if (mark) mark(name); };
    const Dims& d = h->d;
    nl = 0;
    VertP F = vertex_view(h, h->xS);
    VertP Fn = vertex_view(h, h->yS);  // Fbuff, i.e. the new F used by the SDE
    // Independent parts run as concurrent branches (graph capture and batches; sequential when the
    // stages are timed): B = Dyson + bubbles + row sums, C = left K2 BSE, main = momentum averages,
    // caches and left K3 BSE; both branches join the main stream before the right BSEs.
    const bool conc = !mark;
    cudaStream_t sB = conc ? h->st2 : s, sC = conc ? h->st3 : s;
    if (conc) {
        CK(cudaEventRecord(h->evfork, s));
        CK(cudaStreamWaitEvent(sB, h->evfork, 0));
    }
    if (hooks && hooks->after_fork) {
        int r = hooks->after_fork();
        if (r) return r;
    }
    // momentum averages of F (kSW evaluation)
    if (d.Nq > 1) {
        ChanArrays in;
        ChanArraysW out;
        for (int c = 0; c < 3; ++c) {
            in.K1[c] = F.g[c].K1; in.K2[c] = F.g[c].K2; in.K3[c] = F.g[c].K3;
            out.K1[c] = (cplx*)F.g[c].A1; out.K2[c] = (cplx*)F.g[c].A2; out.K3[c] = (cplx*)F.g[c].A3;
        }
        LC(launch_qavg(s, in, out, d));
        stage("qavg");
    }
    if (update_sigma) {
        LC(launch_dyson(sB, h->G, sigmaOf(h, h->xS), h->Gbare, h->nGk));
        LC(launch_g_realspace(sB, h->G, h->GR, h->twm, d));
        if (h->precision == FDGA_MIXED && bubble_f32_supported(d)) {
            // mixed map: bubble and its full-mesh row sums in FP32 from an FP32 copy of G(R)
            LC(launch_to_f32(sB, h->GR, h->GRf, h->nGk));
            LC(launch_bubble_f32(sB, h->GRf, h->Pipp, h->Piph, h->twp, d));
            LC(launch_rowsum(sB, h->Pipp, h->Piph, h->GR, h->SRtmp, h->twp, h->SPi, h->SPi + (size_t)d.Nq * d.NPO, d,
                             h->T0tail, h->GRf));
        } else {
            LC(launch_bubble(sB, h->G, h->GR, h->Pipp, h->Piph, h->twp, d));
            LC(launch_rowsum(sB, h->Pipp, h->Piph, h->GR, h->SRtmp, h->twp, h->SPi, h->SPi + (size_t)d.Nq * d.NPO, d,
                             h->T0tail));
        }
        // the SDE's U² term and the occupation need only G: also on branch B
        LC(launch_u2(sB, h->GR, h->u2C, h->u2R, h->SigU2, h->twp, d));
        nl += 2;
        LC(launch_occupation(sB, h->G, h->nGk, d.T, d.Nk, h->occ));
        stage("dyson_bubble");
    }
    if (conc) CK(cudaEventRecord(h->evB, sB));
    // The mixed map evaluates vertices from an FP32 mirror of the state (converted once per
    // iteration) and keeps the caches, FL.K2 and FL.K3 in FP32: written once, read by the BSEs.
    const bool mixed = h->precision == FDGA_MIXED;
    if (mixed && (!h->cachef || !h->FLK3f || !h->xSf)) return fail(h, FDGA_ERR_STATE, "mixed-precision buffers missing");
    VertPF Ff{}, Fnf{};
    FLPF FLf{};
    if (mixed) {
        LC(launch_to_f32(s, h->xS, h->xSf, 3 * h->nchan));
        if (d.Nq > 1) LC(launch_to_f32(s, h->avg, h->avgf, h->navg));
        for (int i = 0; i < 4; ++i) LC(launch_to_f32(s, h->Fref[i], h->Freff[i], h->nRef));
        Ff = vertex_view_t<cplxf>(h, h->xSf, h->avgf, h->Freff);
        Fnf = vertex_view_t<cplxf>(h, h->ySf, h->avgf, h->Freff);
        for (int c = 0; c < 3; ++c) FLf.K2[c] = h->FLK2f + (size_t)c * h->n2;
    }
    Caches C{};
    for (int i = 0; i < 10; ++i) {
        C.c[i] = h->cache + (size_t)i * h->n3;
        C.f[i] = mixed ? h->cachef + (size_t)i * h->n3 : nullptr;
    }
    if (mixed) LC(launch_build_cache(s, Ff, C, h->d_k3blocks, h->nk3blocks, d));
    else LC(launch_build_cache(s, F, C, h->d_k3blocks, h->nk3blocks, d));
    // strategies that compute FL.K3 (:fdPA, :fdPA_new) write its FP32 copy in the finalize
    const bool left_K3 = strategy == FDGA_FDPA || strategy == FDGA_FDPA_NEW;
    const bool is_new = strategy == FDGA_FDPA_NEW || strategy == FDGA_SCPA_NEW;
    const bool oneloop = strategy == FDGA_FDPA_1LOOP;
    if (mixed && !left_K3) LC(launch_to_f32(s, h->FLK3, h->FLK3f, 3 * h->n3));
    stage("k3_cache");
    FLP FL;
    for (int c = 0; c < 3; ++c) FL.K2[c] = h->FLK2 + (size_t)c * h->n2;
    const int order[3] = {CH_P, CH_A, CH_T};
    BubbleP B{h->Pipp, h->Piph, h->Pi0pp, h->Pi0ph};
    auto Pi = [&](int ch) { return ch == CH_P ? h->Pipp : h->Piph; };
    auto Pi0 = [&](int ch) { return ch == CH_P ? h->Pi0pp : h->Pi0ph; };
    // work lists of the K1 / K2 classes (p uses the pp groups, a and t the ph groups)
    auto work = [&](int cls, cplx* raw) {
        ChanWork cw{};
        const size_t n = cls == 1 ? h->n1 : h->n2;
        for (int ch = 0; ch < 3; ++ch) {
            const Group& g = cls == 1 ? h->gK1 : k2group(h, ch);
            cw.items[ch] = g.trivial ? nullptr : g.d_items;
            cw.nitems[ch] = g.trivial ? (int)n : g.nitems;
            cw.out[ch] = raw + (size_t)ch * n;
            if (cls == 2) k2_rows(h, g, cw, ch);
        }
        return cw;
    };
    auto fin = [&](int cls, cplx* raw, cplx* const out[3], const Group* const grp[3]) {
        Finalize3 f{};
        const size_t n = cls == 1 ? h->n1 : (cls == 2 ? h->n2 : h->n3);
        for (int ch = 0; ch < 3; ++ch) {
            f.raw[ch] = raw + (size_t)ch * n;
            f.out[ch] = out[ch];
            f.map[ch] = grp[ch]->trivial ? nullptr : grp[ch]->d_map;
            f.FL[ch] = h->FLK2 + (size_t)ch * h->n2;
        }
        return f;
    };
    // src/solve.jl:26-82: :fdPA computes FL.K2 and FL.K3, :fdPA_new FL.K3 only
    if (strategy == FDGA_FDPA) {
        {  // left K2 (FL.K2): branch C
            if (conc) {
                CK(cudaEventRecord(h->evA, s));
                CK(cudaStreamWaitEvent(sC, h->evA, 0));
            }
            ChanWork cw = work(2, h->raw2);
            if (mixed) LC(launch_bse_L_K2_all(sC, Ff, B, cw, d));
            else LC(launch_bse_L_K2_all(sC, F, B, cw, d));
            cplx* out[3] = {h->FLK2, h->FLK2 + h->n2, h->FLK2 + 2 * h->n2};
            const Group* grp[3] = {&h->gK2pp, &h->gK2ph, &h->gK2ph};
            Finalize3 f2 = fin(2, h->raw2, out, grp);
            if (mixed)
                for (int c = 0; c < 3; ++c) f2.outf[c] = h->FLK2f + (size_t)c * h->n2;
            LC(launch_finalize3(sC, f2, 0, 1, h->n2));
            if (conc) CK(cudaEventRecord(h->evC, sC));
        }
        stage("bse_L_K2");
    }
    if (left_K3) {
        {  // left K3 (FL.K3)
            K3Args3 a3{};
            K3Args3F a3f{};
            for (int i = 0; i < 3; ++i) {
                const int ch = order[i];
                const int cg = ch == CH_P ? 4 : (ch == CH_A ? 5 : 6), cf0 = ch == CH_P ? 1 : (ch == CH_A ? 2 : 3);
                K3Args& a = a3.a[i];
                a.A = C.c[cg]; a.B0 = C.c[cf0]; a.Pi0 = Pi0(ch);
                a.out = h->raw3 + (size_t)ch * h->n3;
                a3.ch[i] = ch;
                K3ArgsF& af = a3f.a[i];
                af.A = C.f[cg]; af.B0 = C.f[cf0]; af.Pi0 = Pi0(ch);
                af.out = a.out;
                a3f.ch[i] = ch;
            }
            a3.blocks = a3f.blocks = h->d_k3blocks;
            a3.nblocks = a3f.nblocks = h->nk3blocks;
            if (mixed && k3_tensor_cores(h, 0)) LC(launch_k3_tensor_cores(h, s, 0, a3f));
            else if (mixed) LC(launch_bse_K3_f32(s, 0, a3f, 3, d, h->k3_tile[FDGA_MIXED][0]));
            else LC(launch_k3_fp64(h, s, 0, a3));
            stage("bse_L_K3_gemm");
            cplx* out[3] = {h->FLK3, h->FLK3 + h->n3, h->FLK3 + 2 * h->n3};
            const Group* grp[3] = {&h->gK3ppL, &h->gK3phL, &h->gK3phL};
            Finalize3 f3 = fin(3, h->raw3, out, grp);
            if (mixed)
                for (int c = 0; c < 3; ++c) f3.outf[c] = h->FLK3f + (size_t)c * h->n3;
            LC(launch_finalize3(s, f3, 0, 1, h->n3));
        }
        stage("bse_L_K3_finalize");
    }
    if (conc) {  // join: bubbles (B) and FL.K2 (C)
        CK(cudaStreamWaitEvent(s, h->evB, 0));
        if (strategy == FDGA_FDPA) CK(cudaStreamWaitEvent(s, h->evC, 0));
    }
    // the one-loop BSEs (:fdPA_1loop) are the fdPA ones without their FL factor
    FLP FLz = FL;
    FLPF FLzf = FLf;
    if (oneloop) {
        for (int c = 0; c < 3; ++c) {
            FLz.K2[c] = h->FLzero + (size_t)c * h->n2;
            FLzf.K2[c] = h->FLzerof + (size_t)c * h->n2;
        }
    }
    // K1 and K2 (branch D) run concurrently with the K3 contraction (main stream); the SDE joins
    cudaStream_t sD = conc ? h->st3 : s;
    if (conc) {
        CK(cudaEventRecord(h->evD, s));
        CK(cudaStreamWaitEvent(sD, h->evD, 0));
    }
    // ω-sums of the right BSE factor (needs FL.K2 of this iteration)
    if (!is_new) LC(launch_sx(sD, B, h->SPi, h->SPi0, FLz, F, h->SX, d));
    {  // K1
        ChanWork cw = work(1, h->raw1);
        if (is_new && mixed) LC(launch_bse_K1_new(sD, Ff, B, h->SPi, h->SPi0, cw, d));
        else if (is_new) LC(launch_bse_K1_new(sD, F, B, h->SPi, h->SPi0, cw, d));
        else if (mixed) LC(launch_bse_K1_all(sD, Ff, FLzf, B, h->SX, cw, d));
        else LC(launch_bse_K1_all(sD, F, FLz, B, h->SX, cw, d));
        cplx* out[3] = {chanK(h, h->yS, CH_P, 1), chanK(h, h->yS, CH_T, 1), chanK(h, h->yS, CH_A, 1)};
        const Group* grp[3] = {&h->gK1, &h->gK1, &h->gK1};
        LC(launch_finalize3(sD, fin(1, h->raw1, out, grp), 0, 1, h->n1));
    }
    stage("bse_K1");
    {  // K2 (the _new form has no FL epilogue)
        ChanWork cw = work(2, h->raw2);
        if (is_new && mixed) LC(launch_bse_K2_new(sD, Ff, B, h->SPi, h->SPi0, cw, d));
        else if (is_new) LC(launch_bse_K2_new(sD, F, B, h->SPi, h->SPi0, cw, d));
        else if (mixed) LC(launch_bse_K2_all(sD, Ff, FLzf, B, h->SX, cw, d));
        else LC(launch_bse_K2_all(sD, F, FLz, B, h->SX, cw, d));
        cplx* out[3] = {chanK(h, h->yS, CH_P, 2), chanK(h, h->yS, CH_T, 2), chanK(h, h->yS, CH_A, 2)};
        const Group* grp[3] = {&h->gK2pp, &h->gK2ph, &h->gK2ph};
        LC(launch_finalize3(sD, fin(2, h->raw2, out, grp), is_new ? 0 : 1, 1, h->n2));
    }
    stage("bse_K2");
    if (conc) CK(cudaEventRecord(h->evE, sD));
    {  // K3
        K3Args3 a3{};
        K3Args3F a3f{};
        for (int i = 0; i < 3; ++i) {
            const int ch = order[i];
            const int cg = ch == CH_P ? 0 : (ch == CH_A ? 5 : 6), cf = ch == CH_P ? 7 : (ch == CH_A ? 8 : 9);
            const int cf0 = ch == CH_P ? 1 : (ch == CH_A ? 2 : 3);
            K3Args& a = a3.a[i];
            a.A = C.c[cf]; a.B0 = C.c[cf0]; a.G = C.c[cg]; a.Pi = Pi(ch); a.Pi0 = Pi0(ch);
            a.FLc = h->FLK3 + (size_t)ch * h->n3; a.FLt = h->FLK3 + (size_t)CH_T * h->n3; a.FLa = h->FLK3 + (size_t)CH_A * h->n3;
            a.out = h->raw3 + (size_t)ch * h->n3;
            a.flags = oneloop ? (K3F_1LOOP | K3F_NOEPI) : 0;  // :fdPA_1loop: T F (Π - Π0) F0 only
            a3.ch[i] = ch;
            if (mixed) {
                K3ArgsF& af = a3f.a[i];
                af.A = C.f[cf]; af.B0 = C.f[cf0]; af.G = C.f[cg]; af.Pi = a.Pi; af.Pi0 = a.Pi0;
                af.FLc = h->FLK3f + (size_t)ch * h->n3; af.FLt = h->FLK3f + (size_t)CH_T * h->n3;
                af.FLa = h->FLK3f + (size_t)CH_A * h->n3;
                af.out = a.out;
                af.flags = a.flags;
                a3f.ch[i] = ch;
            }
        }
        a3.blocks = a3f.blocks = h->d_k3blocks;
        a3.nblocks = a3f.nblocks = h->nk3blocks;
        if (mixed && k3_tensor_cores(h, 1)) LC(launch_k3_tensor_cores(h, s, 1, a3f));
        else if (mixed) LC(launch_bse_K3_f32(s, 1, a3f, 3, d, h->k3_tile[FDGA_MIXED][1]));
        else LC(launch_k3_fp64(h, s, 1, a3));
        stage("bse_K3_gemm");
        cplx* out[3] = {chanK(h, h->yS, CH_P, 3), chanK(h, h->yS, CH_T, 3), chanK(h, h->yS, CH_A, 3)};
        const Group* grp[3] = {&h->gK3pp, &h->gK3ph, &h->gK3ph};
        LC(launch_finalize3(s, fin(3, h->raw3, out, grp), 0, 1, h->n3));
    }
    stage("bse_K3_finalize");
    if (conc) CK(cudaStreamWaitEvent(s, h->evE, 0));  // join: K1, K2 (D)
    if (hooks && hooks->vertex_done) {
        int r = hooks->vertex_done();
        if (r) return r;
    }
    // SDE (src/SDE.jl:3-33) with the new F
    cplx* SigOut = sigmaOf(h, h->yS);
    if (update_sigma) {
        const double rs = h->ref_nonzero ? 1.0 / 3.0 : 0.0;
        if (mixed) {
            LC(launch_to_f32(s, h->yS, h->ySf, 3 * h->nchan));
            LC(sde_L_pair(h, Fnf, B, h->SPi, h->has0 ? 3 : 1, rs, nl));
        } else {
            LC(sde_L_pair(h, Fn, B, h->SPi, h->has0 ? 3 : 1, rs, nl));
        }
        LC(launch_sde_sigma(s, h->GR, h->Lpp, h->Lph, h->LR, h->SigR, h->SigIn, h->twm, h->twp, d));
        nl += 3;
        LC(launch_sigma_assemble(s, h->SigIn, h->SigU2, h->gSig.trivial ? nullptr : h->gSig.d_map, h->occ, h->C0,
                                 h->Sig0, SigOut, d.U, hartree ? 1 : 0,
                                 strategy_fdpa_sde(strategy) ? (h->fdpa_single_hartree ? 2 : 1) : 0, h->n0, h->nGk));
    } else {
        LC(cudaMemcpyAsync(SigOut, sigmaOf(h, h->xS), h->nGk * sizeof(cplx), cudaMemcpyDeviceToDevice, s));
    }
    stage("sde");
    return FDGA_OK;
}

// ---------------------------------------------------------------------------------------------
// Tangent map (forward-mode derivative, the frule of one iteration): ty = Φ'(x) tx at the base
// point x whose value intermediates (G, G(R), Π, SΠ, caches, FL, S_X, L(R), the U² correlator) the
// last enqueue_iteration of the same precision left in the handle.  The map is a composition of
// vertex-linear stages (momentum averages, caches, left BSEs, symmetrisation and recombination)
// and of products (the bubble G·G, the BSEs F·Π·(F, FL), the SDE G·L and G·G·G); the tangent
// applies the product rule stage by stage:
//   * vertex-linear stages run on the tangent vertex with the RefVertex terms off (it is constant);
//   * dG = -G² dΣ; dΠ and dSΠ from the product-rule bubble kernels (the 1/ν tails are constant);
//   * each bilinear BSE runs as one fused tangent kernel, dK = K(dF; Π, FL) + K(F; dΠ, dFL) (Π0 and
//     the RefVertex caches are constant): K1/K2 evaluate F and dF in the same pass, K3 is one GEMM
//     over the concatenated inner index, [dA | A]·[M ; dM];
//   * dΣ from dL = L(dF, Π) + L(F, dΠ) (one pass), and the product-rule Σ_R and U² kernels.
// ---------------------------------------------------------------------------------------------
int ensure_tangent(fdga_handle* h) {
    auto& t = h->tan;
    const Dims& d = h->d;
    const bool mixed = h->precision == FDGA_MIXED;
    if (!t.x) {  // (the zero-fills run on the solver stream, ahead of any use)
        AL(t.x, h->nstate); AL(t.y, h->nstate);
        if (h->navg) AL(t.avg, h->navg);
        AL(t.G, h->nGk); AL(t.GR, h->nGk);
        AL(t.Pipp, h->nPi); AL(t.Piph, h->nPi);
        AL(t.SPi, 2 * (size_t)d.Nq * d.NPO); AL(t.SX, 3 * (size_t)d.Nq * d.NPO);
        AL(t.FLK2, 3 * h->n2); AL(t.FLK3, 3 * h->n3);
        AL(t.Lpp, h->n2); AL(t.Lph, h->n2); AL(t.LR, 2 * h->n2); AL(t.SR, h->nGk);
        AL(t.SigIn, h->nGk); AL(t.u2C, (size_t)d.Nq * (2 * d.NG - 1)); AL(t.u2R, h->nGk); AL(t.SigU2, h->nGk);
        AL(t.occ, 1);
    }
    if (!mixed && !t.cache) AL(t.cache, 7 * h->n3);
    if (mixed && !t.cachef) {
        int r = ensure_mixed(h);
        if (r) return r;
        AL(t.cachef, 7 * h->n3);
        AL(t.FLK2f, 3 * h->n2); AL(t.FLK3f, 3 * h->n3);
        AL(t.xSf, 3 * h->nchan); AL(t.ySf, 3 * h->nchan);
        if (h->navg) AL(t.avgf, h->navg);
        AL(t.GRf, h->nGk);
    }
    return FDGA_OK;
}

int enqueue_tangent(fdga_handle* h, int strategy, bool update_sigma, bool hartree, int& nl,
                    const StageHook& mark = StageHook()) {
    cudaStream_t s = h->st;
    const Dims& d = h->d;
    auto& t = h->tan;
    auto stage = [&](const char* name) { if (mark) mark(name); };
    nl = 0;
    const bool mixed = h->precision == FDGA_MIXED;
    const size_t nS = (size_t)d.Nq * d.NPO;
    VertP F = vertex_view(h, h->xS), Fn = vertex_view(h, h->yS);
    VertP tF = vertex_view_t<cplx>(h, t.x, t.avg, h->Fref), tFn = vertex_view_t<cplx>(h, t.y, t.avg, h->Fref);
    tF.noref = tFn.noref = 1;
    // as in the value map, the Dyson/bubble tangents (branch B) and the left K2 tangent (branch C)
    // run concurrently with the main stream's caches and left K3 when captured into a graph
    const bool conc = !mark;
    cudaStream_t sB = conc ? h->st2 : s, sC = conc ? h->st3 : s;
    if (conc) {
        CK(cudaEventRecord(h->evfork, s));
        CK(cudaStreamWaitEvent(sB, h->evfork, 0));
    }
    if (d.Nq > 1) {
        ChanArrays in;
        ChanArraysW out;
        for (int c = 0; c < 3; ++c) {
            in.K1[c] = tF.g[c].K1; in.K2[c] = tF.g[c].K2; in.K3[c] = tF.g[c].K3;
            out.K1[c] = (cplx*)tF.g[c].A1; out.K2[c] = (cplx*)tF.g[c].A2; out.K3[c] = (cplx*)tF.g[c].A3;
        }
        LC(launch_qavg(s, in, out, d));
        stage("qavg");
    }
    if (update_sigma) {
        LC(launch_dyson_tan(sB, t.G, h->G, sigmaOf(h, t.x), h->nGk));
        LC(launch_g_realspace(sB, t.G, t.GR, h->twm, d));
        if (mixed && bubble_f32_supported(d)) {
            LC(launch_to_f32(sB, t.GR, t.GRf, h->nGk));
            LC(launch_bubble_f32_tan(sB, h->GRf, t.GRf, t.Pipp, t.Piph, h->twp, d));
            LC(launch_rowsum_tan(sB, t.Pipp, t.Piph, h->GR, t.GR, h->SRtmp, h->twp, t.SPi, t.SPi + nS, d, h->GRf,
                                 t.GRf));
        } else {
            LC(launch_bubble_tan(sB, h->G, t.G, h->GR, t.GR, t.Pipp, t.Piph, h->twp, d));
            LC(launch_rowsum_tan(sB, t.Pipp, t.Piph, h->GR, t.GR, h->SRtmp, h->twp, t.SPi, t.SPi + nS, d));
        }
    } else {  // G and Π are held fixed
        LC(cudaMemsetAsync(t.Pipp, 0, h->nPi * sizeof(cplx), sB));
        LC(cudaMemsetAsync(t.Piph, 0, h->nPi * sizeof(cplx), sB));
        LC(cudaMemsetAsync(t.SPi, 0, 2 * nS * sizeof(cplx), sB));
    }
    if (update_sigma) {  // the U² and occupation tangents need only dG: also on branch B
        LC(launch_u2_tan(sB, h->GR, h->u2C, t.GR, t.u2C, t.u2R, t.SigU2, h->twp, d));
        nl += 2;
        LC(launch_occupation(sB, t.G, h->nGk, d.T, d.Nk, t.occ));  // 1/2 + dn: the Hartree term reads dn
    }
    stage("dyson_bubble");
    if (conc) CK(cudaEventRecord(h->evB, sB));
    // FP32 mirrors of the tangent vertex (mixed map); the value mirrors are the value pass's
    VertPF Ff{}, Fnf{}, tFf{}, tFnf{};
    FLPF FLf{}, tFLf{};
    if (mixed) {
        LC(launch_to_f32(s, t.x, t.xSf, 3 * h->nchan));
        if (d.Nq > 1) LC(launch_to_f32(s, t.avg, t.avgf, h->navg));
        Ff = vertex_view_t<cplxf>(h, h->xSf, h->avgf, h->Freff);
        Fnf = vertex_view_t<cplxf>(h, h->ySf, h->avgf, h->Freff);
        tFf = vertex_view_t<cplxf>(h, t.xSf, t.avgf, h->Freff);
        tFnf = vertex_view_t<cplxf>(h, t.ySf, t.avgf, h->Freff);
        tFf.noref = tFnf.noref = 1;
        for (int c = 0; c < 3; ++c) {
            FLf.K2[c] = h->FLK2f + (size_t)c * h->n2;
            tFLf.K2[c] = t.FLK2f + (size_t)c * h->n2;
        }
    }
    // caches of the tangent vertex (slot -1: a RefVertex cache, constant)
    static const int slot[10] = {0, -1, -1, -1, 1, 2, 3, 4, 5, 6};
    Caches C{}, tC{};
    for (int i = 0; i < 10; ++i) {
        C.c[i] = h->cache + (size_t)i * h->n3;
        C.f[i] = mixed ? h->cachef + (size_t)i * h->n3 : nullptr;
        tC.c[i] = (slot[i] < 0 || mixed) ? nullptr : t.cache + (size_t)slot[i] * h->n3;
        tC.f[i] = (slot[i] < 0 || !mixed) ? nullptr : t.cachef + (size_t)slot[i] * h->n3;
    }
    if (mixed) LC(launch_build_cache(s, tFf, tC, h->d_k3blocks, h->nk3blocks, d));
    else LC(launch_build_cache(s, tF, tC, h->d_k3blocks, h->nk3blocks, d));
    stage("k3_cache");
    FLP FL, tFL;
    for (int c = 0; c < 3; ++c) {
        FL.K2[c] = h->FLK2 + (size_t)c * h->n2;
        tFL.K2[c] = t.FLK2 + (size_t)c * h->n2;
    }
    const int order[3] = {CH_P, CH_A, CH_T};
    auto Pi = [&](int ch) -> const cplx* { return ch == CH_P ? h->Pipp : h->Piph; };
    auto tPi = [&](int ch) -> const cplx* { return ch == CH_P ? t.Pipp : t.Piph; };
    auto Pi0 = [&](int ch) -> const cplx* { return ch == CH_P ? h->Pi0pp : h->Pi0ph; };
    const BubbleP B{h->Pipp, h->Piph, h->Pi0pp, h->Pi0ph};
    auto work = [&](int cls, cplx* raw, int acc) {
        ChanWork cw{};
        const size_t n = cls == 1 ? h->n1 : h->n2;
        for (int ch = 0; ch < 3; ++ch) {
            const Group& g = cls == 1 ? h->gK1 : k2group(h, ch);
            cw.items[ch] = g.trivial ? nullptr : g.d_items;
            cw.nitems[ch] = g.trivial ? (int)n : g.nitems;
            cw.out[ch] = raw + (size_t)ch * n;
            if (cls == 2) k2_rows(h, g, cw, ch);
        }
        cw.acc = acc;
        return cw;
    };
    auto fin = [&](int cls, cplx* raw, cplx* const out[3], const Group* const grp[3]) {
        Finalize3 f{};
        const size_t n = cls == 1 ? h->n1 : (cls == 2 ? h->n2 : h->n3);
        for (int ch = 0; ch < 3; ++ch) {
            f.raw[ch] = raw + (size_t)ch * n;
            f.out[ch] = out[ch];
            f.map[ch] = grp[ch]->trivial ? nullptr : grp[ch]->d_map;
            f.FL[ch] = t.FLK2 + (size_t)ch * h->n2;
        }
        return f;
    };
    // K3 contraction launch in the precision of the map; the tangent (mode 2) takes the tile tuned
    // for the K3 contraction (mode 1), whose operands it shares
    auto k3 = [&](int mode, const K3Args3& a3, const K3Args3F& a3f) -> cudaError_t {
        const int tm = mode == 0 ? 0 : 1;
        if (mixed && k3_tensor_cores(h, mode)) return launch_k3_tensor_cores(h, s, mode, a3f);
        if (mixed) return launch_bse_K3_f32(s, mode, a3f, 3, d, h->k3_tile[FDGA_MIXED][tm]);
        return launch_k3_fp64(h, s, mode, a3);
    };
    if (strategy == FDGA_FDPA) {
        {  // dFL.K2 = L_K2(dF)  (Π0 constant): branch C
            if (conc) {
                CK(cudaEventRecord(h->evA, s));
                CK(cudaStreamWaitEvent(sC, h->evA, 0));
            }
            ChanWork cw = work(2, h->raw2, 0);
            if (mixed) LC(launch_bse_L_K2_all(sC, tFf, B, cw, d));
            else LC(launch_bse_L_K2_all(sC, tF, B, cw, d));
            cplx* out[3] = {t.FLK2, t.FLK2 + h->n2, t.FLK2 + 2 * h->n2};
            const Group* grp[3] = {&h->gK2pp, &h->gK2ph, &h->gK2ph};
            Finalize3 f2 = fin(2, h->raw2, out, grp);
            if (mixed)
                for (int c = 0; c < 3; ++c) f2.outf[c] = t.FLK2f + (size_t)c * h->n2;
            LC(launch_finalize3(sC, f2, 0, 1, h->n2));
            if (conc) CK(cudaEventRecord(h->evC, sC));
        }
        stage("bse_L_K2");
        {  // dFL.K3 = L_K3(dΓ)  (Π0 and the RefVertex caches constant)
            K3Args3 a3{};
            K3Args3F a3f{};
            for (int i = 0; i < 3; ++i) {
                const int ch = order[i];
                const int cg = ch == CH_P ? 4 : (ch == CH_A ? 5 : 6), cf0 = ch == CH_P ? 1 : (ch == CH_A ? 2 : 3);
                K3Args& a = a3.a[i];
                a.A = tC.c[cg]; a.B0 = C.c[cf0]; a.Pi0 = Pi0(ch);
                a.out = h->raw3 + (size_t)ch * h->n3;
                a3.ch[i] = a3f.ch[i] = ch;
                K3ArgsF& af = a3f.a[i];
                af.A = tC.f[cg]; af.B0 = C.f[cf0]; af.Pi0 = Pi0(ch);
                af.out = a.out;
            }
            a3.blocks = a3f.blocks = h->d_k3blocks;
            a3.nblocks = a3f.nblocks = h->nk3blocks;
            LC(k3(0, a3, a3f));
            cplx* out[3] = {t.FLK3, t.FLK3 + h->n3, t.FLK3 + 2 * h->n3};
            const Group* grp[3] = {&h->gK3ppL, &h->gK3phL, &h->gK3phL};
            Finalize3 f3 = fin(3, h->raw3, out, grp);
            if (mixed)
                for (int c = 0; c < 3; ++c) f3.outf[c] = t.FLK3f + (size_t)c * h->n3;
            LC(launch_finalize3(s, f3, 0, 1, h->n3));
        }
        stage("bse_L_K3");
    } else {  // scPA: FL is not iterated
        LC(cudaMemsetAsync(t.FLK2, 0, 3 * h->n2 * sizeof(cplx), s));
        LC(cudaMemsetAsync(t.FLK3, 0, 3 * h->n3 * sizeof(cplx), s));
        if (mixed) {
            LC(cudaMemsetAsync(t.FLK2f, 0, 3 * h->n2 * sizeof(cplxf), s));
            LC(cudaMemsetAsync(t.FLK3f, 0, 3 * h->n3 * sizeof(cplxf), s));
        }
    }
    if (conc) {  // join: dΠ, dSΠ (B) and dFL.K2 (C)
        CK(cudaStreamWaitEvent(s, h->evB, 0));
        if (strategy == FDGA_FDPA) CK(cudaStreamWaitEvent(s, h->evC, 0));
    }
    // dK1 and dK2 (branch D) run concurrently with the K3 tangent (main stream)
    cudaStream_t sD = conc ? h->st3 : s;
    if (conc) {
        CK(cudaEventRecord(h->evD, s));
        CK(cudaStreamWaitEvent(sD, h->evD, 0));
    }
    LC(launch_sx_tan(sD, h->Pipp, h->Piph, t.Pipp, t.Piph, t.SPi, FL, tFL, F, t.SX, d));
    stage("sx");
    // tangent factors of the fused K1/K2/SDE kernels
    const TanArgs T64{tF, tFL, t.Pipp, t.Piph, t.SX, t.SPi, t.SPi + nS};
    const TanArgsF T32{tFf, tFLf, t.Pipp, t.Piph, t.SX, t.SPi, t.SPi + nS};
    {  // dK1 = K1(dF; Π, FL, S_X) + K1(F; dΠ, dFL, dS_X), one pass
        if (mixed) LC(launch_bse_K1_tan(sD, Ff, FLf, B, h->SX, T32, work(1, h->raw1, 0), d));
        else LC(launch_bse_K1_tan(sD, F, FL, B, h->SX, T64, work(1, h->raw1, 0), d));
        cplx* out[3] = {chanK(h, t.y, CH_P, 1), chanK(h, t.y, CH_T, 1), chanK(h, t.y, CH_A, 1)};
        const Group* grp[3] = {&h->gK1, &h->gK1, &h->gK1};
        LC(launch_finalize3(sD, fin(1, h->raw1, out, grp), 0, 1, h->n1));
    }
    stage("bse_K1");
    {  // dK2 likewise, then the FL epilogue with dFL.K2
        if (mixed) LC(launch_bse_K2_tan(sD, Ff, FLf, B, h->SX, T32, work(2, h->raw2, 0), d));
        else LC(launch_bse_K2_tan(sD, F, FL, B, h->SX, T64, work(2, h->raw2, 0), d));
        cplx* out[3] = {chanK(h, t.y, CH_P, 2), chanK(h, t.y, CH_T, 2), chanK(h, t.y, CH_A, 2)};
        const Group* grp[3] = {&h->gK2pp, &h->gK2ph, &h->gK2ph};
        LC(launch_finalize3(sD, fin(2, h->raw2, out, grp), 1, 1, h->n2));
    }
    stage("bse_K2");
    if (conc) CK(cudaEventRecord(h->evE, sD));
    {  // dK3 = T (dF·M + F·dM) + dγL: one GEMM over the concatenated inner index (mode 2)
        K3Args3 a3{};
        K3Args3F a3f{};
        for (int i = 0; i < 3; ++i) {
            const int ch = order[i];
            const int cg = ch == CH_P ? 0 : (ch == CH_A ? 5 : 6), cf = ch == CH_P ? 7 : (ch == CH_A ? 8 : 9);
            const int cf0 = ch == CH_P ? 1 : (ch == CH_A ? 2 : 3);
            K3Args& a = a3.a[i];
            K3ArgsF& af = a3f.a[i];
            a.A = C.c[cf]; af.A = C.f[cf];
            a.tA = tC.c[cf]; af.tA = tC.f[cf];
            a.B0 = C.c[cf0]; af.B0 = C.f[cf0];
            a.G = C.c[cg]; af.G = C.f[cg];
            a.tG = tC.c[cg]; af.tG = tC.f[cg];
            a.Pi = af.Pi = Pi(ch);
            a.tPi = af.tPi = tPi(ch);
            a.Pi0 = af.Pi0 = Pi0(ch);
            a.FLc = h->FLK3 + (size_t)ch * h->n3; a.FLt = h->FLK3 + (size_t)CH_T * h->n3;
            a.FLa = h->FLK3 + (size_t)CH_A * h->n3;
            a.tFLc = t.FLK3 + (size_t)ch * h->n3; a.tFLt = t.FLK3 + (size_t)CH_T * h->n3;
            a.tFLa = t.FLK3 + (size_t)CH_A * h->n3;
            if (mixed) {
                af.FLc = h->FLK3f + (size_t)ch * h->n3; af.FLt = h->FLK3f + (size_t)CH_T * h->n3;
                af.FLa = h->FLK3f + (size_t)CH_A * h->n3;
                af.tFLc = t.FLK3f + (size_t)ch * h->n3; af.tFLt = t.FLK3f + (size_t)CH_T * h->n3;
                af.tFLa = t.FLK3f + (size_t)CH_A * h->n3;
            }
            a.out = af.out = h->raw3 + (size_t)ch * h->n3;
            a3.ch[i] = a3f.ch[i] = ch;
        }
        a3.blocks = a3f.blocks = h->d_k3blocks;
        a3.nblocks = a3f.nblocks = h->nk3blocks;
        LC(k3(2, a3, a3f));
        cplx* out[3] = {chanK(h, t.y, CH_P, 3), chanK(h, t.y, CH_T, 3), chanK(h, t.y, CH_A, 3)};
        const Group* grp[3] = {&h->gK3pp, &h->gK3ph, &h->gK3ph};
        LC(launch_finalize3(s, fin(3, h->raw3, out, grp), 0, 1, h->n3));
    }
    stage("bse_K3");
    if (conc) CK(cudaStreamWaitEvent(s, h->evE, 0));  // join: dK1, dK2 (D)
    cplx* tSig = sigmaOf(h, t.y);
    if (update_sigma) {
        const double rs = h->ref_nonzero ? 1.0 / 3.0 : 0.0;
        ChanWork cw{};
        const Group* g[2] = {&h->gK2pp, &h->gK2ph};
        for (int w = 0; w < 2; ++w) {
            cw.items[w] = g[w]->trivial ? nullptr : g[w]->d_items;
            cw.nitems[w] = g[w]->trivial ? (int)h->n2 : g[w]->nitems;
            cw.out[w] = h->raw2 + (size_t)w * h->n2;
        }
        // dL = L(dF; Π, SΠ) + L(F; dΠ, dSΠ) (+ the RefVertex part with dΠ), one pass
        if (mixed) {
            LC(launch_to_f32(s, t.y, t.ySf, 3 * h->nchan));
            TanArgsF Tn = T32;
            Tn.F = tFnf;
            LC(launch_sde_L_tan(s, Fnf, B, h->SPi, h->SPi + nS, Tn, cw, rs, d));
        } else {
            TanArgs Tn = T64;
            Tn.F = tFn;
            LC(launch_sde_L_tan(s, Fn, B, h->SPi, h->SPi + nS, Tn, cw, rs, d));
        }
        Finalize3 f{};
        f.raw[0] = h->raw2; f.out[0] = t.Lpp; f.map[0] = g[0]->trivial ? nullptr : g[0]->d_map;
        f.raw[2] = h->raw2 + h->n2; f.out[2] = t.Lph; f.map[2] = g[1]->trivial ? nullptr : g[1]->d_map;
        LC(launch_finalize3(s, f, 0, 0, h->n2));
        LC(launch_sde_sigma_tan(s, h->GR, h->LR, t.GR, t.Lpp, t.Lph, t.LR, t.SR, t.SigIn, h->twm, h->twp, d));
        nl += 3;
        LC(launch_sigma_assemble(s, t.SigIn, t.SigU2, h->gSig.trivial ? nullptr : h->gSig.d_map, t.occ, nullptr,
                                 nullptr, tSig, d.U, hartree ? 1 : 0, 0, 0.0, h->nGk));
    } else {
        LC(cudaMemcpyAsync(tSig, sigmaOf(h, t.x), h->nGk * sizeof(cplx), cudaMemcpyDeviceToDevice, s));
    }
    stage("sde");
    return FDGA_OK;
}

int run_tangent(fdga_handle* h, int strategy, bool update_sigma, bool hartree) {
    if (strategy != FDGA_FDPA && strategy != FDGA_SCPA)  // (the graph table holds these two)
        return fail(h, FDGA_ERR_UNSUPPORTED, "the tangent map covers the fdPA and scPA strategies");
    int r = ensure_tangent(h);
    if (r) return r;
    Graph& g = h->tan.graphs[h->precision][strategy][update_sigma][hartree];
    if (!g.exec) {
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
        int nl = 0;
        r = enqueue_tangent(h, strategy, update_sigma, hartree, nl);
        cudaError_t ee = cudaStreamEndCapture(h->st, &graph);
        if (r) {
            if (ee == cudaSuccess) cudaGraphDestroy(graph);
            return r;
        }
        if (ee != cudaSuccess) return cuda_fail(h, ee, "cudaStreamEndCapture");
        ee = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ee != cudaSuccess) { g.exec = nullptr; return cuda_fail(h, ee, "cudaGraphInstantiate"); }
        g.nodes = nl;
    }
    CK(cudaGraphLaunch(g.exec, h->st));
    h->last_launches = g.nodes;
    return FDGA_OK;
}

// ---------------------------------------------------------------------------------------------
// Adjoint map (reverse mode, the rrule of one FP64 iteration): x̄ = Φ'(x)ᵀ ȳ for the real inner
// product, at the base point whose value intermediates the last FP64 enqueue_iteration left in the
// handle.  The stages of enqueue_iteration run backwards: Σ assembly, U² and Σ_R terms, L (SDE),
// the K1/K2/K3 outputs (symmetrisation, FL epilogue, recombination), the K3 GEMMs, K2, K1, S_X, the
// left BSEs, the caches, the bubbles and row sums, G(R), Dyson and the momentum averages.  The
// kernels are in fdga_adjoint.cu.
// ---------------------------------------------------------------------------------------------
int ensure_adjoint(fdga_handle* h) {
    auto& a = h->adj;
    if (a.xb) return FDGA_OK;
    const Dims& d = h->d;
    const size_t NR = (size_t)d.L * d.L, nS = (size_t)d.Nq * d.NPO;
    AL(a.xb, h->nstate); AL(a.yb, h->nstate);
    if (h->navg) AL(a.avgb, h->navg);
    AL(a.Gb, h->nGk); AL(a.GRb, h->nGk);
    AL(a.Pbpp, h->nPi); AL(a.Pbph, h->nPi); AL(a.PbRpp, h->nPi); AL(a.PbRph, h->nPi);
    AL(a.SPib, 2 * nS); AL(a.SRb, 2 * NR * d.NPO); AL(a.SXb, 3 * nS);
    AL(a.cacheb, 10 * h->n3); AL(a.FLK2b, 3 * h->n2); AL(a.FLK3b, 3 * h->n3);
    AL(a.raw1, 3 * h->n1); AL(a.raw2, 3 * h->n2); AL(a.raw3, 3 * h->n3);
    AL(a.M, 3 * h->n3); AL(a.Mb, 3 * h->n3);
    AL(a.SigInb, h->nGk); AL(a.SU2b, h->nGk); AL(a.SigRb, h->nGk); AL(a.u2Rb, h->nGk);
    AL(a.u2Cb, (size_t)d.Nq * (2 * d.NG - 1));
    AL(a.LRb, 2 * h->n2); AL(a.Lb, 2 * h->n2);
    AL(a.nbar, 1);
    return FDGA_OK;
}

int enqueue_adjoint(fdga_handle* h, int strategy, bool update_sigma, bool hartree) {
    cudaStream_t s = h->st;
    const Dims& d = h->d;
    auto& a = h->adj;
    const size_t nS = (size_t)d.Nq * d.NPO;
    auto Z = [&](void* p, size_t bytes) { return cudaMemsetAsync(p, 0, bytes, s); };
    CK(Z(a.xb, h->nstate * sizeof(cplx)));
    if (h->navg) CK(Z(a.avgb, h->navg * sizeof(cplx)));
    CK(Z(a.GRb, h->nGk * sizeof(cplx)));
    CK(Z(a.Pbpp, h->nPi * sizeof(cplx))); CK(Z(a.Pbph, h->nPi * sizeof(cplx)));
    CK(Z(a.SPib, 2 * nS * sizeof(cplx))); CK(Z(a.SXb, 3 * nS * sizeof(cplx)));
    CK(Z(a.cacheb, 10 * h->n3 * sizeof(cplx)));
    CK(Z(a.FLK2b, 3 * h->n2 * sizeof(cplx))); CK(Z(a.FLK3b, 3 * h->n3 * sizeof(cplx)));
    CK(Z(a.SigInb, h->nGk * sizeof(cplx))); CK(Z(a.SU2b, h->nGk * sizeof(cplx)));
    CK(Z(a.nbar, sizeof(double)));
    VertP F = vertex_view(h, h->xS), Fn = vertex_view(h, h->yS);
    // cotangent views: x̄ (with the averages' cotangents) and ȳ (SDE contributions to the new vertex)
    auto bar_view = [&](cplx* st, cplx* avg) {
        VertBar B{};
        for (int c = 0; c < 3; ++c) {
            cplx* base = st + (size_t)c * h->nchan;
            B.g[c].K1 = base; B.g[c].K2 = base + h->n1; B.g[c].K3 = base + h->n1 + h->n2;
            if (d.Nq == 1 || !avg) {
                B.g[c].A1 = B.g[c].K1; B.g[c].A2 = B.g[c].K2; B.g[c].A3 = B.g[c].K3;
            } else {
                const size_t per1 = d.N1, per2 = (size_t)d.N2O * d.N2n, per3 = (size_t)d.N3O * d.N3n * d.N3n;
                cplx* av = avg + (size_t)c * (per1 + per2 + per3);
                B.g[c].A1 = av; B.g[c].A2 = av + per1; B.g[c].A3 = av + per1 + per2;
            }
        }
        return B;
    };
    const VertBar Xb = bar_view(a.xb, a.avgb), Yb = bar_view(a.yb, nullptr);
    FLP FL;
    FLBar FLb;
    for (int c = 0; c < 3; ++c) {
        FL.K2[c] = h->FLK2 + (size_t)c * h->n2;
        FLb.K2[c] = a.FLK2b + (size_t)c * h->n2;
    }
    const BubbleP B{h->Pipp, h->Piph, h->Pi0pp, h->Pi0ph};
    auto work = [&](int cls) {
        ChanWork cw{};
        const size_t n = cls == 1 ? h->n1 : h->n2;
        for (int ch = 0; ch < 3; ++ch) {
            const Group& g = cls == 1 ? h->gK1 : k2group(h, ch);
            cw.items[ch] = g.trivial ? nullptr : g.d_items;
            cw.nitems[ch] = g.trivial ? (int)n : g.nitems;
        }
        return cw;
    };
    // finalize transposed: output cotangents ō (f.raw) -> representative cotangents (f.out)
    auto fin_adj = [&](const cplx* const ob[3], cplx* rb, size_t n, const Group* const grp[3], int k2e, int trec,
                       cplx* const FLbar[3]) -> cudaError_t {
        cudaError_t e = cudaMemsetAsync(rb, 0, 3 * n * sizeof(cplx), s);
        if (e != cudaSuccess) return e;
        Finalize3 f{};
        for (int ch = 0; ch < 3; ++ch) {
            f.raw[ch] = ob[ch];
            f.out[ch] = ob[ch] ? rb + (size_t)ch * n : nullptr;
            f.map[ch] = grp[ch]->trivial ? nullptr : grp[ch]->d_map;
        }
        return launch_adj_finalize3(s, f, k2e, trec, n, FLbar);
    };
    cplx* Sbar_in = sigmaOf(h, a.xb);
    if (update_sigma) {
        // Σ_out = op(Σin + Σ_U²)[rep] + i (n - 1/2) U
        CK(launch_adj_assemble(s, sigmaOf(h, a.yb), h->gSig.trivial ? nullptr : h->gSig.d_map, a.SigInb, a.SU2b,
                               h->nGk, hartree ? 1 : 0, d.U, a.nbar));
        CK(launch_adj_u2(s, h->GR, h->u2C, a.SU2b, a.u2Rb, a.u2Cb, a.GRb, h->twm, d));
        CK(launch_adj_sigma(s, h->GR, h->LR, a.SigInb, a.SigRb, a.LRb, a.Lb, a.GRb, h->twm, h->twp, d));
        // L = symmetrised representatives (K2 groups; slots 0 = pp, 2 = ph)
        {
            const cplx* ob[3] = {a.Lb, nullptr, a.Lb + h->n2};
            const Group* grp[3] = {&h->gK2pp, &h->gK2pp, &h->gK2ph};
            CK(cudaMemsetAsync(a.raw2, 0, 3 * h->n2 * sizeof(cplx), s));
            Finalize3 f{};
            f.raw[0] = ob[0]; f.out[0] = a.raw2; f.map[0] = grp[0]->trivial ? nullptr : grp[0]->d_map;
            f.raw[2] = ob[2]; f.out[2] = a.raw2 + h->n2; f.map[2] = grp[2]->trivial ? nullptr : grp[2]->d_map;
            CK(launch_adj_finalize3(s, f, 0, 0, h->n2, nullptr));
            ChanWork cw{};
            const Group* g2[2] = {&h->gK2pp, &h->gK2ph};
            for (int w = 0; w < 2; ++w) {
                cw.items[w] = g2[w]->trivial ? nullptr : g2[w]->d_items;
                cw.nitems[w] = g2[w]->trivial ? (int)h->n2 : g2[w]->nitems;
            }
            const double rs = h->ref_nonzero ? 1.0 / 3.0 : 0.0;
            CK(launch_adj_sde_L(s, Fn, Yb, B, h->SPi, h->SPi + nS, a.Pbpp, a.Pbph, a.SPib, a.SPib + nS, a.raw2, cw,
                                h->n2, rs, d));
        }
    } else {
        CK(cudaMemcpyAsync(Sbar_in, sigmaOf(h, a.yb), h->nGk * sizeof(cplx), cudaMemcpyDeviceToDevice, s));
    }
    const int order[3] = {CH_P, CH_A, CH_T};
    auto Pi = [&](int ch) -> const cplx* { return ch == CH_P ? h->Pipp : h->Piph; };
    auto Pi0 = [&](int ch) -> const cplx* { return ch == CH_P ? h->Pi0pp : h->Pi0ph; };
    cplx* cb[10];
    for (int i = 0; i < 10; ++i) cb[i] = a.cacheb + (size_t)i * h->n3;
    Caches C{};
    for (int i = 0; i < 10; ++i) C.c[i] = h->cache + (size_t)i * h->n3;
    cplx* FL3b[3] = {a.FLK3b, a.FLK3b + h->n3, a.FLK3b + 2 * h->n3};
    cplx* FL2b[3] = {a.FLK2b, a.FLK2b + h->n2, a.FLK2b + 2 * h->n2};
    {  // K3 outputs -> representatives -> the K3 GEMM transposed (caches F and Γ, Π, FL.K3)
        const cplx* ob[3] = {chanK(h, a.yb, CH_P, 3), chanK(h, a.yb, CH_T, 3), chanK(h, a.yb, CH_A, 3)};
        const Group* grp[3] = {&h->gK3pp, &h->gK3ph, &h->gK3ph};
        CK(fin_adj(ob, a.raw3, h->n3, grp, 0, 1, nullptr));
        K3Args3 a3{};
        const cplx* Ob[3];
        cplx *Ab[3], *Gb[3], *Mb[3], *Mbb[3];
        for (int i = 0; i < 3; ++i) {
            const int ch = order[i];
            const int cg = ch == CH_P ? 0 : (ch == CH_A ? 5 : 6), cf = ch == CH_P ? 7 : (ch == CH_A ? 8 : 9);
            const int cf0 = ch == CH_P ? 1 : (ch == CH_A ? 2 : 3);
            K3Args& k = a3.a[i];
            k.A = C.c[cf]; k.B0 = C.c[cf0]; k.G = C.c[cg]; k.Pi = Pi(ch); k.Pi0 = Pi0(ch);
            k.FLc = h->FLK3 + (size_t)ch * h->n3; k.FLt = h->FLK3 + (size_t)CH_T * h->n3;
            k.FLa = h->FLK3 + (size_t)CH_A * h->n3;
            a3.ch[i] = ch;
            Ob[i] = a.raw3 + (size_t)ch * h->n3;
            Ab[i] = cb[cf];
            Gb[i] = cb[cg];
            Mb[i] = a.M + (size_t)i * h->n3;
            Mbb[i] = a.Mb + (size_t)i * h->n3;
        }
        a3.blocks = h->d_k3blocks;
        a3.nblocks = h->nk3blocks;
        CK(launch_adj_K3(s, 1, a3, Ob, Ab, Gb, Mb, Mbb, a.Pbpp, a.Pbph, FL3b, d));
    }
    {  // K2 outputs (with the FL epilogue) and K2 BSE transposed
        const cplx* ob[3] = {chanK(h, a.yb, CH_P, 2), chanK(h, a.yb, CH_T, 2), chanK(h, a.yb, CH_A, 2)};
        const Group* grp[3] = {&h->gK2pp, &h->gK2ph, &h->gK2ph};
        CK(fin_adj(ob, a.raw2, h->n2, grp, 1, 1, FL2b));
        CK(launch_adj_K2(s, F, FL, B, h->SX, Xb, FLb, a.Pbpp, a.Pbph, a.SXb, a.raw2, work(2), h->n2, d));
    }
    {  // K1
        const cplx* ob[3] = {chanK(h, a.yb, CH_P, 1), chanK(h, a.yb, CH_T, 1), chanK(h, a.yb, CH_A, 1)};
        const Group* grp[3] = {&h->gK1, &h->gK1, &h->gK1};
        CK(fin_adj(ob, a.raw1, h->n1, grp, 0, 1, nullptr));
        CK(launch_adj_K1(s, F, FL, B, h->SX, Xb, FLb, a.Pbpp, a.Pbph, a.SXb, a.raw1, work(1), h->n1, d));
    }
    CK(launch_adj_sx(s, h->Pipp, h->Piph, FL, a.SXb, a.Pbpp, a.Pbph, a.SPib, FLb, d));
    if (strategy == FDGA_FDPA) {  // FL is iterated only in fdPA
        {  // FL.K3 = L_K3(Γ caches)
            const cplx* ob[3] = {FL3b[CH_P], FL3b[CH_T], FL3b[CH_A]};
            const Group* grp[3] = {&h->gK3ppL, &h->gK3phL, &h->gK3phL};
            CK(fin_adj(ob, a.raw3, h->n3, grp, 0, 1, nullptr));
            K3Args3 a3{};
            const cplx* Ob[3];
            cplx *Ab[3], *Mb[3], *Mbb[3];
            for (int i = 0; i < 3; ++i) {
                const int ch = order[i];
                const int cg = ch == CH_P ? 4 : (ch == CH_A ? 5 : 6), cf0 = ch == CH_P ? 1 : (ch == CH_A ? 2 : 3);
                K3Args& k = a3.a[i];
                k.A = C.c[cg]; k.B0 = C.c[cf0]; k.Pi0 = Pi0(ch);
                a3.ch[i] = ch;
                Ob[i] = a.raw3 + (size_t)ch * h->n3;
                Ab[i] = cb[cg];
                Mb[i] = a.M + (size_t)i * h->n3;
                Mbb[i] = a.Mb + (size_t)i * h->n3;
            }
            a3.blocks = h->d_k3blocks;
            a3.nblocks = h->nk3blocks;
            CK(launch_adj_K3(s, 0, a3, Ob, Ab, nullptr, Mb, Mbb, nullptr, nullptr, nullptr, d));
        }
        {  // FL.K2 = L_K2(F)
            const cplx* ob[3] = {FL2b[CH_P], FL2b[CH_T], FL2b[CH_A]};
            const Group* grp[3] = {&h->gK2pp, &h->gK2ph, &h->gK2ph};
            CK(fin_adj(ob, a.raw2, h->n2, grp, 0, 1, nullptr));
            CK(launch_adj_L_K2(s, B, Xb, a.raw2, work(2), h->n2, d));
        }
    }
    {  // caches
        Caches Cb{};
        for (int i = 0; i < 10; ++i) Cb.c[i] = cb[i];
        CK(launch_adj_cache(s, Xb, Cb, h->d_k3blocks, h->nk3blocks, d));
    }
    if (update_sigma) {  // bubbles and row sums -> Ḡ(R) -> Ḡ -> Σ̄ (Dyson)
        CK(launch_adj_bubble(s, h->GR, a.Pbpp, a.Pbph, a.PbRpp, a.PbRph, a.SPib, a.SRb, a.GRb, h->twm, d));
        CK(launch_fft2(s, a.GRb, a.Gb, d.NG, +1, 1.0 / ((double)d.L * d.L), h->twp, d));
        if (hartree) CK(launch_adj_occupation(s, a.Gb, a.nbar, d.T, d.Nk, h->nGk));
        CK(launch_adj_dyson(s, h->G, a.Gb, Sbar_in, h->nGk));
    }
    if (d.Nq > 1) {  // momentum averages
        ChanBarArrays bar{};
        const size_t per1 = d.N1, per2 = (size_t)d.N2O * d.N2n, per3 = (size_t)d.N3O * d.N3n * d.N3n;
        for (int c = 0; c < 3; ++c) {
            const cplx* av = a.avgb + (size_t)c * (per1 + per2 + per3);
            bar.A1[c] = av; bar.A2[c] = av + per1; bar.A3[c] = av + per1 + per2;
            bar.K1[c] = Xb.g[c].K1; bar.K2[c] = Xb.g[c].K2; bar.K3[c] = Xb.g[c].K3;
        }
        CK(launch_adj_qavg(s, bar, d));
    }
    return FDGA_OK;
}

// the adjoint map as one CUDA graph per (strategy, flags), replayed at the base point the last FP64
// map left in the handle, on the cotangent in adj.yb
int run_adjoint(fdga_handle* h, int strategy, bool update_sigma, bool hartree) {
    Graph& g = h->adj.graphs[strategy][update_sigma][hartree];
    if (!g.exec) {
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
        int r = enqueue_adjoint(h, strategy, update_sigma, hartree);
        cudaError_t ee = cudaStreamEndCapture(h->st, &graph);
        if (r) {
            if (ee == cudaSuccess) cudaGraphDestroy(graph);
            return r;
        }
        if (ee != cudaSuccess) return cuda_fail(h, ee, "cudaStreamEndCapture (adjoint)");
        ee = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ee != cudaSuccess) { g.exec = nullptr; return cuda_fail(h, ee, "cudaGraphInstantiate (adjoint)"); }
    }
    CK(cudaGraphLaunch(g.exec, h->st));
    return FDGA_OK;
}

// Strategies of iterate_solver! (src/solve.jl:10): the _new forms exist for the local solver
// (src/BSEa/BSEa_K1.jl:57, BSEa_K2.jl:108), the one-loop form for the nonlocal one
// (src/nonlocal/BSEa/BSE_1loop.jl); elsewhere the reference has no method for them.
// (also allocates the zero FL of the one-loop form, outside any graph capture)
int check_strategy(fdga_handle* h, int strategy) {
    if (strategy < FDGA_FDPA || strategy > FDGA_FDPA_1LOOP) return fail(h, FDGA_ERR_ARG, "unknown strategy");
    if ((strategy == FDGA_FDPA_NEW || strategy == FDGA_SCPA_NEW) && !h->d.local)
        return fail(h, FDGA_ERR_UNSUPPORTED, "the :fdPA_new / :scPA_new BSEs exist for the local solver only");
    if (strategy == FDGA_FDPA_1LOOP && h->d.local)
        return fail(h, FDGA_ERR_UNSUPPORTED, "the :fdPA_1loop BSEs exist for the nonlocal solver only");
    if (strategy == FDGA_FDPA_1LOOP && !h->FLzero) {
        AL(h->FLzero, 3 * h->n2);
        AL(h->FLzerof, 3 * h->n2);
    }
    return FDGA_OK;
}

// Constant reference-system part of the fdPA SDE: C0 = SDE(F0, G0, Π0) without Hartree.
int compute_C0(fdga_handle* h) {
    cudaStream_t s = h->st;
    const Dims& d = h->d;
    int nl = 0;
    // only the reference-vertex fields are read: the RefVertex part (/3) and, for a Vertex F0, its
    // channels (use_vertex bit 2: the Vertex level of the recursion SDE!(Σ, G0, …, F0, …), src/SDE.jl:35-48)
    VertP F0 = vertex_view(h, h->yS);
    BubbleP B0{h->Pi0pp, h->Pi0ph, h->Pi0pp, h->Pi0ph};
    LC(sde_L_pair(h, F0, B0, h->SPi0, h->has0 ? 2 : 0, 1.0 / 3.0, nl));
    LC(launch_g_realspace(s, h->G0, h->GR, h->twm, d));
    LC(launch_sde_sigma(s, h->GR, h->Lpp, h->Lph, h->LR, h->SigR, h->SigIn, h->twm, h->twp, d));
    LC(launch_u2(s, h->GR, h->u2C, h->u2R, h->SigU2, h->twp, d));
    LC(launch_sigma_assemble(s, h->SigIn, h->SigU2, h->gSig.trivial ? nullptr : h->gSig.d_map, h->occ, nullptr,
                             nullptr, h->C0, d.U, 0, 0, 0.0, h->nGk));
    LC(launch_occupation(s, h->G0, h->nGk, d.T, d.Nk, h->occ));
    double n0 = 0.5;
    CK(cudaMemcpyAsync(&n0, h->occ, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    h->n0 = n0;
    h->c0_dirty = false;
    (void)nl;
    return FDGA_OK;
}

template <class A>
void drop_graph_array(A& gs) {
    for (auto& p : gs)
        for (auto& a : p)
            for (auto& b : a)
                for (auto& g : b)
                    if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
}
void drop_graphs(fdga_handle* h) {
    drop_graph_array(h->graphs);
    drop_graph_array(h->tan.graphs);
    for (auto& a : h->adj.graphs)
        for (auto& b : a)
            for (auto& g : b)
                if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
    for (auto& g : h->mf.graphs)
        if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
    for (auto& kv : h->kr_graphs)
        if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    h->kr_graphs.clear();
    if (h->rg.g.exec) cudaGraphExecDestroy(h->rg.g.exec);
    h->rg.g = Graph();
    h->rg.x = nullptr;
    h->rg.R = nullptr;
}

int run_iteration(fdga_handle* h, int strategy, bool update_sigma, bool hartree) {
    if (!h->finalized) return fail(h, FDGA_ERR_STATE, "fdga_finalize has not been called");
    int r0 = check_strategy(h, strategy);
    if (r0) return r0;
    if (h->c0_dirty) {
        int r = compute_C0(h);
        if (r) return r;
    }
    Graph& g = h->graphs[h->precision][strategy][update_sigma][hartree];
    if (!g.exec) {
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
        int nl = 0;
        int r = enqueue_iteration(h, strategy, update_sigma, hartree, nl);
        cudaError_t ee = cudaStreamEndCapture(h->st, &graph);
        if (r) {
            if (ee == cudaSuccess) cudaGraphDestroy(graph);
            return r;
        }
        if (ee != cudaSuccess) return cuda_fail(h, ee, "cudaStreamEndCapture");
        ee = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ee != cudaSuccess) { g.exec = nullptr; return cuda_fail(h, ee, "cudaGraphInstantiate"); }
        g.nodes = nl;
    }
    CK(cudaGraphLaunch(g.exec, h->st));
    h->last_launches = g.nodes;
    return FDGA_OK;
}

double reduce_max(fdga_handle* h, int nblk, int& status) {
    std::vector<double> part(nblk);
    cudaError_t e = cudaMemcpyAsync(part.data(), h->d_part, nblk * sizeof(double), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess) { status = cuda_fail(h, e, "reduce_max"); return 0.0; }
    double m = 0.0;  // the partials are squared magnitudes
    for (double v : part) m = std::max(m, v);
    status = FDGA_OK;
    return std::sqrt(m);
}

bool names_vertex(const std::string& n, std::string& vn, int& ch, int& cls) {
    const size_t dot_ = n.find('.');
    if (dot_ == std::string::npos || n.size() != dot_ + 5) return false;
    vn = n.substr(0, dot_);
    const char c = n[dot_ + 1];
    ch = c == 'p' ? CH_P : (c == 't' ? CH_T : (c == 'a' ? CH_A : -1));
    if (ch < 0 || n[dot_ + 2] != '.' || n[dot_ + 3] != 'K') return false;
    cls = n[dot_ + 4] - '0';
    return cls >= 1 && cls <= 3;
}

// named array -> (device pointer, kind, length)
bool lookup(fdga_handle* h, const std::string& n, cplx*& p, int& kind, size_t& len) {
    if (n == "G") { p = h->G; kind = AK_G; len = h->nGk; return true; }
    if (n == "Sigma") { p = sigmaOf(h, h->xS); kind = AK_G; len = h->nGk; return true; }
    if (n == "Gbare") { p = h->Gbare; kind = AK_G; len = h->nGk; return true; }
    if (n == "G0") { p = h->G0; kind = AK_G; len = h->nGk; return true; }
    if (n == "Sigma0") { p = h->Sig0; kind = AK_G; len = h->nGk; return true; }
    const size_t nPiFull = (size_t)h->d.NPO * h->d.NPn * h->d.Nq;
    if (n == "Pipp") { p = h->Pipp; kind = AK_PI; len = nPiFull; return true; }
    if (n == "Piph") { p = h->Piph; kind = AK_PI; len = nPiFull; return true; }
    if (n == "Pi0pp") { p = h->Pi0pp; kind = AK_PI; len = nPiFull; return true; }
    if (n == "Pi0ph") { p = h->Pi0ph; kind = AK_PI; len = nPiFull; return true; }
    if (n == "Lpp") { p = h->Lpp; kind = AK_K2; len = h->n2; return true; }
    if (n == "Lph") { p = h->Lph; kind = AK_K2; len = h->n2; return true; }
    static const char* cn[10] = {"cache_Gpx", "cache_F0p", "cache_F0a", "cache_F0t", "cache_Gpp",
                                 "cache_Ga",  "cache_Gt",  "cache_Fp",  "cache_Fa",  "cache_Ft"};
    for (int i = 0; i < 10; ++i)
        if (n == cn[i]) { p = h->cache + (size_t)i * h->n3; kind = AK_K3; len = h->n3; return true; }
    std::string vn;
    int ch, cls;
    if (!names_vertex(n, vn, ch, cls)) return false;
    if (vn == "F") {
        p = chanK(h, h->xS, ch, cls);
    } else if (vn == "FL") {
        if (cls == 1) return false;
        p = cls == 2 ? h->FLK2 + (size_t)ch * h->n2 : h->FLK3 + (size_t)ch * h->n3;
    } else {
        return false;
    }
    kind = cls == 1 ? AK_K1 : (cls == 2 ? AK_K2 : AK_K3);
    len = cls == 1 ? h->n1 : (cls == 2 ? h->n2 : h->n3);
    return true;
}


// FDGA_IN_F0_VERTEX: flatten(F0) of a Vertex-valued reference vertex (reference column-major layout,
// src/vertex.jl:152-165) permuted into the device layout of its boxes; then its momentum averages
// (kSW) and, when the mixed map's buffers exist, its FP32 copies.  F0 is constant over the solve.
int set_f0_vertex(fdga_handle* h, const double* re_im, size_t n) {
    if (!h->has0) return fail(h, FDGA_ERR_ARG, "the handle's reference vertex is a RefVertex (f0_vertex = 0)");
    if (n != 3 * h->n0chan)
        return fail(h, FDGA_ERR_ARG, "F0 vertex size mismatch: got " + std::to_string(n) + ", expected " +
                                         std::to_string(3 * h->n0chan));
    for (size_t i = 0; i < 2 * n; ++i)
        if (!std::isfinite(re_im[i])) return fail(h, FDGA_ERR_NONFINITE, "non-finite value in the F0 vertex");
    const Dims d0 = f0_dims(h->d, h->b0);
    const cplx* in = reinterpret_cast<const cplx*>(re_im);
    std::vector<cplx> dev(n);
    size_t j = 0;
    for (int c = 0; c < 3; ++c) {  // γp, γt, γa
        const size_t off = (size_t)c * h->n0chan;
        for (size_t i = 0; i < h->n0_1; ++i) dev[off + dev_index(d0, AK_K1, i)] = in[j++];
        for (size_t i = 0; i < h->n0_2; ++i) dev[off + h->n0_1 + dev_index(d0, AK_K2, i)] = in[j++];
        for (size_t i = 0; i < h->n0_3; ++i) dev[off + h->n0_1 + h->n0_2 + dev_index(d0, AK_K3, i)] = in[j++];
    }
    cudaStream_t s = h->st;
    CK(cudaMemcpyAsync(h->F0v, dev.data(), n * sizeof(cplx), cudaMemcpyHostToDevice, s));
    if (h->d.Nq > 1) {
        ChanArrays a;
        ChanArraysW o;
        const size_t per1 = h->b0.N1, per2 = (size_t)h->b0.N2O * h->b0.N2n;
        const size_t per3 = (size_t)h->b0.N3O * h->b0.N3n * h->b0.N3n;
        for (int c = 0; c < 3; ++c) {
            cplx* base = h->F0v + (size_t)c * h->n0chan;
            a.K1[c] = base; a.K2[c] = base + h->n0_1; a.K3[c] = base + h->n0_1 + h->n0_2;
            cplx* av = h->F0avg + (size_t)c * (per1 + per2 + per3);
            o.K1[c] = av; o.K2[c] = av + per1; o.K3[c] = av + per1 + per2;
        }
        CK(launch_qavg(s, a, o, d0));
    }
    if (h->F0vf) {
        CK(launch_to_f32(s, h->F0v, h->F0vf, 3 * h->n0chan));
        if (h->n0avg) CK(launch_to_f32(s, h->F0avg, h->F0avgf, h->n0avg));
    }
    CK(cudaStreamSynchronize(s));
    h->c0_dirty = true;
    drop_graphs(h);
    return FDGA_OK;
}

}  // namespace

// =============================================================================================
// C ABI
// =============================================================================================
extern "C" {

const char* fdga_create_error(void) { return g_create_error.c_str(); }
const char* fdga_last_error(const fdga_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int fdga_create(const fdga_config* c, fdga_handle** out) {
    if (!c || !out) { g_create_error = "null argument"; return FDGA_ERR_ARG; }
    *out = nullptr;
    auto bad = [&](const std::string& m) { g_create_error = m; return FDGA_ERR_ARG; };
    if (c->nG < 1 || c->nK1 < 1 || c->nK2[0] < 1 || c->nK2[1] < 1 || c->nK3[0] < 1 || c->nK3[1] < 1)
        return bad("mesh sizes must be >= 1");
    if (c->nK1 < c->nK2[0] || c->nK1 < c->nK2[1])
        return bad("No. bosonic frequencies in K1 must be larger than the K2 box (src/channel.jl:33-34)");
    if (c->nK2[0] < c->nK3[0] || c->nK2[1] < c->nK3[1])
        return bad("Number of frequencies in K2 must be larger than in K3 (src/channel.jl:40)");
    if (c->L < 1 || c->mPi_factor < 1 || !(c->T > 0)) return bad("L, mPi_factor and T must be positive");
    if (c->local && c->L != 1) return bad("the local solver has L = 1");
    if (c->LG != c->L) { g_create_error = "L_G != L is not supported by this build"; return FDGA_ERR_UNSUPPORTED; }
    if (c->precision != FDGA_FP64 && c->precision != FDGA_MIXED) {
        g_create_error = "precision must be FDGA_FP64 or FDGA_MIXED";
        return FDGA_ERR_ARG;
    }
    if (c->nR[0] < 1 || c->nR[1] < 1) return bad("RefVertex box must be >= 1");
    if (c->f0_vertex != 0 && c->f0_vertex != 1) return bad("f0_vertex must be 0 or 1");
    if (c->f0_vertex) {
        if (c->nF0K1 < 1 || c->nF0K2[0] < 1 || c->nF0K2[1] < 1 || c->nF0K3[0] < 1 || c->nF0K3[1] < 1)
            return bad("the boxes of the Vertex F0 must be >= 1");
        if (c->nF0K1 < c->nF0K2[0] || c->nF0K1 < c->nF0K2[1])
            return bad("F0: No. bosonic frequencies in K1 must be larger than the K2 box (src/channel.jl:33-34)");
        if (c->nF0K2[0] < c->nF0K3[0] || c->nF0K2[1] < c->nF0K3[1])
            return bad("F0: Number of frequencies in K2 must be larger than in K3 (src/channel.jl:40)");
    }
    fdga_handle* h = new fdga_handle();
    h->cfg = *c;
    h->precision = FDGA_FP64;  // the config's precision is applied once the buffers exist (below)
    make_dims(c, h->d);
    Dims& d = h->d;
    h->nGk = (size_t)d.NG * d.Nk;
    h->n1 = (size_t)d.N1 * d.Nq;
    h->n2 = (size_t)d.N2O * d.N2n * d.Nq;
    h->n3 = (size_t)d.N3O * d.N3n * d.N3n * d.Nq;
    h->nPi = (size_t)d.NPO * d.NPw * d.Nq;
    h->nRef = (size_t)d.NRO * d.NRn * d.NRn;
    h->nchan = h->n1 + h->n2 + h->n3;
    h->nstate = 3 * h->nchan + h->nGk;
    if (c->f0_vertex) {
        Box& b = h->b0;
        b.n1 = c->nF0K1; b.N1 = 2 * c->nF0K1 - 1;
        b.n2O = c->nF0K2[0]; b.N2O = 2 * c->nF0K2[0] - 1; b.n2n = c->nF0K2[1]; b.N2n = 2 * c->nF0K2[1];
        b.n3O = c->nF0K3[0]; b.N3O = 2 * c->nF0K3[0] - 1; b.n3n = c->nF0K3[1]; b.N3n = 2 * c->nF0K3[1];
        h->has0 = true;
        h->n0_1 = (size_t)b.N1 * d.Nq;
        h->n0_2 = (size_t)b.N2O * b.N2n * d.Nq;
        h->n0_3 = (size_t)b.N3O * b.N3n * b.N3n * d.Nq;
        h->n0chan = h->n0_1 + h->n0_2 + h->n0_3;
        if (d.Nq > 1) h->n0avg = 3 * ((size_t)b.N1 + (size_t)b.N2O * b.N2n + (size_t)b.N3O * b.N3n * b.N3n);
    }
    if (h->nstate >= ((size_t)1 << 32) || h->n3 >= ((size_t)1 << 30)) {
        delete h;
        g_create_error = "problem too large for 32-bit index maps";
        return FDGA_ERR_UNSUPPORTED;
    }
    int r = FDGA_OK;
    auto fin_err = [&](int code) { g_create_error = h->err; fdga_destroy(h); return code; };
    if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess || set_fft_twiddles() != cudaSuccess) {
        g_create_error = "cudaStreamCreate failed (no CUDA device?)";
        delete h;
        return FDGA_ERR_CUDA;
    }
    for (auto& e : h->ev) cudaEventCreate(&e);
    if (cudaStreamCreateWithFlags(&h->st2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->st3, cudaStreamNonBlocking) != cudaSuccess) {
        g_create_error = "cudaStreamCreate failed";
        fdga_destroy(h);
        return FDGA_ERR_CUDA;
    }
    for (cudaEvent_t* e : {&h->evfork, &h->evA, &h->evB, &h->evC, &h->evD, &h->evE, &h->evR})
        cudaEventCreateWithFlags(e, cudaEventDisableTiming);
#define ALC(ptr, n) do { r = dalloc(h, &(ptr), (n)); if (r) return fin_err(r); } while (0)
    ALC(h->Gbare, h->nGk); ALC(h->G0, h->nGk); ALC(h->Sig0, h->nGk); ALC(h->G, h->nGk);
    ALC(h->Pi0pp, h->nPi); ALC(h->Pi0ph, h->nPi); ALC(h->Pipp, h->nPi); ALC(h->Piph, h->nPi);
    for (auto& f : h->Fref) ALC(f, h->nRef);
    ALC(h->xS, h->nstate); ALC(h->yS, h->nstate); ALC(h->tmpS, h->nstate);
    if (d.Nq > 1) {
        h->navg = 3 * ((size_t)d.N1 + (size_t)d.N2O * d.N2n + (size_t)d.N3O * d.N3n * d.N3n);
        ALC(h->avg, h->navg);
    }
    if (h->has0) {
        ALC(h->F0v, 3 * h->n0chan);
        if (h->n0avg) ALC(h->F0avg, h->n0avg);
    }
    ALC(h->cache, 10 * h->n3);
    ALC(h->FLK2, 3 * h->n2); ALC(h->FLK3, 3 * h->n3);
    ALC(h->Lpp, h->n2); ALC(h->Lph, h->n2); ALC(h->SigIn, h->nGk); ALC(h->SigU2, h->nGk); ALC(h->C0, h->nGk);
    ALC(h->GR, h->nGk); ALC(h->u2C, (size_t)d.Nq * (2 * d.NG - 1)); ALC(h->u2R, h->nGk);
    ALC(h->twm, d.L); ALC(h->twp, d.L);
    ALC(h->SPi, 2 * (size_t)d.Nq * d.NPO); ALC(h->SPi0, 2 * (size_t)d.Nq * d.NPO); ALC(h->SX, 3 * (size_t)d.Nq * d.NPO);
    ALC(h->SRtmp, 2 * (size_t)d.NPO * d.Nq);
    ALC(h->T0tail, 2 * (size_t)d.NPO);
    ALC(h->LR, 2 * h->n2); ALC(h->SigR, h->nGk);
    ALC(h->raw1, 3 * h->n1); ALC(h->raw2, 3 * h->n2); ALC(h->raw3, 3 * h->n3);
    h->nk3blocks = d.Nq * d.N3O;
    ALC(h->occ, 1);
    ALC(h->perm, h->nstate);
    ALC(h->d_part, NBLK_RED);
    // the zero-fills of dalloc are queued on the (non-blocking) solver stream: finish them before
    // any upload, and keep the uploads on the same stream
    if (cudaStreamSynchronize(h->st) != cudaSuccess) return fin_err(fail(h, FDGA_ERR_CUDA, "create sync"));
    {
        std::vector<cplx> tm(d.L), tp(d.L);
        for (int j = 0; j < d.L; ++j) {
            const double a = 2.0 * M_PI * j / d.L;
            tm[j] = mk(std::cos(a), -std::sin(a));
            tp[j] = mk(std::cos(a), std::sin(a));
        }
        if (cudaMemcpyAsync(h->twm, tm.data(), d.L * sizeof(cplx), cudaMemcpyHostToDevice, h->st) != cudaSuccess ||
            cudaMemcpyAsync(h->twp, tp.data(), d.L * sizeof(cplx), cudaMemcpyHostToDevice, h->st) != cudaSuccess)
            return fin_err(fail(h, FDGA_ERR_CUDA, "twiddle upload"));
        // flatten permutation
        std::vector<uint32_t> perm(h->nstate);
        size_t j = 0;
        for (int ch : {CH_P, CH_T, CH_A}) {
            const size_t off = (size_t)ch * h->nchan;
            for (size_t i = 0; i < h->n1; ++i) perm[j++] = (uint32_t)(off + dev_index(h->d, AK_K1, i));
            for (size_t i = 0; i < h->n2; ++i) perm[j++] = (uint32_t)(off + h->n1 + dev_index(h->d, AK_K2, i));
            for (size_t i = 0; i < h->n3; ++i) perm[j++] = (uint32_t)(off + h->n1 + h->n2 + dev_index(h->d, AK_K3, i));
        }
        for (size_t i = 0; i < h->nGk; ++i) perm[j++] = (uint32_t)(3 * h->nchan + i);
        if (cudaMemcpyAsync(h->perm, perm.data(), h->nstate * sizeof(uint32_t), cudaMemcpyHostToDevice, h->st) !=
                cudaSuccess ||
            cudaStreamSynchronize(h->st) != cudaSuccess)
            return fin_err(fail(h, FDGA_ERR_CUDA, "permutation upload"));
    }
#undef ALC
    if (cudaStreamSynchronize(h->st) != cudaSuccess) return fin_err(fail(h, FDGA_ERR_CUDA, "create sync"));
    if (c->precision == FDGA_MIXED) {
        if ((r = ensure_mixed(h))) return fin_err(r);
        h->precision = FDGA_MIXED;
    }
    *out = h;
    return FDGA_OK;
}

void fdga_destroy(fdga_handle* h) {
    if (!h) return;
    if (h->st) cudaStreamSynchronize(h->st);
    drop_graphs(h);
    if (h->flush_buf) cudaFree(h->flush_buf);
    if (h->kr_st_host) cudaFreeHost(h->kr_st_host);
    for (void* p : h->allocs) cudaFree(p);
    for (auto& e : h->ev) if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : {h->evfork, h->evA, h->evB, h->evC, h->evD, h->evE, h->evR}) if (e) cudaEventDestroy(e);
    for (cudaStream_t t : {h->st2, h->st3}) if (t) { cudaStreamSynchronize(t); cudaStreamDestroy(t); }
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
}

int fdga_set_input(fdga_handle* h, int which, const double* re_im, size_t n) {
    if (!h || !re_im) return fail(h, FDGA_ERR_ARG, "null argument");
    if (which == FDGA_IN_F0_VERTEX) return set_f0_vertex(h, re_im, n);
    cplx* dst = nullptr;
    size_t len = 0;
    switch (which) {
        case FDGA_IN_GBARE: dst = h->Gbare; len = h->nGk; break;
        case FDGA_IN_G0: dst = h->G0; len = h->nGk; break;
        case FDGA_IN_SIGMA0: dst = h->Sig0; len = h->nGk; break;
        case FDGA_IN_FP_P: case FDGA_IN_FP_X: case FDGA_IN_FT_P: case FDGA_IN_FT_X:
            dst = h->Fref[which - FDGA_IN_FP_P]; len = h->nRef; break;
        default: return fail(h, FDGA_ERR_ARG, "unknown input id");
    }
    if (n != len) return fail(h, FDGA_ERR_ARG, "input size mismatch: got " + std::to_string(n) + ", expected " + std::to_string(len));
    for (size_t i = 0; i < 2 * n; ++i)
        if (!std::isfinite(re_im[i])) return fail(h, FDGA_ERR_NONFINITE, "non-finite value in input");
    if (which >= FDGA_IN_FP_P) {
        for (size_t i = 0; i < 2 * n; ++i) if (re_im[i] != 0.0) { h->ref_nonzero = true; break; }
    }
    CK(cudaMemcpyAsync(dst, re_im, n * sizeof(cplx), cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    h->c0_dirty = true;
    drop_graphs(h);
    return FDGA_OK;
}

int fdga_finalize(fdga_handle* h) {
    if (!h) return FDGA_ERR_ARG;
    const Dims& d = h->d;
    cudaStream_t s = h->st;
    CK(launch_g_realspace(s, h->G0, h->GR, h->twm, d));
    CK(launch_bubble(s, h->G0, h->GR, h->Pi0pp, h->Pi0ph, h->twp, d));
    const size_t nS = (size_t)d.Nq * d.NPO;
    CK(launch_tail_const(s, h->T0tail, d));
    CK(launch_rowsum(s, h->Pi0pp, h->Pi0ph, h->GR, h->SRtmp, h->twp, h->SPi0, h->SPi0 + nS, d, h->T0tail));
    CK(cudaMemsetAsync(h->xS, 0, h->nstate * sizeof(cplx), s));
    CK(cudaMemsetAsync(h->yS, 0, h->nstate * sizeof(cplx), s));
    CK(cudaMemsetAsync(h->FLK2, 0, 3 * h->n2 * sizeof(cplx), s));
    CK(cudaMemsetAsync(h->FLK3, 0, 3 * h->n3 * sizeof(cplx), s));
    CK(cudaMemcpyAsync(sigmaOf(h, h->xS), h->Sig0, h->nGk * sizeof(cplx), cudaMemcpyDeviceToDevice, s));
    CK(launch_dyson(s, h->G, sigmaOf(h, h->xS), h->Gbare, h->nGk));
    CK(launch_g_realspace(s, h->G, h->GR, h->twm, d));
    CK(launch_bubble(s, h->G, h->GR, h->Pipp, h->Piph, h->twp, d));
    CK(launch_rowsum(s, h->Pipp, h->Piph, h->GR, h->SRtmp, h->twp, h->SPi, h->SPi + nS, d, h->T0tail));
    if (k3_oz_supported(d)) {
        if (int r = ensure_k3_oz(h)) return r;
        CK(prepare_bse_K3_oz());
    }
    CK(cudaStreamSynchronize(s));
    h->finalized = true;
    h->c0_dirty = true;
    return FDGA_OK;
}

}  // extern "C"

namespace {
// Dyson! and bubbles! (with the full-mesh row sums) of the current state's Σ
int dyson_bubbles(fdga_handle* h) {
    const Dims& d = h->d;
    cudaStream_t s = h->st;
    const size_t nS = (size_t)d.Nq * d.NPO;
    CK(launch_dyson(s, h->G, sigmaOf(h, h->xS), h->Gbare, h->nGk));
    CK(launch_g_realspace(s, h->G, h->GR, h->twm, d));
    CK(launch_bubble(s, h->G, h->GR, h->Pipp, h->Piph, h->twp, d));
    CK(launch_rowsum(s, h->Pipp, h->Piph, h->GR, h->SRtmp, h->twp, h->SPi, h->SPi + nS, d, h->T0tail));
    CK(cudaStreamSynchronize(s));
    return FDGA_OK;
}
// symmetrize_solver! (src/ParquetSolver.jl:246-259): every element of a class takes its
// representative's value under the class operation (Σ and the K1/K2/K3 of the three channels)
int symmetrize_state(fdga_handle* h) {
    cudaStream_t s = h->st;
    CK(cudaMemcpyAsync(h->tmpS, h->xS, h->nstate * sizeof(cplx), cudaMemcpyDeviceToDevice, s));
    auto sym = [&](const Group& g, size_t off, size_t n) -> cudaError_t {
        if (g.trivial) return cudaSuccess;
        Finalize3 f{};
        f.raw[0] = h->tmpS + off;
        f.out[0] = h->xS + off;
        f.map[0] = g.d_map;
        return launch_finalize3(s, f, 0, 0, n);
    };
    CK(sym(h->gSig, 3 * h->nchan, h->nGk));
    for (int ch = 0; ch < 3; ++ch) {
        const size_t o = (size_t)ch * h->nchan;
        CK(sym(h->gK1, o, h->n1));
        CK(sym(ch == CH_P ? h->gK2pp : h->gK2ph, o + h->n1, h->n2));
        CK(sym(ch == CH_P ? h->gK3pp : h->gK3ph, o + h->n1 + h->n2, h->n3));
    }
    CK(cudaStreamSynchronize(s));
    return FDGA_OK;
}
}  // namespace

extern "C" {

int fdga_dyson_bubbles(fdga_handle* h) {
    if (!h) return FDGA_ERR_ARG;
    if (!h->finalized) return fail(h, FDGA_ERR_STATE, "fdga_finalize has not been called");
    return dyson_bubbles(h);
}

int fdga_interpolate_solver(fdga_handle* ho, fdga_handle* hi) {
    if (!ho || !hi) return fail(ho, FDGA_ERR_ARG, "null handle");
    if (ho == hi) return fail(ho, FDGA_ERR_ARG, "source and target must be different solvers");
    if (!ho->finalized || !hi->finalized) return fail(ho, FDGA_ERR_STATE, "fdga_finalize has not been called");
    if (ho->d.local || hi->d.local)
        return fail(ho, FDGA_ERR_UNSUPPORTED, "interpolate_solver! is defined for the nonlocal solver");
    if (ho->d.T != hi->d.T) return fail(ho, FDGA_ERR_ARG, "the two solvers must share the temperature");
    if (ho->d.L * ho->d.L != ho->d.Nk || hi->d.L * hi->d.L != hi->d.Nk)
        return fail(ho, FDGA_ERR_UNSUPPORTED, "Fourier interpolation needs L_G = L");
    const Dims &o = ho->d, &i = hi->d;
    fdga_handle* h = ho;  // errors are reported on the target
    CK(cudaStreamSynchronize(hi->st));
    cudaStream_t s = ho->st;
    // src/interpolate.jl:147-191: Σ, then Dyson and bubbles, then the vertex, then symmetrize
    CK(launch_fourier_interp(s, 0, sigmaOf(hi, hi->xS), sigmaOf(ho, ho->xS), o, i));
    if (int r = dyson_bubbles(ho)) return r;
    for (int ch = 0; ch < 3; ++ch)
        for (int cls = 1; cls <= 3; ++cls)
            CK(launch_fourier_interp(s, cls, chanK(hi, hi->xS, ch, cls), chanK(ho, ho->xS, ch, cls), o, i));
    return symmetrize_state(ho);
}

int fdga_init_sym_grp(fdga_handle* h) {
    if (!h) return FDGA_ERR_ARG;
    std::vector<HostGroup> hg;
    compute_all_groups(h->d, hg);
    ++h->groups_version;
    Group* dst[8] = {&h->gSig, &h->gK1, &h->gK2pp, &h->gK2ph, &h->gK3pp, &h->gK3ph, &h->gK3ppL, &h->gK3phL};
    for (int i = 0; i < 8; ++i) {
        int r = upload_group(h, *dst[i], hg[i], i == 2 || i == 3 ? h->d.N2n : 0);
        if (r) return r;
    }
    // (P, Ω) blocks of the K3 mesh that hold a representative of any K3 group: only these blocks
    // of the caches and of the K3 GEMMs are computed; k_finalize3 fills the rest.
    {
        const size_t bs = (size_t)h->d.N3n * h->d.N3n;
        std::vector<char> used((size_t)h->d.Nq * h->d.N3O, 0);
        for (int i = 4; i < 8; ++i)
            for (int r : hg[i].items) used[(size_t)r / bs] = 1;
        std::vector<int> blocks;
        for (size_t b = 0; b < used.size(); ++b)
            if (used[b]) blocks.push_back((int)b);
        if (!h->d_k3blocks) AL(h->d_k3blocks, used.size());
        CK(cudaMemcpyAsync(h->d_k3blocks, blocks.data(), blocks.size() * sizeof(int), cudaMemcpyHostToDevice, h->st));
        CK(cudaStreamSynchronize(h->st));
        h->nk3blocks = (int)blocks.size();
    }
    drop_graphs(h);
    h->c0_dirty = true;
    return FDGA_OK;
}

int fdga_group_map(const fdga_config* c, int which, uint32_t* map, size_t n, int* nclasses) {
    if (!c || which < 0 || which >= 8) return FDGA_ERR_ARG;
    Dims d;
    int r = make_dims(c, d);
    if (r) return r;
    std::vector<HostGroup> hg;
    compute_all_groups(d, hg);
    if (nclasses) *nclasses = (int)hg[which].items.size();
    if (map) {
        if (n != hg[which].map.size()) return FDGA_ERR_ARG;
        std::memcpy(map, hg[which].map.data(), n * sizeof(uint32_t));
    }
    return FDGA_OK;
}

int fdga_state_len(const fdga_handle* h, size_t* n) {
    if (!h || !n) return FDGA_ERR_ARG;
    *n = h->nstate;
    return FDGA_OK;
}

int fdga_flatten(fdga_handle* h, double* x, size_t n) {
    if (!h || !x) return fail(h, FDGA_ERR_ARG, "null argument");
    if (n != h->nstate) return fail(h, FDGA_ERR_ARG, "state length mismatch");
    CK(launch_gather(h->st, h->tmpS, h->xS, h->perm, n));
    CK(cudaMemcpyAsync(x, h->tmpS, n * sizeof(cplx), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return FDGA_OK;
}

int fdga_unflatten(fdga_handle* h, const double* x, size_t n) {
    if (!h || !x) return fail(h, FDGA_ERR_ARG, "null argument");
    if (n != h->nstate) return fail(h, FDGA_ERR_ARG, "state length mismatch");
    CK(cudaMemcpyAsync(h->tmpS, x, n * sizeof(cplx), cudaMemcpyHostToDevice, h->st));
    CK(launch_scatter(h->st, h->xS, h->tmpS, h->perm, n));
    CK(cudaStreamSynchronize(h->st));
    return FDGA_OK;
}

int fdga_iterate(fdga_handle* h, int strategy, int update_sigma, int compute_hartree) {
    if (!h) return FDGA_ERR_ARG;
    int r = run_iteration(h, strategy, update_sigma != 0, compute_hartree != 0);
    if (r) return r;
    CK(cudaMemcpyAsync(h->xS, h->yS, h->nstate * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    return check_device_error(h);
}

bool page_locked(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// fdga_residual as one graph when x and R are page-locked: the host copies become graph nodes that
// overlap the iteration.  Σ (the last flatten block, stored unpermuted at the end of the device
// state) is copied first, straight into place, so the Dyson/bubble branch starts while the vertex
// is still in flight; the vertex part of R = Φ(x) - x is formed and copied back on a side stream
// while the SDE computes the new Σ.  The state is left at Φ(x), as in the unfused path.
int residual_graph(fdga_handle* h, int strategy, const double* x, double* R) {
    int r0 = check_strategy(h, strategy);
    if (r0) return r0;
    if (h->c0_dirty) {
        int r = compute_C0(h);
        if (r) return r;
    }
    auto& rg = h->rg;
    if (rg.g.exec && (rg.x != x || rg.R != R || rg.precision != h->precision || rg.strategy != strategy)) {
        cudaGraphExecDestroy(rg.g.exec);
        rg.g = Graph();
    }
    if (!rg.g.exec) {
        cudaStream_t s = h->st, sE = h->st2;
        const size_t nv = 3 * h->nchan, nS = h->nGk;
        const cplx* xh = reinterpret_cast<const cplx*>(x);
        cplx* Rh = reinterpret_cast<cplx*>(R);
        IterHooks hk;
        hk.after_fork = [&]() -> int {
            CK(cudaMemcpyAsync(h->tmpS, xh, nv * sizeof(cplx), cudaMemcpyHostToDevice, s));
            CK(launch_scatter(s, h->xS, h->tmpS, h->perm, nv));
            return FDGA_OK;
        };
        hk.vertex_done = [&]() -> int {
            CK(cudaEventRecord(h->evR, s));
            CK(cudaStreamWaitEvent(sE, h->evR, 0));
            CK(launch_gather_sub(sE, h->tmpS, h->yS, h->xS, h->perm, nv));
            CK(cudaMemcpyAsync(Rh, h->tmpS, nv * sizeof(cplx), cudaMemcpyDeviceToHost, sE));
            CK(cudaEventRecord(h->evR, sE));
            return FDGA_OK;
        };
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int nl = 0, r = FDGA_OK;
        cudaError_t ee = cudaMemcpyAsync(sigmaOf(h, h->xS), xh + nv, nS * sizeof(cplx), cudaMemcpyHostToDevice, s);
        if (ee == cudaSuccess) r = enqueue_iteration(h, strategy, true, true, nl, StageHook(), &hk);
        if (ee == cudaSuccess && !r) ee = launch_sub(s, h->tmpS + nv, sigmaOf(h, h->yS), sigmaOf(h, h->xS), nS);
        if (ee == cudaSuccess && !r)
            ee = cudaMemcpyAsync(Rh + nv, h->tmpS + nv, nS * sizeof(cplx), cudaMemcpyDeviceToHost, s);
        if (ee == cudaSuccess && !r) ee = cudaStreamWaitEvent(s, h->evR, 0);
        if (ee == cudaSuccess && !r)
            ee = cudaMemcpyAsync(h->xS, h->yS, h->nstate * sizeof(cplx), cudaMemcpyDeviceToDevice, s);
        cudaError_t ec = cudaStreamEndCapture(s, &graph);
        if (r) {
            if (ec == cudaSuccess) cudaGraphDestroy(graph);
            return r;
        }
        if (ee != cudaSuccess) {
            if (ec == cudaSuccess) cudaGraphDestroy(graph);
            return cuda_fail(h, ee, "residual graph capture");
        }
        if (ec != cudaSuccess) return cuda_fail(h, ec, "cudaStreamEndCapture");
        ee = cudaGraphInstantiate(&rg.g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ee != cudaSuccess) { rg.g.exec = nullptr; return cuda_fail(h, ee, "cudaGraphInstantiate"); }
        rg.g.nodes = nl + 3;  // + scatter, gather-sub, sub
        rg.x = x;
        rg.R = R;
        rg.precision = h->precision;
        rg.strategy = strategy;
    }
    CK(cudaGraphLaunch(rg.g.exec, h->st));
    h->last_launches = rg.g.nodes;
    CK(cudaStreamSynchronize(h->st));
    return check_device_error(h);
}

int fdga_residual(fdga_handle* h, int strategy, const double* x, double* R, size_t n) {
    if (!h || !x || !R) return fail(h, FDGA_ERR_ARG, "null argument");
    if (n != h->nstate) return fail(h, FDGA_ERR_ARG, "state length mismatch");
    if (!h->finalized) return fail(h, FDGA_ERR_STATE, "fdga_finalize has not been called");
    if (h->fused_residual && page_locked(x) && page_locked(R)) return residual_graph(h, strategy, x, R);
    CK(cudaMemcpyAsync(h->tmpS, x, n * sizeof(cplx), cudaMemcpyHostToDevice, h->st));
    CK(launch_scatter(h->st, h->xS, h->tmpS, h->perm, n));
    int r = run_iteration(h, strategy, true, true);
    if (r) return r;
    // R = flatten(Φ(x)) - x, formed in device layout then permuted
    CK(launch_sub(h->st, h->tmpS, h->yS, h->xS, n));
    CK(cudaMemcpyAsync(h->xS, h->yS, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
    CK(launch_gather(h->st, h->yS, h->tmpS, h->perm, n));
    CK(cudaMemcpyAsync(R, h->yS, n * sizeof(cplx), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return check_device_error(h);
}

}  // extern "C"

namespace {

// Anderson solve hooks: before() runs ahead of each map evaluation, after() between the map and the
// residual (it may replace the new state y, e.g. by x + a preconditioned residual)
struct SolveHooks {
    std::function<int()> before, after;
};

int solve_anderson(fdga_handle* h, int strategy, bool update_sigma, int maxiter, double tol, double beta, int mem,
                   int* iters, double* res, double* trace, const SolveHooks* hk) {
    if (!h) return FDGA_ERR_ARG;
    if (maxiter < 1 || mem < 0 || !(tol >= 0)) return fail(h, FDGA_ERR_ARG, "invalid solver parameters");
    const size_t n = h->nstate;
    const int m = (int)std::min<size_t>((size_t)mem, n);
    // buffers: fx g fxold gold | dG[m] | Q[m]
    const size_t need = 4 + 2 * (size_t)m;
    while (h->aa_buf.size() < need) {
        cplx* p = nullptr;
        int r = dalloc(h, &p, n);
        if (r) return r;
        h->aa_buf.push_back(p);
    }
    if (m > AA_MAX) return fail(h, FDGA_ERR_ARG, "Anderson memory exceeds " + std::to_string(AA_MAX));
    if (!h->aa_R) {
        int r = dalloc(h, &h->aa_R, (size_t)AA_MAX * AA_MAX);
        if (!r) r = dalloc(h, &h->aa_rot, 2 * (size_t)AA_MAX);
        if (!r) r = dalloc(h, &h->aa_gam, (size_t)AA_MAX);
        if (!r) r = dalloc(h, &h->aa_part, (size_t)(AA_MAX + 2) * NBLK_RED);
        if (r) return r;
    }
    cplx *fx = h->aa_buf[0], *g = h->aa_buf[1], *fxold = h->aa_buf[2], *gold = h->aa_buf[3];
    std::vector<cplx*> dG(h->aa_buf.begin() + 4, h->aa_buf.begin() + 4 + m);
    AAVecsW Q{};
    for (int i = 0; i < m; ++i) Q.v[i] = h->aa_buf[4 + m + i];
    AAVecs Qc{};
    for (int i = 0; i < m; ++i) Qc.v[i] = Q.v[i];
    cplx* R = h->aa_R;
    cplx* pp[2] = {h->aa_part, h->aa_part + NBLK_RED};  // ping-pong partials of the Gram-Schmidt passes
    cplx* pdot = h->aa_part + 2 * NBLK_RED;              // partials of Qᴴ fx, [AA_MAX][NBLK_RED]
    if (m > 0) CK(cudaMemsetAsync(R, 0, (size_t)m * m * sizeof(cplx), h->st));
    int m_eff = 0, it = 0, status = 0;
    double resid = 0.0;
    bool converged = false;
    for (it = 1; it <= maxiter; ++it) {
        int r = hk && hk->before ? hk->before() : FDGA_OK;
        if (r) return r;
        r = run_iteration(h, strategy, update_sigma, true);
        if (r) return r;
        if (hk && hk->after && (r = hk->after())) return r;
        CK(launch_residual(h->st, h->yS, h->xS, fx, g, beta, h->d_part, NBLK_RED, n));
        resid = reduce_max(h, NBLK_RED, status);
        if (status) return status;
        if (!std::isfinite(resid)) return fail(h, FDGA_ERR_NONFINITE, "non-finite residual in solve");
        if (trace) trace[it - 1] = resid;
        if (resid < tol) { converged = true; break; }
        if (m == 0 || it == 1) {
            CK(cudaMemcpyAsync(h->xS, g, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
            if (m == 0) continue;
            CK(cudaMemcpyAsync(fxold, fx, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
            CK(cudaMemcpyAsync(gold, g, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
            continue;
        }
        m_eff += 1;
        if (m_eff > m) {
            // qrdelete!: Givens rotations on R and Q, Δg columns shift by one (pointer rotation)
            std::rotate(dG.begin(), dG.begin() + 1, dG.end());
            if (m > 1) CK(launch_aa_delete(h->st, NBLK_RED, R, m, h->aa_rot, Q, n));
            m_eff = m;
        }
        const int k = m_eff - 1;
        // qradd!: modified Gram-Schmidt of Δf against Q_0..Q_{k-1}, one pass per column
        CK(launch_aa_diff(h->st, NBLK_RED, dG[k], g, gold, fxold, fx, k > 0 ? Q.v[0] : nullptr, pp[0], n));
        int cur = 0;
        for (int i = 0; i < k; ++i) {
            CK(launch_aa_mgs(h->st, NBLK_RED, fxold, Q.v[i], pp[cur], R + i + (size_t)m * k,
                             i + 1 < k ? Q.v[i + 1] : nullptr, pp[cur ^ 1], n));
            cur ^= 1;
        }
        CK(launch_aa_qnew(h->st, NBLK_RED, Q.v[k], fxold, pp[cur], R + k + (size_t)m * k, n));
        // γ = R⁻¹ Qᴴ fx ; x = g - Σ γ_i Δg_i ; fxold = fx ; gold = g
        CK(launch_aa_gamma(h->st, NBLK_RED, Qc, m_eff, fx, pdot, R, m, h->aa_gam, n));
        AAVecs dGc{};
        for (int i = 0; i < m_eff; ++i) dGc.v[i] = dG[i];
        CK(launch_aa_update(h->st, NBLK_RED, h->xS, g, dGc, h->aa_gam, m_eff, fx, fxold, gold, n));
    }
    if (it > maxiter) it = maxiter;
    // S holds Φ(x) of the last evaluation, as after the reference's solve!
    CK(cudaMemcpyAsync(h->xS, h->yS, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (iters) *iters = converged ? it : -it;
    if (res) *res = resid;
    return FDGA_OK;
}

}  // namespace

extern "C" {

int fdga_solve(fdga_handle* h, int strategy, int maxiter, double tol, double beta, int mem, int* iters, double* res,
               double* trace) {
    return solve_anderson(h, strategy, true, maxiter, tol, beta, mem, iters, res, trace, nullptr);
}

int fdga_solve_mixed(fdga_handle* h, int strategy, int maxiter, double tol, double beta, int mem, int* iters, double* res,
                     double* trace, int* evals) {
    if (!h) return FDGA_ERR_ARG;
    if (maxiter < 2 || mem < 0 || !(tol > 0)) return fail(h, FDGA_ERR_ARG, "invalid solver parameters");
    const size_t n = h->nstate;
    const int m = (int)std::min<size_t>((size_t)mem, n);
    if (m > AA_MAX) return fail(h, FDGA_ERR_ARG, "Anderson memory exceeds " + std::to_string(AA_MAX));
    // FP64: c (defect Φ64 - Φ32 at the outer iterate), g, gold ; FP32: f, Δf, Q[m], Δg[m]
    while (h->ma_buf64.size() < 3) {
        cplx* p = nullptr;
        int r = dalloc(h, &p, n);
        if (r) return r;
        h->ma_buf64.push_back(p);
    }
    while (h->ma_buf32.size() < 2 + 2 * (size_t)m) {
        cplxf* p = nullptr;
        int r = dalloc(h, &p, n);
        if (r) return r;
        h->ma_buf32.push_back(p);
    }
    if (!h->aa_R) {
        int r = dalloc(h, &h->aa_R, (size_t)AA_MAX * AA_MAX);
        if (!r) r = dalloc(h, &h->aa_rot, 2 * (size_t)AA_MAX);
        if (!r) r = dalloc(h, &h->aa_gam, (size_t)AA_MAX);
        if (!r) r = dalloc(h, &h->aa_part, (size_t)(AA_MAX + 2) * NBLK_RED);
        if (r) return r;
    }
    cplx *c = h->ma_buf64[0], *g = h->ma_buf64[1], *gold = h->ma_buf64[2];
    cplxf *f = h->ma_buf32[0], *df = h->ma_buf32[1];
    std::vector<cplxf*> dG(h->ma_buf32.begin() + 2, h->ma_buf32.begin() + 2 + m);
    AAVecs32W Q{};
    AAVecs32 Qc{};
    for (int i = 0; i < m; ++i) Qc.v[i] = Q.v[i] = h->ma_buf32[2 + m + i];
    cplx* R = h->aa_R;
    cplx* pp[2] = {h->aa_part, h->aa_part + NBLK_RED};
    cplx* pdot = h->aa_part + 2 * NBLK_RED;
    if (int r = ensure_mixed(h)) return r;
    const int prec0 = h->precision;
    struct Restore {  // the handle's precision is restored on every exit
        fdga_handle* h; int p;
        ~Restore() { h->precision = p; }
    } restore{h, prec0};
    int n64 = 0, nmix = 0, nouter = 0, status = 0;
    double resid = 0.0;
    bool converged = false;
    auto budget_left = [&]() { return n64 + nmix + 2 <= maxiter; };
    // Anderson with the FP32 history on z -> Φ(z) (+ c), Φ in the handle's current precision, from
    // z = xS with yS = Φ(xS) already evaluated.  Stops when the residual is below tin, after
    // `stagnation` iterations without a new minimum (0: never), or at the evaluation budget.
    // fp64_outer: the residuals are FP64 ones (no c): they are traced and tested against tol.
    auto inner = [&](const cplx* cdef, double tin, int stagnation, bool fp64_outer) -> int {
        if (m > 0) CK(cudaMemsetAsync(R, 0, (size_t)m * m * sizeof(cplx), h->st));
        int m_eff = 0, since = 0;
        double best = INFINITY;
        for (int it = 1;; ++it) {
            CK(launch_ma_residual(h->st, NBLK_RED, h->yS, cdef, h->xS, f, g, beta, h->d_part, n));
            const double rin = reduce_max(h, NBLK_RED, status);
            if (status) return status;
            if (!std::isfinite(rin)) return fail(h, FDGA_ERR_NONFINITE, "non-finite residual in solve_mixed");
            if (fp64_outer) {
                resid = rin;
                if (trace) trace[nouter] = rin;
                ++nouter;
                if (rin < tol) { converged = true; return FDGA_OK; }
            }
            if (rin < tin || !budget_left()) return FDGA_OK;
            if (rin < 0.999 * best) { best = rin; since = 0; }
            else if (stagnation > 0 && ++since >= stagnation) return FDGA_OK;
            if (m == 0 || it == 1) {
                CK(cudaMemcpyAsync(h->xS, g, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
                if (m > 0) {
                    CK(cudaMemcpyAsync(df, f, n * sizeof(cplxf), cudaMemcpyDeviceToDevice, h->st));
                    CK(cudaMemcpyAsync(gold, g, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
                }
            } else {
                m_eff += 1;
                if (m_eff > m) {
                    std::rotate(dG.begin(), dG.begin() + 1, dG.end());
                    if (m > 1) {
                        CK(launch_aa_givens(h->st, R, m, h->aa_rot));
                        CK(launch_ma_qrot(h->st, NBLK_RED, Q, m, h->aa_rot, n));
                    }
                    m_eff = m;
                }
                const int k = m_eff - 1;
                CK(launch_ma_diff(h->st, NBLK_RED, dG[k], g, gold, df, f, k > 0 ? Q.v[0] : nullptr, pp[0], n));
                int cur = 0;
                for (int i = 0; i < k; ++i) {
                    CK(launch_ma_mgs(h->st, NBLK_RED, df, Q.v[i], pp[cur], R + i + (size_t)m * k,
                                     i + 1 < k ? Q.v[i + 1] : nullptr, pp[cur ^ 1], n));
                    cur ^= 1;
                }
                CK(launch_ma_qnew(h->st, NBLK_RED, Q.v[k], df, pp[cur], R + k + (size_t)m * k, n));
                CK(launch_ma_multidot(h->st, NBLK_RED, Qc, m_eff, f, pdot, n));
                CK(launch_aa_gamma_solve(h->st, pdot, NBLK_RED, R, m, m_eff, h->aa_gam));
                AAVecs32 dGc{};
                for (int i = 0; i < m_eff; ++i) dGc.v[i] = dG[i];
                CK(launch_ma_update(h->st, NBLK_RED, h->xS, g, dGc, h->aa_gam, m_eff, f, df, gold, n));
            }
            int r = run_iteration(h, strategy, true, true);
            if (r) return r;
            if (h->precision == FDGA_FP64) ++n64; else ++nmix;
        }
    };
    // Phase 1: iterative refinement.  Inner solves on the mixed map stop at 1e-3 of the outer FP64
    // residual, or when they stagnate at the mixed map's rounding floor.  Phase 2 starts when an
    // outer step reduced the FP64 residual by less than 10x (the floor is reached): the same
    // Anderson iteration then runs on the FP64 map to tol.
    // The inner residual cannot go below the mixed map's rounding floor, about the FP32 unit
    // roundoff times the size of the state; the inner tolerance stops there instead of leaving
    // the inner solve to stagnate.
    const double eta = 1e-3, u32 = 5.96e-8;
    double floor32 = 0.0;
    for (;;) {
        h->precision = FDGA_FP64;
        int r = run_iteration(h, strategy, true, true);
        if (r) return r;
        ++n64;
        if (floor32 == 0.0) {  // max|Φ(x)| at the first outer iterate
            CK(launch_residual(h->st, h->yS, nullptr, nullptr, nullptr, 0.0, h->d_part, NBLK_RED, n));
            floor32 = 2.0 * u32 * reduce_max(h, NBLK_RED, status);
            if (status) return status;
        }
        CK(launch_residual(h->st, h->yS, h->xS, c, nullptr, 0.0, h->d_part, NBLK_RED, n));
        const double rk = reduce_max(h, NBLK_RED, status);
        if (status) return status;
        if (!std::isfinite(rk)) return fail(h, FDGA_ERR_NONFINITE, "non-finite residual in solve_mixed");
        if (trace) trace[nouter] = rk;
        ++nouter;
        const double prev = nouter > 1 ? resid : INFINITY;
        resid = rk;
        if (rk < tol) { converged = true; break; }
        if (!budget_left()) break;
        if (!(rk < 0.1 * prev)) {
            // phase 2 from this iterate (yS = Φ64(x)); its first residual is this outer one
            --nouter;
            r = inner(nullptr, 0.0, 0, true);
            if (r) return r;
            break;
        }
        // defect c = Φ64(x) - Φ32(x): the inner equation z = Φ32(z) + c has the residual Φ64(x) - x at z = x
        CK(cudaMemcpyAsync(c, h->yS, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
        h->precision = FDGA_MIXED;
        r = run_iteration(h, strategy, true, true);
        if (r) return r;
        ++nmix;
        CK(launch_sub(h->st, c, c, h->yS, n));
        r = inner(c, std::max({eta * rk, 0.25 * tol, floor32}), 8, false);
        if (r) return r;
    }
    // S holds Φ64(x) of the last outer evaluation, as after the reference's solve!
    CK(cudaMemcpyAsync(h->xS, h->yS, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (iters) *iters = converged ? nouter : -nouter;
    if (res) *res = resid;
    if (evals) { evals[0] = n64; evals[1] = nmix; }
    return FDGA_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Newton–Krylov and linear response (GMRES on A = I − J, J the forward- or central-difference
// Jacobian of the iteration map, real inner products; the kernels are in fdga_krylov.cu).
// Krylov vectors live in the symmetric subspace: one value per symmetry class of every state
// block, inner products weighted by the class sizes (equal to the full-vector inner products).
// ---------------------------------------------------------------------------------------------
namespace {

// compact (one value per class) index of the state: code[j] = compact*4 + op, pos[i] = full index
int ensure_compact(fdga_handle* h) {
    if (h->kc_code && h->kc_version == h->groups_version) return FDGA_OK;
    const size_t n = h->nstate;
    if (!h->kc_code) {
        AL(h->kc_code, n);
        AL(h->kc_pos, n);
        AL(h->kc_w, n);
    }
    struct Blk { const Group* g; size_t base, len; };
    std::vector<Blk> blk;
    for (int ch : {CH_P, CH_T, CH_A}) {
        const size_t off = (size_t)ch * h->nchan;
        blk.push_back({&h->gK1, off, h->n1});
        blk.push_back({ch == CH_P ? &h->gK2pp : &h->gK2ph, off + h->n1, h->n2});
        blk.push_back({ch == CH_P ? &h->gK3pp : &h->gK3ph, off + h->n1 + h->n2, h->n3});
    }
    blk.push_back({&h->gSig, 3 * h->nchan, h->nGk});
    uint32_t off = 0;
    for (const auto& b : blk) {
        if (b.g == &h->gSig) h->nc_sig = off;
        const bool triv = b.g->trivial;
        CK(launch_kc_codes(h->st, triv ? nullptr : b.g->d_map, triv ? nullptr : b.g->d_items,
                           triv ? (int)b.len : b.g->nitems, b.len, b.base, off, h->kc_code, h->kc_pos));
        off += triv ? (uint32_t)b.len : (uint32_t)b.g->nitems;
    }
    h->nc = off;
    CK(cudaMemsetAsync(h->kc_w, 0, h->nc * sizeof(float), h->st));
    CK(launch_kc_count(h->st, NBLK_RED, h->kc_code, h->kc_w, n));
    CK(cudaStreamSynchronize(h->st));
    h->kc_version = h->groups_version;
    return FDGA_OK;
}

// buffers: compact FP64 [yb, F, dx, r, yp, tmp], compact FP32 [V0..Vm, w, scratch], full FP64 [x]
int ensure_krylov(fdga_handle* h, int m) {
    int r = ensure_compact(h);
    if (r) return r;
    const size_t nc = h->nc;
    if (h->kr_nc != nc) {  // compact length changed (symmetry groups set): drop the compact buffers
        h->kr64.clear();
        h->kr32.clear();
        for (auto& kv : h->kr_graphs)  // (their captured basis pointers)
            if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
        h->kr_graphs.clear();
        h->kr_nc = nc;
    }
    while (h->kr64.size() < 6) {
        cplx* p = nullptr;
        if ((r = dalloc(h, &p, nc))) return r;
        h->kr64.push_back(p);
    }
    while (h->kr32.size() < (size_t)m + 3) {
        cplxf* p = nullptr;
        if ((r = dalloc(h, &p, nc))) return r;
        h->kr32.push_back(p);
    }
    if (!h->kr_x && (r = dalloc(h, &h->kr_x, h->nstate))) return r;
    if (!h->kr_part) {
        r = dalloc(h, &h->kr_part, (size_t)(KR_MAX + 2) * NBLK_RED);
        if (!r) r = dalloc(h, &h->kr_coef, 4 * (size_t)(KR_MAX + 2));
        if (r) return r;
    }
    if (!h->kr_st) {
        AL(h->kr_st, 1);
        CK(cudaHostAlloc((void**)&h->kr_st_host, sizeof(KrDevState), cudaHostAllocDefault));
    }
    return FDGA_OK;
}

// weighted 2-norm of a compact FP64 vector (scratch: a compact FP32 vector)
int cnorm(fdga_handle* h, const cplx* a, cplxf* scratch, double& out) {
    CK(launch_kr_load(h->st, NBLK_RED, a, h->kc_w, scratch, h->kr_part, h->nc));
    CK(launch_kr_reduce(h->st, h->kr_part, NBLK_RED, 1, h->kr_coef));
    double v = 0.0;
    CK(cudaMemcpyAsync(&v, h->kr_coef, sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    out = std::sqrt(std::max(0.0, v));
    return FDGA_OK;
}

// max over the compact entries of |a|  (= the full max norm of a symmetric vector)
int cmax(fdga_handle* h, const cplx* a, double& out) {
    int status = 0;
    CK(launch_residual(h->st, a, nullptr, nullptr, nullptr, 0.0, h->d_part, NBLK_RED, h->nc));
    out = reduce_max(h, NBLK_RED, status);
    return status;
}

// tangent-kernel JVPs: on request, for the strategies the tangent map covers
bool use_tangent(const fdga_handle* h, int strategy) {
    return h->jvp_tangent && (strategy == FDGA_FDPA || strategy == FDGA_SCPA);
}

// A v = v − J v at the base point xb (full) for the unit compact FP32 direction v, into w.
// Tangent kernels (jvp_tangent): J v = Φ'(xb) v; the value intermediates of xb (the last map at xb,
// in the current precision) are in the handle and the state xS is xb.
// Forward difference: J v = (Φ(xb + εv) − yb)/ε (yb compact).  Central: (Φ(xb + εv) − Φ(xb − εv))/(2ε).
int apply_A(fdga_handle* h, int strategy, const cplx* xb, const cplx* yb, const cplxf* v, double eps, bool central,
            cplxf* w, int& nmaps) {
    const size_t n = h->nstate, nc = h->nc;
    if (use_tangent(h, strategy)) {
        CK(launch_kc_point(h->st, NBLK_RED, nullptr, v, h->kc_code, 1.0, h->tan.x, n));
        int r = run_tangent(h, strategy, true, true);
        if (r) return r;
        ++nmaps;
        CK(launch_kc_apply(h->st, NBLK_RED, h->tan.y, nullptr, h->kc_pos, v, 1.0, -1.0, w, nc));
        return FDGA_OK;
    }
    CK(launch_kc_point(h->st, NBLK_RED, xb, v, h->kc_code, eps, h->xS, n));
    int r = run_iteration(h, strategy, true, true);
    if (r) return r;
    ++nmaps;
    if (!central) {
        CK(launch_kc_apply(h->st, NBLK_RED, h->yS, yb, h->kc_pos, v, 1.0, -1.0 / eps, w, nc));
        return FDGA_OK;
    }
    cplx* yp = h->kr64[4];
    CK(launch_kc_gather(h->st, NBLK_RED, h->yS, nullptr, h->kc_pos, 1.0, yp, nc));
    CK(launch_kc_point(h->st, NBLK_RED, xb, v, h->kc_code, -eps, h->xS, n));
    r = run_iteration(h, strategy, true, true);
    if (r) return r;
    ++nmaps;
    CK(launch_kc_apply(h->st, NBLK_RED, h->yS, yp, h->kc_pos, v, 1.0, 0.5 / eps, w, nc));  // v + (y− − y+)/(2ε)
    return FDGA_OK;
}

// The FP32 operands that the tangent of the mixed map reads at its base point (G(R), the mirrors of
// x, Φ(x) and the momentum averages, FL.K2, FL.K3, the ten K3 caches), converted from the FP64
// map's intermediates at the same point: the mixed tangent then linearises at the FP64 value
// pass, and no mixed map is needed to set its base up.  Every other intermediate the tangent reads
// is FP64 and shared by the two precisions.
int mixed_tangent_base_from_fp64(fdga_handle* h) {
    if (int r = ensure_mixed(h)) return r;
    cudaStream_t s = h->st;
    CK(launch_to_f32(s, h->GR, h->GRf, h->nGk));
    CK(launch_to_f32(s, h->xS, h->xSf, 3 * h->nchan));
    CK(launch_to_f32(s, h->yS, h->ySf, 3 * h->nchan));
    if (h->navg) CK(launch_to_f32(s, h->avg, h->avgf, h->navg));
    CK(launch_to_f32(s, h->FLK2, h->FLK2f, 3 * h->n2));
    CK(launch_to_f32(s, h->FLK3, h->FLK3f, 3 * h->n3));
    CK(launch_to_f32(s, h->cache, h->cachef, 10 * h->n3));
    return FDGA_OK;
}

// The operator of a GMRES solve: w = A v for a unit compact FP32 direction v.  apply() adds the map
// evaluations it made to the solve's count; cost is that number, for the budget check.
struct KrylovOp {
    std::function<int(const cplxf* v, cplxf* w)> apply;
    int cost = 1;
    // capture-safe form for the device-resident cycle: enqueue w = A V[st->j] on h->st; key names the
    // operator for the cycle-graph cache (-1: host-driven Arnoldi only)
    std::function<int(const KrVecs& V, const KrDevState* st, cplxf* w)> enqueue_j;
    int key = -1;
};

// The Arnoldi loop of one GMRES cycle as one graph: a WHILE node whose body is the column j = st->j
// (operator, two Gram-Schmidt passes, Hessenberg/Givens update, V[j+1]) and the advance kernel that
// sets its condition.  j grows by one per pass and the condition requires j < m, so the loop ends
// after at most m passes.  Built once per (operator, m) and replayed every cycle.
int kr_cycle_graph(fdga_handle* h, const KrylovOp& op, const KrVecs& V, cplxf* w, int m, Graph*& out) {
    Graph& slot = h->kr_graphs[std::make_pair(op.key, m)];
    out = &slot;
    if (slot.exec) return FDGA_OK;
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0));
    struct Del { cudaGraph_t g; ~Del() { if (g) cudaGraphDestroy(g); } } del{g};
    cudaGraphConditionalHandle cond;
    CK(cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = cond;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    CK(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &p));
    cudaGraph_t body = p.conditional.phGraph_out[0];
    CK(cudaStreamBeginCaptureToGraph(h->st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    int r = op.enqueue_j(V, h->kr_st, w);
    cudaError_t e = cudaSuccess;
    if (!r)
        e = launch_kr_cgs_j(h->st, NBLK_RED, V, h->kr_st, w, h->kc_w, h->kr_part, h->kr_coef,
                            h->kr_coef + (KR_MAX + 2), h->nc);
    if (!r && e == cudaSuccess) e = launch_kr_advance(h->st, h->kr_st, cond);
    cudaGraph_t captured = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(h->st, &captured);
    if (r) return r;
    if (e != cudaSuccess) return cuda_fail(h, e, "GMRES cycle capture");
    if (ee != cudaSuccess) return cuda_fail(h, ee, "cudaStreamEndCapture (GMRES cycle)");
    e = cudaGraphInstantiate(&slot.exec, g, 0);
    if (e != cudaSuccess) { slot.exec = nullptr; return cuda_fail(h, e, "cudaGraphInstantiate (GMRES cycle)"); }
    return FDGA_OK;
}

// Restarted GMRES(m) for A dx = b (compact vectors), dx starting at 0.  Cycles after the first
// restart from the true residual b − A dx.  Stops at ‖b − A dx‖ <= atol + rtol ‖b‖ (estimate);
// relres = final ‖b − A dx‖/‖b‖ estimate.
int gmres_core(fdga_handle* h, const KrylovOp& op, const cplx* b, cplx* dx, int m, int cycles, double rtol,
               double atol, int max_maps, int& nmaps, int& iters, double& relres) {
    const size_t nc = h->nc;
    KrVecs V{};
    for (int i = 0; i <= m; ++i) V.v[i] = h->kr32[i];
    const std::vector<cplxf*>& Vw = h->kr32;  // the same basis, writable
    cplxf* w = h->kr32[m + 1];
    cplxf* sc = h->kr32[m + 2];
    cplx* rr = h->kr64[3];
    const float* W = h->kc_w;
    int r;
    double bnorm = 0.0;
    if ((r = cnorm(h, b, sc, bnorm))) return r;
    const double thr = atol + rtol * bnorm;
    CK(cudaMemsetAsync(dx, 0, nc * sizeof(cplx), h->st));
    relres = 1.0;
    if (bnorm == 0.0) { relres = 0.0; return FDGA_OK; }
    std::vector<double> H((size_t)(m + 1) * m), g(m + 1), cs(m), sn(m), hc(2 * (KR_MAX + 2)), y(m);
    auto Hij = [&](int i, int j) -> double& { return H[(size_t)i + (size_t)(m + 1) * j]; };
    double* c1 = h->kr_coef;
    double* c2 = h->kr_coef + (KR_MAX + 2);
    double* cy = h->kr_coef + 2 * (KR_MAX + 2);
    for (int cyc = 0; cyc < cycles; ++cyc) {
        double beta = bnorm;
        if (cyc == 0) {
            CK(launch_kr_load(h->st, NBLK_RED, b, W, sc, h->kr_part, nc));
            CK(launch_kr_scale(h->st, NBLK_RED, sc, bnorm, Vw[0], nc));
        } else {
            // true residual r = b − A dx, with A dx = ‖dx‖ A(dx/‖dx‖)
            double dn = 0.0;
            if ((r = cnorm(h, dx, sc, dn))) return r;
            if (dn == 0.0) break;
            if (nmaps + op.cost > max_maps) break;
            CK(launch_kr_load(h->st, NBLK_RED, dx, W, sc, h->kr_part, nc));
            CK(launch_kr_scale(h->st, NBLK_RED, sc, dn, sc, nc));
            if ((r = op.apply(sc, w))) return r;
            CK(launch_kr_resid(h->st, NBLK_RED, b, w, -dn, nullptr, nullptr, 0.0, rr, nc));
            if ((r = cnorm(h, rr, sc, beta))) return r;
            relres = beta / bnorm;
            if (beta <= thr) break;
            CK(launch_kr_load(h->st, NBLK_RED, rr, W, sc, h->kr_part, nc));
            CK(launch_kr_scale(h->st, NBLK_RED, sc, beta, Vw[0], nc));
        }
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int k = 0;
        double est = beta;
        const bool dev = op.enqueue_j && op.key >= 0 && h->kr_device_loop;
        if (dev) {
            // device-resident Arnoldi: one graph launch and one state read per cycle
            if (nmaps + op.cost > max_maps) break;
            Graph* cg = nullptr;
            if ((r = kr_cycle_graph(h, op, V, w, m, cg))) return r;
            CK(launch_kr_init(h->st, h->kr_st, m, max_maps - nmaps, op.cost, thr, beta));
            CK(cudaGraphLaunch(cg->exec, h->st));
            CK(cudaMemcpyAsync(h->kr_st_host, h->kr_st, sizeof(KrDevState), cudaMemcpyDeviceToHost, h->st));
            CK(cudaStreamSynchronize(h->st));
            const KrDevState& S = *h->kr_st_host;
            k = S.k;
            iters += k;
            nmaps += S.nmaps;
            est = S.est;
            for (int jj = 0; jj < k; ++jj)
                for (int i = 0; i <= jj; ++i) Hij(i, jj) = S.H[(size_t)i + (size_t)(KR_MAX + 1) * jj];
            for (int i = 0; i <= k; ++i) g[i] = S.g[i];
        }
        for (int j = 0; j < m && !dev; ++j) {
            if (nmaps + op.cost > max_maps) break;
            if ((r = op.apply(V.v[j], w))) return r;
            // classical Gram-Schmidt, twice (weighted inner products)
            CK(launch_kr_dots(h->st, NBLK_RED, V, j + 1, w, W, h->kr_part, -1, nc));
            CK(launch_kr_reduce(h->st, h->kr_part, NBLK_RED, j + 1, c1));
            CK(launch_kr_sub(h->st, NBLK_RED, V, j + 1, c1, w, nc));
            CK(launch_kr_dots(h->st, NBLK_RED, V, j + 1, w, W, h->kr_part, -1, nc));
            CK(launch_kr_reduce(h->st, h->kr_part, NBLK_RED, j + 1, c2));
            CK(launch_kr_sub(h->st, NBLK_RED, V, j + 1, c2, w, nc));
            CK(launch_kr_dots(h->st, NBLK_RED, V, 0, w, W, h->kr_part + (size_t)(KR_MAX + 1) * NBLK_RED, 0, nc));
            CK(launch_kr_reduce(h->st, h->kr_part + (size_t)(KR_MAX + 1) * NBLK_RED, NBLK_RED, 1, c2 + KR_MAX + 1));
            CK(cudaMemcpyAsync(hc.data(), h->kr_coef, 2 * (KR_MAX + 2) * sizeof(double), cudaMemcpyDeviceToHost,
                               h->st));
            CK(cudaStreamSynchronize(h->st));
            for (int i = 0; i <= j; ++i) Hij(i, j) = hc[i] + hc[(KR_MAX + 2) + i];
            const double hn = std::sqrt(std::max(0.0, hc[(KR_MAX + 2) + KR_MAX + 1]));
            Hij(j + 1, j) = hn;
            if (hn > 0.0) CK(launch_kr_scale(h->st, NBLK_RED, w, hn, Vw[j + 1], nc));
            for (int i = 0; i < j; ++i) {  // previous rotations
                const double a = Hij(i, j), bb = Hij(i + 1, j);
                Hij(i, j) = cs[i] * a + sn[i] * bb;
                Hij(i + 1, j) = -sn[i] * a + cs[i] * bb;
            }
            const double a = Hij(j, j), bb = Hij(j + 1, j), rho = std::hypot(a, bb);
            cs[j] = rho > 0 ? a / rho : 1.0;
            sn[j] = rho > 0 ? bb / rho : 0.0;
            Hij(j, j) = rho;
            Hij(j + 1, j) = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            ++iters;
            k = j + 1;
            est = std::fabs(g[j + 1]);
            if (est <= thr || hn == 0.0) break;
        }
        if (k == 0) break;
        for (int i = k - 1; i >= 0; --i) {
            double v = g[i];
            for (int jj = i + 1; jj < k; ++jj) v -= Hij(i, jj) * y[jj];
            y[i] = Hij(i, i) != 0.0 ? v / Hij(i, i) : 0.0;
        }
        CK(cudaMemcpyAsync(cy, y.data(), k * sizeof(double), cudaMemcpyHostToDevice, h->st));
        CK(launch_kr_update(h->st, NBLK_RED, dx, V, k, cy, 1.0, nc));
        relres = est / bnorm;
        if (est <= thr) break;
    }
    CK(cudaStreamSynchronize(h->st));
    return FDGA_OK;
}

// GMRES for the Newton step: A v = v − J v at the base point xb (apply_A); the difference step is
// ε = eps_rel (1 + ‖xb‖).
int gmres_solve(fdga_handle* h, int strategy, const cplx* xb, const cplx* yb, const cplx* b, cplx* dx, int m,
                int cycles, double rtol, double eps_rel, bool central, int max_maps, int& nmaps, int& iters,
                double& relres) {
    cplx* xc = h->kr64[5];
    double xnorm = 0.0;
    CK(launch_kc_gather(h->st, NBLK_RED, xb, nullptr, h->kc_pos, 1.0, xc, h->nc));
    int r = cnorm(h, xc, h->kr32[m + 2], xnorm);
    if (r) return r;
    const double eps = eps_rel * (1.0 + xnorm);
    KrylovOp op;
    op.cost = central && !use_tangent(h, strategy) ? 2 : 1;
    op.apply = [&](const cplxf* v, cplxf* w) { return apply_A(h, strategy, xb, yb, v, eps, central, w, nmaps); };
    if (use_tangent(h, strategy)) {  // v − J v by the tangent kernels: capturable into the cycle graph
        if ((r = ensure_tangent(h))) return r;
        op.key = 10 * h->precision + strategy;
        op.enqueue_j = [h, strategy](const KrVecs& V, const KrDevState* st, cplxf* w) -> int {
            CK(launch_kc_point_j(h->st, NBLK_RED, nullptr, V, st, h->kc_code, 1.0, h->tan.x, h->nstate));
            int nl = 0;
            int rr = enqueue_tangent(h, strategy, true, true, nl);
            if (rr) return rr;
            CK(launch_kc_apply_j(h->st, NBLK_RED, h->tan.y, h->kc_pos, V, st, 1.0, -1.0, w, h->nc));
            return FDGA_OK;
        };
    }
    return gmres_core(h, op, b, dx, m, cycles, rtol, 0.0, max_maps, nmaps, iters, relres);
}

// ---------------------------------------------------------------------------------------------
// mfRG linear map (src/mfRG.jl:20-89): y = x − Φ_mfRG(x·f)/f, f = 1e-2, on the vertex part of the
// state.  Φ_mfRG runs the iteration's BSE sequence on the vertex x·f with the reference system's
// bubble Π0 in every BSE and F0 in the right factors (the is_mfRG branches):
//   caches (fdga_mfrg.cu) → L_K2 (FL.K2) → K1, K2 of the map → L_K3 (FL.K3) → K3 with Π = Π0.
// The map depends on the state only through x (Π0, F0, G0 are the reference system's): it is the
// same linear operator for every application within a solve.  Nonlocal solver; :fdPA and
// :fdPA_1loop run the same map, :fdPA_new (the _new BSEs) is a local-solver strategy here.
// ---------------------------------------------------------------------------------------------
constexpr double kMfrgFactor = 1e-2;

int check_mfrg(fdga_handle* h, int strategy) {
    if (!h->finalized) return fail(h, FDGA_ERR_STATE, "fdga_finalize has not been called");
    if (strategy != FDGA_FDPA && strategy != FDGA_FDPA_NEW && strategy != FDGA_FDPA_1LOOP)
        return fail(h, FDGA_ERR_ARG, "the mfRG map takes the strategies fdPA, fdPA_new and fdPA_1loop");
    if (h->d.local) return fail(h, FDGA_ERR_UNSUPPORTED, "the mfRG map is defined for the nonlocal solver");
    if (strategy == FDGA_FDPA_NEW)
        return fail(h, FDGA_ERR_UNSUPPORTED, "the :fdPA_new BSEs exist for the local solver only");
    if (h->precision == FDGA_MIXED) {
        int r = ensure_mixed(h);
        if (r) return r;
    }
    if (!h->mf.x) {
        AL(h->mf.x, h->nstate);
        AL(h->mf.y, h->nstate);
        AL(h->mf.u, h->nstate);
    }
    return FDGA_OK;
}

// SG(cache, InitFunction(diagram)) of the map's caches: the class broadcast through the K3 groups,
// part 0 the Γ caches (Γpx, Γpp: pp group; Γa, Γt: ph group), part 1 Fp (pp), Fa, Ft (ph)
int mfrg_broadcast(fdga_handle* h, cudaStream_t s, const Caches& C, int part, int& nl) {
    const bool mixed = h->precision == FDGA_MIXED;
    const int pp[2][2] = {{0, 4}, {7, -1}}, ph[2][2] = {{5, 6}, {8, 9}};
    auto run = [&](const Group& g, const int* k) -> int {
        if (g.trivial) return FDGA_OK;
        if (mixed) LC(launch_cache_broadcast(s, C.f[k[0]], k[1] >= 0 ? C.f[k[1]] : nullptr, nullptr, g.d_map, h->n3));
        else LC(launch_cache_broadcast(s, C.c[k[0]], k[1] >= 0 ? C.c[k[1]] : nullptr, nullptr, g.d_map, h->n3));
        return FDGA_OK;
    };
    int r = run(h->gK3pp, pp[part]);
    if (!r) r = run(h->gK3ph, ph[part]);
    return r;
}

// the F0-only caches of the map (once per solve; the iteration overwrites the right ones)
int mfrg_prepare(fdga_handle* h) {
    Caches C{};
    const bool mixed = h->precision == FDGA_MIXED;
    for (int i = 0; i < 10; ++i) {
        C.c[i] = h->cache + (size_t)i * h->n3;
        C.f[i] = mixed ? h->cachef + (size_t)i * h->n3 : nullptr;
    }
    if (mixed) {
        for (int i = 0; i < 4; ++i) CK(launch_to_f32(h->st, h->Fref[i], h->Freff[i], h->nRef));
        VertPF Ff = vertex_view_t<cplxf>(h, h->xSf, h->avgf, h->Freff);
        CK(launch_build_cache_mfrg(h->st, Ff, C, h->d_k3blocks, h->nk3blocks, h->d, 1));
    } else {
        CK(launch_build_cache_mfrg(h->st, vertex_view(h, h->mf.x), C, h->d_k3blocks, h->nk3blocks, h->d, 1));
    }
    int nl = 0;
    return mfrg_broadcast(h, h->st, C, 1, nl);
}

// Φ_mfRG(mf.x) into mf.y.  Branch C: L_K2 → K1, K2 of the map; main: caches → L_K3 → K3.
int enqueue_mfrg(fdga_handle* h, int& nl) {
    cudaStream_t s = h->st, sC = h->st3;
    const Dims& d = h->d;
    nl = 0;
    const bool mixed = h->precision == FDGA_MIXED;
    VertP F = vertex_view(h, h->mf.x);
    if (d.Nq > 1) {
        ChanArrays in;
        ChanArraysW out;
        for (int c = 0; c < 3; ++c) {
            in.K1[c] = F.g[c].K1; in.K2[c] = F.g[c].K2; in.K3[c] = F.g[c].K3;
            out.K1[c] = (cplx*)F.g[c].A1; out.K2[c] = (cplx*)F.g[c].A2; out.K3[c] = (cplx*)F.g[c].A3;
        }
        LC(launch_qavg(s, in, out, d));
    }
    VertPF Ff{};
    if (mixed) {
        LC(launch_to_f32(s, h->mf.x, h->xSf, 3 * h->nchan));
        if (d.Nq > 1) LC(launch_to_f32(s, h->avg, h->avgf, h->navg));
        Ff = vertex_view_t<cplxf>(h, h->xSf, h->avgf, h->Freff);
    }
    CK(cudaEventRecord(h->evA, s));
    CK(cudaStreamWaitEvent(sC, h->evA, 0));
    Caches C{};
    for (int i = 0; i < 10; ++i) {
        C.c[i] = h->cache + (size_t)i * h->n3;
        C.f[i] = mixed ? h->cachef + (size_t)i * h->n3 : nullptr;
    }
    if (mixed) LC(launch_build_cache_mfrg(s, Ff, C, h->d_k3blocks, h->nk3blocks, d, 0));
    else LC(launch_build_cache_mfrg(s, F, C, h->d_k3blocks, h->nk3blocks, d, 0));
    if (int r = mfrg_broadcast(h, s, C, 0, nl)) return r;
    BubbleP B{h->Pipp, h->Piph, h->Pi0pp, h->Pi0ph};
    auto Pi0 = [&](int ch) { return ch == CH_P ? h->Pi0pp : h->Pi0ph; };
    auto work = [&](int cls, cplx* raw) {
        ChanWork cw{};
        const size_t n = cls == 1 ? h->n1 : h->n2;
        for (int ch = 0; ch < 3; ++ch) {
            const Group& g = cls == 1 ? h->gK1 : k2group(h, ch);
            cw.items[ch] = g.trivial ? nullptr : g.d_items;
            cw.nitems[ch] = g.trivial ? (int)n : g.nitems;
            cw.out[ch] = raw + (size_t)ch * n;
        }
        return cw;
    };
    auto fin = [&](int cls, cplx* raw, cplx* const out[3], const Group* const grp[3]) {
        Finalize3 f{};
        const size_t n = cls == 1 ? h->n1 : (cls == 2 ? h->n2 : h->n3);
        for (int ch = 0; ch < 3; ++ch) {
            f.raw[ch] = raw + (size_t)ch * n;
            f.out[ch] = out[ch];
            f.map[ch] = grp[ch]->trivial ? nullptr : grp[ch]->d_map;
            f.FL[ch] = h->FLK2 + (size_t)ch * h->n2;
        }
        return f;
    };
    {  // branch C: FL.K2, then the K1 and K2 of the map (they need FL.K2 only)
        ChanWork cw = work(2, h->raw2);
        if (mixed) LC(launch_bse_L_K2_all(sC, Ff, B, cw, d));
        else LC(launch_bse_L_K2_all(sC, F, B, cw, d));
        cplx* out[3] = {h->FLK2, h->FLK2 + h->n2, h->FLK2 + 2 * h->n2};
        const Group* grp[3] = {&h->gK2pp, &h->gK2ph, &h->gK2ph};
        Finalize3 f2 = fin(2, h->raw2, out, grp);
        if (mixed)
            for (int c = 0; c < 3; ++c) f2.outf[c] = h->FLK2f + (size_t)c * h->n2;
        LC(launch_finalize3(sC, f2, 0, 1, h->n2));
        FLP FL;
        for (int c = 0; c < 3; ++c) FL.K2[c] = h->FLK2 + (size_t)c * h->n2;
        ChanWork c1 = work(1, h->raw1);
        LC(launch_bse_K1_mfrg(sC, F, FL, B, c1, d));
        cplx* o1[3] = {chanK(h, h->mf.y, CH_P, 1), chanK(h, h->mf.y, CH_T, 1), chanK(h, h->mf.y, CH_A, 1)};
        const Group* g1[3] = {&h->gK1, &h->gK1, &h->gK1};
        LC(launch_finalize3(sC, fin(1, h->raw1, o1, g1), 0, 1, h->n1));
        ChanWork c2 = work(2, h->raw2);
        LC(launch_bse_K2_mfrg(sC, F, FL, B, c2, d));
        cplx* o2[3] = {chanK(h, h->mf.y, CH_P, 2), chanK(h, h->mf.y, CH_T, 2), chanK(h, h->mf.y, CH_A, 2)};
        LC(launch_finalize3(sC, fin(2, h->raw2, o2, grp), 1, 1, h->n2));
        CK(cudaEventRecord(h->evC, sC));
    }
    const int order[3] = {CH_P, CH_A, CH_T};
    {  // FL.K3 (BSE_L_K3!, unchanged by the mfRG flag)
        K3Args3 a3{};
        K3Args3F a3f{};
        for (int i = 0; i < 3; ++i) {
            const int ch = order[i];
            const int cg = ch == CH_P ? 4 : (ch == CH_A ? 5 : 6), cf0 = ch == CH_P ? 1 : (ch == CH_A ? 2 : 3);
            K3Args& a = a3.a[i];
            a.A = C.c[cg]; a.B0 = C.c[cf0]; a.Pi0 = Pi0(ch);
            a.out = h->raw3 + (size_t)ch * h->n3;
            a3.ch[i] = ch;
            K3ArgsF& af = a3f.a[i];
            af.A = C.f[cg]; af.B0 = C.f[cf0]; af.Pi0 = Pi0(ch);
            af.out = a.out;
            a3f.ch[i] = ch;
        }
        a3.blocks = a3f.blocks = h->d_k3blocks;
        a3.nblocks = a3f.nblocks = h->nk3blocks;
        if (mixed && k3_tensor_cores(h, 0)) LC(launch_k3_tensor_cores(h, s, 0, a3f));
        else if (mixed) LC(launch_bse_K3_f32(s, 0, a3f, 3, d, h->k3_tile[FDGA_MIXED][0]));
        else LC(launch_k3_fp64(h, s, 0, a3));
        cplx* out[3] = {h->FLK3, h->FLK3 + h->n3, h->FLK3 + 2 * h->n3};
        const Group* grp[3] = {&h->gK3ppL, &h->gK3phL, &h->gK3phL};
        Finalize3 f3 = fin(3, h->raw3, out, grp);
        if (mixed)
            for (int c = 0; c < 3; ++c) f3.outf[c] = h->FLK3f + (size_t)c * h->n3;
        LC(launch_finalize3(s, f3, 0, 1, h->n3));
    }
    {  // K3 of the map: the plain contraction with Π = Π0 (its (Π - Π0) cacheF0 term vanishes)
        K3Args3 a3{};
        K3Args3F a3f{};
        for (int i = 0; i < 3; ++i) {
            const int ch = order[i];
            const int cg = ch == CH_P ? 0 : (ch == CH_A ? 5 : 6), cf = ch == CH_P ? 7 : (ch == CH_A ? 8 : 9);
            const int cf0 = ch == CH_P ? 1 : (ch == CH_A ? 2 : 3);
            K3Args& a = a3.a[i];
            a.A = C.c[cf]; a.B0 = C.c[cf0]; a.G = C.c[cg]; a.Pi = Pi0(ch); a.Pi0 = Pi0(ch);
            a.FLc = h->FLK3 + (size_t)ch * h->n3; a.FLt = h->FLK3 + (size_t)CH_T * h->n3;
            a.FLa = h->FLK3 + (size_t)CH_A * h->n3;
            a.out = h->raw3 + (size_t)ch * h->n3;
            a.flags = 0;
            a3.ch[i] = ch;
            if (mixed) {
                K3ArgsF& af = a3f.a[i];
                af.A = C.f[cf]; af.B0 = C.f[cf0]; af.G = C.f[cg]; af.Pi = a.Pi; af.Pi0 = a.Pi0;
                af.FLc = h->FLK3f + (size_t)ch * h->n3; af.FLt = h->FLK3f + (size_t)CH_T * h->n3;
                af.FLa = h->FLK3f + (size_t)CH_A * h->n3;
                af.out = a.out;
                af.flags = 0;
                a3f.ch[i] = ch;
            }
        }
        a3.blocks = a3f.blocks = h->d_k3blocks;
        a3.nblocks = a3f.nblocks = h->nk3blocks;
        if (mixed && k3_tensor_cores(h, 1)) LC(launch_k3_tensor_cores(h, s, 1, a3f));
        else if (mixed) LC(launch_bse_K3_f32(s, 1, a3f, 3, d, h->k3_tile[FDGA_MIXED][1]));
        else LC(launch_k3_fp64(h, s, 1, a3));
        cplx* out[3] = {chanK(h, h->mf.y, CH_P, 3), chanK(h, h->mf.y, CH_T, 3), chanK(h, h->mf.y, CH_A, 3)};
        const Group* grp[3] = {&h->gK3pp, &h->gK3ph, &h->gK3ph};
        LC(launch_finalize3(s, fin(3, h->raw3, out, grp), 0, 1, h->n3));
    }
    CK(cudaStreamWaitEvent(s, h->evC, 0));
    return FDGA_OK;
}

// one application of Φ_mfRG (mf.x → mf.y) as a captured graph per precision
int run_mfrg(fdga_handle* h) {
    Graph& g = h->mf.graphs[h->precision];
    if (!g.exec) {
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
        int nl = 0;
        int r = enqueue_mfrg(h, nl);
        cudaError_t ee = cudaStreamEndCapture(h->st, &graph);
        if (r) {
            if (ee == cudaSuccess) cudaGraphDestroy(graph);
            return r;
        }
        if (ee != cudaSuccess) return cuda_fail(h, ee, "cudaStreamEndCapture");
        ee = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ee != cudaSuccess) { g.exec = nullptr; return cuda_fail(h, ee, "cudaGraphInstantiate"); }
        g.nodes = nl;
    }
    CK(cudaGraphLaunch(g.exec, h->st));
    h->last_launches = g.nodes;
    return FDGA_OK;
}

// The mfRG operator on compact vectors for GMRES: w = v − Φ_mfRG(f·v)/f (the Σ classes pass through)
KrylovOp mfrg_operator(fdga_handle* h, int& nmaps) {
    KrylovOp op;
    op.cost = 1;
    op.apply = [h, &nmaps](const cplxf* v, cplxf* w) -> int {
        CK(launch_kc_point(h->st, NBLK_RED, nullptr, v, h->kc_code, kMfrgFactor, h->mf.x, 3 * h->nchan));
        int r = run_mfrg(h);
        if (r) return r;
        ++nmaps;
        CK(launch_kc_apply(h->st, NBLK_RED, h->mf.y, nullptr, h->kc_pos, v, 1.0, -1.0 / kMfrgFactor, w, h->nc));
        return FDGA_OK;
    };
    op.key = 100 + h->precision;
    op.enqueue_j = [h](const KrVecs& V, const KrDevState* st, cplxf* w) -> int {
        CK(launch_kc_point_j(h->st, NBLK_RED, nullptr, V, st, h->kc_code, kMfrgFactor, h->mf.x, 3 * h->nchan));
        int nl = 0;
        int rr = enqueue_mfrg(h, nl);
        if (rr) return rr;
        CK(launch_kc_apply_j(h->st, NBLK_RED, h->mf.y, h->kc_pos, V, st, 1.0, -1.0 / kMfrgFactor, w, h->nc));
        return FDGA_OK;
    };
    return op;
}

// Krylov solve of the preconditioner, M z = R_F (src/mfRG.jl:145-155), on the compact state: b is the
// vertex part of (y − x) at the class representatives (Σ's classes zero), z (compact FP64) in
// h->kr64[2].  Restarted GMRES(min(64, maxiter)), at most maxiter map applications, stopping at
// ‖r‖ <= atol + rtol ‖b‖.
int mfrg_krylov(fdga_handle* h, const cplx* y, const cplx* x, int maxiter, double rtol, double atol, int& nmaps,
                int& iters, double& relres) {
    const int m = std::max(1, std::min(KR_MAX - 1, maxiter));
    int r = ensure_krylov(h, m);
    if (r) return r;
    cplx* b = h->kr64[1];
    cplx* z = h->kr64[2];
    CK(launch_kc_gather(h->st, NBLK_RED, y, x, h->kc_pos, 1.0, b, h->nc));
    if (h->nc > h->nc_sig) CK(cudaMemsetAsync(b + h->nc_sig, 0, (h->nc - h->nc_sig) * sizeof(cplx), h->st));
    if ((r = mfrg_prepare(h))) return r;
    const int cycles = (maxiter + m - 1) / m;
    KrylovOp op = mfrg_operator(h, nmaps);
    return gmres_core(h, op, b, z, m, cycles, rtol, atol, maxiter, nmaps, iters, relres);
}

}  // namespace

extern "C" {

int fdga_set_U(fdga_handle* h, double U) {
    if (!h) return FDGA_ERR_ARG;
    if (!std::isfinite(U)) return fail(h, FDGA_ERR_ARG, "U must be finite");
    h->d.U = U;
    h->cfg.U = U;
    h->c0_dirty = true;
    drop_graphs(h);
    return FDGA_OK;
}

int fdga_jvp(fdga_handle* h, int strategy, const double* v, double* Jv, size_t n) {
    if (!h || !v || !Jv) return fail(h, FDGA_ERR_ARG, "null argument");
    if (n != h->nstate) return fail(h, FDGA_ERR_ARG, "state length mismatch");
    int r;
    if (!h->kr_x && (r = dalloc(h, &h->kr_x, n))) return r;
    if (h->jv.size() < 3)
        while (h->jv.size() < 3) {
            cplx* p = nullptr;
            if ((r = dalloc(h, &p, n))) return r;
            h->jv.push_back(p);
        }
    cplx *x = h->kr_x, *tmp = h->jv[0], *dir = h->jv[1], *yp = h->jv[2];
    CK(cudaMemcpyAsync(x, h->xS, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
    CK(cudaMemcpyAsync(tmp, v, n * sizeof(cplx), cudaMemcpyHostToDevice, h->st));
    CK(launch_scatter(h->st, dir, tmp, h->perm, n));  // reference layout -> device layout
    // full-space central difference (v need not be symmetric): Jv = (Φ(x + εv) − Φ(x − εv))/(2ε)
    if (!h->kr_part) {
        r = dalloc(h, &h->kr_part, (size_t)(KR_MAX + 2) * NBLK_RED);
        if (!r) r = dalloc(h, &h->kr_coef, 4 * (size_t)(KR_MAX + 2));
        if (r) return r;
    }
    double vn2 = 0.0, xn2 = 0.0;
    cplxf* scratch = reinterpret_cast<cplxf*>(yp);  // n FP32 pairs fit in an FP64 vector
    for (int k = 0; k < 2; ++k) {
        CK(launch_kr_load(h->st, NBLK_RED, k ? x : dir, nullptr, scratch, h->kr_part, n));
        CK(launch_kr_reduce(h->st, h->kr_part, NBLK_RED, 1, h->kr_coef));
        CK(cudaMemcpyAsync(k ? &xn2 : &vn2, h->kr_coef, sizeof(double), cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
    }
    if (vn2 == 0.0) {
        std::memset(Jv, 0, 2 * n * sizeof(double));
        return FDGA_OK;
    }
    const double eps = 1e-5 * (1.0 + std::sqrt(xn2)) / std::sqrt(vn2);
    CK(launch_kr_axpby(h->st, NBLK_RED, h->xS, x, eps, dir, n));
    if ((r = run_iteration(h, strategy, true, true))) return r;
    CK(cudaMemcpyAsync(yp, h->yS, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
    CK(launch_kr_axpby(h->st, NBLK_RED, h->xS, x, -eps, dir, n));
    if ((r = run_iteration(h, strategy, true, true))) return r;
    CK(launch_kr_resid(h->st, NBLK_RED, nullptr, nullptr, 0.0, yp, h->yS, 0.5 / eps, tmp, n));
    CK(cudaMemcpyAsync(h->xS, x, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
    CK(launch_gather(h->st, h->yS, tmp, h->perm, n));
    CK(cudaMemcpyAsync(Jv, h->yS, n * sizeof(cplx), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return FDGA_OK;
}

int fdga_frule(fdga_handle* h, int strategy, int update_sigma, int compute_hartree, const double* v, double* y,
               double* Jv, size_t n) {
    if (!h || !v || !Jv) return fail(h, FDGA_ERR_ARG, "null argument");
    if (!h->finalized) return fail(h, FDGA_ERR_STATE, "fdga_finalize has not been called");
    if (n != h->nstate) return fail(h, FDGA_ERR_ARG, "state length mismatch");
    if (strategy != FDGA_FDPA && strategy != FDGA_SCPA)
        return fail(h, FDGA_ERR_UNSUPPORTED, "the tangent map covers the fdPA and scPA strategies");
    int r = ensure_tangent(h);
    if (r) return r;
    // value pass at x (leaves the intermediates of the base point in the handle), then the tangent
    if ((r = run_iteration(h, strategy, update_sigma != 0, compute_hartree != 0))) return r;
    CK(cudaMemcpyAsync(h->tmpS, v, n * sizeof(cplx), cudaMemcpyHostToDevice, h->st));
    CK(launch_scatter(h->st, h->tan.x, h->tmpS, h->perm, n));  // reference layout -> device layout
    if ((r = run_tangent(h, strategy, update_sigma != 0, compute_hartree != 0))) return r;
    if ((r = check_device_error(h))) return r;
    CK(launch_gather(h->st, h->tmpS, h->tan.y, h->perm, n));
    CK(cudaMemcpyAsync(Jv, h->tmpS, n * sizeof(cplx), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (y) {
        CK(launch_gather(h->st, h->tmpS, h->yS, h->perm, n));
        CK(cudaMemcpyAsync(y, h->tmpS, n * sizeof(cplx), cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
    }
    return FDGA_OK;
}

int fdga_rrule(fdga_handle* h, int strategy, int update_sigma, int compute_hartree, const double* ybar, double* y,
               double* xbar, size_t n) {
    if (!h || !ybar || !xbar) return fail(h, FDGA_ERR_ARG, "null argument");
    if (!h->finalized) return fail(h, FDGA_ERR_STATE, "fdga_finalize has not been called");
    if (n != h->nstate) return fail(h, FDGA_ERR_ARG, "state length mismatch");
    if (strategy != FDGA_FDPA && strategy != FDGA_SCPA)
        return fail(h, FDGA_ERR_UNSUPPORTED, "the adjoint map covers the fdPA and scPA strategies");
    if (h->has0)
        return fail(h, FDGA_ERR_UNSUPPORTED, "the adjoint map covers a RefVertex reference vertex only (use fdga_frule)");
    int r = ensure_adjoint(h);
    if (r) return r;
    const int prec0 = h->precision;
    h->precision = FDGA_FP64;  // the adjoint runs on the FP64 intermediates
    r = run_iteration(h, strategy, update_sigma != 0, compute_hartree != 0);
    h->precision = prec0;
    if (r) return r;
    CK(cudaMemcpyAsync(h->tmpS, ybar, n * sizeof(cplx), cudaMemcpyHostToDevice, h->st));
    CK(launch_scatter(h->st, h->adj.yb, h->tmpS, h->perm, n));  // reference layout -> device layout
    if ((r = run_adjoint(h, strategy, update_sigma != 0, compute_hartree != 0))) return r;
    CK(launch_gather(h->st, h->tmpS, h->adj.xb, h->perm, n));
    CK(cudaMemcpyAsync(xbar, h->tmpS, n * sizeof(cplx), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (y) {
        CK(launch_gather(h->st, h->tmpS, h->yS, h->perm, n));
        CK(cudaMemcpyAsync(y, h->tmpS, n * sizeof(cplx), cudaMemcpyDeviceToHost, h->st));
        CK(cudaStreamSynchronize(h->st));
    }
    return FDGA_OK;
}

int fdga_solve_newton(fdga_handle* h, int strategy, int maxiter, double tol, int restart, int jvp_precision,
                      int* iters, double* res, double* trace, int* evals) {
    if (!h) return FDGA_ERR_ARG;
    if (maxiter < 2 || !(tol > 0) || restart < 1 || restart >= KR_MAX)
        return fail(h, FDGA_ERR_ARG, "invalid solver parameters");
    if (jvp_precision != FDGA_FP64 && jvp_precision != FDGA_MIXED) return fail(h, FDGA_ERR_ARG, "unknown precision");
    const size_t n = h->nstate;
    int r = ensure_krylov(h, restart);
    if (r) return r;
    const size_t nc = h->nc;
    if (jvp_precision == FDGA_MIXED && (r = ensure_mixed(h))) return r;
    const int prec0 = h->precision;
    if (use_tangent(h, strategy)) {  // tangent buffers of both precisions used below
        for (int p : {(int)FDGA_FP64, jvp_precision}) {
            const int keep = h->precision;
            h->precision = p;
            r = ensure_tangent(h);
            h->precision = keep;
            if (r) return r;
        }
    }
    struct Restore {
        fdga_handle* h; int p;
        ~Restore() { h->precision = p; }
    } restore{h, prec0};
    cplx *x = h->kr_x, *yb = h->kr64[0], *F = h->kr64[1], *dx = h->kr64[2];
    int n64 = 0, nmix = 0, nouter = 0;
    double resid = 0.0, prev = 0.0;
    bool converged = false;
    // Φ(x) at the start; the Newton iterates start from Φ(x), which lies in the symmetric subspace
    h->precision = FDGA_FP64;
    if ((r = run_iteration(h, strategy, true, true))) return r;
    ++n64;
    CK(launch_kc_gather(h->st, NBLK_RED, h->yS, h->xS, h->kc_pos, 1.0, F, nc));
    {
        int status = 0;
        CK(launch_residual(h->st, h->yS, h->xS, nullptr, nullptr, 0.0, h->d_part, NBLK_RED, n));
        resid = reduce_max(h, NBLK_RED, status);
        if (status) return status;
    }
    if (!std::isfinite(resid)) return fail(h, FDGA_ERR_NONFINITE, "non-finite residual in solve_newton");
    if (trace) trace[nouter] = resid;
    ++nouter;
    if (resid < tol) converged = true;
    CK(cudaMemcpyAsync(x, h->yS, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
    bool have_y = false;
    int jvp_prec = jvp_precision;  // mixed JVPs until a step gains less than 2x, FP64 JVPs after that
    while (!converged) {
        h->precision = FDGA_FP64;
        if (!have_y) {
            if (n64 + nmix + 1 > maxiter) break;
            CK(cudaMemcpyAsync(h->xS, x, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
            if ((r = run_iteration(h, strategy, true, true))) return r;
            ++n64;
        }
        // F = Φ(x) − x (compact), yb = Φ(x) (compact)
        CK(launch_kc_gather(h->st, NBLK_RED, h->yS, x, h->kc_pos, 1.0, F, nc));
        CK(launch_kc_gather(h->st, NBLK_RED, h->yS, nullptr, h->kc_pos, 1.0, yb, nc));
        prev = resid;
        if ((r = cmax(h, F, resid))) return r;
        if (!std::isfinite(resid)) return fail(h, FDGA_ERR_NONFINITE, "non-finite residual in solve_newton");
        if (trace) trace[nouter] = resid;
        ++nouter;
        if (resid < tol) { converged = true; break; }
        if (n64 + nmix + 3 > maxiter) break;
        // the rounding floor of mixed JVPs by differences stalls Newton on ill-conditioned Jacobians:
        // switch to FP64 (mixed tangent JVPs carry FP32 rounding only and keep the mixed map)
        if (!use_tangent(h, strategy) && jvp_prec == FDGA_MIXED && nouter > 3 && !(resid < 0.5 * prev))
            jvp_prec = FDGA_FP64;
        // forcing term (Eisenstat–Walker choice 2, bounded); the mixed map's rounding floor bounds it below
        double eta = nouter <= 2 ? 0.1 : std::min(0.1, 0.9 * (resid / prev) * (resid / prev));
        // (tangent JVPs of the mixed map carry FP32 rounding, ~1e-6; differences of it ~1e-4)
        eta = std::max(eta, jvp_prec == FDGA_MIXED ? (use_tangent(h, strategy) ? 1e-5 : 1e-3) : 1e-6);
        // no linear solve beyond what the tolerance asks of this step
        eta = std::min(0.1, std::max(eta, 0.1 * tol / resid));
        if (jvp_prec == FDGA_MIXED && use_tangent(h, strategy)) {
            // the base of the mixed tangent from the FP64 map just run at x (xS = x, yS = Φ64(x))
            if ((r = mixed_tangent_base_from_fp64(h))) return r;
            h->precision = FDGA_MIXED;
        } else if (jvp_prec == FDGA_MIXED) {
            h->precision = FDGA_MIXED;
            CK(cudaMemcpyAsync(h->xS, x, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
            if ((r = run_iteration(h, strategy, true, true))) return r;
            ++nmix;
            CK(launch_kc_gather(h->st, NBLK_RED, h->yS, nullptr, h->kc_pos, 1.0, yb, nc));
        }
        int nmaps = 0, its = 0;
        double relres = 1.0;
        const int left = maxiter - n64 - nmix - 1;
        const double eps_rel = jvp_prec == FDGA_MIXED ? 3e-4 : 1e-7;
        // (I − J) dx = F
        r = gmres_solve(h, strategy, x, yb, F, dx, restart, h->newton_cycles, eta, eps_rel, false, left, nmaps, its,
                        relres);
        if (r) return r;
        if (h->precision == FDGA_FP64) n64 += nmaps; else nmix += nmaps;
        // backtracking on the FP64 residual
        h->precision = FDGA_FP64;
        double lam = 1.0;
        have_y = false;
        for (int ls = 0; ls < 4 && n64 + nmix + 1 <= maxiter; ++ls) {
            CK(launch_kc_axpy(h->st, NBLK_RED, x, dx, h->kc_code, lam, h->xS, n));
            if ((r = run_iteration(h, strategy, true, true))) return r;
            ++n64;
            int status = 0;
            CK(launch_residual(h->st, h->yS, h->xS, nullptr, nullptr, 0.0, h->d_part, NBLK_RED, n));
            const double rn = reduce_max(h, NBLK_RED, status);
            if (status) return status;
            if (std::isfinite(rn) && (rn < (1.0 - 1e-4 * lam) * resid || ls == 3)) {
                CK(cudaMemcpyAsync(x, h->xS, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
                have_y = true;
                break;
            }
            lam *= 0.5;
        }
        if (!have_y) break;
    }
    // S holds Φ64 of the last iterate, as after the reference's solve!
    if (!converged || nouter > 1) {
        if (!have_y) {
            h->precision = FDGA_FP64;
            CK(cudaMemcpyAsync(h->xS, x, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
            if ((r = run_iteration(h, strategy, true, true))) return r;
            ++n64;
        }
        CK(cudaMemcpyAsync(h->xS, h->yS, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
    } else {
        CK(cudaMemcpyAsync(h->xS, x, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
    }
    CK(cudaStreamSynchronize(h->st));
    if (iters) *iters = converged ? nouter : -nouter;
    if (res) *res = resid;
    if (evals) { evals[0] = n64; evals[1] = nmix; }
    return FDGA_OK;
}

int fdga_dchi_dU(fdga_handle* h, int strategy, int channel, double hU, int restart, int cycles, double rtol,
                 double* out, size_t n_out, int* gmres_iters, double* relres_out) {
    if (!h || !out) return fail(h, FDGA_ERR_ARG, "null argument");
    if (channel < FDGA_CHI_M || channel > FDGA_CHI_S) return fail(h, FDGA_ERR_ARG, "unknown susceptibility channel");
    const size_t NO = (size_t)h->d.N1, full = NO * h->d.Nq;
    if (n_out != full) return fail(h, FDGA_ERR_ARG, "dchi_dU length must be NΩ1·Nq");
    if (!(hU > 0) || restart < 1 || restart >= KR_MAX || cycles < 1) return fail(h, FDGA_ERR_ARG, "invalid parameters");
    const size_t n = h->nstate;
    int r = ensure_krylov(h, restart);
    if (r) return r;
    const size_t nc = h->nc;
    const int prec0 = h->precision;
    const double U = h->d.U;
    struct Restore {
        fdga_handle* h; int p; double U;
        ~Restore() { h->precision = p; if (h->d.U != U) fdga_set_U(h, U); }
    } restore{h, prec0, U};
    h->precision = FDGA_FP64;
    cplx *xs = h->kr_x, *b = h->kr64[1], *dx = h->kr64[2], *yp = h->kr64[4];
    CK(cudaMemcpyAsync(xs, h->xS, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
    // ∂Φ/∂U at the fixed point: central difference in U (compact)
    if ((r = fdga_set_U(h, U + hU))) return r;
    if ((r = run_iteration(h, strategy, true, true))) return r;
    CK(launch_kc_gather(h->st, NBLK_RED, h->yS, nullptr, h->kc_pos, 1.0, yp, nc));
    if ((r = fdga_set_U(h, U - hU))) return r;
    if ((r = run_iteration(h, strategy, true, true))) return r;
    CK(launch_kc_gather(h->st, NBLK_RED, h->yS, nullptr, h->kc_pos, 1.0, b, nc));
    CK(launch_kr_resid(h->st, NBLK_RED, nullptr, nullptr, 0.0, yp, b, 0.5 / hU, b, nc));  // b = (y+ − y−)/(2h)
    if ((r = fdga_set_U(h, U))) return r;
    if (use_tangent(h, strategy)) {  // value intermediates at the fixed point for the tangent kernels
        if ((r = ensure_tangent(h))) return r;
        CK(cudaMemcpyAsync(h->xS, xs, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
        if ((r = run_iteration(h, strategy, true, true))) return r;
    }
    // (I − J) dx = ∂Φ/∂U (Jacobian by the tangent kernels, or central differences)
    int nmaps = 0, its = 0;
    double relres = 1.0;
    r = gmres_solve(h, strategy, xs, nullptr, b, dx, restart, cycles, rtol, 1e-5, true, 1 << 30, nmaps, its, relres);
    if (r) return r;
    // dχ/dU = χ(dx) − (2/U) χ(x*)   (χ = K1 combination / U²); dx expanded into the full layout
    CK(cudaMemsetAsync(h->tmpS, 0, n * sizeof(cplx), h->st));
    CK(launch_kc_axpy(h->st, NBLK_RED, h->tmpS, dx, h->kc_code, 1.0, h->tmpS, n));  // tmpS = expand(dx)
    std::vector<cplx> hb(2 * full);  // χ(dx) and χ(x*), staged in yS (2 NΩ1·Nq <= state length)
    CK(launch_chi(h->st, chanK(h, h->tmpS, CH_P, 1), chanK(h, h->tmpS, CH_T, 1), chanK(h, h->tmpS, CH_A, 1), channel, U,
                  (int)NO, h->d.Nq, 0, h->yS));
    CK(launch_chi(h->st, chanK(h, xs, CH_P, 1), chanK(h, xs, CH_T, 1), chanK(h, xs, CH_A, 1), channel, U, (int)NO,
                  h->d.Nq, 0, h->yS + full));
    CK(cudaMemcpyAsync(hb.data(), h->yS, 2 * full * sizeof(cplx), cudaMemcpyDeviceToHost, h->st));
    CK(cudaMemcpyAsync(h->xS, xs, n * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    for (size_t i = 0; i < full; ++i) {
        out[2 * i] = hb[i].x - 2.0 / U * hb[full + i].x;
        out[2 * i + 1] = hb[i].y - 2.0 / U * hb[full + i].y;
    }
    if (gmres_iters) *gmres_iters = its;
    if (relres_out) *relres_out = relres;
    return FDGA_OK;
}

int fdga_named_len(const fdga_handle* h, const char* name, size_t* n) {
    if (!h || !name || !n) return FDGA_ERR_ARG;
    cplx* p;
    int kind;
    if (!lookup(const_cast<fdga_handle*>(h), name, p, kind, *n)) return FDGA_ERR_ARG;
    return FDGA_OK;
}

int fdga_get_named(fdga_handle* h, const char* name, double* out, size_t n) {
    if (!h || !name || !out) return fail(h, FDGA_ERR_ARG, "null argument");
    cplx* p;
    int kind;
    size_t len;
    if (!lookup(h, name, p, kind, len)) return fail(h, FDGA_ERR_ARG, std::string("unknown array ") + name);
    if (n != len) return fail(h, FDGA_ERR_ARG, "size mismatch for " + std::string(name));
    std::vector<cplx> dev(len);
    CK(cudaStreamSynchronize(h->st));
    if (kind == AK_PI) {
        // the iteration stores a window of the bubble mesh; inspection recomputes the whole mesh
        const std::string nm(name);
        const bool ref = nm == "Pi0pp" || nm == "Pi0ph";
        const bool pp = nm == "Pipp" || nm == "Pi0pp";
        Dims df = h->d;
        df.nPw = df.nPn;
        df.NPw = df.NPn;
        cplx *tpp = nullptr, *tph = nullptr;
        CK(cudaMalloc(&tpp, len * sizeof(cplx)));
        cudaError_t e = cudaMalloc(&tph, len * sizeof(cplx));
        if (e == cudaSuccess) e = launch_g_realspace(h->st, ref ? h->G0 : h->G, h->GR, h->twm, df);
        if (e == cudaSuccess) e = launch_bubble(h->st, ref ? h->G0 : h->G, h->GR, tpp, tph, h->twp, df);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dev.data(), pp ? tpp : tph, len * sizeof(cplx), cudaMemcpyDeviceToHost, h->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
        cudaFree(tpp);
        if (tph) cudaFree(tph);
        if (e != cudaSuccess) return cuda_fail(h, e, "full bubble for inspection");
        cplx* o = reinterpret_cast<cplx*>(out);
        for (size_t j = 0; j < len; ++j) o[j] = dev[dev_index(h->d, kind, j)];
        return FDGA_OK;
    }
    CK(cudaMemcpyAsync(dev.data(), p, len * sizeof(cplx), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    cplx* o = reinterpret_cast<cplx*>(out);
    for (size_t j = 0; j < len; ++j) o[j] = dev[dev_index(h->d, kind, j)];
    return FDGA_OK;
}

int fdga_occupation(fdga_handle* h, double* n) {
    if (!h || !n) return FDGA_ERR_ARG;
    CK(launch_occupation(h->st, h->G, h->nGk, h->d.T, h->d.Nk, h->occ));
    CK(cudaMemcpyAsync(n, h->occ, sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return FDGA_OK;
}

int fdga_set_precision(fdga_handle* h, int precision) {
    if (!h) return FDGA_ERR_ARG;
    if (precision != FDGA_FP64 && precision != FDGA_MIXED) return fail(h, FDGA_ERR_ARG, "unknown precision");
    if (precision == FDGA_MIXED) {
        int r = ensure_mixed(h);
        if (r) return r;
    }
    h->precision = precision;
    return FDGA_OK;
}

int fdga_set_option(fdga_handle* h, const char* key, int value) {
    if (h && key && std::string(key) == "gmres_device_loop") {
        h->kr_device_loop = value ? 1 : 0;
        return FDGA_OK;
    }
    if (h && key && std::string(key) == "k3_fp64_tensor_cores") {
        if (value < 0 || value > 3) return fail(h, FDGA_ERR_ARG, "k3_fp64_tensor_cores takes 0, 1, 2 or 3");
        if (value && k3_oz_supported(h->d)) {
            if (int r = ensure_k3_oz(h)) return r;
            CK(prepare_bse_K3_oz());
            CK(cudaStreamSynchronize(h->st));
        }
        h->k3_oz = value;
        drop_graphs(h);
        return FDGA_OK;
    }
    if (!h || !key) return FDGA_ERR_ARG;
    const std::string k(key);
    if (k == "k3_tensor_cores") {
        h->k3_tc = value ? 1 : 0;
        drop_graphs(h);
        return FDGA_OK;
    }
    if (k == "k3_tma") {
        h->k3_tma = value ? 1 : 0;
        drop_graphs(h);
        return FDGA_OK;
    }
    if (k == "jvp_tangent") {
        h->jvp_tangent = value ? 1 : 0;
        return FDGA_OK;
    }
    if (k == "fused_residual") {
        h->fused_residual = value ? 1 : 0;
        return FDGA_OK;
    }
    if (k == "newton_gmres_cycles") {
        if (value < 1 || value > 64) return fail(h, FDGA_ERR_ARG, "newton_gmres_cycles must be in [1, 64]");
        h->newton_cycles = value;
        return FDGA_OK;
    }
    if (k == "fdpa_single_hartree") {
        h->fdpa_single_hartree = value ? 1 : 0;
        drop_graphs(h);
        return FDGA_OK;
    }
    return fail(h, FDGA_ERR_ARG, "unknown option " + k);
}

int fdga_susceptibility(fdga_handle* h, int channel, double* out, size_t n) {
    if (!h || !out) return fail(h, FDGA_ERR_ARG, "null argument");
    if (channel < FDGA_CHI_M || channel > FDGA_CHI_S) return fail(h, FDGA_ERR_ARG, "unknown susceptibility channel");
    const size_t NO = (size_t)h->d.N1, full = NO * h->d.Nq;
    if (n != full && n != NO) return fail(h, FDGA_ERR_ARG, "susceptibility length must be NΩ1·Nq or NΩ1");
    if (!h->finalized) return fail(h, FDGA_ERR_STATE, "fdga_finalize has not been called");
    if (h->d.U == 0.0) return fail(h, FDGA_ERR_ARG, "susceptibility needs U != 0");
    // tmpS holds at least NΩ1·Nq complex (the state contains the three K1 arrays)
    CK(launch_chi(h->st, chanK(h, h->xS, CH_P, 1), chanK(h, h->xS, CH_T, 1), chanK(h, h->xS, CH_A, 1), channel,
                  h->d.U, (int)NO, h->d.Nq, n == NO && full != NO ? 1 : 0, h->tmpS));
    CK(cudaMemcpyAsync(out, h->tmpS, n * sizeof(cplx), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    return FDGA_OK;
}

int fdga_event_record(fdga_handle* h, int slot) {
    if (!h || slot < 0 || slot >= 8) return FDGA_ERR_ARG;
    CK(cudaEventRecord(h->ev[slot], h->st));
    return FDGA_OK;
}
int fdga_event_elapsed_ms(fdga_handle* h, int a, int b, float* ms) {
    if (!h || !ms || a < 0 || a >= 8 || b < 0 || b >= 8) return FDGA_ERR_ARG;
    CK(cudaEventSynchronize(h->ev[b]));
    CK(cudaEventElapsedTime(ms, h->ev[a], h->ev[b]));
    return FDGA_OK;
}
int fdga_synchronize(fdga_handle* h) {
    if (!h) return FDGA_ERR_ARG;
    CK(cudaStreamSynchronize(h->st));
    return FDGA_OK;
}
}  // extern "C"

namespace {
// per-stage device times of an eager launch sequence (the iteration or its tangent)
int stage_times_impl(fdga_handle* h, int strategy, int nrep, char* names, size_t names_cap, double* ms,
                     int max_stages, int* nstages, bool tangent) {
    if (!h || !ms || !nstages || nrep < 1) return FDGA_ERR_ARG;
    if (!h->finalized) return fail(h, FDGA_ERR_STATE, "fdga_finalize has not been called");
    if (tangent && !h->tan.x) return fail(h, FDGA_ERR_STATE, "fdga_frule has not been called");
    if (tangent && strategy != FDGA_FDPA && strategy != FDGA_SCPA)
        return fail(h, FDGA_ERR_UNSUPPORTED, "the tangent map covers the fdPA and scPA strategies");
    {
        int r = check_strategy(h, strategy);
        if (r) return r;
    }
    if (h->c0_dirty) { int r = compute_C0(h); if (r) return r; }
    std::vector<std::string> nm;
    std::vector<double> acc;
    for (int rep = 0; rep < nrep; ++rep) {
        std::vector<cudaEvent_t> evs;
        std::vector<std::string> cur;
        cudaEvent_t e0;
        CK(cudaEventCreate(&e0));
        CK(cudaEventRecord(e0, h->st));
        evs.push_back(e0);
        int nl = 0;
        StageHook hook = [&](const char* name) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return;
            cudaEventRecord(e, h->st);
            evs.push_back(e);
            cur.push_back(name);
        };
        int r = tangent ? enqueue_tangent(h, strategy, true, true, nl, hook)
                        : enqueue_iteration(h, strategy, true, true, nl, hook);
        if (r) return r;
        CK(cudaStreamSynchronize(h->st));
        if (rep == 0) { nm = cur; acc.assign(cur.size(), 0.0); }
        for (size_t i = 0; i + 1 < evs.size() && i < acc.size(); ++i) {
            float t = 0.f;
            cudaEventElapsedTime(&t, evs[i], evs[i + 1]);
            acc[i] += t;
        }
        for (auto e : evs) cudaEventDestroy(e);
        if (!tangent) CK(cudaMemcpyAsync(h->xS, h->yS, h->nstate * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
    }
    CK(cudaStreamSynchronize(h->st));
    const int n = (int)std::min<size_t>(nm.size(), (size_t)max_stages);
    std::string joined;
    for (int i = 0; i < n; ++i) {
        ms[i] = acc[i] / nrep;
        joined += nm[i];
        if (i + 1 < n) joined += ",";
    }
    if (names && names_cap > 0) {
        std::strncpy(names, joined.c_str(), names_cap - 1);
        names[names_cap - 1] = 0;
    }
    *nstages = n;
    return FDGA_OK;
}
}  // namespace

extern "C" {

int fdga_stage_times(fdga_handle* h, int strategy, int nrep, char* names, size_t names_cap, double* ms, int max_stages,
                     int* nstages) {
    return stage_times_impl(h, strategy, nrep, names, names_cap, ms, max_stages, nstages, false);
}
int fdga_tangent_stage_times(fdga_handle* h, int strategy, int nrep, char* names, size_t names_cap, double* ms,
                             int max_stages, int* nstages) {
    return stage_times_impl(h, strategy, nrep, names, names_cap, ms, max_stages, nstages, true);
}

int fdga_map_repeat(fdga_handle* h, int strategy, int n) {
    if (!h || n < 0) return FDGA_ERR_ARG;
    for (int i = 0; i < n; ++i) {
        int r = run_iteration(h, strategy, true, true);
        if (r) return r;
    }
    return FDGA_OK;
}

int fdga_tangent_repeat(fdga_handle* h, int strategy, int n) {
    if (!h || n < 0) return FDGA_ERR_ARG;
    if (!h->tan.x) return fail(h, FDGA_ERR_STATE, "fdga_frule has not been called");
    for (int i = 0; i < n; ++i) {
        int r = run_tangent(h, strategy, true, true);
        if (r) return r;
    }
    return FDGA_OK;
}

// benchmark helper: replay the adjoint graph n times at the base point and cotangent of the last
// fdga_rrule (no host sync)
int fdga_adjoint_repeat(fdga_handle* h, int strategy, int n) {
    if (!h || n < 0) return FDGA_ERR_ARG;
    if (strategy != FDGA_FDPA && strategy != FDGA_SCPA)
        return fail(h, FDGA_ERR_UNSUPPORTED, "the adjoint map covers the fdPA and scPA strategies");
    if (!h->adj.graphs[strategy][1][1].exec) return fail(h, FDGA_ERR_STATE, "fdga_rrule has not been called");
    for (int i = 0; i < n; ++i) {
        int r = run_adjoint(h, strategy, true, true);
        if (r) return r;
    }
    return FDGA_OK;
}

int fdga_host_alloc(size_t bytes, void** p) {
    if (!p) return FDGA_ERR_ARG;
    cudaError_t e = cudaHostAlloc(p, bytes ? bytes : 1, cudaHostAllocDefault);
    if (e != cudaSuccess) { g_create_error = cudaGetErrorString(e); *p = nullptr; return FDGA_ERR_OOM; }
    return FDGA_OK;
}
int fdga_host_free(void* p) {
    return cudaFreeHost(p) == cudaSuccess ? FDGA_OK : FDGA_ERR_CUDA;
}

int fdga_flush_l2(fdga_handle* h, size_t bytes) {
    if (!h || bytes == 0) return FDGA_ERR_ARG;
    if (h->flush_bytes < bytes) {
        if (h->flush_buf) cudaFree(h->flush_buf);
        h->flush_buf = nullptr;
        h->flush_bytes = 0;
        cudaError_t e = cudaMalloc(&h->flush_buf, bytes);
        if (e != cudaSuccess) return fail(h, FDGA_ERR_OOM, std::string("flush buffer: ") + cudaGetErrorString(e));
        h->flush_bytes = bytes;
    }
    CK(cudaMemsetAsync(h->flush_buf, ++h->flush_val, bytes, h->st));  // a new value each time
    return FDGA_OK;
}

int fdga_query(fdga_handle* h, const char* key, double* value) {
    if (!key || !value) return fail(h, FDGA_ERR_ARG, "null argument");
    const std::string k(key);
    if (k == "fp64_gflops") {  // device calibration: FP64 FMA throughput of this GPU
        float ms = 0.f;
        const cudaError_t e = measure_fp64_rate(&ms, value);
        if (e != cudaSuccess) return cuda_fail(h, e, "fp64 calibration");
        return FDGA_OK;
    }
    if (k == "selftest_d2f") {  // mismatches of the integer-path FP64 -> FP32 rounding over 2^26 inputs
        unsigned int mm = 0;
        const cudaError_t e = selftest_d2f((size_t)1 << 26, &mm);
        if (e != cudaSuccess) return cuda_fail(h, e, "d2f self-check");
        *value = mm;
        return FDGA_OK;
    }
    if (!h) return FDGA_ERR_ARG;
    if (k == "k3_blocks") { *value = h->nk3blocks; return FDGA_OK; }
    if (k == "k3_block_dim") { *value = h->d.N3n; return FDGA_OK; }
    if (k == "state_len") { *value = (double)h->nstate; return FDGA_OK; }
    if (k == "launches") { *value = h->last_launches; return FDGA_OK; }
    if (k == "precision") { *value = h->precision; return FDGA_OK; }
    if (k == "k3_fp64_tensor_cores") { *value = use_k3_oz(h) ? 1.0 : 0.0; return FDGA_OK; }
    return fail(h, FDGA_ERR_ARG, "unknown query key " + k);
}

int fdga_autotune(fdga_handle* h, int strategy, int* tiles) {
    if (!h) return FDGA_ERR_ARG;
    if (!h->finalized) return fail(h, FDGA_ERR_STATE, "fdga_finalize has not been called");
    if (int r = check_strategy(h, strategy)) return r;
    if (h->c0_dirty) { int r = compute_C0(h); if (r) return r; }
    if (int r = ensure_mixed(h)) return r;
    // size classes shared by all handles of the process: (Nν3, local, precision) -> (tile L_K3, tile K3)
    static std::mutex mu;
    static std::map<std::tuple<int, int, int>, std::pair<int, int>> cache;
    const int prec0 = h->precision;
    const int cand[6] = {16, 24, 32, 116, 124, 132};
    for (int prec = FDGA_FP64; prec <= FDGA_MIXED; ++prec) {
        const auto key = std::make_tuple(h->d.N3n, h->d.local, prec);
        {
            std::lock_guard<std::mutex> lk(mu);
            auto it = cache.find(key);
            if (it != cache.end()) {
                h->k3_tile[prec][0] = it->second.first;
                h->k3_tile[prec][1] = it->second.second;
                continue;
            }
        }
        double best[2] = {INFINITY, INFINITY};
        int pick[2] = {0, 0};
        h->precision = prec;
        for (int t : cand) {
            h->k3_tile[prec][0] = h->k3_tile[prec][1] = t;
            double acc[2] = {0.0, 0.0};
            for (int rep = 0; rep < 3; ++rep) {
                std::vector<cudaEvent_t> evs;
                std::vector<std::string> names;
                cudaEvent_t e0;
                CK(cudaEventCreate(&e0));
                CK(cudaEventRecord(e0, h->st));
                evs.push_back(e0);
                StageHook hook = [&](const char* name) {
                    cudaEvent_t e;
                    if (cudaEventCreate(&e) != cudaSuccess) return;
                    cudaEventRecord(e, h->st);
                    evs.push_back(e);
                    names.push_back(name);
                };
                int nl = 0;
                int r = enqueue_iteration(h, strategy, true, true, nl, hook);
                if (r) { h->precision = prec0; return r; }
                CK(cudaStreamSynchronize(h->st));
                for (size_t i = 0; i + 1 < evs.size(); ++i) {
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, evs[i], evs[i + 1]);
                    if (rep > 0 && names[i] == std::string("bse_L_K3_gemm")) acc[0] += ms;
                    if (rep > 0 && names[i] == std::string("bse_K3_gemm")) acc[1] += ms;
                }
                for (auto e : evs) cudaEventDestroy(e);
            }
            for (int m = 0; m < 2; ++m)
                if (acc[m] < best[m]) { best[m] = acc[m]; pick[m] = t; }
        }
        h->k3_tile[prec][0] = pick[0];
        h->k3_tile[prec][1] = pick[1];
        std::lock_guard<std::mutex> lk(mu);
        cache[key] = {pick[0], pick[1]};
    }
    h->precision = prec0;
    drop_graphs(h);
    if (tiles)
        for (int p = 0; p < 2; ++p)
            for (int m = 0; m < 2; ++m) tiles[2 * p + m] = h->k3_tile[p][m];
    return FDGA_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Batches of independent solvers: one CUDA graph holds one iteration of every instance, each
// instance a branch forked from and joined into the batch stream.
// ---------------------------------------------------------------------------------------------
struct fdga_batch {
    std::vector<fdga_handle*> hs;
    cudaStream_t st = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaGraphExec_t exec[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};  // [strategy][precision]
    int nodes[2][2] = {{0, 0}, {0, 0}};
    std::string err;
};

extern "C" {

int fdga_batch_create(fdga_handle* const* hs, int n, fdga_batch** out) {
    if (!hs || n < 1 || !out) { g_create_error = "invalid batch arguments"; return FDGA_ERR_ARG; }
    for (int i = 0; i < n; ++i)
        if (!hs[i] || !hs[i]->finalized) { g_create_error = "every batch member must be a finalized handle"; return FDGA_ERR_STATE; }
    {  // each member's state is written by its own branch of the batch graph: no handle twice
        std::vector<const fdga_handle*> v(hs, hs + n);
        std::sort(v.begin(), v.end());
        if (std::adjacent_find(v.begin(), v.end()) != v.end()) {
            g_create_error = "a handle appears twice in the batch";
            return FDGA_ERR_ARG;
        }
    }
    fdga_batch* b = new fdga_batch();
    b->hs.assign(hs, hs + n);
    if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->ev[0]) != cudaSuccess || cudaEventCreate(&b->ev[1]) != cudaSuccess) {
        g_create_error = "batch stream/event creation failed";
        fdga_batch_destroy(b);  // releases what was created
        return FDGA_ERR_CUDA;
    }
    b->join.assign(n, nullptr);
    for (auto& e : b->join) {
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            e = nullptr;
            g_create_error = "batch join event creation failed";
            fdga_batch_destroy(b);
            return FDGA_ERR_CUDA;
        }
    }
    *out = b;
    return FDGA_OK;
}

void fdga_batch_destroy(fdga_batch* b) {
    if (!b) return;
    for (auto& a : b->exec)
        for (auto& g : a)
            if (g) cudaGraphExecDestroy(g);
    for (auto e : b->join) if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    for (auto e : b->ev) if (e) cudaEventDestroy(e);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
}

const char* fdga_batch_last_error(const fdga_batch* b) { return b ? b->err.c_str() : g_create_error.c_str(); }

// S_i <- Φ_i(S_i) for every member (iterate_solver! of each), as one graph launch on the batch stream
int fdga_batch_iterate(fdga_batch* b, int strategy, int precision) {
    if (!b) return FDGA_ERR_ARG;
    if ((strategy != FDGA_FDPA && strategy != FDGA_SCPA) || (precision != FDGA_FP64 && precision != FDGA_MIXED)) {
        b->err = "invalid strategy or precision";
        return FDGA_ERR_ARG;
    }
    cudaGraphExec_t& ex = b->exec[strategy][precision];
    if (!ex) {
        for (auto* h : b->hs)
            if (precision == FDGA_MIXED && ensure_mixed(h)) { b->err = h->err; return FDGA_ERR_OOM; }
        for (auto* h : b->hs)
            if (h->c0_dirty) {
                int r = compute_C0(h);
                if (r) { b->err = h->err; return r; }
            }
        cudaGraph_t graph;
        cudaError_t e = cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) { b->err = cudaGetErrorString(e); return FDGA_ERR_CUDA; }
        e = cudaEventRecord(b->fork, b->st);
        int total = 0, r = FDGA_OK;
        for (size_t i = 0; i < b->hs.size() && e == cudaSuccess && r == FDGA_OK; ++i) {
            fdga_handle* h = b->hs[i];
            e = cudaStreamWaitEvent(h->st, b->fork, 0);
            if (e != cudaSuccess) break;
            const int p0 = h->precision;
            h->precision = precision;
            int nl = 0;
            r = enqueue_iteration(h, strategy, true, true, nl);
            h->precision = p0;
            if (r) { b->err = h->err; break; }
            e = cudaMemcpyAsync(h->xS, h->yS, h->nstate * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st);
            if (e == cudaSuccess) e = cudaEventRecord(b->join[i], h->st);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(b->st, b->join[i], 0);
            total += nl;
        }
        const cudaError_t ee = cudaStreamEndCapture(b->st, &graph);
        if (r || e != cudaSuccess || ee != cudaSuccess) {
            if (ee == cudaSuccess) cudaGraphDestroy(graph);
            if (r) return r;
            b->err = std::string("batch capture: ") + cudaGetErrorString(e != cudaSuccess ? e : ee);
            return FDGA_ERR_CUDA;
        }
        e = cudaGraphInstantiate(&ex, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) { ex = nullptr; b->err = cudaGetErrorString(e); return FDGA_ERR_CUDA; }
        b->nodes[strategy][precision] = total;
    }
    const cudaError_t e = cudaGraphLaunch(ex, b->st);
    if (e != cudaSuccess) { b->err = cudaGetErrorString(e); return FDGA_ERR_CUDA; }
    return FDGA_OK;
}

int fdga_batch_synchronize(fdga_batch* b) {
    if (!b) return FDGA_ERR_ARG;
    const cudaError_t e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) { b->err = cudaGetErrorString(e); return FDGA_ERR_CUDA; }
    return FDGA_OK;
}

// device time of `iters` batch iterations (CUDA events on the batch stream), and the kernels per batch iteration
int fdga_batch_time(fdga_batch* b, int strategy, int precision, int iters, float* ms, int* kernels) {
    if (!b || !ms || iters < 1) return FDGA_ERR_ARG;
    int r = fdga_batch_iterate(b, strategy, precision);  // capture outside the timed region
    if (r) return r;
    cudaError_t e = cudaEventRecord(b->ev[0], b->st);
    for (int i = 0; i < iters && e == cudaSuccess; ++i) {
        r = fdga_batch_iterate(b, strategy, precision);
        if (r) return r;
    }
    if (e == cudaSuccess) e = cudaEventRecord(b->ev[1], b->st);
    if (e == cudaSuccess) e = cudaEventSynchronize(b->ev[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, b->ev[0], b->ev[1]);
    if (e != cudaSuccess) { b->err = cudaGetErrorString(e); return FDGA_ERR_CUDA; }
    if (kernels) *kernels = b->nodes[strategy][precision];
    return FDGA_OK;
}

int fdga_launches_per_iteration(const fdga_handle* h, int* n) {
    if (!h || !n) return FDGA_ERR_ARG;
    *n = h->last_launches;
    return FDGA_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// mfRG / Krylov-preconditioned solver: src/mfRG.jl:20-89 (the map), :93-173 (the preconditioned
// fixed point) and the nlsolve(anderson) driver around it.
// ---------------------------------------------------------------------------------------------
extern "C" {

int fdga_mfrg_apply(fdga_handle* h, int strategy, const double* x, double* y, size_t n) {
    if (!h || !x || !y) return fail(h, FDGA_ERR_ARG, "null argument");
    int r = check_mfrg(h, strategy);
    if (r) return r;
    const size_t nv = 3 * h->nchan;
    if (n != nv) return fail(h, FDGA_ERR_ARG, "the mfRG map acts on the vertex part of the state (length(S.F))");
    cudaStream_t s = h->st;
    CK(cudaMemcpyAsync(h->tmpS, x, nv * sizeof(cplx), cudaMemcpyHostToDevice, s));
    CK(launch_scatter(s, h->mf.u, h->tmpS, h->perm, nv));
    CK(launch_scale(s, h->mf.x, h->mf.u, kMfrgFactor, nv));
    if ((r = mfrg_prepare(h))) return r;
    if ((r = run_mfrg(h))) return r;
    CK(launch_kr_axpby(s, NBLK_RED, h->mf.u, h->mf.u, -1.0 / kMfrgFactor, h->mf.y, nv));
    CK(launch_gather(s, h->tmpS, h->mf.u, h->perm, nv));
    CK(cudaMemcpyAsync(y, h->tmpS, nv * sizeof(cplx), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return check_device_error(h);
}

int fdga_residual_mfrg(fdga_handle* h, int strategy, const double* x, double* R, size_t n, int update_sigma,
                       int krylov_maxiter, double krylov_rtol, double krylov_atol, int* krylov_iters,
                       double* krylov_res) {
    if (!h || !x || !R) return fail(h, FDGA_ERR_ARG, "null argument");
    int r = check_mfrg(h, strategy);
    if (r) return r;
    if (krylov_maxiter < 1 || !(krylov_rtol >= 0) || !(krylov_atol >= 0))
        return fail(h, FDGA_ERR_ARG, "invalid Krylov parameters");
    const size_t nv = 3 * h->nchan, nS = h->nGk;
    if (n != (update_sigma ? h->nstate : nv))
        return fail(h, FDGA_ERR_ARG, update_sigma ? "state length mismatch" : "vertex length mismatch");
    if (h->c0_dirty && (r = compute_C0(h))) return r;
    cudaStream_t s = h->st;
    // x (unsymmetrised) in mf.u; the solver symmetrised from it in xS
    CK(cudaMemcpyAsync(h->tmpS, x, n * sizeof(cplx), cudaMemcpyHostToDevice, s));
    if (!update_sigma) CK(cudaMemcpyAsync(h->mf.u + nv, sigmaOf(h, h->xS), nS * sizeof(cplx), cudaMemcpyDeviceToDevice, s));
    CK(launch_scatter(s, h->mf.u, h->tmpS, h->perm, n));
    CK(cudaMemcpyAsync(h->xS, h->mf.u, h->nstate * sizeof(cplx), cudaMemcpyDeviceToDevice, s));
    if ((r = symmetrize_state(h))) return r;
    if ((r = run_iteration(h, strategy, update_sigma != 0, true))) return r;
    int nmaps = 0, iters = 0;
    double relres = 0.0;
    if ((r = mfrg_krylov(h, h->yS, h->mf.u, krylov_maxiter, krylov_rtol, krylov_atol, nmaps, iters, relres))) return r;
    // R = [z ; Σ(x) - x_Σ]
    CK(cudaMemsetAsync(h->mf.x, 0, nv * sizeof(cplx), s));
    CK(launch_kc_axpy(s, NBLK_RED, h->mf.x, h->kr64[2], h->kc_code, 1.0, h->mf.x, nv));
    if (update_sigma) CK(launch_sub(s, h->mf.x + nv, sigmaOf(h, h->yS), h->mf.u + nv, nS));
    CK(launch_gather(s, h->tmpS, h->mf.x, h->perm, n));
    CK(cudaMemcpyAsync(R, h->tmpS, n * sizeof(cplx), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h->xS, h->yS, h->nstate * sizeof(cplx), cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
    if (krylov_iters) *krylov_iters = iters;
    if (krylov_res) *krylov_res = relres;
    return check_device_error(h);
}

int fdga_solve_mfrg(fdga_handle* h, int strategy, int maxiter, double tol, double beta, int mem, int update_sigma,
                    int krylov_maxiter, double krylov_rtol, double krylov_atol, int* iters, double* res,
                    double* trace, int* krylov_total) {
    if (!h) return FDGA_ERR_ARG;
    int r = check_mfrg(h, strategy);
    if (r) return r;
    if (krylov_maxiter < 1 || !(krylov_rtol >= 0) || !(krylov_atol >= 0))
        return fail(h, FDGA_ERR_ARG, "invalid Krylov parameters");
    const size_t nv = 3 * h->nchan, nS = h->nGk;
    int total = 0;
    SolveHooks hk;
    hk.before = [&]() -> int {  // keep x, iterate from its symmetrised copy (symmetrize_solver!)
        CK(cudaMemcpyAsync(h->mf.u, h->xS, h->nstate * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
        return symmetrize_state(h);
    };
    hk.after = [&]() -> int {  // y ← x + [M⁻¹ R_F ; R_Σ]
        int nmaps = 0, it = 0;
        double relres = 0.0;
        int rr = mfrg_krylov(h, h->yS, h->mf.u, krylov_maxiter, krylov_rtol, krylov_atol, nmaps, it, relres);
        if (rr) return rr;
        total += it;
        CK(launch_kc_axpy(h->st, NBLK_RED, h->mf.u, h->kr64[2], h->kc_code, 1.0, h->yS, nv));
        if (!update_sigma)
            CK(cudaMemcpyAsync(sigmaOf(h, h->yS), h->mf.u + nv, nS * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
        CK(cudaMemcpyAsync(h->xS, h->mf.u, h->nstate * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
        return FDGA_OK;
    };
    r = solve_anderson(h, strategy, update_sigma != 0, maxiter, tol, beta, mem, iters, res, trace, &hk);
    if (krylov_total) *krylov_total = total;
    if (r) return r;
    // unflatten!(S, res.zero); symmetrize_solver!(S): the last evaluated x
    CK(cudaMemcpyAsync(h->xS, h->mf.u, h->nstate * sizeof(cplx), cudaMemcpyDeviceToDevice, h->st));
    if ((r = symmetrize_state(h))) return r;
    return check_device_error(h);
}

}  // extern "C"
