// fdga_oracle.cpp -- CPU ORACLE (test infrastructure only).
//
// A plain C++17/OpenMP restatement of the parquet-iteration hot path of fdDGAsolver.jl,
// used ONLY as the checker in tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
// --impl reference leg.  Nothing in the product library links or calls this file.
//
// It follows the reference loop by loop, in FP64 complex arithmetic, on the reference's own
// column-major storage (first mesh index fastest):
//   * channel/vertex evaluators        src/channel.jl:220-339, src/vertex.jl:209-336,
//                                      src/refvertex.jl:90-216, src/nonlocal/channel.jl:226-382,
//                                      src/nonlocal/vertex.jl:69-379, src/nonlocal/swave.jl:32-88
//   * frequency conversion             src/convention.jl:4-36
//   * Dyson / occupation               src/dyson.jl:5-41
//   * bubbles                          src/bubble.jl:9-36, src/nonlocal/bubble.jl:87-158
//   * K3 caches                        src/build_K3_cache.jl:20-95, src/nonlocal/build_K3_cache.jl:18-94
//   * BSE (K1, L_K2, K2, L_K3, K3)     src/BSE_templates.jl:12-180, src/BSEa/*.jl,
//                                      src/nonlocal/BSEa/*.jl
//   * SDE                              src/SDE.jl:3-364, src/nonlocal/SDE.jl:3-447
//   * iteration / residual             src/solve.jl:4-157, src/ParquetSolver.jl:277-306
//   * symmetry groups                  src/symmetries.jl, src/nonlocal/symmetries.jl,
//                                      src/ParquetSolver.jl:203-231, src/nonlocal/ParquetSolver.jl:198-300
// Third-party algorithms restated from their published descriptions (not vendored):
//   * MatsubaraFunctions.jl 0.1.0 (branch mesh_generalization_v3) SymmetryGroup: a class is the
//     set of mesh points reachable from a seed by the listed symmetries while staying in the
//     box; seeds are taken in linear-index order, so the representative is the first member;
//     evaluation computes the representative and assigns op(value) to every member.
//   * NLsolve.jl 4.5.1 Anderson acceleration (Walker & Ni 2011, type-II, QR-updated least
//     squares with Givens column deletion), beta mixing, history m, ftol on max|f|.
//   * FFTW fft/bfft are replaced by direct separable DFTs with the same sign/normalisation.
//
// The q-averages taken when a momentum argument is the s-wave point kSW (swave.jl:32-88) are
// memoised once per iteration: the sum is the same sum the reference forms at every call.

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using cd = std::complex<double>;

namespace orc {

static const int FINF = -(1 << 30);  // the infinite fermionic frequency νInf
static const int KSW = -1;           // the s-wave momentum point kSW
enum { CH_P = 0, CH_T = 1, CH_A = 2 };
enum { SP_P = 0, SP_X = 1, SP_D = 2 };

static inline bool bin(int m, int N) { return m > -N && m < N; }    // boson mesh, 2N-1 points
static inline bool fin(int n, int N) { return n >= -N && n < N; }   // fermion mesh, 2N points
static inline int imod(int a, int L) { int r = a % L; return r < 0 ? r + L : r; }

// --------------------------------------------------------------------------------------------
// Channel: K1[Ω,P], K2[Ω,ν,P], K3[Ω,ν,ν',P] (column-major).  src/nonlocal/channel.jl:3-45
// --------------------------------------------------------------------------------------------
struct Chan {
    int n1 = 1, n2O = 1, n2n = 1, n3O = 1, n3n = 1, Nq = 1;
    int N1 = 1, N2O = 1, N2n = 2, N3O = 1, N3n = 2;
    std::vector<cd> K1, K2, K3;
    std::vector<cd> A1, A2, A3;  // q-averages (kSW evaluation)

    void init(int nK1, int nK2O, int nK2n, int nK3O, int nK3n, int nq) {
        n1 = nK1; n2O = nK2O; n2n = nK2n; n3O = nK3O; n3n = nK3n; Nq = nq;
        N1 = 2 * n1 - 1; N2O = 2 * n2O - 1; N2n = 2 * n2n; N3O = 2 * n3O - 1; N3n = 2 * n3n;
        K1.assign((size_t)N1 * Nq, 0.0);
        K2.assign((size_t)N2O * N2n * Nq, 0.0);
        K3.assign((size_t)N3O * N3n * N3n * Nq, 0.0);
    }
    size_t len1() const { return (size_t)N1 * Nq; }
    size_t len2() const { return (size_t)N2O * N2n * Nq; }
    size_t len3() const { return (size_t)N3O * N3n * N3n * Nq; }
    size_t length() const { return len1() + len2() + len3(); }
    size_t i1(int m, int P) const { return (size_t)(m + n1 - 1) + (size_t)N1 * P; }
    size_t i2(int m, int n, int P) const {
        return (size_t)(m + n2O - 1) + (size_t)N2O * ((size_t)(n + n2n) + (size_t)N2n * P);
    }
    size_t i3(int m, int n, int np, int P) const {
        return (size_t)(m + n3O - 1) +
               (size_t)N3O * ((size_t)(n + n3n) + (size_t)N3n * ((size_t)(np + n3n) + (size_t)N3n * P));
    }
    // sum(view(f, i..., :)) / length(mesh_P)   (swave.jl:32-72)
    void update_avg() {
        A1.assign(N1, 0.0); A2.assign((size_t)N2O * N2n, 0.0); A3.assign((size_t)N3O * N3n * N3n, 0.0);
        for (int P = 0; P < Nq; ++P) {
            for (size_t i = 0; i < (size_t)N1; ++i) A1[i] += K1[i + (size_t)N1 * P];
            for (size_t i = 0; i < A2.size(); ++i) A2[i] += K2[i + A2.size() * P];
            for (size_t i = 0; i < A3.size(); ++i) A3[i] += K3[i + A3.size() * P];
        }
        for (auto& v : A1) v /= (double)Nq;
        for (auto& v : A2) v /= (double)Nq;
        for (auto& v : A3) v /= (double)Nq;
    }
    cd k1(int m, int P) const { return P == KSW ? A1[m + n1 - 1] : K1[i1(m, P)]; }
    cd k2(int m, int n, int P) const { return P == KSW ? A2[i2(m, n, 0)] : K2[i2(m, n, P)]; }
    cd k3(int m, int n, int np, int P) const { return P == KSW ? A3[i3(m, n, np, 0)] : K3[i3(m, n, np, P)]; }

    // Evaluator, src/channel.jl:220-339 and src/nonlocal/channel.jl:246-382.
    cd eval(int m, int n, int np, int P, bool K1f = true, bool K2f = true, bool K3f = true) const {
        cd val = 0.0;
        const bool ninf = (n == FINF), npinf = (np == FINF);
        if (!ninf && !npinf) {
            if (bin(m, n1)) {
                if (K1f) val += k1(m, P);
                if (bin(m, n2O)) {
                    const bool a = fin(n, n2n), b = fin(np, n2n);
                    if (a && b) {
                        if (K2f) val += k2(m, n, P) + k2(m, np, P);
                        if (K3f && bin(m, n3O) && fin(n, n3n) && fin(np, n3n)) val += k3(m, n, np, P);
                    } else if (a) {
                        if (K2f) val += k2(m, n, P);
                    } else if (b) {
                        if (K2f) val += k2(m, np, P);
                    }
                }
            }
        } else if (ninf && !npinf) {
            if (K1f) {
                if (bin(m, n1)) {
                    val += k1(m, P);
                    if (K2f && bin(m, n2O) && fin(np, n2n)) val += k2(m, np, P);
                }
            } else if (K2f && bin(m, n2O) && fin(np, n2n)) {
                val += k2(m, np, P);
            }
        } else if (!ninf && npinf) {
            if (K1f) {
                if (bin(m, n1)) {
                    val += k1(m, P);
                    if (K2f && bin(m, n2O) && fin(n, n2n)) val += k2(m, n, P);
                }
            } else if (K2f && bin(m, n2O) && fin(n, n2n)) {
                val += k2(m, n, P);
            }
        } else {
            if (K1f && bin(m, n1)) val += k1(m, P);
        }
        return val;
    }
};

// --------------------------------------------------------------------------------------------
// RefVertex: U + local K3-shaped corrections.  src/refvertex.jl:1-216
// --------------------------------------------------------------------------------------------
struct RefV {
    cd U = 0.0;
    int nRO = 1, nRn = 1, NRO = 1, NRn = 2;
    std::vector<cd> Fp_p, Fp_x, Ft_p, Ft_x;
    void init(cd u, int nO, int nn) {
        U = u; nRO = nO; nRn = nn; NRO = 2 * nO - 1; NRn = 2 * nn;
        size_t n = (size_t)NRO * NRn * NRn;
        Fp_p.assign(n, 0.0); Fp_x.assign(n, 0.0); Ft_p.assign(n, 0.0); Ft_x.assign(n, 0.0);
    }
    // MeshFunction call: zero outside the box
    cd call(const std::vector<cd>& f, int m, int n, int np) const {
        if (!bin(m, nRO) || !fin(n, nRn) || !fin(np, nRn)) return 0.0;
        return f[(size_t)(m + nRO - 1) + (size_t)NRO * ((size_t)(n + nRn) + (size_t)NRn * (np + nRn))];
    }
    cd bare(int sp) const { return sp == SP_X ? -U : U; }
    cd eval(int ch, int sp, int m, int n, int np) const {
        if (n == FINF || np == FINF) return bare(sp);
        if (sp == SP_D) return 2.0 * eval(ch, SP_P, m, n, np) + eval(ch, SP_X, m, n, np);
        if (sp == SP_P) {
            if (ch == CH_P) return call(Fp_p, m, n, np) + U;
            if (ch == CH_T) return call(Ft_p, m, n, np) + U;
            return -call(Ft_x, m, np, n) + U;
        }
        if (ch == CH_P) return call(Fp_x, m, n, np) - U;
        if (ch == CH_T) return call(Ft_x, m, n, np) - U;
        return -call(Ft_p, m, np, n) - U;
    }
};

// Frequency conversion on mesh indices, src/convention.jl:4-36 with
// Ω_m - ν_n -> fermion m-n-1, Ω_m + ν_n -> m+n, ν_n - ν_n' -> boson n-n', ν_n + ν_n' -> boson n+n'+1.
static inline void conv(int from, int to, int m, int n, int np, int& mo, int& no, int& npo) {
    if (from == to) { mo = m; no = n; npo = np; return; }
    if (from == CH_P && to == CH_T) { mo = m - n - np - 1; no = np; npo = n; return; }
    if (from == CH_P && to == CH_A) { mo = n - np; no = m - n - 1; npo = np; return; }
    if (from == CH_T && to == CH_P) { mo = m + n + np + 1; no = np; npo = n; return; }
    if (from == CH_T && to == CH_A) { mo = np - n; no = m + n; npo = n; return; }
    if (from == CH_A && to == CH_P) { mo = m + np + n + 1; no = m + np; npo = np; return; }
    /* a -> t */ mo = n - np; no = np; npo = m + np;
}

struct Flags { bool f0 = true, gp = true, gt = true, ga = true; };

struct Vert;
struct AnyV {  // F0 of a vertex: a RefVertex or another Vertex
    const RefV* ref = nullptr;
    const Vert* vert = nullptr;
};

struct Vert {
    AnyV F0;
    Chan g[3];  // p, t, a
    int Nq = 1;
    void init(int nK1, int nK2O, int nK2n, int nK3O, int nK3n, int nq) {
        Nq = nq;
        for (auto& c : g) c.init(nK1, nK2O, nK2n, nK3O, nK3n, nq);
    }
    void update_avg() { for (auto& c : g) c.update_avg(); }
    size_t length() const { return 3 * g[0].length(); }
    cd bare() const;
    cd eval(int ch, int sp, int m, int n, int np, int P, Flags fl = Flags()) const;
};

static inline cd any_eval(const AnyV& v, int ch, int sp, int m, int n, int np, int P) {
    if (v.ref) return v.ref->eval(ch, sp, m, n, np);
    return v.vert->eval(ch, sp, m, n, np, P);
}

cd Vert::bare() const { return F0.ref ? F0.ref->U : F0.vert->bare(); }

// Vertex evaluator with momentum arguments (P, kSW, kSW): src/vertex.jl:209-336,
// src/nonlocal/vertex.jl:69-211 and the s-wave methods :216-379.  A local vertex (Nq = 1)
// ignores momenta (src/nonlocal/channel.jl:385-412).
cd Vert::eval(int ch, int sp, int m, int n, int np, int P, Flags fl) const {
    const int Pv = (Nq == 1) ? 0 : P;
    if (sp == SP_D) {
        cd val = 0.0;
        val += eval(ch, SP_P, m, n, np, P, fl) * 2.0;
        val += eval(ch, SP_X, m, n, np, P, fl);
        return val;
    }
    if (sp == SP_X) {
        Flags sw; sw.f0 = fl.f0; sw.gp = fl.gp; sw.gt = fl.ga; sw.ga = fl.gt;
        if (ch == CH_P) return -eval(CH_P, SP_P, m, n, (np == FINF) ? FINF : m - np - 1, P, sw);
        if (ch == CH_T) return -eval(CH_A, SP_P, m, n, np, P, sw);
        return -eval(CH_T, SP_P, m, n, np, P, sw);
    }
    cd val = 0.0;
    if (fl.f0) val += any_eval(F0, ch, SP_P, m, n, np, P);
    if (n == FINF || np == FINF) {
        if (ch == CH_P && fl.gp) val += g[CH_P].eval(m, n, np, Pv);
        if (ch == CH_T && fl.gt) val += g[CH_T].eval(m, n, np, Pv);
        if (ch == CH_A && fl.ga) val += g[CH_A].eval(m, n, np, Pv);
        return val;
    }
    const bool on[3] = {fl.gp, fl.gt, fl.ga};
    for (int r = 0; r < 3; ++r) {
        if (!on[r]) continue;
        int mo, no, npo;
        conv(ch, r, m, n, np, mo, no, npo);
        val += g[r].eval(mo, no, npo, (r == ch) ? Pv : (Nq == 1 ? 0 : KSW));
    }
    return val;
}

// --------------------------------------------------------------------------------------------
// Symmetry groups (MatsubaraFunctions SymmetryGroup semantics, restated).
// A shape is up to 4 axes, each boson(N) / fermion(N) / momentum(L*L), column-major.
// --------------------------------------------------------------------------------------------
enum AxisKind { AX_B = 0, AX_F = 1, AX_K = 2 };
struct Shape {
    int nax = 0;
    int kind[4] = {0, 0, 0, 0};
    int N[4] = {0, 0, 0, 0};   // mesh parameter (boson/fermion N, or L for momentum)
    int len[4] = {1, 1, 1, 1};
    void add(int k, int n) {
        kind[nax] = k; N[nax] = n;
        len[nax] = (k == AX_B) ? 2 * n - 1 : (k == AX_F ? 2 * n : n * n);
        ++nax;
    }
    size_t size() const { size_t s = 1; for (int a = 0; a < nax; ++a) s *= (size_t)len[a]; return s; }
    void decode(size_t idx, int w[4]) const {
        for (int a = 0; a < nax; ++a) {
            int p = (int)(idx % (size_t)len[a]); idx /= (size_t)len[a];
            w[a] = (kind[a] == AX_B) ? p - (N[a] - 1) : (kind[a] == AX_F ? p - N[a] : p);
        }
    }
    bool inb(const int w[4]) const {
        for (int a = 0; a < nax; ++a) {
            if (kind[a] == AX_B && !bin(w[a], N[a])) return false;
            if (kind[a] == AX_F && !fin(w[a], N[a])) return false;
        }
        return true;
    }
    size_t encode(const int w[4]) const {
        size_t idx = 0, stride = 1;
        for (int a = 0; a < nax; ++a) {
            int p = (kind[a] == AX_B) ? w[a] + N[a] - 1 : (kind[a] == AX_F ? w[a] + N[a] : w[a]);
            idx += stride * (size_t)p; stride *= (size_t)len[a];
        }
        return idx;
    }
};

// Momentum helpers on index P = x + L*y (src/nonlocal/symmetries.jl:4-12).
static inline int k_neg(int P, int L) { int x = P % L, y = P / L; return imod(-x, L) + L * imod(-y, L); }
static inline int k_ref(int P, int L) { int x = P % L, y = P / L; return y + L * x; }
static inline int k_rot(int P, int L) { int x = P % L, y = P / L; return y + L * imod(-x, L); }

// op bits: 1 = sgn, 2 = con
typedef int (*SymFn)(const int w[4], int o[4], int L);

// local symmetries src/symmetries.jl:2-94, extended with momentum (src/nonlocal/symmetries.jl)
static int s_sigma(const int w[4], int o[4], int L) { o[0] = -w[0] - 1; o[1] = L > 1 ? k_neg(w[1], L) : w[1]; return 3; }
static int s_sigma_ref(const int w[4], int o[4], int L) { o[0] = w[0]; o[1] = k_ref(w[1], L); return 0; }
static int s_sigma_rot(const int w[4], int o[4], int L) { o[0] = w[0]; o[1] = k_rot(w[1], L); return 0; }
static int s_k1_conj(const int w[4], int o[4], int L) { o[0] = -w[0]; o[1] = L > 1 ? k_neg(w[1], L) : w[1]; return 2; }
static int s_k1_ref(const int w[4], int o[4], int L) { o[0] = w[0]; o[1] = k_ref(w[1], L); return 0; }
static int s_k1_rot(const int w[4], int o[4], int L) { o[0] = w[0]; o[1] = k_rot(w[1], L); return 0; }
static int s_k2pp1(const int w[4], int o[4], int L) { o[0] = -w[0]; o[1] = -w[1] - 1; o[2] = L > 1 ? k_neg(w[2], L) : w[2]; return 2; }
static int s_k2pp2(const int w[4], int o[4], int L) { (void)L; o[0] = w[0]; o[1] = w[0] - w[1] - 1; o[2] = w[2]; return 0; }
static int s_k2ph2(const int w[4], int o[4], int L) { o[0] = -w[0]; o[1] = w[0] + w[1]; o[2] = L > 1 ? k_neg(w[2], L) : w[2]; return 0; }
static int s_k2_ref(const int w[4], int o[4], int L) { o[0] = w[0]; o[1] = w[1]; o[2] = k_ref(w[2], L); return 0; }
static int s_k2_rot(const int w[4], int o[4], int L) { o[0] = w[0]; o[1] = w[1]; o[2] = k_rot(w[2], L); return 0; }
static int s_k3pp1(const int w[4], int o[4], int L) { o[0] = -w[0]; o[1] = -w[1] - 1; o[2] = -w[2] - 1; o[3] = L > 1 ? k_neg(w[3], L) : w[3]; return 2; }
static int s_k3pp2(const int w[4], int o[4], int L) { (void)L; o[0] = w[0]; o[1] = w[2]; o[2] = w[1]; o[3] = w[3]; return 0; }
static int s_k3pp3(const int w[4], int o[4], int L) { (void)L; o[0] = w[0]; o[1] = w[0] - w[1] - 1; o[2] = w[0] - w[2] - 1; o[3] = w[3]; return 0; }
static int s_k3ph3(const int w[4], int o[4], int L) { o[0] = -w[0]; o[1] = w[0] + w[1]; o[2] = w[0] + w[2]; o[3] = L > 1 ? k_neg(w[3], L) : w[3]; return 0; }
static int s_k3_ref(const int w[4], int o[4], int L) { o[0] = w[0]; o[1] = w[1]; o[2] = w[2]; o[3] = k_ref(w[3], L); return 0; }
static int s_k3_rot(const int w[4], int o[4], int L) { o[0] = w[0]; o[1] = w[1]; o[2] = w[2]; o[3] = k_rot(w[3], L); return 0; }

struct SymGroup {
    bool trivial = true;
    std::vector<int> cstart;   // CSR over classes
    std::vector<int> members;  // linear indices; first member of a class is the representative
    std::vector<uint8_t> ops;  // op bits per member
    size_t nclass() const { return trivial ? 0 : cstart.size() - 1; }
};

static SymGroup build_group(const Shape& sh, const std::vector<SymFn>& syms, int L) {
    SymGroup G;
    G.trivial = false;
    const size_t n = sh.size();
    std::vector<uint8_t> checked(n, 0);
    G.cstart.push_back(0);
    std::vector<std::pair<size_t, int>> todo;
    for (size_t idx = 0; idx < n; ++idx) {
        if (checked[idx]) continue;
        checked[idx] = 1;
        G.members.push_back((int)idx); G.ops.push_back(0);
        todo.clear(); todo.push_back({idx, 0});
        while (!todo.empty()) {
            auto cur = todo.back(); todo.pop_back();
            int w[4]; sh.decode(cur.first, w);
            for (auto s : syms) {
                int o[4] = {0, 0, 0, 0};
                int op = s(w, o, L);
                if (!sh.inb(o)) continue;
                size_t j = sh.encode(o);
                if (checked[j]) continue;
                checked[j] = 1;
                int nop = cur.second ^ op;
                G.members.push_back((int)j); G.ops.push_back((uint8_t)nop);
                todo.push_back({j, nop});
            }
        }
        G.cstart.push_back((int)G.members.size());
    }
    return G;
}

static inline cd apply_op(int op, cd v) {
    if (op & 2) v = std::conj(v);
    if (op & 1) v = -v;
    return v;
}

// SG(f, InitFunction(diagram)): evaluate representatives, broadcast with op.
template <class Fn>
static void sg_eval(const SymGroup& G, const Shape& sh, cd* out, Fn diagram) {
    if (G.trivial) {
        const long n = (long)sh.size();
#pragma omp parallel for schedule(dynamic, 16)
        for (long i = 0; i < n; ++i) { int w[4]; sh.decode((size_t)i, w); out[i] = diagram(w); }
        return;
    }
    const long nc = (long)G.nclass();
#pragma omp parallel for schedule(dynamic, 4)
    for (long c = 0; c < nc; ++c) {
        int w[4]; sh.decode((size_t)G.members[G.cstart[c]], w);
        cd v = diagram(w);
        for (int j = G.cstart[c]; j < G.cstart[c + 1]; ++j) out[G.members[j]] = apply_op(G.ops[j], v);
    }
}
// SG(f): symmetrize in place from the representative values.
static void sg_symmetrize(const SymGroup& G, cd* f) {
    if (G.trivial) return;
    for (size_t c = 0; c < G.nclass(); ++c) {
        cd v = f[G.members[G.cstart[c]]];
        for (int j = G.cstart[c] + 1; j < G.cstart[c + 1]; ++j) f[G.members[j]] = apply_op(G.ops[j], v);
    }
}

// --------------------------------------------------------------------------------------------
// DFT helpers over an L x L momentum grid, index x + L*y.  sign -1: fft, +1: bfft (unnormalised)
// --------------------------------------------------------------------------------------------
static void dft2(std::vector<cd>& data, size_t inner, size_t outer_stride, int L, int sign) {
    // data layout [inner, L, L] column-major (inner fastest)
    const size_t N = (size_t)L * L;
    std::vector<cd> w(L);
    for (int j = 0; j < L; ++j) w[j] = std::polar(1.0, sign * 2.0 * M_PI * j / L);
    std::vector<cd> tmp(N);
    (void)outer_stride;
    for (size_t i = 0; i < inner; ++i) {
        // along x
        for (int y = 0; y < L; ++y)
            for (int kx = 0; kx < L; ++kx) {
                cd s = 0.0;
                for (int x = 0; x < L; ++x) s += data[i + inner * (size_t)(x + L * y)] * w[(size_t)(kx * x) % L];
                tmp[kx + L * y] = s;
            }
        for (int kx = 0; kx < L; ++kx)
            for (int ky = 0; ky < L; ++ky) {
                cd s = 0.0;
                for (int y = 0; y < L; ++y) s += tmp[kx + L * y] * w[(size_t)(ky * y) % L];
                data[i + inner * (size_t)(kx + L * ky)] = s;
            }
    }
}

// --------------------------------------------------------------------------------------------
// Solver state: src/ParquetSolver.jl:5-157 and src/nonlocal/ParquetSolver.jl:1-153
// --------------------------------------------------------------------------------------------
struct Dims {
    int nG, nK1, nK2O, nK2n, nK3O, nK3n;
    int L, LG;          // vertex / Green-function momentum meshes (L = LG = 1 for local)
    int fPi;            // bubble fermionic mesh factor
    int local;          // 1: ParquetSolver, 0: NL_ParquetSolver
    double T, U;
    int nRO, nRn;       // RefVertex correction box (1, 1 = null vertex)
    int f0_is_vertex;   // 1: the reference vertex is a Vertex (with RefVertex U) of box nF0*
    int nF0K1, nF0K2O, nF0K2n, nF0K3O, nF0K3n;
};

struct Solver {
    Dims d;
    int Nq = 1, Nk = 1, NG = 0, NPO = 0, NPn = 0, nPO = 0, nPn = 0;
    std::vector<cd> Gbare, G0, Sig0, G, Sig;
    std::vector<cd> Pi0pp, Pi0ph, Pipp, Piph;
    RefV ref;          // RefVertex of the reference (PA) or of the reference vertex
    RefV zero_ref;     // RefVertex(T, 0) used by Fbuff and FL
    Vert F0v;          // reference vertex when f0_is_vertex
    AnyV F0;
    Vert F, Fbuff, FL;
    std::vector<cd> Lpp, Lph, L0pp, L0ph;
    std::vector<cd> cache[10];  // Γpx F0p F0a F0t Γpp Γa Γt Fp Fa Ft
    Shape shK1, shK2, shK3, shSig;
    // symmetry groups: Σ, pp[3], ph[3], ppL[3], phL[3], 0pp2, 0ph2
    SymGroup sgSig, sgpp[3], sgph[3], sgppL[3], sgphL[3], sg0pp2, sg0ph2;
    std::string err;
    // Test-only variant: skip the explicit subtraction of the reference Hartree term at the end
    // of SDE!(S; strategy=:fdPA) (src/SDE.jl:19-24).  The literal source subtracts it there and
    // inside SDE(F0, G0); the golden value of test/test_siam_fdPA.jl:179 matches one subtraction.
    int variant_single_hartree = 0;

    size_t iG(int n, int k) const { return (size_t)(n + d.nG) + (size_t)NG * k; }
    size_t iPi(int m, int n, int P) const { return (size_t)(m + nPO - 1) + (size_t)NPO * ((size_t)(n + nPn) + (size_t)NPn * P); }
    double T() const { return d.T; }
};

enum { C_GPX = 0, C_F0P, C_F0A, C_F0T, C_GPP, C_GA, C_GT, C_FP, C_FA, C_FT };

// --------------------------------------------------------------------------------------------
// Dyson and occupation: src/dyson.jl:5-41
// --------------------------------------------------------------------------------------------
static void dyson(std::vector<cd>& G, const std::vector<cd>& S, const std::vector<cd>& Gb) {
    for (size_t i = 0; i < G.size(); ++i) G[i] = 1.0 / (1.0 / Gb[i] + S[i]);
}
static double occupation(const Solver& s, const std::vector<cd>& G) {
    cd sum = 0.0;
    for (auto v : G) sum += v;
    return 0.5 + sum.imag() * s.d.T / (double)s.Nk;
}

// --------------------------------------------------------------------------------------------
// Bubbles: local src/bubble.jl:9-36; nonlocal real-space src/nonlocal/bubble.jl:87-158
// --------------------------------------------------------------------------------------------
static void bubbles(Solver& s, std::vector<cd>& pp, std::vector<cd>& ph, const std::vector<cd>& G) {
    const double T = s.d.T;
    auto fval = [&](int n) { return (2.0 * n + 1.0) * M_PI * T; };
    if (s.d.local) {
#pragma omp parallel for collapse(2)
        for (int m = -(s.nPO - 1); m <= s.nPO - 1; ++m)
            for (int n = -s.nPn; n < s.nPn; ++n) {
                auto Gt = [&](int k) -> cd { return fin(k, s.d.nG) ? G[s.iG(k, 0)] : cd(1.0 / fval(k), 0.0); };
                cd Gn = Gt(n), Gm = Gt(m - n - 1), Gp = Gt(m + n);
                pp[s.iPi(m, n, 0)] = Gn * Gm;
                ph[s.iPi(m, n, 0)] = Gn * Gp;
            }
        return;
    }
    const int LG = s.d.LG, L = s.d.L, NG = s.NG;
    const size_t NkG = (size_t)LG * LG;
    std::vector<cd> GR(G.begin(), G.end());   // [ν, x, y]
    dft2(GR, NG, 0, LG, -1);
    for (auto& v : GR) v /= (double)NkG;
    std::fill(pp.begin(), pp.end(), 0.0);
    std::fill(ph.begin(), ph.end(), 0.0);
    const int h = L / 2;
    for (int R1 = -h; R1 <= h; ++R1)
        for (int R2 = -h; R2 <= h; ++R2) {
            double weight = 1.0;
            if (LG % 2 == 0) {
                if (std::abs(R1) == LG / 2) weight /= 2;
                if (std::abs(R2) == LG / 2) weight /= 2;
            }
            const int ipR = imod(R1, LG) + LG * imod(R2, LG);
            const int imR = imod(-R1, LG) + LG * imod(-R2, LG);
            const int iRP = imod(R1, L) + L * imod(R2, L);
            const bool R0 = (R1 == 0 && R2 == 0);
            auto Gp = [&](int n) -> cd { return fin(n, s.d.nG) ? GR[s.iG(n, ipR)] : cd(0.0); };
            auto Gm = [&](int n) -> cd { return fin(n, s.d.nG) ? GR[s.iG(n, imR)] : cd(0.0); };
            auto Gpt = [&](int n) -> cd { return fin(n, s.d.nG) ? GR[s.iG(n, ipR)] : cd(1.0 / fval(n), 0.0); };
            auto Gmt = [&](int n) -> cd { return fin(n, s.d.nG) ? GR[s.iG(n, imR)] : cd(1.0 / fval(n), 0.0); };
#pragma omp parallel for collapse(2)
            for (int m = -(s.nPO - 1); m <= s.nPO - 1; ++m)
                for (int n = -s.nPn; n < s.nPn; ++n) {
                    const size_t i = s.iPi(m, n, iRP);
                    if (R0) {
                        pp[i] += Gpt(m - n - 1) * Gpt(n) * weight;
                        ph[i] += Gpt(m + n) * Gmt(n) * weight;
                    } else {
                        pp[i] += Gp(m - n - 1) * Gp(n) * weight;
                        ph[i] += Gp(m + n) * Gm(n) * weight;
                    }
                }
        }
    const size_t inner = (size_t)s.NPO * s.NPn;
    dft2(pp, inner, 0, L, +1);
    dft2(ph, inner, 0, L, +1);
}

// --------------------------------------------------------------------------------------------
// K3 caches: src/build_K3_cache.jl:20-95, src/nonlocal/build_K3_cache.jl:18-94
// --------------------------------------------------------------------------------------------
static void build_K3_cache(Solver& s) {
    const Shape& sh = s.shK3;
    const long n = (long)sh.size();
    const Vert& F = s.F;
    const AnyV& F0 = s.F0;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
        int w[4]; sh.decode((size_t)i, w);
        const int m = w[0], a = w[1], b = w[2], P = (s.Nq == 1) ? 0 : w[3];
        // left: (Ω, ω, ν', P)
        {
            Flags fl; fl.f0 = false; fl.gp = false;
            s.cache[C_GPX][i] = F.eval(CH_P, SP_X, m, a, b, P, fl);
            s.cache[C_F0P][i] = any_eval(F0, CH_P, SP_X, m, a, b, P) - any_eval(F0, CH_P, SP_X, m, a, FINF, P);
            s.cache[C_F0A][i] = any_eval(F0, CH_A, SP_P, m, a, b, P) - any_eval(F0, CH_A, SP_P, m, a, FINF, P);
            cd f0t = any_eval(F0, CH_T, SP_P, m, a, b, P) - any_eval(F0, CH_T, SP_P, m, a, FINF, P);
            s.cache[C_F0T][i] = 2.0 * f0t - s.cache[C_F0A][i];
        }
        // right: (Ω, ν, ω, P)
        {
            Flags fp; fp.f0 = false; fp.gp = false;
            Flags fa; fa.f0 = false; fa.ga = false;
            Flags ft; ft.f0 = false; ft.gt = false;
            cd Gpp = F.eval(CH_P, SP_P, m, a, b, P, fp);
            cd Ga = F.eval(CH_A, SP_P, m, a, b, P, fa);
            cd Gt = F.eval(CH_T, SP_P, m, a, b, P, ft);
            Flags rp; rp.ga = false; rp.gt = false;
            Flags ra; ra.gp = false; ra.gt = false;
            Flags rt; rt.gp = false; rt.ga = false;
            cd Fp = F.eval(CH_P, SP_P, m, a, b, P, rp) - F.eval(CH_P, SP_P, m, FINF, b, P, rp) + Gpp;
            cd Fa = F.eval(CH_A, SP_P, m, a, b, P, ra) - F.eval(CH_A, SP_P, m, FINF, b, P, ra) + Ga;
            cd Ft = F.eval(CH_T, SP_P, m, a, b, P, rt) - F.eval(CH_T, SP_P, m, FINF, b, P, rt) + Gt;
            s.cache[C_GPP][i] = Gpp;
            s.cache[C_GA][i] = Ga;
            s.cache[C_GT][i] = Gt * 2.0 - Ga;
            s.cache[C_FP][i] = Fp;
            s.cache[C_FA][i] = Fa;
            s.cache[C_FT][i] = Ft * 2.0 - Fa;
        }
    }
}

static inline int cross(int ch, int m, int n) { return ch == CH_P ? m - n - 1 : n; }  // BSE_templates.jl:4-6
static inline int spin_of(int ch) { return ch == CH_T ? SP_D : SP_P; }
static inline double sign_of(int ch) { return ch == CH_T ? -1.0 : 1.0; }

// --------------------------------------------------------------------------------------------
// BSE: src/BSE_templates.jl:12-180, src/BSEa/*.jl, src/nonlocal/BSEa/*.jl (fdPA / scPA forms)
// --------------------------------------------------------------------------------------------
static void bse_K1(Solver& s, int ch) {
    const int sp = spin_of(ch);
    const double sgn = sign_of(ch), T = s.d.T;
    Chan& out = s.Fbuff.g[ch];
    const SymGroup& G = (ch == CH_P) ? s.sgpp[0] : s.sgph[0];
    sg_eval(G, s.shK1, out.K1.data(), [&](const int* w) -> cd {
        const int m = w[0], P = (s.Nq == 1) ? 0 : w[1];
        cd val = 0.0;
        for (int n = -s.nPn; n < s.nPn; ++n) {
            const int wt = cross(ch, m, n);
            cd Fl = s.F.eval(ch, sp, m, FINF, n, P);
            cd F0r = any_eval(s.F0, ch, sp, m, wt, FINF, P);
            cd FLr = s.FL.eval(ch, sp, m, wt, FINF, P);
            cd pi = ((ch == CH_P) ? s.Pipp : s.Piph)[s.iPi(m, n, P)];
            cd pi0 = ((ch == CH_P) ? s.Pi0pp : s.Pi0ph)[s.iPi(m, n, P)];
            val += Fl * ((pi - pi0) * F0r + pi * FLr);
        }
        return T * val * sgn;
    });
    if (ch == CH_T) {
        for (size_t i = 0; i < out.K1.size(); ++i) out.K1[i] = (out.K1[i] + s.Fbuff.g[CH_A].K1[i]) / 2.0;
    }
}

static void bse_L_K2(Solver& s, int ch) {
    const int sp = spin_of(ch);
    const double sgn = sign_of(ch), T = s.d.T;
    Chan& out = s.FL.g[ch];
    const SymGroup& G = (ch == CH_P) ? s.sgppL[1] : s.sgphL[1];
    const std::vector<cd>& Pi0 = (ch == CH_P) ? s.Pi0pp : s.Pi0ph;
    Flags fl; fl.f0 = false; fl.ga = (ch != CH_A); fl.gp = (ch != CH_P); fl.gt = (ch != CH_T);
    sg_eval(G, s.shK2, out.K2.data(), [&](const int* w) -> cd {
        const int m = w[0], nu = w[1], P = (s.Nq == 1) ? 0 : w[2];
        cd val = 0.0;
        if (s.d.local) {
            // src/BSEa/BSEa_K2.jl:1-40: ω over the bubble mesh, crossing on F0's argument
            for (int n = -s.nPn; n < s.nPn; ++n) {
                cd Gp = s.F.eval(ch, sp, m, nu, n, P, fl);
                cd F0p = any_eval(s.F0, ch, sp, m, cross(ch, m, n), FINF, P);
                val += Gp * Pi0[s.iPi(m, n, P)] * F0p;
            }
        } else {
            // src/nonlocal/BSEa/BSEa_K2.jl:1-39: ω over the K2 mesh, crossing on Γ's argument
            for (int n = -s.d.nK2n; n < s.d.nK2n; ++n) {
                cd Gl = s.F.eval(ch, sp, m, nu, cross(ch, m, n), P, fl);
                cd F0r = any_eval(s.F0, ch, sp, m, n, FINF, P);
                val += Gl * Pi0[s.iPi(m, n, P)] * F0r;
            }
        }
        return T * val * sgn;
    });
    if (ch == CH_T) {
        for (size_t i = 0; i < out.K2.size(); ++i) out.K2[i] = (out.K2[i] + s.FL.g[CH_A].K2[i]) / 2.0;
    }
}

static void bse_K2(Solver& s, int ch) {
    const int sp = spin_of(ch);
    const double sgn = sign_of(ch), T = s.d.T;
    Chan& out = s.Fbuff.g[ch];
    const SymGroup& G = (ch == CH_P) ? s.sgpp[1] : s.sgph[1];
    const std::vector<cd>& Pi0 = (ch == CH_P) ? s.Pi0pp : s.Pi0ph;
    const std::vector<cd>& Pi = (ch == CH_P) ? s.Pipp : s.Piph;
    sg_eval(G, s.shK2, out.K2.data(), [&](const int* w) -> cd {
        const int m = w[0], nu = w[1], P = (s.Nq == 1) ? 0 : w[2];
        cd val = 0.0;
        for (int n = -s.nPn; n < s.nPn; ++n) {
            const int wt = cross(ch, m, n);
            cd Fl = s.F.eval(ch, sp, m, nu, n, P) - s.F.eval(ch, sp, m, FINF, n, P);
            cd F0r = any_eval(s.F0, ch, sp, m, wt, FINF, P);
            cd FLr = s.FL.eval(ch, sp, m, wt, FINF, P);
            const size_t ip = s.iPi(m, n, P);
            val += Fl * ((Pi[ip] - Pi0[ip]) * F0r + Pi[ip] * FLr);
        }
        return T * val * sgn;
    });
    if (ch == CH_T) {
        for (size_t i = 0; i < out.K2.size(); ++i) {
            out.K2[i] += s.FL.g[CH_T].K2[i] * 2.0;
            out.K2[i] += s.FL.g[CH_A].K2[i] * -1.0;
        }
        for (size_t i = 0; i < out.K2.size(); ++i) out.K2[i] = (out.K2[i] + s.Fbuff.g[CH_A].K2[i]) / 2.0;
    } else {
        for (size_t i = 0; i < out.K2.size(); ++i) out.K2[i] += s.FL.g[ch].K2[i];
    }
}

static void bse_L_K3(Solver& s, int ch) {
    const double sgn = (ch == CH_A) ? 1.0 : -1.0, T = s.d.T;  // BSE_templates.jl:117-146
    Chan& out = s.FL.g[ch];
    const SymGroup& G = (ch == CH_P) ? s.sgppL[2] : s.sgphL[2];
    const std::vector<cd>& cG = s.cache[ch == CH_P ? C_GPP : (ch == CH_A ? C_GA : C_GT)];
    const std::vector<cd>& cF0 = s.cache[ch == CH_P ? C_F0P : (ch == CH_A ? C_F0A : C_F0T)];
    const std::vector<cd>& Pi0 = (ch == CH_P) ? s.Pi0pp : s.Pi0ph;
    const Chan& K = s.F.g[0];
    sg_eval(G, s.shK3, out.K3.data(), [&](const int* w) -> cd {
        const int m = w[0], nu = w[1], nup = w[2], P = (s.Nq == 1) ? 0 : w[3];
        cd val = 0.0;
        for (int o = -K.n3n; o < K.n3n; ++o)
            val += cG[K.i3(m, nu, o, P)] * Pi0[s.iPi(m, o, P)] * cF0[K.i3(m, o, nup, P)];
        return T * val * sgn;
    });
    if (ch == CH_T) {
        for (size_t i = 0; i < out.K3.size(); ++i) out.K3[i] = (out.K3[i] + s.FL.g[CH_A].K3[i]) / 2.0;
    }
}

static void bse_K3(Solver& s, int ch) {
    // signs (sign1, sign2): a (+1,+1), p (-1,+1), t (-1,-1)   BSE_templates.jl:151-180
    const double s1 = (ch == CH_A) ? 1.0 : -1.0, s2 = (ch == CH_T) ? -1.0 : 1.0, T = s.d.T;
    Chan& out = s.Fbuff.g[ch];
    const SymGroup& G = (ch == CH_P) ? s.sgpp[2] : s.sgph[2];
    const std::vector<cd>& cG = s.cache[ch == CH_P ? C_GPX : (ch == CH_A ? C_GA : C_GT)];
    const std::vector<cd>& cF = s.cache[ch == CH_P ? C_FP : (ch == CH_A ? C_FA : C_FT)];
    const std::vector<cd>& cF0 = s.cache[ch == CH_P ? C_F0P : (ch == CH_A ? C_F0A : C_F0T)];
    const std::vector<cd>& Pi0 = (ch == CH_P) ? s.Pi0pp : s.Pi0ph;
    const std::vector<cd>& Pi = (ch == CH_P) ? s.Pipp : s.Piph;
    const Chan& K = s.F.g[0];
    const Chan& gL = s.FL.g[ch];
    const Chan& gLt = s.FL.g[CH_T];
    const Chan& gLa = s.FL.g[CH_A];
    sg_eval(G, s.shK3, out.K3.data(), [&](const int* w) -> cd {
        const int m = w[0], nu = w[1], nup = w[2], P = (s.Nq == 1) ? 0 : w[3];
        cd val = 0.0;
        for (int o = -K.n3n; o < K.n3n; ++o) {
            const size_t ip = s.iPi(m, o, P);
            cd pi0 = Pi0[ip], pi = Pi[ip];
            cd Fs = cF[K.i3(m, nu, o, P)];
            cd Gs = (ch == CH_P) ? cG[K.i3(m, o, nup, P)] : cG[K.i3(m, nup, o, P)];
            val += Fs * ((pi - pi0) * cF0[K.i3(m, o, nup, P)] + pi * Gs) * s1;
            const int ot = cross(ch, m, o);
            if (fin(ot, K.n3n)) {
                if (ch == CH_T)
                    val += Fs * pi * (2.0 * gLt.K3[K.i3(m, ot, nup, P)] - gLa.K3[K.i3(m, ot, nup, P)]) * s2;
                else
                    val += Fs * pi * gL.K3[K.i3(m, ot, nup, P)] * s2;
            }
        }
        const size_t io = K.i3(m, nu, nup, P);
        if (ch == CH_T) return T * val + 2.0 * gLt.K3[io] - gLa.K3[io];
        return T * val + gL.K3[io];
    });
    if (ch == CH_T) {
        for (size_t i = 0; i < out.K3.size(); ++i) out.K3[i] = (out.K3[i] + s.Fbuff.g[CH_A].K3[i]) / 2.0;
    }
}

// --------------------------------------------------------------------------------------------
// Strategy variants.  :fdPA_new / :scPA_new (local solver): the K1 and K2 classes in the form
// K = (F Π - F0 Π0) U (src/BSEa/BSEa_K1.jl:57-100, src/BSEa/BSEa_K2.jl:104-150, wrappers and the
// t-channel recombination src/BSE_templates.jl:185-250).  :fdPA_1loop (nonlocal solver): the
// one-loop BSEs with F0 on the right, K = F (Π - Π0) F0 (src/nonlocal/BSEa/BSE_1loop.jl:1-180,
// wrappers src/BSE_templates.jl:252-360).  U = bare_vertex(F, Sp) is U for pSp and dSp.
// --------------------------------------------------------------------------------------------
static void bse_K1_new(Solver& s, int ch) {
    const int sp = spin_of(ch);
    const double sgn = sign_of(ch), T = s.d.T, U = s.d.U;
    Chan& out = s.Fbuff.g[ch];
    const SymGroup& G = (ch == CH_P) ? s.sgpp[0] : s.sgph[0];
    const std::vector<cd>& Pi0 = (ch == CH_P) ? s.Pi0pp : s.Pi0ph;
    const std::vector<cd>& Pi = (ch == CH_P) ? s.Pipp : s.Piph;
    sg_eval(G, s.shK1, out.K1.data(), [&](const int* w) -> cd {
        const int m = w[0], P = (s.Nq == 1) ? 0 : w[1];
        cd val = 0.0;
        for (int n = -s.nPn; n < s.nPn; ++n) {
            const size_t ip = s.iPi(m, n, P);
            const cd Fl = s.F.eval(ch, sp, m, FINF, n, P);
            const cd F0l = any_eval(s.F0, ch, sp, m, FINF, n, P);
            val += (Fl * Pi[ip] - F0l * Pi0[ip]) * U;
        }
        return T * val * sgn;
    });
    if (ch == CH_T) {
        for (size_t i = 0; i < out.K1.size(); ++i) out.K1[i] = (out.K1[i] + s.Fbuff.g[CH_A].K1[i]) / 2.0;
    }
}

static void bse_K2_new(Solver& s, int ch) {
    const int sp = spin_of(ch);
    const double sgn = sign_of(ch), T = s.d.T, U = s.d.U;
    Chan& out = s.Fbuff.g[ch];
    const SymGroup& G = (ch == CH_P) ? s.sgpp[1] : s.sgph[1];
    const std::vector<cd>& Pi0 = (ch == CH_P) ? s.Pi0pp : s.Pi0ph;
    const std::vector<cd>& Pi = (ch == CH_P) ? s.Pipp : s.Piph;
    sg_eval(G, s.shK2, out.K2.data(), [&](const int* w) -> cd {
        const int m = w[0], nu = w[1], P = (s.Nq == 1) ? 0 : w[2];
        cd val = 0.0;
        for (int n = -s.nPn; n < s.nPn; ++n) {
            const size_t ip = s.iPi(m, n, P);
            const cd Fl = s.F.eval(ch, sp, m, nu, n, P) - s.F.eval(ch, sp, m, FINF, n, P);
            const cd F0l = any_eval(s.F0, ch, sp, m, nu, n, P) - any_eval(s.F0, ch, sp, m, FINF, n, P);
            val += (Fl * Pi[ip] - F0l * Pi0[ip]) * U;
        }
        return T * val * sgn;
    });
    if (ch == CH_T) {
        for (size_t i = 0; i < out.K2.size(); ++i) out.K2[i] = (out.K2[i] + s.Fbuff.g[CH_A].K2[i]) / 2.0;
    }
}

static void bse_K1_1loop(Solver& s, int ch) {
    const int sp = spin_of(ch);
    const double sgn = sign_of(ch), T = s.d.T;
    Chan& out = s.Fbuff.g[ch];
    const SymGroup& G = (ch == CH_P) ? s.sgpp[0] : s.sgph[0];
    const std::vector<cd>& Pi0 = (ch == CH_P) ? s.Pi0pp : s.Pi0ph;
    const std::vector<cd>& Pi = (ch == CH_P) ? s.Pipp : s.Piph;
    sg_eval(G, s.shK1, out.K1.data(), [&](const int* w) -> cd {
        const int m = w[0], P = (s.Nq == 1) ? 0 : w[1];
        cd val = 0.0;
        for (int n = -s.nPn; n < s.nPn; ++n) {
            const size_t ip = s.iPi(m, n, P);
            const cd Fl = s.F.eval(ch, sp, m, FINF, n, P);
            const cd F0r = any_eval(s.F0, ch, sp, m, cross(ch, m, n), FINF, P);
            val += Fl * (Pi[ip] - Pi0[ip]) * F0r;
        }
        return T * val * sgn;
    });
    if (ch == CH_T) {
        for (size_t i = 0; i < out.K1.size(); ++i) out.K1[i] = (out.K1[i] + s.Fbuff.g[CH_A].K1[i]) / 2.0;
    }
}

static void bse_K2_1loop(Solver& s, int ch) {
    const int sp = spin_of(ch);
    const double sgn = sign_of(ch), T = s.d.T;
    Chan& out = s.Fbuff.g[ch];
    const SymGroup& G = (ch == CH_P) ? s.sgpp[1] : s.sgph[1];
    const std::vector<cd>& Pi0 = (ch == CH_P) ? s.Pi0pp : s.Pi0ph;
    const std::vector<cd>& Pi = (ch == CH_P) ? s.Pipp : s.Piph;
    sg_eval(G, s.shK2, out.K2.data(), [&](const int* w) -> cd {
        const int m = w[0], nu = w[1], P = (s.Nq == 1) ? 0 : w[2];
        cd val = 0.0;
        for (int n = -s.nPn; n < s.nPn; ++n) {
            const size_t ip = s.iPi(m, n, P);
            const cd Fl = s.F.eval(ch, sp, m, nu, n, P) - s.F.eval(ch, sp, m, FINF, n, P);
            const cd F0r = any_eval(s.F0, ch, sp, m, cross(ch, m, n), FINF, P);
            val += Fl * (Pi[ip] - Pi0[ip]) * F0r;
        }
        return T * val * sgn;
    });
    if (ch == CH_T) {
        for (size_t i = 0; i < out.K2.size(); ++i) {
            out.K2[i] += s.FL.g[CH_T].K2[i] * 2.0;
            out.K2[i] += s.FL.g[CH_A].K2[i] * -1.0;
        }
        for (size_t i = 0; i < out.K2.size(); ++i) out.K2[i] = (out.K2[i] + s.Fbuff.g[CH_A].K2[i]) / 2.0;
    } else {
        for (size_t i = 0; i < out.K2.size(); ++i) out.K2[i] += s.FL.g[ch].K2[i];
    }
}

static void bse_K3_1loop(Solver& s, int ch) {
    const double s1 = (ch == CH_A) ? 1.0 : -1.0, T = s.d.T;
    Chan& out = s.Fbuff.g[ch];
    const SymGroup& G = (ch == CH_P) ? s.sgpp[2] : s.sgph[2];
    const std::vector<cd>& cF = s.cache[ch == CH_P ? C_FP : (ch == CH_A ? C_FA : C_FT)];
    const std::vector<cd>& cF0 = s.cache[ch == CH_P ? C_F0P : (ch == CH_A ? C_F0A : C_F0T)];
    const std::vector<cd>& Pi0 = (ch == CH_P) ? s.Pi0pp : s.Pi0ph;
    const std::vector<cd>& Pi = (ch == CH_P) ? s.Pipp : s.Piph;
    const Chan& K = s.F.g[0];
    sg_eval(G, s.shK3, out.K3.data(), [&](const int* w) -> cd {
        const int m = w[0], nu = w[1], nup = w[2], P = (s.Nq == 1) ? 0 : w[3];
        cd val = 0.0;
        for (int o = -K.n3n; o < K.n3n; ++o) {
            const size_t ip = s.iPi(m, o, P);
            val += cF[K.i3(m, nu, o, P)] * (Pi[ip] - Pi0[ip]) * cF0[K.i3(m, o, nup, P)] * s1;
        }
        return T * val;
    });
    if (ch == CH_T) {
        for (size_t i = 0; i < out.K3.size(); ++i) out.K3[i] = (out.K3[i] + s.Fbuff.g[CH_A].K3[i]) / 2.0;
    }
}

// --------------------------------------------------------------------------------------------
// SDE: src/SDE.jl:3-364, src/nonlocal/SDE.jl:3-447
// --------------------------------------------------------------------------------------------
// L_pp, L_ph for a vertex (γ contributions only) or for a RefVertex (F - U).
static void sde_L(Solver& s, std::vector<cd>& Lpp, std::vector<cd>& Lph, const std::vector<cd>& Pipp,
                  const std::vector<cd>& Piph, const AnyV& F, const SymGroup& Gpp, const SymGroup& Gph) {
    const double T = s.d.T;
    const cd U = F.ref ? F.ref->U : F.vert->bare();
    sg_eval(Gpp, s.shK2, Lpp.data(), [&](const int* w) -> cd {
        const int m = w[0], nu = w[1], P = (s.Nq == 1) ? 0 : w[2];
        cd val = 0.0;
        for (int n = -s.nPn; n < s.nPn; ++n) {
            const cd pi = Pipp[s.iPi(m, n, P)];
            if (F.ref) {
                val += U * pi * (F.ref->eval(CH_P, SP_P, m, m - n - 1, nu) - F.ref->bare(SP_P));
            } else {
                const int Pv = (F.vert->Nq == 1) ? 0 : P;
                val += U * pi * F.vert->g[CH_P].eval(m, m - n - 1, nu, Pv);
            }
        }
        return T * val;
    });
    sg_eval(Gph, s.shK2, Lph.data(), [&](const int* w) -> cd {
        const int m = w[0], nu = w[1], P = (s.Nq == 1) ? 0 : w[2];
        cd val = 0.0;
        for (int n = -s.nPn; n < s.nPn; ++n) {
            const cd pi = Piph[s.iPi(m, n, P)];
            if (F.ref) {
                val += U * pi * (F.ref->eval(CH_A, SP_P, m, nu, n) + F.ref->eval(CH_T, SP_P, m, nu, n) -
                                 F.ref->bare(SP_P) - F.ref->bare(SP_P));
            } else {
                const int Pv = (F.vert->Nq == 1) ? 0 : P;
                if (s.d.local)
                    val += U * pi * (F.vert->g[CH_A].eval(m, nu, n, Pv) + F.vert->g[CH_T].eval(m, nu, n, Pv));
                else
                    val += U * pi * (F.vert->g[CH_T].eval(m, nu, n, Pv) + F.vert->g[CH_A].eval(m, nu, n, Pv));
            }
        }
        return T * val;
    });
}

// Σ from L: local src/SDE.jl:241-263; nonlocal real space src/nonlocal/SDE.jl:192-280
static void sde_inner(Solver& s, std::vector<cd>& Sig, const std::vector<cd>& G, const std::vector<cd>& Lpp,
                      const std::vector<cd>& Lph) {
    const double T = s.d.T;
    const int nG = s.d.nG, n2O = s.d.nK2O, n2n = s.d.nK2n, N2O = 2 * n2O - 1;
    auto iL = [&](int m, int n, int P) { return (size_t)(m + n2O - 1) + (size_t)N2O * ((size_t)(n + n2n) + (size_t)(2 * n2n) * P); };
    if (s.d.local) {
        sg_eval(s.sgSig, s.shSig, Sig.data(), [&](const int* w) -> cd {
            const int nu = w[0];
            cd val = 0.0;
            if (fin(nu, n2n)) {
                for (int m = -(n2O - 1); m <= n2O - 1; ++m) {
                    cd g1 = fin(m - nu - 1, nG) ? G[s.iG(m - nu - 1, 0)] : cd(0.0);
                    cd g2 = fin(m + nu, nG) ? G[s.iG(m + nu, 0)] : cd(0.0);
                    val += g1 * Lpp[iL(m, nu, 0)];
                    val += g2 * Lph[iL(m, nu, 0)];
                }
            }
            return T * val;
        });
        return;
    }
    const int L = s.d.L, LG = s.d.LG, LS = s.d.LG;  // Σ lives on the G momentum mesh
    std::vector<cd> GR(G.begin(), G.end());
    dft2(GR, s.NG, 0, LG, -1);
    for (auto& v : GR) v /= (double)(LG * LG);
    std::vector<cd> LppR(Lpp.begin(), Lpp.end()), LphR(Lph.begin(), Lph.end());
    const size_t inner = (size_t)N2O * 2 * n2n;
    dft2(LppR, inner, 0, L, -1);
    dft2(LphR, inner, 0, L, -1);
    for (auto& v : LppR) v /= (double)(L * L);
    for (auto& v : LphR) v /= (double)(L * L);
    std::vector<cd> SR((size_t)s.NG * LS * LS, 0.0);
    const int h = L / 2;
    for (int R1 = -h; R1 <= h; ++R1)
        for (int R2 = -h; R2 <= h; ++R2) {
            double weight = 1.0;
            if (L % 2 == 0) {
                if (std::abs(R1) == L / 2) weight /= 2;
                if (std::abs(R2) == L / 2) weight /= 2;
            }
            const int iRL = imod(R1, L) + L * imod(R2, L);
            const int imRG = imod(-R1, LG) + LG * imod(-R2, LG);
            const int ipRS = imod(R1, LS) + LS * imod(R2, LS);
            const int imRS = imod(-R1, LS) + LS * imod(-R2, LS);
            for (int nu = -n2n; nu < n2n; ++nu) {
                if (!fin(nu, nG)) continue;
                for (int m = -(n2O - 1); m <= n2O - 1; ++m) {
                    if (fin(m - nu - 1, nG))
                        SR[s.iG(nu, ipRS)] += GR[s.iG(m - nu - 1, imRG)] * LppR[iL(m, nu, iRL)] * weight;
                    if (fin(m + nu, nG))
                        SR[s.iG(nu, imRS)] += GR[s.iG(m + nu, imRG)] * LphR[iL(m, nu, iRL)] * weight;
                }
            }
        }
    for (auto& v : SR) v *= T;
    dft2(SR, s.NG, 0, LS, +1);
    Sig = SR;
    sg_symmetrize(s.sgSig, Sig.data());
}

// second-order term: local src/SDE.jl:328-364; nonlocal src/nonlocal/SDE.jl:400-447
static void sde_U2(Solver& s, std::vector<cd>& out, const std::vector<cd>& G, cd U) {
    const double T = s.d.T;
    const int nG = s.d.nG;
    if (s.d.local) {
        sg_eval(s.sgSig, s.shSig, out.data(), [&](const int* w) -> cd {
            const int nu = w[0];
            cd val = 0.0;
            for (int n2 = -nG; n2 < nG; ++n2)
                for (int n1 = -nG; n1 < nG; ++n1) {
                    const int n3 = n1 - n2 + nu;
                    if (fin(n3, nG)) val += G[s.iG(n1, 0)] * G[s.iG(n2, 0)] * G[s.iG(n3, 0)];
                }
            return val * U * U * T * T;
        });
        return;
    }
    const int L = s.d.LG;
    std::vector<cd> Gp(G.begin(), G.end()), Gm(G.begin(), G.end());
    dft2(Gp, s.NG, 0, L, -1);
    dft2(Gm, s.NG, 0, L, +1);
    for (auto& v : Gp) v /= (double)(L * L);
    for (auto& v : Gm) v /= (double)(L * L);
    std::vector<cd> SR((size_t)s.NG * L * L, 0.0);
#pragma omp parallel for
    for (int R = 0; R < L * L; ++R) {
        for (int n2 = -nG; n2 < nG; ++n2)
            for (int n1 = -nG; n1 < nG; ++n1) {
                cd gg = Gm[s.iG(n1, R)] * Gp[s.iG(n2, R)];
                for (int nu = -nG; nu < nG; ++nu) {
                    const int n3 = n1 - n2 + nu;
                    if (fin(n3, nG)) SR[s.iG(nu, R)] += gg * Gp[s.iG(n3, R)];
                }
            }
    }
    for (auto& v : SR) v *= U * U * T * T;
    dft2(SR, s.NG, 0, L, +1);
    out = SR;
    sg_symmetrize(s.sgSig, out.data());
}

// SDE_compute!: src/SDE.jl:219-283, src/nonlocal/SDE.jl:146-190
static void sde_compute(Solver& s, std::vector<cd>& Sig, const std::vector<cd>& G, const std::vector<cd>& Pipp,
                        const std::vector<cd>& Piph, std::vector<cd>& Lpp, std::vector<cd>& Lph, const AnyV& F,
                        const SymGroup& Gpp, const SymGroup& Gph, bool incU2, bool incH) {
    sde_L(s, Lpp, Lph, Pipp, Piph, F, Gpp, Gph);
    sde_inner(s, Sig, G, Lpp, Lph);
    if (F.ref) for (auto& v : Sig) v *= 1.0 / 3.0;
    const cd U = F.ref ? F.ref->U : F.vert->bare();
    if (incU2) {
        std::vector<cd> u2(Sig.size(), 0.0);
        sde_U2(s, u2, G, U);
        for (size_t i = 0; i < Sig.size(); ++i) Sig[i] += u2[i];
    }
    if (incH) {
        const double n = occupation(s, G);
        const cd h = (n - 0.5) * U * cd(0.0, 1.0);
        for (auto& v : Sig) v += h;
    }
}

// SDE!(Σ, G, ..., F, ...) with the recursion over F.F0: src/SDE.jl:35-48
static void sde_rec(Solver& s, std::vector<cd>& Sig, const std::vector<cd>& G, const std::vector<cd>& Pipp,
                    const std::vector<cd>& Piph, std::vector<cd>& Lpp, std::vector<cd>& Lph, const AnyV& F,
                    const SymGroup& Gpp, const SymGroup& Gph, bool incU2, bool incH) {
    std::vector<cd> tmp(Sig.size(), 0.0);
    sde_compute(s, tmp, G, Pipp, Piph, Lpp, Lph, F, Gpp, Gph, incU2, incH);
    for (size_t i = 0; i < Sig.size(); ++i) Sig[i] += tmp[i];
    if (F.vert) sde_rec(s, Sig, G, Pipp, Piph, Lpp, Lph, F.vert->F0, Gpp, Gph, false, false);
}

// SDE!(S; strategy): src/SDE.jl:3-33
static void sde_solver(Solver& s, bool fdpa, bool incH) {
    AnyV Fa; Fa.vert = &s.F;
    std::fill(s.Sig.begin(), s.Sig.end(), 0.0);
    sde_rec(s, s.Sig, s.G, s.Pipp, s.Piph, s.Lpp, s.Lph, Fa, s.sgpp[1], s.sgph[1], true, incH);
    if (!fdpa) return;
    std::vector<cd> s0(s.Sig.size(), 0.0);
    sde_rec(s, s0, s.G0, s.Pi0pp, s.Pi0ph, s.L0pp, s.L0ph, s.F0, s.sg0pp2, s.sg0ph2, true, incH);
    for (size_t i = 0; i < s.Sig.size(); ++i) s.Sig[i] += s0[i] * -1.0;
    for (size_t i = 0; i < s.Sig.size(); ++i) s.Sig[i] += s.Sig0[i];
    if (incH && !s.variant_single_hartree) {
        const double n0 = occupation(s, s.G0);
        const cd h = (n0 - 0.5) * s.F.bare() * cd(0.0, 1.0);
        for (auto& v : s.Sig) v -= h;
    }
}

// --------------------------------------------------------------------------------------------
// One parquet iteration: src/solve.jl:4-116
// --------------------------------------------------------------------------------------------
enum { STRAT_FDPA = 0, STRAT_SCPA = 1, STRAT_FDPA_NEW = 2, STRAT_SCPA_NEW = 3, STRAT_FDPA_1LOOP = 4 };

static void iterate(Solver& s, int strategy, bool update_sigma, bool incH) {
    s.F.update_avg();
    if (update_sigma) {
        dyson(s.G, s.Sig, s.Gbare);
        bubbles(s, s.Pipp, s.Piph, s.G);
    }
    build_K3_cache(s);
    // src/solve.jl:26-82
    if (strategy == STRAT_FDPA_NEW || strategy == STRAT_SCPA_NEW) {
        if (strategy == STRAT_FDPA_NEW) { bse_L_K3(s, CH_P); bse_L_K3(s, CH_A); bse_L_K3(s, CH_T); }
        bse_K3(s, CH_P); bse_K3(s, CH_A); bse_K3(s, CH_T);
        bse_K1_new(s, CH_P); bse_K1_new(s, CH_A); bse_K1_new(s, CH_T);
        bse_K2_new(s, CH_P); bse_K2_new(s, CH_A); bse_K2_new(s, CH_T);
    } else if (strategy == STRAT_FDPA_1LOOP) {
        bse_K3_1loop(s, CH_P); bse_K3_1loop(s, CH_A); bse_K3_1loop(s, CH_T);
        bse_K1_1loop(s, CH_P); bse_K1_1loop(s, CH_A); bse_K1_1loop(s, CH_T);
        bse_K2_1loop(s, CH_P); bse_K2_1loop(s, CH_A); bse_K2_1loop(s, CH_T);
    } else {
        if (strategy == STRAT_FDPA) {
            bse_L_K2(s, CH_P); bse_L_K2(s, CH_A); bse_L_K2(s, CH_T);
            bse_L_K3(s, CH_P); bse_L_K3(s, CH_A); bse_L_K3(s, CH_T);
        }
        bse_K1(s, CH_P); bse_K1(s, CH_A); bse_K1(s, CH_T);
        bse_K2(s, CH_P); bse_K2(s, CH_A); bse_K2(s, CH_T);
        bse_K3(s, CH_P); bse_K3(s, CH_A); bse_K3(s, CH_T);
    }
    for (int c = 0; c < 3; ++c) {
        s.F.g[c].K1 = s.Fbuff.g[c].K1;
        s.F.g[c].K2 = s.Fbuff.g[c].K2;
        s.F.g[c].K3 = s.Fbuff.g[c].K3;
    }
    if (update_sigma) {
        s.F.update_avg();
        // src/SDE.jl:3-33: the _new and _1loop variants take the SDE of their base strategy
        sde_solver(s, strategy == STRAT_FDPA || strategy == STRAT_FDPA_NEW || strategy == STRAT_FDPA_1LOOP, incH);
    }
}

// --------------------------------------------------------------------------------------------
// mfRG linear map of the Krylov-preconditioned solver (nonlocal solver): src/mfRG.jl:20-89.  The
// map calls the two-argument cache builder, whose method for the nonlocal solvers lives in
// src/nonlocal_2/build_K3_cache.jl:97-165: the Γ caches are F(γr = false) - F.F0(γr = false)
// (for a Vertex-valued F0 this keeps F0's own γr) and the right F caches come from F0 alone, each
// evaluated on the class representatives of the K3 symmetry group.  The BSEs are the is_mfRG
// branches of src/nonlocal/BSEa/BSEa_K1.jl:29-37, BSEa_K2.jl:70-77 and BSEa_K3.jl:83-97.
// --------------------------------------------------------------------------------------------
static cd f0_eval_flags(const AnyV& F0, int ch, int sp, int m, int n, int np, int P, Flags fl) {
    if (F0.ref) return F0.ref->eval(ch, sp, m, n, np);  // RefVertex ignores the channel flags
    return F0.vert->eval(ch, sp, m, n, np, P, fl);
}

static void build_K3_cache_mfrg(Solver& s) {
    build_K3_cache(s);  // the left F0 caches (F0 alone, unchanged by the map)
    const Shape& sh = s.shK3;
    const Vert& F = s.F;
    const AnyV& F0 = s.F0;
    auto Pof = [&](const int* w) { return (s.Nq == 1) ? 0 : w[3]; };
    Flags np_; np_.gp = false;
    Flags na_; na_.ga = false;
    Flags nt_; nt_.gt = false;
    sg_eval(s.sgpp[2], sh, s.cache[C_GPX].data(), [&](const int* w) -> cd {
        const int P = Pof(w);
        return F.eval(CH_P, SP_X, w[0], w[1], w[2], P, np_) - f0_eval_flags(F0, CH_P, SP_X, w[0], w[1], w[2], P, np_);
    });
    sg_eval(s.sgpp[2], sh, s.cache[C_GPP].data(), [&](const int* w) -> cd {
        const int P = Pof(w);
        return F.eval(CH_P, SP_P, w[0], w[1], w[2], P, np_) - f0_eval_flags(F0, CH_P, SP_P, w[0], w[1], w[2], P, np_);
    });
    sg_eval(s.sgph[2], sh, s.cache[C_GA].data(), [&](const int* w) -> cd {
        const int P = Pof(w);
        return F.eval(CH_A, SP_P, w[0], w[1], w[2], P, na_) - f0_eval_flags(F0, CH_A, SP_P, w[0], w[1], w[2], P, na_);
    });
    sg_eval(s.sgph[2], sh, s.cache[C_GT].data(), [&](const int* w) -> cd {
        const int P = Pof(w);
        return F.eval(CH_T, SP_P, w[0], w[1], w[2], P, nt_) - f0_eval_flags(F0, CH_T, SP_P, w[0], w[1], w[2], P, nt_);
    });
    sg_eval(s.sgpp[2], sh, s.cache[C_FP].data(), [&](const int* w) -> cd {
        const int P = Pof(w);
        return any_eval(F0, CH_P, SP_P, w[0], w[1], w[2], P) - any_eval(F0, CH_P, SP_P, w[0], FINF, w[2], P);
    });
    sg_eval(s.sgph[2], sh, s.cache[C_FA].data(), [&](const int* w) -> cd {
        const int P = Pof(w);
        return any_eval(F0, CH_A, SP_P, w[0], w[1], w[2], P) - any_eval(F0, CH_A, SP_P, w[0], FINF, w[2], P);
    });
    sg_eval(s.sgph[2], sh, s.cache[C_FT].data(), [&](const int* w) -> cd {
        const int P = Pof(w);
        return any_eval(F0, CH_T, SP_P, w[0], w[1], w[2], P) - any_eval(F0, CH_T, SP_P, w[0], FINF, w[2], P);
    });
    const size_t n = sh.size();
    for (size_t i = 0; i < n; ++i) {
        s.cache[C_GT][i] = s.cache[C_GT][i] * 2.0 - s.cache[C_GA][i];
        s.cache[C_FT][i] = s.cache[C_FT][i] * 2.0 - s.cache[C_FA][i];
    }
}

// K1 = T s Σ_ω F0(Ω,∞,ω) Π0(Ω,ω) FL(Ω,ω̃,∞)
static void bse_K1_mfrg(Solver& s, int ch) {
    const int sp = spin_of(ch);
    const double sgn = sign_of(ch), T = s.d.T;
    Chan& out = s.Fbuff.g[ch];
    const SymGroup& G = (ch == CH_P) ? s.sgpp[0] : s.sgph[0];
    const std::vector<cd>& Pi0 = (ch == CH_P) ? s.Pi0pp : s.Pi0ph;
    sg_eval(G, s.shK1, out.K1.data(), [&](const int* w) -> cd {
        const int m = w[0], P = (s.Nq == 1) ? 0 : w[1];
        cd val = 0.0;
        for (int n = -s.nPn; n < s.nPn; ++n) {
            const int wt = cross(ch, m, n);
            cd F0l = any_eval(s.F0, ch, sp, m, FINF, n, P);
            cd FLr = s.FL.eval(ch, sp, m, wt, FINF, P);
            val += F0l * Pi0[s.iPi(m, n, P)] * FLr;
        }
        return T * val * sgn;
    });
    if (ch == CH_T) {
        for (size_t i = 0; i < out.K1.size(); ++i) out.K1[i] = (out.K1[i] + s.Fbuff.g[CH_A].K1[i]) / 2.0;
    }
}

// K2 = T s Σ_ω [F0(Ω,ν,ω̃) - F0(Ω,∞,ω̃)] Π0(Ω,ω) FL(Ω,ω,∞) + the FL.K2 epilogue
static void bse_K2_mfrg(Solver& s, int ch) {
    const int sp = spin_of(ch);
    const double sgn = sign_of(ch), T = s.d.T;
    Chan& out = s.Fbuff.g[ch];
    const SymGroup& G = (ch == CH_P) ? s.sgpp[1] : s.sgph[1];
    const std::vector<cd>& Pi0 = (ch == CH_P) ? s.Pi0pp : s.Pi0ph;
    sg_eval(G, s.shK2, out.K2.data(), [&](const int* w) -> cd {
        const int m = w[0], nu = w[1], P = (s.Nq == 1) ? 0 : w[2];
        cd val = 0.0;
        for (int n = -s.nPn; n < s.nPn; ++n) {
            const int wt = cross(ch, m, n);
            cd F0l = any_eval(s.F0, ch, sp, m, nu, wt, P) - any_eval(s.F0, ch, sp, m, FINF, wt, P);
            cd FLr = s.FL.eval(ch, sp, m, n, FINF, P);
            val += F0l * Pi0[s.iPi(m, n, P)] * FLr;
        }
        return T * val * sgn;
    });
    if (ch == CH_T) {
        for (size_t i = 0; i < out.K2.size(); ++i) {
            out.K2[i] += s.FL.g[CH_T].K2[i] * 2.0;
            out.K2[i] += s.FL.g[CH_A].K2[i] * -1.0;
        }
        for (size_t i = 0; i < out.K2.size(); ++i) out.K2[i] = (out.K2[i] + s.Fbuff.g[CH_A].K2[i]) / 2.0;
    } else {
        for (size_t i = 0; i < out.K2.size(); ++i) out.K2[i] += s.FL.g[ch].K2[i];
    }
}

// K3 = T Σ_ω cacheF(ν,ω) Π0(ω) [s1 Γ(ω,ν') + s2 γL(ω̃,ν') (ω̃ in the box)] + γL(ν,ν')
static void bse_K3_mfrg(Solver& s, int ch) {
    const double s1 = (ch == CH_A) ? 1.0 : -1.0, s2 = (ch == CH_T) ? -1.0 : 1.0, T = s.d.T;
    Chan& out = s.Fbuff.g[ch];
    const SymGroup& G = (ch == CH_P) ? s.sgpp[2] : s.sgph[2];
    const std::vector<cd>& cG = s.cache[ch == CH_P ? C_GPX : (ch == CH_A ? C_GA : C_GT)];
    const std::vector<cd>& cF = s.cache[ch == CH_P ? C_FP : (ch == CH_A ? C_FA : C_FT)];
    const std::vector<cd>& Pi0 = (ch == CH_P) ? s.Pi0pp : s.Pi0ph;
    const Chan& K = s.F.g[0];
    const Chan& gL = s.FL.g[ch];
    const Chan& gLt = s.FL.g[CH_T];
    const Chan& gLa = s.FL.g[CH_A];
    sg_eval(G, s.shK3, out.K3.data(), [&](const int* w) -> cd {
        const int m = w[0], nu = w[1], nup = w[2], P = (s.Nq == 1) ? 0 : w[3];
        cd val = 0.0;
        for (int o = -K.n3n; o < K.n3n; ++o) {
            cd pi0 = Pi0[s.iPi(m, o, P)];
            cd Fs = cF[K.i3(m, nu, o, P)];
            cd Gs = (ch == CH_P) ? cG[K.i3(m, o, nup, P)] : cG[K.i3(m, nup, o, P)];
            val += Fs * pi0 * Gs * s1;
            const int ot = cross(ch, m, o);
            if (fin(ot, K.n3n)) {
                if (ch == CH_T)
                    val += Fs * pi0 * (2.0 * gLt.K3[K.i3(m, ot, nup, P)] - gLa.K3[K.i3(m, ot, nup, P)]) * s2;
                else
                    val += Fs * pi0 * gL.K3[K.i3(m, ot, nup, P)] * s2;
            }
        }
        if (ch == CH_T) return T * val + 2.0 * gLt.K3[K.i3(m, nu, nup, P)] - gLa.K3[K.i3(m, nu, nup, P)];
        return T * val + gL.K3[K.i3(m, nu, nup, P)];
    });
    if (ch == CH_T) {
        for (size_t i = 0; i < out.K3.size(); ++i) out.K3[i] = (out.K3[i] + s.Fbuff.g[CH_A].K3[i]) / 2.0;
    }
}

// y = x - Φ_mfRG(x f)/f with f = 1e-2 (vertex part of the state only; the map is linear in x)
static void mfrg_apply(Solver& s, const cd* x, cd* y) {
    const double factor = 1e-2;
    size_t o = 0;
    for (int c : {CH_P, CH_T, CH_A}) {
        Chan& g = s.F.g[c];
        for (auto& v : g.K1) v = x[o++] * factor;
        for (auto& v : g.K2) v = x[o++] * factor;
        for (auto& v : g.K3) v = x[o++] * factor;
    }
    s.F.update_avg();
    build_K3_cache_mfrg(s);
    bse_L_K2(s, CH_P); bse_L_K2(s, CH_A); bse_L_K2(s, CH_T);
    bse_K1_mfrg(s, CH_P); bse_K1_mfrg(s, CH_A); bse_K1_mfrg(s, CH_T);
    bse_K2_mfrg(s, CH_P); bse_K2_mfrg(s, CH_A); bse_K2_mfrg(s, CH_T);
    bse_L_K3(s, CH_P); bse_L_K3(s, CH_A); bse_L_K3(s, CH_T);
    bse_K3_mfrg(s, CH_P); bse_K3_mfrg(s, CH_A); bse_K3_mfrg(s, CH_T);
    o = 0;
    for (int c : {CH_P, CH_T, CH_A}) {
        const Chan& g = s.Fbuff.g[c];
        for (const auto& v : g.K1) { y[o] = x[o] - v / factor; ++o; }
        for (const auto& v : g.K2) { y[o] = x[o] - v / factor; ++o; }
        for (const auto& v : g.K3) { y[o] = x[o] - v / factor; ++o; }
    }
    for (int c = 0; c < 3; ++c) {  // set!(S.F, S.Fbuff)
        s.F.g[c].K1 = s.Fbuff.g[c].K1;
        s.F.g[c].K2 = s.Fbuff.g[c].K2;
        s.F.g[c].K3 = s.Fbuff.g[c].K3;
    }
}

static size_t state_len(const Solver& s) { return s.F.length() + s.Sig.size(); }

static void flatten(const Solver& s, cd* x) {
    size_t o = 0;
    for (int c : {CH_P, CH_T, CH_A}) {
        const Chan& g = s.F.g[c];
        std::copy(g.K1.begin(), g.K1.end(), x + o); o += g.K1.size();
        std::copy(g.K2.begin(), g.K2.end(), x + o); o += g.K2.size();
        std::copy(g.K3.begin(), g.K3.end(), x + o); o += g.K3.size();
    }
    std::copy(s.Sig.begin(), s.Sig.end(), x + o);
}

static void unflatten(Solver& s, const cd* x) {
    size_t o = 0;
    for (int c : {CH_P, CH_T, CH_A}) {
        Chan& g = s.F.g[c];
        std::copy(x + o, x + o + g.K1.size(), g.K1.begin()); o += g.K1.size();
        std::copy(x + o, x + o + g.K2.size(), g.K2.begin()); o += g.K2.size();
        std::copy(x + o, x + o + g.K3.size(), g.K3.begin()); o += g.K3.size();
    }
    std::copy(x + o, x + o + s.Sig.size(), s.Sig.begin());
}

// --------------------------------------------------------------------------------------------
// Construction: src/ParquetSolver.jl:277-352, src/nonlocal/ParquetSolver.jl:77-152
// (inputs Gbare, G0, Σ0 and the reference vertex are uploaded before finalize()).
// --------------------------------------------------------------------------------------------
static Solver* create(const Dims& d) {
    auto s = new Solver();
    s->d = d;
    s->Nq = d.local ? 1 : d.L * d.L;
    s->Nk = d.local ? 1 : d.LG * d.LG;
    s->NG = 2 * d.nG;
    s->nPO = d.nK1; s->nPn = d.nK1 * d.fPi;
    s->NPO = 2 * s->nPO - 1; s->NPn = 2 * s->nPn;
    const size_t nGk = (size_t)s->NG * s->Nk;
    s->Gbare.assign(nGk, 0.0); s->G0.assign(nGk, 0.0); s->Sig0.assign(nGk, 0.0);
    s->G.assign(nGk, 0.0); s->Sig.assign(nGk, 0.0);
    const size_t nPi = (size_t)s->NPO * s->NPn * s->Nq;
    s->Pi0pp.assign(nPi, 0.0); s->Pi0ph.assign(nPi, 0.0); s->Pipp.assign(nPi, 0.0); s->Piph.assign(nPi, 0.0);
    s->ref.init(d.U, d.nRO, d.nRn);
    s->zero_ref.init(0.0, 1, 1);
    if (d.f0_is_vertex) {
        s->F0v.init(d.nF0K1, d.nF0K2O, d.nF0K2n, d.nF0K3O, d.nF0K3n, s->Nq);
        s->F0v.F0.ref = &s->ref;
        s->F0.vert = &s->F0v;
    } else {
        s->F0.ref = &s->ref;
    }
    s->F.init(d.nK1, d.nK2O, d.nK2n, d.nK3O, d.nK3n, s->Nq);
    s->F.F0 = s->F0;
    s->Fbuff.init(d.nK1, d.nK2O, d.nK2n, d.nK3O, d.nK3n, s->Nq);
    s->Fbuff.F0.ref = &s->zero_ref;
    s->FL.init(d.nK1, d.nK2O, d.nK2n, d.nK3O, d.nK3n, s->Nq);
    s->FL.F0.ref = &s->zero_ref;
    const size_t n2 = s->F.g[0].len2();
    s->Lpp.assign(n2, 0.0); s->Lph.assign(n2, 0.0); s->L0pp.assign(n2, 0.0); s->L0ph.assign(n2, 0.0);
    for (auto& c : s->cache) c.assign(s->F.g[0].len3(), 0.0);
    const int L = d.local ? 1 : d.L;
    s->shK1.add(AX_B, d.nK1); if (!d.local) s->shK1.add(AX_K, L);
    s->shK2.add(AX_B, d.nK2O); s->shK2.add(AX_F, d.nK2n); if (!d.local) s->shK2.add(AX_K, L);
    s->shK3.add(AX_B, d.nK3O); s->shK3.add(AX_F, d.nK3n); s->shK3.add(AX_F, d.nK3n); if (!d.local) s->shK3.add(AX_K, L);
    s->shSig.add(AX_F, d.nG); if (!d.local) s->shSig.add(AX_K, d.LG);
    return s;
}

// constructor tail: Π0 from G0, G = Dyson(Σ = Σ0), Π from G
static void finalize(Solver& s) {
    if (s.F0.vert) s.F0v.update_avg();
    bubbles(s, s.Pi0pp, s.Pi0ph, s.G0);
    s.Sig = s.Sig0;
    dyson(s.G, s.Sig, s.Gbare);
    bubbles(s, s.Pipp, s.Piph, s.G);
}

// init_sym_grp!: src/ParquetSolver.jl:203-231, src/nonlocal/ParquetSolver.jl:198-300
static void init_sym_grp(Solver& s) {
    const bool nl = !s.d.local;
    const int L = nl ? s.d.L : 1, LG = nl ? s.d.LG : 1;
    std::vector<SymFn> sig = {s_sigma}, k1 = {s_k1_conj};
    std::vector<SymFn> k2pp = {s_k2pp1, s_k2pp2}, k2ph = {s_k2pp1, s_k2ph2};
    std::vector<SymFn> k3pp = {s_k3pp1, s_k3pp2, s_k3pp3}, k3ppL = {s_k3pp1, s_k3pp3};
    std::vector<SymFn> k3ph = {s_k3pp1, s_k3pp2, s_k3ph3}, k3phL = {s_k3pp1, s_k3ph3};
    if (nl) {
        sig.push_back(s_sigma_ref); sig.push_back(s_sigma_rot);
        k1.push_back(s_k1_ref); k1.push_back(s_k1_rot);
        for (auto* v : {&k2pp, &k2ph}) { v->push_back(s_k2_ref); v->push_back(s_k2_rot); }
        for (auto* v : {&k3pp, &k3ppL, &k3ph, &k3phL}) { v->push_back(s_k3_ref); v->push_back(s_k3_rot); }
    }
    s.sgSig = build_group(s.shSig, sig, LG);
    s.sgpp[0] = build_group(s.shK1, k1, L);
    s.sgpp[1] = build_group(s.shK2, k2pp, L);
    s.sgpp[2] = build_group(s.shK3, k3pp, L);
    s.sgppL[0] = s.sgpp[0]; s.sgppL[1] = s.sgpp[1];
    s.sgppL[2] = build_group(s.shK3, k3ppL, L);
    s.sgph[0] = s.sgpp[0];
    s.sgph[1] = build_group(s.shK2, k2ph, L);
    s.sgph[2] = build_group(s.shK3, k3ph, L);
    s.sgphL[0] = s.sgph[0]; s.sgphL[1] = s.sgph[1];
    s.sgphL[2] = build_group(s.shK3, k3phL, L);
    s.sg0pp2 = s.sgpp[1];
    s.sg0ph2 = s.sgph[1];
}

// --------------------------------------------------------------------------------------------
// Anderson acceleration (NLsolve 4.5.1 method=:anderson, restated; Walker & Ni 2011)
// --------------------------------------------------------------------------------------------
struct AndersonOut { int iterations; int converged; double last_res; };

static void givens(cd f, cd g, double& c, cd& sn) {
    const double af = std::abs(f), ag = std::abs(g);
    if (ag == 0.0) { c = 1.0; sn = 0.0; return; }
    if (af == 0.0) { c = 0.0; sn = std::conj(g) / ag; return; }
    const double r = std::hypot(af, ag);
    c = af / r;
    sn = (f / af) * std::conj(g) / r;
}

static AndersonOut anderson(Solver& s, int strategy, bool update_sigma, bool incH, int maxiter, double ftol, double beta,
                            int mem, double* trace) {
    const size_t n = state_len(s);
    std::vector<cd> x(n), fx(n), g(n), fxold, gold;
    flatten(s, x.data());
    const int mmax = (int)std::min<size_t>(n, (size_t)mem);
    std::vector<std::vector<cd>> dG(mmax, std::vector<cd>(n)), Q(mmax, std::vector<cd>(n));
    std::vector<cd> R((size_t)mmax * mmax, 0.0), gam(mmax);
    fxold.assign(n, 0.0); gold.assign(n, 0.0);
    auto Rr = [&](int i, int j) -> cd& { return R[(size_t)i + (size_t)mmax * j]; };
    int m_eff = 0;
    AndersonOut out{0, 0, 0.0};
    for (int it = 1; it <= maxiter; ++it) {
        // fixed_point!: R = Φ(x) - x   (src/solve.jl:119-157)
        unflatten(s, x.data());
        iterate(s, strategy, update_sigma, incH);
        flatten(s, fx.data());
        double res = 0.0;
        for (size_t i = 0; i < n; ++i) { fx[i] -= x[i]; res = std::max(res, std::abs(fx[i])); }
        for (size_t i = 0; i < n; ++i) g[i] = x[i] + beta * fx[i];
        if (trace) trace[it - 1] = res;
        out.iterations = it; out.last_res = res;
        if (res < ftol) { out.converged = 1; break; }
        x = g;
        if (mmax == 0) continue;
        if (it == 1) {
            fxold = fx; gold = g;
            continue;
        }
        m_eff += 1;
        if (m_eff > mmax) {
            // circular shift of Δg and deletion of the first QR column by Givens rotations
            std::vector<cd> first = std::move(dG[0]);
            for (int i = 0; i < mmax - 1; ++i) dG[i] = std::move(dG[i + 1]);
            dG[mmax - 1] = std::move(first);
            const int k = mmax;
            for (int i = 1; i < k; ++i) {
                double c; cd sn;
                givens(Rr(i - 1, i), Rr(i, i), c, sn);
                for (int j = 0; j < k; ++j) {
                    cd a = Rr(i - 1, j), b = Rr(i, j);
                    Rr(i - 1, j) = c * a + sn * b;
                    Rr(i, j) = -std::conj(sn) * a + c * b;
                }
                std::vector<cd>& qa = Q[i - 1];
                std::vector<cd>& qb = Q[i];
                for (size_t t = 0; t < n; ++t) {
                    cd a = qa[t], b = qb[t];
                    qa[t] = c * a + std::conj(sn) * b;
                    qb[t] = -sn * a + c * b;
                }
            }
            for (int j = 0; j < k - 1; ++j)
                for (int i = 0; i < k - 1; ++i) Rr(i, j) = Rr(i, j + 1);
            m_eff = mmax;
        }
        std::vector<cd>& dg = dG[m_eff - 1];
        for (size_t t = 0; t < n; ++t) dg[t] = g[t] - gold[t];
        for (size_t t = 0; t < n; ++t) fxold[t] = fx[t] - fxold[t];
        // qradd!: modified Gram-Schmidt of the new column
        const int k = m_eff - 1;
        for (int i = 0; i < k; ++i) {
            cd r = 0.0;
            for (size_t t = 0; t < n; ++t) r += std::conj(Q[i][t]) * fxold[t];
            Rr(i, k) = r;
            for (size_t t = 0; t < n; ++t) fxold[t] -= r * Q[i][t];
        }
        double nr = 0.0;
        for (size_t t = 0; t < n; ++t) nr += std::norm(fxold[t]);
        nr = std::sqrt(nr);
        Rr(k, k) = nr;
        for (size_t t = 0; t < n; ++t) Q[k][t] = fxold[t] / nr;
        // γ = R \ (Q^H fx)
        for (int i = 0; i < m_eff; ++i) {
            cd r = 0.0;
            for (size_t t = 0; t < n; ++t) r += std::conj(Q[i][t]) * fx[t];
            gam[i] = r;
        }
        for (int i = m_eff - 1; i >= 0; --i) {
            cd v = gam[i];
            for (int j = i + 1; j < m_eff; ++j) v -= Rr(i, j) * gam[j];
            gam[i] = v / Rr(i, i);
        }
        for (int i = 0; i < m_eff; ++i)
            for (size_t t = 0; t < n; ++t) x[t] -= gam[i] * dG[i][t];
        fxold = fx; gold = g;
    }
    return out;
}

// --------------------------------------------------------------------------------------------
// Model inputs: src/models/siam.jl:9-29, src/models/hubbard.jl:8-44
// --------------------------------------------------------------------------------------------
static void siam_bare(Solver& s, std::vector<cd>& out, double e, double Delta, double D) {
    for (int n = -s.d.nG; n < s.d.nG; ++n) {
        const double nu = (2.0 * n + 1.0) * M_PI * s.d.T;
        const double sg = (nu > 0) - (nu < 0);
        cd v = std::isinf(D) ? 1.0 / (nu + cd(0.0, e) + Delta * sg)
                             : 1.0 / (nu + cd(0.0, e) + 2.0 * Delta / M_PI * std::atan(D / nu));
        out[s.iG(n, 0)] = v;
    }
}

static void hubbard_bare(Solver& s, std::vector<cd>& out, double mu, double t1, double t2, double t3) {
    const int L = s.d.LG;
    for (int k = 0; k < L * L; ++k) {
        const double k1 = 2.0 * M_PI * (k % L) / L, k2 = 2.0 * M_PI * (k / L) / L;
        double ek = -2.0 * t1 * (std::cos(k1) + std::cos(k2));
        ek += -4.0 * t2 * std::cos(k1) * std::cos(k2);
        ek += -2.0 * t3 * (std::cos(2 * k1) + std::cos(2 * k2));
        for (int n = -s.d.nG; n < s.d.nG; ++n) {
            const double nu = (2.0 * n + 1.0) * M_PI * s.d.T;
            out[s.iG(n, k)] = 1.0 / (cd(0.0, nu) + mu - ek) * cd(0.0, 1.0);
        }
    }
}

}  // namespace orc

// ============================================================================================
// C interface (ctypes)
// ============================================================================================
using namespace orc;

extern "C" {

struct orc_dims {
    int nG, nK1, nK2O, nK2n, nK3O, nK3n, L, LG, fPi, local;
    double T, U;
    int nRO, nRn;
    int f0_is_vertex, nF0K1, nF0K2O, nF0K2n, nF0K3O, nF0K3n;
};

void* orc_create(const orc_dims* dd) {
    Dims d;
    d.nG = dd->nG; d.nK1 = dd->nK1; d.nK2O = dd->nK2O; d.nK2n = dd->nK2n; d.nK3O = dd->nK3O; d.nK3n = dd->nK3n;
    d.L = dd->L; d.LG = dd->LG; d.fPi = dd->fPi; d.local = dd->local; d.T = dd->T; d.U = dd->U;
    d.nRO = dd->nRO; d.nRn = dd->nRn;
    d.f0_is_vertex = dd->f0_is_vertex; d.nF0K1 = dd->nF0K1; d.nF0K2O = dd->nF0K2O; d.nF0K2n = dd->nF0K2n;
    d.nF0K3O = dd->nF0K3O; d.nF0K3n = dd->nF0K3n;
    return create(d);
}
void orc_destroy(void* h) { delete (Solver*)h; }
void orc_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int orc_max_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static std::vector<cd>* named(Solver* s, const char* name) {
    std::string n(name);
    if (n == "Gbare") return &s->Gbare;
    if (n == "G0") return &s->G0;
    if (n == "Sigma0") return &s->Sig0;
    if (n == "G") return &s->G;
    if (n == "Sigma") return &s->Sig;
    if (n == "Pi0pp") return &s->Pi0pp;
    if (n == "Pi0ph") return &s->Pi0ph;
    if (n == "Pipp") return &s->Pipp;
    if (n == "Piph") return &s->Piph;
    if (n == "Lpp") return &s->Lpp;
    if (n == "Lph") return &s->Lph;
    if (n == "Fp_p") return &s->ref.Fp_p;
    if (n == "Fp_x") return &s->ref.Fp_x;
    if (n == "Ft_p") return &s->ref.Ft_p;
    if (n == "Ft_x") return &s->ref.Ft_x;
    static const char* cn[10] = {"cache_Gpx", "cache_F0p", "cache_F0a", "cache_F0t", "cache_Gpp",
                                 "cache_Ga",  "cache_Gt",  "cache_Fp",  "cache_Fa",  "cache_Ft"};
    for (int i = 0; i < 10; ++i) if (n == cn[i]) return &s->cache[i];
    // vertex blocks: "<F|Fbuff|FL|F0>.<p|t|a>.<K1|K2|K3>"
    Vert* v = nullptr;
    size_t dot = n.find('.');
    if (dot == std::string::npos) return nullptr;
    std::string vn = n.substr(0, dot), rest = n.substr(dot + 1);
    if (vn == "F") v = &s->F; else if (vn == "Fbuff") v = &s->Fbuff; else if (vn == "FL") v = &s->FL;
    else if (vn == "F0") v = &s->F0v; else return nullptr;
    if (rest.size() != 4) return nullptr;
    int c = rest[0] == 'p' ? CH_P : (rest[0] == 't' ? CH_T : (rest[0] == 'a' ? CH_A : -1));
    if (c < 0) return nullptr;
    std::string k = rest.substr(2);
    if (k == "K1") return &v->g[c].K1;
    if (k == "K2") return &v->g[c].K2;
    if (k == "K3") return &v->g[c].K3;
    return nullptr;
}

long orc_len(void* h, const char* name) {
    auto* v = named((Solver*)h, name);
    return v ? (long)v->size() : -1;
}
int orc_set(void* h, const char* name, const double* re_im, long n) {
    auto* v = named((Solver*)h, name);
    if (!v || (long)v->size() != n) return 1;
    std::memcpy(static_cast<void*>(v->data()), re_im, sizeof(cd) * n);  // std::complex<double>: (re, im) pairs
    return 0;
}
int orc_get(void* h, const char* name, double* re_im, long n) {
    auto* v = named((Solver*)h, name);
    if (!v || (long)v->size() != n) return 1;
    std::memcpy(re_im, v->data(), sizeof(cd) * n);
    return 0;
}
void orc_set_variant_single_hartree(void* h, int on) { ((Solver*)h)->variant_single_hartree = on; }
void orc_finalize(void* h) { finalize(*(Solver*)h); }
void orc_init_sym_grp(void* h) { init_sym_grp(*(Solver*)h); }
long orc_state_len(void* h) { return (long)state_len(*(Solver*)h); }
void orc_flatten(void* h, double* x) { flatten(*(Solver*)h, (cd*)x); }
void orc_unflatten(void* h, const double* x) { unflatten(*(Solver*)h, (const cd*)x); }
void orc_iterate(void* h, int strategy, int update_sigma, int compute_hartree) {
    iterate(*(Solver*)h, strategy, update_sigma != 0, compute_hartree != 0);
}
// symmetrize_solver!(S) (src/ParquetSolver.jl:246-259): every class takes its representative's value
void orc_symmetrize(void* h) {
    Solver& s = *(Solver*)h;
    sg_symmetrize(s.sgSig, s.Sig.data());
    for (int c : {CH_A, CH_P, CH_T}) {
        const SymGroup* G = (c == CH_P) ? s.sgpp : s.sgph;
        sg_symmetrize(G[0], s.F.g[c].K1.data());
        sg_symmetrize(G[1], s.F.g[c].K2.data());
        sg_symmetrize(G[2], s.F.g[c].K3.data());
    }
}
// mfRG linear map: y = x - Φ_mfRG(x f)/f on the vertex part (length F.length()); nonlocal solver only
int orc_mfrg_apply(void* h, const double* x, double* y) {
    Solver& s = *(Solver*)h;
    if (s.d.local) return 1;
    mfrg_apply(s, (const cd*)x, (cd*)y);
    return 0;
}
void orc_dyson(void* h) { Solver& s = *(Solver*)h; dyson(s.G, s.Sig, s.Gbare); }
void orc_bubbles(void* h) { Solver& s = *(Solver*)h; bubbles(s, s.Pipp, s.Piph, s.G); }
void orc_build_cache(void* h) { Solver& s = *(Solver*)h; s.F.update_avg(); build_K3_cache(s); }
double orc_occupation(void* h, const char* name) { Solver& s = *(Solver*)h; return occupation(s, *named(&s, name)); }
void orc_siam_bare(void* h, const char* name, double e, double Delta, double D) {
    Solver& s = *(Solver*)h; siam_bare(s, *named(&s, name), e, Delta, D);
}
void orc_hubbard_bare(void* h, const char* name, double mu, double t1, double t2, double t3) {
    Solver& s = *(Solver*)h; hubbard_bare(s, *named(&s, name), mu, t1, t2, t3);
}
int orc_solve(void* h, int strategy, int update_sigma, int compute_hartree, int maxiter, double tol, double beta, int mem,
              double* trace, double* last_res) {
    auto r = anderson(*(Solver*)h, strategy, update_sigma != 0, compute_hartree != 0, maxiter, tol, beta, mem, trace);
    if (last_res) *last_res = r.last_res;
    return r.converged ? r.iterations : -r.iterations;
}
// class count and representatives of a named group, for cross-checking the product's builder
long orc_group_info(void* h, const char* name, int* cstart, int* members, int* ops, long cap) {
    Solver& s = *(Solver*)h;
    std::string n(name);
    const SymGroup* G = nullptr;
    if (n == "Sigma") G = &s.sgSig;
    else if (n == "pp1") G = &s.sgpp[0]; else if (n == "pp2") G = &s.sgpp[1]; else if (n == "pp3") G = &s.sgpp[2];
    else if (n == "ph1") G = &s.sgph[0]; else if (n == "ph2") G = &s.sgph[1]; else if (n == "ph3") G = &s.sgph[2];
    else if (n == "ppL3") G = &s.sgppL[2]; else if (n == "phL3") G = &s.sgphL[2];
    if (!G || G->trivial) return -1;
    const long nm = (long)G->members.size(), nc = (long)G->nclass();
    if (cap >= nm && members) {
        for (long i = 0; i < nm; ++i) { members[i] = G->members[i]; ops[i] = G->ops[i]; }
        for (long i = 0; i <= nc; ++i) cstart[i] = G->cstart[i];
    }
    return nc;
}
}
