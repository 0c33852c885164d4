"""Host-side mirror of fdDGAsolver.jl's solver API over libfdga.

Names, arguments and defaults follow the reference:
  ParquetSolver(nK1, nK2, nK3, Gbare, G0, Σ0, F0; mΠν_factor=6)        src/ParquetSolver.jl:277-352
  NL_ParquetSolver(nK1, nK2, nK3, L, Gbare, G0, Σ0, F0; mΠν_factor=32) src/nonlocal/ParquetSolver.jl:77-152
  parquet_solver_siam_parquet_approximation(nG, nK1, nK2, nK3; e, Δ, D, T, U)   src/ParquetSolver.jl:170-200
  parquet_solver_hubbard_parquet_approximation(nG, nK1, nK2, nK3, L; T, U, μ, t1, t2, t3)
                                                                       src/nonlocal/ParquetSolver.jl:166-194
  init_sym_grp!(S)                    -> init_sym_grp(S)              src/ParquetSolver.jl:203-231
  iterate_solver!(S; strategy, update_Σ, compute_Hartree) -> iterate_solver(S, ...)  src/solve.jl:4-116
  fixed_point!(R, x, S)               -> fixed_point(S, x)            src/solve.jl:119-157
  solve!(S; maxiter, tol, δ, mem)     -> solve(S, ...)                src/solve.jl:160-196
  flatten(S) / unflatten!(S, x)       -> flatten(S) / unflatten(S, x) src/ParquetSolver.jl:277-306
Complex arrays are numpy complex128 in the reference's column-major order.
"""
import ctypes

import numpy as np

from . import _lib
from .models import hubbard_bare_Green, siam_bare_Green

STRATEGIES = {"fdPA": _lib.FDGA_FDPA, "scPA": _lib.FDGA_SCPA, "fdPA_new": _lib.FDGA_FDPA_NEW,
              "scPA_new": _lib.FDGA_SCPA_NEW, "fdPA_1loop": _lib.FDGA_FDPA_1LOOP}


class RefVertex:
    """RefVertex(U, Fp_p, Fp_x, Ft_p, Ft_x) (src/refvertex.jl:1-35); corrections optional.

    Correction arrays have the K3 shape (2nR0-1, 2nR1, 2nR1), column-major [Ω, ν, ν']."""

    def __init__(self, T, U, Fp_p=None, Fp_x=None, Ft_p=None, Ft_x=None):
        self.T = float(T)
        self.U = float(U)
        arrs = [Fp_p, Fp_x, Ft_p, Ft_x]
        if all(a is None for a in arrs):
            self.nR = (1, 1)
            self.arrays = [np.zeros((1, 2, 2), dtype=np.complex128) for _ in range(4)]
        else:
            shp = next(a.shape for a in arrs if a is not None)
            if len(shp) != 3 or shp[1] != shp[2] or shp[0] % 2 != 1 or shp[1] % 2 != 0:
                raise ValueError("RefVertex corrections must have shape (2nΩ-1, 2nν, 2nν)")
            self.nR = ((shp[0] + 1) // 2, shp[1] // 2)
            self.arrays = [np.zeros(shp, dtype=np.complex128) if a is None else np.asarray(a, dtype=np.complex128)
                           for a in arrs]
            if any(a.shape != shp for a in self.arrays):
                raise ValueError("all RefVertex corrections must share one shape")


class Vertex:
    """Vertex(F0, γp, γt, γa) (src/vertex.jl:7-35): a channel-decomposed vertex whose own reference
    vertex F0 is a RefVertex.  As the reference vertex of a solver it makes the fdDΓA solve of
    ParquetSolver(nK1, nK2, nK3, Gbare, S0.G, S0.Σ, S0.F) (test/test_siam_fdPA.jl:79-84).

    flat = flatten(F) = [γp(K1,K2,K3), γt, γa] in the reference's column-major layout of its boxes
    nK1, nK2, nK3 (src/vertex.jl:152-165); L is the momentum mesh (1 for a local vertex)."""

    def __init__(self, F0, nK1, nK2, nK3, flat, L=1):
        if not isinstance(F0, RefVertex):
            raise TypeError("the reference vertex of a Vertex is a RefVertex")
        self.F0 = F0
        self.T, self.U = F0.T, F0.U
        self.nK1, self.nK2, self.nK3, self.L = int(nK1), tuple(nK2), tuple(nK3), int(L)
        self.flat = np.ascontiguousarray(np.asarray(flat, dtype=np.complex128).reshape(-1))
        Nq = self.L * self.L
        n = 3 * Nq * ((2 * self.nK1 - 1) + (2 * self.nK2[0] - 1) * 2 * self.nK2[1] +
                      (2 * self.nK3[0] - 1) * (2 * self.nK3[1]) ** 2)
        if self.flat.size != n:
            raise ValueError(f"flatten(F) has {self.flat.size} values, the boxes need {n}")

    @property
    def nR(self):
        return self.F0.nR

    @property
    def arrays(self):
        return self.F0.arrays


def _as_f(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.complex128).reshape(-1, order="F"))


class _Solver:
    local = True

    def __init__(self, nK1, nK2, nK3, L, Gbare, G0, Sigma0, F0, *, mPi_factor, precision=0):
        if not isinstance(F0, (RefVertex, Vertex)):
            raise TypeError("the reference vertex F0 is a RefVertex or a Vertex")
        if isinstance(F0, Vertex) and F0.L != int(L):
            raise ValueError("a Vertex reference vertex has the solver's momentum mesh")
        lib = _lib.load()
        Gbare = np.asarray(Gbare, dtype=np.complex128)
        nG = Gbare.shape[0] // 2
        c = _lib.fdga_config()
        c.nG, c.nK1 = nG, int(nK1)
        c.nK2[0], c.nK2[1] = nK2
        c.nK3[0], c.nK3[1] = nK3
        c.L = c.LG = int(L)
        c.mPi_factor = int(mPi_factor)
        c.local = 1 if self.local else 0
        c.T, c.U = F0.T, F0.U
        c.nR[0], c.nR[1] = F0.nR
        c.precision = int(precision)
        if isinstance(F0, Vertex):
            c.f0_vertex = 1
            c.nF0K1 = F0.nK1
            c.nF0K2[0], c.nF0K2[1] = F0.nK2
            c.nF0K3[0], c.nF0K3[1] = F0.nK3
        h = ctypes.c_void_p()
        _lib.check(lib.fdga_create(ctypes.byref(c), ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self.T, self.U = F0.T, F0.U
        self.nG, self.nK1, self.nK2, self.nK3, self.L = nG, nK1, tuple(nK2), tuple(nK3), L
        self.F0 = F0
        self._set(_lib.IN_GBARE, Gbare)
        self._set(_lib.IN_G0, G0)
        self._set(_lib.IN_SIGMA0, Sigma0)
        for k, a in enumerate(F0.arrays):
            self._set(_lib.IN_FP_P + k, a)
        if isinstance(F0, Vertex):
            self._check(lib.fdga_set_input(h, _lib.IN_F0_VERTEX, F0.flat.ctypes.data, F0.flat.size))
        self._check(lib.fdga_finalize(h))
        n = ctypes.c_size_t()
        self._check(lib.fdga_state_len(h, ctypes.byref(n)))
        self.state_len = n.value

    # -- plumbing --
    def _check(self, rc):
        _lib.check(rc, self._h)

    def _set(self, which, a):
        a = _as_f(a)
        self._check(self._lib.fdga_set_input(self._h, which, a.ctypes.data, a.size))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fdga_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- reference API --
    def init_sym_grp(self):
        self._check(self._lib.fdga_init_sym_grp(self._h))

    @property
    def F(self):
        """S.F: the current vertex as a host Vertex (its reference vertex is this solver's RefVertex),
        to become the reference vertex F0 of another solver."""
        if isinstance(self.F0, Vertex):
            raise NotImplementedError("S.F of a solver whose own F0 is a Vertex (a reference chain of depth > 2)")
        nS = 2 * self.nG * self.L * self.L
        return Vertex(self.F0, self.nK1, self.nK2, self.nK3, self.flatten()[:-nS], L=self.L)

    def flatten(self):
        x = np.empty(self.state_len, dtype=np.complex128)
        self._check(self._lib.fdga_flatten(self._h, x.ctypes.data, x.size))
        return x

    def unflatten(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        if x.size != self.state_len:
            raise ValueError("state length mismatch")
        self._check(self._lib.fdga_unflatten(self._h, x.ctypes.data, x.size))

    def iterate_solver(self, strategy="fdPA", update_Sigma=True, compute_Hartree=True):
        self._check(self._lib.fdga_iterate(self._h, STRATEGIES[strategy], int(update_Sigma), int(compute_Hartree)))

    def fixed_point(self, x, strategy="fdPA"):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        R = np.empty_like(x)
        self._check(self._lib.fdga_residual(self._h, STRATEGIES[strategy], x.ctypes.data, R.ctypes.data, x.size))
        return R

    def solve(self, strategy="fdPA", maxiter=100, tol=1e-4, delta=0.85, mem=8):
        trace = np.zeros(maxiter, dtype=np.float64)
        it = ctypes.c_int()
        res = ctypes.c_double()
        self._check(self._lib.fdga_solve(self._h, STRATEGIES[strategy], int(maxiter), float(tol), float(delta), int(mem),
                                         ctypes.byref(it), ctypes.byref(res), trace.ctypes.data))
        n = abs(it.value)
        return {"converged": it.value > 0, "iterations": n, "residual": res.value, "trace": trace[:n]}

    def solve_mixed(self, strategy="fdPA", maxiter=300, tol=1e-8, delta=0.85, mem=8):
        """The FP64 fixed point by iterative refinement around mixed-precision inner Anderson solves."""
        trace = np.zeros(maxiter, dtype=np.float64)
        it = ctypes.c_int()
        res = ctypes.c_double()
        ev = np.zeros(2, dtype=np.int32)
        self._check(self._lib.fdga_solve_mixed(self._h, STRATEGIES[strategy], int(maxiter), float(tol), float(delta),
                                               int(mem), ctypes.byref(it), ctypes.byref(res), trace.ctypes.data,
                                               ev.ctypes.data))
        n = abs(it.value)
        return {"converged": it.value > 0, "outer": n, "residual": res.value, "trace": trace[:n],
                "evals_fp64": int(ev[0]), "evals_mixed": int(ev[1])}

    def solve_newton(self, strategy="fdPA", maxiter=300, tol=1e-8, restart=30, jvp="fp64"):
        """Newton–Krylov (GMRES(restart), forward-difference JVPs in 'fp64' or 'mixed') to max|R| < tol."""
        trace = np.zeros(maxiter, dtype=np.float64)
        it = ctypes.c_int()
        res = ctypes.c_double()
        ev = np.zeros(2, dtype=np.int32)
        self._check(self._lib.fdga_solve_newton(self._h, STRATEGIES[strategy], int(maxiter), float(tol), int(restart),
                                                {"fp64": 0, "mixed": 1}[jvp], ctypes.byref(it), ctypes.byref(res),
                                                trace.ctypes.data, ev.ctypes.data))
        n = abs(it.value)
        return {"converged": it.value > 0, "newton": n, "residual": res.value, "trace": trace[:n],
                "evals_fp64": int(ev[0]), "evals_mixed": int(ev[1])}

    def mfrg_apply(self, x, strategy="fdPA"):
        """mfRGLinearMap(S, strategy) * x (src/mfRG.jl:20-89): x - Φ_mfRG(x·1e-2)/1e-2 on a vertex
        vector of length(S.F) (the vertex part of flatten(S)); nonlocal solver."""
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.empty_like(x)
        self._check(self._lib.fdga_mfrg_apply(self._h, STRATEGIES[strategy], x.ctypes.data, y.ctypes.data, x.size))
        return y

    def fixed_point_preconditioned(self, x, strategy="fdPA", update_sigma=False, krylov_maxiter=400,
                                   krylov_rtol=1e-6, krylov_atol=1e-6):
        """fixed_point_preconditioned!(R, x, S; strategy, update_Σ) (src/mfRG.jl:93-173): the residual
        of one iteration with its vertex part solved against the mfRG map (GMRES on the device).
        x is flatten(S) when update_sigma, else the vertex part flatten(S.F).  Returns
        (R, info) with info = {"krylov_iterations", "krylov_residual"}."""
        x = np.ascontiguousarray(x, dtype=np.complex128)
        R = np.empty_like(x)
        it = ctypes.c_int()
        rel = ctypes.c_double()
        self._check(self._lib.fdga_residual_mfrg(self._h, STRATEGIES[strategy], x.ctypes.data, R.ctypes.data, x.size,
                                                 int(bool(update_sigma)), int(krylov_maxiter), float(krylov_rtol),
                                                 float(krylov_atol), ctypes.byref(it), ctypes.byref(rel)))
        return R, {"krylov_iterations": it.value, "krylov_residual": rel.value}

    def solve_mfrg(self, strategy="fdPA", maxiter=40, tol=1e-4, delta=0.85, mem=50, update_sigma=False,
                   krylov_maxiter=400, krylov_rtol=1e-6, krylov_atol=1e-6):
        """solve_using_mfRG_without_mixing!(S; tol, strategy, update_Σ, maxiter, memory, mixing)
        (src/mfRG.jl:686-776): nlsolve(anderson) over fixed_point_preconditioned!, on the device from the
        current state; S ends at the last evaluated x, symmetrized."""
        trace = np.zeros(maxiter, dtype=np.float64)
        it = ctypes.c_int()
        res = ctypes.c_double()
        kt = ctypes.c_int()
        self._check(self._lib.fdga_solve_mfrg(self._h, STRATEGIES[strategy], int(maxiter), float(tol), float(delta),
                                              int(mem), int(bool(update_sigma)), int(krylov_maxiter),
                                              float(krylov_rtol), float(krylov_atol), ctypes.byref(it),
                                              ctypes.byref(res), trace.ctypes.data, ctypes.byref(kt)))
        n = abs(it.value)
        return {"converged": it.value > 0, "iterations": n, "residual": res.value, "trace": trace[:n],
                "krylov_iterations": kt.value}

    def jvp(self, v, strategy="fdPA"):
        """dΦ/dx · v at the current state (flatten layout)."""
        v = np.ascontiguousarray(v, dtype=np.complex128)
        out = np.empty_like(v)
        self._check(self._lib.fdga_jvp(self._h, STRATEGIES[strategy], v.ctypes.data, out.ctypes.data, v.size))
        return out

    def frule(self, v, strategy="fdPA", update_sigma=True, compute_hartree=True):
        """(Φ(x), Φ'(x)·v) at the current state x from the tangent kernels (forward mode, no finite
        differences), the frule of one fixed_point! iteration; v in the flatten layout."""
        v = np.ascontiguousarray(v, dtype=np.complex128)
        y = np.empty_like(v)
        jv = np.empty_like(v)
        self._check(self._lib.fdga_frule(self._h, STRATEGIES[strategy], int(bool(update_sigma)),
                                         int(bool(compute_hartree)), v.ctypes.data, y.ctypes.data,
                                         jv.ctypes.data, v.size))
        return y, jv

    def rrule(self, ybar, strategy="fdPA", update_sigma=True, compute_hartree=True):
        """(Φ(x), Φ'(x)ᵀ·ȳ) at the current state x from the adjoint kernels (reverse mode), the rrule
        of one fixed_point! iteration; the transpose is for the real inner product Re Σ conj(a) b."""
        ybar = np.ascontiguousarray(ybar, dtype=np.complex128)
        y = np.empty_like(ybar)
        xbar = np.empty_like(ybar)
        self._check(self._lib.fdga_rrule(self._h, STRATEGIES[strategy], int(bool(update_sigma)),
                                         int(bool(compute_hartree)), ybar.ctypes.data, y.ctypes.data,
                                         xbar.ctypes.data, ybar.size))
        return y, xbar

    def set_U(self, U):
        self._check(self._lib.fdga_set_U(self._h, float(U)))

    def dchi_dU(self, channel="m", strategy="fdPA", hU=1e-4, restart=40, cycles=4, rtol=1e-10):
        """dχ/dU(Ω, q) at the converged state (linear response through GMRES), flat [Ω, q] layout."""
        n = self.get_len("F.a.K1")
        out = np.empty(n, dtype=np.complex128)
        its = ctypes.c_int()
        rel = ctypes.c_double()
        self._check(self._lib.fdga_dchi_dU(self._h, STRATEGIES[strategy], {"m": 0, "d": 1, "s": 2}[channel],
                                           float(hU), int(restart), int(cycles), float(rtol), out.ctypes.data, n,
                                           ctypes.byref(its), ctypes.byref(rel)))
        return out, {"gmres_iterations": its.value, "relres": rel.value}

    def autotune(self, strategy="fdPA"):
        """Pick the K3 GEMM tiles per size class by timing; returns {fp64: (L_K3, K3), mixed: (L_K3, K3)}."""
        t = np.zeros(4, dtype=np.int32)
        self._check(self._lib.fdga_autotune(self._h, STRATEGIES[strategy], t.ctypes.data))
        return {"fp64": (int(t[0]), int(t[1])), "mixed": (int(t[2]), int(t[3]))}

    def get(self, name):
        n = ctypes.c_size_t()
        self._check(self._lib.fdga_named_len(self._h, name.encode(), ctypes.byref(n)))
        out = np.empty(n.value, dtype=np.complex128)
        self._check(self._lib.fdga_get_named(self._h, name.encode(), out.ctypes.data, out.size))
        return out

    def set_option(self, key, value):
        self._check(self._lib.fdga_set_option(self._h, key.encode(), int(value)))

    def set_precision(self, precision):
        """'fp64' (plain path) or 'mixed' (K3 contractions in FP32) for later iterate/residual calls."""
        self._check(self._lib.fdga_set_precision(self._h, {"fp64": 0, "mixed": 1}[precision]))

    def susceptibility(self, channel="m", local=False):
        """Connected χ_m / χ_d / χ_s from K1 (K1_r = -U² χ_r, src/utility/load_triqs.jl:67-75,106-114).

        Flat array in the reference's column-major [Ω, q] layout (length NΩ1·Nq), or the momentum
        average χ_loc(Ω) (length NΩ1) when local."""
        which = {"m": 0, "d": 1, "s": 2}[channel]
        n = 2 * self.nK1 - 1 if local else self.get_len("F.a.K1")
        out = np.empty(n, dtype=np.complex128)
        self._check(self._lib.fdga_susceptibility(self._h, which, out.ctypes.data, n))
        return out

    def get_len(self, name):
        n = ctypes.c_size_t()
        self._check(self._lib.fdga_named_len(self._h, name.encode(), ctypes.byref(n)))
        return n.value

    def occupation(self):
        v = ctypes.c_double()
        self._check(self._lib.fdga_occupation(self._h, ctypes.byref(v)))
        return v.value

    # -- timing helpers on the solver's stream --
    def event_record(self, slot):
        self._check(self._lib.fdga_event_record(self._h, slot))

    def event_elapsed_ms(self, a, b):
        v = ctypes.c_float()
        self._check(self._lib.fdga_event_elapsed_ms(self._h, a, b, ctypes.byref(v)))
        return v.value

    def synchronize(self):
        self._check(self._lib.fdga_synchronize(self._h))

    def stage_times(self, strategy="fdPA", nrep=3, tangent=False):
        """Per-stage device milliseconds of an eager iteration (CUDA events on the solver stream);
        tangent=True: of the tangent map at the last frule's base point and direction."""
        names = ctypes.create_string_buffer(1024)
        ms = np.zeros(32, dtype=np.float64)
        n = ctypes.c_int()
        fn = self._lib.fdga_tangent_stage_times if tangent else self._lib.fdga_stage_times
        self._check(fn(self._h, STRATEGIES[strategy], int(nrep), names, 1024, ms.ctypes.data, 32, ctypes.byref(n)))
        keys = names.value.decode().split(",") if n.value else []
        return dict(zip(keys, ms[: n.value].tolist()))

    def map_repeat(self, n, strategy="fdPA"):
        """Apply the iteration map n times to the unchanged device state (no host sync)."""
        self._check(self._lib.fdga_map_repeat(self._h, STRATEGIES[strategy], int(n)))

    def adjoint_repeat(self, n, strategy="fdPA"):
        """Replay the adjoint map n times at the base point and cotangent of the last rrule call."""
        self._check(self._lib.fdga_adjoint_repeat(self._h, STRATEGIES[strategy], int(n)))

    def tangent_repeat(self, n, strategy="fdPA"):
        """Apply the tangent map n times at the base point and direction of the last frule call."""
        self._check(self._lib.fdga_tangent_repeat(self._h, STRATEGIES[strategy], int(n)))

    def flush_l2(self, nbytes=256 << 20):
        """Overwrite the L2 with a device buffer write on the solver's stream."""
        self._check(self._lib.fdga_flush_l2(self._h, int(nbytes)))

    def fixed_point_ptr(self, x_ptr, R_ptr, strategy="fdPA"):
        """fixed_point! on caller-owned host buffers (e.g. pinned) of state_len complex values."""
        self._check(self._lib.fdga_residual(self._h, STRATEGIES[strategy], x_ptr, R_ptr, self.state_len))

    def query(self, key):
        v = ctypes.c_double()
        self._check(self._lib.fdga_query(self._h, key.encode(), ctypes.byref(v)))
        return v.value

    def launches_per_iteration(self):
        v = ctypes.c_int()
        self._check(self._lib.fdga_launches_per_iteration(self._h, ctypes.byref(v)))
        return v.value


class ParquetSolver(_Solver):
    local = True

    def __init__(self, nK1, nK2, nK3, Gbare, G0, Sigma0, F0, *, mPi_factor=6, precision=0):
        super().__init__(nK1, nK2, nK3, 1, Gbare, G0, Sigma0, F0, mPi_factor=mPi_factor, precision=precision)


class NL_ParquetSolver(_Solver):
    local = False

    def __init__(self, nK1, nK2, nK3, L, Gbare, G0, Sigma0, F0, *, mPi_factor=32, precision=0):
        super().__init__(nK1, nK2, nK3, L, Gbare, G0, Sigma0, F0, mPi_factor=mPi_factor, precision=precision)


def parquet_solver_siam_parquet_approximation(nG, nK1, nK2, nK3, *, e, Delta, D, T, U, mPi_factor=6, F0=None):
    Gbare = siam_bare_Green(T, nG, Delta=Delta, e=e, D=D)
    z = np.zeros_like(Gbare)
    return ParquetSolver(nK1, nK2, nK3, Gbare, z, z, F0 or RefVertex(T, U), mPi_factor=mPi_factor)


def parquet_solver_hubbard_parquet_approximation(nG, nK1, nK2, nK3, L, *, T, U, mu, t1, t2=0.0, t3=0.0,
                                                 mPi_factor=32, F0=None):
    Gbare = hubbard_bare_Green(T, nG, L, mu=mu, t1=t1, t2=t2, t3=t3)
    z = np.zeros_like(Gbare)
    return NL_ParquetSolver(nK1, nK2, nK3, L, Gbare, z, z, F0 or RefVertex(T, U), mPi_factor=mPi_factor)


class PinnedBuffer:
    """Page-locked host buffer of complex128 values (fdga_host_alloc)."""

    def __init__(self, n):
        lib = _lib.load()
        self._lib = lib
        p = ctypes.c_void_p()
        _lib.check(lib.fdga_host_alloc(int(n) * 16, ctypes.byref(p)))
        self.ptr = p.value
        self.n = int(n)
        self.array = np.ctypeslib.as_array((ctypes.c_double * (2 * self.n)).from_address(self.ptr)).view(np.complex128)

    def free(self):
        if self.ptr:
            self._lib.fdga_host_free(ctypes.c_void_p(self.ptr))
            self.ptr = None


# Julia-style free functions
def init_sym_grp(S):
    S.init_sym_grp()


def iterate_solver(S, strategy="fdPA", update_Sigma=True, compute_Hartree=True):
    S.iterate_solver(strategy, update_Sigma, compute_Hartree)


def _lib_query(key):
    """fdga_query without a handle (device-level keys: fp64_gflops, selftest_d2f)."""
    from ._lib import load
    lib = load()
    v = ctypes.c_double()
    rc = lib.fdga_query(None, key.encode(), ctypes.byref(v))
    if rc != 0:
        raise RuntimeError(f"fdga_query({key}) failed with status {rc}")
    return v.value


def fixed_point(S, x, strategy="fdPA"):
    return S.fixed_point(x, strategy)


class mfRGLinearMap:
    """mfRGLinearMap(S, strategy) (src/mfRG.jl:20-32): a linear map on length(S.F) vectors;
    A * x and A @ x apply it on the device."""

    def __init__(self, S, strategy="fdPA"):
        if strategy not in ("fdPA", "fdPA_new", "fdPA_1loop"):
            raise ValueError(f"Invalid strategy {strategy}. Must be fdPA or fdPA_new or fdPA_1loop.")
        self.S, self.strategy = S, strategy
        n = S.state_len - 2 * S.nG * S.L * S.L  # length(S.F): flatten(S) without Σ
        self.shape = (n, n)

    def __mul__(self, x):
        return self.S.mfrg_apply(x, self.strategy)

    __matmul__ = __mul__


def fixed_point_preconditioned(S, x, strategy="fdPA", update_sigma=False, krylov_maxiter=400):
    """fixed_point_preconditioned!(R, x, S; strategy, update_Σ, krylov_maxiter) (src/mfRG.jl:93-173)."""
    return S.fixed_point_preconditioned(x, strategy, update_sigma, krylov_maxiter)[0]


def solve_using_mfRG_without_mixing(S, strategy="fdPA", tol=1e-4, update_sigma=False, maxiter=100, memory=50,
                                    mixing=0.85, krylov_maxiter=400):
    """solve_using_mfRG_without_mixing!(S; ...) (src/mfRG.jl:686-776) on the device."""
    return S.solve_mfrg(strategy, maxiter, tol, mixing, memory, update_sigma, krylov_maxiter)


def solve(S, strategy="fdPA", maxiter=100, tol=1e-4, delta=0.85, mem=8):
    return S.solve(strategy, maxiter, tol, delta, mem)


def flatten(S):
    return S.flatten()


def unflatten(S, x):
    S.unflatten(x)


def dyson_bubbles(S):
    """Dyson!(S); bubbles!(S) of the current state (src/dyson.jl:5-31, src/bubble.jl)."""
    S._check(S._lib.fdga_dyson_bubbles(S._h))


def interpolate_solver(So, Si, occ_target=None, hubbard_params=None):
    """interpolate_solver!(So, Si; occ_target, hubbard_params) (src/interpolate.jl:147-191): Σ and
    the vertex of Si Fourier-interpolated to So's lattice, So's G and bubbles updated and So
    symmetrized.  With occ_target, μ is then fixed to the occupation (src/dyson.jl:45-58) and Gbare,
    G and the bubbles follow."""
    So._check(So._lib.fdga_interpolate_solver(So._h, Si._h))
    if occ_target is not None:
        from .models import compute_hubbard_chemical_potential, hubbard_bare_Green
        hp = dict(hubbard_params or {})
        sig = So.get("Sigma").reshape(2 * So.nG, So.L * So.L, order="F")
        mu = compute_hubbard_chemical_potential(occ_target, sig, So.T, So.nG, So.L, **hp)
        So._set(_lib.IN_GBARE, hubbard_bare_Green(So.T, So.nG, So.L, mu=mu, **hp))
        dyson_bubbles(So)
        return mu
    return None


class Batch:
    """Independent solvers iterated together: one CUDA graph launch performs one iterate_solver! of
    every member, the members' kernels running as concurrent graph branches."""

    def __init__(self, solvers):
        from . import _lib
        self._lib = _lib.load()
        self.solvers = list(solvers)
        arr = (ctypes.c_void_p * len(self.solvers))(*[s._h for s in self.solvers])
        b = ctypes.c_void_p()
        rc = self._lib.fdga_batch_create(arr, len(self.solvers), ctypes.byref(b))
        if rc != 0:
            raise _lib.FdgaError(rc, self._lib.fdga_create_error().decode())
        self._b = b

    def _check(self, rc):
        if rc != 0:
            from . import _lib
            raise _lib.FdgaError(rc, (self._lib.fdga_batch_last_error(self._b) or b"").decode())

    def iterate(self, strategy="fdPA", precision="fp64"):
        self._check(self._lib.fdga_batch_iterate(self._b, STRATEGIES[strategy], {"fp64": 0, "mixed": 1}[precision]))

    def synchronize(self):
        self._check(self._lib.fdga_batch_synchronize(self._b))

    def time(self, iters, strategy="fdPA", precision="fp64"):
        """(device ms of `iters` batch iterations, kernels per batch iteration)."""
        ms = ctypes.c_float()
        k = ctypes.c_int()
        self._check(self._lib.fdga_batch_time(self._b, STRATEGIES[strategy], {"fp64": 0, "mixed": 1}[precision],
                                              int(iters), ctypes.byref(ms), ctypes.byref(k)))
        return ms.value, k.value

    def close(self):
        if getattr(self, "_b", None):
            self._lib.fdga_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
