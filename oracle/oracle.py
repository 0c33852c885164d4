"""ctypes front-end of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this module, and only as
the checker.  It mirrors the reference constructors so tests read like the reference's own:

* ``siam_pa(...)``     -> parquet_solver_siam_parquet_approximation   (src/ParquetSolver.jl:170-200)
* ``hubbard_pa(...)``  -> parquet_solver_hubbard_parquet_approximation (src/nonlocal/ParquetSolver.jl:166-194)
* ``OracleSolver.iterate`` -> iterate_solver!  (src/solve.jl:4-116)
* ``OracleSolver.solve``   -> solve!           (src/solve.jl:160-196)
"""
import ctypes
import os

import numpy as np

from . import build as _build

_LIB = None


class orc_dims(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("nG", "nK1", "nK2O", "nK2n", "nK3O", "nK3n", "L", "LG", "fPi", "local")] + [
        ("T", ctypes.c_double), ("U", ctypes.c_double)] + [
        (n, ctypes.c_int) for n in ("nRO", "nRn", "f0_is_vertex", "nF0K1", "nF0K2O", "nF0K2n", "nF0K3O", "nF0K3n")]


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        vp, cp, dp, ip = ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [ctypes.POINTER(orc_dims)]
        L.orc_destroy.argtypes = [vp]
        L.orc_len.restype = ctypes.c_long
        L.orc_len.argtypes = [vp, cp]
        L.orc_set.argtypes = [vp, cp, dp, ctypes.c_long]
        L.orc_get.argtypes = [vp, cp, dp, ctypes.c_long]
        L.orc_finalize.argtypes = [vp]
        L.orc_init_sym_grp.argtypes = [vp]
        L.orc_state_len.restype = ctypes.c_long
        L.orc_state_len.argtypes = [vp]
        L.orc_flatten.argtypes = [vp, dp]
        L.orc_unflatten.argtypes = [vp, dp]
        L.orc_iterate.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_dyson.argtypes = [vp]
        L.orc_bubbles.argtypes = [vp]
        L.orc_build_cache.argtypes = [vp]
        L.orc_occupation.restype = ctypes.c_double
        L.orc_occupation.argtypes = [vp, cp]
        L.orc_siam_bare.argtypes = [vp, cp, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.orc_hubbard_bare.argtypes = [vp, cp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.orc_solve.restype = ctypes.c_int
        L.orc_solve.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                ctypes.c_double, ctypes.c_int, dp, dp]
        L.orc_group_info.restype = ctypes.c_long
        L.orc_group_info.argtypes = [vp, cp, ip, ip, ip, ctypes.c_long]
        L.orc_set_variant_single_hartree.argtypes = [vp, ctypes.c_int]
        L.orc_symmetrize.argtypes = [vp]
        L.orc_mfrg_apply.restype = ctypes.c_int
        L.orc_mfrg_apply.argtypes = [vp, dp, dp]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_max_threads.restype = ctypes.c_int
        _LIB = L
    return _LIB


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def max_threads() -> int:
    return int(lib().orc_max_threads())


STRATEGIES = {"fdPA": 0, "scPA": 1, "fdPA_new": 2, "scPA_new": 3, "fdPA_1loop": 4}


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class OracleSolver:
    """CPU restatement of ParquetSolver / NL_ParquetSolver (FP64 complex)."""

    def __init__(self, *, nG, nK1, nK2, nK3, T, U, L=1, LG=None, local=True, mPi_factor=None,
                 nR=(1, 1), f0_vertex_box=None):
        d = orc_dims()
        d.nG, d.nK1 = nG, nK1
        d.nK2O, d.nK2n = nK2
        d.nK3O, d.nK3n = nK3
        d.L = 1 if local else L
        d.LG = 1 if local else (LG or L)
        d.fPi = mPi_factor if mPi_factor is not None else (6 if local else 32)
        d.local = 1 if local else 0
        d.T, d.U = float(T), float(U)
        d.nRO, d.nRn = nR
        if f0_vertex_box is not None:
            d.f0_is_vertex = 1
            d.nF0K1 = f0_vertex_box[0]
            d.nF0K2O, d.nF0K2n = f0_vertex_box[1]
            d.nF0K3O, d.nF0K3n = f0_vertex_box[2]
        self.dims = d
        self.h = lib().orc_create(ctypes.byref(d))
        self.local = bool(local)
        self.T = float(T)
        self.U = float(U)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().orc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    # ---- arrays (column-major, reference layout) ----
    def length(self, name):
        n = lib().orc_len(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        return n

    def get(self, name):
        n = self.length(name)
        out = np.zeros(n, dtype=np.complex128)
        if lib().orc_get(self.h, name.encode(), _dp(out.view(np.float64)), n) != 0:
            raise KeyError(name)
        return out

    def set(self, name, data):
        data = np.ascontiguousarray(np.asarray(data, dtype=np.complex128).reshape(-1, order="F"))
        if lib().orc_set(self.h, name.encode(), _dp(data.view(np.float64)), data.size) != 0:
            raise ValueError(f"{name}: size {data.size} != {self.length(name)}")

    def finalize(self):
        lib().orc_finalize(self.h)

    def set_variant_single_hartree(self, on=True):
        """Test-only: subtract the reference Hartree term once in the fdPA SDE (see the C++ note)."""
        lib().orc_set_variant_single_hartree(self.h, int(on))

    def init_sym_grp(self):
        lib().orc_init_sym_grp(self.h)

    def flatten(self):
        n = lib().orc_state_len(self.h)
        x = np.zeros(n, dtype=np.complex128)
        lib().orc_flatten(self.h, _dp(x.view(np.float64)))
        return x

    def unflatten(self, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        assert x.size == lib().orc_state_len(self.h)
        lib().orc_unflatten(self.h, _dp(x.view(np.float64)))

    def mfrg_apply(self, x):
        """mfRGLinearMap(S) * x (src/mfRG.jl:36-89): the vertex part of the state; nonlocal solver."""
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.zeros_like(x)
        if lib().orc_mfrg_apply(self.h, _dp(x.view(np.float64)), _dp(y.view(np.float64))) != 0:
            raise ValueError("the mfRG linear map is defined for the nonlocal solver")
        return y

    def symmetrize(self):
        """symmetrize_solver!(S) (src/ParquetSolver.jl:246-259)."""
        lib().orc_symmetrize(self.h)

    def fixed_point_preconditioned(self, x, strategy="fdPA", update_sigma=False, rtol=1e-12, maxiter=2000):
        """fixed_point_preconditioned!(R, x, S; strategy, update_Σ) (src/mfRG.jl:93-173) with the Krylov
        solve M z = R_F done to rtol by real GMRES (scipy) on the real-linear map: the map conjugates
        under the symmetry operations, so it acts on (Re, Im) pairs.  Test-only restatement."""
        import scipy.sparse.linalg as sla
        x = np.ascontiguousarray(x, dtype=np.complex128)
        full = self.flatten()
        nS = full.size - self.vertex_len()
        if update_sigma:
            self.unflatten(x)
        else:
            full[: x.size] = x
            self.unflatten(full)
        self.symmetrize()
        self.iterate(strategy, update_sigma=update_sigma)
        y = self.flatten()
        nF = y.size - nS
        RF = y[:nF] - x[:nF]
        RS = y[nF:] - x[nF:] if update_sigma else None
        n = nF

        def mv(v):
            z = self.mfrg_apply(v[:n] + 1j * v[n:])
            return np.concatenate([z.real, z.imag])

        A = sla.LinearOperator((2 * n, 2 * n), matvec=mv, dtype=np.float64)
        b = np.concatenate([RF.real, RF.imag])
        sol, info = sla.gmres(A, b, rtol=rtol, atol=0.0, restart=200, maxiter=maxiter)
        if info != 0:
            raise RuntimeError(f"oracle GMRES did not converge (info={info})")
        z = sol[:n] + 1j * sol[n:]
        return np.concatenate([z, RS]) if update_sigma else z

    def vertex_len(self):
        return lib().orc_state_len(self.h) - self.length("Sigma")

    def iterate(self, strategy="fdPA", update_sigma=True, compute_hartree=True):
        lib().orc_iterate(self.h, STRATEGIES[strategy], int(update_sigma), int(compute_hartree))

    def residual(self, x, strategy="fdPA"):
        """fixed_point!: R = Φ(x) - x (src/solve.jl:119-157)."""
        self.unflatten(x)
        self.iterate(strategy)
        return self.flatten() - x

    def solve(self, strategy="fdPA", maxiter=100, tol=1e-4, beta=0.85, mem=8, update_sigma=True,
              compute_hartree=True):
        trace = np.zeros(maxiter, dtype=np.float64)
        last = np.zeros(1, dtype=np.float64)
        it = lib().orc_solve(self.h, STRATEGIES[strategy], int(update_sigma), int(compute_hartree), maxiter, tol,
                             beta, mem, _dp(trace), _dp(last))
        n = abs(it)
        return {"converged": it > 0, "iterations": n, "trace": trace[:n], "residual": float(last[0])}

    def occupation(self, name="G"):
        return lib().orc_occupation(self.h, name.encode())

    def group(self, name):
        n = self.length({"Sigma": "Sigma", "pp1": "F.p.K1", "ph1": "F.p.K1", "pp2": "F.p.K2", "ph2": "F.p.K2"}.get(
            name, "F.p.K3"))
        cs = np.zeros(n + 1, dtype=np.int32)
        mem = np.zeros(n, dtype=np.int32)
        ops = np.zeros(n, dtype=np.int32)
        ip = ctypes.POINTER(ctypes.c_int)
        nc = lib().orc_group_info(self.h, name.encode(), cs.ctypes.data_as(ip), mem.ctypes.data_as(ip),
                                  ops.ctypes.data_as(ip), n)
        if nc < 0:
            return None
        return cs[: nc + 1].copy(), mem.copy(), ops.copy()

    # ---- model inputs (src/models/*.jl) ----
    def siam_bare_green(self, name="Gbare", *, e, Delta, D):
        lib().orc_siam_bare(self.h, name.encode(), e, Delta, D)

    def hubbard_bare_green(self, name="Gbare", *, mu, t1, t2=0.0, t3=0.0):
        lib().orc_hubbard_bare(self.h, name.encode(), mu, t1, t2, t3)


def siam_pa(nG, nK1, nK2, nK3, *, e, Delta, D, T, U, mPi_factor=6, sym=False):
    """parquet_solver_siam_parquet_approximation: G0 = Σ0 = 0, F0 = RefVertex(U)."""
    s = OracleSolver(nG=nG, nK1=nK1, nK2=nK2, nK3=nK3, T=T, U=U, local=True, mPi_factor=mPi_factor)
    s.siam_bare_green("Gbare", e=e, Delta=Delta, D=D)
    s.finalize()
    if sym:
        s.init_sym_grp()
    return s


def hubbard_pa(nG, nK1, nK2, nK3, L, *, T, U, mu, t1, t2=0.0, t3=0.0, LG=None, mPi_factor=32, nR=(1, 1),
               refvertex=None, sym=False):
    """parquet_solver_hubbard_parquet_approximation (+ optional RefVertex corrections)."""
    s = OracleSolver(nG=nG, nK1=nK1, nK2=nK2, nK3=nK3, T=T, U=U, L=L, LG=LG or L, local=False,
                     mPi_factor=mPi_factor, nR=nR)
    s.hubbard_bare_green("Gbare", mu=mu, t1=t1, t2=t2, t3=t3)
    if refvertex is not None:
        for k, v in refvertex.items():
            s.set(k, v)
    s.finalize()
    if sym:
        s.init_sym_grp()
    return s
