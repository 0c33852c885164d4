#!/usr/bin/env python
"""Benchmark of the parquet-iteration hot path (one JSON line on stdout).

Metric: seconds per parquet iteration (one iterate_solver!, fdPA, update_Σ) on the plain FP64 GPU
path, with time-to-converge at max|R| < 1e-8 reported beside it for the plain FP64 solver and the
mixed-precision iterative-refinement solver (and the mixed map's error per result).  Workload: the Hubbard 8x8
nonlocal fdPA configuration (t=1, t'=0, μ=0, U=2, β=5, nK1=32, nK2=(16,16), nK3=(8,12), nG=32,
mΠν_factor=32, seeded synthetic RefVertex), init_sym_grp! symmetry groups.

  value  device-resident: the iteration graph replayed K times on a fixed state, CUDA events on
         the solver's stream around each iteration, L2 flushed (256 MB write) before each.
  e2e    fixed_point!(R, x, S) through the C ABI with pinned host x and R: H2D + iteration + D2H
         (one graph whose copies overlap the iteration), host wall clock per call, L2 flushed
         before each call.
  --impl reference  the CPU oracle (C++ restatement of the reference algorithm, all host threads);
         the reference itself is Julia and cannot run on this machine.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "fddgasolver.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC_LABEL = {
    "siam_b10_nk3_16": "SIAM local config",
    "hubbard8x8_b5_nk3_8x12": "Hubbard 8x8 config",
    "hubbard16x16_n09_nk3_20x40": "Hubbard 16x16 n=0.9 config",
    "hubbard4x4_n09_nk3_20x40": "Hubbard 4x4 lattice with the 16x16 config's boxes",
    "hubbard24x24_b8_nk3_24x48": "Hubbard 24x24 config",
}


def metric_for(config):
    """The metric string of a workload's line (the default workload's is the headline metric)."""
    return f"s per parquet iteration (plain FP64, fdPA, {METRIC_LABEL.get(config, config)})"


WORKLOADS = {
    "siam_b10_nk3_16": "SIAM local fdPA: beta=10 U=1 Gamma=0.5 flat band nK1=64 nK2=(32,32) nK3=(16,16) nG=64 mPi=6, init_sym_grp",
    "hubbard8x8_b5_nk3_8x12": "Hubbard 8x8 NL fdPA: t=1 t'=0 mu=0 U=2 beta=5 nK1=32 nK2=(16,16) nK3=(8,12) nG=32 mPi=32, "
               "synthetic RefVertex, init_sym_grp",
    "hubbard16x16_n09_nk3_20x40": "Hubbard 16x16 NL fdPA: t=1 t'=-0.2 n=0.9 U=3 beta=10 nK1=80 nK2=(40,40) nK3=(20,40) nG=80 mPi=32, "
               "init_sym_grp",
    "hubbard4x4_n09_nk3_20x40": "Hubbard 4x4 NL fdPA with the 16x16 workload's boxes: t=1 t'=-0.2 n=0.9 U=3 beta=10 nK1=80 nK2=(40,40) "
                "nK3=(20,40) nG=80 mPi=32, init_sym_grp (profiling size)",
    "hubbard24x24_b8_nk3_24x48": "Hubbard 24x24 NL fdPA: t=1 t'=0 mu=0 U=2.5 beta=8 nK1=96 nK2=(48,48) nK3=(24,48) nG=96 mPi=32, "
               "init_sym_grp",
}
UNIT = "s/iteration"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 200 for siam_b10_nk3_16/hubbard8x8_b5_nk3_8x12, enough to span several clock samples; "
                         "fewer for the larger configurations)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="hubbard8x8_b5_nk3_8x12")
    ap.add_argument("--no-converge", action="store_true", help="skip the time-to-converge leg")
    ap.add_argument("--U", type=float, default=None, help="override the configuration's U (differentiation runs)")
    ap.add_argument("--restart", type=int, default=20, help="GMRES restart of the Newton solves (differentiation runs)")
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the oracle timing (for the large configurations, where one oracle iteration takes hours)")
    args = ap.parse_args()
    if args.steps is None:  # the whole default run stays within a few minutes
        if args.impl == "reference":
            args.steps = 5
        else:
            args.steps = {"siam_b10_nk3_16": 200, "hubbard8x8_b5_nk3_8x12": 200, "hubbard16x16_n09_nk3_20x40": 10, "siam_batch48": 10}.get(args.config, 3)
    return args


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier and max-over-ranks on the host (gloo); a no-op for one process."""

    def __init__(self, world):
        self.world = world
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, v):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def has_sample(self):
        try:
            return self.path is not None and os.path.getsize(self.path) > 0
        except OSError:
            return False

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_problem(cfg_name, impl):
    from fdgasolver.workloads import CONFIGS, make_solver
    cfg = dict(CONFIGS[cfg_name])
    if impl == "ours":
        return cfg, make_solver(cfg, True)
    return cfg, oracle_problem(cfg)


def oracle_problem(cfg):
    """The oracle solver of a workload dict (CPU baseline legs only)."""
    from fdgasolver.workloads import make_inputs
    from oracle import oracle as O
    Gb, G0, S0, rv = make_inputs(cfg)
    local = cfg["kind"] == "siam"
    s = O.OracleSolver(nG=cfg["nG"], nK1=cfg["nK1"], nK2=cfg["nK2"], nK3=cfg["nK3"], T=cfg["T"], U=cfg["U"],
                       L=1 if local else cfg["L"], local=local, mPi_factor=cfg["mPi_factor"], nR=rv.nR)
    for name, a in (("Gbare", Gb), ("G0", G0), ("Sigma0", S0)):
        s.set(name, a)
    for name, a in zip(["Fp_p", "Fp_x", "Ft_p", "Ft_x"], rv.arrays):
        s.set(name, a)
    s.finalize()
    s.init_sym_grp()
    return s


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


def flatten_blocks(cfg):
    """(name, start, stop) of the flatten(S) blocks: γp(K1,K2,K3), γt, γa, Σ."""
    local = cfg["kind"] == "siam"
    Nq = 1 if local else cfg["L"] ** 2
    n1 = (2 * cfg["nK1"] - 1) * Nq
    n2 = (2 * cfg["nK2"][0] - 1) * 2 * cfg["nK2"][1] * Nq
    n3 = (2 * cfg["nK3"][0] - 1) * (2 * cfg["nK3"][1]) ** 2 * Nq
    out, o = [], 0
    for ch in "pta":
        for nm, n in (("K1", n1), ("K2", n2), ("K3", n3)):
            out.append((f"{ch}.{nm}", o, o + n))
            o += n
    out.append(("Sigma", o, o + 2 * cfg["nG"] * Nq))
    return out


def profile_traffic(name):
    """DRAM bytes per launch of a kernel, from the committed ncu summary under profiles/ (or None)."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.strip().startswith("dram_bytes_per_launch"):
                return int(line.split("=")[1].split()[0].replace(",", ""))
    except (OSError, ValueError, IndexError):
        pass
    return None


def k3_gemm_roofline(S, stages, cfg_name):
    """Roofline of the fused K3 BSE GEMM (MODE 1): one complex Nν3 x Nν3 x Nν3 product per (channel,
    representative (P, Ω) block); complex MAC = 8 real flops.  On the FP64 CUDA-core kernel
    (k_bse_K3_gemm) the FP64 pipe bounds it; on the digit-sliced tensor-core kernel (k_bse_K3_oz,
    the default from Nν3 = 32 on) the BF16 MMAs it issues are compared with the measured bf16 peak
    and its FP64-equivalent rate with the FP64 pipe."""
    nb, N = S.query("k3_blocks"), S.query("k3_block_dim")
    ms = stages["bse_K3_gemm"]
    flops = 3 * nb * 8 * N ** 3
    byts = 16 * nb * N * N * 16  # A, B0, Γ, FL (two for t) and the output, per channel: 16 N² complex
    fp64_peak = S.query("fp64_gflops") / 1e3
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs", 6800.0)
    achieved = flops / (ms * 1e-3) / 1e12
    if S.query("k3_fp64_tensor_cores") == 1:
        # 36 BF16 MMAs (M = 128 rows, K = 16) per K chunk over all 2N real columns and 2N real K
        mma_flops = 3 * nb * 36 * 2 * 128 * (2 * N) * (2 * N)
        bf16 = peaks.get("bf16_tflops", 1900.0)
        tc = mma_flops / (ms * 1e-3) / 1e12
        return {"bound": "tensor", "kernel": "k_bse_K3_oz<1> (fused K3 BSE, FP64 by digit slicing on tcgen05)",
                "achieved": tc, "peak": bf16, "unit": "TFLOP/s", "frac": tc / bf16,
                "peak_source": "fallback" if peaks.get("fallback") else "measured (bf16_tflops)",
                "flops_per_launch": mma_flops, "fp64_equivalent_tflops": achieved, "fp64_pipe_peak": fp64_peak,
                "fp64_equivalent_frac": achieved / fp64_peak,
                "traffic": profile_traffic(f"k_bse_K3_oz_{cfg_name}.md"), "algorithmic_bytes": byts,
                "hbm_achieved_gbs": byts / (ms * 1e-3) / 1e9, "hbm_peak_gbs": hbm,
                "hbm_frac": byts / (ms * 1e-3) / 1e9 / hbm, "launch_ms": ms,
                "share_of_iteration": ms / sum(stages.values()),
                "stage_ms": {k: round(v, 4) for k, v in stages.items()}}
    traffic = profile_traffic(f"k_bse_K3_gemm_{cfg_name}.md")
    tile = 16 if N <= 16 else (24 if N <= 24 else 32)
    return {"bound": "fp64", "kernel": f"k_bse_K3_gemm<1,{tile},cplx> (fused K3 BSE, FP64)", "achieved": achieved,
            "peak": fp64_peak, "unit": "TFLOP/s", "frac": achieved / fp64_peak,
            "peak_source": "measured: the library's FP64 FMA calibration kernel on this GPU (fdga_query fp64_gflops)",
            "traffic": traffic, "algorithmic_bytes": byts, "hbm_achieved_gbs": byts / (ms * 1e-3) / 1e9,
            "hbm_peak_gbs": hbm, "hbm_frac": byts / (ms * 1e-3) / 1e9 / hbm,
            "hbm_peak_source": "fallback" if peaks.get("fallback") else "measured",
            "launch_ms": ms, "flops_per_launch": flops, "share_of_iteration": ms / sum(stages.values()),
            "stage_ms": {k: round(v, 4) for k, v in stages.items()}}


def precision_report(cfg, S, x):
    """Mixed map vs FP64 map at the same state: max relative error per flatten block and of χ."""
    import numpy as np
    y64 = S.fixed_point(x) + x
    U = cfg["U"]
    S.set_precision("mixed")
    y32 = S.fixed_point(x) + x
    S.set_precision("fp64")
    rep = {}
    for name, a, b in flatten_blocks(cfg):
        ref = np.abs(y64[a:b]).max()
        rep[name] = float(np.abs(y32[a:b] - y64[a:b]).max() / ref) if ref > 0 else 0.0
    blk = {n: (a, b) for n, a, b in flatten_blocks(cfg)}
    k1 = {c: (y64[slice(*blk[f"{c}.K1"])], y32[slice(*blk[f"{c}.K1"])]) for c in "ta"}
    for ch, f in (("chi_m", lambda a, t: a / U ** 2), ("chi_d", lambda a, t: (a - 2 * t) / U ** 2)):
        r64, r32 = f(k1["a"][0], k1["t"][0]), f(k1["a"][1], k1["t"][1])
        rep[ch] = float(np.abs(r32 - r64).max() / np.abs(r64).max())
    return rep


def run_ours(args, rank, world, dist):
    import numpy as np
    from fdgasolver.solver import PinnedBuffer
    cfg, S = build_problem(args.config, "ours")
    rng = np.random.default_rng(1)
    # a representative state: a few damped iterations from the PA start
    x = S.flatten()
    for _ in range(3):
        x = x + 0.5 * S.fixed_point(x)
    x = x + 1e-3 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))
    S.unflatten(x)
    for _ in range(max(args.warmup, 3)):
        S.map_repeat(1)
    S.synchronize()
    launches = S.launches_per_iteration()
    # ---- device-resident timed region ----
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    # keep the GPU loaded (untimed iterations) until the sampler's first line, so that every clock
    # sample is taken under load (nvidia-smi needs a few hundred ms to start)
    t_wait = time.perf_counter()
    while clocks.proc and not clocks.has_sample() and time.perf_counter() - t_wait < 3.0:
        S.map_repeat(20)
        S.synchronize()
    dist.barrier()
    S.synchronize()
    ms_dev = 0.0
    for _ in range(args.steps):
        S.flush_l2(256 << 20)  # 256 MB write: L2 (129 MB) holds nothing of the previous iteration
        S.event_record(0)
        S.map_repeat(1)
        S.event_record(1)
        ms_dev += S.event_elapsed_ms(0, 1)
    S.synchronize()
    dist.barrier()
    ms_dev /= args.steps
    # ---- e2e through the C ABI with pinned host buffers ----
    xb, Rb = PinnedBuffer(S.state_len), PinnedBuffer(S.state_len)
    xb.array[:] = x
    for _ in range(max(args.warmup, 3)):
        S.fixed_point_ptr(xb.ptr, Rb.ptr)
    dist.barrier()
    t_e2e = 0.0
    for _ in range(args.steps):
        S.flush_l2(256 << 20)  # as for `value`: no intermediate of the previous step stays in L2
        S.synchronize()
        t0 = time.perf_counter()
        S.fixed_point_ptr(xb.ptr, Rb.ptr)
        t_e2e += time.perf_counter() - t0
    t_e2e /= args.steps
    # kernels launched in the two timed regions: the iteration graph's per device-resident step, the
    # fused residual graph's per e2e step (the L2 flushes are memsets, outside the timed spans)
    e2e_launches = S.launches_per_iteration()
    gpu_launches = args.steps * launches + args.steps * e2e_launches
    dist.barrier()
    clk = clocks.stop()
    xb.free()
    Rb.free()
    ms_dev = dist.max(ms_dev)
    t_e2e = dist.max(t_e2e)
    # ---- per-stage device times (eager run, CUDA events between stages) ----
    S.unflatten(x)
    stages = S.stage_times("fdPA", nrep=3)
    roofline = k3_gemm_roofline(S, stages, args.config)
    precision = precision_report(cfg, S, x)
    # ---- time to converge at max|R| < 1e-8 (Anderson with the reference's solve! defaults δ=0.85, m=8) ----
    conv = None
    if not args.no_converge:
        conv = {}
        res = {}
        for mode in ("plain", "mixed", "newton", "newton_mixed", "newton_mixed_differences"):
            cfg2, S2 = build_problem(args.config, "ours")
            x0 = S2.flatten()
            S2.iterate_solver("fdPA")  # captures the iteration graphs outside the timed solves
            S2.set_precision("mixed"); S2.iterate_solver("fdPA"); S2.set_precision("fp64")
            S2.unflatten(x0)
            S2.synchronize()
            t0 = time.perf_counter()
            if mode == "plain":
                r = S2.solve("fdPA", maxiter=300, tol=1e-8, delta=0.85, mem=8)
                info = {"iterations": r["iterations"],
                        "method": "Anderson m=8, beta=0.85 (NLsolve restated, device-resident QR), FP64 map"}
            elif mode.startswith("newton"):
                jvp = "fp64" if mode == "newton" else "mixed"
                tangent = 0 if mode.endswith("differences") else 1
                S2.set_option("jvp_tangent", tangent)
                r = S2.solve_newton("fdPA", maxiter=600, tol=1e-8, restart=30, jvp=jvp)
                how = ("the hand-written tangent kernels (fdga_frule) of the " if tangent else
                       "forward differences of the ")
                info = {"newton_steps": r["newton"], "fp64_maps": r["evals_fp64"],
                        "mixed_maps_or_tangents": r["evals_mixed"],
                        "method": f"Newton-Krylov: GMRES(30) on (I-J)dx = R with JVPs from {how}{jvp} map, "
                                  f"Eisenstat-Walker forcing, backtracking on the FP64 residual"}
            else:
                r = S2.solve_mixed("fdPA", maxiter=600, tol=1e-8, delta=0.85, mem=8)
                info = {"fp64_maps": r["evals_fp64"], "mixed_maps": r["evals_mixed"],
                        "method": "iterative refinement: FP64 residual outside, Anderson m=8 beta=0.85 with FP32 "
                                  "history on the mixed map (FP32 K3 contractions) inside; FP64 Anderson phase "
                                  "once the mixed map's rounding floor is reached"}
            t = time.perf_counter() - t0
            conv[mode] = {"seconds": dist.max(t), "converged": r["converged"], "final_residual": r["residual"], **info}
            res[mode] = {c: S2.susceptibility(c) for c in ("m", "d")}
            res[mode]["Sigma"] = S2.get("Sigma")
            S2.close()
        import numpy as np
        for mode in ("mixed", "newton", "newton_mixed", "newton_mixed_differences"):
            conv[f"speedup_{mode}_vs_plain"] = conv["plain"]["seconds"] / conv[mode]["seconds"]
            conv[f"{mode}_vs_plain_solution_rel_err"] = {
                k: float(np.abs(res[mode][k] - res["plain"][k]).max() / np.abs(res["plain"][k]).max())
                for k in ("m", "d", "Sigma")}
        # linear response at the fixed point: dχ_m/dU(Ω = 0, q = (π, π)) through GMRES on (I − J)
        cfg2, S2 = build_problem(args.config, "ours")
        S2.solve_newton("fdPA", maxiter=600, tol=1e-12, restart=30, jvp="fp64")
        t0 = time.perf_counter()
        d, info = S2.dchi_dU("m", hU=1e-4, restart=40, cycles=4, rtol=1e-8)
        t = time.perf_counter() - t0
        nO = 2 * cfg2["nK1"] - 1
        L = cfg2.get("L", 1)
        iq = (L // 2 + L * (L // 2)) if cfg2["kind"] != "siam" else 0
        v = d[iq * nO + cfg2["nK1"] - 1]
        conv["dchi_m_dU"] = {"value_Omega0_q_pipi": [v.real, v.imag], "seconds": t, **info,
                             "method": "GMRES(40) on (I-J) dx/dU = dPhi/dU at the converged state, JVPs by the "
                                       "tangent kernels, dPhi/dU by central differences (h = 1e-4)"}
        S2.close()
    # ---- derivatives of one iteration at this workload: tangent (frule) and adjoint (rrule) ----
    diff = derivative_report(S, x)
    nstate = S.state_len
    out = {
        "metric": metric_for(args.config), "value": ms_dev * 1e-3, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_dev, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128 (FP64 complex)", "data": "synthetic (seeded; reference inputs restated)",
        "config": {"workload": WORKLOADS.get(args.config, args.config),
                   "name": args.config, "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "L2 flushed (256 MB device write) before every timed iteration; flush not timed"},
        "e2e": {"value": t_e2e, "unit": UNIT, "h2d_bytes_per_step": nstate * 16, "d2h_bytes_per_step": nstate * 16},
        "gpu_launches": gpu_launches,
        "launches_per_iteration": launches,
        "e2e_launches_per_call": e2e_launches,
        "time_to_converge": conv,
        "roofline": roofline,
        "precision_mixed_map_vs_fp64": precision,
        "derivatives": diff,
        "clocks": clk,
    }
    S.close()
    return out


def derivative_report(S, x):
    """Tangent (fdga_frule) and adjoint (fdga_rrule) of one iteration at x: device time per application
    of the tangent map (CUDA graph replays) next to the map, the transpose identity <ȳ, J v> = <Jᵀ ȳ, v>,
    and the tangent against central differences of the FP64 map."""
    import numpy as np
    rng = np.random.default_rng(3)
    v = rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size)
    yb = rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size)
    out = {}
    for prec in ("fp64", "mixed"):
        S.set_precision(prec)
        S.unflatten(x)
        _, jv = S.frule(v)
        S.synchronize()
        ms = {}
        for what, f in (("map", S.map_repeat), ("tangent", S.tangent_repeat)):
            f(3)
            S.synchronize()
            S.event_record(0)
            f(20)
            S.event_record(1)
            S.synchronize()
            ms[what] = S.event_elapsed_ms(0, 1) / 20
        out[f"{prec}_ms"] = ms
        if prec == "fp64":
            j64 = jv
        else:
            out["mixed_tangent_rel_err_vs_fp64"] = float(np.abs(jv - j64).max() / np.abs(j64).max())
    S.set_precision("fp64")
    h = 1e-6 * max(1.0, float(np.abs(x).max()))
    d = (S.fixed_point(x + h * v) - S.fixed_point(x - h * v)) / (2 * h) + v
    out["tangent_vs_central_difference_rel"] = float(np.abs(j64 - d).max() / np.abs(d).max())
    S.unflatten(x)
    if x.size > 50_000_000:  # the adjoint's cotangent buffers would not fit beside the state
        out["adjoint"] = "skipped: its buffers (about 9 state-sized K3 arrays) exceed the HBM left at this size"
        return out
    t0 = time.perf_counter()
    _, xb = S.rrule(yb)
    out["adjoint_host_ms_incl_value_pass_and_copies"] = (time.perf_counter() - t0) * 1e3
    lhs, rhs = float(np.real(np.vdot(yb, j64))), float(np.real(np.vdot(xb, v)))
    out["transpose_identity_rel"] = abs(lhs - rhs) / (np.linalg.norm(yb) * np.linalg.norm(j64))
    S.unflatten(x)
    return out


def run_batch(args, rank, world, dist):
    """Config 4: 48 SIAM instances iterated together, one CUDA graph launch per batch iteration."""
    import numpy as np
    from fdgasolver.solver import Batch
    from fdgasolver.workloads import batch_instances, make_solver
    inst = batch_instances(48)
    solvers = [make_solver(c, True) for c in inst]
    tiles = {}
    for S, c in zip(solvers, inst):
        tiles[str(c["nK3"][1])] = S.autotune()
    for S in solvers:  # a populated state: one damped step from the PA start
        x = S.flatten()
        S.unflatten(x + 0.5 * S.fixed_point(x))
    xs = [S.flatten() for S in solvers]
    batch = Batch(solvers)
    for _ in range(max(args.warmup, 3)):
        batch.iterate("fdPA", "fp64")
    batch.synchronize()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    ms64, kernels = batch.time(args.steps, "fdPA", "fp64")
    ms32, _ = batch.time(args.steps, "fdPA", "mixed")
    clk = clocks.stop()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for S in solvers:
            S.iterate_solver("fdPA")  # one graph launch and one stream synchronisation per instance
    t_seq = (time.perf_counter() - t0) / args.steps
    for S in solvers:
        S.set_precision("mixed")
        S.iterate_solver("fdPA")
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for S in solvers:
            S.iterate_solver("fdPA")
    t_seq32 = (time.perf_counter() - t0) / args.steps
    for S in solvers:
        S.set_precision("fp64")
    # the FP64 K3 GEMM work of all members (2 GEMMs x 3 channels x representative blocks x N^3
    # complex products, 3 real FMAs = 6 flops each in the CUDA-core kernel's 3M form) at the measured
    # FP64 FMA rate: the floor of a batch iteration whose K3 GEMMs run on the FP64 pipe; members with
    # Nν3 ≥ 32 run them on the tensor cores instead (digit slicing), which this floor does not bound
    from fdgasolver.solver import _lib_query
    fp64_rate = _lib_query("fp64_gflops") * 1e9
    gemm_flops = sum(6.0 * S.query("k3_blocks") * 6.0 * S.query("k3_block_dim") ** 3 for S in solvers)
    tc_members = sum(int(S.query("k3_fp64_tensor_cores")) for S in solvers)
    errs = []
    for S, x in zip(solvers, xs):
        y64 = S.fixed_point(x) + x
        S.set_precision("mixed")
        y32 = S.fixed_point(x) + x
        S.set_precision("fp64")
        errs.append(float(np.abs(y32 - y64).max() / np.abs(y64).max()))
    batch.close()
    for S in solvers:
        S.close()
    t64 = ms64 / args.steps * 1e-3
    return {
        "metric": "s per batch iteration (48 SIAM instances, one iterate_solver! each)", "value": t64,
        "unit": "s/batch-iteration", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t64 * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 (FP64 complex)", "data": "synthetic (seeded instance parameters)",
        "config": {"workload": "48 SIAM local fdPA instances: U~U[0.5,3], beta in {5,10,20,40}, Gamma~U[0.3,1], "
                               "nK3=(nu/2,nu), nu=16/32/48/64 by beta, nK2=(nu,nu), nK1=nG=2nu, mPi=6",
                   "name": "siam_batch48", "parallelism": "single GPU, one graph with 48 branches"},
        "mixed_s_per_batch_iteration": ms32 / args.steps * 1e-3,
        "sequential_s_per_round": t_seq,
        "speedup_batch_vs_sequential": t_seq / t64,
        "sequential_mixed_s_per_round": t_seq32,
        "speedup_mixed_batch_vs_sequential": t_seq32 / (ms32 / args.steps * 1e-3),
        "fp64_k3_gemm_cuda_core_floor_s": gemm_flops / fp64_rate,
        "members_with_tensor_core_fp64_k3": tc_members,
        "kernels_per_batch_iteration": kernels, "gpu_launches": kernels * args.steps,
        "autotuned_k3_tiles_by_nu": tiles,
        "mixed_map_rel_err": {"max": max(errs), "median": float(np.median(errs))},
        "clocks": clk,
    }


def run_differentiation(args, rank, world, dist):
    """Config 5: Newton–Krylov solve to the FP64 fixed point, then dχ_m(Ω=0, q=(π,π))/dU by the linear
    response (GMRES on (I − J) dx/dU = ∂Φ/∂U), checked against central differences h = 1e-4 of
    the converged χ_m at U ± h (same solver, re-solved from the fixed point)."""
    import numpy as np
    from fdgasolver.workloads import CONFIGS, make_solver
    cfg = dict(CONFIGS[args.config])
    if args.U is not None:
        cfg["U"] = args.U
    S = make_solver(cfg, True)
    nO, L = 2 * cfg["nK1"] - 1, cfg["L"]
    iq = L // 2 + L * (L // 2)
    k0 = iq * nO + cfg["nK1"] - 1
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    t0 = time.perf_counter()
    r = S.solve_newton("fdPA", maxiter=400, tol=1e-10, restart=args.restart, jvp="mixed")
    t_solve = time.perf_counter() - t0
    t0 = time.perf_counter()
    d, info = S.dchi_dU("m", hU=1e-4, restart=30, cycles=3, rtol=1e-7)
    t_lr = time.perf_counter() - t0
    clk = clocks.stop()
    U, h = cfg["U"], 1e-4
    chi = {}
    for sgn in (+1, -1):
        S.set_U(U + sgn * h)
        rs = S.solve_newton("fdPA", maxiter=400, tol=1e-11, restart=args.restart, jvp="fp64")
        chi[sgn] = S.susceptibility("m")
        S.set_U(U)
    fd = (chi[+1] - chi[-1]) / (2 * h)
    S.close()
    return {
        "metric": "dchi_m(Omega=0,q=(pi,pi))/dU by linear response (Hubbard 24x24 NL fdPA)",
        "value": t_lr, "unit": "s (linear response at the fixed point)", "n_gpus": world, "steps": 1, "warmup": 0,
        "ms_per_step": t_lr * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 (FP64 complex)", "data": "synthetic (model inputs restated)",
        "config": {"workload": WORKLOADS["hubbard24x24_b8_nk3_24x48"] + ("" if args.U is None else f" (U overridden: {args.U})"),
                   "name": "hubbard24x24_b8_nk3_24x48", "parallelism": "single GPU", "U": cfg["U"], "gmres_restart": args.restart},
        "solve": {"seconds": t_solve, "converged": r["converged"], "residual": r["residual"],
                  "newton_steps": r["newton"], "fp64_maps": r["evals_fp64"], "mixed_maps": r["evals_mixed"]},
        "dchi_m_dU": {"value": [d[k0].real, d[k0].imag], **info},
        "central_difference_check": {"value": [fd[k0].real, fd[k0].imag],
                                     "rel_diff_at_point": float(abs(d[k0] - fd[k0]) / abs(fd[k0])),
                                     "rel_diff_max_all_Omega_q": float(np.abs(d - fd).max() / np.abs(fd).max()),
                                     "last_fd_solve_converged": rs["converged"]},
        "clocks": clk,
    }


def run_mfrg(args, rank, world, dist):
    """The mfRG / Krylov-preconditioned solver (src/mfRG.jl) on the config-2 lattice and boxes as an
    fdDΓA problem: the reference system's G0 is the bare G at μ = +0.25 (Π0 ≠ 0), F0 the bare U
    (the map is then linear), Σ0 = 0.  Reports the time of one mfRG map application on the device
    (graph replays inside a GMRES solve, per application), the preconditioned Anderson solve
    (nlsolve m = 50, β = 0.85, Krylov rtol = atol = 1e-6, the reference's settings) against the plain
    FP64 Anderson solve to the same tolerance, and the oracle's map on the host cores."""
    import numpy as np
    from fdgasolver.models import hubbard_bare_Green
    from fdgasolver.workloads import CONFIGS, make_solver
    cfg = dict(CONFIGS["hubbard8x8_b5_nk3_8x12"])
    cfg.pop("refvertex_noise", None)
    if args.U is not None:
        cfg["U"] = args.U
    cfg["G0"] = hubbard_bare_Green(cfg["T"], cfg["nG"], cfg["L"], mu=0.25, t1=cfg["t1"], t2=cfg.get("t2", 0.0))
    S = make_solver(cfg, True)
    x0 = S.flatten()
    nF = x0.size - 2 * cfg["nG"] * cfg["L"] ** 2
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    S.synchronize()
    t0 = time.perf_counter()
    rp = S.solve("fdPA", maxiter=600, tol=1e-8, delta=0.85, mem=8)
    t_plain = time.perf_counter() - t0
    xp = S.flatten()
    S.unflatten(x0)
    S.solve_mfrg("fdPA", maxiter=1, tol=1e-8, delta=0.85, mem=50, update_sigma=True)  # capture the graphs
    S.unflatten(x0)
    S.synchronize()
    t0 = time.perf_counter()
    rm = S.solve_mfrg("fdPA", maxiter=40, tol=1e-8, delta=0.85, mem=50, update_sigma=True, krylov_maxiter=400)
    t_mfrg = time.perf_counter() - t0
    xm = S.flatten()
    # one preconditioned residual: its Krylov iterations give the per-application cost
    S.unflatten(xp + 1e-3 * (x0 - xp))
    S.synchronize()
    t0 = time.perf_counter()
    _, info = S.fixed_point_preconditioned(xp + 1e-3 * (x0 - xp), "fdPA", update_sigma=True, krylov_maxiter=400,
                                           krylov_rtol=1e-6, krylov_atol=1e-6)
    t_res = time.perf_counter() - t0
    clk = clocks.stop()
    S.close()
    # the oracle's map on the host cores (bounded sample)
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    orc = oracle_problem(cfg)
    v = xp[:nF]
    orc.mfrg_apply(v)
    t0 = time.perf_counter()
    orc.mfrg_apply(v)
    t_orc = time.perf_counter() - t0
    rel = float(np.abs(xm - xp).max() / np.abs(xp).max())
    return {
        "metric": "time to converge to max|R| < 1e-8, mfRG-preconditioned Anderson (Hubbard 8x8 fdDGA, G0 != 0)",
        "value": t_mfrg, "unit": "s", "n_gpus": world, "steps": 1, "warmup": 1, "ms_per_step": t_mfrg * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "c128 (FP64 complex)",
        "data": "synthetic (model inputs restated)",
        "config": {"workload": "Hubbard 8x8 NL fdDGA: config-2 lattice and boxes, reference system G0 = bare G at "
                               f"mu=0.25, Sigma0 = 0, F0 = bare U (U={cfg['U']}), init_sym_grp", "name": "hubbard8x8_b5_mfrg",
                   "parallelism": "single GPU"},
        "mfrg": {"seconds": t_mfrg, "converged": rm["converged"], "outer_iterations": rm["iterations"],
                 "krylov_iterations": rm["krylov_iterations"], "residual": rm["residual"]},
        "plain": {"seconds": t_plain, "converged": rp["converged"], "iterations": rp["iterations"],
                  "residual": rp["residual"]},
        "speedup_mfrg_vs_plain": t_plain / t_mfrg,
        "mfrg_vs_plain_solution_rel_err": rel,
        "preconditioned_residual": {"seconds": t_res, "krylov_iterations": info["krylov_iterations"],
                                    "krylov_residual": info["krylov_residual"],
                                    "ms_per_krylov_iteration": t_res * 1e3 / max(info["krylov_iterations"], 1)},
        "cpu_baseline": {"value": t_orc, "unit": "s per mfRG map application", "cores": threads, "kind": "port",
                         "sample": "1 application of the oracle's mfRG map after 1 warm-up (C++ restatement, OpenMP)"},
        "clocks": clk,
    }


def run_reference(args, rank, world):
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    cfg, S = build_problem(args.config, "reference")
    x = S.flatten()
    for _ in range(args.warmup):
        S.residual(x)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        S.residual(x)
    dt = (time.perf_counter() - t0) / args.steps
    return {
        "impl": "reference", "metric": metric_for(args.config), "value": dt, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128 (FP64 complex)", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOADS.get(args.config, args.config), "name": args.config,
                   "parallelism": "host cores (OpenMP), rank 0 only"},
        "cpu_baseline": {"value": dt, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full iterations of the workload (C++ restatement of the reference "
                                   f"algorithm; Julia reference not runnable here)"},
        "e2e": {"value": dt, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def cpu_baseline_sample(args):
    """Oracle timed on the host cores for one iteration of the same workload (bounded sample)."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    cfg, S = build_problem(args.config, "reference")
    x = S.flatten()
    S.residual(x)
    t0 = time.perf_counter()
    S.residual(x)
    dt = time.perf_counter() - t0
    return {"value": dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "1 iteration of the workload after 1 warm-up (C++ restatement, OpenMP)"}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args, rank, 1)))
        return 0
    if world > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    dist = Dist(world)
    if args.config in ("siam_batch48", "hubbard24x24_b8_newton", "hubbard8x8_b5_mfrg"):
        if args.config == "hubbard8x8_b5_mfrg":
            out = run_mfrg(args, rank, world, dist)
        elif args.config == "hubbard24x24_b8_newton":
            args.config = "hubbard24x24_b8_nk3_24x48"
            out = run_differentiation(args, rank, world, dist)
        else:
            out = run_batch(args, rank, world, dist)
        if rank == 0:
            print(json.dumps(out))
        return 0
    out = run_ours(args, rank, world, dist)
    if rank == 0:
        out["cpu_baseline"] = None if args.no_cpu_baseline else cpu_baseline_sample(args)
        print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
