"""Benchmark of the matrix-free Hubbard H|psi> on one GB300 (or N replicas).

Workload (N=1 line): 2D square-lattice Hubbard 4x4 periodic, t=1, U=8,
N_up = N_down = 6 -- 64,128,064 states, 16-byte complex elements (1.026 GB
per vector).  A step is one H|psi> over the whole sector on device-resident
block-floating-point vectors (int64 mantissas, one exponent per vector: the
engine's FP64-class format; plain FP64 arithmetic runs at 1/57 of the FP32
rate on this GPU and is reported beside it in `extras`).  `value` is the algorithmic
bandwidth 2 * 16 B * dim / (device time per apply); `e2e` is the same metric
through the reference-facing C-ABI call with complex128 host buffers in
reference order (mb_op_apply_host: x read over the host link and scattered to
tensor order, FP64->Q64 conversion, the apply in row groups, each finished
reference-order prefix converted back and copied to the host while later
groups run).

Inputs (1 GB each) are larger than the 129 MB L2, so no flush is needed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference's CPU path for the same metric: its
compute_matrix_elements matrix applied by a serial CSC column scatter (the
reference builds Armadillo with ARMA_OPENMP_THREADS=1), restated in the CPU
oracle because Armadillo is absent; run on a bounded sample (a smaller sector
of the same lattice) so the run ends in minutes.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0
# Sectors a run can use; the default is the 4x4, 6+6 workload of the N=1 line.
# The smaller ones serve profiling captures (inputs still larger than L2).
CASES = {
    "4x4_6+6": dict(workload="hubbard2d_4x4_n6+6_u8_apply", lattice=(4, 4), n_up=6, n_down=6,
                    t=1.0, U=8.0),
    "4x4_5+5": dict(workload="hubbard2d_4x4_n5+5_u8_apply", lattice=(4, 4), n_up=5, n_down=5,
                    t=1.0, U=8.0),
    "1d16_8+8": dict(workload="hubbard1d_L16_n8+8_u4_apply", lattice=(16,), n_up=8, n_down=8,
                     t=1.0, U=4.0),
}
METRIC = "hubbard_hpsi_GBps"


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return HBM_FALLBACK_GBS, "fallback"


FP64_NOMINAL_TFLOPS = 1.25  # GB300 dense FP64, nominal


def mean_hops(lattice, n_up: int, n_down: int) -> float:
    """Mean number of hops (both spins) of a state of the sector: a bond with
    exactly one end occupied gives one hop, so per spin the mean is
    B * 2 n (N - n) / (N (N - 1)) for B bonds (a size-2 side's doubled bond
    counts twice, a size-1 side's self bond none) on N sites."""
    N = 1
    for d in lattice:
        N *= d
    B = sum(N for d in lattice if d >= 2)
    if N < 2:
        return 0.0
    return sum(B * 2.0 * n * (N - n) / (N * (N - 1)) for n in (n_up, n_down))


def committed_traffic(kernel_key: str):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        v = d.get(kernel_key)
        if isinstance(v, dict):
            return v.get("dram_bytes_per_launch")
    return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(value: float, dist=None) -> float:
    """MAX of a per-rank float over the process group (NCCL or gloo)."""
    if dist is None or not dist.is_initialized():
        return value
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(bytes_per_step: float, steps: int, world: int, max_ms: float) -> float:
    """Whole-job GB/s of N independent replicas: all ranks' bytes over the slowest rank's time."""
    return world * bytes_per_step * steps / (max_ms * 1e-3) / 1e9


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def time_loop(torch, stream, fn, steps, warmup):
    """CUDA-event time of `steps` calls (after `warmup`); returns (total_ms, per-call ms list)."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for i in range(steps):
        ev[i][0].record(stream)
        fn()
        ev[i][1].record(stream)
    t1.record(stream)
    torch.cuda.synchronize()
    return t0.elapsed_time(t1), [a.elapsed_time(b) for a, b in ev]


def run_gpu(args):
    import torch

    import manybody_gb300 as mb

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        pg = dist

    def barrier():
        if pg:
            pg.barrier()

    w = dict(CASES[args.case])
    L = 1
    for d in w["lattice"]:
        L *= d
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(L, w["n_up"] + w["n_down"],
                                                                w["n_up"] - w["n_down"])
    model = mb._Hubbard(w["t"], w["U"], w["lattice"])
    opq = mb.GpuHubbardOperator(basis, model, mb.PREC_Q64)
    dim = opq.dimension()
    # the apply's kernel shape from the project's autotuner (every candidate
    # timed on this GPU; all give the same bits)
    apply_shape, _ = opq.autotune()
    w.update(dim=dim, lattice="x".join(str(d) for d in w["lattice"]), order="tensor",
             apply_shape=apply_shape,
             vector="16-byte complex elements (int64 mantissa pairs)",
             l2=f"inputs ({16 * dim / 1e9:.2f} GB) larger than L2 (129 MB); no flush")
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    alg_bytes = 2 * 16 * dim

    # --- headline: H|psi> on device-resident Q64 vectors (tensor order) --------
    x = opq.seed_vector(0, order=mb.ORDER_TENSOR)
    xq, ex = opq.q64_from_f64(x, order=mb.ORDER_TENSOR)
    del x
    yq = opq.q64_empty()

    def step():
        opq.apply_q64(xq, ex, out=yq, stream=sp)

    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        total_ms, per = time_loop(torch, stream, step, args.steps, args.warmup)
        barrier()
    total_ms = max_over_ranks(total_ms, pg)
    ms_per_step = total_ms / args.steps
    value = replica_throughput(alg_bytes, args.steps, world, total_ms)
    kernel_ms = statistics.mean(per)
    achieved = alg_bytes / (kernel_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    del yq, xq
    torch.cuda.empty_cache()
    if args.only_apply:
        if rank == 0:
            print(json.dumps({"case": args.case, "ms_per_apply": round(kernel_ms, 5),
                              "GBps": round(achieved, 2), "frac": round(achieved / peak, 4)}))
        if pg:
            pg.destroy_process_group()
        return

    # --- end to end: reference-order host buffers through the C ABI ------------
    xh = torch.empty(dim, dtype=torch.complex128).pin_memory()
    yh = torch.empty(dim, dtype=torch.complex128).pin_memory()
    xh.copy_(opq.seed_vector(0).cpu())
    for _ in range(max(1, args.warmup // 2)):
        opq.apply_host(xh, yh)
    e2e_steps = max(2, min(args.steps, 10))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        opq.apply_host(xh, yh)
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, pg)
    e2e_value = world * alg_bytes / e2e_s / 1e9
    del xh, yh
    del opq
    torch.cuda.empty_cache()

    # --- the same operator in plain FP64 and in FP32 (context, not headline) --
    extras = {}
    for name, prec, nbytes in (("f64_fp64_pipe", mb.PREC_F64, 16), ("c64_fp32", mb.PREC_F32, 8)):
        op = mb.GpuHubbardOperator(basis, model, prec)
        shape, _ = op.autotune()
        xv = op.seed_vector(0, order=mb.ORDER_TENSOR)
        yv = op.empty()
        n_steps = 3 if prec == mb.PREC_F64 else max(5, args.steps // 2)
        tot, pr = time_loop(torch, stream, lambda: op.apply(xv, out=yv, order=mb.ORDER_TENSOR,
                                                             stream=sp), n_steps, 2)
        ms = statistics.mean(pr)
        gbs = 2 * nbytes * dim / (ms * 1e-3) / 1e9
        extras[name] = {"ms_per_apply": round(ms, 4), "GBps": round(gbs, 2),
                        "frac_of_hbm": round(gbs / peak, 4), "apply_shape": shape}
        if prec == mb.PREC_F64:
            # the FP64 ALU roofline: ~(2 hops + 6) real FP64 operations an element,
            # against the nominal 1.25 TFLOP/s of this part (no measured FP64 peak)
            cw = CASES[args.case]
            flops = (2.0 * mean_hops(cw["lattice"], cw["n_up"], cw["n_down"]) + 6.0) * dim
            tf = flops / (ms * 1e-3) / 1e12
            extras[name]["fp64_roofline"] = {
                "flops_per_element": round(flops / dim, 2), "achieved_tflops": round(tf, 4),
                "nominal_peak_tflops": FP64_NOMINAL_TFLOPS,
                "frac_of_nominal": round(tf / FP64_NOMINAL_TFLOPS, 4)}
        del op, xv, yv
        torch.cuda.empty_cache()

    if not args.no_extras:
        runs = [("cfg2_solve", run_cfg2_extra)]
        if not args.skip_cfg2_reorth:  # about a minute
            runs.append(("cfg2_reorth", run_cfg2_reorth_extra))
        for name, fn in (*runs, ("momentum", run_momentum_extra),
                         ("batch", run_batch_extra),
                         ("precision", run_precision_extra), ("serve", run_serve_extra)):
            try:
                extras[name] = fn(mb, torch)
            except Exception as exc:  # reported, never hidden
                extras[name] = {"error": f"{type(exc).__name__}: {exc}"}
            torch.cuda.empty_cache()

    if rank != 0:
        if pg:
            pg.destroy_process_group()
        return
    clocks = clk.summary()
    out = {
        "metric": METRIC,
        "value": round(value, 2),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int64",
        "data": "synthetic: Philox4x32-10 seed-0 uniform(-1,1) complex start vector",
        "config": dict(w, parallelism=f"replicas{world}" if world > 1 else "single_gpu",
                       vector_format="block floating point: int64 mantissas (re, im), one "
                                     "exponent per vector; FP64-class (>=56-bit) accuracy"),
        "roofline": {
            "bound": "hbm",
            "achieved": round(achieved, 2),
            "peak": peak,
            "unit": "GB/s",
            "frac": round(achieved / peak, 4),
            "traffic": committed_traffic("hubbard2d_4x4_q64_apply"),
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "kernel": "k_apply_q",
            "algorithmic_bytes_per_launch": alg_bytes,
            "kernel_ms": round(kernel_ms, 5),
        },
        "e2e": {
            "value": round(e2e_value, 2),
            "unit": "GB/s",
            "h2d_bytes_per_step": 16 * dim,
            "d2h_bytes_per_step": 16 * dim,
            "call": "mb_op_apply_host(order=reference) on complex128 host buffers",
            "ms_per_step": round(e2e_s * 1e3, 3),
        },
        "gpu_launches": args.steps,
        "clocks": clocks,
        "extras": extras,
    }
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    print(json.dumps(out), flush=True)
    if pg:
        pg.destroy_process_group()


# ---------------------------------------------------------------------------
# Other workloads (reported in `extras`): batching, precision, serving.
# ---------------------------------------------------------------------------
def philox_rng(seed):
    import numpy as np
    return np.random.Generator(np.random.Philox(key=seed))


def batch_sectors(n=512, seed=2024):
    """512 1D periodic sectors: L uniform in {8,10,12}, N_up=N_down uniform in
    {L/2-1, L/2}, U uniform(0,8), t=1."""
    rng = philox_rng(seed)
    out = []
    for _ in range(n):
        L = int(rng.choice([8, 10, 12]))
        nn = int(rng.choice([L // 2 - 1, L // 2]))
        out.append(((L,), nn, nn, float(rng.uniform(0.0, 8.0))))
    return out


def fp64_solve(mb, dims, nu, nd, u, k, seed, conv_tol=0.0):
    L = 1
    for d in dims:
        L *= d
    b = mb.FermionBasis.with_fixed_particle_number_and_spin(L, nu + nd, nu - nd)
    op = mb.GpuHubbardOperator(b, mb._Hubbard(1.0, u, dims), mb.PREC_F64)
    s = op.seed_vector(seed, order=mb.ORDER_TENSOR)
    r = mb.find_min_eigenpair(op, min(k, op.dimension()), s, order=mb.ORDER_TENSOR,
                              conv_tol=conv_tol, want_vector=False)
    return r.value


def run_batch_extra(mb, torch):
    secs = batch_sectors()
    descs = [mb.sector(d, nu, nd, 1.0, u) for d, nu, nd, u in secs]
    seeds = list(range(len(secs)))
    mb.batch_ground_states(descs[:8], seeds[:8], kmax=20)  # warm up tables / kernels
    torch.cuda.synchronize()
    # cold: a new engine (its memory pool maps the kept bases, its sector
    # tables are built); warm: the same batch again on that engine
    t0 = time.perf_counter()
    eng = mb.Engine()
    res = mb.batch_ground_states(descs, seeds, kmax=150, refine=True, use_graph=True,
                                 engine=eng)
    t_batch = time.perf_counter() - t0
    t0 = time.perf_counter()
    res_warm = mb.batch_ground_states(descs, seeds, kmax=150, refine=True, use_graph=True,
                                      engine=eng)
    t_warm = time.perf_counter() - t0
    warm_same = all(a.e0 == b.e0 for a, b in zip(res, res_warm))
    engine_shape = eng.shape()
    del eng
    # the plain per-instance FP64 GPU solver timed on a sample (same 150
    # steps); every instance checked against a converged FP64 solve
    idx = list(range(0, len(secs), 64))
    t0 = time.perf_counter()
    ref = [fp64_solve(mb, *secs[i], 150, i) for i in idx]
    t_ref = (time.perf_counter() - t0) / len(idx)
    t0 = time.perf_counter()
    conv = [fp64_solve(mb, *secs[i], 500, i, conv_tol=1e-13) for i in range(len(secs))]
    t_check = time.perf_counter() - t0
    errs = [abs(res[i].e0 - r) / abs(r) for i, r in zip(idx, ref)]
    errs_conv = [abs(r.e0 - c) / abs(c) for r, c in zip(res, conv)]
    errs_fp64_150 = [abs(a - conv[i]) / abs(conv[i]) for i, a in zip(idx, ref)]
    return {
        "instances": len(secs), "lanczos_steps": 150, "vectors": "complex64",
        "recurrence": "FP64 alpha/beta + FP64 Rayleigh-Ritz refinement",
        "solves_per_s": round(len(secs) / t_batch, 2),
        "solves_per_s_warm_engine": round(len(secs) / t_warm, 2),
        "warm_engine_same_energies": warm_same,
        "fp64_per_instance_solves_per_s": round(1.0 / t_ref, 2),
        "speedup_vs_fp64_per_instance": round((len(secs) / t_batch) * t_ref, 2),
        "max_rel_dE0_vs_fp64_same_steps": float(max(errs)),
        "max_rel_dE0_vs_converged_fp64": float(max(errs_conv)),
        "fp64_150_steps_max_rel_dE0_vs_converged": float(max(errs_fp64_150)),
        "instances_checked": len(errs_conv),
        "instances_within_1e-8": int(sum(e <= 1e-8 for e in errs_conv)),
        "check_seconds": round(t_check, 2),
        "fp64_timing_sample": len(idx), "cuda_graph": True, "autotuned": True,
        "engine_shape": engine_shape,
        "step": "one persistent cooperative launch of the fused step kernel per fixed-length "
                "phase (all its steps), captured as a CUDA graph" if engine_shape["persistent"]
                else "grouped kernels per step, captured as a CUDA graph",
    }


def run_cfg2_extra(mb, torch, n_probes=16, n_moments=1024):
    """4x4, 6+6, U=8 on Q64 vectors: the ground state by plain Lanczos (the
    reference's find_min_eigenpair) to Ritz stability 1e-12, at most 300 steps;
    the top of the spectrum the same way; then DOS Chebyshev moments with
    bounds from those extremal Ritz values, padding 0.01, random-phase probes
    (Philox streams 1..R).  Full re-orthogonalisation to 300 steps would hold
    308 GB of Krylov vectors, more than the GPU's memory."""
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(16, 12, 0)
    model = mb.HubbardModel2D(1.0, 8.0, 4, 4)
    op = mb.GpuHubbardOperator(basis, model, mb.PREC_Q64)
    op.autotune()  # the apply shape (cached per sector), outside the timed solves
    seed = op.seed_vector(0, order=mb.ORDER_TENSOR)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lo = mb.find_min_eigenpair(op, 300, seed, order=mb.ORDER_TENSOR, conv_tol=1e-12,
                               check_every=10, want_vector=False)
    t_lo = time.perf_counter() - t0
    t0 = time.perf_counter()
    hi = mb.find_max_eigenpair(op, 300, seed, order=mb.ORDER_TENSOR, conv_tol=1e-10,
                               check_every=10, want_vector=False)
    t_hi = time.perf_counter() - t0
    del seed
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mu = mb.kpm_dos_moments(op, n_moments, n_probes, 1, lo.value, hi.value, 0.01)
    t_kpm = time.perf_counter() - t0
    dim = op.dimension()
    peak, _ = measured_peaks()

    def step_roofline(seconds, steps, vector_passes):
        """A step's algorithmic bytes: the matvec (read x, write y) and
        `vector_passes` more 16-byte vector passes, over its mean wall time."""
        ms = 1e3 * seconds / max(steps, 1)
        gbs = (2 + vector_passes) * 16 * dim / (ms * 1e-3) / 1e9
        return {"ms_per_step": round(ms, 3), "algorithmic_bytes": (2 + vector_passes) * 16 * dim,
                "GBps": round(gbs, 1), "frac_of_hbm": round(gbs / peak, 4)}

    kpm_steps = n_probes * (n_moments // 2)
    return {
        "workload": "2D 4x4 periodic, t=1, U=8, N_up=N_down=6 (64,128,064 states), Q64 vectors",
        "e0": lo.value, "e0_lanczos_steps": lo.steps, "e0_seconds": round(t_lo, 3),
        # a Lanczos step: the matvec, then read v, v_prev, w and write w
        "lanczos_step": step_roofline(t_lo, lo.steps, 4),
        "e_max": hi.value, "e_max_lanczos_steps": hi.steps, "e_max_seconds": round(t_hi, 3),
        "kpm": {"moments": n_moments, "probes": n_probes, "seconds": round(t_kpm, 3),
                "seconds_per_probe": round(t_kpm / n_probes, 3),
                # a Chebyshev step (two moments by the doubling identities): the
                # matvec, then read T_n-1 and write T_n+1
                "chebyshev_step": step_roofline(t_kpm, kpm_steps, 2),
                "mu0": float(mu[0]), "mu_1_to_4": [float(v) for v in mu[1:5]]},
    }


def run_cfg2_reorth_extra(mb, torch, k=300):
    """4x4, 6+6, U=8: Lanczos with full re-orthogonalisation (classical
    Gram-Schmidt against every stored Krylov vector, a second pass by the DGKS
    test) for all 300 steps, as the 4x4 configuration names it.
    300 complex128 or Q64 vectors would be 308 GB, so the FP64 operator keeps
    its Krylov basis in complex64 (154 GB); the recurrence, the projections
    and the tridiagonal eigensolve stay FP64."""
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(16, 12, 0)
    op = mb.GpuHubbardOperator(basis, mb.HubbardModel2D(1.0, 8.0, 4, 4), mb.PREC_F64)
    op.autotune()
    seed = op.seed_vector(0, order=mb.ORDER_TENSOR)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = mb.find_min_eigenpair(op, k, seed, order=mb.ORDER_TENSOR, reorth=True,
                              basis_precision=mb.PREC_F32, want_vector=False)
    t = time.perf_counter() - t0
    del seed, op
    return {"workload": "2D 4x4 periodic, t=1, U=8, N_up=N_down=6, FP64 operator",
            "lanczos_steps": r.steps, "reorth": "classical Gram-Schmidt against every stored vector, second pass by the DGKS test",
            "krylov_basis": "complex64, 154 GB", "e0": r.value, "seconds": round(t, 3)}


def run_momentum_extra(mb, torch):
    """4x4, 6+6, U=8 on the total-momentum sector K = (0, 0) (the sector of the
    ground state): the sector basis and its H built on the GPU, the apply in
    FP64, FP32 and block floating point (Q64: exact integer sums of the +-U/N
    entries), the ground state by plain Lanczos to Ritz stability 1e-12 in
    FP64 and Q64."""
    dims = (4, 4)
    model = mb.HubbardModelMomentum(1.0, 8.0, dims)
    t0 = time.perf_counter()
    basis = mb.FermionBasis.with_fixed_particle_number_spin_momentum(16, 12, 0, dims, (0, 0))
    t_basis = time.perf_counter() - t0
    out = {"workload": "2D 4x4, U=8, N_up=N_down=6, total momentum (0,0)", "dim": basis.size(),
           "basis_seconds": round(t_basis, 3)}
    stream = torch.cuda.current_stream()
    for name, prec in (("f64", mb.PREC_F64), ("f32", mb.PREC_F32), ("q64", mb.PREC_Q64)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op = mb.GpuHubbardOperator(basis, model, prec)
        torch.cuda.synchronize()
        t_build = time.perf_counter() - t0
        shape, _ = op.autotune()  # lanes a CSR row
        x = op.seed_vector(0)
        y = op.empty()
        _, per = time_loop(torch, stream, lambda: op.apply(x, out=y, stream=stream.cuda_stream), 10, 3)
        out[f"{name}_build_seconds"] = round(t_build, 3)
        out[f"{name}_apply_ms"] = round(statistics.mean(per), 3)
        out[f"{name}_csr_lanes"] = shape["csr_lanes"]
        if prec != mb.PREC_F32:
            t0 = time.perf_counter()
            r = mb.find_min_eigenpair(op, 300, x, conv_tol=1e-12, check_every=10,
                                      want_vector=False)
            pre = "" if prec == mb.PREC_F64 else "q64_"
            out.update({pre + "e0": r.value, pre + "lanczos_steps": r.steps,
                        pre + "e0_seconds": round(time.perf_counter() - t0, 3)})
        del op, x, y
        torch.cuda.empty_cache()
    return out


def run_precision_extra(mb, torch, k=150):
    """1D L=16, N_up=N_down=8 (165,636,900 states), U in {2, 4, 8}: FP32
    (complex64) vectors and apply, Lanczos with full re-orthogonalisation
    against a complex64 Krylov basis (k vectors, 1.33 GB each) with FP64
    alpha/beta and projections, one FP64 Rayleigh-Ritz refinement; against
    the plain FP64 GPU solver (complex128, FP64 arithmetic, Ritz stability
    1e-12) on the same problem, timed at every U.  The FP32 run without
    re-orthogonalisation is reported beside them."""
    out = {}
    b = mb.FermionBasis.with_fixed_particle_number_and_spin(16, 16, 0)
    for u in (2.0, 4.0, 8.0):
        model = mb.HubbardModel(1.0, u, 16)
        op64 = mb.GpuHubbardOperator(b, model, mb.PREC_F64)
        op64.autotune()  # the apply shape, outside the timed solve
        s64 = op64.seed_vector(0, order=mb.ORDER_TENSOR)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r64 = mb.find_min_eigenpair(op64, 400, s64, order=mb.ORDER_TENSOR, conv_tol=1e-12,
                                    check_every=10, want_vector=False)
        t64 = time.perf_counter() - t0
        del op64, s64
        torch.cuda.empty_cache()
        op32 = mb.GpuHubbardOperator(b, model, mb.PREC_F32)
        op32.autotune()
        s32 = op32.seed_vector(0, order=mb.ORDER_TENSOR)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rr = mb.find_min_eigenpair(op32, k, s32, order=mb.ORDER_TENSOR, reorth=True,
                                   basis_precision=mb.PREC_F32, conv_tol=1e-10, check_every=10,
                                   want_vector=False, refine=True)
        t_re = time.perf_counter() - t0
        torch.cuda.empty_cache()
        t0 = time.perf_counter()
        rp = mb.find_min_eigenpair(op32, 300, s32, order=mb.ORDER_TENSOR, conv_tol=1e-10,
                                   check_every=10, want_vector=False, refine=True)
        t_plain = time.perf_counter() - t0
        raw = mb.find_min_eigenpair(op32, rr.steps, s32, order=mb.ORDER_TENSOR, reorth=True,
                                    basis_precision=mb.PREC_F32, want_vector=False).value
        del op32, s32
        torch.cuda.empty_cache()
        e = r64.value
        out[f"U={u:g}"] = {
            "e0_fp64": e, "steps_fp64": r64.steps, "seconds_fp64": round(t64, 3),
            "e0_fp32_reorth_refined": rr.value, "steps_fp32_reorth": rr.steps,
            "seconds_fp32_reorth_refined": round(t_re, 3),
            "rel_dE0_fp32_reorth_refined_vs_fp64": abs(rr.value - e) / abs(e),
            "e0_fp32_reorth_unrefined": raw,
            "rel_dE0_fp32_reorth_unrefined_vs_fp64": abs(raw - e) / abs(e),
            "e0_fp32_plain_refined": rp.value, "steps_fp32_plain": rp.steps,
            "seconds_fp32_plain_refined": round(t_plain, 3),
            "rel_dE0_fp32_plain_refined_vs_fp64": abs(rp.value - e) / abs(e),
            "speedup_fp32_reorth_refined_vs_fp64": round(t64 / t_re, 2),
            "speedup_fp32_plain_refined_vs_fp64": round(t64 / t_plain, 2),
        }
    return {"workload": "1D L=16 N_up=N_down=8 (165,636,900 states), t=1",
            "fp32_reorth": f"full re-orthogonalisation, complex64 basis of at most {k} vectors "
                           "(1.33 GB each), FP64 alpha/beta/projections, stop at Ritz stability "
                           "1e-10, then FP64 Rayleigh-Ritz on span{x, Hx, ...} (3-8 Krylov directions, until the lowest Ritz value settles)",
            "fp64": "plain Lanczos on complex128 with FP64 arithmetic, Ritz stability 1e-12",
            "runs": out}


SERVE_LATTICES = [(6,), (7,), (8,), (9,), (10,), (11,), (12,), (13,), (14,), (3, 3), (2, 4), (3, 4)]


def serve_requests(n, rate, seed=77):
    """Poisson arrivals (mean `rate`/s); lattice uniform over SERVE_LATTICES;
    N_up = N_down uniform over the non-trivial sectors 1..L-1; U ~ U(0,10);
    half ground states (1e-8 relative), half 512-moment DOS requests."""
    rng = philox_rng(seed)
    t = 0.0
    reqs = []
    for i in range(n):
        t += float(rng.exponential(1.0 / rate))
        dims = SERVE_LATTICES[int(rng.integers(len(SERVE_LATTICES)))]
        L = 1
        for d in dims:
            L *= d
        nn = int(rng.integers(1, L))
        kind = int(rng.integers(2))
        reqs.append((t, dims, nn, float(rng.uniform(0.0, 10.0)), kind, i))
    return reqs


def fp64_dos(mb, dims, nn, u, n_moments, seed):
    L = 1
    for d in dims:
        L *= d
    b = mb.FermionBasis.with_fixed_particle_number_and_spin(L, 2 * nn, 0)
    op = mb.GpuHubbardOperator(b, mb._Hubbard(1.0, u, dims), mb.PREC_F64)
    s = op.seed_vector(seed, order=mb.ORDER_TENSOR)
    k = min(40, op.dimension())
    lo = mb.find_min_eigenpair(op, k, s, order=mb.ORDER_TENSOR, want_vector=False).value
    hi = mb.find_max_eigenpair(op, k, s, order=mb.ORDER_TENSOR, want_vector=False).value
    pad = 0.05 * (hi - lo) + 1e-6
    return mb.kpm_dos_moments(op, n_moments, 1, seed, lo - pad, hi + pad, 0.01)


def q64_dos(mb, dims, nn, u, n_moments, seed, lo, hi, padding=0.01):
    """DOS moments of one probe (Philox stream 1, key `seed`: the engine's
    probe) on an FP64-class (Q64) operator with the given bounds."""
    L = 1
    for d in dims:
        L *= d
    b = mb.FermionBasis.with_fixed_particle_number_and_spin(L, 2 * nn, 0)
    op = mb.GpuHubbardOperator(b, mb._Hubbard(1.0, u, dims), mb.PREC_Q64)
    return mb.kpm_dos_moments(op, n_moments, 1, seed, lo, hi, padding)


def run_serve_extra(mb, torch, n_requests=400, rate=200.0):
    import numpy as np
    reqs = serve_requests(n_requests, rate)
    eng = mb.Engine()
    pending, live, lat, e_served, dos_served = [], {}, {}, {}, {}
    nxt = 0
    t0 = time.perf_counter()
    while len(lat) < len(reqs):
        now = time.perf_counter() - t0
        while nxt < len(reqs) and reqs[nxt][0] <= now:
            pending.append(reqs[nxt])
            nxt += 1
        while pending:
            a, dims, nn, u, kind, i = pending[0]
            d = mb.sector(dims, nn, nn, 1.0, u)
            rid = (eng.try_submit(d, seed=i, kmax=400, rel_tol=1e-10, refine=True) if kind == 0
                   else eng.try_submit_dos(d, n_moments=512, n_probes=1, seed=i))
            if rid is None:
                break
            live[rid] = (a, kind, i)
            pending.pop(0)
        if live:
            eng.step(1)
            for rid in eng.completed():
                a, kind, i = live.pop(rid)
                r = eng.poll(rid) if kind == 0 else eng.poll_dos(rid)
                lat[i] = (time.perf_counter() - t0) - a
                if kind == 0:
                    e_served[i] = r.e0
                else:
                    dos_served[i] = (np.asarray(r[0]), r[1], r[2])
        elif nxt < len(reqs):
            time.sleep(max(0.0, reqs[nxt][0] - (time.perf_counter() - t0)))
    wall = time.perf_counter() - t0
    n_steps, step_wall_ms, step_dev_ms = eng.stats()
    lv = np.array(sorted(lat.values()))
    # the same stream through the plain per-request FP64 GPU solver, FIFO
    lat_ref, e_ref = [], {}
    t0 = time.perf_counter()
    for a, dims, nn, u, kind, i in reqs:
        wait = a - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        if kind == 0:
            e_ref[i] = fp64_solve(mb, dims, nn, nn, u, 400, i, conv_tol=1e-10)
        else:
            fp64_dos(mb, dims, nn, u, 512, i)
        lat_ref.append((time.perf_counter() - t0) - a)
    wall_ref = time.perf_counter() - t0
    lr = np.array(sorted(lat_ref))
    # accuracy of every result: each ground state against a converged FP64
    # solve; each DOS request's moments against the FP64-class (Q64) Chebyshev
    # moments of the same probe with the bounds the engine used
    by_idx = {r[5]: r for r in reqs}
    t_chk = time.perf_counter()
    dE = []
    for i in sorted(e_served):
        a, dims, nn, u, kind, _ = by_idx[i]
        e_conv = fp64_solve(mb, dims, nn, nn, u, 500, i, conv_tol=1e-13)
        dE.append(abs(e_served[i] - e_conv) / max(abs(e_conv), 1e-300))
    # a rounding-error model of the FP32 Chebyshev recurrence: mu_n comes from
    # the k = ceil(n / 2) + 1 steps behind it; each step adds up to ~8 u_32
    # (u_32 = 2^-24: the apply's sums, the doubling and the subtraction), and
    # an error made at step j reaches step k through U_(k-j)(H~) (norm <=
    # k - j + 1 on [-1, 1]), so |d mu_n| <= 8 k^2 u_32
    dmu, dmu_ratio = [], []
    for i in sorted(dos_served):
        a, dims, nn, u, kind, _ = by_idx[i]
        mu, lo, hi = dos_served[i]
        d = np.abs(mu - q64_dos(mb, dims, nn, u, len(mu), i, lo, hi))
        k = np.ceil(np.arange(len(mu)) / 2.0) + 1.0
        dmu.append(float(np.max(d)))
        dmu_ratio.append(float(np.max(d / (8.0 * k * k * 2.0 ** -24))))
    t_chk = time.perf_counter() - t_chk
    return {
        "requests": len(reqs), "arrival_rate_per_s": rate,
        "mix": "50 % ground state (Ritz stability 1e-10 + FP64 Rayleigh refinement), "
               "50 % 512-moment KPM DOS (1 random-phase probe)",
        "engine": {"wall_s": round(wall, 3), "solves_per_s": round(len(reqs) / wall, 2),
                   "latency_p50_s": round(float(np.percentile(lv, 50)), 4),
                   "latency_p99_s": round(float(np.percentile(lv, 99)), 4),
                   "steps": n_steps, "step_ms": round(step_wall_ms / max(n_steps, 1), 4),
                   "step_device_ms": round(step_dev_ms / max(n_steps, 1), 4)},
        "fp64_per_request_fifo": {"wall_s": round(wall_ref, 3),
                                  "solves_per_s": round(len(reqs) / wall_ref, 2),
                                  "latency_p50_s": round(float(np.percentile(lr, 50)), 4),
                                  "latency_p99_s": round(float(np.percentile(lr, 99)), 4)},
        "solves_per_s_ratio": round(wall_ref / wall, 2),
        "max_rel_dE0_vs_converged_fp64": float(max(dE)) if dE else None,
        "ground_states_checked": len(dE),
        "ground_states_within_1e-8": int(sum(x <= 1e-8 for x in dE)),
        "max_abs_dmu_vs_fp64class": float(max(dmu)) if dmu else None,
        "dos_requests_checked": len(dmu),
        "dos_within_1e-4": int(sum(x <= 1e-4 for x in dmu)),
        "max_dmu_over_fp32_rounding_bound": float(max(dmu_ratio)) if dmu_ratio else None,
        "dos_within_fp32_rounding_bound": int(sum(x <= 1.0 for x in dmu_ratio)),
        "check_seconds": round(t_chk, 2),
    }


# ---------------------------------------------------------------------------
# CPU reference path (oracle restatement of compute_matrix_elements + serial
# CSC apply), on a bounded sample.
# ---------------------------------------------------------------------------
def cpu_sample_matrix():
    """The sample's H by the restated compute_matrix_elements (normal ordering
    of H|key_j>, OpenMP over columns), with the wall time of building it: the
    reference's CPU path builds H once, then applies it serially."""
    import oracle
    # same lattice and interaction, a sector small enough to build in seconds
    t0 = time.perf_counter()
    H = oracle.hubbard_csc([4, 4], 1.0, 8.0, 3, 3)
    build = {"build_seconds": round(time.perf_counter() - t0, 3),
             "build_cores": oracle.max_threads()}
    return H, "4x4 U=8 sector N_up=N_down=3 (313,600 states)", build


def concurrent_applies(H, x, seconds):
    """Every host thread applies H to its own vector, the serial column scatter
    each, as the reference's OpenMP drivers call apply on one const operator
    from every thread; returns (GB/s over all threads, threads, applies, s)."""
    import concurrent.futures as cf
    nthreads = max(1, len(os.sched_getaffinity(0)))
    xs = [x.copy() for _ in range(nthreads)]
    with cf.ThreadPoolExecutor(nthreads) as pool:
        list(pool.map(H.apply, xs))
        n, t0 = 0, time.perf_counter()
        while True:
            list(pool.map(H.apply, xs))  # the foreign call releases the GIL
            n += 1
            el = time.perf_counter() - t0
            if el >= seconds or n >= 10000:
                break
    return nthreads * n * 2 * 16 * H.dim / el / 1e9, nthreads, nthreads * n, el


def cpu_baseline(seconds: float = 10.0):
    """The reference's CPU apply on the host cores: the serial column scatter
    of Armadillo's sp_cx_mat * cx_vec on every host thread at once (one vector
    a thread), with the single-thread rate beside it."""
    import numpy as np
    H, sample, build = cpu_sample_matrix()
    x = np.ascontiguousarray(
        np.random.default_rng(0).uniform(-1, 1, H.dim) + 1j * np.random.default_rng(1).uniform(-1, 1, H.dim))
    H.apply(x)
    n, t0 = 0, time.perf_counter()
    while True:
        H.apply(x)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds / 2 or n >= 10000:
            break
    per = el / n
    gbs, nthreads, napp, elc = concurrent_applies(H, x, seconds / 2)
    return {"value": round(gbs, 4), "unit": "GB/s", "cores": nthreads, "kind": "port",
            "sample": f"{sample}; serial CSC column-scatter apply on each of {nthreads} threads, "
                      f"one vector a thread, {napp} applies in {elc:.1f}s, nnz={H.nnz}",
            **build,
            "single_thread": {"value": round(2 * 16 * H.dim / per / 1e9, 4), "unit": "GB/s",
                              "cores": 1, "sample": f"{n} applies in {el:.1f}s"},
            "best_effort_all_cores": cpu_parallel(H, x, sample, seconds / 4)}


def cpu_parallel(H, x, sample, seconds):
    """Best-effort context: a multi-core row gather of the same Hermitian matrix
    (not the reference's algorithm, whose Armadillo product is serial)."""
    import oracle
    H.apply_parallel(x)
    n, t0 = 0, time.perf_counter()
    while True:
        H.apply_parallel(x)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds or n >= 20000:
            break
    per = el / n
    return {"value": round(2 * 16 * H.dim / per / 1e9, 4), "unit": "GB/s",
            "cores": oracle.max_threads(), "kind": "port",
            "sample": f"{sample}; OpenMP row gather (column i of the Hermitian H = conj of "
                      f"row i), {n} applies in {el:.1f}s"}


def run_reference(args):
    """The reference's CPU apply on the machine's host cores, with every host thread:
    each thread applies the sample H to its own vector, as the reference's
    OpenMP drivers call apply on one const operator from every thread
    (examples/hubbard_momentum_optical_conductivity.cpp:351-400); the apply
    itself is the serial column scatter of Armadillo's sp_cx_mat * cx_vec.  A
    step is one apply on every thread; the single-thread rate is reported
    beside it."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import numpy as np
    H, sample, build = cpu_sample_matrix()
    x = np.ascontiguousarray(np.random.default_rng(0).uniform(-1, 1, H.dim) + 0j)
    # single thread
    for _ in range(args.warmup):
        H.apply(x)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        H.apply(x)
        times.append(time.perf_counter() - t0)
    per1 = sum(times) / len(times)
    value1 = 2 * 16 * H.dim / per1 / 1e9
    # every host thread, one vector each; a step is one apply on every thread
    import concurrent.futures as cf
    nthreads = max(1, len(os.sched_getaffinity(0)))
    xs = [x.copy() for _ in range(nthreads)]
    with cf.ThreadPoolExecutor(nthreads) as pool:
        for _ in range(args.warmup):
            list(pool.map(H.apply, xs))
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            list(pool.map(H.apply, xs))  # the foreign call releases the GIL
            times.append(time.perf_counter() - t0)
    per = sum(times) / len(times)
    value = nthreads * 2 * 16 * H.dim / per / 1e9
    out = {
        "metric": METRIC,
        "value": round(value, 4),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(per * 1e3, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic uniform(-1,1) vector",
        "config": dict(CASES["4x4_6+6"], lattice="4x4", dim=64128064, sample=sample),
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 4), "unit": "GB/s", "cores": nthreads,
                         "kind": "port",
                         "sample": f"{sample}; the reference's compute_matrix_elements H "
                                   f"(restated) applied by the serial CSC column scatter of "
                                   f"Armadillo's sp_cx_mat*cx_vec, one apply per thread on its "
                                   f"own vector, {nthreads} threads concurrently (a step: one "
                                   f"apply on every thread)",
                         **build,
                         "single_thread": {"value": round(value1, 4), "unit": "GB/s",
                                           "cores": 1},
                         "best_effort_all_cores": cpu_parallel(H, x, sample, 5.0)},
        "e2e": {"value": round(value, 4), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------
# Kernel probes for profiling captures: a few launches of one kernel's
# workload, nothing timed (ncu measures).  Each prints one JSON line.
# ---------------------------------------------------------------------------
PROBES = ("q64_apply", "fp64_apply", "fp32_apply", "engine_persistent", "engine_grouped",
          "engine_persistent_fixed", "engine_fused", "momentum_csr", "momentum_csr_q64",
          "q64_lanczos", "fp32_lanczos_refined")


def run_probe(args):
    import torch

    import manybody_gb300 as mb
    torch.cuda.set_device(0)
    name = args.probe
    if name in ("q64_apply", "fp64_apply", "fp32_apply"):
        w = CASES[args.case]
        L = 1
        for d in w["lattice"]:
            L *= d
        basis = mb.FermionBasis.with_fixed_particle_number_and_spin(L, w["n_up"] + w["n_down"],
                                                                    w["n_up"] - w["n_down"])
        prec = {"q64_apply": mb.PREC_Q64, "fp64_apply": mb.PREC_F64,
                "fp32_apply": mb.PREC_F32}[name]
        op = mb.GpuHubbardOperator(basis, mb._Hubbard(w["t"], w["U"], w["lattice"]), prec)
        if args.apply_shape:  # a given shape; else the default (a profiler distorts the tuner's timings)
            op.set_apply_shape(**json.loads(args.apply_shape))
        shape = op.apply_shape()
        x = op.seed_vector(0, order=mb.ORDER_TENSOR)
        if prec == mb.PREC_Q64:
            xq, ex = op.q64_from_f64(x, order=mb.ORDER_TENSOR)
            yq = op.q64_empty()
            for _ in range(args.steps):
                op.apply_q64(xq, ex, out=yq)
        else:
            y = op.empty()
            for _ in range(args.steps):
                op.apply(x, out=y, order=mb.ORDER_TENSOR)
        torch.cuda.synchronize()
        out = {"probe": name, "case": args.case, "dim": op.dimension(), "apply_shape": shape,
               "launches": args.steps}
    elif name == "fp32_lanczos_refined":
        # --steps plain Lanczos steps on complex64 vectors with FP64 alpha/beta,
        # then the FP64 Rayleigh-Ritz refinement (the precision path), on
        # --case
        w = CASES[args.case]
        L = 1
        for d in w["lattice"]:
            L *= d
        basis = mb.FermionBasis.with_fixed_particle_number_and_spin(L, w["n_up"] + w["n_down"],
                                                                    w["n_up"] - w["n_down"])
        op = mb.GpuHubbardOperator(basis, mb._Hubbard(w["t"], w["U"], w["lattice"]), mb.PREC_F32)
        x = op.seed_vector(0, order=mb.ORDER_TENSOR)
        r = mb.find_min_eigenpair(op, args.steps, x, order=mb.ORDER_TENSOR, want_vector=False,
                                  refine=True)
        torch.cuda.synchronize()
        out = {"probe": name, "case": args.case, "dim": op.dimension(), "steps": r.steps,
               "e0": r.value}
    elif name == "q64_lanczos":
        # --steps plain Lanczos steps on the Q64 operator of --case (the
        # ground-state solve's recurrence: apply with fused dots, w -= alpha v,
        # v = w / beta)
        w = CASES[args.case]
        L = 1
        for d in w["lattice"]:
            L *= d
        basis = mb.FermionBasis.with_fixed_particle_number_and_spin(L, w["n_up"] + w["n_down"],
                                                                    w["n_up"] - w["n_down"])
        op = mb.GpuHubbardOperator(basis, mb._Hubbard(w["t"], w["U"], w["lattice"]), mb.PREC_Q64)
        x = op.seed_vector(0, order=mb.ORDER_TENSOR)
        r = mb.find_min_eigenpair(op, args.steps, x, order=mb.ORDER_TENSOR, want_vector=False)
        torch.cuda.synchronize()
        out = {"probe": name, "case": args.case, "dim": op.dimension(), "steps": r.steps}
    elif name in ("engine_persistent", "engine_grouped", "engine_persistent_fixed"):
        # engine_persistent_fixed: all --steps steps in one launch (a fixed-length
        # batch), the others one launch a step
        secs = batch_sectors(n=64)
        descs = [mb.sector(d, nu, nd, 1.0, u) for d, nu, nd, u in secs]
        eng = mb.Engine()
        eng.set_persistent(name != "engine_grouped")
        for i, d in enumerate(descs):
            eng.try_submit(d, seed=i, kmax=150, rel_tol=0.0)
        if name == "engine_persistent_fixed":
            eng.step_fixed(args.steps, False)
        else:
            eng.step(args.steps)
        torch.cuda.synchronize()
        import math
        states = sum(math.comb(d[0], nu) * math.comb(d[0], nd) for d, nu, nd, _ in secs)
        out = {"probe": name, "requests": len(descs), "steps": args.steps, "states": states,
               "shape": eng.shape()}
    elif name == "engine_fused":
        # four 4x4 5+5 requests (19,079,424 states each): large enough for the
        # grouped engine's fused apply (k_eng_fused)
        descs = [mb.sector((4, 4), 5, 5, 1.0, u) for u in (2.0, 4.0, 6.0, 8.0)]
        eng = mb.Engine()
        eng.set_persistent(False)
        for i, d in enumerate(descs):
            eng.try_submit(d, seed=i, kmax=150, rel_tol=0.0)
        eng.step(args.steps)
        torch.cuda.synchronize()
        out = {"probe": name, "requests": len(descs), "steps": args.steps,
               "states": 4 * 19079424, "shape": eng.shape()}
    else:  # momentum_csr(_q64): the K = (0, 0) sector of 4x4, N_up = N_down = 4
        dims = (4, 4)
        basis = mb.FermionBasis.with_fixed_particle_number_spin_momentum(16, 8, 0, dims, (0, 0))
        prec = mb.PREC_Q64 if name.endswith("q64") else mb.PREC_F64
        op = mb.GpuHubbardOperator(basis, mb.HubbardModelMomentum(1.0, 8.0, dims), prec)
        x = op.seed_vector(0)
        y = op.empty()
        for _ in range(args.steps):
            op.apply(x, out=y)
        torch.cuda.synchronize()
        out = {"probe": name, "dim": op.dimension(), "launches": args.steps}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--case", default="4x4_6+6", choices=sorted(CASES))
    ap.add_argument("--only-apply", action="store_true",
                    help="time only the device apply (profiling captures)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batching / precision / serving extras")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--skip-cfg2-reorth", action="store_true",
                    help="leave out the 300-step fully re-orthogonalised Lanczos at 4x4 6+6")
    ap.add_argument("--apply-shape", default=None,
                    help="with --probe q64_apply / fp64_apply / fp32_apply: the apply shape as "
                         "JSON, e.g. '{\"table_bits\": 16, \"row_split\": 2}'")
    ap.add_argument("--probe", choices=PROBES,
                    help="run a few launches of one kernel's workload for a profiler "
                         "(--steps launches; nothing timed, no bench line)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.probe:
        run_probe(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
