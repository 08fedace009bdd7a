#!/usr/bin/env python
"""Benchmark: MsFEM basis solves/s on one GB300 (per rank), one JSON line.

Workload (one step = one pass of the hot path over the batch):
  2D unit square, 64x64 coarse Q1 cells (4096), 32x32 fine Q1 cells per
  coarse cell (1089 nodes), 4 Dirichlet basis solves per cell (16384 solves),
  random-Fourier SPD tensor A = R(theta) diag(e^g1, e^g2) R(theta)^T (64
  modes per field, |k| <= 128 pi, amplitudes N(0, 1/64), seeds 2/20/200),
  f = 1, CG to 1e-10 relative residual.  Synthetic, seeded; the coefficient is
  tabulated at the QGauss(2) points once (input data, 403 MB, larger than L2)
  and stays resident in HBM.

value      device-resident FP64 form (the drop-in), CUDA events on the
           launching stream, max over ranks.
mixed      same workload, FP32 inner CG + FP64 refinement.
e2e        the public C-ABI call with pinned HOST buffers: H2D of the corners
           and the tabulated field, D2H of M and F, every step.
roofline   FP64 FMA pipe (the kernel is bound by it; HBM fraction reported too).
cpu_baseline  the oracle's restatement of the reference algorithm (SSOR(1.6)
           preconditioned CG on CSR, QGauss(2) assembly, 2^d x 2^d SpMV
           epilogue) on a bounded sample of the same workload, all host cores.

--impl reference  the reference algorithm on the host cores only (the
           reference itself cannot be built: deal.II/p4est/Trilinos/MPI absent).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
import __graft_entry__ as graft  # noqa: E402

METRIC = "MsFEM basis solves/s at 1e-10 rel residual, plain FP64 vs mixed+surrogate, 1 GB300"
UNIT = "basis solves/s"
TOL = 1e-10
K_COARSE, N_FINE = 64, 32
WORKLOAD = ("2D MsFEM local basis: 64x64 coarse Q1 cells, 32x32 fine Q1 per cell, 4 RHS per cell, "
            "random-Fourier SPD tensor (seeds 2/20/200), f=1, CG to 1e-10 rel residual")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def flops_per_solve_iter(N):
    """Algorithmic work of one CG iteration of one 2D solve: 2 nnz(A_II) +
    11 n_I, nnz(A_II) = (3N-5)^2, n_I = (N-1)^2."""
    return 2 * (3 * N - 5) ** 2 + 11 * (N - 1) ** 2


def flops_per_solve_iter_3d(N):
    """Algorithmic work of one CG iteration of one 3D solve: 2 nnz(A_II) +
    11 n_I, nnz(A_II) = (3N-5)^3, n_I = (N-1)^3."""
    return 2 * (3 * N - 5) ** 3 + 11 * (N - 1) ** 3


def inner_flops_per_iter(N, poly, coarse=0):
    """Inner FP32 iteration of the mixed 2D form, per right-hand side.

    Polynomial preconditioner of degree `poly` (poly + 1 stencils, two
    dot-product pairs and the vector updates): (poly + 1) 2 nnz(A_II) +
    (11 + 4 poly) n_I.  Two-level V-cycle (`coarse` = coarse spacing > 0,
    smoothing degree poly = M - 1): 2M + 1 stencils (search direction, M
    pre-smoothing, the coarse correction's, M - 1 post-smoothing), 10 M + 22
    vector operations per node, the restriction and prolongation
    (28 per coarse node) and the dense coarse solve 2 n_c^2, n_c the
    interior coarse nodes."""
    nnz, n_i = (3 * N - 5) ** 2, (N - 1) ** 2
    if coarse and N % coarse == 0 and N // coarse >= 2:
        m = poly + 1
        n_c = (N // coarse - 1) ** 2
        return (2 * m + 1) * 2 * nnz + (10 * m + 22) * n_i + 2 * n_c * n_c + 28 * n_c
    return (poly + 1) * 2 * nnz + (11 + 4 * poly) * n_i


def flops_one_off_per_cell(N):
    """Epilogue 2^d 2 nnz + (2^2d + 2^d) 2 n^d, assembly N^d 2^d (2^2d (2d+1))."""
    n = N + 1
    return 4 * 2 * (3 * n - 2) ** 2 + (16 + 4) * 2 * n * n + N * N * 4 * (16 * 5)


def load_probe(pkg):
    lib = ctypes.CDLL(os.path.join(pkg.build.LIB_DIR, "libmsfem_probe.so"))
    lib.msfem_probe_fma_flops.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    lib.msfem_probe_fma_flops.restype = ctypes.c_int
    return lib


def read_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def read_profile_traffic(name):
    """dram bytes per launch recorded from an ncu capture (profiles/*.txt)."""
    path = os.path.join(REPO, "profiles", name)
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                mhz.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not mhz:
            return None
        busy = [m for m in mhz if mx and m > 0.5 * mx] or mhz
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(mhz)}


def cpu_reference(pkg, oracle, prob_cells, nthreads, steps=1, warmup=0, min_seconds=0.0):
    """The reference algorithm (SSOR(1.6)-PCG, CSR, QGauss(2) assembly) on a
    sample of cells; the tabulated coefficient is prepared untimed.  Timed
    passes repeat until `steps` passes and at least `min_seconds` (at most
    30 s) have run."""
    tab = oracle.tabulate(prob_cells, 3)
    tprob = dict(prob_cells)
    tprob["coef"] = {"kind": pkg._abi.COEF_TABULATED, "ncomp": 3, "qp_values": tab}
    times = []
    res = None
    it = 0
    while it < warmup + steps or (sum(times) < min_seconds and sum(times) < 30.0):
        t0 = time.perf_counter()
        res = oracle.run(tprob, solver=oracle.SOLVER_SSOR_CG, tol=TOL, tol_absolute=False,
                         maxit=1000, omega=1.6, ordering=oracle.ORDER_DEALII, nthreads=nthreads)
        dt = time.perf_counter() - t0
        if it >= warmup:
            times.append(dt)
        it += 1
    solves = prob_cells["corners"].shape[0] * 4
    return solves, times, res


def run_reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    pkg = graft.load_package()
    oracle = graft.load_oracle()
    oracle.build()
    W = pkg.workloads
    full = W.fourier_square(K=K_COARSE, N=N_FINE)
    nthreads = os.cpu_count() or 1
    n_sample = max(16, min(4096, 64 * nthreads))
    cells = np.linspace(0, K_COARSE * K_COARSE - 1, n_sample).astype(int)
    sample = W.subset(full, cells)
    solves, times, res = cpu_reference(pkg, oracle, sample, nthreads, steps=args.steps,
                                       warmup=args.warmup)
    t = sum(times) / len(times)
    value = solves / t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded random-Fourier coefficient)",
        "config": {"workload": WORKLOAD, "precision": "fp64", "sample_cells": int(n_sample)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"{n_sample} of 4096 coarse cells per step ({solves} solves), "
                                   "SSOR(1.6)-PCG to 1e-10 rel, deal.II dof order"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "mean_iterations": float(res["iters"].mean()),
        "note": ("reference cannot be built here (deal.II/p4est/Trilinos/MPI absent); this is "
                 "the oracle's restatement of its local-basis algorithm"),
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile", default=None, choices=["fp64_2d", "mixed_2d", "fp64_3d", "mixed_3d", "cnn"],
                    help="run one small single-kernel case (for ncu captures) and exit")
    ap.add_argument("--variant", type=int, default=None, help="--profile: launch shape index to use")
    ap.add_argument("--inner-tol", type=float, default=1e-6, help="--profile 2D mixed: inner FP32 reduction")
    ap.add_argument("--cheb-ratio", type=float, default=30.0, help="--profile 2D mixed: Chebyshev interval ratio")
    ap.add_argument("--no-fourier-256", action="store_true", help="skip the 256x256-cell (65536) Fourier-field timing")
    ap.add_argument("--no-surrogate", action="store_true", help="skip training / evaluating the warm start")
    ap.add_argument("--no-spheres-3d", action="store_true", help="skip the 3D uneven-N sphere-field timing")
    ap.add_argument("--coarse", type=int, default=K_COARSE, help="coarse cells per direction")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference_arm(args)
        return

    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pkg = graft.load_package()
    pkg.build.build_all()
    abi = pkg._abi
    W = pkg.workloads
    eng = pkg.Engine(local)
    # a dedicated (non-default) stream, current for torch and used by the
    # library, so the CUDA events below bracket the kernels themselves
    stream = torch.cuda.Stream(device=local)
    torch.cuda.set_stream(stream)
    eng.set_stream(stream.cuda_stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def max_over_ranks(x):
        return pkg.sharding.max_over_ranks(x, torch.distributed if world > 1 else None, f"cuda:{local}")

    tab_times = {}

    def make_ws(prob, shift):
        """Device workload: corners + the coefficient tabulated at the Gauss
        points (input data, tabulated once by the library's field kernel;
        the tabulation's device time is kept in tab_times by cell count)."""
        corners_h = pkg.sharding.weak_shard_corners(prob["corners"], shift)
        n = corners_h.shape[0]
        corners_d = torch.from_numpy(corners_h).to(f"cuda:{local}")
        modes_d = torch.from_numpy(np.ascontiguousarray(prob["coef"]["modes"])).to(f"cuda:{local}")
        dt = abi.BatchDesc()
        dt.dim, dt.n_cells, dt.n_fine = 2, n, N_FINE
        dt.corners = corners_d.data_ptr()
        dt.coef.kind = abi.COEF_FOURIER
        dt.coef.modes = modes_d.data_ptr()
        dt.coef.n_modes = modes_d.shape[1]
        dt.memory = abi.MEM_DEVICE
        dt.tol, dt.maxit = TOL, 1000
        size = eng.lib.msfem_tabulated_size(ctypes.byref(dt), 3)
        tab_d = torch.empty(size, dtype=torch.float64, device=f"cuda:{local}")
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        rc = eng.lib.msfem_tabulate_coefficient(eng.handle, ctypes.byref(dt), 3, tab_d.data_ptr())
        ev1.record(stream)
        if rc != abi.OK:
            raise abi.MsfemError(rc, abi.last_error(eng.lib))
        torch.cuda.synchronize()
        tab_times[n] = {"ms": ev0.elapsed_time(ev1), "bytes": int(size * 8)}
        ws = {"n": n, "corners_h": corners_h, "corners_d": corners_d, "tab_d": tab_d, "size": size,
              "M": torch.empty((n, 4, 4), dtype=torch.float64, device=f"cuda:{local}"),
              "F": torch.empty((n, 4), dtype=torch.float64, device=f"cuda:{local}"),
              "st": torch.empty(n, dtype=torch.int32, device=f"cuda:{local}"),
              "it": torch.empty((n, 4), dtype=torch.int32, device=f"cuda:{local}")}
        return ws

    def device_desc(ws, precision):
        d = abi.BatchDesc()
        d.dim, d.n_cells, d.n_fine = 2, ws["n"], N_FINE
        d.precision = precision
        d.corners = ws["corners_d"].data_ptr()
        d.coef.kind = abi.COEF_TABULATED
        d.coef.ncomp = 3
        d.coef.qp_values = ws["tab_d"].data_ptr()
        d.f_value = 1.0
        d.tol, d.maxit = TOL, 1000
        d.memory = abi.MEM_DEVICE
        return d

    def timed_ws(ws, precision, steps, warmup, sample_clocks=False):
        d = device_desc(ws, precision)
        args_ = (ws["M"].data_ptr(), ws["F"].data_ptr(), None, ws["st"].data_ptr(), ws["it"].data_ptr())
        for _ in range(warmup):
            eng.run_desc(d, *args_, stats=False)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        sampler = ClockSampler(local) if sample_clocks else None
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            eng.run_desc(d, *args_, stats=False)
        e1.record(stream)
        torch.cuda.synchronize()
        clocks = sampler.stop() if sampler else None
        barrier()
        ms = e0.elapsed_time(e1) / steps
        # correctness / work accounting of the same workload (untimed)
        _, st = eng.run_desc(d, *args_, stats=True)
        return max_over_ranks(ms), st, clocks

    def solve_with_basis(ws, precision, tol, warm=abi.WARM_NONE, desc=None):
        """One untimed solve of a device workload with the basis output."""
        d = desc if desc is not None else device_desc(ws, precision)
        d.precision, d.tol, d.warm_start = precision, tol, warm
        n = d.n_cells
        out = {"M": torch.empty((n, 4, 4), dtype=torch.float64, device=f"cuda:{local}"),
               "F": torch.empty((n, 4), dtype=torch.float64, device=f"cuda:{local}"),
               "basis": torch.empty((n, 4, (N_FINE + 1) ** 2), dtype=torch.float64, device=f"cuda:{local}"),
               "st": torch.empty(n, dtype=torch.int32, device=f"cuda:{local}"),
               "it": torch.empty((n, 4), dtype=torch.int32, device=f"cuda:{local}")}
        _, out["stats"] = eng.run_desc(d, out["M"].data_ptr(), out["F"].data_ptr(), out["basis"].data_ptr(),
                                       out["st"].data_ptr(), out["it"].data_ptr(), stats=True)
        d.warm_start = abi.WARM_NONE
        d.tol = TOL
        return out

    def basis_errors(ws, got, ref, desc=None):
        """Energy-norm error of every basis function (msfem_energy_error) and
        the coarse-matrix error of every cell, got against ref."""
        d = desc if desc is not None else device_desc(ws, abi.PREC_FP64)
        n, nv = d.n_cells, 1 << d.dim
        err = torch.empty((n, nv), dtype=torch.float64, device=f"cuda:{local}")
        nrm = torch.empty((n, nv), dtype=torch.float64, device=f"cuda:{local}")
        rc = eng.lib.msfem_energy_error(eng.handle, ctypes.byref(d), got["basis"].data_ptr(),
                                        ref["basis"].data_ptr(), err.data_ptr(), nrm.data_ptr())
        if rc != abi.OK:
            raise abi.MsfemError(rc, abi.last_error(eng.lib))
        torch.cuda.synchronize()
        rel = err / nrm
        scale = ref["M"].abs().amax(dim=(1, 2), keepdim=True)
        mrel = ((got["M"] - ref["M"]).abs() / scale).amax(dim=(1, 2))
        frel = ((got["F"] - ref["F"]).abs() / ref["F"].abs().amax(dim=1, keepdim=True)).amax(dim=1)
        return {"max_rel_energy_error": float(rel.max()), "mean_rel_energy_error": float(rel.mean()),
                "max_rel_M_error": float(mrel.max()), "mean_rel_M_error": float(mrel.mean()),
                "max_rel_F_error": float(frel.max()),
                "max_rel_residual": got["stats"]["max_rel_residual"],
                "cells_failed": got["stats"]["cells_failed"]}

    # ---- small single-kernel cases for ncu captures (--profile KIND): W
    # warm-up launches, then K timed ones; nothing else runs
    if args.profile:
        kind = args.profile
        t_ms = None
        if kind in ("fp64_2d", "mixed_2d"):
            # 48x48 cells: a 226 MB tabulated field, larger than L2
            wsp = make_ws(W.fourier_square(K=48, N=N_FINE), 0)
            prec = abi.PREC_FP64 if kind == "fp64_2d" else abi.PREC_MIXED
            if args.variant is not None:
                eng.set_tuning({"dim": 2, "n_max": N_FINE, "precision": prec, "variant": args.variant,
                                "check_interval": 0, "inner_tol": args.inner_tol,
                                "cheb_ratio": args.cheb_ratio})
            t_ms, _, _ = timed_ws(wsp, prec, args.steps, args.warmup)
        elif kind in ("fp64_3d", "mixed_3d"):
            # the first 256 cells of the 3D sphere field (uneven N, 1e4-contrast spheres)
            sub = W.subset(W.spheres_cube(), np.arange(256))
            prec = "fp64" if kind == "fp64_3d" else "mixed"
            if args.variant is not None:
                eng.set_tuning({"dim": 3, "n_max": 24, "precision": 0 if prec == "fp64" else 1,
                                "variant": args.variant, "check_interval": 0, "inner_tol": args.inner_tol})
            for _ in range(args.warmup):
                eng.run(sub, precision=prec, tol=TOL)
            t_ms = 0.0
            for _ in range(args.steps):
                t_ms += eng.run(sub, precision=prec, tol=TOL)["stats"]["kernel_ms"] / args.steps
        elif kind == "cnn":
            # inference of 2048 cells and training steps of batch 256 (random weights)
            S = pkg.surrogate
            desc_p, keep_p = S.device_problem(eng, W.subset(W.fourier_square(K=64, N=N_FINE), np.arange(2048)), torch)
            feats = S.features(eng, desc_p, torch)
            sur = S.Surrogate(eng, seed=7)
            out = torch.empty((2048, 4, 33, 33), dtype=torch.float32, device=f"cuda:{local}")
            tg = torch.zeros((256, 4, 33, 33), dtype=torch.float32, device=f"cuda:{local}")
            for _ in range(args.warmup):
                sur.predict(feats, out)
                sur.train_step(feats[:256].contiguous(), tg, 1e-3)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.steps):
                sur.predict(feats, out)
            e1.record(stream)
            torch.cuda.synchronize()
            t_ms = e0.elapsed_time(e1) / args.steps
            for _ in range(args.steps):
                sur.train_step(feats[:256].contiguous(), tg, 1e-3)
            torch.cuda.synchronize()
            sur.close()
        print(json.dumps({"profile": kind, "ms_per_step": t_ms, "steps": args.steps, "warmup": args.warmup}))
        return

    # ---- workload on the device (weak scaling: every rank owns its own
    # 64x64 block of coarse cells, shifted by the rank along x)
    prob = W.fourier_square(K=args.coarse, N=N_FINE)
    ws2 = make_ws(prob, rank)
    n_cells, size, corners_h = ws2["n"], ws2["size"], ws2["corners_h"]
    solves_rank = 4 * n_cells
    M_d, F_d = ws2["M"], ws2["F"]

    def timed(precision, steps, warmup, sample_clocks=False):
        return timed_ws(ws2, precision, steps, warmup, sample_clocks)

    def autotune_ws(ws, precision, sample=1024):
        """The library's autotuner on a prefix of the workload (untimed); the
        choice stays in the handle for every later call with the same key."""
        d = device_desc(ws, precision)
        t = abi.Tuning()
        rc = eng.lib.msfem_autotune(eng.handle, ctypes.byref(d), sample, ctypes.byref(t))
        if rc != abi.OK:
            raise abi.MsfemError(rc, abi.last_error(eng.lib))
        return t.as_dict()

    # ---- FP64 form (headline)
    tune64 = autotune_ws(ws2, abi.PREC_FP64)
    ms64, st64, clocks = timed(abi.PREC_FP64, args.steps, args.warmup, sample_clocks=True)
    value = pkg.sharding.job_throughput(world * solves_rank, ms64 * 1e-3)
    probe = load_probe(pkg)
    fp64_peak = ctypes.c_double(0.0)
    fp32_peak = ctypes.c_double(0.0)
    probe_sampler = ClockSampler(local)
    probe.msfem_probe_fma_flops(1, ctypes.byref(fp64_peak))
    probe.msfem_probe_fma_flops(0, ctypes.byref(fp32_peak))
    probe_clocks = probe_sampler.stop()
    flops64 = (st64["iterations_total"] * flops_per_solve_iter(N_FINE)
               + n_cells * flops_one_off_per_cell(N_FINE))
    achieved = flops64 / (ms64 * 1e-3) / 1e12
    peaks, peak_src = read_peaks()
    alg_bytes = size * 8 + n_cells * (8 * 2 * 4 + 8 * 20 + 4 * 5)  # field + corners + outputs
    traffic = read_profile_traffic("msfem2d_fp64_fourier64x64.txt")
    roofline = {
        "bound": "fp64", "achieved": achieved, "peak": fp64_peak.value / 1e12, "unit": "TFLOP/s",
        "frac": achieved / (fp64_peak.value / 1e12),
        "traffic": traffic,
        "peak_source": "measured in this run: FP64 FMA probe (libmsfem_probe.so), 8 independent "
                       "FMA chains per thread, 8 CTAs x 256 threads per SM",
        "peak_method": {"kernel": "fma_chain<double>", "ctas": "8 per SM", "threads": 256,
                        "fma_per_thread": 8 * 4096, "launches": "1 warm-up + 3 timed, best of 3",
                        "launch_ms": (2.0 * 8 * 4096 * 256 * 8
                                      * torch.cuda.get_device_properties(local).multi_processor_count
                                      / fp64_peak.value * 1e3) if fp64_peak.value else None,
                        "clocks_during_probe": probe_clocks,
                        "note": "MEASURED_PEAKS.json has no FP64 figure; the FP64 pipe bounds this kernel"},
        "kernel": "msfem2d_kernel<32,256,FP64>",
        "flops_per_launch": flops64,
        "algorithmic_bytes_per_launch": alg_bytes,
        "hbm": {"achieved": alg_bytes / (ms64 * 1e-3) / 1e9, "peak": peaks.get("hbm_gbs"),
                "unit": "GB/s", "frac": alg_bytes / (ms64 * 1e-3) / 1e9 / peaks.get("hbm_gbs", 1),
                "peak_source": peak_src},
    }
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms64, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded random-Fourier SPD coefficient, tabulated at Gauss points)",
        "config": {"workload": WORKLOAD if args.coarse == K_COARSE else
                   WORKLOAD.replace("64x64", f"{args.coarse}x{args.coarse}"),
                   "precision": "fp64", "coarse_cells_per_gpu": n_cells,
                   "fine_cells_per_coarse": N_FINE * N_FINE, "rhs_per_cell": 4,
                   "solves_per_step_per_gpu": solves_rank, "tol": TOL,
                   "l2": "inputs larger than L2 (403 MB tabulated field per step)",
                   "parallelism": f"replicas: {world} GPU(s), cells sharded, no collective"},
        "roofline": roofline,
        "gpu_launches": args.steps * st64["kernel_launches"],
        "clocks": clocks,
        "stats": {"mean_iterations": st64["iterations_total"] / max(1, st64["solves"]),
                  "max_iterations": st64["iterations_max"],
                  "max_rel_residual": st64["max_rel_residual"],
                  "cells_failed": st64["cells_failed"], "ctas_per_sm": st64["ctas_per_sm"], "tuning": tune64},
    }
    M64 = M_d.cpu().numpy().copy()
    # ---- mixed form
    if not args.no_mixed:
        tunemx = autotune_ws(ws2, abi.PREC_MIXED)
        msmx, stmx, _ = timed(abi.PREC_MIXED, args.steps, args.warmup)
        line["mixed"] = {
            "tuning": tunemx,
            "value": world * solves_rank / (msmx * 1e-3), "ms_per_step": msmx,
            "speedup_vs_fp64": ms64 / msmx,
            "mean_inner_iterations": stmx["iterations_total"] / max(1, stmx["solves"]),
            "max_refinements": stmx["refinements_max"],
            "max_rel_residual": stmx["max_rel_residual"], "cells_failed": stmx["cells_failed"],
            "fp32_peak_tflops": fp32_peak.value / 1e12,
        }
        # achieved FP32 work of the inner loop (algorithmic flops per inner
        # iteration times the iterations executed) over the whole step time
        fl32 = stmx["iterations_total"] * inner_flops_per_iter(N_FINE, int(tunemx.get("poly_degree", 0)),
                                                              int(tunemx.get("coarse_spacing", 0)))
        line["mixed"]["inner_fp32_tflops"] = fl32 / (msmx * 1e-3) / 1e12
        line["mixed"]["inner_fp32_frac_of_measured_peak"] = line["mixed"]["inner_fp32_tflops"] / (fp32_peak.value / 1e12)
    # ---- e2e through the public C-ABI with pinned host buffers
    if not args.no_e2e:
        tab_h = torch.empty(size, dtype=torch.float64, pin_memory=True)
        tab_h.copy_(ws2["tab_d"].cpu())
        corners_pin = torch.from_numpy(np.ascontiguousarray(corners_h)).pin_memory()
        M_h = torch.empty((n_cells, 4, 4), dtype=torch.float64, pin_memory=True)
        F_h = torch.empty((n_cells, 4), dtype=torch.float64, pin_memory=True)
        st_h = torch.empty(n_cells, dtype=torch.int32, pin_memory=True)
        d = device_desc(ws2, abi.PREC_FP64)
        d.memory = abi.MEM_HOST
        d.corners = corners_pin.data_ptr()
        d.coef.qp_values = tab_h.data_ptr()
        for _ in range(2):
            eng.run_desc(d, M_h.data_ptr(), F_h.data_ptr(), None, st_h.data_ptr(), None, stats=False)
        torch.cuda.synchronize()
        barrier()
        e_steps = max(3, args.steps // 2)
        t0 = time.perf_counter()
        for _ in range(e_steps):
            eng.run_desc(d, M_h.data_ptr(), F_h.data_ptr(), None, st_h.data_ptr(), None, stats=False)
        torch.cuda.synchronize()
        e2e_s = max_over_ranks((time.perf_counter() - t0) / e_steps)
        line["e2e"] = {"value": world * solves_rank / e2e_s, "unit": UNIT,
                       "ms_per_step": e2e_s * 1e3,
                       "h2d_bytes_per_step": int(size * 8 + corners_h.nbytes),
                       "d2h_bytes_per_step": int(M_h.numel() * 8 + F_h.numel() * 8 + st_h.numel() * 4)}
        # sanity: host result equals the device-resident one
        line["e2e"]["matches_device"] = bool(np.array_equal(M_h.numpy(), M64))
        line["e2e"]["note"] = ("pinned host table read in place by the kernel over the CPU-GPU link "
                               "(counted in h2d_bytes_per_step); M/F/status copied back")
        # the mixed form through the same host call
        if not args.no_mixed:
            dm = device_desc(ws2, abi.PREC_MIXED)
            dm.memory = abi.MEM_HOST
            dm.corners = corners_pin.data_ptr()
            dm.coef.qp_values = tab_h.data_ptr()
            for _ in range(2):
                eng.run_desc(dm, M_h.data_ptr(), F_h.data_ptr(), None, st_h.data_ptr(), None, stats=False)
            torch.cuda.synchronize()
            barrier()
            t0 = time.perf_counter()
            for _ in range(e_steps):
                eng.run_desc(dm, M_h.data_ptr(), F_h.data_ptr(), None, st_h.data_ptr(), None, stats=False)
            torch.cuda.synchronize()
            e2e_m = max_over_ranks((time.perf_counter() - t0) / e_steps)
            line["mixed"]["e2e"] = {"value": world * solves_rank / e2e_m, "unit": UNIT, "ms_per_step": e2e_m * 1e3,
                                    "h2d_bytes_per_step": line["e2e"]["h2d_bytes_per_step"],
                                    "d2h_bytes_per_step": line["e2e"]["d2h_bytes_per_step"]}
    # ---- 256x256 coarse cells (65536) of the evaluation Fourier field, mixed vs FP64
    if not args.no_fourier_256 and world == 1 and args.coarse == K_COARSE:
        ws3 = make_ws(W.fourier_square(K=256, N=32, seeds=W.EVAL_SEEDS), 0)
        st3 = max(2, min(5, args.steps))
        ms3m, s3m, _ = timed_ws(ws3, abi.PREC_MIXED, st3, 3)
        ms3f, s3f, _ = timed_ws(ws3, abi.PREC_FP64, 2, 3)
        n3 = ws3["n"]
        line["fourier_256x256"] = {
            "workload": "2D 256x256 coarse cells, 32x32 fine Q1, 4 RHS, random-Fourier SPD tensor "
                        "(seeds 3/30/300), f=1, 1e-10 rel residual",
            "mixed": {"value": 4 * n3 / (ms3m * 1e-3), "unit": UNIT, "ms_per_step": ms3m,
                      "mean_inner_iterations": s3m["iterations_total"] / max(1, s3m["solves"]),
                      "max_refinements": s3m["refinements_max"],
                      "max_rel_residual": s3m["max_rel_residual"], "cells_failed": s3m["cells_failed"]},
            "fp64": {"value": 4 * n3 / (ms3f * 1e-3), "unit": UNIT, "ms_per_step": ms3f,
                     "mean_iterations": s3f["iterations_total"] / max(1, s3f["solves"]),
                     "max_rel_residual": s3f["max_rel_residual"], "cells_failed": s3f["cells_failed"]},
            "speedup_mixed_vs_fp64": ms3f / ms3m,
        }
        line["gpu_launches_fourier_256x256"] = st3 + 2
        # field generation: the random-Fourier tensor tabulated at the Gauss
        # points on the device (phase recurrence along lattice rows)
        tt = tab_times.get(ws3["n"])
        if tt:
            line["fourier_256x256"]["tabulation"] = {
                "ms": tt["ms"], "bytes_written": tt["bytes"],
                "hbm_frac_of_measured": tt["bytes"] / (tt["ms"] * 1e-3) / 1e9 / read_peaks()[0].get("hbm_gbs", 1),
                "note": "3 fields x 64 modes per Gauss point in FP64; bound by the FP64 pipe, not HBM"}
        # per-basis energy-norm and coarse-matrix errors of every cell against
        # the FP64 form solved to 1e-12 (untimed)
        ref3 = solve_with_basis(ws3, abi.PREC_FP64, 1e-12)
        errs = {}
        for prec, pname in ((abi.PREC_MIXED, "mixed"), (abi.PREC_FP64, "fp64")):
            errs[pname] = basis_errors(ws3, solve_with_basis(ws3, prec, TOL), ref3)
        line["fourier_256x256"]["errors_vs_fp64_1e-12"] = {
            "reference": "FP64 form solved to 1e-12 relative residual, same cells and field; "
                         "energy norm ||phi - phi_ref||_A / ||phi_ref||_A per basis function, "
                         "coarse entries |M_ij - M_ref,ij| / max_ij |M_ref,ij| per cell",
            "reference_max_rel_residual": ref3["stats"]["max_rel_residual"], **errs}
        del ws3
        if args.no_surrogate:
            del ref3
        torch.cuda.empty_cache()
    # ---- 3D unit cube, 16^3 coarse cells with uneven N in {8,16,24},
    # 1e4-contrast spheres, 8 RHS; one persistent kernel per call, autotuned
    # on a sample of the batch, FP64 and mixed
    if not args.no_spheres_3d and world == 1 and args.coarse == K_COARSE:
        t0 = time.time()
        prob4 = W.spheres_cube()
        t_rsa = time.time() - t0
        nc4 = prob4["corners"].shape[0]
        nf4_h = np.ascontiguousarray(prob4["n_fine_per_cell"], dtype=np.int32)
        corners4 = torch.from_numpy(np.ascontiguousarray(prob4["corners"])).to(f"cuda:{local}")
        nf4 = torch.from_numpy(nf4_h).to(f"cuda:{local}")
        sp4 = np.ascontiguousarray(prob4["coef"]["spheres"])
        size4 = int(np.sum(8 * nf4_h.astype(np.int64) ** 3))
        tab4 = torch.empty(size4, dtype=torch.float64, device=f"cuda:{local}")
        dt = abi.BatchDesc()
        dt.dim, dt.n_cells, dt.n_fine = 3, nc4, 24
        dt.corners, dt.n_fine_per_cell = corners4.data_ptr(), nf4.data_ptr()
        dt.coef.kind = abi.COEF_SPHERES
        dt.coef.params[0] = float(prob4["coef"]["params"][0])
        dt.coef.spheres = sp4.ctypes.data
        dt.coef.n_spheres = sp4.shape[0]
        dt.memory = abi.MEM_DEVICE
        dt.f_value, dt.tol, dt.maxit = 1.0, TOL, 1000
        rc = eng.lib.msfem_tabulate_coefficient(eng.handle, ctypes.byref(dt), 1, tab4.data_ptr())
        if rc != abi.OK:
            raise abi.MsfemError(rc, abi.last_error(eng.lib))

        def desc4(precision, n=nc4):
            d = abi.BatchDesc()
            d.dim, d.n_cells, d.n_fine = 3, n, 24
            d.precision = precision
            d.corners, d.n_fine_per_cell = corners4.data_ptr(), nf4.data_ptr()
            d.coef.kind, d.coef.ncomp, d.coef.qp_values = abi.COEF_TABULATED, 1, tab4.data_ptr()
            d.f_value, d.tol, d.maxit, d.memory = 1.0, TOL, 1000, abi.MEM_DEVICE
            return d

        M4 = torch.empty((nc4, 8, 8), dtype=torch.float64, device=f"cuda:{local}")
        F4 = torch.empty((nc4, 8), dtype=torch.float64, device=f"cuda:{local}")
        st4 = torch.empty(nc4, dtype=torch.int32, device=f"cuda:{local}")
        it4 = torch.empty((nc4, 8), dtype=torch.int32, device=f"cuda:{local}")
        res4 = {"workload": "3D 16^3 coarse cells, N per cell uniform over {8,16,24} (seed 4), "
                            "a = 1 + (1e4 - 1) [x in spheres], spheres r in [0.004, 0.012] at volume "
                            "fraction 0.2 (seed 44, random sequential addition), f=1, 8 RHS, "
                            "1e-10 rel residual",
                "cells_by_N": {str(v): int((nf4_h == v).sum()) for v in (8, 16, 24)},
                "spheres": int(sp4.shape[0]), "sphere_generation_s": t_rsa}
        for prec, pname in ((abi.PREC_FP64, "fp64"), (abi.PREC_MIXED, "mixed")):
            # autotune on the first half of the batch (the same N mix; a
            # sample large enough that every CTA works through several cells,
            # as in the full batch), then time the batch
            tn = abi.Tuning()
            n_tune = nc4 // 2
            rc = eng.lib.msfem_autotune(eng.handle, ctypes.byref(desc4(prec, n_tune)), n_tune, ctypes.byref(tn))
            if rc != abi.OK:
                raise abi.MsfemError(rc, abi.last_error(eng.lib))
            d = desc4(prec)
            outs = (M4.data_ptr(), F4.data_ptr(), None, st4.data_ptr(), it4.data_ptr())
            eng.run_desc(d, *outs, stats=False)  # warm-up
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.run_desc(d, *outs, stats=False)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            _, s4 = eng.run_desc(d, *outs, stats=True)
            it_h = it4.cpu().numpy()
            res4[pname] = {"value": 8 * nc4 / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms,
                           "mean_iterations": s4["iterations_total"] / s4["solves"],
                           "mean_iterations_by_N": {str(v): float(it_h[nf4_h == v].mean()) for v in (8, 16, 24)},
                           "max_refinements": s4["refinements_max"],
                           "max_rel_residual": s4["max_rel_residual"], "cells_failed": s4["cells_failed"],
                           "tuning": tn.as_dict()}
            # algorithmic CG work of the step (per solve: its iterations x the
            # per-iteration flops of its N) against the FP64 / FP32 FMA peak
            flw = float(sum(int(it_h[c].sum()) * flops_per_solve_iter_3d(int(nf4_h[c])) for c in range(nc4)))
            peak = fp64_peak.value if prec == abi.PREC_FP64 else fp32_peak.value
            res4[pname]["cg_tflops"] = flw / (ms * 1e-3) / 1e12
            res4[pname]["cg_frac_of_measured_" + ("fp64" if prec == abi.PREC_FP64 else "fp32") + "_peak"] = \
                flw / (ms * 1e-3) / peak
        res4["speedup_mixed_vs_fp64"] = res4["fp64"]["ms_per_step"] / res4["mixed"]["ms_per_step"]
        # per-basis energy errors and coarse-matrix errors of both forms
        # against the FP64 form solved to 1e-12 (untimed)
        bsz4 = int(np.sum(8 * (nf4_h.astype(np.int64) + 1) ** 3))

        def solve4(precision, tol):
            d = desc4(precision)
            d.tol = tol
            out = {"M": torch.empty((nc4, 8, 8), dtype=torch.float64, device=f"cuda:{local}"),
                   "F": torch.empty((nc4, 8), dtype=torch.float64, device=f"cuda:{local}"),
                   "basis": torch.empty(bsz4, dtype=torch.float64, device=f"cuda:{local}")}
            _, out["stats"] = eng.run_desc(d, out["M"].data_ptr(), out["F"].data_ptr(), out["basis"].data_ptr(),
                                           st4.data_ptr(), it4.data_ptr(), stats=True)
            return out

        ref4 = solve4(abi.PREC_FP64, 1e-12)
        res4["errors_reference"] = ("FP64 form solved to 1e-12 relative residual (max "
                                    f"{ref4['stats']['max_rel_residual']:.2e}); energy norm ||phi - phi_ref||_A / "
                                    "||phi_ref||_A per basis function, |M_ij - M_ref,ij| / max |M_ref| per cell")
        for prec, pname in ((abi.PREC_FP64, "fp64"), (abi.PREC_MIXED, "mixed")):
            got4 = solve4(prec, TOL)
            res4[pname]["errors_vs_fp64_1e-12"] = basis_errors(None, got4, ref4, desc=desc4(abi.PREC_FP64))
            del got4
        del ref4
        line["spheres_3d"] = res4
        del tab4, M4, F4, st4, it4, corners4, nf4
        torch.cuda.empty_cache()
    # ---- learned warm start (the surrogate): trained here with the library's
    # own BF16 tensor-core forward/backward kernels, evaluated on the unseen
    # 256x256-cell evaluation field (65536 cells) against the cold start
    if not args.no_surrogate and world == 1 and args.coarse == K_COARSE:
        S = pkg.surrogate
        t0 = time.time()
        feats, tgts = S.training_set(eng, torch)
        torch.cuda.synchronize()
        t_data = time.time() - t0
        sur = S.Surrogate(eng, seed=1)
        t0 = time.time()
        hist = S.train(sur, feats, tgts, torch, epochs=20, batch=256, lr=1e-3)
        torch.cuda.synchronize()
        t_train = time.time() - t0
        del feats, tgts
        desc5, keep5 = S.device_problem(eng, W.fourier_square(K=256, N=32, seeds=W.EVAL_SEEDS), torch)
        ev = {}
        for prec, pname in ((abi.PREC_MIXED, "mixed"), (abi.PREC_FP64, "fp64")):
            for warm, wname in ((abi.WARM_NONE, "cold"), (abi.WARM_SURROGATE, "surrogate")):
                if warm == abi.WARM_SURROGATE:
                    sur.attach()
                S.solve_device(eng, desc5, torch, precision=prec, warm=warm)  # warm-up
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                r = S.solve_device(eng, desc5, torch, precision=prec, warm=warm)
                e1.record(stream)
                torch.cuda.synchronize()
                sur.detach()
                st = r["stats"]
                ms = e0.elapsed_time(e1)
                ev[f"{pname}_{wname}"] = {
                    "value": st["solves"] / (ms * 1e-3), "unit": UNIT, "ms": ms,
                    "mean_iterations": st["iterations_total"] / st["solves"],
                    "max_rel_residual": st["max_rel_residual"], "cells_failed": st["cells_failed"]}
        if not args.no_fourier_256:
            sur.attach()
            for prec, pname in ((abi.PREC_MIXED, "mixed"), (abi.PREC_FP64, "fp64")):
                got = solve_with_basis(None, prec, TOL, warm=abi.WARM_SURROGATE, desc=desc5)
                ev[f"{pname}_surrogate"]["errors_vs_fp64_1e-12"] = basis_errors(None, got, ref3, desc=desc5)
                del got
            sur.detach()
            del ref3
        # cost of the prediction itself, timed apart: node features and the
        # network's forward pass over all 65536 cells (the warm-started solve
        # also composes Q1 + delta and evaluates the FP64 initial residual)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e2 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        f5 = S.features(eng, desc5, torch)
        e1.record(stream)
        p5 = torch.empty((desc5.n_cells, 4, 33, 33), dtype=torch.float32, device=f"cuda:{local}")
        sur.predict(f5, p5)
        e2.record(stream)
        torch.cuda.synchronize()
        infer = {"features_ms": e0.elapsed_time(e1), "network_ms": e1.elapsed_time(e2)}
        del f5, p5
        for pname in ("mixed", "fp64"):
            c, w = ev[f"{pname}_cold"], ev[f"{pname}_surrogate"]
            w["iterations_saved"] = 1.0 - w["mean_iterations"] / c["mean_iterations"]
            w["speedup_vs_cold"] = c["ms"] / w["ms"]
            # what the fewer iterations save, against what the prediction costs
            w["breakdown_ms"] = {"cold_solve": c["ms"], "warm_total": w["ms"], **infer,
                                 "warm_without_prediction": w["ms"] - infer["features_ms"] - infer["network_ms"],
                                 "saved_by_fewer_iterations": c["ms"] - (w["ms"] - infer["features_ms"]
                                                                         - infer["network_ms"])}
        ev["mixed_surrogate"]["speedup_vs_fp64_cold"] = ev["fp64_cold"]["ms"] / ev["mixed_surrogate"]["ms"]
        line["surrogate"] = {
            "network": "6 conv3x3 layers 3-32-32-32-32-32-4, dilations 1/2/4/8/2/1, BF16 weights and "
                       "activations, FP32 accumulation (tcgen05.mma kind::f16, TMEM accumulators, TMA-staged windows) "
                       "for the forward pass, the input gradient and the weight/bias gradient; Adam lr 1e-3",
            "training": {"solves": int(4 * 12 * 4096), "epochs": 20, "batch": 256,
                         "data_seconds": t_data, "train_seconds": t_train,
                         "loss_first_epoch": hist[0], "loss_last_epoch": hist[-1]},
            "eval_workload": "256x256-cell random-Fourier field (seeds 3/30/300, not in the training set), 65536 cells",
            "results": ev,
        }
        sur.close()
        del keep5
        torch.cuda.empty_cache()
    # ---- CPU baseline (rank 0, N = 1 only)
    if rank == 0 and world == 1 and not args.no_cpu:
        oracle = graft.load_oracle()
        oracle.build()
        nthreads = os.cpu_count() or 1
        n_sample = max(16, min(2048, 128 * nthreads))
        cells = np.linspace(0, n_cells - 1, n_sample).astype(int)
        sample = W.subset(prob, cells)
        # passes over the sample repeat until about 10 s of wall time have run
        solves, times, res = cpu_reference(pkg, oracle, sample, nthreads, steps=1, warmup=0, min_seconds=10.0)
        cv = solves * len(times) / sum(times)
        line["cpu_baseline"] = {
            "value": cv, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{n_sample} of {n_cells} coarse cells ({solves} solves) x {len(times)} passes, "
                      "SSOR(1.6)-PCG to 1e-10 rel, CSR, QGauss(2) assembly, 16-SpMV epilogue",
            "seconds": sum(times), "mean_iterations": float(res["iters"].mean())}
        # parity of the sampled cells against the GPU result
        got_M = M64[cells]
        line["cpu_baseline"]["max_rel_diff_M_vs_gpu"] = float(
            np.abs(got_M - res["M"]).max() / np.abs(res["M"]).max())
    if rank == 0:
        print(json.dumps(line))
    eng.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
