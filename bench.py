#!/usr/bin/env python
"""MGPCG time-to-solve on one GB300 (SGLDBench's solve path).

Workload (default): the SIMP-graded 256 x 128 x 128 cantilever -- a solid
cuboid of 4,194,304 voxels (12,830,211 DOFs), densities = seeded U[0,1) noise
Gaussian-smoothed (sigma 2 voxels) and mapped to [1e-3, 1], E = 1e-9 +
rho^3 (1 - 1e-9), nu = 0.3, all nodes at x = 0 fixed, a unit -z load spread
over the x = max bottom edge, 5 dyadic multigrid levels, damped Jacobi
omega = 0.6, PCG to relative residual 1e-6.  Synthetic, seeded inputs stand
in for the reference's voxelized models.

One step = one full solve for a given modulus field: set E, assemble the
Galerkin hierarchy and the coarsest factor, run PCG to 1e-6.  `value` is the
device time per step with E and F already in HBM, for the mixed-precision
solve (FP64 flexible PCG, FP32 inner CG with the FP32 V-cycle, double-float
outer K*u) unless --precision says otherwise; `plain_fp64` is the reference
form (FP64 PCG, FP64 V-cycle) timed the same way right after; `e2e` is the
headline solve through the public C ABI with host buffers (E and F copied in,
U copied out).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision fp64|mixed|mixed_df] [--size NX NY NZ]

Under torchrun (N > 1) every rank solves its own replica on its own GPU (the
solve path has no data-parallel split; replicas only) and rank 0 reports.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MGPCG time-to-solve at rel.res 1e-6, mixed+learned vs plain FP64, 1 GB300"
TOL = 1e-6
OMEGA = 0.6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["fp64", "mixed", "mixed_df"], default="mixed_df")
    ap.add_argument("--fp64-steps", type=int, default=2, help="plain FP64 solves timed beside the headline")
    ap.add_argument("--size", type=int, nargs=3, default=[256, 128, 128], metavar=("NX", "NY", "NZ"))
    ap.add_argument("--levels", type=int, default=5)
    ap.add_argument("--maxit", type=int, default=2000)
    ap.add_argument("--inner-its", type=int, default=0,
                    help="initial cap on the FP32 inner CG iterations per outer step of the mixed solves (0 = "
                         "library default 64, doubled after a capped inner solve up to 16x); exact count when "
                         "--inner-tol is 0 and this is > 0")
    ap.add_argument("--inner-tol", type=float, default=0.0,
                    help="inner CG stops at ||s|| <= inner_tol ||r|| (0 = library default 3e-4)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-iters", type=int, default=5, help="PCG iterations in the CPU sample")
    return ap.parse_args()


def workload(nx, ny, nz):
    from sgldbench_gb300 import domains as D

    vox = D.cuboid(nx, ny, nz)
    rho = D.graded_density(nx, ny, nz, seed=0, sigma=2.0, rho_min=1e-3)
    E = D.simp_modulus(rho, E0=1.0, Emin=1e-9, p=3.0)
    return vox, E


def workload_config(args):
    nx, ny, nz = args.size
    return {"workload": f"SIMP-graded cantilever {nx}x{ny}x{nz} voxels (config 1)", "grid": [nx, ny, nz],
            "levels": args.levels, "dyadic": True, "omega": OMEGA, "tol": TOL, "precision": args.precision,
            "inner_its": args.inner_its, "inner_tol": args.inner_tol,
            "l2": "inputs larger than L2 (each DOF vector > 100 MB at the default size)"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
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
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU path (oracle): restated reference, timed on a bounded sample
# ---------------------------------------------------------------------------
def cpu_time_to_solve(vox, E, levels, its_full, sample_iters, steps=1, warmup=0):
    """Times the oracle (C + numpy restatement of the reference's MEX kernels
    and MATLAB glue) on the host cores: assembly + `sample_iters` PCG
    iterations, extrapolated to `its_full` iterations.  Returns a dict."""
    from oracle import glue as G

    t0 = time.perf_counter()
    m = G.build_model(vox, non_dyadic=0, omega=OMEGA, num_levels=levels)
    t_setup = time.perf_counter() - t0
    G.set_modulus(m, E)
    spent = {"kbyu": 0.0, "vcycle": 0.0}

    def timed(name, fn):
        def call(v):
            t = time.perf_counter()
            out = fn(v)
            spent[name] += time.perf_counter() - t
            return out
        return call

    AtX = timed("kbyu", lambda u: G.kbyu(m, u))
    PtV = timed("vcycle", lambda r: G.vcycle(m, r))
    times = []
    for k in range(warmup + steps):
        t0 = time.perf_counter()
        G.assemble_stencil(m)
        spent["kbyu"] = spent["vcycle"] = 0.0
        t1 = time.perf_counter()
        G.pcg(AtX, PtV, m.F, 0.0, sample_iters)
        t2 = time.perf_counter()
        if k >= warmup:
            times.append((t1 - t0, (t2 - t1) / sample_iters, spent["kbyu"] / sample_iters,
                          spent["vcycle"] / sample_iters))
    t_asm, t_it, t_kbyu, t_vc = (float(np.mean([t[i] for t in times])) for i in range(4))
    # the SpMV / PtV / rest split of QuickAccess/zTmp_Benchmarking_SpMV.m:63-111, per iteration
    return {"seconds": t_asm + t_it * its_full, "assemble_s": t_asm, "iter_s": t_it, "kbyu_s": t_kbyu,
            "vcycle_s": t_vc, "glue_s": t_it - t_kbyu - t_vc, "setup_s": t_setup,
            "levels": m.numLevels, "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    nx, ny, nz = args.size
    vox, E = workload(nx, ny, nz)
    its_full = _known_iterations(args)
    r = cpu_time_to_solve(vox, E, args.levels, its_full, args.cpu_iters, steps=args.steps,
                          warmup=min(args.warmup, 1))
    from oracle import mexcall

    kind = "reference" if mexcall.ref_lib() is not None else "port"
    line = {"impl": "reference", "metric": METRIC, "value": r["seconds"], "unit": "s", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["seconds"] * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded graded-density cuboid)", "config": workload_config(args),
            "cpu_baseline": {"value": r["seconds"], "unit": "s", "cores": r["cores"], "kind": kind,
                             "sample": f"assembly + {args.cpu_iters} PCG iterations per step, "
                                       f"extrapolated to {its_full} iterations"},
            "e2e": {"value": r["seconds"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "detail": r}
    print(json.dumps(line), flush=True)


def _known_iterations(args):
    """Iteration count of the FP64 solve of this workload.  The GPU solve and the
    oracle run the same algorithm (equal counts in the parity tests), and a full
    oracle solve does not fit a bounded CPU sample, so the count recorded from
    the GPU run (profiles/iterations.json) is used to extrapolate."""
    path = os.path.join(ROOT, "profiles", "iterations.json")
    key = "x".join(map(str, args.size)) + f"_L{args.levels}"
    try:
        with open(path) as f:
            return int(json.load(f)[key])
    except (OSError, KeyError, ValueError):
        return 100


# ---------------------------------------------------------------------------
# GPU path
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch

    from sgldbench_gb300 import VoxelSolver, replicas
    from sgldbench_gb300 import domains as D
    from sgldbench_gb300.solver import kernel_launches

    rank, world, local = replicas.dist_env()
    torch.cuda.set_device(local)
    replicas.init("nccl")
    nx, ny, nz = args.size
    vox, E = workload(nx, ny, nz)
    s = VoxelSolver(vox, num_levels=args.levels, non_dyadic=0, omega=OMEGA, device=local, pad=False)
    nodes = s.nodMapBack(1)
    F, fixed = D.cantilever3(vox, nodes)
    s.set_fixed_dofs(fixed)
    dev = torch.device("cuda", local)
    E_d = torch.from_numpy(E).to(dev)
    F_d = torch.from_numpy(F).to(dev)
    U_d = torch.zeros_like(F_d)
    stream = torch.cuda.ExternalStream(s.stream, device=dev)

    def step(profile=False):
        s.set_modulus_device(E_d.data_ptr())
        s.Solving_AssembleFEAstencil()
        return s.pcg_device(F_d.data_ptr(), U_d.data_ptr(), TOL, args.maxit, precision=args.precision,
                            inner_its=args.inner_its, inner_tol=args.inner_tol, profile=profile)

    for _ in range(max(args.warmup, 0)):
        info = step()
    sampler = ClockSampler(local)
    sampler.start()
    replicas.barrier()
    torch.cuda.synchronize()
    l0 = kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    infos = []
    for _ in range(args.steps):
        infos.append(step())
    e1.record(stream)
    torch.cuda.synchronize()
    launches = (kernel_launches() - l0) / max(args.steps, 1)
    clocks = sampler.stop()
    t_step = e0.elapsed_time(e1) / 1e3 / args.steps
    replicas.barrier()
    torch.cuda.synchronize()
    # the slowest replica's time per solve; every rank solved `steps` replicas
    t_step, solves = replicas.aggregate(t_step, args.steps, device=dev)
    its = infos[-1]["its"]
    # split: one profiled solve (outer K*u launches timed with events on the library stream)
    pinfo = step(profile=True)
    # the reference form, same workload, timed the same way (device events)
    fp64 = None
    if args.precision != "fp64" and args.fp64_steps > 0:
        def step64():
            s.set_modulus_device(E_d.data_ptr())
            s.Solving_AssembleFEAstencil()
            return s.pcg_device(F_d.data_ptr(), U_d.data_ptr(), TOL, args.maxit, precision="fp64")
        step64()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        f0.record(stream)
        for _ in range(args.fp64_steps):
            i64 = step64()
        f1.record(stream)
        torch.cuda.synchronize()
        t64 = f0.elapsed_time(f1) / 1e3 / args.fp64_steps
        fp64 = {"value": t64, "unit": "s", "iterations": i64["its"], "true_relres": i64["true_relres"],
                "steps": args.fp64_steps, "speedup_of_headline": t64 / t_step}
    # end to end through the public API with host buffers (page-locked, as a
    # caller streaming load cases would hold them)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    E_h = torch.from_numpy(E).pin_memory().numpy()
    F_h = torch.from_numpy(F).pin_memory().numpy()
    U_h = torch.zeros(F.size, dtype=torch.float64).pin_memory().numpy()
    def step_e2e():
        s.set_modulus(E_h)
        s.Solving_AssembleFEAstencil()
        return s.pcg(F_h, tol=TOL, maxIT=args.maxit, precision=args.precision, inner_its=args.inner_its,
                     inner_tol=args.inner_tol, out=U_h)

    # warm-up of the host-buffer path too: its first calls pay one-time costs
    # (pinned-buffer registration lookups, the host entry point's first solve)
    for _ in range(max(args.warmup, 0)):
        step_e2e()
    e2e = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0.record(stream)
        U_h, inf = step_e2e()
        t1.record(stream)
        torch.cuda.synchronize()
        e2e.append(t0.elapsed_time(t1) / 1e3)
    h2d = E.nbytes + F.nbytes
    d2h = U_h.nbytes
    ndof = s.numDOFs
    # roofline of the dominant kernel: the K*u of the solve's inner loop
    NN = (nx + 1) * (ny + 1) * (nz + 1)
    NE = nx * ny * nz
    peaks = _peaks()
    if args.precision == "fp64":
        kname, kbytes = "k_kbyu<double> (FP64 K*u)", NN * (3 * 8 * 2 + 1) + NE * 8
        kb_avg = pinfo["kbyu_seconds"] / max(pinfo["kbyu_launches"], 1)
        how = "CUDA events around every K*u launch of one solve on the library stream"
        note = "FP64 K*u is FP64-issue-bound on GB300 (ncu: FP64 pipe ~84 % busy)"
    else:
        kname, kbytes = "k_kbyu_x2 (FP32 K*u of the inner CG, f32x2 packed)", NN * (3 * 4 * 2 + 1) + NE * 4
        kb_avg = s.time_op("kbyu32", 20) * 1e-3
        how = ("CUDA events around 20 back-to-back launches on the library stream (sgld_time_op) right after "
               "the timed region; inside the timed region the kernel runs in the inner CG's graph")
        note = ("FP32 K*u is issue/latency-bound, not HBM-bound; the HBM fraction is reported against the "
                "measured copy bandwidth. Autotuned tile: %s" % json.dumps(s.kbyu_tile()))
    achieved = kbytes / kb_avg / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": _ncu_traffic(args.precision),
                "kernel": kname, "avg_launch_ms": kb_avg * 1e3, "launch_timing": how,
                "algorithmic_bytes_per_launch": kbytes, "peak_source": peaks["source"],
                "dense_equiv_tflops": 1152.0 * NE / kb_avg / 1e12, "note": note}
    line = {"metric": METRIC, "value": t_step, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": {"fp64": "f64", "mixed": "f64+f32", "mixed_df": "f64+f32+df32"}[args.precision],
            "data": "synthetic (seeded graded-density cuboid)", "config": workload_config(args),
            "iterations": its, "dof": ndof, "dof_it_per_s": world * ndof * its / t_step,
            "replica_solves_per_s": solves / (t_step * args.steps),
            "split": {"pcg_s": infos[-1]["seconds"], "assemble_s": t_step - infos[-1]["seconds"],
                      "kbyu_s": pinfo["kbyu_seconds"], "precond_s": pinfo["precond_seconds"]},
            "true_relres": infos[-1]["true_relres"], "converged": infos[-1]["converged"],
            "e2e": {"value": float(np.mean(e2e)), "unit": "s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "samples": [round(v, 6) for v in e2e]},
            "gpu_launches": int(round(launches)), "roofline": roofline, "clocks": clocks}
    if fp64:
        line["plain_fp64"] = fp64
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        its_ref = fp64["iterations"] if fp64 else (its if args.precision == "fp64" else _known_iterations(args))
        r = cpu_time_to_solve(vox, E, args.levels, its_ref, args.cpu_iters, steps=1, warmup=0)
        line["cpu_baseline"] = {"value": r["seconds"], "unit": "s", "cores": r["cores"], "kind": "port",
                                "sample": f"oracle assembly + {args.cpu_iters} PCG iterations of the reference "
                                          f"(FP64) algorithm, extrapolated to its {its_ref} iterations",
                                "detail": r}
    if rank == 0:
        print(json.dumps(line), flush=True)
    s.close()
    replicas.shutdown()


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured (MEASURED_PEAKS.json)"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "source": "fallback"}


def _ncu_traffic(precision):
    """DRAM bytes per launch of the roofline kernel from the committed ncu
    capture (profiles/kbyu_traffic.json), if recorded."""
    p = os.path.join(ROOT, "profiles", "kbyu_traffic.json")
    try:
        with open(p) as f:
            d = json.load(f)
    except (OSError, ValueError):
        return None
    if precision == "fp64":
        return d.get("dram_bytes_per_launch_full")
    return d.get("k_kbyu_x2", {}).get("dram_bytes_per_launch")


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
