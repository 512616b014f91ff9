#!/usr/bin/env python
"""MGPCG time-to-solve on one GB300 (SGLDBench's solve path): the large stress
analysis with a learned start for held-out load cases.

Workload (default): a 1024 x 512 x 512 voxel box holding a seeded random
smooth shape -- the sum of 64 Gaussian blobs thresholded to keep ~30 % of the
voxels, largest face-connected component (about 231 M DOFs) -- E = 1, nu = 0.3,
all nodes of the lowest 4 voxel layers fixed, 7 dyadic multigrid levels, damped
Jacobi omega = 0.6, PCG to relative residual 1e-6.  Load cases are perturbed
versions of one surface load (a unit force spread over the boundary nodes
within 10 voxels of a centre; the centre moves by up to 8 voxels and the
direction turns by up to 30 degrees between cases).  Synthetic, seeded inputs
stand in for the reference's voxelized models.

Protocol: 20 training cases are solved first and teach the learned start
(sgld_cases_*: a K-orthonormal basis of their solutions and a coarse-level
U-Net trained on the corrections the solves found); then each step solves one
held-out case from the learned start with the mixed-precision solve (FP64
flexible PCG, FP32 inner CG with the FP32 V-cycle, double-float outer K*u).
`value` is the device time per held-out solve with the loads resident in HBM;
`e2e` the same through the host-buffer C ABI call (load copied in, U copied
out); `plain_fp64` the reference form (FP64 PCG and V-cycle from zero) on the
same case; `learned` compares the held-out cases' starts (zero, basis only,
basis + network).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--size NX NY NZ] [--levels L] [--train T]

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


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, nargs=3, default=[1024, 512, 512], metavar=("NX", "NY", "NZ"))
    ap.add_argument("--levels", type=int, default=7)
    ap.add_argument("--fill", type=float, default=0.3)
    ap.add_argument("--blobs", type=int, default=64)
    ap.add_argument("--train", type=int, default=20, help="training load cases solved before the held-out ones")
    ap.add_argument("--held-out", type=int, default=20, help="distinct held-out load cases (steps cycle over them)")
    ap.add_argument("--precision", choices=["mixed", "mixed_df"], default="mixed_df")
    ap.add_argument("--maxit", type=int, default=20000)
    ap.add_argument("--fp64-steps", type=int, default=1, help="plain FP64 solves timed beside the headline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-iters", type=int, default=5, help="PCG iterations per CPU sample")
    return ap.parse_args(argv)


def patch_scale(args):
    """Patch radius and centre shift in voxels (10 and 8 at 1024 voxels in x)."""
    f = args.size[0] / 1024.0
    return max(10.0 * f, 2.5), max(8.0 * f, 2.0)


def workload(args):
    from sgldbench_gb300 import domains as D

    nx, ny, nz = args.size
    return D.gaussian_blobs(nx, ny, nz, seed=0, n_blobs=args.blobs, fill=args.fill)


def load_cases(vox, nodes, args):
    from sgldbench_gb300 import domains as D

    radius, shift = patch_scale(args)
    kw = dict(base_seed=0, radius=radius, shift=shift, max_angle_deg=30.0)
    train = D.perturbed_patch_cases(vox, nodes, args.train, seed=1, **kw)
    held = D.perturbed_patch_cases(vox, nodes, args.held_out, seed=2, **kw)
    return train, held


def workload_config(args, extra=None):
    nx, ny, nz = args.size
    radius, shift = patch_scale(args)
    cfg = {"workload": f"stress analysis of {args.blobs} thresholded Gaussian blobs in a {nx}x{ny}x{nz} voxel box "
                       f"(~{args.fill:.0%} solid), learned start for held-out perturbed load cases",
           "grid": [nx, ny, nz], "levels": args.levels, "dyadic": True, "omega": OMEGA, "tol": TOL,
           "precision": args.precision, "train_cases": args.train, "held_out_cases": args.held_out,
           "load": f"unit force over boundary nodes within {radius:g} voxels of a centre moved by up to {shift:g} "
                   "voxels, direction turned by up to 30 degrees", "fixed": "lowest 4 voxel layers",
           "l2": "inputs larger than L2 (each DOF vector > 1 GB)"}
    if extra:
        cfg.update(extra)
    return cfg


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 500 ms while running
    (started before the warm-up, so that its start-up is not in a timed step)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []
        self.marks = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "500"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append((time.monotonic(), ln.strip()))

    def mark(self):
        """Start of a timed region; summary() keeps samples after the first mark."""
        self.marks.append(time.monotonic())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        t0 = self.marks[0] if self.marks else 0.0
        if not any(t >= t0 for t, _ in self.lines):   # a timed region shorter than the interval
            t0 = 0.0
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if t < t0 or len(parts) < 9:
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
                "samples": len(sm), "interval_ms": 500}


# ---------------------------------------------------------------------------
# CPU path (oracle): the restated reference on a bounded sample of the workload
# ---------------------------------------------------------------------------
def crop_of(vox, args):
    """The CPU sample's model: a window of the workload's box, a quarter of
    each extent (at least 32 voxels, at most the extent), centred in x and y
    and resting on z = 0 so that it holds fixed layers, reduced to its largest
    face-connected component.  Returns (voxels, levels)."""
    from sgldbench_gb300 import domains as D

    ny, nx, nz = vox.shape
    cy, cx, cz = (min(n, max(n // 4, 32)) for n in (ny, nx, nz))
    y0, x0 = (ny - cy) // 2, (nx - cx) // 2
    crop = D._largest_component(vox[y0:y0 + cy, x0:x0 + cx, :cz].copy())
    levels = max(2, args.levels - int(round(np.log2(nx / cx))))
    return crop, levels


def cpu_sample(vox, args, iterations, steps=1, warmup=0):
    """Times the oracle (C + numpy restatement of the reference's MEX kernels
    and MATLAB glue) on the host cores: per step, assembly + args.cpu_iters PCG
    iterations of the reference (FP64) algorithm on the crop of crop_of(); the
    time to solve the whole workload is extrapolated by the ratio of active
    elements and to `iterations` iterations.  Returns a dict."""
    from oracle import glue as G
    from sgldbench_gb300 import domains as D

    crop, levels = crop_of(vox, args)
    ne_full, ne_crop = int(vox.sum()), int(crop.sum())
    t0 = time.perf_counter()
    # the crop's own fixed DOFs (its lowest 4 layers) and one load on its boundary
    l1 = G.voxel_discretization(crop, 50000, levels)[0]
    fixed = D.fix_bottom_layers(crop, l1.nodMapBack, layers=4)
    m = G.build_model_fixed(crop, fixed, non_dyadic=0, omega=OMEGA, num_levels=levels)
    case = D.perturbed_patch_cases(crop, m.levels[0].nodMapBack, 1, seed=2, base_seed=0,
                                   radius=min(10.0, crop.shape[1] / 8), shift=2.0)[0]
    m.F = D.dense_load(m.levels[0].numNodes, case)
    t_setup = time.perf_counter() - t0
    G.set_modulus(m, np.ones(m.levels[0].numElements))
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
    rec = []
    for k in range(warmup + steps):
        t0 = time.perf_counter()
        G.assemble_stencil(m)
        spent["kbyu"] = spent["vcycle"] = 0.0
        t1 = time.perf_counter()
        G.pcg(AtX, PtV, m.F, 0.0, args.cpu_iters)
        t2 = time.perf_counter()
        if k >= warmup:
            rec.append((t1 - t0, (t2 - t1) / args.cpu_iters, spent["kbyu"] / args.cpu_iters,
                        spent["vcycle"] / args.cpu_iters))
    t_asm, t_it, t_kbyu, t_vc = (float(np.mean([r[i] for r in rec])) for i in range(4))
    scale = ne_full / ne_crop
    seconds = (t_asm + t_it * iterations) * scale
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"seconds": seconds, "extrapolated": True, "sampled_iterations": args.cpu_iters, "iterations": iterations,
            "scale_active_elements": scale, "crop_voxels": list(crop.shape), "crop_active_elements": ne_crop,
            "crop_levels": m.numLevels, "assemble_s": t_asm, "iter_s": t_it, "kbyu_s": t_kbyu, "vcycle_s": t_vc,
            "glue_s": t_it - t_kbyu - t_vc, "crop_setup_s": t_setup, "cores": cores,
            "split": "per-iteration K*u / V-cycle / rest, as QuickAccess/zTmp_Benchmarking_SpMV.m:63-111"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    from sgldbench_gb300.workloads import fp64_iterations

    vox = workload(args)
    its, provenance = fp64_iterations(args.size, args.levels, args.fill, args.blobs)
    r = cpu_sample(vox, args, its, steps=args.steps, warmup=min(args.warmup, 1))
    from oracle import mexcall

    kind = "reference" if mexcall.ref_lib() is not None else "port"
    sample = (f"per step: oracle assembly + {args.cpu_iters} PCG iterations of the reference (FP64) algorithm on a "
              f"{'x'.join(map(str, r['crop_voxels']))} crop of the box ({r['crop_active_elements']} active "
              f"elements), scaled by the active-element ratio {r['scale_active_elements']:.1f} and to {its} "
              f"iterations ({provenance})")
    line = {"impl": "reference", "metric": METRIC, "value": r["seconds"], "unit": "s", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["seconds"] * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Gaussian-blob shape, perturbed surface loads)",
            "config": workload_config(args),
            "cpu_baseline": {"value": r["seconds"], "unit": "s", "cores": r["cores"], "kind": kind,
                             "sample": sample, "extrapolated": True},
            "e2e": {"value": r["seconds"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "detail": r}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU path
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch

    from sgldbench_gb300 import LoadCases, VoxelSolver, replicas
    from sgldbench_gb300 import domains as D
    from sgldbench_gb300.solver import kernel_launches

    rank, world, local = replicas.dist_env()
    torch.cuda.set_device(local)
    replicas.init("nccl")
    dev = torch.device("cuda", local)
    t_host = time.perf_counter()
    vox = workload(args)
    s = VoxelSolver(vox, num_levels=args.levels, non_dyadic=0, omega=OMEGA, device=local, pad=False)
    nodes = s.nodMapBack(1)
    fixed = D.fix_bottom_layers(vox, nodes, layers=4)
    s.set_fixed_dofs(fixed)
    s.set_modulus(np.ones(s.numElements))
    s.Solving_AssembleFEAstencil()
    train, held = load_cases(vox, nodes, args)
    nn, nd = s.numNodes, s.numDOFs
    t_host = time.perf_counter() - t_host
    stream = torch.cuda.ExternalStream(s.stream, device=dev)

    def dev_load(case):
        f = torch.zeros(nd, dtype=torch.float64, device=dev)
        sel, v = case
        f.view(-1, 3)[torch.from_numpy(sel).to(dev)] = torch.tensor(v, dtype=torch.float64, device=dev)
        return f

    sampler = ClockSampler(local)
    sampler.start()
    # training: the learned start sees the training cases one after another
    lc = LoadCases(s, max_basis=args.train, net_level=0, train_steps=8)
    U_d = torch.empty(nd, dtype=torch.float64, device=dev)
    t0 = time.perf_counter()
    train_rec = []
    for case in train:
        F_d = dev_load(case)
        info, st = lc.solve_device(F_d.data_ptr(), U_d.data_ptr(), mode="learned", train=True, tol=TOL,
                                   maxIT=args.maxit, precision=args.precision)
        train_rec.append((info["its"], info["inner_its"], st["t_solve"], st["t_train"], st["net_loss_before"],
                          st["net_loss"]))
        del F_d
    t_train = time.perf_counter() - t0
    held_d = [dev_load(c) for c in held]
    torch.cuda.synchronize()

    def step(j):
        return lc.solve_device(held_d[j % len(held_d)].data_ptr(), U_d.data_ptr(), mode="learned", tol=TOL,
                               maxIT=args.maxit, precision=args.precision)

    for k in range(max(args.warmup, 0)):
        step(k)
    replicas.barrier()
    torch.cuda.synchronize()
    sampler.mark()
    l0 = kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    recs = []
    for k in range(args.steps):
        recs.append(step(k)[0])
    e1.record(stream)
    torch.cuda.synchronize()
    launches = (kernel_launches() - l0) / max(args.steps, 1)
    t_step = e0.elapsed_time(e1) / 1e3 / args.steps
    replicas.barrier()
    torch.cuda.synchronize()
    t_step, solves = replicas.aggregate(t_step, args.steps, device=dev)
    # end to end through the host-buffer C ABI call: the load copied in from
    # page-locked memory, U copied out, every step
    F_pin = torch.zeros(nd, dtype=torch.float64).pin_memory().numpy()
    U_pin = torch.zeros(nd, dtype=torch.float64).pin_memory().numpy()
    t0e, t1e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2e = []
    for k in range(-1, args.steps):   # one warm-up call of the host path
        D.dense_load(nn, held[max(k, 0) % len(held)], out=F_pin)
        torch.cuda.synchronize()
        t0e.record(stream)
        lc.solve(F_pin, mode="learned", tol=TOL, maxIT=args.maxit, precision=args.precision, out=U_pin)
        t1e.record(stream)
        torch.cuda.synchronize()
        if k >= 0:
            e2e.append(t0e.elapsed_time(t1e) / 1e3)
    clocks = sampler.stop()
    # the starts compared on the first held-out cases (untimed): zero, basis only, basis + network
    cmp = {"zero": [], "basis": [], "learned": []}
    U_mx = None
    for j in range(min(2, len(held))):
        for mode in ("zero", "basis", "learned"):
            info, st = lc.solve_device(held_d[j].data_ptr(), U_d.data_ptr(), mode=mode, tol=TOL, maxIT=args.maxit,
                                       precision=args.precision, diagnostics=True)
            cmp[mode].append({"its": info["its"], "inner_its": info["inner_its"], "seconds": st["t_start"] +
                              st["t_solve"], "start_ratio": st["start_ratio"], "net_accepted": st["net_accepted"]})
            if j == 0 and mode == "learned":
                U_mx = U_d.clone()   # case 0 from the learned start, the headline's answer
    gain = {m: float(np.mean([r["inner_its"] for r in cmp[m]])) for m in cmp}
    net_gain = {"inner_its_basis_only": gain["basis"], "inner_its_with_network": gain["learned"],
                "inner_its_zero_start": gain["zero"],
                "network_vs_basis": gain["basis"] / gain["learned"] if gain["learned"] else None,
                "learned_vs_zero": gain["zero"] / gain["learned"] if gain["learned"] else None}
    # the reference form on case 0: FP64 PCG with the FP64 V-cycle from zero
    fp64 = None
    if args.fp64_steps > 0:
        U64_d = torch.empty_like(U_d)
        s.pcg_device(held_d[0].data_ptr(), U64_d.data_ptr(), TOL, 3, precision="fp64")   # one-time set-up
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        f0.record(stream)
        for _ in range(args.fp64_steps):
            i64 = s.pcg_device(held_d[0].data_ptr(), U64_d.data_ptr(), TOL, args.maxit, precision="fp64")
        f1.record(stream)
        torch.cuda.synchronize()
        t64 = f0.elapsed_time(f1) / 1e3 / args.fp64_steps
        fp64 = {"value": t64, "unit": "s", "iterations": i64["its"], "true_relres": i64["true_relres"],
                "steps": args.fp64_steps, "speedup_of_headline": t64 / t_step,
                "speedup_of_e2e": t64 / float(np.mean(e2e))}
        # errors of the mixed + learned answer of case 0 against the FP64 one
        U64 = U64_d.cpu().numpy()
        Um = U_mx.cpu().numpy()
        F0 = D.dense_load(nn, held[0])
        c64, cm = float(F0 @ U64), float(F0 @ Um)
        _, _, vm64 = s.FEA_StressAnalysis(U64)
        _, _, vmm = s.FEA_StressAnalysis(Um)
        fp64["error_of_headline_vs_fp64"] = {
            "compliance_rel": abs(cm - c64) / abs(c64),
            "displacement_rel_l2": float(np.linalg.norm(Um - U64) / np.linalg.norm(U64)),
            "von_mises_elem_rel_max": float(np.abs(vmm - vm64).max() / np.abs(vm64).max()),
            "note": "both solves at relative residual 1e-6 on their true residual"}
    # roofline of the dominant kernel: the FP32 K*u of the inner CG
    from sgldbench_gb300 import roofline as R

    rl = R.kbyu_f32_roofline(s, vox, reps=20)
    free, total = torch.cuda.mem_get_info()
    inner = [r["inner_its"] for r in recs]
    outer = [r["its"] for r in recs]
    line = {"metric": METRIC, "value": t_step, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": {"mixed": "f64+f32", "mixed_df": "f64+f32+df32"}[args.precision],
            "data": "synthetic (seeded Gaussian-blob shape, perturbed surface loads)",
            "config": workload_config(args, {"dofs": nd, "active_fraction": float(vox.mean())}),
            "iterations": {"outer": outer, "inner": inner},
            "dof_it_per_s": {"outer": world * nd * float(np.mean(outer)) / t_step,
                             "inner": world * nd * float(np.mean(inner)) / t_step},
            "replica_solves_per_s": solves / (t_step * args.steps),
            "converged": all(r["converged"] for r in recs),
            "max_true_relres": max(r["true_relres"] for r in recs),
            "fallbacks": sum(int(r["fallback"]) for r in recs),
            "e2e": {"value": float(np.mean(e2e)), "unit": "s", "h2d_bytes_per_step": 8 * nd,
                    "d2h_bytes_per_step": 8 * nd, "samples": [round(v, 4) for v in e2e]},
            "gpu_launches": int(round(launches)), "roofline": rl, "clocks": clocks,
            "learned": {"train_cases": len(train), "basis": lc.basis_size,
                        "train_s_wall": t_train,
                        "train": [{"its": a, "inner_its": b, "t_solve": c, "t_train": d, "net_loss_before": e,
                                   "net_loss": f} for a, b, c, d, e, f in train_rec],
                        "held_out_compare": cmp, "gain": net_gain,
                        "start": "energy-optimal combination of the training solutions' basis plus the "
                                 "coarse-level network's correction when it lowers r'Mr"},
            "memory_bytes": int(total - free), "host_setup_s": t_host}
    if fp64:
        line["plain_fp64"] = fp64
    if rank == 0 and world == 1 and not args.no_cpu_baseline and fp64:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        r = cpu_sample(vox, args, fp64["iterations"])
        line["cpu_baseline"] = {
            "value": r["seconds"], "unit": "s", "cores": r["cores"], "kind": "port", "extrapolated": True,
            "sample": (f"oracle assembly + {args.cpu_iters} PCG iterations of the reference (FP64) algorithm on a "
                       f"{'x'.join(map(str, r['crop_voxels']))} crop of the box, scaled by the active-element ratio "
                       f"{r['scale_active_elements']:.1f} and to the {fp64['iterations']} iterations of the "
                       "reference-form solve of the same case in this run"),
            "detail": r}
    if rank == 0:
        print(json.dumps(line), flush=True)
    lc.close()
    s.close()
    replicas.shutdown()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
