"""Measurements of the five workloads of SGLDBench's solve path on one GPU:

  0  solid 64 x 32 x 32 cuboid, E = 1, cantilever, 3 levels (first step 4:1), omega 0.6
  1  SIMP-graded 256 x 128 x 128 cantilever, 5 dyadic levels
  2  512 x 256 x 256 union of spheres and boxes grown to ~40 % solid, lowest 4 layers fixed,
     8 load cases over surface patches, block right-hand side, 6 dyadic levels
  3  SIMP loop on config 1's cantilever: volume fraction 0.3, p = 3, rmin 1.5, OC, 60 iterations
  4  1024 x 512 x 512 thresholded Gaussian blobs (~30 % solid), lowest 4 layers fixed,
     2 load cases, 7 dyadic levels

    python -m sgldbench_gb300.config_bench --config 0 1 2 3 4

Each config prints one JSON line: device times (CUDA events) of the reference-form
FP64 solve and of the mixed-precision solve, iteration counts, DOF*iterations/s,
and the errors of every solve against an FP64 solve of the same system to
relative residual 1e-10 (compliance, displacement relative L2, per-element von
Mises).  Synthetic seeded inputs stand in for the reference's voxel models.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import domains as D
from .solver import VoxelSolver


def _events():
    import torch

    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _timed(s, fn, reps=1):
    import torch

    stream = torch.cuda.ExternalStream(s.stream)
    fn()   # warm-up (graph capture, first-touch allocation)
    a, b = _events()
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(reps):
        out = fn()
    b.record(stream)
    torch.cuda.synchronize()
    return out, a.elapsed_time(b) / 1e3 / reps


def _errors(s, U, U_ref):
    _, c = s.TopOpti_ComputeUnitCompliance(U)
    _, c_ref = s.TopOpti_ComputeUnitCompliance(U_ref)
    _, _, vm = s.FEA_StressAnalysis(U)
    _, _, vm_ref = s.FEA_StressAnalysis(U_ref)
    return {"compliance_rel": abs(c - c_ref) / abs(c_ref),
            "displacement_rel_l2": float(np.linalg.norm(U - U_ref) / np.linalg.norm(U_ref)),
            "vm_elem_rel_max": float(np.abs(vm - vm_ref).max() / np.abs(vm_ref).max())}


def _solve_pair(s, F, tol=1e-6, maxit=5000, reps=2):
    """FP64 and mixed_df solves of one load case, each with its assembly."""
    out = {}
    s.Solving_AssembleFEAstencil()
    U_ref, _ = s.pcg(F, tol=1e-10, maxIT=20000)
    for prec in ("fp64", "mixed_df"):
        def run():
            s.Solving_AssembleFEAstencil()
            return s.pcg(F, tol=tol, maxIT=maxit, precision=prec)
        (U, info), t = _timed(s, run, reps)
        rec = {"seconds": t, "iterations": info["its"], "inner_iterations": info["inner_its"],
               "true_relres": info["true_relres"], "dof_it_per_s": s.numDOFs * info["its"] / t}
        rec.update(_errors(s, U, U_ref))
        out[prec] = rec
    out["speedup_mixed_vs_fp64"] = out["fp64"]["seconds"] / out["mixed_df"]["seconds"]
    return out


def _device_mem():
    import torch

    free, total = torch.cuda.mem_get_info()
    return total - free


def config0():
    vox = D.cuboid(64, 32, 32)
    s = VoxelSolver(vox, non_dyadic=1, omega=0.6)
    F, fixed = D.cantilever3(vox, s.nodMapBack(1))
    s.set_fixed_dofs(fixed)
    s.set_modulus(np.ones(s.numElements))
    return {"config": 0, "dofs": s.numDOFs, "levels": s.numLevels, **_solve_pair(s, F)}


def config1():
    nx, ny, nz = 256, 128, 128
    vox = D.cuboid(nx, ny, nz)
    E = D.simp_modulus(D.graded_density(nx, ny, nz, seed=0, sigma=2.0, rho_min=1e-3), Emin=1e-9)
    s = VoxelSolver(vox, num_levels=5, non_dyadic=0, omega=0.6, pad=False)
    F, fixed = D.cantilever3(vox, s.nodMapBack(1))
    s.set_fixed_dofs(fixed)
    s.set_modulus(E)
    return {"config": 1, "dofs": s.numDOFs, "levels": s.numLevels, **_solve_pair(s, F)}


def config_block(nx, ny, nz, vox, levels, nrhs, cfg):
    t0 = time.perf_counter()
    s = VoxelSolver(vox, num_levels=levels, non_dyadic=0, omega=0.6, pad=False)
    nodes = s.nodMapBack(1)
    fixed = D.fix_bottom_layers(vox, nodes, layers=4)
    F = D.patch_loads(vox, nodes, nrhs, seed=cfg, radius=10.0)
    s.set_fixed_dofs(fixed)
    s.set_modulus(np.ones(s.numElements))
    setup = time.perf_counter() - t0
    s.Solving_AssembleFEAstencil()
    mem = _device_mem()
    rec = {"config": cfg, "dofs": s.numDOFs, "active_fraction": float(vox.mean()), "levels": s.numLevels,
           "nrhs": nrhs, "host_setup_s": setup, "device_bytes_in_use": mem}
    U_ref, _ = s.solve_block(F, tol=1e-10, maxIT=20000)
    for prec in ("fp64", "mixed_df"):
        def run():
            s.Solving_AssembleFEAstencil()
            return s.solve_block(F, tol=1e-6, maxIT=5000, precision=prec)
        (U, infos), t = _timed(s, run, 1)
        errs = [_errors(s, U[j], U_ref[j]) for j in range(nrhs)]
        rec[prec] = {"seconds_block": t, "seconds_per_rhs": t / nrhs,
                     "iterations": [i["its"] for i in infos],
                     "max_true_relres": max(i["true_relres"] for i in infos),
                     "dof_it_per_s": s.numDOFs * sum(i["its"] for i in infos) / t,
                     **{k: max(e[k] for e in errs) for k in errs[0]}}
    rec["speedup_mixed_vs_fp64"] = rec["fp64"]["seconds_block"] / rec["mixed_df"]["seconds_block"]
    return rec


def config2():
    vox = D.blobby_union(512, 256, 256, seed=0, fill=0.4)
    return config_block(512, 256, 256, vox, 6, 8, 2)


def config3():
    nx, ny, nz = 256, 128, 128
    vox = D.cuboid(nx, ny, nz)
    s = VoxelSolver(vox, num_levels=5, non_dyadic=0, omega=0.6, pad=False)
    F, fixed = D.cantilever3(vox, s.nodMapBack(1))
    s.set_fixed_dofs(fixed)
    rec = {"config": 3, "dofs": s.numDOFs, "levels": s.numLevels}
    xs = {}
    for prec, tol in (("fp64", 1e-6), ("mixed_df", 1e-6)):
        t0 = time.perf_counter()
        x, hist = s.TopOpti_GlobalVolumeConstraint(F, volfrac=0.3, rMin=1.5, nLoop=60, tol=tol, maxIT=5000,
                                                   precision=prec)
        wall = time.perf_counter() - t0
        xs[prec] = x
        rec[prec] = {"wall_s": wall, "iterations": len(hist),
                     "solve_s": float(sum(h["t_solve"] for h in hist)),
                     "assemble_s": float(sum(h["t_assemble"] for h in hist)),
                     "cg_iterations": int(sum(h["cg_iterations"] for h in hist)),
                     "final_compliance": hist[-1]["compliance"], "final_volume": hist[-1]["volume"]}
    rec["final_compliance_rel_diff"] = abs(rec["mixed_df"]["final_compliance"] - rec["fp64"]["final_compliance"]) \
        / abs(rec["fp64"]["final_compliance"])
    rec["xphys_max_abs_diff"] = float(np.abs(xs["mixed_df"] - xs["fp64"]).max())
    rec["speedup_mixed_vs_fp64_solve"] = rec["fp64"]["solve_s"] / rec["mixed_df"]["solve_s"]
    return rec


def config4():
    vox = D.gaussian_blobs(1024, 512, 512, seed=0, fill=0.3)
    return config_block(1024, 512, 512, vox, 7, 2, 4)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, nargs="+", default=[0, 1])
    args = ap.parse_args()
    fns = {0: config0, 1: config1, 2: config2, 3: config3, 4: config4}
    for c in args.config:
        print(json.dumps(fns[c]()), flush=True)


if __name__ == "__main__":
    main()
