"""Per-operator device timings of the solve path (CUDA events), for rooflines
and as the small driver of kernel-level profiler captures.

  python -m sgldbench_gb300.kernel_bench [--size NX NY NZ] [--levels L]
                                         [--ops kbyu64 kbyu32 kbyu_df vcycle64 vcycle32 assemble]
                                         [--reps N] [--domain graded|blobs] [--fill F]
                                         [--solve PRECISION] [--net NY NX NZ]

Builds the SIMP-graded cantilever of the given size (or, with --domain blobs,
the thresholded Gaussian-blob shape of the large stress analysis with its
lowest 4 voxel layers fixed), assembles it and prints one JSON line per
operator with the mean milliseconds per application and the algorithmic bytes
/ flops that its roofline uses (active nodes and elements).  --solve then
runs one solve to relative residual 1e-6 in the given precision (the
cantilever load, or one patch load of the blob shape) and prints its
iterations and device time; with SGLD_INNER_LOOP=host its inner loop runs
from the host, so that a profiler's launch list shows every kernel.

--net NY NX NZ times the learned start's U-Net alone (8 input channels, 3
outputs, 4 levels of widths 16/32/48/64) on that node grid instead: forward
passes and training steps (host copies of its small inputs included); with
SGLD_NET_CUDA_CORES=1 its convolutions run on the FP32 pipes instead of the
tensor cores.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import domains as D
from .solver import VoxelSolver


def bytes_and_flops(op: str, nn: int, ne: int) -> tuple[int, float]:
    if op in ("kbyu64", "kbyu_df"):   # read u, write y (3 doubles per node), node flags, E per element
        return nn * (48 + 1) + ne * 8, 1176.0 * ne
    if op == "kbyu32":
        return nn * (24 + 1) + ne * 4, 1176.0 * ne
    return 0, 0.0


def net_bench(dims, reps: int):
    import os
    import time

    from .net import UNet

    cin = 8
    net = UNet(tuple(dims), cin, 3, levels=4, widths=[16, 32, 48, 64], seed=0)
    V = int(np.prod(dims))
    rng = np.random.default_rng(0)
    x = rng.standard_normal((V, cin)).astype(np.float32)
    t = rng.standard_normal((V, 3)).astype(np.float32)
    for _ in range(3):
        net.forward(x)
        net.train_step(x, t, lr=1e-4)
    t0 = time.perf_counter()
    for _ in range(reps):
        net.forward(x)
    t1 = time.perf_counter()
    for _ in range(reps):
        net.train_step(x, t, lr=1e-4)
    t2 = time.perf_counter()
    print(json.dumps({"net": list(dims), "convolutions": "fp32 pipes" if os.environ.get("SGLD_NET_CUDA_CORES") == "1"
                      else "tensor cores", "forward_ms": (t1 - t0) / reps * 1e3,
                      "train_step_ms": (t2 - t1) / reps * 1e3}), flush=True)
    net.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, nargs=3, default=[256, 128, 128])
    ap.add_argument("--levels", type=int, default=5)
    ap.add_argument("--ops", nargs="+", default=["kbyu64", "kbyu32", "kbyu_df", "vcycle64", "vcycle32", "assemble"])
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--domain", choices=["graded", "blobs"], default="graded")
    ap.add_argument("--fill", type=float, default=0.3)
    ap.add_argument("--solve", choices=["fp64", "mixed", "mixed_df"], default=None)
    ap.add_argument("--net", type=int, nargs=3, default=None, metavar=("NY", "NX", "NZ"))
    args = ap.parse_args()
    if args.net:
        net_bench(args.net, args.reps)
        return
    nx, ny, nz = args.size
    if args.domain == "blobs":
        vox = D.gaussian_blobs(nx, ny, nz, seed=0, n_blobs=64, fill=args.fill)
    else:
        vox = D.cuboid(nx, ny, nz)
    s = VoxelSolver(vox, num_levels=args.levels, non_dyadic=0, omega=0.6, pad=False)
    if args.domain == "blobs":
        fixed = D.fix_bottom_layers(vox, s.nodMapBack(1), layers=4)
        E = np.ones(s.numElements)
    else:
        E = D.simp_modulus(D.graded_density(nx, ny, nz, seed=0), Emin=1e-9)
        F, fixed = D.cantilever3(vox, s.nodMapBack(1))
    s.set_fixed_dofs(fixed)
    s.set_modulus(E)
    s.Solving_AssembleFEAstencil()
    for op in args.ops:
        ms = s.time_op(op, args.reps)
        b, f = bytes_and_flops(op, s.numNodes, s.numElements)
        rec = {"op": op, "size": args.size, "domain": args.domain, "ms": ms}
        if b:
            rec.update({"bytes": b, "GBps": b / ms / 1e6, "dense_equiv_TFLOPs": f / ms / 1e9})
        if op == "kbyu32":
            rec["tile"] = s.kbyu_tile()
        print(json.dumps(rec), flush=True)
    if args.solve:
        if args.domain == "blobs":
            case = D.perturbed_patch_cases(vox, s.nodMapBack(1), 1, seed=2, base_seed=0,
                                           radius=max(10.0 * nx / 1024, 2.5), shift=0.0)[0]
            F = D.dense_load(s.numNodes, case)
        U, info = s.pcg(F, tol=1e-6, maxIT=20000, precision=args.solve)
        print(json.dumps({"solve": args.solve, "size": args.size, "domain": args.domain, "its": info["its"],
                          "inner_its": info["inner_its"], "seconds": info["seconds"],
                          "true_relres": info["true_relres"], "converged": info["converged"]}), flush=True)
    s.close()


if __name__ == "__main__":
    main()
