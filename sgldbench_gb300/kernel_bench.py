"""Per-operator device timings of the solve path (CUDA events), for rooflines
and as the small driver of kernel-level profiler captures.

  python -m sgldbench_gb300.kernel_bench [--size NX NY NZ] [--levels L]
                                         [--ops kbyu64 kbyu32 kbyu_df vcycle64 vcycle32 assemble]
                                         [--reps N]

Builds the SIMP-graded cantilever of the given size, assembles it and prints
one JSON line per operator with the mean milliseconds per application and the
algorithmic bytes / flops that its roofline uses.
"""
from __future__ import annotations

import argparse
import json

from . import domains as D
from .solver import VoxelSolver


def bytes_and_flops(op: str, nx: int, ny: int, nz: int) -> tuple[int, float]:
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    ne = nx * ny * nz
    if op in ("kbyu64", "kbyu_df"):   # read u, write y (3 doubles per node), node flags, E per element
        return nn * (48 + 1) + ne * 8, 1176.0 * ne
    if op == "kbyu32":
        return nn * (24 + 1) + ne * 4, 1176.0 * ne
    return 0, 0.0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, nargs=3, default=[256, 128, 128])
    ap.add_argument("--levels", type=int, default=5)
    ap.add_argument("--ops", nargs="+", default=["kbyu64", "kbyu32", "kbyu_df", "vcycle64", "vcycle32", "assemble"])
    ap.add_argument("--reps", type=int, default=10)
    args = ap.parse_args()
    nx, ny, nz = args.size
    vox = D.cuboid(nx, ny, nz)
    E = D.simp_modulus(D.graded_density(nx, ny, nz, seed=0), Emin=1e-9)
    s = VoxelSolver(vox, num_levels=args.levels, non_dyadic=0, omega=0.6, pad=False)
    F, fixed = D.cantilever3(vox, s.nodMapBack(1))
    s.set_fixed_dofs(fixed)
    s.set_modulus(E)
    s.Solving_AssembleFEAstencil()
    for op in args.ops:
        ms = s.time_op(op, args.reps)
        b, f = bytes_and_flops(op, nx, ny, nz)
        rec = {"op": op, "size": args.size, "ms": ms}
        if b:
            rec.update({"bytes": b, "GBps": b / ms / 1e6, "dense_equiv_TFLOPs": f / ms / 1e9})
        if op == "kbyu32":
            rec["tile"] = s.kbyu_tile()
        print(json.dumps(rec), flush=True)
    s.close()


if __name__ == "__main__":
    main()
