"""Measured facts about the seeded benchmark workloads that a run without a GPU
needs.  bench.py's reference arm times the reference algorithm on a bounded
sample and extrapolates to the iteration count of the reference-form (FP64
PCG, FP64 additive V-cycle) solve of the same system; the oracle cannot reach
that count within a bounded sample, so the count measured by the GPU's
reference-form solve -- the same algorithm, whose iteration counts equal the
oracle's in the parity tests -- is recorded here with its provenance.
"""
from __future__ import annotations

# (nx, ny, nz, levels, fill, blobs) -> (iterations, provenance)
FP64_ITERATIONS: dict = {
    (1024, 512, 512, 7, 0.3, 64): (
        507, "measured: the reference-form FP64 PCG of held-out case 0 on a GB300 (bench.py plain_fp64, "
             "two runs, 507 iterations each)"),
}

# used when no measurement is recorded for a workload
DEFAULT_ITERATIONS = 500


def fp64_iterations(size, levels, fill, blobs):
    key = (int(size[0]), int(size[1]), int(size[2]), int(levels), float(fill), int(blobs))
    if key in FP64_ITERATIONS:
        return FP64_ITERATIONS[key]
    return DEFAULT_ITERATIONS, "no measurement recorded for this workload: a default estimate"
