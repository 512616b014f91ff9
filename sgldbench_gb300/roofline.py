"""Roofline figures of the solve's dominant kernel, the FP32 K*u of the inner
CG (k_kbyu_tma), for bench.py and kernel_bench.py.

Algorithmic bytes per launch follow the operator's own data (per active node:
u read and y written, 3 FP32 values each, plus one flag byte; per active
element: its FP32 modulus), the same count the reference's K*u kernel would
have to move (src/MEXfuncs/Solving_KbyU_MatrixFree_mex.cpp:53-138 reads u, E
and writes y).  The launch time is measured live with CUDA events on the
library's stream (sgld_time_op).  The DRAM traffic of a launch comes from an
ncu capture (dram__bytes_read.sum + dram__bytes_write.sum) recorded below with
the command that produced it; captures on a case smaller than the workload are
scaled by the full-grid node count, which the kernel's traffic follows.
"""
from __future__ import annotations

import json
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# ncu DRAM bytes per full-grid node of one k_kbyu_tma launch, by workload kind.
# "blobs": dram__bytes_read.sum + dram__bytes_write.sum = 160,872,448 + 31,981,824
# bytes for one launch on the 384 x 192 x 192 thresholded-blob shape (30 % solid,
# 385 * 193 * 193 = 14,340,865 grid nodes; default tile 32 x 8 x 26 layers) on a
# GB300, from
#   SGLD_AUTOTUNE=0 ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum
#       --clock-control none -k regex:k_kbyu_tma -c 1 --csv python -m sgldbench_gb300.kernel_bench
#       --domain blobs --size 384 192 192 --levels 6 --ops kbyu32 --reps 3
# The same shape family at 1024 x 512 x 512 is too large for a capture; its
# traffic is scaled by the grid nodes (the launch reads the rows of the tiles
# that hold active elements and writes the active nodes, both in proportion).
DRAM_BYTES_PER_GRID_NODE: dict = {"blobs": (160872448 + 31981824) / 14340865}


def peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured (MEASURED_PEAKS.json)"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "source": "fallback (6.8 TB/s, one earlier GB300 measurement)"}


def kbyu_f32_bytes(active_nodes: int, active_elements: int) -> int:
    return active_nodes * (3 * 4 * 2 + 1) + active_elements * 4


# The reference's K*u applies the dense 24 x 24 Ke to each element (576 multiply-adds,
# src/MEXfuncs/Solving_KbyU_MatrixFree_mex.cpp:105-138) and scales by its modulus: 1152 + 24
# flops per active element.  The FP32 CUDA-core peak is nominal: 152 SMs x 128 FP32 lanes x 2
# flops per FMA at the maximum SM clock of 2070 MHz (no measured figure exists for it).
KBYU_FLOPS_PER_ELEMENT = 1152 + 24
FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.070e9 / 1e12


def kbyu_f32_record(nn: int, ne: int, ms: float, grid_nodes: int, reps: int, tile=None, kind: str = "blobs") -> dict:
    """Roofline record of one k_kbyu_tma launch of `ms` milliseconds on nn active nodes and ne
    active elements.  The binding roof reported is HBM (algorithmic bytes / time against the
    measured copy bandwidth).  `fp32_dense_equivalent` adds the compute view: the reference
    algorithm's flops for the same product / time against the nominal FP32 CUDA-core peak.  The
    sum-factorised kernel executes about a fifth of those flops, so that fraction says how fast
    the product is, not how busy the FP32 pipes are (ncu: FMA pipe active 46 % of cycles)."""
    alg = kbyu_f32_bytes(nn, ne)
    p = peaks()
    achieved = alg / (ms * 1e-3) / 1e9
    per = DRAM_BYTES_PER_GRID_NODE.get(kind)
    tflops = KBYU_FLOPS_PER_ELEMENT * ne / (ms * 1e-3) / 1e12
    return {"bound": "hbm", "achieved": achieved, "peak": p["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / p["hbm_gbs"], "traffic": None if per is None else per * grid_nodes,
            "kernel": "k_kbyu_tma (FP32 K*u of the inner CG)", "avg_launch_ms": ms,
            "launch_timing": f"CUDA events around {reps} back-to-back launches on the library stream "
                             "(sgld_time_op) after the timed region; inside it the kernel runs in the inner CG's "
                             "graph", "algorithmic_bytes_per_launch": alg,
            "algorithmic_bytes": "active nodes x (3 x 4 B in + 3 x 4 B out + 1 B flags) + active elements x 4 B",
            "active_nodes": nn, "active_elements": ne, "grid_nodes": grid_nodes,
            "peak_source": p["source"], "tile": tile,
            "fp32_dense_equivalent": {
                "flops_per_element": KBYU_FLOPS_PER_ELEMENT, "achieved_tflops": tflops,
                "peak_tflops": FP32_NOMINAL_TFLOPS, "frac": tflops / FP32_NOMINAL_TFLOPS,
                "peak_source": "nominal (152 SMs x 128 FP32 lanes x 2 flops x 2070 MHz)",
                "note": "flops of the reference's dense per-element product; the sum-factorised kernel "
                        "executes about a fifth of them"}}


def kbyu_f32_roofline(s, voxels=None, reps: int = 20, kind: str = "blobs") -> dict:
    """Roofline record of k_kbyu_tma on solver s (assembled)."""
    ms = s.time_op("kbyu32", reps)
    grid_nodes = (s.resY + 1) * (s.resX + 1) * (s.resZ + 1)
    return kbyu_f32_record(s.numNodes, s.numElements, ms, grid_nodes, reps, s.kbyu_tile(), kind)
