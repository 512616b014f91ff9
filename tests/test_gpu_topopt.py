"""GPU: the cone density filter and the SIMP loop (config 3's caller) against
the oracle (restatement of TopOpti_GlobalVolumeConstraint_Tmp.m with the C
restatement of the filter MEX kernels).

Tolerances: filter and weight sums 1e-14 relative (same weights, same
summation order; only FMA contraction differs).  SIMP loop: both sides solve
every MGPCG to 1e-10 so the designs follow the same path; per-iteration
compliance within 1e-6 relative, volume within 1e-9, final xPhys within 1e-5.
"""
import numpy as np
import pytest

from oracle import glue as G
from oracle import kernels as OK

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@pytest.fixture(scope="module")
def irregular(built_lib):
    from sgldbench_gb300 import VoxelSolver

    rng = np.random.default_rng(4)
    vox = rng.random((16, 24, 16)) < 0.75
    m = G.build_model(vox, omega=0.6)
    s = VoxelSolver(vox, omega=0.6)
    s.set_fixed_dofs(m.levels[0].fixedDOFs)
    return m, s


@pytest.mark.parametrize("rmin", [1.5, 2.6])
def test_density_filter(irregular, rmin):
    m, s = irregular
    l1 = m.levels[0]
    x = np.random.default_rng(1).random(l1.numElements)
    args = (l1.eleMapForward, l1.resX, l1.resY, l1.resZ)
    assert _rel(s.TopOpti_SetupDensityFilter(rmin), OK.density_filter(None, rmin, *args)) <= 1e-14
    assert _rel(s.TopOpti_PerformDensityFiltering(x, rmin), OK.density_filter(x, rmin, *args)) <= 1e-14


def test_simp_loop_matches_oracle(built_lib):
    from sgldbench_gb300 import VoxelSolver

    vox = np.ones((8, 16, 8), bool)
    m = G.build_model(vox, omega=0.6)
    s = VoxelSolver(vox, omega=0.6)
    s.set_fixed_dofs(m.levels[0].fixedDOFs)
    opt = G.TopOptOptions(n_loop=6, tol=1e-10, maxit=2000, Emin=1e-9)
    xp_o, hist_o = G.topopt_global_volume(m, opt)
    xp, hist = s.TopOpti_GlobalVolumeConstraint(m.F, volfrac=0.3, rMin=1.5, nLoop=6, tol=1e-10, maxIT=2000,
                                                Emin=1e-9)
    assert len(hist) == len(hist_o)
    for a, b in zip(hist, hist_o):
        assert abs(a["compliance"] - b["c"]) <= 1e-6 * abs(b["c"])
        assert abs(a["volume"] - b["vol"]) <= 1e-9
        assert abs(a["change"] - b["change"]) <= 1e-5
        assert abs(a["sharpness"] - b["sharp"]) <= 1e-6
    assert _rel(xp, xp_o) <= 1e-5
    assert hist[-1]["compliance"] < hist[0]["compliance"]


def test_simp_loop_mixed_precision(built_lib):
    """The mixed solve inside the loop reaches the same designs to the loop's
    tolerance: compliance history within 1e-4 of the FP64 loop."""
    from sgldbench_gb300 import VoxelSolver

    vox = np.ones((8, 16, 8), bool)
    m = G.build_model(vox, omega=0.6)
    s = VoxelSolver(vox, omega=0.6)
    s.set_fixed_dofs(m.levels[0].fixedDOFs)
    _, h64 = s.TopOpti_GlobalVolumeConstraint(m.F, nLoop=4, tol=1e-8, maxIT=2000, Emin=1e-9)
    _, hmx = s.TopOpti_GlobalVolumeConstraint(m.F, nLoop=4, tol=1e-8, maxIT=500, Emin=1e-9, precision="mixed")
    for a, b in zip(hmx, h64):
        assert abs(a["compliance"] - b["compliance"]) <= 1e-4 * abs(b["compliance"])
