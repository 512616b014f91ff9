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


def test_pde_filter_matches_oracle(built_lib):
    """PDE (Helmholtz) filter (TopOpti_PDEFiltering_matrixFree.m) against the
    oracle: same PCG iteration count (+-1) and filtered field to 1e-9 at tol
    1e-10; the filter preserves a constant field on a solid box."""
    from sgldbench_gb300 import VoxelSolver

    rng = np.random.default_rng(12)
    vox = rng.random((12, 16, 8)) < 0.8
    m = G.build_model(vox, omega=0.6)
    s = VoxelSolver(vox, omega=0.6)
    x = rng.random(m.levels[0].numElements)
    for rhat in (1.5, 3.0):
        y, its = s.TopOpti_PDEFiltering(x, rhat, tol=1e-10, maxIT=1000)
        y_o, its_o = G.pde_filter(m, x, rhat, tol=1e-10, maxIT=1000)
        assert abs(its - its_o) <= 1
        assert np.abs(y - y_o).max() <= 1e-9 * np.abs(y_o).max()
    box = np.ones((8, 8, 8), bool)
    sb = VoxelSolver(box, omega=0.6)
    ones = np.ones(sb.numElements)
    yb, _ = sb.TopOpti_PDEFiltering(ones, 2.0, tol=1e-12, maxIT=1000)
    assert np.abs(yb - 1.0).max() <= 1e-9


def test_mma_update_matches_oracle(built_lib):
    """sgld_mma_update (MMA_mex's drop-in, one volume constraint) against the
    oracle restatement of MMAseq (pinned to the compiled reference by the CPU
    tests): new design to 1e-9, xold1/xold2 exactly as MMAseq::Update sets them."""
    from oracle import mma
    from sgldbench_gb300 import VoxelSolver

    s = VoxelSolver(np.ones((8, 8, 8), bool), omega=0.6)
    rng = np.random.default_rng(21)
    for n in (1000, 200_000):
        x = rng.uniform(0.0, 1.0, n)
        xmin, xmax = np.maximum(0, x - 0.1), np.minimum(1, x + 0.1)
        df0 = -rng.uniform(1e-4, 3.0, n)
        dg = np.full(n, 1.0 / (n * 0.3))
        fval = x.sum() / (n * 0.3) - 1
        xo1, xo2 = x * 0.99, x * 0.98
        xn, o1, o2 = s.MMA(x, xmin, xmax, xo1, xo2, df0, fval, dg)
        rn, r1, r2 = mma.mma_update(1, n, x, xmin, xmax, xo1, xo2, df0, fval, dg)
        assert np.abs(xn - rn).max() <= 1e-9
        assert np.array_equal(o1, r1) and np.array_equal(o2, r2)
        assert np.all(xn >= xmin - 1e-15) and np.all(xn <= xmax + 1e-15)


@pytest.mark.parametrize("optimizer", ["OC", "MMA"])
def test_simp_loop_optimizer_and_passive(built_lib, optimizer):
    """The SIMP loop with the MMA update (TopOpti_GlobalVolumeConstraint.m:
    139-156) or OC, with passive elements kept solid (:162, :179), against the
    oracle: compliance per iteration within 1e-6, final xPhys within 1e-5,
    passive xPhys exactly 1."""
    from sgldbench_gb300 import VoxelSolver

    vox = np.ones((8, 16, 8), bool)
    m = G.build_model(vox, omega=0.6)
    s = VoxelSolver(vox, omega=0.6)
    s.set_fixed_dofs(m.levels[0].fixedDOFs)
    n = m.levels[0].numElements
    passive = np.arange(0, n, 17)
    s.set_passive(passive)
    opt = G.TopOptOptions(n_loop=5, tol=1e-10, maxit=2000, Emin=1e-9, optimizer=optimizer, passive=passive)
    xp_o, hist_o = G.topopt_global_volume(m, opt)
    xp, hist = s.TopOpti_GlobalVolumeConstraint(m.F, volfrac=0.3, rMin=1.5, nLoop=5, tol=1e-10, maxIT=2000,
                                                Emin=1e-9, optimizer=optimizer)
    s.set_passive([])
    assert len(hist) == len(hist_o)
    for a, b in zip(hist, hist_o):
        assert abs(a["compliance"] - b["c"]) <= 1e-6 * abs(b["c"])
        assert abs(a["change"] - b["change"]) <= 1e-5
    assert _rel(xp, xp_o) <= 1e-5
    assert np.all(xp[passive] == 1.0)


def test_local_volume_loop_matches_oracle(built_lib):
    """The porous-infill loop (TopOpti_LocalVolumeConstraint.m): PDE-filtered
    local volume p-norm constraint, MMA, Heaviside projection, with the beta
    doubling and the penalty increment both exercised (short intervals), and
    passive elements.  Both sides solve every MGPCG and PDE filter to 1e-10, so
    the designs follow the same path: compliance per iteration within 1e-6,
    the constraint value within 1e-8, final xPhys within 1e-5, passive
    xPhys exactly 1."""
    from sgldbench_gb300 import VoxelSolver

    vox = np.ones((8, 16, 8), bool)
    m = G.build_model(vox, omega=0.6)
    s = VoxelSolver(vox, omega=0.6)
    s.set_fixed_dofs(m.levels[0].fixedDOFs)
    n = m.levels[0].numElements
    passive = np.arange(3, n, 23)
    s.set_passive(passive)
    kw = dict(rmin=1.5, rhat=3.0, alpha=0.6, pnorm=16.0, n_loop=5, penalty=2.8, penalty_increment=0.1,
              penalty_interval=2, beta_interval=2, tol=1e-10, maxit=2000)
    opt = G.LocalOptions(passive=passive, **kw)
    xp_o, hist_o = G.topopt_local_volume(m, opt)
    xp, hist = s.TopOpti_LocalVolumeConstraint(
        m.F, rMin=kw["rmin"], rHat=kw["rhat"], alpha=kw["alpha"], p=kw["pnorm"], nLoop=kw["n_loop"],
        penalty=kw["penalty"], penalty_increment=kw["penalty_increment"], penalty_interval=kw["penalty_interval"],
        beta_interval=kw["beta_interval"], tol=kw["tol"], maxIT=kw["maxit"])
    s.set_passive([])
    assert len(hist) == len(hist_o)
    assert [h["beta"] for h in hist_o][-1] > 1.0     # the continuation ran
    for a, b in zip(hist, hist_o):
        assert abs(a["compliance"] - b["c"]) <= 1e-6 * abs(b["c"])
        assert abs(a["constraint"] - b["fval"]) <= 1e-8
        assert abs(a["volume"] - b["vol"]) <= 1e-9
        assert abs(a["change"] - b["change"]) <= 1e-5
    assert _rel(xp, xp_o) <= 1e-5
    assert np.all(xp[passive] == 1.0)


def test_projected_volume_loop_matches_oracle(built_lib):
    """TopOpti_GlobalVolumeConstraint.m's full loop with MMA (Heaviside projection,
    beta and penalty continuation, solid-normalised compliance) against the
    oracle, same tolerances as the local-volume loop."""
    from sgldbench_gb300 import VoxelSolver

    vox = np.ones((8, 16, 8), bool)
    m = G.build_model(vox, omega=0.6)
    s = VoxelSolver(vox, omega=0.6)
    s.set_fixed_dofs(m.levels[0].fixedDOFs)
    kw = dict(volfrac=0.4, rmin=1.5, n_loop=5, penalty=2.8, penalty_increment=0.1, penalty_interval=2,
              beta_interval=3, tol=1e-10, maxit=2000)
    xp_o, hist_o = G.topopt_local_volume(m, G.LocalOptions(constraint="volume", **kw))
    xp, hist = s.TopOpti_GlobalVolumeConstraintProjected(
        m.F, volfrac=kw["volfrac"], rMin=kw["rmin"], nLoop=kw["n_loop"], penalty=kw["penalty"],
        penalty_increment=kw["penalty_increment"], penalty_interval=kw["penalty_interval"],
        beta_interval=kw["beta_interval"], tol=kw["tol"], maxIT=kw["maxit"])
    assert len(hist) == len(hist_o)
    assert [h["beta"] for h in hist_o][-1] > 1.0
    for a, b in zip(hist, hist_o):
        assert abs(a["compliance"] - b["c"]) <= 1e-6 * abs(b["c"])
        assert abs(a["constraint"] - b["fval"]) <= 1e-8
        assert abs(a["change"] - b["change"]) <= 1e-5
    assert _rel(xp, xp_o) <= 1e-5


@pytest.mark.parametrize("optimizer", ["OC", "MMA"])
def test_simp_loop_checkpoint_resume(built_lib, tmp_path, optimizer):
    """A loop stopped after 3 iterations, saved to a checkpoint file, loaded and
    resumed to 7 runs iterations 4-7 exactly as the uninterrupted 7-iteration
    loop does: same history, bitwise-equal final xPhys."""
    from sgldbench_gb300 import VoxelSolver
    from sgldbench_gb300 import checkpoint as CK

    vox = np.ones((8, 16, 8), bool)
    m = G.build_model(vox, omega=0.6)
    s = VoxelSolver(vox, omega=0.6)
    s.set_fixed_dofs(m.levels[0].fixedDOFs)
    kw = dict(volfrac=0.3, rMin=1.5, tol=1e-8, maxIT=2000, optimizer=optimizer, precision="mixed_df")
    xp_full, h_full = s.TopOpti_GlobalVolumeConstraint(m.F, nLoop=7, **kw)
    _, h_a, st = s.TopOpti_GlobalVolumeConstraint(m.F, nLoop=3, return_state=True, **kw)
    p = str(tmp_path / "loop.ckpt")
    CK.save(p, st)
    xp_b, h_b = s.TopOpti_GlobalVolumeConstraint(m.F, nLoop=7, resume=CK.load(p), **kw)
    assert [h["loop"] for h in h_a + h_b] == list(range(1, 8))
    for a, b in zip(h_a + h_b, h_full):
        assert a["compliance"] == b["compliance"] and a["change"] == b["change"]
        assert a["cg_iterations"] == b["cg_iterations"]
    assert np.array_equal(xp_b, xp_full)
