"""GPU parity at the benchmark configurations' own sizes, against the oracle.

* The SIMP-graded 256 x 128 x 128 cantilever (12.8 M DOF, 5 dyadic levels,
  omega 0.6): the FP64 solve takes the oracle's iteration count (+-1) and its
  displacement within 1e-8 (relative L2) of the oracle's solve at the same
  tolerance 1e-6; the mixed solve (mixed_df) meets 1e-6 on the true residual
  and agrees with the oracle's FP64 solve continued to 1e-10 within 1e-6 in
  compliance and 1e-5 in displacement.
* One iteration of the SIMP loop (TopOpti_GlobalVolumeConstraint_Tmp.m) on
  the same 256 x 128 x 128 cantilever: compliance, volume, change, sharpness
  and xPhys against the oracle's loop.
* The real model data/part_R256.TopVoxel (1.85 M voxels): FP64 and mixed
  solves against the oracle's FP64 solve of the same system, on 5 dyadic
  levels and on the reference's own default hierarchy (coarsestResolution-
  Control_ = 50000 and nonDyadic_ = 1, Data_GlobalVariables.m:13-15: the
  grid padded to multiples of 8, a 4:1 first step and a 2:1 second one, so
  3 levels with a 32 x 20 x 14-element coarsest grid).

The oracle (C + numpy restatement of the reference) takes about half a
minute of host time per solve at these sizes.
"""
import os

import numpy as np
import pytest

from oracle import glue as G

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def config1(built_lib):
    from sgldbench_gb300 import VoxelSolver
    from sgldbench_gb300 import domains as D

    nx, ny, nz = 256, 128, 128
    vox = D.cuboid(nx, ny, nz)
    E = D.simp_modulus(D.graded_density(nx, ny, nz, seed=0, sigma=2.0, rho_min=1e-3), Emin=1e-9)
    m = G.build_model(vox, non_dyadic=0, omega=0.6, num_levels=5)
    s = VoxelSolver(vox, num_levels=5, non_dyadic=0, omega=0.6, pad=False)
    assert s.numLevels == m.numLevels == 5 and s.numDOFs == 12830211
    F, fixed = D.cantilever3(vox, s.nodMapBack(1))
    assert np.array_equal(fixed, m.levels[0].fixedDOFs) and np.array_equal(F, m.F)
    G.set_modulus(m, E)
    G.assemble_stencil(m)
    s.set_fixed_dofs(fixed)
    s.set_modulus(E)
    s.Solving_AssembleFEAstencil()
    U_o, its_o = G.solve(m, tol=1e-6, maxIT=2000)
    U_c, _ = G.solve(m, tol=1e-10, maxIT=4000, x0=U_o)   # the oracle's solve continued to 1e-10
    yield m, s, U_o, its_o, U_c
    s.close()


def test_config1_fp64_matches_oracle(config1):
    m, s, U_o, its_o, _ = config1
    U, info = s.pcg(m.F, tol=1e-6, maxIT=2000)
    assert info["converged"]
    assert abs(info["its"] - its_o) <= 1, (info["its"], its_o)
    assert np.linalg.norm(U - U_o) / np.linalg.norm(U_o) <= 1e-8


def test_config1_mixed_matches_oracle(config1):
    m, s, _, _, U_c = config1
    U, info = s.pcg(m.F, tol=1e-6, maxIT=2000, precision="mixed_df")
    assert info["converged"] and info["true_relres"] <= 1e-6 and not info["fallback"], info
    c_ref = G.compliance(m, U_c)
    _, c = s.TopOpti_ComputeUnitCompliance(U)
    assert abs(c - c_ref) / abs(c_ref) <= 1e-6
    assert np.linalg.norm(U - U_c) / np.linalg.norm(U_c) <= 1e-5


def test_config3_simp_iteration_matches_oracle(config1):
    """First iteration of config 3's SIMP loop (volume fraction 0.3, p = 3,
    rmin 1.5, OC with move 0.1) at its full size."""
    m, s, _, _, _ = config1
    opt = G.TopOptOptions(n_loop=1, tol=1e-6, maxit=2000, Emin=1e-9)
    xp_o, hist_o = G.topopt_global_volume(m, opt)
    xp, hist = s.TopOpti_GlobalVolumeConstraint(m.F, volfrac=0.3, rMin=1.5, nLoop=1, tol=1e-6, maxIT=2000,
                                                Emin=1e-9)
    assert len(hist) == len(hist_o) == 1
    a, b = hist[0], hist_o[0]
    assert abs(a["cg_iterations"] - b["its"]) <= 1
    assert abs(a["compliance"] - b["c"]) <= 1e-6 * abs(b["c"])
    assert abs(a["volume"] - b["vol"]) <= 1e-9
    assert abs(a["change"] - b["change"]) <= 1e-5
    assert abs(a["sharpness"] - b["sharp"]) <= 1e-6
    assert np.abs(xp - xp_o).max() <= 1e-5


@pytest.fixture(scope="module")
def part(built_lib):
    from sgldbench_gb300 import VoxelSolver
    from sgldbench_gb300 import topvoxel as T

    tv = T.model_from_npz(os.path.join(HERE, "golden", "part_R256_model.npz"))
    s = VoxelSolver(tv.voxels, num_levels=5, non_dyadic=0, omega=0.6)
    fixed, F = T.boundary_conditions(tv, s)
    m = G.build_model_fixed(s.voxels, fixed, non_dyadic=0, omega=0.6, num_levels=5)
    assert m.numLevels == 5 and m.levels[0].numDOFs == s.numDOFs
    m.F = F
    E = np.ones(s.numElements)
    G.set_modulus(m, E)
    G.assemble_stencil(m)
    s.set_fixed_dofs(fixed)
    s.set_modulus(E)
    s.Solving_AssembleFEAstencil()
    U_o, its_o = G.solve(m, tol=1e-6, maxIT=5000)
    U_c, _ = G.solve(m, tol=1e-10, maxIT=10000, x0=U_o)
    yield m, s, U_o, its_o, U_c
    s.close()


def test_part_fp64_matches_oracle(part):
    m, s, U_o, its_o, _ = part
    U, info = s.pcg(m.F, tol=1e-6, maxIT=5000)
    assert info["converged"]
    assert abs(info["its"] - its_o) <= 1, (info["its"], its_o)
    assert np.linalg.norm(U - U_o) / np.linalg.norm(U_o) <= 1e-8


def test_part_mixed_matches_oracle(part):
    m, s, _, _, U_c = part
    U, info = s.pcg(m.F, tol=1e-6, maxIT=5000, precision="mixed_df")
    assert info["converged"] and info["true_relres"] <= 1e-6, info
    c_ref = G.compliance(m, U_c)
    _, c = s.TopOpti_ComputeUnitCompliance(U)
    assert abs(c - c_ref) / abs(c_ref) <= 1e-6
    assert np.linalg.norm(U - U_c) / np.linalg.norm(U_c) <= 1e-4


@pytest.fixture(scope="module")
def part_default(built_lib):
    """part_R256 with the reference's default level rule and first step."""
    from sgldbench_gb300 import VoxelSolver
    from sgldbench_gb300 import topvoxel as T

    tv = T.model_from_npz(os.path.join(HERE, "golden", "part_R256_model.npz"))
    s = VoxelSolver(tv.voxels, omega=0.6)   # num_levels from the reference rule, non_dyadic = 1
    fixed, F = T.boundary_conditions(tv, s)
    m = G.build_model_fixed(s.voxels, fixed, omega=0.6)
    assert m.numLevels == s.numLevels == 3
    assert (s.levels[-1]["resX"], s.levels[-1]["resY"], s.levels[-1]["resZ"]) == (32, 20, 14)
    for i, lv in enumerate(m.levels, 1):
        info = s.levels[i - 1]
        assert (info["resX"], info["resY"], info["resZ"]) == (lv.resX, lv.resY, lv.resZ)
    m.F = F
    E = np.ones(s.numElements)
    G.set_modulus(m, E)
    G.assemble_stencil(m)
    s.set_fixed_dofs(fixed)
    s.set_modulus(E)
    s.Solving_AssembleFEAstencil()
    U_o, its_o = G.solve(m, tol=1e-6, maxIT=5000)
    yield m, s, U_o, its_o
    s.close()


def test_part_default_hierarchy_matches_oracle(part_default):
    m, s, U_o, its_o = part_default
    U, info = s.pcg(m.F, tol=1e-6, maxIT=5000)
    assert info["converged"]
    assert abs(info["its"] - its_o) <= 1, (info["its"], its_o)
    assert np.linalg.norm(U - U_o) / np.linalg.norm(U_o) <= 1e-8
    Um, im = s.pcg(m.F, tol=1e-6, maxIT=5000, precision="mixed_df")
    assert im["converged"] and im["true_relres"] <= 1e-6
    c_o = float(m.F @ U_o)
    assert abs(float(m.F @ Um) - c_o) <= 1e-5 * abs(c_o)
