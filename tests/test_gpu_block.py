"""GPU: block right-hand side (config-2 style): an irregular union of spheres
and boxes, nodes of the lowest voxel layers fixed, load cases that are unit
forces in random directions over surface patches, all solved through
sgld_solve_block on one assembly.

Checks, per load case: the FP64 solve matches the oracle's solve of the same
case (iterations +-1, displacement relative L2 <= 1e-8 at tol 1e-6); the
mixed_df solve meets the tolerance on the true residual and its compliance is
within 1e-6 of an FP64 solve to 1e-10."""
import numpy as np
import pytest

from oracle import glue as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def block_case(built_lib):
    from sgldbench_gb300 import VoxelSolver
    from sgldbench_gb300 import domains as D

    nx, ny, nz = 64, 32, 32
    vox = D.blobby_union(nx, ny, nz, seed=4)
    s = VoxelSolver(vox, num_levels=3, non_dyadic=0, omega=0.6, pad=False)
    nodes = s.nodMapBack(1)
    fixed = D.fix_bottom_layers(vox, nodes, layers=4)
    F = D.patch_loads(vox, nodes, 2, seed=2, radius=5.0)
    s.set_fixed_dofs(fixed)
    E = np.ones(s.numElements)
    s.set_modulus(E)
    s.Solving_AssembleFEAstencil()
    m = G.build_model_fixed(vox, fixed, non_dyadic=0, omega=0.6, num_levels=3)
    G.set_modulus(m, E)
    G.assemble_stencil(m)
    return m, s, F


def test_block_fp64_matches_oracle(block_case):
    m, s, F = block_case
    U, infos = s.solve_block(F, tol=1e-6, maxIT=500)
    assert len(infos) == F.shape[0]
    for j in range(F.shape[0]):
        m.F = F[j]
        U_o, its_o = G.solve(m, tol=1e-6, maxIT=500)
        assert infos[j]["converged"] and abs(infos[j]["its"] - its_o) <= 1
        assert np.linalg.norm(U[j] - U_o) / np.linalg.norm(U_o) <= 1e-8


def test_block_mixed_df(block_case):
    m, s, F = block_case
    U, infos = s.solve_block(F, tol=1e-6, maxIT=500, precision="mixed_df")
    U64, _ = s.solve_block(F, tol=1e-10, maxIT=2000)
    for j in range(F.shape[0]):
        assert infos[j]["converged"] and infos[j]["true_relres"] <= 1e-6
        _, c = s.TopOpti_ComputeUnitCompliance(U[j])
        _, c64 = s.TopOpti_ComputeUnitCompliance(U64[j])
        assert abs(c - c64) / abs(c64) <= 1e-6


def test_block_warm_start_and_empty(block_case):
    m, s, F = block_case
    U, _ = s.solve_block(F, tol=1e-8, maxIT=1000)
    U2, infos = s.solve_block(F, tol=1e-6, maxIT=500, U0=U)
    assert all(i["its"] <= 1 for i in infos)
    Z, zi = s.solve_block(np.zeros((0, s.numDOFs)))
    assert Z.shape == (0, s.numDOFs) and zi == []
