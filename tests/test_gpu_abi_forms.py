"""GPU: the entry points in the form the solve path's boundary lists them.

* sgld_kbyu_prec / sgld_vcycle_prec: K*u and the V-cycle with a precision
  argument (FP64 = the reference form; the FP32 and double-float operators of
  the mixed solves), against the FP64 operators;
* sgld_build_hierarchy: Solving_BuildingMeshHierarchy as a call of its own,
  against contexts created with that level count, keeping a user-set Ke, and
  leaving the context unchanged on error;
* sgld_solve: several load cases with plain arguments, against sgld_solve_block;
* sgld_vonmises: against sgld_stress.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _make(vox, levels, seed=3, **kw):
    from sgldbench_gb300 import VoxelSolver
    from sgldbench_gb300 import domains as D

    s = VoxelSolver(vox, num_levels=levels, non_dyadic=0, omega=0.6, pad=False, **kw)
    F, fixed = D.cantilever3(vox, s.nodMapBack(1))
    E = np.random.default_rng(seed).uniform(0.2, 1.0, s.numElements)
    s.set_fixed_dofs(fixed)
    s.set_modulus(E)
    s.Solving_AssembleFEAstencil()
    return s, F, fixed, E


@pytest.fixture(scope="module")
def vox(built_lib):
    from sgldbench_gb300 import domains as D

    return D.cuboid(32, 16, 16)


def test_operators_at_each_precision(vox):
    s, F, _, _ = _make(vox, 3)
    rng = np.random.default_rng(0)
    u = rng.standard_normal(s.numDOFs)
    y64 = s.Solving_KbyU_MatrixFree(u)
    assert np.array_equal(s.Solving_KbyU_MatrixFree(u, "fp64"), y64)
    ydf = s.Solving_KbyU_MatrixFree(u, "mixed_df")
    assert np.array_equal(ydf, s.kbyu_double_float(u))
    assert _rel(ydf, y64) <= 1e-12                    # double-float: ~2^-48 per operation
    assert _rel(s.Solving_KbyU_MatrixFree(u, "mixed"), y64) <= 5e-5   # FP32 u, moduli and sums
    r = F + 1e-3 * rng.standard_normal(s.numDOFs)
    z64 = s.Solving_Vcycle(r)
    z32 = s.Solving_Vcycle(r, "mixed")
    assert np.array_equal(s.Solving_Vcycle(r, "mixed_df"), z32)   # both modes precondition in FP32
    assert _rel(z32, z64) <= 2e-3                     # FP32 V-cycle incl. the FP32 coarse inverse
    s.close()


def test_build_hierarchy_matches_create(vox):
    from sgldbench_gb300._lib import SgldError

    s, F, fixed, E = _make(vox, 3)
    U3, i3 = s.pcg(F, tol=1e-8, maxIT=300)
    s.Solving_BuildingMeshHierarchy(2)
    assert s.numLevels == 2
    s.set_fixed_dofs(fixed)
    s.set_modulus(E)
    s.Solving_AssembleFEAstencil()
    U2, i2 = s.pcg(F, tol=1e-8, maxIT=300)
    t, *_ = _make(vox, 2)
    Ut, it = t.pcg(F, tol=1e-8, maxIT=300)
    assert i2["its"] == it["its"] and np.array_equal(U2, Ut)
    t.close()
    # back to 3 levels: the first solve again, bit for bit
    s.Solving_BuildingMeshHierarchy(3)
    s.set_fixed_dofs(fixed)
    s.set_modulus(E)
    s.Solving_AssembleFEAstencil()
    U3b, i3b = s.pcg(F, tol=1e-8, maxIT=300)
    assert i3b["its"] == i3["its"] and np.array_equal(U3b, U3)
    # an invalid level count is refused and leaves the context as it was
    with pytest.raises(SgldError):
        s.Solving_BuildingMeshHierarchy(1)
    assert s.lib.sgld_num_levels(s.ctx) == 3
    U3c, _ = s.pcg(F, tol=1e-8, maxIT=300)
    assert np.array_equal(U3c, U3)
    # a Ke set by the caller survives the rebuild
    o, *_ = _make(vox, 2, poisson_ratio=0.4)
    Ke = o.Ke
    o.close()
    s.set_ke(Ke)
    s.Solving_BuildingMeshHierarchy(2)
    assert np.array_equal(s.Ke, Ke)
    s.close()


def test_solve_and_vonmises(vox):
    s, F, fixed, _ = _make(vox, 3)
    noise = 1e-3 * np.random.default_rng(1).standard_normal(F.size)
    noise[np.asarray(fixed, bool)] = 0.0   # a load on a fixed DOF would keep a residual there
    Fb = np.stack([F, 0.5 * F + noise])
    for prec in ("fp64", "mixed_df"):
        U, its, relres = s.solve(Fb, tol=1e-8, maxIT=300, precision=prec)
        Ub, infos = s.solve_block(Fb, tol=1e-8, maxIT=300, precision=prec)
        assert np.array_equal(U, Ub)
        assert list(its) == [i["its"] for i in infos]
        assert np.array_equal(relres, np.array([i["relres"] for i in infos]))
        assert np.all(relres < 1e-8)
    _, vmn, vme = s.FEA_StressAnalysis(U[0])
    vme2, vmn2 = s.vonmises(U[0])
    assert np.array_equal(vme2, vme) and np.array_equal(vmn2, vmn)
    s.close()
