"""GPU: edge cases of the solve path's inputs.

* a zero load: the solution is exactly 0 (the reference's PCG would divide
  by ||b|| = 0 and return NaN; here every precision and the block path return
  U = 0, converged, no iterations);
* every DOF fixed: assembly succeeds with an empty coarsest system;
* no DOF fixed (a floating body): the coarsest matrix is singular and the
  library reports SGLD_ERR_NUMERIC instead of iterating;
* the smallest domain, one 2x2x2 voxel block on 2 levels, against the oracle;
* an empty block (nrhs = 0) is covered in test_gpu_block.py;
* two live contexts of different materials, called in turn.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small(built_lib):
    from sgldbench_gb300 import VoxelSolver
    from sgldbench_gb300 import domains as D

    vox = D.cuboid(16, 8, 8)
    s = VoxelSolver(vox, num_levels=2, non_dyadic=0, omega=0.6, pad=False)
    F, fixed = D.cantilever3(vox, s.nodMapBack(1))
    s.set_fixed_dofs(fixed)
    s.set_modulus(np.ones(s.numElements))
    s.Solving_AssembleFEAstencil()
    return s, F, vox


@pytest.mark.parametrize("prec", ["fp64", "mixed", "mixed_df"])
def test_zero_load(small, prec):
    s, F, _ = small
    U, info = s.pcg(np.zeros_like(F), tol=1e-6, maxIT=50, precision=prec)
    assert info["converged"] and info["its"] == 0 and not info["fallback"]
    assert np.all(U == 0.0)
    U0 = np.random.default_rng(0).standard_normal(F.size)
    U, info = s.pcg(np.zeros_like(F), tol=1e-6, maxIT=50, precision=prec, x0=U0)
    assert info["converged"] and np.all(U == 0.0)
    Ub, infos = s.solve_block(np.stack([np.zeros_like(F), F]), tol=1e-6, maxIT=200, precision=prec)
    assert np.all(Ub[0] == 0.0) and infos[0]["converged"]
    assert infos[1]["converged"] and np.abs(Ub[1]).max() > 0


def test_all_fixed_and_floating(small):
    from sgldbench_gb300 import VoxelSolver
    from sgldbench_gb300._lib import SgldError

    _, F, vox = small
    s = VoxelSolver(vox, num_levels=2, non_dyadic=0, omega=0.6, pad=False)
    s.set_fixed_dofs(np.ones(s.numDOFs, bool))
    s.set_modulus(np.ones(s.numElements))
    s.Solving_AssembleFEAstencil()
    U, info = s.pcg(np.zeros(s.numDOFs), tol=1e-6, maxIT=50)
    assert info["converged"] and np.all(U == 0.0)
    s.close()
    s = VoxelSolver(vox, num_levels=2, non_dyadic=0, omega=0.6, pad=False)
    s.set_fixed_dofs(np.zeros(s.numDOFs, bool))
    s.set_modulus(np.ones(s.numElements))
    with pytest.raises(SgldError) as e:
        s.Solving_AssembleFEAstencil()
    assert e.value.code == 4   # SGLD_ERR_NUMERIC: the coarsest matrix is not positive definite
    s.close()


def test_single_voxel_block(built_lib):
    from oracle import glue as G
    from sgldbench_gb300 import VoxelSolver

    vox = np.ones((2, 2, 2), bool)
    m = G.build_model(vox, omega=0.6, num_levels=2)
    s = VoxelSolver(vox, num_levels=2, omega=0.6)
    s.set_fixed_dofs(m.levels[0].fixedDOFs)
    E = np.array([1.0, 0.5, 0.25, 1.0, 0.75, 1.0, 0.3, 0.9])[: m.levels[0].numElements]
    G.set_modulus(m, E)
    G.assemble_stencil(m)
    s.set_modulus(E)
    s.Solving_AssembleFEAstencil()
    U_o, its_o = G.solve(m, tol=1e-10, maxIT=100)
    U, info = s.pcg(m.F, tol=1e-10, maxIT=100)
    assert info["converged"] and abs(info["its"] - its_o) <= 1
    assert np.linalg.norm(U - U_o) <= 1e-8 * np.linalg.norm(U_o)


def test_contexts_of_different_materials_alternate(built_lib, monkeypatch):
    """The element matrix sits in device constant memory shared by all contexts
    on a device.  Two live contexts with different Poisson ratios, called in
    turn, must each apply their own matrix: K*u and the FP64 and mixed solves
    match bit for bit what each context gives when it runs alone (with the
    default FP32 tile, so that both runs use the same one)."""
    from sgldbench_gb300 import VoxelSolver
    from sgldbench_gb300 import domains as D

    monkeypatch.setenv("SGLD_AUTOTUNE", "0")
    vox = D.cuboid(16, 8, 8)

    def make(nu):
        s = VoxelSolver(vox, num_levels=2, non_dyadic=0, omega=0.6, pad=False, poisson_ratio=nu)
        F, fixed = D.cantilever3(vox, s.nodMapBack(1))
        s.set_fixed_dofs(fixed)
        s.set_modulus(np.ones(s.numElements))
        s.Solving_AssembleFEAstencil()
        return s, F

    u = np.random.default_rng(1).standard_normal(3 * 17 * 9 * 9)

    def run(s, F):
        y = s.Solving_KbyU_MatrixFree(u[: F.size])
        U, _ = s.pcg(F, tol=1e-8, maxIT=200)
        Um, _ = s.pcg(F, tol=1e-8, maxIT=200, precision="mixed")
        return y, U, Um

    a, Fa = make(0.3)
    alone_a = run(a, Fa)
    a.close()
    b, Fb = make(0.45)
    alone_b = run(b, Fb)
    b.close()

    a, Fa = make(0.3)
    b, Fb = make(0.45)   # created last: its matrix is the one held
    for _ in range(2):
        got_a = run(a, Fa)
        got_b = run(b, Fb)
        for x, y in zip(got_a, alone_a):
            assert np.array_equal(x, y)
        for x, y in zip(got_b, alone_b):
            assert np.array_equal(x, y)
    assert not np.allclose(alone_a[0], alone_b[0])
    a.close()
    b.close()


def test_contexts_of_one_material_in_threads(built_lib, monkeypatch):
    """Contexts of equal element matrices may be used from concurrent host
    threads (ctypes releases the GIL during each call).  Two contexts run a
    mixed solve, a density filter and a PDE filter with different radii at the
    same time; every result matches the same calls made one after another."""
    import threading

    from sgldbench_gb300 import VoxelSolver
    from sgldbench_gb300 import domains as D

    monkeypatch.setenv("SGLD_AUTOTUNE", "0")
    vox = D.cuboid(32, 16, 16)
    rng = np.random.default_rng(4)

    def make(seed):
        s = VoxelSolver(vox, num_levels=3, non_dyadic=0, omega=0.6, pad=False)
        F, fixed = D.cantilever3(vox, s.nodMapBack(1))
        s.set_fixed_dofs(fixed)
        s.set_modulus(np.random.default_rng(seed).uniform(0.2, 1.0, s.numElements))
        s.Solving_AssembleFEAstencil()
        return s, F

    x = rng.random(32 * 16 * 16)
    jobs = [(make(1), 1.5, 2.0), (make(2), 3.0, 4.0)]

    def work(job):
        (s, F), rmin, rhat = job
        U, _ = s.pcg(F, tol=1e-8, maxIT=300, precision="mixed")
        return U, s.TopOpti_PerformDensityFiltering(x, rmin), s.TopOpti_PDEFiltering(x, rhat, tol=1e-10)[0]

    alone = [work(j) for j in jobs]
    for _ in range(3):
        got = [None, None]

        def run(i):
            got[i] = work(jobs[i])

        ts = [threading.Thread(target=run, args=(i,)) for i in range(2)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        for g, a in zip(got, alone):
            assert g is not None
            for u, v in zip(g, a):
                assert np.array_equal(u, v)
    for (s, _), _, _ in jobs:
        s.close()
