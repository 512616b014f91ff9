"""GPU parity: every operator of the solve path, through the C ABI, against
the oracle (CPU restatement of the reference, pinned to the reference's own
compiled MEX kernels by the CPU tests).

Tolerances (relative, max-norm unless stated):
  K*u, restriction, interpolation, Jacobi diagonals   1e-13
  FP32 K*u of the mixed solve's inner loop              1e-5
  FP32 restriction of the inner V-cycle                 1e-6
  Galerkin element matrices Ks                          1e-12
  V-cycle (coarsest solve through an explicit inverse)  1e-9
  PCG: iteration count equal to the oracle's (+-1); displacement relative L2
  vs the oracle's solve at the same tolerance 1e-6; against an FP64 solve to
  1e-10: displacement relative L2 <= 1e-5 and compliance <= 1e-6.
"""
import numpy as np
import pytest

from oracle import glue as G

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def make_pair(vox, non_dyadic=1, omega=0.6, E=None, seed=0, crc=50000):
    from sgldbench_gb300 import VoxelSolver

    m = G.build_model(vox, coarsest_control=crc, non_dyadic=non_dyadic, omega=omega)
    s = VoxelSolver(vox, non_dyadic=non_dyadic, omega=omega, coarsest_resolution_control=crc)
    l1 = m.levels[0]
    if E is None:
        E = np.random.default_rng(seed).uniform(0.05, 1.0, l1.numElements)
    G.set_modulus(m, E)
    s.set_fixed_dofs(l1.fixedDOFs)
    s.set_modulus(E)
    G.assemble_stencil(m)
    s.Solving_AssembleFEAstencil()
    return m, s


@pytest.fixture(scope="module", params=["solid_nondyadic", "irregular", "solid_dyadic"])
def pair(request, built_lib):
    rng = np.random.default_rng(7)
    if request.param == "solid_nondyadic":
        vox = np.ones((8, 16, 8), bool)
        return make_pair(vox, non_dyadic=1)
    if request.param == "irregular":
        vox = rng.random((16, 24, 16)) < 0.7
        return make_pair(vox, non_dyadic=1, seed=3)
    vox = np.ones((16, 32, 16), bool)
    return make_pair(vox, non_dyadic=0, seed=5)


def test_hierarchy_matches(pair):
    m, s = pair
    assert s.numLevels == m.numLevels
    for i, lv in enumerate(m.levels, 1):
        info = s.levels[i - 1]
        assert (info["resX"], info["resY"], info["resZ"]) == (lv.resX, lv.resY, lv.resZ)
        assert info["numElements"] == lv.numElements
        assert info["numNodes"] == lv.numNodes
        assert np.array_equal(s.eleMapBack(i), lv.eleMapBack.astype(np.int64))
    assert np.array_equal(s.nodMapBack(1), m.levels[0].nodMapBack.astype(np.int64))


def test_coarse_free_dofs(pair):
    m, s = pair
    for ii in range(2, m.numLevels + 1):
        assert np.array_equal(s.free_dofs(ii), m.levels[ii - 1].freeDOFs)


def test_kbyu(pair):
    m, s = pair
    u = np.random.default_rng(1).standard_normal(m.levels[0].numDOFs)
    assert _rel(s.Solving_KbyU_MatrixFree(u), G.kbyu(m, u)) <= 1e-13


def test_kbyu_fp32(pair):
    """The FP32 K*u of the inner solve (its 8-value form: the reference's
    isotropic element matrix has the cube's symmetry): FP32 u, moduli and sums,
    so 1e-5."""
    m, s = pair
    u = np.random.default_rng(11).standard_normal(m.levels[0].numDOFs)
    assert _rel(s.Solving_KbyU_MatrixFree(u, "mixed"), G.kbyu(m, u)) <= 1e-5


def _hadamard_to_ke(Ke, scale_blocks):
    """Ke with some of its Hadamard-basis blocks scaled: the transform of
    sgld_set_ke's check (corner order k = ks | kt<<1 | kp<<2, H the 8-point
    Hadamard matrix), applied, scaled blockwise and undone.  Scaling a whole
    diagonal block keeps the block pattern and the symmetry but, for unequal
    factors, breaks the cube's symmetry."""
    kmap = [0, 1, 3, 2, 4, 5, 7, 6]
    P = np.zeros((24, 24))
    for j in range(8):
        for c in range(3):
            P[3 * kmap[j] + c, 3 * j + c] = 1.0
    H = np.array([[np.prod([(1.0 if (k >> a) & 1 else -1.0) if (mm >> a) & 1 else 1.0 for a in range(3)])
                   for k in range(8)] for mm in range(8)])
    HH = np.kron(H, np.eye(3))
    Kh = HH @ (P @ Ke @ P.T) @ HH.T / 64.0
    for idx, f in scale_blocks:
        ix = np.ix_(idx, idx)
        Kh[ix] *= f
    return P.T @ (HH.T @ Kh @ HH) @ P


def test_kbyu_fp32_general_element_matrix(built_lib):
    """An element matrix with the Hadamard block pattern but without the
    cube's symmetry takes the FP32 K*u's 45-value form; both forms against the
    oracle with that matrix."""
    from oracle import kernels as OK

    rng = np.random.default_rng(12)
    vox = rng.random((12, 20, 10)) < 0.8
    m, s = make_pair(vox, non_dyadic=0, seed=6)
    l1 = m.levels[0]
    Ke2 = _hadamard_to_ke(m.Ke, [([9, 20], 1.2), ([11, 16, 18], 0.9)])
    assert np.allclose(Ke2, Ke2.T) and not np.allclose(Ke2, m.Ke)
    u = rng.standard_normal(l1.numDOFs)
    y_iso = G.kbyu(m, u)
    assert _rel(s.Solving_KbyU_MatrixFree(u, "mixed"), y_iso) <= 1e-5
    s.set_ke(Ke2)
    y2 = OK.kbyu(u, l1.eNodMat, Ke2, l1.eleModulus, l1.colors)
    y2[l1.fixedDOFs] = 0.0
    assert _rel(y2, y_iso) > 1e-3
    assert _rel(s.Solving_KbyU_MatrixFree(u, "mixed"), y2) <= 1e-5
    assert _rel(s.Solving_KbyU_MatrixFree(u), y2) <= 1e-13
    s.set_ke(m.Ke)
    assert _rel(s.Solving_KbyU_MatrixFree(u, "mixed"), y_iso) <= 1e-5
    s.close()


def test_mixed_solve_after_element_matrix_change(built_lib):
    """The captured solve graphs hold the FP32 K*u form chosen for the element
    matrix they were built with (the 8-value form for the reference's
    isotropic Ke).  After sgld_set_ke with a matrix without the cube's symmetry
    a mixed solve runs the general form: it converges without the FP64
    fallback, to the FP64 solve of the new system (displacement 1e-5)."""
    from sgldbench_gb300 import VoxelSolver
    from sgldbench_gb300 import domains as D

    vox = D.cuboid(32, 16, 16)
    s = VoxelSolver(vox, num_levels=3, non_dyadic=0, omega=0.6, pad=False)
    F, fixed = D.cantilever3(vox, s.nodMapBack(1))
    s.set_fixed_dofs(fixed)
    s.set_modulus(np.random.default_rng(4).uniform(0.2, 1.0, s.numElements))
    s.Solving_AssembleFEAstencil()
    for prec in ("mixed", "mixed_df"):
        _, info = s.pcg(F, tol=1e-6, maxIT=500, precision=prec)
        assert info["converged"] and not info["fallback"], info
    s.set_ke(_hadamard_to_ke(s.Ke, [([9, 20], 1.2), ([11, 16, 18], 0.9)]))
    s.Solving_AssembleFEAstencil()
    U64, _ = s.pcg(F, tol=1e-10, maxIT=2000, precision="fp64")
    for prec in ("mixed", "mixed_df"):
        U, info = s.pcg(F, tol=1e-6, maxIT=500, precision=prec)
        assert info["converged"] and not info["fallback"], info
        assert np.linalg.norm(U - U64) <= 1e-5 * np.linalg.norm(U64)
    s.close()


def test_restrict_interpolate(pair):
    m, s = pair
    rng = np.random.default_rng(2)
    for ii in range(2, m.numLevels + 1):
        rf = rng.standard_normal(m.levels[ii - 2].numDOFs)
        assert _rel(s.Solving_RestrictResidual(rf, ii), G.restrict(m.levels, rf, ii)) <= 1e-13
        xc = rng.standard_normal(m.levels[ii - 1].numDOFs)
        assert _rel(s.Solving_InterpolationDeviation(xc, ii), G.interpolate(m.levels, xc, ii)) <= 1e-13


def test_restrict_fp32(pair):
    """The FP32 restriction of the inner V-cycle against the oracle's: FP32
    input and sums of up to 27 taps, so 1e-6."""
    m, s = pair
    rng = np.random.default_rng(13)
    for ii in range(2, m.numLevels + 1):
        rf = rng.standard_normal(m.levels[ii - 2].numDOFs)
        assert _rel(s.Solving_RestrictResidual(rf, ii, "mixed"), G.restrict(m.levels, rf, ii)) <= 1e-6


def test_diag_and_stencils(pair):
    m, s = pair
    for ii in range(1, m.numLevels):
        assert _rel(s.diagK(ii), m.levels[ii - 1].diagK) <= 1e-13
    for ii in range(2, m.numLevels + 1):
        assert _rel(s.Ks(ii), m.levels[ii - 1].Ks) <= 1e-12


def test_vcycle(pair):
    m, s = pair
    r = np.random.default_rng(4).standard_normal(m.levels[0].numDOFs)
    r[m.levels[0].fixedDOFs] = 0.0
    assert _rel(s.Solving_Vcycle(r), G.vcycle(m, r)) <= 1e-9


def test_compliance_and_stress(pair):
    m, s = pair
    u = np.random.default_rng(5).standard_normal(m.levels[0].numDOFs)
    ce, c = s.TopOpti_ComputeUnitCompliance(u)
    ce_o = G.unit_compliance(m, u)
    assert _rel(ce, ce_o) <= 1e-13
    assert abs(c - G.compliance(m, u)) <= 1e-12 * abs(c)
    s6, vmn, vme = s.FEA_StressAnalysis(u)
    s6_o, vmn_o = G.stress_analysis(m, u)
    assert _rel(s6, s6_o) <= 1e-12
    assert _rel(vmn, vmn_o) <= 1e-12
    assert _rel(vme, G.per_element_von_mises(m, s6_o)) <= 1e-12


@pytest.fixture(scope="module")
def config0(built_lib):
    """Config 0: solid 64x32x32 cantilever, 3 levels (4:1 then 2:1), omega 0.6."""
    vox = np.ones((32, 64, 32), bool)
    m = G.build_model(vox, omega=0.6)
    from sgldbench_gb300 import VoxelSolver

    s = VoxelSolver(vox, omega=0.6)
    E = np.ones(m.levels[0].numElements)
    G.set_modulus(m, E)
    s.set_fixed_dofs(m.levels[0].fixedDOFs)
    s.set_modulus(E)
    G.assemble_stencil(m)
    s.Solving_AssembleFEAstencil()
    return m, s


def test_pcg_config0_matches_oracle(config0):
    m, s = config0
    U_o, its_o = G.solve(m, tol=1e-6, maxIT=500)
    U, info = s.pcg(m.F, tol=1e-6, maxIT=500)
    assert info["converged"]
    assert abs(info["its"] - its_o) <= 1, (info["its"], its_o)
    assert np.linalg.norm(U - U_o) / np.linalg.norm(U_o) <= 1e-8
    assert info["true_relres"] < 1.01e-6


def test_pcg_config0_vs_converged_fp64(config0):
    m, s = config0
    U_ref, _ = G.solve(m, tol=1e-10, maxIT=1000)
    U, info = s.pcg(m.F, tol=1e-6, maxIT=500)
    c_ref = G.compliance(m, U_ref)
    _, c = s.TopOpti_ComputeUnitCompliance(U)
    assert abs(c - c_ref) / abs(c_ref) <= 1e-6
    U10, _ = s.pcg(m.F, tol=1e-10, maxIT=1000)
    assert np.linalg.norm(U10 - U_ref) / np.linalg.norm(U_ref) <= 1e-5


def test_pcg_warm_start(config0):
    m, s = config0
    U1, info1 = s.pcg(m.F, tol=1e-6, maxIT=500)
    U2, info2 = s.pcg(m.F, tol=1e-6, maxIT=500, x0=U1)
    assert info2["its"] <= 2
    y_o, its_o = G.pcg(lambda u: G.kbyu(m, u), lambda r: G.vcycle(m, r), m.F, 1e-6, 500, x0=U1)
    assert abs(info2["its"] - its_o) <= 1


def test_principal_stress(pair):
    """Principal stresses per node and the dominant direction per element
    (FEA_ComputePrincipalStress.m, Common_ExtractDominantDirections...m)
    against the oracle: eigenvalues to 1e-10 of the largest |l| of the node;
    eigenvectors to 1e-7 where the eigenvalue gap exceeds 1e-3 of |l|max."""
    m, s = pair
    U, _ = s.pcg(m.F, tol=1e-8, maxIT=1000)
    s6, _ = G.stress_analysis(m, U)
    ps, dd = s.FEA_ComputePrincipalStress(U)
    ref = G.principal_stress(s6)
    lam, lam_r = ps[:, [0, 4, 8]], ref[:, [0, 4, 8]]
    scale = np.abs(lam_r).max(axis=1) + 1e-300
    assert (np.abs(lam - lam_r).max(axis=1) / scale).max() <= 1e-10
    for k in range(3):
        gaps = np.min([np.abs(lam_r[:, k] - lam_r[:, j]) for j in range(3) if j != k], axis=0) / scale
        ok = gaps > 1e-3
        assert ok.sum() > 0.5 * len(ok)
        v, vr = ps[ok, 4 * k + 1:4 * k + 4], ref[ok, 4 * k + 1:4 * k + 4]
        assert np.abs(v - vr).max() <= 1e-7
    # dominant direction: compare where the dominant |l| is separated from the others
    l1 = m.levels[0]
    cent = s6[l1.eNodMat - 1].mean(axis=1)
    pc = G.principal_stress(cent)
    a = np.sort(np.abs(pc[:, [0, 4, 8]]), axis=1)
    sep = (a[:, 2] - a[:, 1]) > 1e-3 * a[:, 2]
    ddr = G.dominant_directions(m, s6)
    assert np.abs(dd[sep] - ddr[sep]).max() <= 1e-7
