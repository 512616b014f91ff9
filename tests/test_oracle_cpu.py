"""CPU tests: the oracle is pinned to the reference.

* The oracle's C restatement of the MEX kernels reproduces the golden outputs
  of the reference's own compiled MEX kernels (tests/golden/ref_kernels.npz,
  made by tests/golden/make_golden.py): bit-exact for K*u, restriction,
  interpolation and the density filter, <= 1e-15 relative for the kernels
  whose inner summation order differs (assembly, unit compliance).
* The oracle's glue regenerates the reference's index tables for the same
  model and the hard-coded transfer tables of the MATLAB source.
* When the compiled reference kernels are present (this container), the
  oracle is also compared with them live on fresh inputs.
* Analytic invariants of the discretisation (Ke, P, the V-cycle).
"""
import os

import numpy as np
import pytest

from oracle import glue as G
from oracle import kernels as K
from oracle import mexcall

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(os.path.join(GOLD, "ref_kernels.npz")))


@pytest.fixture(scope="module")
def tables():
    return dict(np.load(os.path.join(GOLD, "ref_tables.npz")))


@pytest.fixture(scope="module")
def model(gold):
    m = G.build_model(gold["vox"], omega=0.6)
    G.set_modulus(m, gold["E"])
    return m


def _colors(gold, pre):
    return [gold[f"{pre}color{c}"] for c in range(8)]


def test_tables_match_reference_source(tables):
    for s in (2, 4):
        assert np.array_equal(G.ri_inNODE(s), tables[f"inNODE_{s}"])
        assert np.array_equal(G.ri_inDOF(s), tables[f"inDOF_{s}"])
        assert np.array_equal(G.sub_ele_nod_mat(s), tables[f"SubEleNodMat_{s}"])
    s, t, p, _ = G.gauss_points()
    assert np.array_equal(s, tables["gauss_s"]) and np.array_equal(t, tables["gauss_t"])
    assert np.array_equal(p, tables["gauss_p"])


def test_glue_reproduces_index_tables(gold, model):
    assert model.numLevels == int(gold["num_levels"])
    l1 = model.levels[0]
    assert np.array_equal(l1.eNodMat, gold["l1_eNodMat"])
    assert np.array_equal(l1.eleMapForward, gold["l1_eleMapForward"])
    for c in range(8):
        assert np.array_equal(l1.colors[c], gold[f"l1_color{c}"])
    for ii in range(2, model.numLevels + 1):
        lv = model.levels[ii - 1]
        for k in ("transferMat", "transferMatCoeffi", "solidNodeMapCoarser2Finer", "eNodMat", "elementUpwardMap",
                  "eleMapBack"):
            assert np.array_equal(getattr(lv, k), gold[f"l{ii}_{k}"]), (ii, k)


def test_kbyu_bit_exact(gold):
    y = K.kbyu(gold["u"], gold["l1_eNodMat"], gold["Ke"], gold["E"], _colors(gold, "l1_"))
    assert np.array_equal(y, gold["y_kbyu"])


def test_transfers_bit_exact(gold, model):
    for ii in range(2, int(gold["num_levels"]) + 1):
        pre = f"l{ii}_"
        nc, ng, nf, _ = gold[pre + "sizes"]
        RI = model.levels[ii - 1].multiGridOperatorRI
        rc = K.restriction(gold[pre + "rf"], gold[pre + "transferMat"], RI, gold[pre + "eNodMat"], nc, ng,
                           gold[pre + "solidNodeMapCoarser2Finer"], gold[pre + "transferMatCoeffi"],
                           _colors(gold, pre))
        assert np.array_equal(rc, gold[pre + "rc"]), ii
        xf = K.interpolation(gold[pre + "xc"], gold[pre + "transferMat"], RI, gold[pre + "eNodMat"], nf, ng,
                             gold[pre + "solidNodeMapCoarser2Finer"], gold[pre + "transferMatCoeffi"],
                             _colors(gold, pre))
        assert np.array_equal(xf, gold[pre + "xf"]), ii


def test_compliance_and_assembly(gold, model):
    ce = K.unit_compliance(gold["u"], gold["l1_eNodMat"], gold["Ke"])
    assert np.abs(ce - gold["ce"]).max() <= 1e-15 * np.abs(gold["ce"]).max() * 10
    c2 = model.levels[1]
    s2 = c2.spanWidth
    Ks2 = K.assemble_from_finest(gold["Ke"], gold["E"], gold["l2_elementUpwardMap"], G.ri_inDOF(s2),
                                 G.local_mapping(s2), (s2 + 1) ** 3)
    assert np.abs(Ks2 - gold["Ks2"]).max() <= 1e-14 * np.abs(gold["Ks2"]).max()
    s3 = model.levels[2].spanWidth
    Ks3 = K.assemble_from_nonfinest(gold["Ks2"], gold["l3_elementUpwardMap"], G.ri_inDOF(s3),
                                    G.local_mapping(s3), (s3 + 1) ** 3)
    assert np.abs(Ks3 - gold["Ks3"]).max() <= 1e-14 * np.abs(gold["Ks3"]).max()


def test_density_filter_bit_exact(gold):
    nx, ny, nz = gold["l1_res"]
    hs = K.density_filter(None, 1.5, gold["l1_eleMapForward"], nx, ny, nz)
    assert np.array_equal(hs, gold["Hs"])
    f = K.density_filter(gold["filter_x"], 1.5, gold["l1_eleMapForward"], nx, ny, nz)
    assert np.array_equal(f, gold["filtered"])


@pytest.mark.skipif(mexcall.ref_lib() is None, reason="reference MEX kernels not built here")
def test_live_against_reference_kernels():
    R = mexcall.ref_lib()
    rng = np.random.default_rng(11)
    vox = rng.random((8, 16, 8)) < 0.8
    m = G.build_model(vox, omega=0.6)
    l1 = m.levels[0]
    E = rng.uniform(0.1, 1.0, l1.numElements)
    u = rng.standard_normal(l1.numDOFs)
    y = R.call("ref_Solving_KbyU_MatrixFree_mex", 1, u, l1.eNodMat, m.Ke, E, l1.colors).ravel()
    assert np.array_equal(y, K.kbyu(u, l1.eNodMat, m.Ke, E, l1.colors))
    with pytest.raises(mexcall.MexError):   # the reference's own argument checks (mex:32-46)
        R.call("ref_Solving_KbyU_MatrixFree_mex", 1, u, l1.eNodMat.astype(np.float64), m.Ke, E, l1.colors)


# ---------------------------------------------------------------------------
# invariants
# ---------------------------------------------------------------------------
def test_element_stiffness_invariants():
    Ke = G.element_stiffness(0.3)
    assert np.allclose(Ke, Ke.T, atol=1e-15)
    ev = np.linalg.eigvalsh(Ke)
    assert (np.abs(ev[:6]) < 1e-12).all() and (ev[6:] > 1e-3).all()   # 6 rigid-body modes


def test_prolongation_reproduces_linear_fields():
    vox = np.ones((8, 16, 8), bool)
    m = G.build_model(vox, omega=0.6)
    for ii in range(2, m.numLevels + 1):
        c, f = m.levels[ii - 1], m.levels[ii - 2]

        # coordinates of the coarse and fine nodes on their own grids
        def coords(lv):
            full = np.unique(_enod_full(lv)) - 1
            NY, NX = lv.resY + 1, lv.resX + 1
            return np.stack([full % NY, (full // NY) % NX, full // (NY * NX)], 1).astype(float)

        cc = coords(c) * c.spanWidth
        fc = coords(f)
        a = np.array([0.3, -1.2, 0.7])
        xc = np.repeat((cc @ a)[:, None], 3, axis=1).reshape(-1)
        xf = G.interpolate(m.levels, xc, ii).reshape(-1, 3)
        assert np.allclose(xf[:, 0], fc @ a, atol=1e-12)
        for row in c.multiGridOperatorRI:
            assert abs(row.sum() - 1.0) < 1e-15


def _enod_full(lv):
    return G._full_enodmat(lv.resX, lv.resY, lv.resZ)[lv.eleMapBack.astype(np.int64) - 1]


def test_vcycle_symmetric_and_compliance_identity():
    rng = np.random.default_rng(3)
    vox = rng.random((8, 16, 8)) < 0.85
    m = G.build_model(vox, omega=0.6)
    G.set_modulus(m, rng.uniform(0.2, 1.0, m.levels[0].numElements))
    G.assemble_stencil(m)
    free = m.levels[0].freeDOFs
    a = rng.standard_normal(m.levels[0].numDOFs) * free
    b = rng.standard_normal(m.levels[0].numDOFs) * free
    assert abs(G.vcycle(m, a) @ b - a @ G.vcycle(m, b)) <= 1e-10 * abs(a @ G.vcycle(m, b))
    U, its = G.solve(m, tol=1e-10, maxIT=2000)
    assert abs(G.compliance(m, U) - m.F @ U) <= 1e-8 * abs(m.F @ U)


def test_pde_kbyu_matches_reference_kernel():
    """The oracle's scalar 8 x 8 product against the reference's own
    Solving_KbyU_MatrixFree8x8_mex.cpp (compiled from the checkout)."""
    from oracle import mexcall

    R = mexcall.ref_lib()
    if R is None:
        pytest.skip("reference kernels not built (oracle/_ref)")
    rng = np.random.default_rng(5)
    vox = rng.random((8, 12, 6)) < 0.8
    m = G.build_model(vox, omega=0.6)
    l1 = m.levels[0]
    Ke8 = G.pde_element_matrix(1.5 * 2)
    u = rng.standard_normal(l1.numNodes)
    y_ref = R.call("ref_Solving_KbyU_MatrixFree8x8_mex", 1, u, l1.eNodMat, Ke8, l1.colors).ravel()
    assert np.abs(G.pde_kbyu(l1, Ke8, u) - y_ref).max() <= 1e-13 * np.abs(y_ref).max()
    # element matrix: symmetric, rows of the Laplacian part sum to zero, mass part sums to the volume
    s, t, p, w = G.gauss_points()
    dN = G.shape_derivatives(s, t, p)
    assert np.allclose(Ke8, Ke8.T) and abs((dN.T @ dN).sum()) < 1e-12
    assert abs(G.pde_element_matrix(0.0).sum() - 1.0) < 1e-12


@pytest.mark.parametrize("m", [1, 2])
def test_mma_restatement_matches_reference(m):
    """oracle/mma.py against the reference's own MMA_mex.cpp + MMAseq.cpp
    (compiled from the checkout): one update of a SIMP-like problem."""
    from oracle import mma, mexcall

    R = mexcall.ref_lib()
    if R is None:
        pytest.skip("reference kernels not built (oracle/_ref)")
    rng = np.random.default_rng(7 + m)
    n = 3000
    x = rng.uniform(0.05, 0.95, n)
    xmin, xmax = np.maximum(0, x - 0.1), np.minimum(1, x + 0.1)
    df0 = -rng.uniform(0.001, 2.0, n)
    dfdx = np.stack([np.ones(n) / (n * 0.3), rng.uniform(-1, 1, n) / n][:m], axis=1).reshape(-1)
    fval = np.array([x.sum() / (n * 0.3) - 1, 0.05][:m])
    xo1, xo2 = x * 0.98, x * 0.97
    ref = R.call("ref_MMA_mex", 3, float(m), float(n), x, xmin, xmax, xo1, xo2, df0, fval, dfdx)
    out = mma.mma_update(m, n, x, xmin, xmax, xo1, xo2, df0, fval, dfdx)
    for a, b in zip(out, ref):
        assert np.abs(a - np.asarray(b).ravel()).max() <= 1e-12


@pytest.mark.parametrize("levels,widths", [(1, [4]), (2, [4, 8]), (3, [4, 8, 8])])
def test_net_oracle_gradient(levels, widths):
    """The U-Net restatement's backward pass equals central finite differences
    of its loss (float64, no rounding): pins the oracle the GPU is checked against."""
    from oracle.net import UNet

    rng = np.random.default_rng(levels)
    dims = (7, 5, 4)
    n = UNet(dims, 4, 3, levels, widths, emulate=False)
    V = int(np.prod(dims))
    p = rng.standard_normal(n.nparam) * 0.3
    x = rng.standard_normal((V, 4))
    t = rng.standard_normal((V, 3))
    m = (rng.random(V) > 0.2).astype(float)
    _, g, _ = n.value_and_grad(p, x, t, m)
    h = 1e-6
    for _ in range(3):
        d = rng.standard_normal(n.nparam)
        lp, _, _ = n.value_and_grad(p + h * d, x, t, m)
        lm, _, _ = n.value_and_grad(p - h * d, x, t, m)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g @ d) <= 1e-7 * abs(g @ d)


def test_net_oracle_bf16_rounding():
    """Round to nearest even at the BF16 boundary (8 mantissa bits)."""
    from oracle.net import bf16

    v = bf16(np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -9, -3.14159, 0.0]))
    assert v.tolist() == [1.0, 1.0, 1.0078125, -3.140625, 0.0]
