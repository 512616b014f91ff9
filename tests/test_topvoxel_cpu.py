"""CPU: the .TopVoxel reader (src/IO_ImportTopVoxels.m) and the mapping of
its boundary conditions onto the solver's compact DOFs.

The compact fixture tests/golden/part_R256_model.npz (made from the
reference's data/part_R256.TopVoxel by tests/golden/make_topvoxel_fixture.py)
carries the header counts the reference's file declares: 256 x 160 x 112,
1,845,040 solid voxels, 74,546 passive elements, 13,042 fixed nodes, 7,788
loaded nodes."""
import os

import numpy as np
import pytest

from oracle import glue as G
from oracle.refpath import reference_root
from sgldbench_gb300 import topvoxel as T

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "part_R256_model.npz")
_REF = reference_root()
REF_FILE = os.path.join(_REF, "data", "part_R256.TopVoxel") if _REF else ""


def test_fixture_counts():
    m = T.model_from_npz(FIXTURE)
    assert (m.nelx, m.nely, m.nelz) == (256, 160, 112)
    assert int(m.voxels.sum()) == 1845040
    assert m.passive.size == 74546 and m.fixing.shape == (13042, 4) and m.loading.shape == (7788, 4)
    assert np.all(m.fixing[:, 1:] == 1)
    assert abs(m.loading[:, 3].sum() + 1.0) < 1e-4 and np.all(m.loading[:, 1:3] == 0)
    # passive elements are solid voxels
    flat = m.voxels.reshape(-1, order="F")
    assert flat[m.passive - 1].all()


@pytest.mark.skipif(not os.path.exists(REF_FILE), reason="reference checkout not found (SGLD_REFERENCE)")
def test_reader_matches_fixture():
    a = T.read_topvoxel(REF_FILE)
    b = T.model_from_npz(FIXTURE)
    assert np.array_equal(a.voxels, b.voxels)
    assert np.array_equal(np.sort(a.passive), b.passive)
    assert np.array_equal(a.fixing, b.fixing) and np.array_equal(a.loading, b.loading)


def test_roundtrip_and_errors(tmp_path):
    rng = np.random.default_rng(0)
    vox = rng.random((6, 8, 5)) < 0.6
    NY, NX = 7, 9
    fixing = np.array([[1 + 0 + NY * 0, 1, 1, 1], [1 + 2 + NY * 3, 1, 0, 1]], float)
    loading = np.array([[1 + 6 + NY * (8 + NX * 5), 0.0, 0.5, -0.25]], float)
    dens = rng.random(int(vox.sum()))
    p = str(tmp_path / "m.TopVoxel")
    T.write_topvoxel(p, vox, fixing, loading, passive=[1, 3], density=dens)
    m = T.read_topvoxel(p)
    assert np.array_equal(m.voxels, vox) and m.passive.tolist() == [1, 3]
    assert np.allclose(m.density, dens, rtol=1e-4)
    assert np.array_equal(m.fixing, fixing[np.argsort(fixing[:, 0])]) and np.allclose(m.loading, loading)
    bad = str(tmp_path / "bad.TopVoxel")
    with open(p) as f, open(bad, "w") as g:
        g.write(f.read().replace("Fixations:", "Fixings:"))
    with pytest.raises(T.TopVoxelFormatError):
        T.read_topvoxel(bad)


class _FakeSolver:
    """resY/resX/resZ and the compact maps of level 1, as VoxelSolver exposes them."""

    def __init__(self, l1, pad_shape):
        self.resY, self.resX, self.resZ = pad_shape
        self._n, self._e = l1.nodMapBack.astype(np.int64), l1.eleMapBack.astype(np.int64)

    def nodMapBack(self, level=1):
        return self._n

    def eleMapBack(self, level=1):
        return self._e


def test_boundary_conditions_follow_apply_boundary_condition():
    """On a padded synthetic model, the mapped fixed mask and loads equal
    FEA_ApplyBoundaryCondition's on the same nodes (the reference indexes them
    through nodesOnBoundary after AdaptBCExternalMdl)."""
    rng = np.random.default_rng(3)
    vox = np.ones((10, 14, 6), bool)
    vox[rng.random(vox.shape) < 0.1] = False
    l1, nlev, pad, _ = G.voxel_discretization(vox, 50000, 3)
    NY, NX = vox.shape[0] + 1, vox.shape[1] + 1
    bn = l1.nodMapBack[l1.nodesOnBoundary - 1] - 1                    # padded full, 0-based
    PY, PX = pad.shape[0] + 1, pad.shape[1] + 1
    iy, ix, iz = bn % PY, (bn // PY) % PX, bn // (PY * PX)
    inside = (iy < NY) & (ix < NX) & (iz < vox.shape[2] + 1)
    pick = np.nonzero(inside)[0][:12]
    file_nodes = 1 + iy[pick] + NY * (ix[pick] + NX * iz[pick])
    model = T.TopVoxelModel(vox.shape[1], vox.shape[0], vox.shape[2], vox, None,
                            np.nonzero(vox.reshape(-1, order="F"))[0] + 1, np.zeros(0, np.int64),
                            T._unique_sorted(np.column_stack([file_nodes[:8], np.ones((8, 3))])),
                            T._unique_sorted(np.column_stack([file_nodes[6:], np.tile([0.0, 0.0, -1.0], (6, 1))])))
    fixed, F = T.boundary_conditions(model, _FakeSolver(l1, pad.shape))
    # the reference: node numbers -> boundary-node indices -> FEA_ApplyBoundaryCondition
    fixing = np.column_stack([pick[np.argsort(file_nodes[:8])] + 1, np.ones((8, 3))])
    loading = np.column_stack([pick[6:] + 1, np.tile([0.0, 0.0, -1.0], (6, 1))])
    F_ref = G.apply_boundary_condition(l1, fixing, loading)
    assert np.array_equal(fixed, l1.fixedDOFs)
    assert np.array_equal(F, F_ref)


def test_checkpoint_roundtrip(tmp_path):
    """The checkpoint format stores the loop state exactly and rejects foreign files."""
    import numpy as np
    import pytest

    from sgldbench_gb300 import checkpoint as CK

    rng = np.random.default_rng(0)
    st = {"loop": 7, "x": rng.random(100), "xPhys": rng.random(100), "U": rng.standard_normal(303)}
    p = str(tmp_path / "state.ckpt")
    CK.save(p, st)
    back = CK.load(p)
    assert back["loop"] == 7
    for k in ("x", "xPhys", "U"):
        assert np.array_equal(back[k], st[k])
    bad = tmp_path / "bad.ckpt"
    bad.write_bytes(b"NOTACKPT" + bytes(40))
    with pytest.raises(ValueError):
        CK.load(str(bad))
    good = (tmp_path / "state.ckpt").read_bytes()
    cut = tmp_path / "cut.ckpt"
    cut.write_bytes(good[:-8])          # last U entry missing
    with pytest.raises(ValueError):
        CK.load(str(cut))
