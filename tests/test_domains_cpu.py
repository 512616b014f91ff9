"""CPU: the seeded synthetic models and load cases that stand in for the
reference's voxelized datasets have the shapes, fractions and invariants the
workloads state, and are reproducible from their seeds.

* graded_density (config 1): values in [rho_min, 1] reaching both ends,
  compact element order, SIMP modulus E = Emin + rho^p (E0 - Emin);
* blobby_union (config 2): one face-connected component at about the
  requested fill;
* gaussian_blobs (config 4): one face-connected component a little under the
  30 % threshold (the largest component of it);
* fix_bottom_layers: exactly the nodes of the lowest voxel layers;
* patch_loads / perturbed_patch_cases: unit total force on boundary nodes
  above the fixed layers; perturbed directions within the stated angle of the
  base direction and patch centres within the stated shift; training and
  held-out seeds give different cases of one distribution.

Node maps come from the voxel grid itself (nodes touched by a solid voxel, in
column-major order, 1-based), which is the level-1 map of an unpadded grid.
"""
import numpy as np
from scipy.ndimage import generate_binary_structure, label

from sgldbench_gb300 import domains as D


def _node_map(vox):
    ny, nx, nz = vox.shape
    cnt = np.zeros((ny + 1, nx + 1, nz + 1), np.int16)
    v = vox.astype(np.int16)
    for dy in (0, 1):
        for dx in (0, 1):
            for dz in (0, 1):
                cnt[dy:dy + ny, dx:dx + nx, dz:dz + nz] += v
    return np.nonzero(cnt.reshape(-1, order="F") > 0)[0] + 1


def _face_components(m):
    return label(m, structure=generate_binary_structure(3, 1))[1]


def test_graded_density_and_simp():
    rho = D.graded_density(32, 16, 16, seed=1)
    assert rho.shape == (32 * 16 * 16,)
    assert abs(rho.min() - 1e-3) <= 1e-15 and abs(rho.max() - 1.0) <= 1e-15
    assert np.array_equal(rho, D.graded_density(32, 16, 16, seed=1))
    assert not np.array_equal(rho, D.graded_density(32, 16, 16, seed=2))
    # smoothing with sigma = 2 voxels: neighbours along y (fastest index) differ far less than
    # independent samples would
    g = rho.reshape((16, 32, 16), order="F")
    assert np.abs(np.diff(g, axis=0)).mean() < 0.1 * np.abs(g - g.mean()).mean() + 0.05
    E = D.simp_modulus(rho)
    assert np.allclose(E, 1e-9 + rho ** 3 * (1.0 - 1e-9), rtol=0, atol=1e-15)


def test_blobby_union_fill_and_connectivity():
    m = D.blobby_union(128, 64, 64, seed=0, fill=0.4)
    assert m.shape == (64, 128, 64)
    assert _face_components(m) == 1
    assert abs(m.mean() - 0.4) <= 0.02
    assert np.array_equal(m, D.blobby_union(128, 64, 64, seed=0, fill=0.4))


def test_gaussian_blobs_fill_and_connectivity():
    a = D.gaussian_blobs(64, 32, 32, seed=3, fill=0.3)
    assert a.shape == (32, 64, 32)
    assert _face_components(a) == 1
    assert 0.2 <= a.mean() <= 0.3 + 1e-3
    assert np.array_equal(a, D.gaussian_blobs(64, 32, 32, seed=3, fill=0.3))
    assert not np.array_equal(a, D.gaussian_blobs(64, 32, 32, seed=4, fill=0.3))


def test_fixed_layers_and_patch_loads():
    vox = D.gaussian_blobs(64, 32, 32, seed=0, fill=0.3)
    nmap = _node_map(vox)
    ny, nx, _ = vox.shape
    ix, iy, iz = D.node_coords(nmap, ny, nx)
    fixed = D.fix_bottom_layers(vox, nmap, layers=4).reshape(-1, 3)
    assert np.array_equal(fixed[:, 0], iz <= iz.min() + 4)
    assert np.array_equal(fixed[:, 0], fixed[:, 1]) and np.array_equal(fixed[:, 0], fixed[:, 2])
    bnd = D.boundary_nodes(vox, nmap)
    F = D.patch_loads(vox, nmap, 4, seed=5)
    assert F.shape == (4, 3 * len(nmap))
    for f in F:
        f3 = f.reshape(-1, 3)
        on = np.any(f3 != 0, axis=1)
        assert on.any() and np.all(bnd[on]) and np.all(iz[on] > iz.min() + 4)
        assert abs(np.linalg.norm(f3.sum(axis=0)) - 1.0) <= 1e-12
        assert not np.any(fixed.reshape(-1)[f != 0])


def test_perturbed_cases():
    vox = D.gaussian_blobs(64, 32, 32, seed=0, fill=0.3)
    nmap = _node_map(vox)
    ny, nx, _ = vox.shape
    ix, iy, iz = D.node_coords(nmap, ny, nx)
    pos = np.stack([ix, iy, iz], axis=1).astype(float)
    train = D.perturbed_patch_cases(vox, nmap, 6, seed=1)
    held = D.perturbed_patch_cases(vox, nmap, 6, seed=2)
    dirs = []
    for sel, v in train + held:
        assert abs(np.linalg.norm(v) * len(sel) - 1.0) <= 1e-12   # unit total force
        dirs.append(v / np.linalg.norm(v))
    dirs = np.array(dirs)
    # every direction lies within 30 degrees of the base direction, so any two within 60
    cos = dirs @ dirs.T
    assert cos.min() >= np.cos(np.deg2rad(60.0)) - 1e-12
    # the patch centres (mean of the loaded nodes) stay near one another: centre moves of at
    # most 8 voxels, patches of radius 10
    cen = np.array([pos[sel].mean(axis=0) for sel, _ in train + held])
    assert np.linalg.norm(cen - cen.mean(axis=0), axis=1).max() <= 8.0 + 10.0
    assert any(not np.array_equal(a[0], b[0]) or not np.allclose(a[1], b[1]) for a, b in zip(train, held))
    Fd = D.perturbed_patch_loads(vox, nmap, 3, seed=1)
    for k in range(3):
        assert np.array_equal(Fd[k], D.dense_load(len(nmap), train[k]))
