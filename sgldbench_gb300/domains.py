"""Seeded synthetic voxel models and boundary conditions for the solve path.

The reference's benchmark models are surface meshes voxelized in MATLAB; the
workloads here are synthetic stand-ins with the shapes, sizes and value
distributions of the benchmark configurations:

* ``cuboid``: a solid box (configs 0 and 1);
* ``graded_density``: seeded U[0,1) noise, Gaussian-smoothed, mapped to
  [rho_min, 1] (config 1), with ``simp_modulus`` for E;
* ``blobby_union``: union of seeded spheres and boxes, largest 26-connected
  component (config 2);
* ``gaussian_blobs``: thresholded sum of seeded Gaussian blobs (config 4).

Boundary conditions follow the reference's conventions: node indices are the
compact node numbering, DOFs are node-major [ux uy uz].
"""
from __future__ import annotations

import numpy as np


def cuboid(nx: int, ny: int, nz: int) -> np.ndarray:
    """Solid (ny, nx, nz) voxel grid (MATLAB size order [nely nelx nelz])."""
    return np.ones((ny, nx, nz), dtype=bool)


def node_coords(nodMapBack: np.ndarray, resY: int, resX: int) -> np.ndarray:
    """(ix, iy_row, iz) grid coordinates of compact nodes (1-based nodMapBack)."""
    n = np.asarray(nodMapBack, dtype=np.int64) - 1
    NY, NX = resY + 1, resX + 1
    iy = n % NY
    ix = (n // NY) % NX
    iz = n // (NY * NX)
    return ix, iy, iz


def boundary_nodes(voxels: np.ndarray, nodMapBack: np.ndarray) -> np.ndarray:
    """Mask of compact nodes shared by fewer than 8 solid voxels
    (FEA_VoxelBasedDiscretization.m:229-235)."""
    ny, nx, nz = voxels.shape
    cnt = np.zeros((ny + 1, nx + 1, nz + 1), np.int16)
    v = voxels.astype(np.int16)
    for dy in (0, 1):
        for dx in (0, 1):
            for dz in (0, 1):
                cnt[dy:dy + ny, dx:dx + nx, dz:dz + nz] += v
    flat = cnt.reshape(-1, order="F")
    return flat[np.asarray(nodMapBack, np.int64) - 1] < 8


def cantilever3(voxels: np.ndarray, nodMapBack: np.ndarray, nelx: int | None = None):
    """'Cuboid - Cantilever 3' (FEA_BuiltInBoundaryConditions4CuboidDesignDomain.m:34-44):
    fix the boundary nodes at the minimal x; a total unit -z load spread evenly
    over the boundary nodes with x == nelx and z == minimal z.
    Returns (F (numDOFs,), fixed mask (numDOFs,))."""
    ny, nx, nz = voxels.shape
    nelx = nx if nelx is None else nelx
    ix, iy, iz = node_coords(nodMapBack, ny, nx)
    bnd = boundary_nodes(voxels, nodMapBack)
    xb, zb = ix[bnd], iz[bnd]
    fixed_nodes = np.nonzero(bnd & (ix == xb.min()))[0]
    loaded = np.nonzero(bnd & (ix == nelx) & (iz == zb.min()))[0]
    nn = len(nodMapBack)
    fixed_nodes = np.setdiff1d(fixed_nodes, loaded)   # FEA_ApplyBoundaryCondition.m:9-10
    F = np.zeros((nn, 3))
    F[loaded, 2] = -1.0 / max(len(loaded), 1)
    fixed = np.zeros((nn, 3), bool)
    fixed[fixed_nodes, :] = True
    return F.reshape(-1), fixed.reshape(-1)


def graded_density(nx: int, ny: int, nz: int, seed: int = 0, sigma: float = 2.0, rho_min: float = 1e-3):
    """Config-1 style density: U[0,1) noise, Gaussian smoothing (sigma in
    voxels), affine map to [rho_min, 1].  Returned in compact element order
    (column-major over (ny, nx, nz))."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    r = rng.random((ny, nx, nz))
    s = gaussian_filter(r, sigma=sigma, mode="nearest")
    s = (s - s.min()) / max(s.max() - s.min(), 1e-300)
    rho = rho_min + s * (1.0 - rho_min)
    return rho.reshape(-1, order="F")


def simp_modulus(rho, E0: float = 1.0, Emin: float = 1e-9, p: float = 3.0):
    """E = Emin + rho^p (E0 - Emin) (TopOpti_MaterialInterpolationSIMP.m:5)."""
    return Emin + np.asarray(rho, dtype=np.float64) ** p * (E0 - Emin)


def _largest_component(mask: np.ndarray, connectivity: int = 6) -> np.ndarray:
    """Largest connected component: face-connected (6) by default, so that no
    part hangs on a shared node or edge (a mechanical hinge that makes the
    stiffness matrix near-singular); 26 gives the corner-connected component."""
    from scipy.ndimage import generate_binary_structure, label

    rank = {6: 1, 18: 2, 26: 3}[connectivity]
    lab, n = label(mask, structure=generate_binary_structure(3, rank))
    if n <= 1:
        return mask
    sizes = np.bincount(lab.reshape(-1))
    sizes[0] = 0
    return lab == sizes.argmax()


def blobby_union(nx: int, ny: int, nz: int, seed: int = 0, n_spheres: int = 12, n_boxes: int = 8,
                 r_range=(20, 60), edge_range=(30, 120), fill: float | None = None) -> np.ndarray:
    """Config-2 style domain: union of seeded spheres and axis-aligned boxes,
    largest face-connected component (26-connected parts joined only through
    a node or an edge would hinge).  Radii / edges scale with the grid when it
    is smaller than 512 x 256 x 256.  With ``fill``, every radius and edge is
    multiplied by one common factor (>= 1, found by bisection) so that the
    largest component covers about that fraction of the box: at the literal
    sizes twelve spheres and eight boxes cover only 10-20 % of a 512 x 256 x
    256 box and split into several components."""
    rng = np.random.default_rng(seed)
    scale = min(nx / 512, ny / 256, nz / 256)
    spheres = [(rng.uniform(*r_range) * scale, rng.uniform([0, 0, 0], [ny, nx, nz])) for _ in range(n_spheres)]
    boxes = [(rng.uniform(*edge_range, size=3) * scale, rng.uniform([0, 0, 0], [ny, nx, nz])) for _ in range(n_boxes)]
    y, x, z = np.ogrid[:ny, :nx, :nz]

    def build(k):
        m = np.zeros((ny, nx, nz), bool)
        for r, c in spheres:
            m |= (y - c[0]) ** 2 + (x - c[1]) ** 2 + (z - c[2]) ** 2 <= (k * r) ** 2
        for e, lo in boxes:
            hi = lo + k * e
            m[int(lo[0]):int(hi[0]), int(lo[1]):int(hi[1]), int(lo[2]):int(hi[2])] = True
        return _largest_component(m)

    if fill is None:
        return build(1.0)
    lo_k, hi_k = 1.0, 4.0
    best = build(lo_k)
    if best.mean() >= fill:
        return best
    for _ in range(12):
        mid = 0.5 * (lo_k + hi_k)
        m = build(mid)
        if m.mean() >= fill:
            hi_k, best = mid, m
        else:
            lo_k = mid
        if abs(m.mean() - fill) < 0.01:
            return m
    return best


def gaussian_blobs(nx: int, ny: int, nz: int, seed: int = 0, n_blobs: int = 64, fill: float = 0.3) -> np.ndarray:
    """Config-4 style domain: sum of seeded Gaussian blobs thresholded at the
    quantile that keeps about `fill` of the voxels, largest component."""
    rng = np.random.default_rng(seed)
    f = np.zeros((ny, nx, nz), np.float32)
    yy = np.arange(ny, dtype=np.float32)[:, None, None]
    xx = np.arange(nx, dtype=np.float32)[None, :, None]
    zz = np.arange(nz, dtype=np.float32)[None, None, :]
    for _ in range(n_blobs):
        c = rng.uniform([0, 0, 0], [ny, nx, nz])
        s = rng.uniform(0.05, 0.15) * min(nx, ny, nz)
        gy = np.exp(-((yy - c[0]) ** 2) / (2 * s * s))
        gx = np.exp(-((xx - c[1]) ** 2) / (2 * s * s))
        gz = np.exp(-((zz - c[2]) ** 2) / (2 * s * s))
        f += gy * gx * gz
    thr = np.quantile(f, 1.0 - fill)
    return _largest_component(f >= thr)


def fix_bottom_layers(voxels: np.ndarray, nodMapBack: np.ndarray, layers: int = 4) -> np.ndarray:
    """Fixed mask: every DOF of the nodes in the lowest `layers` voxel layers (z)."""
    ny, nx, _ = voxels.shape
    _, _, iz = node_coords(nodMapBack, ny, nx)
    zmin = iz.min()
    fixed = np.repeat((iz <= zmin + layers)[:, None], 3, axis=1)
    return fixed.reshape(-1)


def patch_loads(voxels: np.ndarray, nodMapBack: np.ndarray, nrhs: int, seed: int = 0, radius: float = 10.0,
                exclude_below: int = 4):
    """nrhs load cases, each a unit force in a random direction spread evenly
    over the boundary nodes within `radius` of a random boundary node."""
    ny, nx, _ = voxels.shape
    ix, iy, iz = node_coords(nodMapBack, ny, nx)
    bnd = np.nonzero(boundary_nodes(voxels, nodMapBack) & (iz > iz.min() + exclude_below))[0]
    rng = np.random.default_rng(seed)
    nn = len(nodMapBack)
    out = np.zeros((nrhs, 3 * nn))
    for k in range(nrhs):
        c = bnd[rng.integers(len(bnd))]
        d = ((ix[bnd] - ix[c]) ** 2 + (iy[bnd] - iy[c]) ** 2 + (iz[bnd] - iz[c]) ** 2) <= radius ** 2
        sel = bnd[d]
        v = rng.standard_normal(3)
        v /= np.linalg.norm(v)
        f = np.zeros((nn, 3))
        f[sel] = v / len(sel)
        out[k] = f.reshape(-1)
    return out


def perturbed_patch_cases(voxels: np.ndarray, nodMapBack: np.ndarray, n: int, seed: int = 0, base_seed: int = 0,
                          radius: float = 10.0, shift: float = 8.0, max_angle_deg: float = 30.0,
                          exclude_below: int = 4):
    """n perturbed versions of one load case (a unit force spread evenly over
    the boundary nodes within `radius` of a boundary node), as a list of
    (compact node indices, force per node (3,)).  The base case's centre node
    and direction come from `base_seed`; each perturbed case moves the centre
    to a random boundary node within `shift` voxels of the base centre and
    turns the direction by a random rotation of at most `max_angle_deg`
    degrees; cases from another `seed` are held-out cases of the same
    distribution.  The reference's robustness study turns its loads by Euler
    angles (GUIs/Mtd_StructuralRobustnessExploration.m, UpdateButtonPushed);
    here the patch moves as well, so that a case is not a combination of
    others."""
    ny, nx, _ = voxels.shape
    ix, iy, iz = node_coords(nodMapBack, ny, nx)
    bnd = np.nonzero(boundary_nodes(voxels, nodMapBack) & (iz > iz.min() + exclude_below))[0]
    base = np.random.default_rng(base_seed)
    c0 = bnd[base.integers(len(bnd))]
    d0 = base.standard_normal(3)
    d0 /= np.linalg.norm(d0)
    near = bnd[((ix[bnd] - ix[c0]) ** 2 + (iy[bnd] - iy[c0]) ** 2 + (iz[bnd] - iz[c0]) ** 2) <= shift ** 2]
    rng = np.random.default_rng(seed)
    cases = []
    for _ in range(n):
        c = near[rng.integers(len(near))]
        sel = bnd[((ix[bnd] - ix[c]) ** 2 + (iy[bnd] - iy[c]) ** 2 + (iz[bnd] - iz[c]) ** 2) <= radius ** 2]
        axis = rng.standard_normal(3)
        axis /= np.linalg.norm(axis)
        ang = np.deg2rad(max_angle_deg) * rng.random()
        # Rodrigues' rotation of d0 about `axis` by `ang`
        v = d0 * np.cos(ang) + np.cross(axis, d0) * np.sin(ang) + axis * (axis @ d0) * (1.0 - np.cos(ang))
        cases.append((sel, v / len(sel)))
    return cases


def dense_load(num_nodes: int, case, out: np.ndarray | None = None) -> np.ndarray:
    """The load vector (3 num_nodes,) of one (nodes, force per node) case."""
    f = np.zeros(3 * num_nodes) if out is None else out
    if out is not None:
        f[...] = 0.0
    sel, v = case
    f.reshape(-1, 3)[sel] = v
    return f


def perturbed_patch_loads(voxels: np.ndarray, nodMapBack: np.ndarray, n: int, **kw) -> np.ndarray:
    """perturbed_patch_cases as a dense (n, numDOFs) array."""
    nn = len(nodMapBack)
    return np.stack([dense_load(nn, c) for c in perturbed_patch_cases(voxels, nodMapBack, n, **kw)])
