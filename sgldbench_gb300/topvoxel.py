"""Reader of SGLDBench's ``.TopVoxel`` voxel models and their boundary
conditions (src/IO_ImportTopVoxels.m:12-82, BC remap :84-134).

Format, version 1.0 (text):

    # Voxel Model for SGLDBench
    Version: 1.0
    Resolution: nelx nely nelz
    Density values: 0|1
    Solid voxels: N
    N lines: linear voxel index (1-based, column-major over (nely, nelx, nelz))
             [and its density when density values are included]
    Passive elements: P
    P lines: linear voxel index
    Fixations: F
    F lines: node fx fy fz   (node: 1-based, column-major over (nely+1, nelx+1, nelz+1);
                              f* = 1 fixes that displacement component)
    Loads: L
    L lines: node Fx Fy Fz

``read_topvoxel`` parses the file; ``boundary_conditions`` maps the fixations
and loads onto a ``VoxelSolver``'s compact DOFs after the grid was padded to
the multigrid multiple (what AdaptBCExternalMdl does before the reference
indexes its boundary nodes), and ``passive_elements`` maps the passive voxels
to compact element indices (AdaptPassiveElementsExternalMdl + eleMapForward).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class TopVoxelModel:
    nelx: int
    nely: int
    nelz: int
    voxels: np.ndarray            # bool (nely, nelx, nelz)
    density: np.ndarray | None    # per solid voxel, in file order, when included
    solid: np.ndarray             # 1-based linear voxel indices (file order)
    passive: np.ndarray           # 1-based linear voxel indices
    fixing: np.ndarray            # (F, 4): node, fx, fy, fz  (unique nodes, ascending)
    loading: np.ndarray           # (L, 4): node, Fx, Fy, Fz (unique nodes, ascending)


class TopVoxelFormatError(ValueError):
    pass


def _expect(tok, want):
    if tok != want:
        raise TopVoxelFormatError(f"Incompatible Mesh Data Format! expected {want!r}, found {tok!r}")


def _unique_sorted(rows: np.ndarray) -> np.ndarray:
    """unique(rows(:,1)) keeping the first occurrence, then sorted by node
    (IO_ImportTopVoxels.m:60-63 and :70-73)."""
    if rows.size == 0:
        return rows.reshape(0, 4)
    _, first = np.unique(rows[:, 0], return_index=True)
    rows = rows[first]
    return rows[np.argsort(rows[:, 0], kind="stable")]


def read_topvoxel(path: str) -> TopVoxelModel:
    with open(path, "rb") as f:
        toks = f.read().split()
    pos = 0

    def take(n=1):
        nonlocal pos
        out = toks[pos:pos + n]
        if len(out) < n:
            raise TopVoxelFormatError("unexpected end of file")
        pos += n
        return out

    take(4)                                  # "# Voxel Model for" ... (fscanf '%s %s %s %s')
    # the header's remaining words run up to "Version:"
    while toks[pos] != b"Version:":
        pos += 1
    take(1)
    version = float(take(1)[0])
    if version != 1.0:
        raise TopVoxelFormatError(f"Unsupported Data! version {version}")
    _expect(take(1)[0], b"Resolution:")
    nelx, nely, nelz = (int(t) for t in take(3))
    take(2)                                  # "Density values:"
    has_density = int(take(1)[0])
    take(2)                                  # "Solid voxels:"
    n_solid = int(take(1)[0])
    if has_density:
        vals = np.array(take(2 * n_solid), dtype=np.float64).reshape(n_solid, 2)
        solid = vals[:, 0].astype(np.int64)
        density = vals[:, 1].copy()
    else:
        solid = np.array(take(n_solid), dtype=np.int64)
        density = None
    _expect(take(1)[0], b"Passive")
    _expect(take(1)[0], b"elements:")
    n_passive = int(take(1)[0])
    passive = np.array(take(n_passive), dtype=np.int64)
    _expect(take(1)[0], b"Fixations:")
    n_fixed = int(take(1)[0])
    fixing = np.array(take(4 * n_fixed), dtype=np.float64).reshape(n_fixed, 4)
    _expect(take(1)[0], b"Loads:")
    n_loaded = int(take(1)[0])
    loading = np.array(take(4 * n_loaded), dtype=np.float64).reshape(n_loaded, 4)
    n = nelx * nely * nelz
    if solid.size and (solid.min() < 1 or solid.max() > n):
        raise TopVoxelFormatError("solid voxel index out of range")
    vol = np.zeros(n, dtype=bool)
    vol[solid - 1] = True
    voxels = vol.reshape((nely, nelx, nelz), order="F")
    return TopVoxelModel(nelx, nely, nelz, voxels, density, solid, passive, _unique_sorted(fixing),
                         _unique_sorted(loading))


def _node_yxz(model: TopVoxelModel, nodes_1based: np.ndarray):
    """1-based node numbers of the file's (nely+1, nelx+1, nelz+1) grid -> (iy, ix, iz)."""
    NY, NX = model.nely + 1, model.nelx + 1
    k = nodes_1based.astype(np.int64) - 1
    return k % NY, (k // NY) % NX, k // (NY * NX)


def boundary_conditions(model: TopVoxelModel, solver):
    """(fixed DOF mask, F) in ``solver``'s compact DOF order.

    The node numbers of the file refer to the unpadded grid; padding adds
    voxels at the high end of each axis, so a node keeps its (iy, ix, iz)
    (AdaptBCExternalMdl).  FEA_ApplyBoundaryCondition.m:9-42 then drops
    fixations of loaded nodes and fixes the components whose flag is 1."""
    NYp, NXp = solver.resY + 1, solver.resX + 1
    nodmap = solver.nodMapBack(1) - 1                       # compact -> padded full (0-based)
    fwd = np.full(NYp * NXp * (solver.resZ + 1), -1, dtype=np.int64)
    fwd[nodmap] = np.arange(nodmap.size)

    def compact(rows):
        iy, ix, iz = _node_yxz(model, rows[:, 0])
        full = iy + NYp * (ix + NXp * iz)
        c = fwd[full]
        if (c < 0).any():
            raise TopVoxelFormatError(f"{int((c < 0).sum())} boundary-condition nodes are not solid nodes")
        return c

    fixing = model.fixing[~np.isin(model.fixing[:, 0], model.loading[:, 0])]
    fixed = np.zeros((nodmap.size, 3), dtype=bool)
    if fixing.size:
        fixed[compact(fixing)] = fixing[:, 1:4] == 1
    F = np.zeros((nodmap.size, 3))
    if model.loading.size:
        F[compact(model.loading)] = model.loading[:, 1:4]
    return fixed.reshape(-1), F.reshape(-1)


def passive_elements(model: TopVoxelModel, solver) -> np.ndarray:
    """Compact (0-based) element indices of the passive voxels in ``solver``'s
    padded grid (AdaptPassiveElementsExternalMdl, then eleMapForward)."""
    if model.passive.size == 0:
        return np.zeros(0, dtype=np.int64)
    k = np.sort(model.passive) - 1
    iy, ix, iz = k % model.nely, (k // model.nely) % model.nelx, k // (model.nely * model.nelx)
    full = iy + solver.resY * (ix + solver.resX * iz)
    elemap = solver.eleMapBack(1) - 1
    fwd = np.full(solver.resY * solver.resX * solver.resZ, -1, dtype=np.int64)
    fwd[elemap] = np.arange(elemap.size)
    c = fwd[full]
    return c[c >= 0]


def model_from_npz(path: str) -> TopVoxelModel:
    """A TopVoxelModel from the compact fixture written by
    tests/golden/make_topvoxel_fixture.py (bit-packed masks in the file's
    column-major voxel order, fixations and loads)."""
    z = np.load(path)
    nelx, nely, nelz = (int(v) for v in z["res"])
    n = nelx * nely * nelz
    solid_mask = np.unpackbits(z["solid_bits"])[:n].astype(bool)
    passive_mask = np.unpackbits(z["passive_bits"])[:n].astype(bool)
    fixing = np.column_stack([z["fix_nodes"].astype(np.float64), z["fix_flags"].astype(np.float64)])
    loading = np.column_stack([z["load_nodes"].astype(np.float64), z["load_values"]])
    return TopVoxelModel(nelx, nely, nelz, solid_mask.reshape((nely, nelx, nelz), order="F"), None,
                         np.nonzero(solid_mask)[0] + 1, np.nonzero(passive_mask)[0] + 1,
                         _unique_sorted(fixing), _unique_sorted(loading))


def write_topvoxel(path: str, voxels: np.ndarray, fixing=None, loading=None, passive=None, density=None):
    """Writes a version-1.0 file (used to make synthetic models and fixtures)."""
    ny, nx, nz = voxels.shape
    solid = np.nonzero(voxels.reshape(-1, order="F"))[0] + 1
    fixing = np.zeros((0, 4)) if fixing is None else np.asarray(fixing)
    loading = np.zeros((0, 4)) if loading is None else np.asarray(loading)
    passive = np.zeros(0, dtype=np.int64) if passive is None else np.asarray(passive, dtype=np.int64)
    with open(path, "w") as f:
        f.write("# Voxel Model for SGLDBench\nVersion: 1.0\n")
        f.write(f"Resolution: {nx} {ny} {nz}\n")
        f.write(f"Density values: {0 if density is None else 1}\n")
        f.write(f"Solid voxels: {solid.size}\n")
        if density is None:
            f.write("".join(f"{i}\n" for i in solid))
        else:
            f.write("".join(f"{i} {d:.4e}\n" for i, d in zip(solid, density)))
        f.write(f"Passive elements: {passive.size}\n")
        f.write("".join(f"{i}\n" for i in passive))
        f.write(f"Fixations: {len(fixing)}\n")
        f.write("".join(f"{int(r[0])} {int(r[1])} {int(r[2])} {int(r[3])}\n" for r in fixing))
        f.write(f"Loads: {len(loading)}\n")
        f.write("".join(f"{int(r[0])} {r[1]:.4e} {r[2]:.4e} {r[3]:.4e}\n" for r in loading))
