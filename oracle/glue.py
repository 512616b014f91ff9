"""CPU restatement (numpy) of SGLDBench's MATLAB glue for the MGPCG solve.

TEST INFRASTRUCTURE ONLY.  This module is the oracle: the product
(``sgldbench_gb300``) never imports it.  It is used by ``tests/``, by
``__graft_entry__.smoke()`` as the checker and by ``bench.py``'s CPU baseline.

Each function restates one MATLAB function of the reference line by line, in
the reference's own data formats (1-based int32 index tables, column-major
arrays, node-major interleaved DOFs [ux uy uz] per node, n-by-3 arrays for the
transfer operators).  The citations are file:line within the SGLDBench
repository.  The element kernels (K*u, restriction, interpolation, stencil
assembly, unit compliance, density filter) come from ``oracle/sgld_oracle.c``
(a C restatement of the reference's MEX kernels) through ``oracle.kernels``;
the compiled reference kernels themselves (``oracle/_ref``) pin that
restatement in the tests.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp

from . import kernels as K

# ---------------------------------------------------------------------------
# constants and small helpers
# ---------------------------------------------------------------------------
GAUSS = 0.577350269189626  # src/FEA_GaussianIntegral.m:10-15 (15 digits, as written)

# Corner offsets (dy, dx, dz) of the 8 element nodes relative to element
# (iy, ix, iz): eNodMat = base + [0, ny+1, ny, -1, Nxy, Nxy+ny+1, Nxy+ny, Nxy-1]
# with base = nodenrs(iy, ix, iz) + 1  (src/FEA_VoxelBasedDiscretization.m:72-79)
CORNER_DYX = np.array([[1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 0],
                       [1, 0, 1], [1, 1, 1], [0, 1, 1], [0, 0, 1]], dtype=np.int64)


def mround(x):
    """MATLAB round(): half away from zero."""
    return math.floor(abs(x) + 0.5) * (1 if x >= 0 else -1)


def f_index(iy, ix, iz, ny, nx):
    """0-based column-major linear index of (iy, ix, iz) in a (ny, nx, *) array."""
    return iy + ny * (ix + nx * iz)


# ---------------------------------------------------------------------------
# element stiffness (src/FEA_VoxelBasedElementStiffnessMatrix.m:1-24 and helpers)
# ---------------------------------------------------------------------------
def gauss_points():
    """src/FEA_GaussianIntegral.m:10-16."""
    g = GAUSS
    s = np.array([-g, g, g, -g, -g, g, g, -g])
    t = np.array([-g, -g, g, g, -g, -g, g, g])
    p = np.array([-g, -g, -g, -g, g, g, g, g])
    w = np.ones(8)
    return s, t, p, w


def shape_functions(s, t, p):
    """src/FEA_ShapeFunction.m:10-23; rows = points, cols = nodes 1..8."""
    s, t, p = (np.atleast_1d(np.asarray(v, dtype=float)) for v in (s, t, p))
    return 0.125 * np.stack([(1 - s) * (1 - t) * (1 - p), (1 + s) * (1 - t) * (1 - p),
                             (1 + s) * (1 + t) * (1 - p), (1 - s) * (1 + t) * (1 - p),
                             (1 - s) * (1 - t) * (1 + p), (1 + s) * (1 - t) * (1 + p),
                             (1 + s) * (1 + t) * (1 + p), (1 - s) * (1 + t) * (1 + p)], axis=1)


def shape_derivatives(s, t, p):
    """src/FEA_DeShapeFunction.m:1-22: (3*npts) x 8, rows d/ds, d/dt, d/dp per point."""
    dNds = np.stack([-0.125 * (1 - t) * (1 - p), 0.125 * (1 - t) * (1 - p), 0.125 * (1 + t) * (1 - p),
                     -0.125 * (1 + t) * (1 - p), -0.125 * (1 - t) * (1 + p), 0.125 * (1 - t) * (1 + p),
                     0.125 * (1 + t) * (1 + p), -0.125 * (1 + t) * (1 + p)], axis=1)
    dNdt = np.stack([-0.125 * (1 - s) * (1 - p), -0.125 * (1 + s) * (1 - p), 0.125 * (1 + s) * (1 - p),
                     0.125 * (1 - s) * (1 - p), -0.125 * (1 - s) * (1 + p), -0.125 * (1 + s) * (1 + p),
                     0.125 * (1 + s) * (1 + p), 0.125 * (1 - s) * (1 + p)], axis=1)
    dNdp = np.stack([-0.125 * (1 - s) * (1 - t), -0.125 * (1 + s) * (1 - t), -0.125 * (1 + s) * (1 + t),
                     -0.125 * (1 - s) * (1 + t), 0.125 * (1 - s) * (1 - t), 0.125 * (1 + s) * (1 - t),
                     0.125 * (1 + s) * (1 + t), 0.125 * (1 - s) * (1 + t)], axis=1)
    n = len(s)
    d = np.zeros((3 * n, 8))
    d[0::3], d[1::3], d[2::3] = dNds, dNdt, dNdp
    return d


def strain_matrix(cell_size=1.0):
    """src/FEA_ElementStrainMatrix.m:1-94 with invJ = 2/h (FEA_VoxelBasedElementStiffnessMatrix.m:13).
    48 x 24; strain order xx, yy, zz, yz, zx, xy per Gauss point."""
    s, t, p, _ = gauss_points()
    der = (2.0 / cell_size) * shape_derivatives(s, t, p)
    B = np.zeros((48, 24))
    for i in range(8):
        ds, dt, dp = der[3 * i], der[3 * i + 1], der[3 * i + 2]
        for j in range(8):
            B[6 * i:6 * i + 6, 3 * j:3 * j + 3] = [[ds[j], 0, 0], [0, dt[j], 0], [0, 0, dp[j]],
                                                   [0, dp[j], dt[j]], [dp[j], 0, ds[j]],
                                                   [dt[j], ds[j], 0]]
    return B


def hooke(nu=0.3, E=1.0):
    """src/FEA_HookeLaw.m:4-13 (the reference always uses E = 1 here)."""
    c1 = (1 + nu) * (1 - 2 * nu)
    c2 = 2 * (1 + nu)
    S = np.zeros((6, 6))
    S[0, 0] = E * (1 - nu) / c1
    S[0, 1] = E * nu / c1
    S[0, 2] = S[0, 1]
    S[1, 0] = S[0, 1]
    S[1, 1] = S[0, 0]
    S[1, 2] = S[1, 0]
    S[2, 0] = S[0, 2]
    S[2, 1] = S[1, 2]
    S[2, 2] = S[1, 1]
    S[3, 3] = E / c2
    S[4, 4] = S[3, 3]
    S[5, 5] = S[4, 4]
    return S


def element_stiffness(nu=0.3, cell_size=1.0):
    """src/FEA_VoxelBasedElementStiffnessMatrix.m:10-23: Ke = B'(D.*w)B, 24 x 24."""
    B = strain_matrix(cell_size)
    D = np.kron(np.eye(8), hooke(nu))
    wgt = np.repeat(np.ones(8) * (cell_size ** 3 / 8.0), 6)
    return B.T @ (D * wgt[None, :]) @ B


def stress_extrapolation():
    """src/FEA_StressAnalysis.m:64-93: inv(sFM), 48 x 48 (GP stresses -> corner stresses)."""
    s, t, p, _ = gauss_points()
    N = shape_functions(s, t, p)
    sFM = np.zeros((48, 48))
    for g in range(8):
        for k in range(6):
            sFM[6 * g + k, k::6] = N[g, :]
    return np.linalg.inv(sFM)


# ---------------------------------------------------------------------------
# multigrid transfer tables (src/Solving_Operator4MultiGridRestrictionAndInterpolation.m)
# ---------------------------------------------------------------------------
def ri_inNODE(span):
    """(span+1)^3 x 8 trilinear weights.  Row order: the local (span+1)^3 fine node
    block reshaped column-major in (y, x, z) (Solving_BuildingMeshHierarchy.m:58-59);
    columns: coarse element nodes 1..8.  Local row a (y) maps to t = 1 - 2a/span
    (row index grows downward), b (x) to s = -1 + 2b/span, c (z) to p = -1 + 2c/span.
    Equal to the hard-coded tables in the reference (pinned by tests)."""
    n = span + 1
    rows = []
    for c in range(n):
        for b in range(n):
            for a in range(n):
                rows.append(shape_functions(-1 + 2 * b / span, 1 - 2 * a / span, -1 + 2 * c / span)[0])
    return np.array(rows)


def ri_inDOF(span):
    """3(span+1)^3 x 24: inNODE expanded to interleaved DOFs."""
    return np.kron(ri_inNODE(span), np.eye(3))


def sub_ele_nod_mat(span):
    """src/Solving_SubEleNodMat.m: for each child element (column-major order in the
    span^3 block) the 8 local node numbers (1-based) in the (span+1)^3 block."""
    n = span + 1
    out = []
    for cz in range(span):
        for cx in range(span):
            for cy in range(span):
                row = []
                for dy, dx, dz in CORNER_DYX:
                    row.append(1 + (cy + dy) + n * (cx + dx) + n * n * (cz + dz))
                out.append(row)
    return np.array(out, dtype=np.int32)


# ---------------------------------------------------------------------------
# mesh levels
# ---------------------------------------------------------------------------
@dataclass
class Level:
    resX: int
    resY: int
    resZ: int
    spanWidth: int = 1
    eleMapBack: np.ndarray = None       # int32, 1-based full-grid element indices of active elements
    eleMapForward: np.ndarray = None    # int32, full grid -> compact (1-based, 0 = void)
    numElements: int = 0
    eNodMat: np.ndarray = None          # int32 (numElements, 8), 1-based compact node numbers
    nodMapBack: np.ndarray = None       # int32, compact node -> full grid node (1-based)
    nodMapForward: np.ndarray = None
    numNodes: int = 0
    numDOFs: int = 0
    colors: list = field(default_factory=list)
    # coarse levels only
    elementUpwardMap: np.ndarray = None
    transferMat: np.ndarray = None      # int32 ((s+1)^3, numElements), ghost numbering
    transferMatCoeffi: np.ndarray = None
    solidNodeMapCoarser2Finer: np.ndarray = None
    intermediateNumNodes: int = 0
    multiGridOperatorRI: np.ndarray = None
    # finest only
    numNod2ElesVec: np.ndarray = None
    nodesOnBoundary: np.ndarray = None
    boundaryNodeCoords: np.ndarray = None
    # boundary conditions / solver data
    fixedDOFs: np.ndarray = None        # bool mask (numDOFs,)
    freeDOFs: np.ndarray = None
    diagK: np.ndarray = None
    eleModulus: np.ndarray = None
    Ke: np.ndarray = None
    Ks: np.ndarray = None


def coloring(eleMapForward, nx, ny, nz):
    """src/Solving_Coloring.m:2-12: 8 parity classes of elements."""
    v = eleMapForward.reshape((ny, nx, nz), order="F")
    out = []
    for (oy, ox, oz) in [(0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0), (0, 0, 1), (1, 0, 1), (0, 1, 1), (1, 1, 1)]:
        samp = v[oy::2, ox::2, oz::2].flatten(order="F")
        out.append(samp[samp > 0].astype(np.int32))
    return out


def _full_enodmat(nx, ny, nz):
    """eNodMat over all elements of an (ny, nx, nz) grid, 1-based full node numbers.
    src/FEA_VoxelBasedDiscretization.m:71-80."""
    iy, ix, iz = np.meshgrid(np.arange(ny), np.arange(nx), np.arange(nz), indexing="ij")
    iy, ix, iz = (a.flatten(order="F").astype(np.int64) for a in (iy, ix, iz))
    out = np.empty((iy.size, 8), dtype=np.int64)
    for k, (dy, dx, dz) in enumerate(CORNER_DYX):
        out[:, k] = 1 + f_index(iy + dy, ix + dx, iz + dz, ny + 1, nx + 1)
    return out


def _discretize_level(lv: Level):
    """Node numbering, eNodMat, nodMap* for the active elements of a level."""
    nx, ny, nz = lv.resX, lv.resY, lv.resZ
    full = _full_enodmat(nx, ny, nz)
    act = full[lv.eleMapBack.astype(np.int64) - 1]
    lv.nodMapBack = np.unique(act).astype(np.int32)
    lv.numNodes = int(lv.nodMapBack.size)
    lv.numDOFs = 3 * lv.numNodes
    lv.nodMapForward = np.zeros((nx + 1) * (ny + 1) * (nz + 1), dtype=np.int32)
    lv.nodMapForward[lv.nodMapBack - 1] = np.arange(1, lv.numNodes + 1, dtype=np.int32)
    lv.eNodMat = lv.nodMapForward[act - 1].astype(np.int32)
    return full


def voxel_discretization(vox, coarsest_control=50000, num_levels=None):
    """src/FEA_VoxelBasedDiscretization.m:26-106 (node coordinate caches excluded).
    vox: bool (ny, nx, nz).  Returns (level1, numLevels, padded vox, (nely, nelx, nelz)).
    num_levels, when given, replaces the level-count heuristic (:168-173), as
    setting the global numLevels_ would."""
    vox = np.asarray(vox, dtype=bool)
    nely, nelx, nelz = vox.shape
    num_voxels = int(vox.sum())
    if num_levels is not None:
        L = int(num_levels) - 1
    else:
        crc = min(coarsest_control, mround(mround(num_voxels / 8) / 8))
        if crc <= 0:
            raise ValueError("domain too small to build a mesh hierarchy")
        L = 0
        nv = num_voxels
        while nv >= crc:
            L += 1
            nv = mround(nv / 8)
    ax = int(math.ceil(nelx / 2 ** L) * 2 ** L)
    ay = int(math.ceil(nely / 2 ** L) * 2 ** L)
    az = int(math.ceil(nelz / 2 ** L) * 2 ** L)
    num_levels = L + 1
    pad = np.zeros((ay, ax, az), dtype=bool)
    pad[:nely, :nelx, :nelz] = vox
    lv = Level(resX=ax, resY=ay, resZ=az)
    flat = pad.flatten(order="F")
    lv.eleMapBack = (np.nonzero(flat)[0] + 1).astype(np.int32)
    lv.numElements = int(lv.eleMapBack.size)
    lv.eleMapForward = np.zeros(flat.size, dtype=np.int32)
    lv.eleMapForward[lv.eleMapBack - 1] = np.arange(1, lv.numElements + 1, dtype=np.int32)
    lv.colors = coloring(lv.eleMapForward, ax, ay, az)
    _discretize_level(lv)
    # boundary info (:92-106)
    cnt = np.zeros(lv.numNodes)
    np.add.at(cnt, lv.eNodMat.flatten() - 1, 1)
    lv.numNod2ElesVec = cnt
    lv.nodesOnBoundary = (np.nonzero(cnt < 8)[0] + 1).astype(np.int32)
    # node coordinates (:123-156): x = column, y = ny - row, z = page (cell size 1)
    full = lv.nodMapBack.astype(np.int64) - 1
    iy = full % (ay + 1)
    ix = (full // (ay + 1)) % (ax + 1)
    iz = full // ((ay + 1) * (ax + 1))
    coords = np.stack([ix, ay - iy, iz], axis=1).astype(np.float64)
    lv.boundaryNodeCoords = coords[lv.nodesOnBoundary - 1]
    return lv, num_levels, pad, (nely, nelx, nelz)


def build_hierarchy(level1: Level, num_levels: int, non_dyadic: int = 1):
    """src/Solving_BuildingMeshHierarchy.m:9-165.  Returns the list of levels and the
    (possibly reduced) level count."""
    levels = [level1]
    if non_dyadic == 1 and num_levels >= 4:
        num_levels -= 1
    else:
        non_dyadic = 0
    fine_full = _full_enodmat(level1.resX, level1.resY, level1.resZ)
    for ii in range(2, num_levels + 1):
        fl = levels[-1]
        s = 4 if (ii == 2 and non_dyadic == 1) else 2
        nx, ny, nz = fl.resX // s, fl.resY // s, fl.resZ // s
        lv = Level(resX=nx, resY=ny, resZ=nz, spanWidth=s)
        FY, FX = s * ny, s * nx
        # children of each coarse element, column-major within the s^3 block (:45-66)
        cy, cx, cz = np.meshgrid(np.arange(ny), np.arange(nx), np.arange(nz), indexing="ij")
        cy, cx, cz = (a.flatten(order="F").astype(np.int64) for a in (cy, cx, cz))
        oy, ox, oz = np.meshgrid(np.arange(s), np.arange(s), np.arange(s), indexing="ij")
        oy, ox, oz = (a.flatten(order="F") for a in (oy, ox, oz))
        child_full = f_index(s * cy[:, None] + oy[None, :], s * cx[:, None] + ox[None, :],
                             s * cz[:, None] + oz[None, :], FY, FX)  # 0-based
        eum_all = fl.eleMapForward[child_full]
        n1 = s + 1
        ny1, nx1, nz1 = np.meshgrid(np.arange(n1), np.arange(n1), np.arange(n1), indexing="ij")
        ny1, nx1, nz1 = (a.flatten(order="F") for a in (ny1, nx1, nz1))
        tm_full = 1 + f_index(s * cy[:, None] + ny1[None, :], s * cx[:, None] + nx1[None, :],
                              s * cz[:, None] + nz1[None, :], FY + 1, FX + 1)  # 1-based fine nodes
        unempty = np.nonzero(eum_all.sum(axis=1) > 0)[0]
        # ghost (intermediate) fine nodes: all nodes of all children of non-empty elements (:79-85)
        ghost = np.unique(fine_full[child_full[unempty].flatten()])
        lv.intermediateNumNodes = int(ghost.size)
        tmp = np.zeros((FX + 1) * (FY + 1) * (s * nz + 1), dtype=np.int32)
        tmp[ghost - 1] = np.arange(1, ghost.size + 1, dtype=np.int32)
        lv.transferMat = tmp[tm_full[unempty] - 1].T.copy(order="F")
        coeffi = np.zeros(lv.intermediateNumNodes)
        np.add.at(coeffi, lv.transferMat.flatten() - 1, 1.0)
        lv.transferMatCoeffi = coeffi
        # fine active nodes in ghost numbering (:95-100)
        fine_nodes = np.unique(fine_full[fl.eleMapBack.astype(np.int64) - 1])
        lv.solidNodeMapCoarser2Finer = (np.searchsorted(ghost, fine_nodes) + 1).astype(np.int32)
        # coarse elements (:103-109)
        lv.eleMapForward = np.zeros(nx * ny * nz, dtype=np.int32)
        lv.eleMapBack = (unempty + 1).astype(np.int32)
        lv.numElements = int(unempty.size)
        lv.eleMapForward[unempty] = np.arange(1, lv.numElements + 1, dtype=np.int32)
        lv.colors = coloring(lv.eleMapForward, nx, ny, nz)
        lv.elementUpwardMap = eum_all[unempty].astype(np.int32)
        # discretize (:112-133)
        fine_full = _discretize_level(lv)
        kk = ii if non_dyadic == 1 else ii - 1
        st = 2 ** kk
        R1 = level1
        fy = np.arange(0, R1.resY + 1, st)
        fx = np.arange(0, R1.resX + 1, st)
        fz = np.arange(0, R1.resZ + 1, st)
        gy, gx, gz = np.meshgrid(fy, fx, fz, indexing="ij")
        node_vol = 1 + f_index(gy.flatten(order="F"), gx.flatten(order="F"), gz.flatten(order="F"),
                               R1.resY + 1, R1.resX + 1)
        lv.nodMapBack = node_vol[lv.nodMapBack - 1].astype(np.int32)
        lv.multiGridOperatorRI = ri_inNODE(s)
        levels.append(lv)
    return levels, num_levels, non_dyadic


# ---------------------------------------------------------------------------
# boundary conditions
# ---------------------------------------------------------------------------
def cantilever3(level1: Level, nelx: int):
    """'Cuboid - Cantilever 3' (src/FEA_BuiltInBoundaryConditions4CuboidDesignDomain.m:34-44):
    fix the boundary nodes with minimal x; a total unit -z load spread over the boundary
    nodes with x == nelx and z == min z.  Returns (fixingCond, loadingCond) with node
    indices into nodesOnBoundary (1-based)."""
    c = level1.boundaryNodeCoords
    DL = c.min(axis=0)
    fixed = np.nonzero(c[:, 0] == DL[0])[0] + 1
    fixing = np.column_stack([fixed, np.ones((fixed.size, 3))])
    tmp = np.nonzero(c[:, 0] == nelx * 1.0)[0]
    loaded = tmp[c[tmp, 2] == DL[2]] + 1
    f = np.array([0.0, 0.0, -1.0]) / loaded.size
    loading = np.column_stack([loaded, np.tile(f, (loaded.size, 1))])
    return fixing, loading


def apply_boundary_condition(level1: Level, fixing, loading):
    """src/FEA_ApplyBoundaryCondition.m:9-42.  Returns F (numDOFs,) and sets the
    level's fixedDOFs/freeDOFs logical masks."""
    fixing = np.asarray(fixing, dtype=float)
    loading = np.asarray(loading, dtype=float)
    keep = ~np.isin(fixing[:, 0], loading[:, 0])
    fixing = fixing[keep]
    _, ui = np.unique(fixing[:, 0], return_index=True)
    fixing = fixing[np.sort(ui)]
    _, ul = np.unique(loading[:, 0], return_index=True)
    loading = loading[np.sort(ul)]
    F = np.zeros((level1.numNodes, 3))
    nodes = level1.nodesOnBoundary[loading[:, 0].astype(np.int64) - 1] - 1
    F[nodes, :] = loading[:, 1:4]
    fixed_nodes = level1.nodesOnBoundary[fixing[:, 0].astype(np.int64) - 1].astype(np.int64)
    dofs = (3 * fixed_nodes[:, None] - np.array([2, 1, 0])[None, :])
    state = fixing[:, 1:4] == 1
    fixed = np.zeros(level1.numDOFs, dtype=bool)
    fixed[dofs[state] - 1] = True
    level1.fixedDOFs = fixed
    level1.freeDOFs = ~fixed
    return F.reshape(-1)


# ---------------------------------------------------------------------------
# transfer operators (src/Solving_RestrictResidual.m, src/Solving_InterpolationDeviation.m)
# ---------------------------------------------------------------------------
def restrict(levels, r_fine, ii):
    """Solving_RestrictResidual(rFiner, ii); ii is the MATLAB (1-based) coarse level."""
    c, f = levels[ii - 1], levels[ii - 2]
    rf = np.asarray(r_fine, dtype=float).reshape(f.numNodes, 3)
    rc = K.restriction(rf, c.transferMat, c.multiGridOperatorRI, c.eNodMat, c.numNodes,
                       c.intermediateNumNodes, c.solidNodeMapCoarser2Finer, c.transferMatCoeffi,
                       c.colors)
    return rc.reshape(-1)


def interpolate(levels, x_coarse, ii):
    """Solving_InterpolationDeviation(xCoarser, ii)."""
    c, f = levels[ii - 1], levels[ii - 2]
    xc = np.asarray(x_coarse, dtype=float).reshape(c.numNodes, 3)
    xf = K.interpolation(xc, c.transferMat, c.multiGridOperatorRI, c.eNodMat, f.numNodes,
                         c.intermediateNumNodes, c.solidNodeMapCoarser2Finer, c.transferMatCoeffi,
                         c.colors)
    return xf.reshape(-1)


# ---------------------------------------------------------------------------
# solver setup
# ---------------------------------------------------------------------------
@dataclass
class Model:
    levels: list
    numLevels: int
    nonDyadic: int
    Ke: np.ndarray
    F: np.ndarray = None
    U: np.ndarray = None
    omega: float = 0.35
    chol: object = None      # (L, perm) for the coarsest level's free DOFs
    nely: int = 0
    nelx: int = 0
    nelz: int = 0


def setup_voxel_based(levels, num_levels, Ke):
    """src/FEA_SetupVoxelBased.m:6-27: coarse fixed masks by restricting the fine
    fixed indicator (fixed iff the restricted value is nonzero)."""
    levels[0].Ke = Ke
    ind = levels[0].fixedDOFs.astype(float)
    for ii in range(2, num_levels + 1):
        fc = restrict(levels, ind, ii)
        levels[ii - 1].freeDOFs = fc == 0
        levels[ii - 1].fixedDOFs = ~levels[ii - 1].freeDOFs
        ind = fc
    levels[0].Ks = Ke


def simp_modulus(x, E0=1.0, Emin=1e-6, p=3.0):
    """src/TopOpti_MaterialInterpolationSIMP.m:5."""
    return Emin + np.asarray(x, dtype=float).reshape(-1) ** p * (E0 - Emin)


_REORDER = np.array([1, 9, 17, 2, 10, 18, 3, 11, 19, 4, 12, 20, 5, 13, 21, 6, 14, 22, 7, 15, 23, 8, 16, 24]) - 1


def local_mapping(span):
    """Solving_AssembleFEAstencil.m:8-20: linear index into the 3(s+1)^3 square
    tmpK for every (Ke entry, child) pair; int32, 1-based, length 576*s^3."""
    en = sub_ele_nod_mat(span).astype(np.int64)
    edof = np.concatenate([3 * en - 2, 3 * en - 1, 3 * en], axis=1)[:, _REORDER]  # (s^3, 24)
    rows = np.tile(np.arange(24), 24)          # find(ones(24)) column-major
    cols = np.repeat(np.arange(24), 24)
    iK = edof[:, rows].T                         # (576, s^3)
    jK = edof[:, cols].T
    nd = 3 * (span + 1) ** 3
    return (iK.flatten(order="F") + (jK.flatten(order="F") - 1) * nd).astype(np.int32)


def assemble_stencil(model: Model):
    """src/Solving_AssembleFEAstencil.m:7-135: Galerkin per-element stiffness on the
    coarse levels (kept on each level as Ks, 24x24xM), Jacobi diagonals on levels
    1..L-1 and the coarsest-level Cholesky factor (free DOFs only)."""
    levels, L = model.levels, model.numLevels
    Ks = None
    for ii in range(2, L + 1):
        lv = levels[ii - 1]
        s = lv.spanWidth
        P = ri_inDOF(s)
        lm = local_mapping(s)
        npn = (s + 1) ** 3
        if ii == 2:
            Ks = K.assemble_from_finest(model.Ke, levels[0].eleModulus, lv.elementUpwardMap, P, lm, npn)
        else:
            Ks = K.assemble_from_nonfinest(Ks, lv.elementUpwardMap, P, lm, npn)
        lv.Ks = Ks
        if ii < L:
            d = Ks[np.arange(24), np.arange(24), :]      # (24, M): diagonal of every Ks page
            dg = np.zeros((lv.numNodes, 3))
            for c in range(3):
                np.add.at(dg[:, c], lv.eNodMat.T.flatten(order="F") - 1, d[c::3, :].flatten(order="F"))
            lv.diagK = dg.reshape(-1)
    # finest diagonal (:103-121)
    l1 = levels[0]
    dke = np.diag(model.Ke)
    dg = np.zeros((l1.numNodes, 3))
    Em = l1.eleModulus.reshape(-1)
    for c in range(3):
        vals = (dke[c::3][:, None] * Em[None, :])  # (8, numEl)
        np.add.at(dg[:, c], l1.eNodMat.T.flatten(order="F") - 1, vals.flatten(order="F"))
    l1.diagK = dg.reshape(-1)
    # coarsest direct solver (:124-135)
    lc = levels[L - 1]
    if L == 1:
        Ks = np.repeat(model.Ke[:, :, None], 1, axis=2) * l1.eleModulus[None, None, :]
    Kc = coarse_matrix(lc, Ks)
    free = lc.freeDOFs
    Kf = Kc[np.ix_(free, free)]
    model.chol = sla.cho_factor(Kf, lower=True)
    return model


def coarse_matrix(lc: Level, Ks):
    """Assemble the coarsest-level stiffness matrix (dense) from per-element Ks."""
    edof = np.concatenate([3 * lc.eNodMat - 2, 3 * lc.eNodMat - 1, 3 * lc.eNodMat], axis=1)[:, _REORDER] - 1
    n = lc.numDOFs
    rows = np.repeat(edof[:, :, None], 24, axis=2)   # (M, 24 row, 24 col)
    cols = np.repeat(edof[:, None, :], 24, axis=1)
    vals = np.transpose(Ks, (2, 0, 1))                # Ks(row, col, e)
    Kc = sp.coo_matrix((vals.flatten(), (rows.flatten(), cols.flatten())), shape=(n, n)).toarray()
    return Kc


# ---------------------------------------------------------------------------
# operators used by PCG
# ---------------------------------------------------------------------------
def kbyu(model: Model, u):
    """src/Solving_KbyU_MatrixFree.m:1-41 (MEX branch) incl. y(fixedDOFs) = 0."""
    l1 = model.levels[0]
    y = K.kbyu(np.asarray(u, dtype=float), l1.eNodMat, model.Ke, l1.eleModulus, l1.colors)
    y[l1.fixedDOFs] = 0.0
    return y


def vcycle(model: Model, r):
    """src/Solving_Vcycle.m:12-50 (additive multilevel Jacobi + coarsest Cholesky)."""
    levels, L, w = model.levels, model.numLevels, model.omega
    r = np.asarray(r, dtype=float)
    xs = [None] * (L + 1)
    rs = [None] * (L + 1)
    rtilde = None
    for ii in range(2, L + 1):
        if ii == 2:
            rtilde = w * r / levels[0].diagK
            rs[ii] = restrict(levels, r, ii)
        else:
            xs[ii - 1] = w * rs[ii - 1] / levels[ii - 2].diagK
            rs[ii] = restrict(levels, rs[ii - 1], ii)
    lc = levels[L - 1]
    xc = np.zeros(lc.numDOFs)
    xc[lc.freeDOFs] = sla.cho_solve(model.chol, rs[L][lc.freeDOFs])
    xs[L] = xc
    for ii in range(L, 1, -1):
        if ii == 2:
            rtilde = rtilde + interpolate(levels, xs[ii], ii)
            rtilde = rtilde + w * r / levels[0].diagK
        else:
            xs[ii - 1] = xs[ii - 1] + interpolate(levels, xs[ii], ii)
            xs[ii - 1] = xs[ii - 1] + w * rs[ii - 1] / levels[ii - 2].diagK
    rtilde[levels[0].fixedDOFs] = 0.0
    return rtilde


def pcg(AtX, PtV, b, tol, maxIT, x0=None, history=None):
    """src/Solving_PreconditionedConjugateGradientSolver.m:7-36.  Returns (y, its)."""
    b = np.asarray(b, dtype=float)
    normB = np.linalg.norm(b)
    y = np.zeros_like(b) if x0 is None else np.array(x0, dtype=float)
    r = b - AtX(y)
    z = PtV(r)
    p = z.copy()
    x1 = z @ r
    its = 0
    for its in range(1, maxIT + 1):
        z = AtX(p)
        lam = x1 / (p @ z)
        y = y + lam * p
        r = r - lam * z
        res = np.linalg.norm(r) / normB
        if history is not None:
            history.append(res)
        if res < tol:
            break
        z = PtV(r)
        x2 = z @ r
        p = z + x2 / x1 * p
        x1 = x2
    return y, its


def unit_compliance(model: Model, U):
    """src/TopOpti_ComputeUnitCompliance.m:1-21 -> per-element u_e' Ke u_e."""
    l1 = model.levels[0]
    return K.unit_compliance(np.asarray(U, dtype=float), l1.eNodMat, model.Ke)


def compliance(model: Model, U):
    """src/FEA_ComputeComplianceVoxel.m:20-22: c = sum(E .* ce)."""
    return float(np.sum(model.levels[0].eleModulus * unit_compliance(model, U)))


def stress_analysis(model: Model, U, nu=0.3, cell_size=1.0):
    """src/FEA_StressAnalysis.m:17-60: nodal Cartesian stress (numNodes x 6, averaged
    over the elements sharing each node) and nodal von Mises stress."""
    l1 = model.levels[0]
    B = strain_matrix(cell_size)
    D = np.kron(np.eye(8), hooke(nu))
    OTP = stress_extrapolation()
    M = OTP @ (D @ B)                                   # 48 x 24
    Un = np.asarray(U, dtype=float).reshape(l1.numNodes, 3)
    ue = Un[l1.eNodMat - 1].reshape(l1.numElements, 24)  # interleaved per corner
    sig = (ue @ M.T) * l1.eleModulus[:, None]           # (numEl, 48): corner-major, 6 comps
    field_ = np.zeros((l1.numNodes, 6))
    for k in range(8):
        np.add.at(field_, l1.eNodMat[:, k] - 1, sig[:, 6 * k:6 * k + 6])
    field_ = field_ / l1.numNod2ElesVec[:, None]
    return field_, von_mises(field_)


def von_mises(s):
    """src/FEA_ComputeVonMisesStress.m:2-6 (order xx, yy, zz, yz, zx, xy)."""
    return np.sqrt(0.5 * ((s[:, 0] - s[:, 1]) ** 2 + (s[:, 1] - s[:, 2]) ** 2 + (s[:, 2] - s[:, 0]) ** 2)
                   + 3 * (s[:, 5] ** 2 + s[:, 3] ** 2 + s[:, 4] ** 2))


def per_element_von_mises(model: Model, cartesian):
    """src/FEA_ComputePerElementVonMisesStress.m:10-19, including the final .^(1/2)."""
    l1 = model.levels[0]
    cent = cartesian[l1.eNodMat - 1].mean(axis=1) if False else \
        np.einsum("k,ekc->ec", shape_functions(0.0, 0.0, 0.0)[0], cartesian[l1.eNodMat - 1])
    return von_mises(cent) ** 0.5


# ---------------------------------------------------------------------------
# end-to-end helpers
# ---------------------------------------------------------------------------
def build_model(vox, coarsest_control=50000, non_dyadic=1, nu=0.3, omega=0.35,
                bc="cantilever3", fixing=None, loading=None, num_levels=None):
    """Discretize, apply boundary conditions and set up the hierarchy, as
    QuickAccess/QuickAccess_Mtd0_StressAnalysis.m:24-25 does."""
    l1, nlev, pad, (nely, nelx, nelz) = voxel_discretization(vox, coarsest_control, num_levels)
    levels, nlev, nd = build_hierarchy(l1, nlev, non_dyadic)
    if bc == "cantilever3":
        fixing, loading = cantilever3(l1, nelx)
    F = apply_boundary_condition(l1, fixing, loading)
    Ke = element_stiffness(nu)
    setup_voxel_based(levels, nlev, Ke)
    m = Model(levels=levels, numLevels=nlev, nonDyadic=nd, Ke=Ke, F=F, omega=omega,
              nely=nely, nelx=nelx, nelz=nelz)
    m.U = np.zeros(l1.numDOFs)
    return m


def pde_element_matrix(rhat):
    """src/TopOpti_BuildPDEfilter_matrixFree.m:9-20: KePDE = r^2 dN'dN + N'diag(w detJ)N,
    unit cell (detJ = 1/8, w = 1), r = rHatMin / 2 / sqrt(3); 8 x 8, reference node order."""
    s, t, p, w = gauss_points()
    N = shape_functions(s, t, p)
    dN = shape_derivatives(s, t, p)
    wgt = w * (1.0 / 8.0)
    r = rhat / 2.0 / np.sqrt(3.0)
    return r * r * (dN.T @ dN) + N.T @ np.diag(wgt) @ N


def pde_kbyu(l1, Ke8, u):
    """y = sum_e Ke8 u_e over eNodMat (the product of Solving_KbyU_MatrixFree8x8_mex.cpp)."""
    ue = np.asarray(u, float)[l1.eNodMat - 1]
    return np.bincount((l1.eNodMat - 1).ravel(), weights=(ue @ Ke8).ravel(), minlength=l1.numNodes)


def pde_filter(model, x, rhat, tol=1e-6, maxIT=500):
    """src/TopOpti_PDEFiltering_matrixFree.m:1-36: element -> node (x/8 to each corner),
    Jacobi-preconditioned PCG on KePDE, node -> element (mean of the 8 corners).
    Returns (filtered field, PCG iterations)."""
    l1 = model.levels[0]
    Ke8 = pde_element_matrix(rhat)
    vals = np.asarray(x, float) * (1.0 / 8.0)
    src = np.zeros(l1.numNodes)
    for jj in range(8):
        src += np.bincount(l1.eNodMat[:, jj] - 1, weights=vals, minlength=l1.numNodes)
    diag = np.zeros(l1.numNodes)
    for jj in range(8):
        diag += np.bincount(l1.eNodMat[:, jj] - 1, weights=np.full(l1.numElements, Ke8[jj, jj]),
                            minlength=l1.numNodes)
    dinv = 1.0 / diag
    t, its = pcg(lambda v: pde_kbyu(l1, Ke8, v), lambda r: dinv * r, src, tol, maxIT)
    return t[l1.eNodMat - 1].sum(axis=1) * (1.0 / 8.0), its


def principal_stress(cartesian):
    """src/FEA_ComputePrincipalStress.m:1-8 for every row of a (n, 6) field
    [xx yy zz yz zx xy]: rows [l1 v1 l2 v2 l3 v3], eigenvalues ascending (as eig
    returns them for a symmetric matrix), each eigenvector signed so that its
    largest-magnitude entry is positive (eig leaves the sign open)."""
    s = np.asarray(cartesian, float)
    A = np.empty((s.shape[0], 3, 3))
    A[:, 0, 0], A[:, 1, 1], A[:, 2, 2] = s[:, 0], s[:, 1], s[:, 2]
    A[:, 0, 1] = A[:, 1, 0] = s[:, 5]
    A[:, 0, 2] = A[:, 2, 0] = s[:, 4]
    A[:, 1, 2] = A[:, 2, 1] = s[:, 3]
    w, V = np.linalg.eigh(A)
    big = np.abs(V).argmax(axis=1)                       # (n, 3): row of the largest entry per vector
    sign = np.sign(np.take_along_axis(V, big[:, None, :], axis=1))[:, 0, :]
    sign[sign == 0] = 1.0
    V = V * sign[:, None, :]
    out = np.empty((s.shape[0], 12))
    for k in range(3):
        out[:, 4 * k] = w[:, k]
        out[:, 4 * k + 1:4 * k + 4] = V[:, :, k]
    return out


def dominant_directions(model, cartesian):
    """src/Common_ExtractDominantDirectionsFromPrincipalStressDirections.m:9-38:
    per element, the centroid stress (shape functions at the centroid = 1/8
    each) and the eigenvector of the principal stress of largest magnitude."""
    l1 = model.levels[0]
    cent = cartesian[l1.eNodMat - 1].mean(axis=1)
    ps = principal_stress(cent)
    lam = np.abs(ps[:, [0, 4, 8]])
    k = lam.argmax(axis=1)
    return np.stack([ps[np.arange(len(k)), 4 * k + 1 + i] for i in range(3)], axis=1)


def build_model_fixed(vox, fixed, coarsest_control=50000, non_dyadic=1, nu=0.3, omega=0.35, num_levels=None):
    """build_model with a caller-given level-1 fixed-DOF mask instead of a
    named boundary condition (FEA_ApplyBoundaryCondition.m:37-41 sets the same
    mask from a fixing table); loads are set per solve through model.F."""
    l1, nlev, pad, (nely, nelx, nelz) = voxel_discretization(vox, coarsest_control, num_levels)
    levels, nlev, nd = build_hierarchy(l1, nlev, non_dyadic)
    l1.fixedDOFs = np.asarray(fixed, dtype=bool).reshape(-1).copy()
    l1.freeDOFs = ~l1.fixedDOFs
    Ke = element_stiffness(nu)
    setup_voxel_based(levels, nlev, Ke)
    m = Model(levels=levels, numLevels=nlev, nonDyadic=nd, Ke=Ke, F=np.zeros(l1.numDOFs), omega=omega,
              nely=nely, nelx=nelx, nelz=nelz)
    m.U = np.zeros(l1.numDOFs)
    return m


def set_modulus(model: Model, E):
    model.levels[0].eleModulus = np.asarray(E, dtype=float).reshape(-1)


def solve(model: Model, tol=1e-6, maxIT=500, x0=None, history=None):
    return pcg(lambda u: kbyu(model, u), lambda r: vcycle(model, r), model.F, tol, maxIT,
               x0=x0, history=history)


# ---------------------------------------------------------------------------
# SIMP loop (src/TopOpti_GlobalVolumeConstraint_Tmp.m:26-120, ft = 2 branch)
# ---------------------------------------------------------------------------
@dataclass
class TopOptOptions:
    volfrac: float = 0.3          # V_
    rmin: float = 1.5             # rMin_
    move: float = 0.1             # move_ (Data_GlobalVariables.m:65)
    n_loop: int = 60              # nLoop_
    min_change: float = 1.0e-4    # minChange_ (Data_GlobalVariables.m:68)
    max_sharpness: float = 0.05   # maxSharpness_ (Data_GlobalVariables.m:67)
    penalty: float = 3.0          # SIMPpenalty_ / penalty_
    E0: float = 1.0               # modulus_
    Emin: float = 1.0e-9          # modulusMin_
    tol: float = 1.0e-6           # tol_
    optimizer: str = "OC"         # optimizer_: "OC" (the _Tmp loop's bisection) or "MMA"
    passive: np.ndarray = None    # passiveElements_ (compact 0-based), kept solid
    maxit: int = 500              # maxIT_


def topopt_global_volume(model: Model, opt: TopOptOptions, history=None):
    """TopOpti_GlobalVolumeConstraint_Tmp.m:26-120 with ft = 2 (density filter on
    sensitivities and densities), OC bisection on the linearised volume
    constraint, warm-started MGPCG (Solving_CG_GMGS.m:7).  Returns xPhys and a
    list of per-iteration records (compliance, volume, sharpness, change, its)."""
    l1 = model.levels[0]
    n = l1.numElements
    emf, (rx, ry, rz) = l1.eleMapForward, (l1.resX, l1.resY, l1.resZ)
    Hs = K.density_filter(None, opt.rmin, emf, rx, ry, rz)                    # :35
    x = np.full(n, opt.volfrac)                                               # TopOpti_CallTopOpti.m:34
    xPhys = x.copy()
    U = np.zeros(l1.numDOFs)
    loop, change, sharp = 0, 1.0, 1.0
    hist = [] if history is None else history
    while loop < opt.n_loop and change > opt.min_change and sharp > opt.max_sharpness:   # :47
        loop += 1
        E = simp_modulus(xPhys, opt.E0, opt.Emin, opt.penalty)               # :52
        set_modulus(model, E)
        assemble_stencil(model)                                              # :54
        U, its = pcg(lambda u: kbyu(model, u), lambda r: vcycle(model, r), model.F, opt.tol, opt.maxit, x0=U)
        ce = unit_compliance(model, U)                                       # :59
        c = float(E @ ce)                                                    # :63 (complianceSolid_ = 1)
        vol = float(xPhys.sum() / n)                                         # :65
        dc = -(opt.penalty * (opt.E0 - opt.Emin) * xPhys ** (opt.penalty - 1)) * ce   # :66, TopOpti_DeMaterialInterpolation.m:5
        dv = np.ones(n)
        dc = K.density_filter(dc / Hs, opt.rmin, emf, rx, ry, rz)            # :76
        dv = K.density_filter(dv / Hs, opt.rmin, emf, rx, ry, rz)            # :77
        g = float(xPhys.mean() - opt.volfrac)                                # :83
        pas = np.zeros(n, bool) if opt.passive is None else np.isin(np.arange(n), opt.passive)
        if opt.optimizer == "MMA":
            # TopOpti_GlobalVolumeConstraint.m:139-156 (one volume constraint)
            from oracle import mma
            var = np.nonzero(~pas)[0]
            xval = x[var]
            xmin, xmax = np.maximum(0.0, xval - opt.move), np.minimum(1.0, xval + opt.move)
            fval = xPhys.sum() / (n * opt.volfrac) - 1.0
            xmma, _, _ = mma.mma_update(1, var.size, xval, xmin, xmax, xval, xval, dc[var], fval,
                                        dv[var] / (n * opt.volfrac))
            change = float(np.abs(xmma - xval).max())
            xnew = np.ones(n)
            xnew[var] = xmma
        else:
            lo, hi = 0.0, 1e9                                                # :84
            while (hi - lo) / (lo + hi) > 1e-6:                              # :85-90
                lmid = 0.5 * (hi + lo)
                xnew = np.maximum(0.0, np.maximum(x - opt.move, np.minimum(1.0, np.minimum(
                    x + opt.move, x * np.sqrt(-dc / dv / lmid)))))
                xnew[pas] = 1.0                                              # GlobalVolumeConstraint.m:162
                gt = g + float(np.sum(dv * (xnew - x)))
                if gt > 0:
                    lo = lmid
                else:
                    hi = lmid
            change = float(np.abs(xnew - x).max())                          # :91
        x = xnew
        xPhys = K.density_filter(xnew, opt.rmin, emf, rx, ry, rz) / Hs       # :99
        xPhys[pas] = 1.0                                                     # GlobalVolumeConstraint.m:179
        sharp = float(4.0 * np.sum(xPhys * (1.0 - xPhys)) / n)               # :102
        hist.append({"loop": loop, "c": c, "vol": vol, "sharp": sharp, "change": change, "g": g, "its": its})
    return xPhys, hist


# ---------------------------------------------------------------------------
# Local-volume-constrained loop (porous infill): src/TopOpti_LocalVolumeConstraint.m
# ---------------------------------------------------------------------------
@dataclass
class LocalOptions:
    constraint: str = "local"      # "local" (TopOpti_LocalVolumeConstraint.m) or "volume"
                                   # (TopOpti_GlobalVolumeConstraint.m, optimizer_ = 'MMA')
    volfrac: float = 0.3           # V_ ("volume")
    rmin: float = 1.5              # rMin_ (density filter)
    rhat: float = 8.0              # rHatMin_ (Data_GlobalVariables.m:62), PDE filter of the local volume
    alpha: float = 0.5             # alphaMin_ = alphaMax_ (Data_GlobalVariables.m:63; Initialize4GradedPorosity)
    pnorm: float = 16.0            # p_ (Data_GlobalVariables.m:75)
    move: float = 0.1              # move_
    n_loop: int = 300              # nLoop_
    min_change: float = 1.0e-4     # minChange_
    max_sharpness: float = 0.05    # maxSharpness_
    simp_penalty: float = 3.0      # SIMPpenalty_ (TopOpti_MaterialInterpolationSIMP.m)
    penalty: float = 3.0           # penalty_ (TopOpti_DeMaterialInterpolation.m), continued
    penalty_increment: float = 0.2  # penaltyIncrement_ (Data_GlobalVariables.m:73)
    penalty_interval: int = 30     # penaltyUpdateIterations_ (:74)
    beta: float = 1.0              # beta_ (:76)
    eta: float = 0.5               # eta_ (:77)
    beta_max: float = 128.0        # pMax_ (:59)
    beta_interval: int = 40        # TopOpti_LocalVolumeConstraint.m:246
    E0: float = 1.0                # modulus_
    Emin: float = 1.0e-6           # modulusMin_
    tol: float = 1.0e-6            # tol_ (elasticity and PDE-filter PCG)
    maxit: int = 500               # maxIT_
    passive: np.ndarray = None     # passiveElements_ (compact 0-based)


def heaviside(xt, beta, eta):
    """TopOpti_DualizeDesignVariable.m:4."""
    return (np.tanh(beta * eta) + np.tanh(beta * (xt - eta))) / (np.tanh(beta * eta) + np.tanh(beta * (1 - eta)))


def heaviside_derivative(xt, beta, eta):
    """TopOpti_DeDualizeDesignVariable.m:4."""
    t = np.tanh(beta * (xt - eta))
    return beta * (1 - t * t) / (np.tanh(beta * eta) + np.tanh(beta * (1 - eta)))


def topopt_local_volume(model: Model, opt: LocalOptions, history=None):
    """TopOpti_LocalVolumeConstraint.m:33-269 (MEX branch, PDE filter matrix-free)
    or, with opt.constraint == "volume", TopOpti_GlobalVolumeConstraint.m:50-228
    with MMA (volume constraint sum(xPhys) <= V n, x starting at V, beta also
    doubled once change <= 1e-3):
    solid-domain compliance, then per iteration SIMP E, warm-started MGPCG,
    normalised compliance and its sensitivity, the p-norm of the PDE-filtered
    local volume against alpha and its sensitivity, density-filter chain rule
    through the Heaviside projection, one MMA update (m = 1, passive elements
    excluded), filter + projection of the new design, beta and penalty
    continuation.  Returns xPhys and per-iteration records."""
    from oracle import mma

    l1 = model.levels[0]
    n = l1.numElements
    emf, (rx, ry, rz) = l1.eleMapForward, (l1.resX, l1.resY, l1.resZ)
    Hs = K.density_filter(None, opt.rmin, emf, rx, ry, rz)                       # :37
    pas = np.zeros(n, bool) if opt.passive is None else np.isin(np.arange(n), opt.passive)
    act = np.nonzero(~pas)[0]                                                    # :63
    vol_max = np.full(n, opt.alpha)                                              # :290-301
    vol_max[pas] = 1.0
    local = opt.constraint == "local"
    x = np.full(n, opt.alpha if local else opt.volfrac)                          # TopOpti_CallTopOpti.m:34-45
    x[pas] = 1.0
    beta, penalty = opt.beta, opt.penalty
    xTilde = x.copy()                                                            # :69
    xPhys = heaviside(xTilde, beta, opt.eta)                                     # :70
    # :79-86 compliance of the fully solid domain
    E = np.full(n, opt.E0)
    set_modulus(model, E)
    assemble_stencil(model)
    U, _ = pcg(lambda u: kbyu(model, u), lambda r: vcycle(model, r), model.F, opt.tol, opt.maxit,
               x0=np.zeros(l1.numDOFs))
    c_solid = float(E @ unit_compliance(model, U))
    loopbeta, loop, change, sharp = 0, 0, 1.0, 1.0
    hist = [] if history is None else history
    while loop < opt.n_loop and change > opt.min_change and sharp > opt.max_sharpness:   # :116
        loopbeta += 1
        loop += 1
        E = simp_modulus(xPhys, opt.E0, opt.Emin, opt.simp_penalty)             # :121
        set_modulus(model, E)
        assemble_stencil(model)                                                  # :123
        U, its = pcg(lambda u: kbyu(model, u), lambda r: vcycle(model, r), model.F, opt.tol, opt.maxit, x0=U)
        ce_norm = unit_compliance(model, U) / c_solid                            # :128, :132
        c = float(E @ ce_norm) * c_solid                                         # :133-134
        vol = float(xPhys.sum() / n)                                             # :135
        dc = -(penalty * (opt.E0 - opt.Emin) * xPhys ** (penalty - 1)) * ce_norm  # :136
        dx = heaviside_derivative(xTilde, beta, opt.eta)                         # :151
        dc = K.density_filter(dc * dx / Hs, opt.rmin, emf, rx, ry, rz)           # :153
        if local:
            xh, _ = pde_filter(model, xPhys, opt.rhat, opt.tol, opt.maxit)       # :142
            s = float(np.sum(xh ** opt.pnorm / vol_max ** opt.pnorm) / n)
            dfdx_pde = s ** (1.0 / opt.pnorm - 1.0) * (xh ** (opt.pnorm - 1) / vol_max ** opt.pnorm) / n   # :146
            dfdx, _ = pde_filter(model, dfdx_pde, opt.rhat, opt.tol, opt.maxit)  # :162
            dfdx = K.density_filter(dfdx * dx / Hs, opt.rmin, emf, rx, ry, rz)   # :169
            fval = s ** (1.0 / opt.pnorm) - 1.0                                  # :179
        else:   # TopOpti_GlobalVolumeConstraint.m:119, :128-129, :139-141
            dfdx = K.density_filter(dx / Hs, opt.rmin, emf, rx, ry, rz) / (n * opt.volfrac)
            fval = float(xPhys.sum()) / (n * opt.volfrac) - 1.0
        xval = x[act]
        xmin, xmax = np.maximum(0.0, xval - opt.move), np.minimum(1.0, xval + opt.move)   # :184-185
        xmma, _, _ = mma.mma_update(1, act.size, xval, xmin, xmax, xval, xval, dc[act], fval, dfdx[act])
        change = float(np.abs(xmma - xval).max())                                # :191
        x = np.ones(n)
        x[act] = xmma                                                            # :192
        xTilde = K.density_filter(x, opt.rmin, emf, rx, ry, rz) / Hs             # :197
        xPhys = heaviside(xTilde, beta, opt.eta)                                 # :201
        xPhys[pas] = 1.0                                                         # :204
        sharp = float(4.0 * np.sum(xPhys * (1.0 - xPhys)) / n)                   # :205
        hist.append({"loop": loop, "c": c, "vol": vol, "sharp": sharp, "change": change, "fval": fval,
                     "its": its, "beta": beta, "penalty": penalty})
        if beta < opt.beta_max and (loopbeta >= opt.beta_interval or (not local and change <= 1e-3)):   # :246 / Global :212
            beta, loopbeta, change, sharp = 2 * beta, 0, 1.0, 1.0
        if opt.penalty_interval > 0 and loop % opt.penalty_interval == 0:        # :256-261
            penalty = min(penalty + opt.penalty_increment, 3.0)
    return xPhys, hist
