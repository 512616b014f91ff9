"""Python host interface over the C ABI, mirroring SGLDBench's solve path.

``VoxelSolver`` owns one device context (``sgld_ctx``).  Its methods carry
the reference's function names and argument meaning:

==========================================  =====================================================
reference (SGLDBench)                       here
==========================================  =====================================================
FEA_VoxelBasedDiscretization.m + Solving_   ``VoxelSolver(voxels, ...)``
BuildingMeshHierarchy.m
FEA_ApplyBoundaryCondition.m (fixedDOFs)    ``set_fixed_dofs(mask)``
  + FEA_SetupVoxelBased.m (coarse masks)
TopOpti_MaterialInterpolationSIMP.m         ``set_modulus(E)``  (``simp_modulus`` computes E)
Solving_AssembleFEAstencil.m                ``Solving_AssembleFEAstencil()``
Solving_KbyU_MatrixFree.m                   ``Solving_KbyU_MatrixFree(u)``
Solving_RestrictResidual.m                  ``Solving_RestrictResidual(r, ii)``
Solving_InterpolationDeviation.m            ``Solving_InterpolationDeviation(x, ii)``
Solving_Vcycle.m                            ``Solving_Vcycle(r)``
Solving_PreconditionedConjugate...m         ``Solving_PreconditionedConjugateGradientSolver(...)``
Solving_CG_GMGS.m                           ``Solving_CG_GMGS(F, U0)``
TopOpti_ComputeUnitCompliance.m             ``TopOpti_ComputeUnitCompliance(U)``
FEA_StressAnalysis.m /                      ``FEA_StressAnalysis(U)``
FEA_ComputePerElementVonMisesStress.m
==========================================  =====================================================

Vectors use the reference's compact layout: DOF vectors of length
3 * numNodes (node-major [ux uy uz]), element vectors of length numElements.
All computation happens in the CUDA library; errors raise ``SgldError``.
"""
from __future__ import annotations

import ctypes as C
import math
import warnings

import numpy as np

from . import _lib as L


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def reference_num_levels(num_voxels: int, coarsest_resolution_control: int = 50000) -> int:
    """Level count of FEA_VoxelBasedDiscretization.m:168-177 (before nonDyadic)."""
    return int(L.load().sgld_reference_num_levels(int(num_voxels), int(coarsest_resolution_control)))


def pad_voxels(voxels: np.ndarray, num_levels: int) -> np.ndarray:
    """Pads the (ny, nx, nz) grid to multiples of 2^(num_levels-1) with void,
    as FEA_VoxelBasedDiscretization.m:174-186 does."""
    m = 2 ** (num_levels - 1)
    ny, nx, nz = voxels.shape
    out = np.zeros((int(math.ceil(ny / m) * m), int(math.ceil(nx / m) * m), int(math.ceil(nz / m) * m)), bool)
    out[:ny, :nx, :nz] = voxels
    return out


_PRECISIONS = {"fp64": L.SGLD_PREC_FP64, "mixed": L.SGLD_PREC_MIXED, "mixed_df": L.SGLD_PREC_MIXED_DF}


def _precision(name: str) -> int:
    """'fp64' (the reference's form), 'mixed' or 'mixed_df' -> SGLD_PREC_*."""
    if name not in _PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(_PRECISIONS)}, not {name!r}")
    return _PRECISIONS[name]


def _info_dict(info) -> dict:
    return {"its": info.iterations, "converged": bool(info.converged), "relres": info.relres,
            "true_relres": info.true_relres, "inner_its": info.inner_iterations, "seconds": info.seconds,
            "kbyu_seconds": info.kbyu_seconds, "kbyu_launches": info.kbyu_launches,
            "precond_seconds": info.precond_seconds, "fallback": bool(info.fallback),
            "replacements": info.replacements}


def kernel_launches() -> int:
    """Kernels the CUDA library has launched so far from the calling thread."""
    return int(L.load().sgld_kernel_launches())


def simp_modulus(x, E0: float = 1.0, Emin: float = 1e-6, p: float = 3.0) -> np.ndarray:
    """TopOpti_MaterialInterpolationSIMP.m:5: E = Emin + x^p (E0 - Emin)."""
    return Emin + np.asarray(x, dtype=np.float64).reshape(-1) ** p * (E0 - Emin)


class VoxelSolver:
    """One GB300 solver context for a padded voxel grid (ny, nx, nz)."""

    def __init__(self, voxels: np.ndarray, num_levels: int | None = None, non_dyadic: int = 1,
                 coarsest_resolution_control: int = 50000, poisson_ratio: float = 0.3,
                 cell_size: float = 1.0, omega: float = 0.35, device: int = 0, pad: bool = True):
        self.lib = L.load()
        vox = np.asarray(voxels, dtype=bool)
        if num_levels is None:
            num_levels = reference_num_levels(int(vox.sum()), coarsest_resolution_control)
            if num_levels < 0:
                raise ValueError("domain too small to build a mesh hierarchy")
        if pad:
            vox = pad_voxels(vox, num_levels)
        self.voxels = vox
        self.resY, self.resX, self.resZ = vox.shape
        opts = L.Options()
        self.lib.sgld_default_options(C.byref(opts))
        opts.num_levels, opts.non_dyadic = int(num_levels), int(non_dyadic)
        opts.poisson_ratio, opts.cell_size, opts.omega, opts.device = poisson_ratio, cell_size, omega, device
        buf = np.ascontiguousarray(vox.flatten(order="F").astype(np.uint8))
        ctx = C.c_void_p()
        rc = self.lib.sgld_create(self.resY, self.resX, self.resZ, _p(buf), C.byref(opts), C.byref(ctx))
        self.ctx = ctx
        if rc != L.SGLD_OK:
            msg = self.lib.sgld_last_error(ctx).decode() if ctx else "create failed"
            if ctx:
                self.lib.sgld_destroy(ctx)
                self.ctx = None
            raise L.SgldError(rc, msg)
        self.numLevels = int(self.lib.sgld_num_levels(ctx))
        self.levels = [self.level_info(i + 1) for i in range(self.numLevels)]
        self.numElements = self.levels[0]["numElements"]
        self.numNodes = self.levels[0]["numNodes"]
        self.numDOFs = 3 * self.numNodes
        self.omega = omega

    # -- housekeeping -------------------------------------------------------
    def _check(self, rc: int):
        if rc != L.SGLD_OK:
            raise L.SgldError(rc, self.lib.sgld_last_error(self.ctx).decode())

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.sgld_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def level_info(self, level: int) -> dict:
        res = (C.c_int * 3)()
        span = C.c_int()
        ne, nn = C.c_int64(), C.c_int64()
        self._check(self.lib.sgld_level_info(self.ctx, level, res, C.byref(span), C.byref(ne), C.byref(nn)))
        return {"resY": res[0], "resX": res[1], "resZ": res[2], "spanWidth": span.value,
                "numElements": ne.value, "numNodes": nn.value, "numDOFs": 3 * nn.value}

    def nodMapBack(self, level: int = 1) -> np.ndarray:
        out = np.zeros(self.levels[level - 1]["numNodes"], np.int64)
        self._check(self.lib.sgld_node_map(self.ctx, level, _p(out)))
        return out

    def eleMapBack(self, level: int = 1) -> np.ndarray:
        out = np.zeros(self.levels[level - 1]["numElements"], np.int64)
        self._check(self.lib.sgld_element_map(self.ctx, level, _p(out)))
        return out

    @property
    def Ke(self) -> np.ndarray:
        k = np.zeros(576)
        self._check(self.lib.sgld_get_ke(self.ctx, _p(k)))
        return k.reshape(24, 24, order="F")

    def set_ke(self, Ke: np.ndarray):
        k = np.asfortranarray(np.asarray(Ke, dtype=np.float64)).reshape(-1, order="F").copy()
        self._check(self.lib.sgld_set_ke(self.ctx, _p(k)))

    # -- setup ----------------------------------------------------------------
    def set_fixed_dofs(self, fixed_mask: np.ndarray):
        m = np.ascontiguousarray(np.asarray(fixed_mask, dtype=bool).reshape(-1).astype(np.uint8))
        if m.size != self.numDOFs:
            raise ValueError("fixed mask must have numDOFs entries")
        self._check(self.lib.sgld_set_fixed_dofs(self.ctx, _p(m)))

    def free_dofs(self, level: int) -> np.ndarray:
        out = np.zeros(self.levels[level - 1]["numDOFs"], np.uint8)
        self._check(self.lib.sgld_get_free_dofs(self.ctx, level, _p(out)))
        return out.astype(bool)

    def set_modulus(self, E: np.ndarray):
        e = np.ascontiguousarray(np.asarray(E, dtype=np.float64).reshape(-1))
        if e.size != self.numElements:
            raise ValueError("modulus must have numElements entries")
        self._check(self.lib.sgld_set_modulus(self.ctx, _p(e)))

    def set_modulus_device(self, ptr: int):
        self._check(self.lib.sgld_set_modulus_device(self.ctx, C.c_void_p(ptr)))

    def Solving_AssembleFEAstencil(self):
        self._check(self.lib.sgld_assemble(self.ctx))

    def diagK(self, level: int) -> np.ndarray:
        out = np.zeros(self.levels[level - 1]["numDOFs"])
        self._check(self.lib.sgld_get_diag(self.ctx, level, _p(out)))
        return out

    def Ks(self, level: int) -> np.ndarray:
        ne = self.levels[level - 1]["numElements"]
        out = np.zeros(576 * ne)
        self._check(self.lib.sgld_get_ks(self.ctx, level, _p(out)))
        return out.reshape(ne, 24, 24).transpose(2, 1, 0).copy(order="F")  # (24, 24, ne), column-major pages

    # -- operators ----------------------------------------------------------------
    def _vec(self, v, n):
        a = np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1))
        if a.size != n:
            raise ValueError(f"vector must have {n} entries, got {a.size}")
        return a

    def Solving_KbyU_MatrixFree(self, uVec, precision: str = "fp64") -> np.ndarray:
        """K u; ``precision`` 'mixed' applies the FP32 operator of the inner
        solve, 'mixed_df' the double-float one (sgld_kbyu_prec)."""
        u = self._vec(uVec, self.numDOFs)
        y = np.zeros_like(u)
        if precision == "fp64":
            self._check(self.lib.sgld_kbyu(self.ctx, _p(u), _p(y)))
        else:
            self._check(self.lib.sgld_kbyu_prec(self.ctx, _p(u), _p(y), _precision(precision)))
        return y

    def kbyu_double_float(self, uVec) -> np.ndarray:
        """K u in double-float arithmetic: the outer operator of precision "mixed_df"."""
        u = self._vec(uVec, self.numDOFs)
        y = np.zeros_like(u)
        self._check(self.lib.sgld_kbyu_df(self.ctx, _p(u), _p(y)))
        return y

    def Solving_RestrictResidual(self, rFiner, ii: int, precision: str = "fp64") -> np.ndarray:
        """R r; ``precision`` 'mixed' / 'mixed_df' applies the FP32 restriction
        of the inner solve's V-cycle (sgld_restrict_prec)."""
        r = self._vec(rFiner, self.levels[ii - 2]["numDOFs"])
        out = np.zeros(self.levels[ii - 1]["numDOFs"])
        if precision == "fp64":
            self._check(self.lib.sgld_restrict(self.ctx, ii, _p(r), _p(out)))
        else:
            self._check(self.lib.sgld_restrict_prec(self.ctx, ii, _p(r), _p(out), _precision(precision)))
        return out

    def Solving_InterpolationDeviation(self, xCoarser, ii: int) -> np.ndarray:
        x = self._vec(xCoarser, self.levels[ii - 1]["numDOFs"])
        out = np.zeros(self.levels[ii - 2]["numDOFs"])
        self._check(self.lib.sgld_interpolate(self.ctx, ii, _p(x), _p(out)))
        return out

    def Solving_Vcycle(self, r, precision: str = "fp64") -> np.ndarray:
        """z = M^-1 r; ``precision`` 'mixed' / 'mixed_df' applies the FP32 V-cycle
        of the inner solve (sgld_vcycle_prec)."""
        rv = self._vec(r, self.numDOFs)
        z = np.zeros_like(rv)
        if precision == "fp64":
            self._check(self.lib.sgld_vcycle(self.ctx, _p(rv), _p(z)))
        else:
            self._check(self.lib.sgld_vcycle_prec(self.ctx, _p(rv), _p(z), _precision(precision)))
        return z

    def Solving_BuildingMeshHierarchy(self, num_levels: int, non_dyadic: int = 0):
        """Rebuilds the coarse levels for another level count (sgld_build_hierarchy).
        Fixed DOFs and moduli must be set again afterwards."""
        self._check(self.lib.sgld_build_hierarchy(self.ctx, int(num_levels), int(non_dyadic)))
        self.numLevels = int(self.lib.sgld_num_levels(self.ctx))
        self.levels = [self.level_info(i + 1) for i in range(self.numLevels)]

    def pcg(self, b, tol: float = 1e-3, maxIT: int = 500, x0=None, precision: str = "fp64",
            inner_its: int = 0, history: bool = False, inner_tol: float = 0.0, out=None):
        """Runs the whole PCG on the device.  Returns (x, info dict).  ``out``:
        optional float64 array of numDOFs entries to receive x (for example
        page-locked host memory)."""
        bv = self._vec(b, self.numDOFs)
        # without x0 the library starts from zero on the device and never reads x;
        # it writes every entry of x on return
        if out is not None:
            if out.dtype != np.float64 or out.size != self.numDOFs or not out.flags.c_contiguous:
                raise ValueError("out must be a contiguous float64 array of numDOFs entries")
            x = out
            if x0 is not None:
                x[...] = self._vec(x0, self.numDOFs)
        else:
            x = np.empty_like(bv) if x0 is None else self._vec(x0, self.numDOFs).copy()
        hist = np.zeros(maxIT) if history else None
        o = L.SolveOpts(tol=tol, maxit=maxIT, use_x0=int(x0 is not None),
                        precision=_precision(precision),
                        inner_its=inner_its, history=hist.ctypes.data if history else None,
                        inner_tol=inner_tol)
        info = L.SolveInfo()
        self._check(self.lib.sgld_pcg(self.ctx, _p(bv), _p(x), C.byref(o), C.byref(info)))
        d = _info_dict(info)
        if history:
            d["history"] = hist[: info.iterations].copy()
        return x, d

    def solve_block(self, F, tol: float = 1e-6, maxIT: int = 500, U0=None, precision: str = "fp64",
                    inner_its: int = 0, inner_tol: float = 0.0):
        """Block right-hand side: F is (nrhs, numDOFs); returns (U (nrhs, numDOFs), list of info dicts)."""
        Fb = np.ascontiguousarray(np.asarray(F, dtype=np.float64).reshape(-1, self.numDOFs))
        nrhs = Fb.shape[0]
        U = np.zeros_like(Fb) if U0 is None else np.ascontiguousarray(
            np.asarray(U0, dtype=np.float64).reshape(nrhs, self.numDOFs)).copy()
        o = L.SolveOpts(tol=tol, maxit=maxIT, use_x0=int(U0 is not None), precision=_precision(precision),
                        inner_its=inner_its, history=None, profile=0, inner_tol=inner_tol)
        infos = (L.SolveInfo * max(nrhs, 1))()
        self._check(self.lib.sgld_solve_block(self.ctx, nrhs, _p(Fb), _p(U), C.byref(o), infos))
        return U, [_info_dict(infos[j]) for j in range(nrhs)]

    def pcg_device(self, b_ptr: int, x_ptr: int, tol: float, maxIT: int, use_x0: bool = False,
                   precision: str = "fp64", inner_its: int = 0, profile: bool = False,
                   inner_tol: float = 0.0) -> dict:
        o = L.SolveOpts(tol=tol, maxit=maxIT, use_x0=int(use_x0),
                        precision=_precision(precision),
                        inner_its=inner_its, history=None, profile=int(profile), inner_tol=inner_tol)
        info = L.SolveInfo()
        self._check(self.lib.sgld_pcg_device(self.ctx, C.c_void_p(b_ptr), C.c_void_p(x_ptr), C.byref(o),
                                             C.byref(info)))
        return _info_dict(info)

    OPS = {"kbyu64": 0, "kbyu32": 1, "vcycle64": 2, "vcycle32": 3, "assemble": 4, "kbyu_df": 5}

    def time_op(self, op: str, reps: int = 10) -> float:
        """Mean device milliseconds of one internal operator (CUDA events)."""
        ms = C.c_double()
        self._check(self.lib.sgld_time_op(self.ctx, self.OPS[op], int(reps), C.byref(ms)))
        return ms.value

    def inject_fault(self, kind: int = 1):
        """Test hook: kind 1 puts a NaN into the FP32 inner operator's moduli (until
        the next assembly), so that a mixed solve fails and falls back to FP64;
        kind 2 scales the next single-load mixed solve's converged iterate by
        1 + 1e-3 before its true residual is checked, so that residual
        replacement runs."""
        self._check(self.lib.sgld_inject_fault(self.ctx, int(kind)))

    def kbyu_tile(self) -> dict:
        """Tile of the FP32 K*u on the finest level (x width, node layers per CTA)."""
        tx, zc = C.c_int(), C.c_int()
        self._check(self.lib.sgld_kbyu_tile(self.ctx, C.byref(tx), C.byref(zc)))
        return {"tile_x": tx.value, "z_chunk": zc.value}

    @property
    def stream(self) -> int:
        """cudaStream_t of this context (every call runs on it)."""
        return int(self.lib.sgld_get_stream(self.ctx) or 0)

    def Solving_PreconditionedConjugateGradientSolver(self, AtX, PtV, b, tol, maxIT, printP="printP_OFF",
                                                      x0=None):
        """Solving_PreconditionedConjugateGradientSolver.m:1-37.  With this
        solver's own operators (AtX = Solving_KbyU_MatrixFree, PtV =
        Solving_Vcycle) the whole loop runs on the device; other callables are
        not supported (the reference's function-handle form is a MATLAB
        feature)."""
        if AtX != self.Solving_KbyU_MatrixFree or PtV != self.Solving_Vcycle:
            raise NotImplementedError("only this solver's KbyU / Vcycle operators are supported")
        x, info = self.pcg(b, tol, maxIT, x0=x0, history=(printP == "printP_ON"))
        if printP == "printP_ON":
            for k, r in enumerate(info["history"], 1):
                print(f" It.: {k:4d} Res.: {r:16.6e}")
        if info["converged"]:
            print(f"CG solver converged at iteration{info['its']:5d} to a solution with relative residual"
                  f"{info['relres']:16.6e}")
        else:
            warnings.warn("Exceed the maximum iterate numbers")
            print(f"The iterative process stops at residual = {info['relres']:10.4f}")
        return x, info["its"]

    def Solving_CG_GMGS(self, F, U0, tol: float, maxIT: int, printP="printP_OFF"):
        """Solving_CG_GMGS.m:7: PCG warm-started from the previous U."""
        return self.Solving_PreconditionedConjugateGradientSolver(
            self.Solving_KbyU_MatrixFree, self.Solving_Vcycle, F, tol, maxIT, printP, U0)

    def TopOpti_ComputeUnitCompliance(self, U):
        """Returns (ceList, c) with c = sum(E .* ce) (FEA_ComputeComplianceVoxel.m:20-22)."""
        u = self._vec(U, self.numDOFs)
        ce = np.zeros(self.numElements)
        c = C.c_double()
        self._check(self.lib.sgld_compliance(self.ctx, _p(u), _p(ce), C.byref(c)))
        return ce, c.value

    def solve(self, F, tol: float = 1e-6, maxIT: int = 500, precision: str = "fp64"):
        """sgld_solve: F is (nrhs, numDOFs) or one vector; returns (U, its, relres)
        with one entry per load case."""
        Fb = np.ascontiguousarray(np.asarray(F, dtype=np.float64).reshape(-1, self.numDOFs))
        nrhs = Fb.shape[0]
        U = np.empty_like(Fb)
        its = np.zeros(nrhs, np.int32)
        relres = np.zeros(nrhs)
        self._check(self.lib.sgld_solve(self.ctx, nrhs, _p(Fb), _p(U), float(tol), int(maxIT),
                                        _precision(precision), _p(its), _p(relres)))
        return U, its, relres

    def vonmises(self, U):
        """sgld_vonmises: (per-element von Mises, per-node von Mises)."""
        u = self._vec(U, self.numDOFs)
        vme = np.zeros(self.numElements)
        vmn = np.zeros(self.numNodes)
        self._check(self.lib.sgld_vonmises(self.ctx, _p(u), _p(vme), _p(vmn)))
        return vme, vmn

    def FEA_StressAnalysis(self, U):
        """Returns (cartesianStressField numNodes x 6, vonMises per node,
        per-element von Mises with the reference's extra square root)."""
        u = self._vec(U, self.numDOFs)
        s6 = np.zeros(6 * self.numNodes)
        vmn = np.zeros(self.numNodes)
        vme = np.zeros(self.numElements)
        self._check(self.lib.sgld_stress(self.ctx, _p(u), _p(s6), _p(vmn), _p(vme)))
        return s6.reshape(self.numNodes, 6), vmn, vme

    def FEA_ComputePrincipalStress(self, U):
        """Principal stresses of the nodal stress field: (numNodes x 12 rows
        [l1 v1 l2 v2 l3 v3], ascending l, eigenvectors signed so that their
        largest-magnitude entry is positive) and the per-element dominant
        principal direction (numElements x 3)."""
        u = self._vec(U, self.numDOFs)
        ps = np.zeros(12 * self.numNodes)
        dd = np.zeros(3 * self.numElements)
        self._check(self.lib.sgld_principal_stress(self.ctx, _p(u), _p(ps), _p(dd)))
        return ps.reshape(self.numNodes, 12), dd.reshape(self.numElements, 3)

    # -- SIMP loop (TopOpti_GlobalVolumeConstraint_Tmp.m) ---------------------------
    def TopOpti_PerformDensityFiltering(self, x, rMin: float) -> np.ndarray:
        """Cone filter of an element field (TopOpti_PerformDensityFiltering_mex)."""
        xv = self._vec(x, self.numElements)
        y = np.zeros(self.numElements)
        self._check(self.lib.sgld_density_filter(self.ctx, float(rMin), _p(xv), _p(y)))
        return y

    def set_passive(self, elements):
        """Passive elements (compact 0-based indices) kept solid by the SIMP loop."""
        idx = np.ascontiguousarray(np.asarray(elements, dtype=np.int64).ravel())
        self._check(self.lib.sgld_set_passive(self.ctx, idx.size, _p(idx) if idx.size else None))

    def TopOpti_PDEFiltering(self, x, rHatMin: float, tol: float = 1e-6, maxIT: int = 500):
        """PDE (Helmholtz) filter of an element field (TopOpti_PDEFiltering_matrixFree.m).
        Returns (filtered field, PCG iterations)."""
        xv = self._vec(x, self.numElements)
        y = np.zeros(self.numElements)
        its = C.c_int()
        self._check(self.lib.sgld_pde_filter(self.ctx, float(rHatMin), _p(xv), _p(y), float(tol), int(maxIT),
                                             C.byref(its)))
        return y, its.value

    def MMA(self, xval, xmin, xmax, xold1, xold2, df0dx, fval, dfdx):
        """One MMA update with one constraint (MMA_mex's arguments and outputs):
        returns (xnew, xold1, xold2)."""
        xv = np.ascontiguousarray(xval, dtype=np.float64).ravel()
        n = xv.size
        arr = [np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (xmin, xmax, xold1, xold2, df0dx)]
        fv = np.atleast_1d(np.asarray(fval, dtype=np.float64)).copy()
        dg = np.ascontiguousarray(dfdx, dtype=np.float64).ravel()
        xn, o1, o2 = np.zeros(n), np.zeros(n), np.zeros(n)
        self._check(self.lib.sgld_mma_update(self.ctx, 1, n, _p(xv), _p(arr[0]), _p(arr[1]), _p(arr[2]), _p(arr[3]),
                                             _p(arr[4]), _p(fv), _p(dg), _p(xn), _p(o1), _p(o2)))
        return xn, o1, o2

    def TopOpti_SetupDensityFilter(self, rMin: float) -> np.ndarray:
        """Weight sums Hs of the cone filter (TopOpti_SetupDensityFilter_mex)."""
        y = np.zeros(self.numElements)
        self._check(self.lib.sgld_density_filter(self.ctx, float(rMin), None, _p(y)))
        return y

    def TopOpti_LocalVolumeConstraint(self, F, rMin: float = 1.5, rHat: float = 8.0, alpha: float = 0.5,
                                      p: float = 16.0, nLoop: int = 300, move: float = 0.1,
                                      minChange: float = 1e-4, maxSharpness: float = 0.05,
                                      simp_penalty: float = 3.0, penalty: float = 3.0,
                                      penalty_increment: float = 0.2, penalty_interval: int = 30,
                                      beta: float = 1.0, eta: float = 0.5, beta_max: float = 128.0,
                                      beta_interval: int = 40, E0: float = 1.0, Emin: float = 1e-6,
                                      tol: float = 1e-6, maxIT: int = 500, precision: str = "fp64"):
        """TopOpti_LocalVolumeConstraint.m on the device (porous infill: p-norm of
        the PDE-filtered local volume <= alpha, MMA, Heaviside projection with
        beta continuation).  Passive elements (``set_passive``) stay solid.
        Returns (xPhys, history list); history ``constraint`` is fval."""
        return self._projected(0, 0.0, F, rMin, rHat, alpha, p, nLoop, move, minChange, maxSharpness,
                               simp_penalty, penalty, penalty_increment, penalty_interval, beta, eta, beta_max,
                               beta_interval, E0, Emin, tol, maxIT, precision)

    def TopOpti_GlobalVolumeConstraintProjected(self, F, volfrac: float = 0.3, rMin: float = 1.5,
                                                nLoop: int = 300, move: float = 0.1, minChange: float = 1e-4,
                                                maxSharpness: float = 0.05, simp_penalty: float = 3.0,
                                                penalty: float = 3.0, penalty_increment: float = 0.2,
                                                penalty_interval: int = 30, beta: float = 1.0, eta: float = 0.5,
                                                beta_max: float = 128.0, beta_interval: int = 40, E0: float = 1.0,
                                                Emin: float = 1e-6, tol: float = 1e-6, maxIT: int = 500,
                                                precision: str = "fp64"):
        """TopOpti_GlobalVolumeConstraint.m (the full loop: Heaviside projection with
        beta/penalty continuation, solid-normalised compliance) with MMA, on the
        device.  Returns (xPhys, history list)."""
        return self._projected(1, volfrac, F, rMin, 8.0, 0.5, 16.0, nLoop, move, minChange, maxSharpness,
                               simp_penalty, penalty, penalty_increment, penalty_interval, beta, eta, beta_max,
                               beta_interval, E0, Emin, tol, maxIT, precision)

    def _projected(self, constraint, volfrac, F, rMin, rHat, alpha, p, nLoop, move, minChange, maxSharpness,
                   simp_penalty, penalty, penalty_increment, penalty_interval, beta, eta, beta_max, beta_interval,
                   E0, Emin, tol, maxIT, precision):
        Fv = self._vec(F, self.numDOFs)
        so = L.SolveOpts(tol=tol, maxit=maxIT, use_x0=1, precision=_precision(precision), inner_its=0,
                         history=None, profile=0, inner_tol=0.0)
        o = L.TopOptProjectedOpts(constraint=constraint, volfrac=volfrac, rmin=rMin, rhat=rHat, alpha=alpha, pnorm=p, move=move, n_loop=nLoop,
                              min_change=minChange, max_sharpness=maxSharpness, simp_penalty=simp_penalty,
                              penalty=penalty, penalty_increment=penalty_increment,
                              penalty_interval=penalty_interval, beta=beta, eta=eta, beta_max=beta_max,
                              beta_interval=beta_interval, E0=E0, Emin=Emin, solve=so)
        xp = np.zeros(self.numElements)
        hist = (L.TopOptIter * nLoop)()
        nit = C.c_int()
        self._check(self.lib.sgld_topopt_projected(self.ctx, C.byref(o), _p(Fv), _p(xp), hist, C.byref(nit)))
        return xp, [{k: getattr(hist[i], k) for k, _ in L.TopOptIter._fields_} for i in range(nit.value)]

    def TopOpti_GlobalVolumeConstraint(self, F, volfrac: float = 0.3, rMin: float = 1.5, nLoop: int = 60,
                                       move: float = 0.1, minChange: float = 1e-4, maxSharpness: float = 0.05,
                                       penalty: float = 3.0, E0: float = 1.0, Emin: float = 1e-9,
                                       tol: float = 1e-6, maxIT: int = 500, precision: str = "fp64",
                                       inner_its: int = 0, x0=None, inner_tol: float = 0.0,
                                       optimizer: str = "OC", learned: int = 0, net_level: int = 0,
                                       net_train_steps: int = 0, net_lr: float = 0.0, resume=None,
                                       return_state: bool = False):
        """The whole SIMP loop on the device.  Returns (xPhys, history list), and
        with return_state=True also the loop state {"loop", "x", "xPhys", "U"}
        (what ``sgldbench_gb300.checkpoint`` saves).

        learned=1 turns on the learned warm start (a U-Net on the grid of
        level ``net_level`` trained online on the loop's solves, combined with
        the previous displacement change); learned=2 uses the previous change
        alone.  The solves still run to ``tol``, so only iteration counts
        change.  resume=state continues a loop from its state (x0 is then
        ignored); nLoop stays the total iteration cap."""
        Fv = self._vec(F, self.numDOFs)
        so = L.SolveOpts(tol=tol, maxit=maxIT, use_x0=1,
                         precision=_precision(precision),
                         inner_its=inner_its, history=None, profile=0, inner_tol=inner_tol)
        if optimizer not in ("OC", "MMA"):
            raise ValueError("optimizer must be 'OC' or 'MMA'")
        o = L.TopOptOpts(volfrac=volfrac, rmin=rMin, move=move, n_loop=nLoop, min_change=minChange,
                         max_sharpness=maxSharpness, penalty=penalty, E0=E0, Emin=Emin, solve=so,
                         optimizer=1 if optimizer == "MMA" else 0, learned=int(learned),
                         net_level=net_level, net_train_steps=net_train_steps, net_lr=net_lr)
        xp = np.zeros(self.numElements)
        hist = (L.TopOptIter * nLoop)()
        nit = C.c_int()
        keep = []
        if resume is not None:
            x0 = resume["x"]
            xph0 = self._vec(resume["xPhys"], self.numElements)
            U0 = self._vec(resume["U"], self.numDOFs)
            keep += [xph0, U0]
            o.xphys0, o.U0, o.loop0 = _p(xph0), _p(U0), int(resume["loop"])
        xout = np.zeros(self.numElements)
        o.x_out = _p(xout)
        x0v = self._vec(x0, self.numElements) if x0 is not None else None
        self._check(self.lib.sgld_topopt(self.ctx, C.byref(o), _p(Fv), _p(x0v) if x0v is not None else None,
                                         _p(xp), hist, C.byref(nit)))
        recs = []
        for i in range(nit.value):
            h = hist[i]
            recs.append({k: getattr(h, k) for k, _ in L.TopOptIter._fields_})
        if not return_state:
            return xp, recs
        U = np.zeros(self.numDOFs)
        self._check(self.lib.sgld_topopt_displacement(self.ctx, _p(U)))
        loop = (int(resume["loop"]) if resume is not None else 0) + nit.value
        return xp, recs, {"loop": loop, "x": xout, "xPhys": xp.copy(), "U": U}


class LoadCases:
    """Learned start for a sequence of load cases on one VoxelSolver
    (sgld_cases_* of the C ABI; no counterpart in the reference, which starts
    every new load case from zero).  Training cases add their solutions to a
    K-orthonormal basis and train a coarse-level U-Net on the correction the
    solve found beyond the basis start; a new case starts from the basis
    projection (mode 1) plus the network's correction when it lowers r'Mr
    (mode 2).  Every solve still runs to its tolerance on the true residual."""

    MODES = {"zero": 0, "basis": 1, "learned": 2}

    def __init__(self, solver: VoxelSolver, max_basis: int = 20, net_level: int = 0, train_steps: int = 8):
        self.s = solver
        self.lib = solver.lib
        h = C.c_void_p()
        solver._check(self.lib.sgld_cases_create(solver.ctx, int(max_basis), int(net_level), int(train_steps),
                                                  C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.sgld_cases_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def basis_size(self) -> int:
        return int(self.lib.sgld_cases_basis_size(self.h))

    def _opts(self, tol, maxIT, precision, inner_its, inner_tol):
        return L.SolveOpts(tol=tol, maxit=maxIT, use_x0=0, precision=_precision(precision), inner_its=inner_its,
                           history=None, profile=0, inner_tol=inner_tol)

    @staticmethod
    def _stats(st) -> dict:
        return {k: getattr(st, k) for k, _ in L.CasesStats._fields_ if k != "diagnostics"}

    def solve(self, F, mode: str = "learned", train: bool = False, tol: float = 1e-6, maxIT: int = 5000,
              precision: str = "mixed_df", inner_its: int = 0, inner_tol: float = 0.0, diagnostics: bool = False,
              out=None):
        """One load case from host vectors.  Returns (U, info dict, stats dict)."""
        bv = self.s._vec(F, self.s.numDOFs)
        x = np.empty_like(bv) if out is None else out
        o = self._opts(tol, maxIT, precision, inner_its, inner_tol)
        info, st = L.SolveInfo(), L.CasesStats(diagnostics=int(diagnostics))
        self.s._check(self.lib.sgld_cases_solve(self.h, _p(bv), _p(x), C.byref(o), self.MODES[mode], int(train),
                                                C.byref(info), C.byref(st)))
        return x, _info_dict(info), self._stats(st)

    def solve_device(self, F_ptr: int, U_ptr: int, mode: str = "learned", train: bool = False, tol: float = 1e-6,
                     maxIT: int = 5000, precision: str = "mixed_df", inner_its: int = 0, inner_tol: float = 0.0,
                     diagnostics: bool = False):
        """One load case from compact device vectors.  Returns (info dict, stats dict)."""
        o = self._opts(tol, maxIT, precision, inner_its, inner_tol)
        info, st = L.SolveInfo(), L.CasesStats(diagnostics=int(diagnostics))
        self.s._check(self.lib.sgld_cases_solve_device(self.h, C.c_void_p(F_ptr), C.c_void_p(U_ptr), C.byref(o),
                                                       self.MODES[mode], int(train), C.byref(info), C.byref(st)))
        return _info_dict(info), self._stats(st)
