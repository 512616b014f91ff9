"""GPU: the two C++ hosts over the C ABI.

* The MEX gateway (sgldbench_gb300/mex/sgld_gpu_mex.cpp) compiled against the
  oracle's MEX API stand-in and driven the way MATLAB calls it (mxArrays in,
  mxArrays out): create / fixed / modulus / assemble / kbyu / vcycle / pcg /
  compliance / stress / filter, checked against the oracle, and its error
  behaviour (mexErrMsgIdAndTxt) on bad input; the callers' commands; kbyu and
  vcycle with a precision argument and the hierarchy rebuild; clear mex.
* The standalone harness (sgldbench_gb300/harness/sgld_harness.cpp) on config 0.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import glue as G
from oracle import mexcall

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@pytest.fixture(scope="module")
def gateway(built_lib, tmp_path_factory):
    from sgldbench_gb300 import build as B

    out = str(tmp_path_factory.mktemp("mex") / "libsgld_gpu_mex_test.so")
    B.build_mex_gateway(os.path.join(ROOT, "oracle", "mexshim"), out)
    return mexcall.MexLib(out)


def test_gateway_solve_path(gateway):
    M = gateway
    rng = np.random.default_rng(9)
    vox = rng.random((8, 16, 8)) < 0.85
    m = G.build_model(vox, omega=0.6)
    _, nlev0, padded, _ = G.voxel_discretization(vox)
    nlev = M.call("sgld_gpu_mex", 1, "create", padded, float(nlev0), 1.0, 0.3, 1.0, 0.6)
    assert int(np.asarray(nlev).ravel()[0]) == m.numLevels
    l1 = m.levels[0]
    E = rng.uniform(0.2, 1.0, l1.numElements)
    G.set_modulus(m, E)
    G.assemble_stencil(m)
    M.call("sgld_gpu_mex", 0, "fixed", l1.fixedDOFs)
    M.call("sgld_gpu_mex", 0, "modulus", E)
    M.call("sgld_gpu_mex", 0, "assemble")
    u = rng.standard_normal(l1.numDOFs)
    assert _rel(M.call("sgld_gpu_mex", 1, "kbyu", u).ravel(), G.kbyu(m, u)) <= 1e-13
    r = u * l1.freeDOFs
    assert _rel(M.call("sgld_gpu_mex", 1, "vcycle", r).ravel(), G.vcycle(m, r)) <= 1e-9
    U, its = M.call("sgld_gpu_mex", 2, "pcg", m.F, 1e-6, 500.0)
    U_o, its_o = G.solve(m, tol=1e-6, maxIT=500)
    assert abs(int(np.asarray(its).ravel()[0]) - its_o) <= 1
    assert np.linalg.norm(U.ravel() - U_o) / np.linalg.norm(U_o) <= 1e-8
    # on a solution field u_e'Ke u_e cancels strongly (near-rigid element motion),
    # so the element energies agree to 1e-11 of the largest, not 1e-13
    ce, c = M.call("sgld_gpu_mex", 2, "compliance", U.ravel())
    assert _rel(ce.ravel(), G.unit_compliance(m, U.ravel())) <= 1e-11
    s, vm, vme = M.call("sgld_gpu_mex", 3, "stress", U.ravel())
    s_o, vm_o = G.stress_analysis(m, U.ravel())
    assert _rel(s, s_o) <= 1e-11 and _rel(vm.ravel(), vm_o) <= 1e-11
    assert _rel(vme.ravel(), G.per_element_von_mises(m, s_o)) <= 1e-11
    x = rng.random(l1.numElements)
    from oracle import kernels as OK

    f = M.call("sgld_gpu_mex", 1, "filter", x, 1.5).ravel()
    assert _rel(f, OK.density_filter(x, 1.5, l1.eleMapForward, l1.resX, l1.resY, l1.resZ)) <= 1e-14
    # the reference's error behaviour: bad input raises (mexErrMsgIdAndTxt)
    with pytest.raises(mexcall.MexError):
        M.call("sgld_gpu_mex", 1, "kbyu", u[:-3])
    with pytest.raises(mexcall.MexError):
        M.call("sgld_gpu_mex", 0, "nonsense")
    M.call("sgld_gpu_mex", 0, "destroy")
    with pytest.raises(mexcall.MexError):
        M.call("sgld_gpu_mex", 1, "kbyu", u)


def test_gateway_callers(gateway):
    """The gateway's commands for the callers around the solve, driven as MATLAB
    would: principal stresses, the PDE filter, MMA and the two SIMP loops
    (with passive elements given as 1-based indices), against the oracle."""
    from oracle import mma as OM

    M = gateway
    vox = np.ones((8, 16, 8), bool)
    m = G.build_model(vox, omega=0.6)
    _, nlev0, padded, _ = G.voxel_discretization(vox)
    M.call("sgld_gpu_mex", 1, "create", padded, float(nlev0), 1.0, 0.3, 1.0, 0.6)
    l1 = m.levels[0]
    n = l1.numElements
    rng = np.random.default_rng(3)
    E = rng.uniform(0.3, 1.0, n)
    G.set_modulus(m, E)
    G.assemble_stencil(m)
    M.call("sgld_gpu_mex", 0, "fixed", l1.fixedDOFs)
    M.call("sgld_gpu_mex", 0, "modulus", E)
    M.call("sgld_gpu_mex", 0, "assemble")
    U_o, _ = G.solve(m, tol=1e-10, maxIT=2000)
    ps, dirs = M.call("sgld_gpu_mex", 2, "principal", U_o)
    s_o, _ = G.stress_analysis(m, U_o)
    ps_o = G.principal_stress(s_o)
    assert ps.shape == (l1.numNodes, 12) and dirs.shape == (n, 3)
    lam = ps[:, [0, 4, 8]]
    assert _rel(lam, ps_o[:, [0, 4, 8]]) <= 1e-9
    x = rng.random(n)
    y, its = M.call("sgld_gpu_mex", 2, "pdefilter", x, 3.0, 1e-10, 1000.0)
    y_o, its_o = G.pde_filter(m, x, 3.0, tol=1e-10, maxIT=1000)
    assert _rel(y.ravel(), y_o) <= 1e-9 and abs(int(np.asarray(its).ravel()[0]) - its_o) <= 1
    nv = 50
    xv = rng.uniform(0.2, 0.8, nv)
    xmin, xmax = np.maximum(0, xv - 0.1), np.minimum(1, xv + 0.1)
    df0, dg = -rng.random(nv), rng.random(nv) / nv
    out = M.call("sgld_gpu_mex", 3, "mma", 1.0, float(nv), xv, xmin, xmax, xv, xv, df0, np.array([0.05]), dg)
    x_o, _, _ = OM.mma_update(1, nv, xv, xmin, xmax, xv, xv, df0, 0.05, dg)
    assert _rel(out[0].ravel(), x_o) <= 1e-10
    # the _Tmp loop with MMA and passive elements, and the local-volume loop
    passive = np.arange(0, n, 17)
    M.call("sgld_gpu_mex", 0, "passive", (passive + 1).astype(float))
    xp, hist = M.call("sgld_gpu_mex", 2, "topopt", m.F, 0.3, 1.5, 4.0, 1e-10, 2000.0, "MMA")
    xp_o, hist_o = G.topopt_global_volume(m, G.TopOptOptions(n_loop=4, tol=1e-10, maxit=2000, Emin=1e-6,
                                                             optimizer="MMA", passive=passive))
    assert hist.shape == (len(hist_o), 6)
    assert _rel(hist[:, 0], np.array([h["c"] for h in hist_o])) <= 1e-6
    assert _rel(xp.ravel(), xp_o) <= 1e-5 and np.all(xp.ravel()[passive] == 1.0)
    xl, hl = M.call("sgld_gpu_mex", 2, "topopt_local", m.F, 0.6, 1.5, 3.0, 16.0, 3.0, 1e-10, 2000.0)
    xl_o, hl_o = G.topopt_local_volume(m, G.LocalOptions(rmin=1.5, rhat=3.0, alpha=0.6, n_loop=3, tol=1e-10,
                                                         maxit=2000, passive=passive))
    assert _rel(hl[:, 0], np.array([h["c"] for h in hl_o])) <= 1e-6
    assert np.abs(hl[:, 4] - np.array([h["fval"] for h in hl_o])).max() <= 1e-8
    assert _rel(xl.ravel(), xl_o) <= 1e-5
    M.call("sgld_gpu_mex", 0, "passive", np.zeros(0))
    with pytest.raises(mexcall.MexError):
        M.call("sgld_gpu_mex", 0, "passive", np.array([float(n + 1)]))
    M.call("sgld_gpu_mex", 0, "destroy")


def test_harness_config0(built_lib):
    from sgldbench_gb300 import build as B

    exe = B.build_harness()
    out = subprocess.run([exe, "--size", "64", "32", "32", "--levels", "4", "--nondyadic", "1", "--omega", "0.6",
                          "--tol", "1e-6"], capture_output=True, text=True, check=True)
    rec = json.loads(out.stdout.strip().splitlines()[-1])
    assert rec["converged"] == 1 and rec["levels"] == 3 and rec["dofs"] == 212355
    vox = np.ones((32, 64, 32), bool)
    m = G.build_model(vox, omega=0.6)
    G.set_modulus(m, np.ones(m.levels[0].numElements))
    G.assemble_stencil(m)
    U_o, its_o = G.solve(m, tol=1e-6, maxIT=500)
    assert abs(rec["iterations"] - its_o) <= 1
    assert abs(rec["compliance"] - G.compliance(m, U_o)) <= 1e-6 * G.compliance(m, U_o)
    # the headline mode from the command line: same compliance to 1e-6
    out = subprocess.run([exe, "--size", "64", "32", "32", "--levels", "4", "--nondyadic", "1", "--omega", "0.6",
                          "--tol", "1e-6", "--precision", "mixed_df"], capture_output=True, text=True, check=True)
    mix = json.loads(out.stdout.strip().splitlines()[-1])
    assert mix["precision"] == "mixed_df" and mix["converged"] == 1 and mix["true_relres"] < 1e-6
    assert abs(mix["compliance"] - G.compliance(m, U_o)) <= 1e-6 * G.compliance(m, U_o)


def test_gateway_clear_releases_context(gateway):
    """`clear mex` runs the gateway's mexAtExit function, which destroys the
    context: the next command that needs one is refused until 'create'."""
    M = gateway
    vox = np.ones((8, 16, 8), bool)
    _, nlev0, padded, _ = G.voxel_discretization(vox)
    M.call("sgld_gpu_mex", 1, "create", padded, float(nlev0), 1.0, 0.3, 1.0, 0.6)
    M.clear()
    with pytest.raises(mexcall.MexError, match="create"):
        M.call("sgld_gpu_mex", 0, "assemble")
    M.call("sgld_gpu_mex", 1, "create", padded, float(nlev0), 1.0, 0.3, 1.0, 0.6)
    M.call("sgld_gpu_mex", 0, "destroy")
    M.clear()   # nothing left to release


def test_gateway_precision_and_hierarchy(gateway):
    """'kbyu' / 'vcycle' with a precision argument give the library's
    operators of that solve mode; 'hierarchy' rebuilds the levels."""
    from sgldbench_gb300 import VoxelSolver

    M = gateway
    vox = np.ones((8, 16, 8), bool)
    m = G.build_model(vox, omega=0.6)
    _, nlev0, padded, _ = G.voxel_discretization(vox)
    assert int(np.asarray(M.call("sgld_gpu_mex", 1, "create", padded, float(nlev0), 0.0, 0.3, 1.0, 0.6)).ravel()[0]) == nlev0
    l1 = m.levels[0]
    E = np.random.default_rng(5).uniform(0.3, 1.0, l1.numElements)
    s = VoxelSolver(padded, num_levels=nlev0, non_dyadic=0, omega=0.6, pad=False)
    M.call("sgld_gpu_mex", 0, "fixed", l1.fixedDOFs)
    M.call("sgld_gpu_mex", 0, "modulus", E)
    M.call("sgld_gpu_mex", 0, "assemble")
    s.set_fixed_dofs(l1.fixedDOFs)
    s.set_modulus(E)
    s.Solving_AssembleFEAstencil()
    u = np.random.default_rng(6).standard_normal(s.numDOFs)
    for mode, prec in (("fp64", "fp64"), ("mixed", "mixed_df"), ("mixed64", "mixed")):
        y = M.call("sgld_gpu_mex", 1, "kbyu", u, mode).ravel()
        assert np.array_equal(y, s.Solving_KbyU_MatrixFree(u, prec))
        z = M.call("sgld_gpu_mex", 1, "vcycle", u, mode).ravel()
        assert np.array_equal(z, s.Solving_Vcycle(u, prec))
    with pytest.raises(mexcall.MexError, match="precision"):
        M.call("sgld_gpu_mex", 1, "kbyu", u, "half")
    assert int(np.asarray(M.call("sgld_gpu_mex", 1, "hierarchy", 2.0)).ravel()[0]) == 2
    with pytest.raises(mexcall.MexError):
        M.call("sgld_gpu_mex", 1, "hierarchy", 1.0)
    s.close()
    M.call("sgld_gpu_mex", 0, "destroy")
