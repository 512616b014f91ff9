"""GPU: the two C++ hosts over the C ABI.

* The MEX gateway (sgldbench_gb300/mex/sgld_gpu_mex.cpp) compiled against the
  oracle's MEX API stand-in and driven the way MATLAB calls it (mxArrays in,
  mxArrays out): create / fixed / modulus / assemble / kbyu / vcycle / pcg /
  compliance / stress / filter, checked against the oracle, and its error
  behaviour (mexErrMsgIdAndTxt) on bad input.
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
