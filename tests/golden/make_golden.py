"""Generates the golden fixtures of the CPU parity tests.

Run where the SGLDBench checkout is available (it is read, never modified):

    sh oracle/build_ref.sh && python tests/golden/make_golden.py

1. ``ref_tables.npz``: the hard-coded tables of the reference's MATLAB code,
   parsed from its source text: the trilinear transfer tables 'inNODE' and
   'inDOF' for span widths 2 and 4
   (src/Solving_Operator4MultiGridRestrictionAndInterpolation.m), the child
   node tables (src/Solving_SubEleNodMat.m) and the Gauss points
   (src/FEA_GaussianIntegral.m).
2. ``ref_kernels.npz``: inputs and outputs of the reference's own C++ MEX
   kernels (compiled unmodified into oracle/_ref/libref_mex.so against the
   oracle's MEX shim) on a seeded irregular voxel model: K*u, restriction,
   interpolation (every level), unit compliance, both stencil-assembly
   kernels and the two density-filter kernels.  The index tables fed to the
   kernels come from the oracle's restatement of the MATLAB glue and are
   stored with the fixture.
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.refpath import reference_root  # noqa: E402

REF = reference_root()
if REF is None:
    sys.exit("reference checkout not found: set SGLD_REFERENCE to its root")


def _parse_matrix(text: str) -> np.ndarray:
    rows = []
    for ln in text.strip().splitlines():
        ln = ln.split("%")[0].strip().rstrip(";").strip()
        if not ln:
            continue
        rows.append([float(v) for v in ln.replace("[", " ").replace("]", " ").split()])
    return np.array(rows)


def parse_tables():
    src = open(os.path.join(REF, "src", "Solving_Operator4MultiGridRestrictionAndInterpolation.m")).read()
    out = {}
    for span in (2, 4):
        block = src.split(f"case {span}")[1]
        for opt in ("inNODE", "inDOF"):
            part = block.split(f"strcmp(opt, '{opt}')")[1]
            body = part[part.index("ss = [") + len("ss = ["):]
            body = body[:body.index("];")]
            out[f"{opt}_{span}"] = _parse_matrix(body)
    sub = open(os.path.join(REF, "src", "Solving_SubEleNodMat.m")).read()
    for span in (2, 4):
        part = sub.split(f"case {span}")[1]
        body = part[part.index("val = [") + len("val = ["):]
        body = body[:body.index("];")]
        out[f"SubEleNodMat_{span}"] = _parse_matrix(body).astype(np.int32)
    g = open(os.path.join(REF, "src", "FEA_GaussianIntegral.m")).read()
    for name in ("s", "t", "p"):
        body = re.search(rf"\b{name}\s*=\s*\[([^\]]*)\]'", g).group(1)
        out[f"gauss_{name}"] = np.array([float(v) for v in body.replace("...", " ").replace(",", " ").split()])
    return out


def make_kernels():
    from oracle import glue as G
    from oracle import mexcall

    R = mexcall.ref_lib()
    if R is None:
        raise SystemExit("oracle/_ref/libref_mex.so is not built (run oracle/build_ref.sh)")
    rng = np.random.default_rng(20240601)
    vox = rng.random((16, 24, 16)) < 0.7
    m = G.build_model(vox, omega=0.6)
    l1 = m.levels[0]
    E = rng.uniform(0.05, 1.0, l1.numElements)
    u = rng.standard_normal(l1.numDOFs)
    d = {"vox": vox, "E": E, "u": u, "Ke": m.Ke, "num_levels": m.numLevels}
    d["l1_eNodMat"] = l1.eNodMat
    d["l1_eleMapForward"] = l1.eleMapForward
    d["l1_res"] = np.array([l1.resX, l1.resY, l1.resZ])
    d["y_kbyu"] = R.call("ref_Solving_KbyU_MatrixFree_mex", 1, u, l1.eNodMat, m.Ke, E, l1.colors).ravel()
    d["ce"] = R.call("ref_TopOpti_CmptUnitCompliance_mex", 1, u, l1.eNodMat, m.Ke).ravel()
    for c in range(8):
        d[f"l1_color{c}"] = l1.colors[c]
    for ii in range(2, m.numLevels + 1):
        c, f = m.levels[ii - 1], m.levels[ii - 2]
        pre = f"l{ii}_"
        for k in ("transferMat", "transferMatCoeffi", "solidNodeMapCoarser2Finer", "eNodMat", "elementUpwardMap",
                  "eleMapBack"):
            d[pre + k] = getattr(c, k)
        d[pre + "sizes"] = np.array([c.numNodes, c.intermediateNumNodes, f.numNodes, c.spanWidth])
        for cc in range(8):
            d[pre + f"color{cc}"] = c.colors[cc]
        rf = rng.standard_normal((f.numNodes, 3))
        xc = rng.standard_normal((c.numNodes, 3))
        d[pre + "rf"] = rf
        d[pre + "xc"] = xc
        d[pre + "rc"] = R.call("ref_Solving_Restriction_MatrixFree_mex", 1, rf, c.transferMat,
                               np.ascontiguousarray(c.multiGridOperatorRI.T), c.eNodMat, float(c.numNodes),
                               float(c.intermediateNumNodes), c.solidNodeMapCoarser2Finer, c.transferMatCoeffi,
                               c.colors)
        d[pre + "xf"] = R.call("ref_Solving_Interpolation_MatrixFree_mex", 1, xc, c.transferMat,
                               c.multiGridOperatorRI, c.eNodMat, float(f.numNodes), float(c.intermediateNumNodes),
                               c.solidNodeMapCoarser2Finer, c.transferMatCoeffi, c.colors)
    c2 = m.levels[1]
    s2 = c2.spanWidth
    d["Ks2"] = R.call("ref_Solving_AssembleCmptStencilFromFinestLevel", 1, m.Ke, E, c2.elementUpwardMap,
                      sp.csc_matrix(G.ri_inDOF(s2)), G.local_mapping(s2).reshape(-1, 1), float((s2 + 1) ** 3))
    c3 = m.levels[2]
    s3 = c3.spanWidth
    d["Ks3"] = R.call("ref_Solving_AssembleCmptStencilFromNonFinestLevel", 1, d["Ks2"], c3.elementUpwardMap,
                      sp.csc_matrix(G.ri_inDOF(s3)), G.local_mapping(s3).reshape(-1, 1), float((s3 + 1) ** 3))
    x = rng.random(l1.numElements)
    d["filter_x"] = x
    args = (float(l1.numElements), l1.eleMapForward, float(l1.resX), float(l1.resY), float(l1.resZ))
    d["Hs"] = R.call("ref_TopOpti_SetupDensityFilter_mex", 1, 1.5, *args).ravel()
    d["filtered"] = R.call("ref_TopOpti_PerformDensityFiltering_mex", 1, x, 1.5, *args).ravel()
    return d


def main():
    tables = parse_tables()
    np.savez_compressed(os.path.join(HERE, "ref_tables.npz"), **tables)
    kern = make_kernels()
    np.savez_compressed(os.path.join(HERE, "ref_kernels.npz"), **kern)
    print("wrote", sorted(tables), "and", len(kern), "kernel arrays")


if __name__ == "__main__":
    main()
