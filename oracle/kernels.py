"""ctypes bindings of the oracle's C kernels (``oracle/sgld_oracle.c``).

TEST INFRASTRUCTURE ONLY.  ``build()`` compiles the C restatement with gcc
into ``oracle/_build/libsgld_oracle.so`` (done by ``__graft_entry__.build()``
and on first use).  Argument formats follow the reference MEX kernels: 1-based
int32 tables stored column-major, interleaved DOF vectors for K*u and n-by-3
arrays for the transfer operators.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libsgld_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "sgld_oracle.c")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(_SO), exist_ok=True)
        tmp = _SO + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11",
                               "-o", tmp, src, "-lm"])
        os.replace(tmp, _SO)
    return _SO


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _i32(a):
    return np.asfortranarray(np.asarray(a, dtype=np.int32))


def _f64(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def _colors(colors):
    offs = np.zeros(len(colors) + 1, dtype=np.int64)
    offs[1:] = np.cumsum([len(c) for c in colors])
    idx = np.concatenate([np.asarray(c, dtype=np.int32).reshape(-1) for c in colors]) if colors else \
        np.zeros(0, np.int32)
    return np.ascontiguousarray(idx, dtype=np.int32), offs


_I64 = C.c_int64


def kbyu(u, eNodMat, Ke, E, colors):
    u, en, Ke, E = _f64(u).reshape(-1), _i32(eNodMat), _f64(Ke), _f64(E).reshape(-1)
    ci, co = _colors(colors)
    y = np.zeros(u.size)
    lib().orc_kbyu(_p(u), _p(en), _I64(en.shape[0]), _p(Ke), _p(E), _p(ci), _p(co), C.c_int(len(colors)),
                   _p(y), _I64(u.size))
    return y


def restriction(rF, transferMat, RI, eNodMat, nCoarse, nGhost, solidMap, coeffi, colors):
    rF, tm, RI, en = _f64(rF), _i32(transferMat), _f64(RI), _i32(eNodMat)
    sm, cf = _i32(solidMap).reshape(-1), _f64(coeffi).reshape(-1)
    ci, co = _colors(colors)
    out = np.zeros((int(nCoarse), 3), order="F")
    lib().orc_restriction(_p(rF), _I64(rF.shape[0]), _p(tm), C.c_int(tm.shape[0]), _p(RI), _p(en),
                          _I64(en.shape[0]), _I64(nCoarse), _I64(nGhost), _p(sm), _p(cf), _p(ci), _p(co),
                          C.c_int(len(colors)), _p(out))
    return out


def interpolation(xC, transferMat, RI, eNodMat, nFine, nGhost, solidMap, coeffi, colors):
    xC, tm, RI, en = _f64(xC), _i32(transferMat), _f64(RI), _i32(eNodMat)
    sm, cf = _i32(solidMap).reshape(-1), _f64(coeffi).reshape(-1)
    ci, co = _colors(colors)
    out = np.zeros((int(nFine), 3), order="F")
    lib().orc_interpolation(_p(xC), _I64(xC.shape[0]), _p(tm), C.c_int(tm.shape[0]), _p(RI), _p(en),
                            _I64(en.shape[0]), _I64(nFine), _I64(nGhost), _p(sm), _p(cf), _p(ci), _p(co),
                            C.c_int(len(colors)), _p(out))
    return out


def unit_compliance(U, eNodMat, Ke):
    U, en, Ke = _f64(U).reshape(-1), _i32(eNodMat), _f64(Ke)
    ce = np.zeros(en.shape[0])
    lib().orc_unit_compliance(_p(U), _p(en), _I64(en.shape[0]), _p(Ke), _p(ce))
    return ce


def assemble_from_finest(Ke, E, eum, P, lmap, nProjNodes):
    Ke, E, eum, P, lm = _f64(Ke), _f64(E).reshape(-1), _i32(eum), _f64(P), _i32(lmap).reshape(-1)
    Mc, nq = eum.shape
    Ks = np.zeros((24, 24, Mc), order="F")
    lib().orc_assemble_finest(_p(Ke), _p(E), _p(eum), _I64(Mc), C.c_int(nq), _p(P), _p(lm),
                              C.c_int(nProjNodes), _p(Ks))
    return Ks


def assemble_from_nonfinest(KsPrev, eum, P, lmap, nProjNodes):
    Kp, eum, P, lm = _f64(KsPrev), _i32(eum), _f64(P), _i32(lmap).reshape(-1)
    Mc, nq = eum.shape
    Ks = np.zeros((24, 24, Mc), order="F")
    lib().orc_assemble_nonfinest(_p(Kp), _p(eum), _I64(Mc), C.c_int(nq), _p(P), _p(lm),
                                 C.c_int(nProjNodes), _p(Ks))
    return Ks


def density_filter(x, rmin, eleMapForward, resX, resY, resZ):
    """x=None returns the weight sums Hs (TopOpti_SetupDensityFilter_mex)."""
    emf = _i32(eleMapForward).reshape(-1)
    n = int((emf > 0).sum())
    y = np.zeros(n)
    xp = _f64(x).reshape(-1) if x is not None else None
    lib().orc_density_filter(_p(xp) if xp is not None else None, C.c_double(rmin), _p(emf),
                             C.c_int(resX), C.c_int(resY), C.c_int(resZ), _p(y))
    return y
