"""ctypes bridge from numpy to mexFunction-style entry points.

TEST INFRASTRUCTURE ONLY (oracle side).  Builds mxArrays through the oracle's
MEX shim (``oracle/mexshim``), calls an entry point that has MATLAB's
``mexFunction(nlhs, plhs, nrhs, prhs)`` signature, and converts the outputs
back to numpy.  Used to run the reference's own MEX kernels (compiled into
``oracle/_ref/libref_mex.so`` by ``oracle/build_ref.sh``) and this project's
MEX gateway the way MATLAB would call them.

Conversion rules (MATLAB column-major semantics):
  float64 ndarray -> double array      int32 ndarray -> int32 array
  bool ndarray    -> logical array     python float/int -> double scalar
  list/tuple      -> cell array        scipy.sparse      -> sparse double
  str             -> char array
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

MX_CELL, MX_LOGICAL, MX_CHAR, MX_DOUBLE, MX_SINGLE, MX_INT32 = 1, 3, 4, 6, 7, 12
_CLS_TO_DTYPE = {MX_DOUBLE: np.float64, MX_SINGLE: np.float32, MX_INT32: np.int32,
                 MX_LOGICAL: np.uint8}


class MexError(RuntimeError):
    """Raised when the called entry point signalled mexErrMsgIdAndTxt."""


class MexLib:
    def __init__(self, path: str):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        L = self.lib
        vp = C.c_void_p
        L.shim_new_numeric.restype = vp
        L.shim_new_numeric.argtypes = [C.c_int, C.c_size_t, C.c_size_t, vp]
        L.shim_new_nd.restype = vp
        L.shim_new_nd.argtypes = [C.c_int, C.c_size_t, C.POINTER(C.c_size_t), vp]
        L.shim_new_cell.restype = vp
        L.shim_new_cell.argtypes = [C.c_size_t]
        L.shim_cell_set.argtypes = [vp, C.c_size_t, vp]
        L.shim_new_sparse.restype = vp
        L.shim_new_sparse.argtypes = [C.c_size_t, C.c_size_t, C.c_size_t, vp, vp, vp]
        L.shim_new_string.restype = vp
        L.shim_new_string.argtypes = [C.c_char_p]
        L.shim_class.restype = C.c_int
        L.shim_class.argtypes = [vp]
        L.shim_ndim.restype = C.c_size_t
        L.shim_ndim.argtypes = [vp]
        L.shim_dim.restype = C.c_size_t
        L.shim_dim.argtypes = [vp, C.c_size_t]
        L.shim_data.restype = vp
        L.shim_data.argtypes = [vp]
        L.shim_destroy.argtypes = [vp]
        if hasattr(L, "shim_run_at_exit"):   # absent from libraries built before the shim had it
            L.shim_run_at_exit.argtypes = []
        L.shim_call.restype = C.c_int
        L.shim_call.argtypes = [vp, C.c_int, vp, C.c_int, vp, C.c_char_p, C.c_size_t]

    # -- conversion -------------------------------------------------------
    def _to_mx(self, x):
        L = self.lib
        if isinstance(x, str):
            return L.shim_new_string(x.encode())
        if isinstance(x, (list, tuple)):
            cell = L.shim_new_cell(len(x))
            for i, e in enumerate(x):
                L.shim_cell_set(cell, i, self._to_mx(e))
            return cell
        if hasattr(x, "tocsc") and hasattr(x, "nnz"):
            csc = x.tocsc()
            csc.sort_indices()
            jc = np.ascontiguousarray(csc.indptr, dtype=np.int64)
            ir = np.ascontiguousarray(csc.indices, dtype=np.int64)
            pr = np.ascontiguousarray(csc.data, dtype=np.float64)
            return L.shim_new_sparse(csc.shape[0], csc.shape[1], csc.nnz,
                                     jc.ctypes.data, ir.ctypes.data, pr.ctypes.data)
        if np.isscalar(x):
            a = np.array([[float(x)]])
        else:
            a = np.asarray(x)
        if a.dtype == np.bool_:
            cls, a = MX_LOGICAL, a.astype(np.uint8)
        elif a.dtype == np.int32:
            cls = MX_INT32
        elif a.dtype == np.float32:
            cls = MX_SINGLE
        else:
            cls, a = MX_DOUBLE, a.astype(np.float64)
        if a.ndim == 0:
            a = a.reshape(1, 1)
        if a.ndim == 1:
            a = a.reshape(-1, 1)
        buf = np.asfortranarray(a)
        dims = (C.c_size_t * a.ndim)(*a.shape)
        return L.shim_new_nd(cls, a.ndim, dims, buf.ctypes.data)

    def _from_mx(self, p):
        L = self.lib
        cls = L.shim_class(p)
        nd = L.shim_ndim(p)
        shape = tuple(L.shim_dim(p, i) for i in range(nd))
        dt = _CLS_TO_DTYPE.get(cls)
        if dt is None:
            raise MexError(f"unsupported output class {cls}")
        n = int(np.prod(shape))
        ptr = L.shim_data(p)
        raw = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dt))),
                                    shape=(max(n, 1),))[:n].copy()
        return raw.reshape(shape, order="F")

    def clear(self):
        """What MATLAB's `clear mex` does to the loaded file: runs the function
        it registered with mexAtExit."""
        self.lib.shim_run_at_exit()

    # -- call ---------------------------------------------------------------
    def call(self, name: str, nlhs: int, *args):
        fn = getattr(self.lib, name)
        prhs_list = [self._to_mx(a) for a in args]
        prhs = (C.c_void_p * max(len(prhs_list), 1))(*prhs_list)
        plhs = (C.c_void_p * max(nlhs, 1))()
        err = C.create_string_buffer(1024)
        try:
            rc = self.lib.shim_call(C.cast(fn, C.c_void_p), nlhs, plhs, len(prhs_list), prhs,
                                    err, 1024)
            if rc != 0:
                raise MexError(err.value.decode(errors="replace"))
            outs = [self._from_mx(plhs[i]) for i in range(nlhs)]
        finally:
            for p in prhs_list:
                self.lib.shim_destroy(p)
            for i in range(nlhs):
                if plhs[i]:
                    self.lib.shim_destroy(plhs[i])
        return outs[0] if nlhs == 1 else tuple(outs)


_REF = None


def ref_lib_path() -> str:
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "libref_mex.so")


def ref_lib() -> MexLib | None:
    """The reference's compiled MEX kernels, or None when they are not built
    (they are built only where the reference sources exist)."""
    global _REF
    if _REF is None and os.path.exists(ref_lib_path()):
        _REF = MexLib(ref_lib_path())
    return _REF
