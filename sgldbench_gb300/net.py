"""The learned warm start's U-Net on its own (C ABI ``sgld_net_*``).

No counterpart in the reference.  The SIMP loop uses the same network inside
the library (``TopOpti_GlobalVolumeConstraint(..., learned=True)``); this
wrapper exposes it for tests and experiments: forward pass, loss gradients
and Adam steps on host arrays, parameters in the packed order of
include/sgld_gpu.h.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


class UNet:
    def __init__(self, dims, cin, cout, levels=4, widths=None, seed=0):
        self.lib = _lib.load()
        self.dims = tuple(int(d) for d in dims)   # (ny, nx, nz)
        self.cin, self.cout = int(cin), int(cout)
        self.V = int(np.prod(self.dims))
        h = C.c_void_p()
        w = (C.c_int * len(widths))(*widths) if widths is not None else None
        rc = self.lib.sgld_net_create(self.dims[0], self.dims[1], self.dims[2], self.cin, self.cout, int(levels), w,
                                      C.c_ulonglong(seed), C.byref(h))
        if rc != _lib.SGLD_OK:
            raise _lib.SgldError(rc, "sgld_net_create failed")
        self.h = h

    def _check(self, rc):
        if rc != _lib.SGLD_OK:
            raise _lib.SgldError(rc, self.lib.sgld_net_last_error(self.h).decode())

    @property
    def num_params(self) -> int:
        return int(self.lib.sgld_net_num_params(self.h))

    def get_params(self) -> np.ndarray:
        p = np.empty(self.num_params, np.float32)
        self._check(self.lib.sgld_net_get_params(self.h, p.ctypes.data))
        return p

    def set_params(self, p):
        p = _f32(p)
        assert p.size == self.num_params
        self._check(self.lib.sgld_net_set_params(self.h, p.ctypes.data))

    def forward(self, x) -> np.ndarray:
        x = _f32(x).reshape(self.V, self.cin)
        y = np.empty((self.V, self.cout), np.float32)
        self._check(self.lib.sgld_net_forward(self.h, x.ctypes.data, y.ctypes.data))
        return y

    def grad(self, x, t, m=None):
        x = _f32(x).reshape(self.V, self.cin)
        t = _f32(t).reshape(self.V, self.cout)
        mp = _f32(m).reshape(self.V) if m is not None else None
        loss = C.c_double()
        g = np.empty(self.num_params, np.float32)
        self._check(self.lib.sgld_net_grad(self.h, x.ctypes.data, t.ctypes.data,
                                           mp.ctypes.data if mp is not None else None, C.byref(loss), g.ctypes.data))
        return loss.value, g

    def train_step(self, x, t, m=None, lr=1e-3) -> float:
        x = _f32(x).reshape(self.V, self.cin)
        t = _f32(t).reshape(self.V, self.cout)
        mp = _f32(m).reshape(self.V) if m is not None else None
        loss = C.c_double()
        self._check(self.lib.sgld_net_train_step(self.h, x.ctypes.data, t.ctypes.data,
                                                 mp.ctypes.data if mp is not None else None, C.c_float(lr),
                                                 C.byref(loss)))
        return loss.value

    def close(self):
        if self.h:
            self.lib.sgld_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
