"""The learned subgrid-stress closure (include/chgpu_closure.h).

``Mlp`` binds the pointwise network: parameters, normalisation, resident
training set, gradient, Adam training and inference, all on the tensor
cores of the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .lib import ChannelError, load_library

NIN, NOUT, NPARAMS = 10, 6, 9734
FEATURES = ("du/dx", "du/dy", "du/dz", "dv/dx", "dv/dy", "dv/dz", "dw/dx", "dw/dy", "dw/dz", "y")
STRESSES = ("uu", "vv", "ww", "uv", "vw", "uw")

_FP = C.POINTER(C.c_float)
_DP = C.POINTER(C.c_double)


class Norm(C.Structure):
    _fields_ = [("mu_in", C.c_float * NIN), ("sd_in", C.c_float * NIN),
                ("mu_out", C.c_float * NOUT), ("sd_out", C.c_float * NOUT)]


def _f32(a, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None and a.shape != shape:
        raise ValueError(f"shape {a.shape} != {shape}")
    return a


class Mlp:
    """The 10 -> 64 -> 64 -> 64 -> 6 SiLU network on the current CUDA device."""

    def __init__(self, seed: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        rc = self.lib.chgpu_mlp_create(C.c_ulonglong(seed), C.byref(h))
        if rc != 0:
            if h:
                self.lib.chgpu_mlp_destroy(h)
            raise ChannelError(rc, self.lib.chgpu_mlp_last_error(None).decode())
        self.h = h

    def _check(self, rc: int):
        if rc != 0:
            raise ChannelError(rc, self.lib.chgpu_mlp_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.chgpu_mlp_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self) -> np.ndarray:
        t = np.empty(NPARAMS, np.float32)
        self._check(self.lib.chgpu_mlp_get_params(self.h, t.ctypes.data_as(_FP)))
        return t

    @params.setter
    def params(self, theta):
        t = _f32(theta, (NPARAMS,))
        self._check(self.lib.chgpu_mlp_set_params(self.h, t.ctypes.data_as(_FP)))

    @property
    def norm(self) -> dict:
        n = Norm()
        self._check(self.lib.chgpu_mlp_get_norm(self.h, C.byref(n)))
        return {k: np.array(getattr(n, k)[:], np.float32) for k in ("mu_in", "sd_in", "mu_out", "sd_out")}

    @norm.setter
    def norm(self, d: dict):
        n = Norm()
        for k, size in (("mu_in", NIN), ("sd_in", NIN), ("mu_out", NOUT), ("sd_out", NOUT)):
            v = np.asarray(d[k], np.float32)
            if v.shape != (size,):
                raise ValueError(f"{k}: shape {v.shape} != ({size},)")
            getattr(n, k)[:] = list(map(float, v))
        self._check(self.lib.chgpu_mlp_set_norm(self.h, C.byref(n)))

    def set_data(self, feat, targ):
        """feat (10, n), targ (6, n) in physical units."""
        f = _f32(feat)
        t = _f32(targ)
        if f.ndim != 2 or f.shape[0] != NIN or t.shape != (NOUT, f.shape[1]):
            raise ValueError("need feat (10, n) and targ (6, n)")
        self._check(self.lib.chgpu_mlp_set_data(self.h, f.ctypes.data_as(_FP), t.ctypes.data_as(_FP), f.shape[1]))

    @property
    def data_size(self) -> int:
        return int(self.lib.chgpu_mlp_data_size(self.h))

    def gradient(self, first: int = 0, count: int | None = None):
        """(loss, gradient) on resident points first .. first+count-1."""
        count = self.data_size if count is None else count
        g = np.empty(NPARAMS, np.float32)
        loss = C.c_double()
        self._check(self.lib.chgpu_mlp_gradient(self.h, first, count, g.ctypes.data_as(_FP), C.byref(loss)))
        return loss.value, g

    def train(self, steps: int, batch: int, lr: float) -> np.ndarray:
        """Adam steps on consecutive windows of the resident set; per-step losses."""
        out = np.zeros(max(steps, 1), np.float64)
        self._check(self.lib.chgpu_mlp_train(self.h, steps, batch, C.c_float(lr), out.ctypes.data_as(_DP)))
        return out[:steps]

    def predict(self, feat) -> np.ndarray:
        f = _f32(feat)
        if f.ndim != 2 or f.shape[0] != NIN:
            raise ValueError("need feat (10, n)")
        out = np.empty((NOUT, f.shape[1]), np.float32)
        self._check(self.lib.chgpu_mlp_predict(self.h, f.ctypes.data_as(_FP), f.shape[1], out.ctypes.data_as(_FP)))
        return out
