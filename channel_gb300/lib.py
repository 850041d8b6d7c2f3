"""ctypes binding of libchgpu.so (include/chgpu.h).

``Channel`` mirrors the module procedures channel.f90 calls on its hot path:
``start`` (the start-up CFL pass, flow rate and first outstats,
channel.f90:64-116), ``buildrhs(ODE, compute_cfl)`` (dnsdata.f90:611),
``linsolve(lambda)`` (linsolve_blocking.inc:3), ``outstats()``
(dnsdata.f90:853) and ``step()`` (one whole time-loop iteration,
channel.f90:118-167, replayed from a CUDA graph).  Fields cross the boundary
in the restart-file layout: numpy complex128 of shape (3, nx+1, 2nz+1, ny+3).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from .dnsin import DnsIn

PKG = Path(__file__).resolve().parent
RK = [(120.0 / 32.0, 2.0, 0.0), (120.0 / 8.0, 50.0 / 8.0, 34.0 / 8.0), (120.0 / 20.0, 90.0 / 20.0, 50.0 / 20.0)]
FP64, MIXED, FP64DD = 0, 1, 2


class ChannelError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("alfa0", C.c_double), ("beta0", C.c_double), ("ni", C.c_double),
        ("a", C.c_double), ("ymin", C.c_double), ("ymax", C.c_double),
        ("cpi", C.c_int), ("cpi_type", C.c_int), ("gamma", C.c_double),
        ("meanpx", C.c_double), ("meanpz", C.c_double),
        ("meanflowx", C.c_double), ("meanflowz", C.c_double),
        ("u0", C.c_double), ("uN", C.c_double),
        ("deltat", C.c_double), ("cflmax", C.c_double), ("time", C.c_double),
        ("dt_field", C.c_double), ("dt_save", C.c_double), ("t_max", C.c_double),
        ("time_from_restart", C.c_int), ("nstep", C.c_longlong), ("npy", C.c_int),
        ("precision", C.c_int),
    ]


class Stats(C.Structure):
    _fields_ = [("line", C.c_double * 11), ("fr", C.c_double * 3), ("corrpx", C.c_double), ("corrpz", C.c_double),
                ("meanpx", C.c_double), ("meanpz", C.c_double), ("cfl", C.c_double), ("deltat", C.c_double),
                ("time", C.c_double), ("istep", C.c_longlong)]


# name -> (restype, argtypes), one per declaration in include/chgpu.h
class ExportOpts(C.Structure):
    _fields_ = [("fluct_only", C.c_int), ("part", C.c_int), ("z_threshold", C.c_int), ("undersample", C.c_float)]


EXPORT_PART = {"all": 0, "large": 1, "small": 2}

_P = C.c_void_p
_DP = C.POINTER(C.c_double)
_FP = C.POINTER(C.c_float)
SIGNATURES = {
    "chgpu_create": (C.c_int, [C.POINTER(Params), C.POINTER(C.c_void_p)]),
    "chgpu_destroy": (C.c_int, [_P]),
    "chgpu_upload_field": (C.c_int, [_P, _DP]),
    "chgpu_download_field": (C.c_int, [_P, _DP]),
    "chgpu_field_doubles": (C.c_size_t, [_P]),
    "chgpu_start": (C.c_int, [_P, C.c_double, C.c_double, C.POINTER(Stats)]),
    "chgpu_set_wall_velocity": (C.c_int, [_P, C.c_double, C.c_double]),
    "chgpu_buildrhs": (C.c_int, [_P, _DP, C.c_int]),
    "chgpu_linsolve": (C.c_int, [_P, C.c_double]),
    "chgpu_outstats": (C.c_int, [_P, C.POINTER(Stats)]),
    "chgpu_step": (C.c_int, [_P, C.POINTER(Stats)]),
    "chgpu_get_stats": (C.c_int, [_P, C.POINTER(Stats)]),
    "chgpu_synchronize": (C.c_int, [_P]),
    "chgpu_stream": (C.c_void_p, [_P]),
    "chgpu_launch_count": (C.c_longlong, [_P]),
    "chgpu_last_error": (C.c_char_p, [_P]),
    "chgpu_set_profiling": (C.c_int, [_P, C.c_int]),
    "chgpu_kernel_times": (C.c_int, [_P, _DP, C.POINTER(C.c_longlong)]),
    "chgpu_kernel_kind_name": (C.c_char_p, [C.c_int]),
    "chgpu_set_body_force": (C.c_int, [_P, _DP]),
    "chgpu_ensemble_create": (C.c_int, [C.POINTER(Params), C.c_int, C.POINTER(C.c_void_p)]),
    "chgpu_ensemble_destroy": (C.c_int, [_P]),
    "chgpu_ensemble_size": (C.c_int, [_P]),
    "chgpu_ensemble_member": (C.c_void_p, [_P, C.c_int]),
    "chgpu_ensemble_step": (C.c_int, [_P, C.POINTER(Stats)]),
    "chgpu_ensemble_synchronize": (C.c_int, [_P]),
    "chgpu_ensemble_stream": (C.c_void_p, [_P]),
    "chgpu_ensemble_last_error": (C.c_char_p, [_P]),
    "chgpu_autotune": (C.c_int, [_P]),
    "chgpu_tiles": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "chgpu_set_tiles": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "chgpu_set_step_halves": (C.c_int, [_P, C.c_int]),
    "chgpu_set_wait_limit": (C.c_int, [_P, C.c_int]),
    "chgpu_export_dims": (C.c_int, [_P, C.c_float, C.POINTER(C.c_int)]),
    "chgpu_export_physical": (C.c_int, [_P, C.POINTER(ExportOpts), _DP]),
    "chgpu_stats_reset": (C.c_int, [_P]),
    "chgpu_stats_accumulate": (C.c_int, [_P]),
    "chgpu_profiles": (C.c_int, [_P, _DP, _DP, C.POINTER(C.c_longlong)]),
    "chgpu_snapshot_async": (C.c_int, [_P]),
    "chgpu_snapshot_wait": (C.c_int, [_P, C.POINTER(_DP)]),
    "chgpu_linsolve_noalloc": (C.c_int, [C.POINTER(Params), C.c_double, C.c_void_p, _DP, C.c_void_p,
                                         C.c_char_p, C.c_size_t]),
    "chgpu_measure_peaks": (C.c_int, [_DP, _DP, _DP, C.c_char_p, C.c_size_t]),
    "chgpu_pivot_reciprocal": (C.c_int, [_DP, _DP, C.c_size_t, C.c_char_p, C.c_size_t]),
    "chgpu_tke_reset": (C.c_int, [_P, _DP]),
    "chgpu_tke_accumulate": (C.c_int, [_P, _DP]),
    "chgpu_tke_result": (C.c_int, [_P, C.c_int, _DP, _DP, _DP, C.POINTER(C.c_longlong)]),
    # include/chgpu_closure.h
    "chgpu_mlp_create": (C.c_int, [C.c_ulonglong, C.POINTER(C.c_void_p)]),
    "chgpu_mlp_destroy": (C.c_int, [_P]),
    "chgpu_mlp_last_error": (C.c_char_p, [_P]),
    "chgpu_mlp_set_params": (C.c_int, [_P, _FP]),
    "chgpu_mlp_get_params": (C.c_int, [_P, _FP]),
    "chgpu_mlp_set_norm": (C.c_int, [_P, C.c_void_p]),
    "chgpu_mlp_get_norm": (C.c_int, [_P, C.c_void_p]),
    "chgpu_mlp_set_data": (C.c_int, [_P, _FP, _FP, C.c_longlong]),
    "chgpu_mlp_data_size": (C.c_longlong, [_P]),
    "chgpu_mlp_gradient": (C.c_int, [_P, C.c_longlong, C.c_longlong, _FP, _DP]),
    "chgpu_mlp_train": (C.c_int, [_P, C.c_int, C.c_longlong, C.c_float, _DP]),
    "chgpu_mlp_predict": (C.c_int, [_P, _FP, C.c_longlong, _FP]),
    "chgpu_closure_dims": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "chgpu_closure_attach": (C.c_int, [_P, _P, C.c_int]),
    "chgpu_closure_set_tau": (C.c_int, [_P, _FP]),
    "chgpu_closure_features": (C.c_int, [_P, _FP]),
    "chgpu_closure_physical": (C.c_int, [_P, _DP, C.c_int, _FP]),
    "chgpu_products": (C.c_int, [_P, _DP]),
}
NKINDS = 6


def library_path() -> Path:
    return Path(os.environ.get("CHGPU_LIB", PKG / "_build" / "libchgpu.so"))


_lib = None


def load_library():
    """Load libchgpu.so; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is None:
        path = library_path()
        if not path.exists():
            raise FileNotFoundError(f"{path} not built: run `python -m channel_gb300.build`")
        L = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def measure_peaks(copy: bool = True) -> dict:
    """FP64 / FP32 FMA throughput (TFLOP/s) and device copy rate (GB/s) of
    the current device (chgpu_measure_peaks)."""
    L = load_library()
    f64, f32, cp = C.c_double(), C.c_double(), C.c_double()
    err = C.create_string_buffer(256)
    rc = L.chgpu_measure_peaks(C.byref(f64), C.byref(f32), C.byref(cp) if copy else None, err, 256)
    if rc != 0:
        raise ChannelError(rc, err.value.decode())
    out = {"fp64_tflops": f64.value, "fp32_tflops": f32.value}
    if copy:
        out["copy_gbs"] = cp.value
    return out


def pivot_reciprocal(x) -> np.ndarray:
    """1/x as the banded solves form their pivot reciprocals
    (chgpu_pivot_reciprocal), for an array of float64 values."""
    L = load_library()
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    err = C.create_string_buffer(256)
    rc = L.chgpu_pivot_reciprocal(x.ctypes.data_as(_DP), y.ctypes.data_as(_DP), x.size, err, 256)
    if rc != 0:
        raise ChannelError(rc, err.value.decode())
    return y


def params_struct(p: DnsIn, precision: int = FP64) -> Params:
    return Params(p.nx, p.ny, p.nz, p.alfa0, p.beta0, p.ni, p.a, p.ymin, p.ymax, int(p.cpi), p.cpi_type, p.gamma,
                  p.meanpx, p.meanpz, p.meanflowx, p.meanflowz, p.u0, p.uN, p.deltat, p.cflmax, p.time,
                  p.dt_field, p.dt_save, p.t_max, int(p.time_from_restart), p.nstep, p.npy, precision)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def _precision(precision: str | int) -> int:
    return {"fp64": FP64, "mixed": MIXED, "fp64dd": FP64DD}[precision] if isinstance(precision, str) else precision


class Channel:
    """One channel run on the current CUDA device."""

    def __init__(self, p: DnsIn, precision: str | int = "fp64", _handle=None):
        self.lib = load_library()
        self.p = p
        prec = _precision(precision)
        self.precision = prec
        self._params = params_struct(p, prec)
        self._owned = _handle is None
        if _handle is None:
            h = C.c_void_p()
            rc = self.lib.chgpu_create(C.byref(self._params), C.byref(h))
            if rc != 0:
                raise ChannelError(rc, self.lib.chgpu_last_error(None).decode())
        else:
            h = C.c_void_p(_handle)
        self.h = h
        self.shape = (3, p.nx + 1, 2 * p.nz + 1, p.ny + 3)

    def _check(self, rc: int):
        if rc != 0:
            raise ChannelError(rc, self.lib.chgpu_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            if self._owned:
                self.lib.chgpu_destroy(self.h)
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

    def upload(self, V: np.ndarray):
        a = np.ascontiguousarray(V, dtype=np.complex128)
        if a.shape != self.shape:
            raise ValueError(f"field shape {a.shape} != {self.shape}")
        self._check(self.lib.chgpu_upload_field(self.h, _dp(a.view(np.float64))))

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        a = out if out is not None else np.empty(self.shape, dtype=np.complex128)
        self._check(self.lib.chgpu_download_field(self.h, _dp(a.view(np.float64))))
        return a

    def start(self, time: float | None = None, deltat: float | None = None) -> np.ndarray:
        st = Stats()
        t = self.p.time if time is None else time
        dt = self.p.deltat if deltat is None else deltat
        self._check(self.lib.chgpu_start(self.h, t, dt, C.byref(st)))
        return np.array(st.line)

    def set_wall_velocity(self, u0: float, uN: float):
        self._check(self.lib.chgpu_set_wall_velocity(self.h, u0, uN))

    def buildrhs(self, ode, compute_cfl: bool):
        o = np.array(ode, dtype=np.float64)
        self._check(self.lib.chgpu_buildrhs(self.h, _dp(o), int(compute_cfl)))

    def linsolve(self, lam: float):
        self._check(self.lib.chgpu_linsolve(self.h, lam))

    def outstats(self) -> Stats:
        st = Stats()
        self._check(self.lib.chgpu_outstats(self.h, C.byref(st)))
        return st

    def step(self, sync: bool = True) -> np.ndarray | None:
        if not sync:
            self._check(self.lib.chgpu_step(self.h, None))
            return None
        st = Stats()
        self._check(self.lib.chgpu_step(self.h, C.byref(st)))
        return np.array(st.line)

    def stats(self) -> Stats:
        st = Stats()
        self._check(self.lib.chgpu_get_stats(self.h, C.byref(st)))
        return st

    def synchronize(self):
        self._check(self.lib.chgpu_synchronize(self.h))

    def set_profiling(self, on: bool):
        self._check(self.lib.chgpu_set_profiling(self.h, int(on)))

    def kernel_times(self) -> dict:
        """{kernel kind: (summed device ms, launches)} since profiling was enabled."""
        ms = np.zeros(NKINDS)
        n = (C.c_longlong * NKINDS)()
        self._check(self.lib.chgpu_kernel_times(self.h, _dp(ms), n))
        return {self.lib.chgpu_kernel_kind_name(k).decode(): (float(ms[k]), int(n[k])) for k in range(NKINDS)}

    def autotune(self) -> tuple:
        """Times the transform tiles on this handle and keeps the fastest;
        returns them (see tiles())."""
        self._check(self.lib.chgpu_autotune(self.h))
        return self.tiles()

    def tiles(self) -> tuple:
        """(z columns, x rows, x-row variant, z threads, x threads, solve form,
        step halves)."""
        t = (C.c_int * 7)()
        self._check(self.lib.chgpu_tiles(self.h, t))
        return tuple(t)

    def set_tiles(self, tiles) -> None:
        """Tiles of tiles(); five values keep this handle's solve form and halves."""
        tiles = tuple(tiles)
        if len(tiles) == 5:
            tiles = tiles + self.tiles()[5:]
        self._check(self.lib.chgpu_set_tiles(self.h, (C.c_int * 7)(*tiles)))

    def set_wait_limit(self, polls: int) -> None:
        """Poll count of the first device-side wait (generic z kernels); < 0: default."""
        self._check(self.lib.chgpu_set_wait_limit(self.h, polls))

    def set_step_halves(self, halves: int) -> None:
        """1: the step on one stream; 2: rhs / solve split in two kx halves on two streams."""
        self._check(self.lib.chgpu_set_step_halves(self.h, halves))

    def export_dims(self, undersample: float = 1.0) -> tuple[int, int, int]:
        d = (C.c_int * 3)()
        self._check(self.lib.chgpu_export_dims(self.h, undersample, d))
        return d[0], d[1], d[2]

    def export_physical(self, fluct_only: bool = False, part: str = "all", z_threshold: int = 0,
                        undersample: float = 1.0) -> np.ndarray:
        """The current field in physical space as the exporter writes it:
        vec(3, nxtot, 0:ny, nztot) in Fortran order = an array
        [nztot][ny+1][nxtot][3]."""
        nxtot, nytot, nztot = self.export_dims(undersample)
        out = np.empty((nztot, nytot, nxtot, 3))
        o = ExportOpts(int(bool(fluct_only)), EXPORT_PART[part], int(z_threshold), undersample)
        self._check(self.lib.chgpu_export_physical(self.h, C.byref(o), _dp(out)))
        return out

    def set_body_force(self, F: np.ndarray | None):
        """Body force in the restart-file layout (None switches it off)."""
        if F is None:
            self._check(self.lib.chgpu_set_body_force(self.h, None))
            return
        a = np.ascontiguousarray(F, dtype=np.complex128)
        if a.shape != self.shape:
            raise ValueError(f"force shape {a.shape} != {self.shape}")
        self._check(self.lib.chgpu_set_body_force(self.h, _dp(a.view(np.float64))))

    def stats_reset(self):
        self._check(self.lib.chgpu_stats_reset(self.h))

    def stats_accumulate(self):
        self._check(self.lib.chgpu_stats_accumulate(self.h))

    def profiles(self):
        """(mean, var, nsamples): mean and variance profiles, arrays (3, ny+3)."""
        n = 3 * (self.p.ny + 3)
        mean, var = np.empty(n), np.empty(n)
        ns = C.c_longlong()
        self._check(self.lib.chgpu_profiles(self.h, _dp(mean), _dp(var), C.byref(ns)))
        return mean.reshape(3, -1), var.reshape(3, -1), int(ns.value)

    def tke_reset(self, mean_u: np.ndarray, mean_w: np.ndarray, mean_p: np.ndarray | None = None):
        """Reynolds-stress budget spectra: clears the sums; the mean profiles
        (ny+3 each) are removed from every sample."""
        ny3 = self.p.ny + 3
        m = np.zeros(3 * ny3)
        m[:ny3] = mean_u
        m[ny3:2 * ny3] = mean_w
        if mean_p is not None:
            m[2 * ny3:] = mean_p
        self._check(self.lib.chgpu_tke_reset(self.h, _dp(m)))

    def tke_accumulate(self, pressure: np.ndarray | None = None):
        """One sample of the current field; pressure (nx+1, 2nz+1, ny+3) complex or None."""
        if pressure is None:
            self._check(self.lib.chgpu_tke_accumulate(self.h, None))
            return
        a = np.ascontiguousarray(pressure, dtype=np.complex128)
        assert a.shape == (self.p.nx + 1, 2 * self.p.nz + 1, self.p.ny + 3)
        # C order of (nx+1, 2nz+1, ny+3) is the restart-file order (iy fastest)
        self._check(self.lib.chgpu_tke_accumulate(self.h, _dp(a.view(np.float64))))

    def tke_result(self, timestwo: bool = False):
        """(mean (7, ny+3), spectra (6, 10, 2nz+1, ny+3), profiles (6, 10, ny+3), samples)."""
        ny3, nzt = self.p.ny + 3, 2 * self.p.nz + 1
        mean = np.empty(7 * ny3)
        sp = np.empty(60 * nzt * ny3)
        pr = np.empty(60 * ny3)
        n = C.c_longlong()
        self._check(self.lib.chgpu_tke_result(self.h, int(timestwo), _dp(mean), _dp(sp), _dp(pr), C.byref(n)))
        return (mean.reshape((7, ny3), order="F"), sp.reshape((6, 10, nzt, ny3), order="F"),
                pr.reshape((6, 10, ny3), order="F"), n.value)

    def snapshot_async(self):
        self._check(self.lib.chgpu_snapshot_async(self.h))

    def snapshot_wait(self) -> np.ndarray:
        ptr = _DP()
        self._check(self.lib.chgpu_snapshot_wait(self.h, C.byref(ptr)))
        n = int(np.prod(self.shape))
        return np.ctypeslib.as_array(ptr, shape=(2 * n,)).view(np.complex128).reshape(self.shape).copy()

    # ---- learned closure (include/chgpu_closure.h) ----
    def closure_dims(self) -> tuple[int, int, int]:
        """(2 nxd, nzd, ny-1): the closure points, x fastest."""
        d = (C.c_int * 3)()
        self._check(self.lib.chgpu_closure_dims(self.h, d))
        return tuple(d)

    def closure_points(self) -> int:
        a, b, c = self.closure_dims()
        return a * b * c

    def products(self) -> np.ndarray:
        """The six product spectra of the current field, (6, nx+1, 2nz+1, ny+3) complex128."""
        out = np.empty((6,) + self.shape[1:], dtype=np.complex128)
        self._check(self.lib.chgpu_products(self.h, _dp(out.view(np.float64))))
        return out

    def closure_features(self) -> np.ndarray:
        out = np.empty((10, self.closure_points()), dtype=np.float32)
        self._check(self.lib.chgpu_closure_features(self.h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def closure_physical(self, spec: np.ndarray) -> np.ndarray:
        """Physical values at the closure points of (3|6|9, nx+1, 2nz+1, ny+3) spectra."""
        a = np.ascontiguousarray(spec, dtype=np.complex128)
        if a.shape[1:] != self.shape[1:] or a.shape[0] not in (3, 6, 9):
            raise ValueError(f"spectra shape {a.shape}")
        out = np.empty((a.shape[0], self.closure_points()), dtype=np.float32)
        self._check(self.lib.chgpu_closure_physical(self.h, _dp(a.view(np.float64)), a.shape[0],
                                                    out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def closure_set_tau(self, tau: np.ndarray | None):
        if tau is None:
            self._check(self.lib.chgpu_closure_set_tau(self.h, None))
            return
        t = np.ascontiguousarray(tau, dtype=np.float32)
        if t.shape != (6, self.closure_points()):
            raise ValueError(f"tau shape {t.shape}")
        self._check(self.lib.chgpu_closure_set_tau(self.h, t.ctypes.data_as(C.POINTER(C.c_float))))

    def closure_attach(self, mlp, enable: bool = True):
        """Evaluate the network in every convolution pass (enable=False: the plain solver)."""
        self._closure_mlp = mlp  # keeps the network alive while attached
        self._check(self.lib.chgpu_closure_attach(self.h, mlp.h if mlp is not None else None, int(enable)))

    @property
    def launches(self) -> int:
        return int(self.lib.chgpu_launch_count(self.h))

    @property
    def stream(self) -> int:
        return int(self.lib.chgpu_stream(self.h) or 0)


class Ensemble:
    """Independent channel runs (uneven sizes allowed) advanced together: one
    graph launch per step.  members[i] is a Channel view of member i (upload,
    start, download, statistics, tiles); closing the ensemble frees them."""

    def __init__(self, params: list, precision: str | int | list = "mixed"):
        self.lib = load_library()
        precs = precision if isinstance(precision, list) else [precision] * len(params)
        arr = (Params * len(params))(*[params_struct(p, _precision(q)) for p, q in zip(params, precs)])
        e = C.c_void_p()
        rc = self.lib.chgpu_ensemble_create(arr, len(params), C.byref(e))
        if rc != 0:
            raise ChannelError(rc, self.lib.chgpu_ensemble_last_error(None).decode())
        self.e = e
        self.members = [Channel(p, q, _handle=self.lib.chgpu_ensemble_member(e, i))
                        for i, (p, q) in enumerate(zip(params, precs))]
        self._stats = (Stats * len(params))()

    def _check(self, rc: int):
        if rc != 0:
            raise ChannelError(rc, self.lib.chgpu_ensemble_last_error(self.e).decode())

    def step(self, sync: bool = True):
        """One RK3 step of every member; with sync, the Runtimedata records."""
        if not sync:
            self._check(self.lib.chgpu_ensemble_step(self.e, None))
            return None
        self._check(self.lib.chgpu_ensemble_step(self.e, self._stats))
        return [np.array(s.line) for s in self._stats]

    def synchronize(self):
        self._check(self.lib.chgpu_ensemble_synchronize(self.e))

    @property
    def stream(self) -> int:
        return self.lib.chgpu_ensemble_stream(self.e)

    def close(self):
        if getattr(self, "e", None):
            for m in self.members:
                m.close()
            self.lib.chgpu_ensemble_destroy(self.e)
            self.e = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
