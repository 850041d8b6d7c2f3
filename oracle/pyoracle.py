"""ctypes binding of the CPU oracle (test infrastructure only).

Loaded by the tests, the smoke check and the benchmark's CPU-baseline leg as
the checker of the CUDA library; never by the library itself.  Builds
oracle/_build/liboracle.so with the Makefile beside this file when missing.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"


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
    ]


class Line(C.Structure):
    _fields_ = [("v", C.c_double * 11)]


class Scalars(C.Structure):
    _fields_ = [("time", C.c_double), ("deltat", C.c_double), ("cfl", C.c_double),
                ("fr", C.c_double * 3), ("corrpx", C.c_double), ("corrpz", C.c_double),
                ("meanpx", C.c_double), ("meanpz", C.c_double), ("istep", C.c_longlong)]


def build(force: bool = False) -> Path:
    # make rebuilds when the sources are newer than the library
    subprocess.run(["make", "-s", "-C", str(HERE)] + (["-B"] if force else []), check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        D = C.POINTER(C.c_double)
        L.orc_create.restype = P
        L.orc_create.argtypes = [C.POINTER(Params), C.c_int]
        L.orc_sizes.argtypes = [C.POINTER(Params), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.orc_destroy.argtypes = [P]
        L.orc_set_field.argtypes = [P, D]
        L.orc_get_field.argtypes = [P, D]
        L.orc_field_len.restype = C.c_longlong
        L.orc_field_len.argtypes = [P]
        L.orc_tables.argtypes = [P, D, D, D, D, D]
        L.orc_buildrhs.argtypes = [P, D, C.c_int]
        L.orc_linsolve.argtypes = [P, C.c_double]
        L.orc_initial_cfl.restype = C.c_double
        L.orc_initial_cfl.argtypes = [P]
        L.orc_initial_flowrate.argtypes = [P]
        L.orc_yintegr.restype = C.c_double
        L.orc_yintegr.argtypes = [P, D]
        L.orc_convolve_plane.restype = C.c_double
        L.orc_convolve_plane.argtypes = [P, C.c_int, D]
        L.orc_get_scalars.argtypes = [P, C.POINTER(Scalars)]
        L.orc_set_scalars.argtypes = [P, C.POINTER(Scalars)]
        L.orc_outstats.argtypes = [P, C.POINTER(Line)]
        L.orc_step.argtypes = [P, C.POINTER(Line)]
        L.orc_start.argtypes = [P, C.POINTER(Line)]
        L.orc_fft.argtypes = [C.c_int, C.c_int, C.c_int, D]
        L.orc_deriv.argtypes = [P, D, D]
        L.orc_deriv2.argtypes = [P, D, D]
        L.orc_set_body_force.argtypes = [P, D]
        L.orc_set_tau.argtypes = [P, D]
        L.orc_fftfit.restype = C.c_int
        L.orc_fftfit.argtypes = [C.c_int]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def params_from(p) -> Params:
    """Params from a channel_gb300.dnsin.DnsIn."""
    return Params(p.nx, p.ny, p.nz, p.alfa0, p.beta0, p.ni, p.a, p.ymin, p.ymax, int(p.cpi), p.cpi_type,
                  p.gamma, p.meanpx, p.meanpz, p.meanflowx, p.meanflowz, p.u0, p.uN, p.deltat, p.cflmax,
                  p.time, p.dt_field, p.dt_save, p.t_max, int(p.time_from_restart), p.nstep, p.npy)


def fft(x: np.ndarray, sign: int) -> np.ndarray:
    """Batched unnormalised FFT over the last axis; sign -1 forward, +1 backward."""
    a = np.ascontiguousarray(x, dtype=np.complex128).copy()
    n = a.shape[-1]
    lib().orc_fft(n, sign, a.size // n, _dp(a.view(np.float64)))
    return a


RK = [(120.0 / 32.0, 2.0, 0.0), (120.0 / 8.0, 50.0 / 8.0, 34.0 / 8.0), (120.0 / 20.0, 90.0 / 20.0, 50.0 / 20.0)]


class Oracle:
    """One oracle run: the reference's module state plus its routines."""

    def __init__(self, p, nthreads: int | None = None):
        self.p = p
        self.nthreads = nthreads or int(os.environ.get("ORACLE_THREADS", os.cpu_count() or 1))
        self._cp = params_from(p)
        self.h = lib().orc_create(C.byref(self._cp), self.nthreads)
        if not self.h:
            raise ValueError("oracle rejected the parameters")
        self.shape = (3, p.nx + 1, 2 * p.nz + 1, p.ny + 3)
        nxd, nzd = C.c_int(), C.c_int()
        lib().orc_sizes(C.byref(self._cp), C.byref(nxd), C.byref(nzd))
        self.nxd, self.nzd = nxd.value, nzd.value

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_field(self, V: np.ndarray):
        a = np.ascontiguousarray(V, dtype=np.complex128)
        assert a.shape == self.shape
        lib().orc_set_field(self.h, _dp(a.view(np.float64)))

    def field(self) -> np.ndarray:
        a = np.empty(self.shape, dtype=np.complex128)
        lib().orc_get_field(self.h, _dp(a.view(np.float64)))
        return a

    def tables(self) -> dict:
        ny = self.p.ny
        y = np.empty(ny + 3)
        der = np.empty((ny - 1, 4, 5))
        wall = np.empty((10, 5))
        bc = np.empty((8, 5))
        d0 = np.empty((ny + 1, 5))
        lib().orc_tables(self.h, _dp(y), _dp(der), _dp(wall), _dp(bc), _dp(d0))
        names = ["d040", "d140", "d240", "d14m1", "d24m1", "d04n", "d14n", "d24n", "d14np1", "d24np1"]
        bnames = ["v0bc", "v0m1bc", "eta0bc", "eta0m1bc", "vnbc", "vnp1bc", "etanbc", "etanp1bc"]
        out = {"y": y, "der": der, "D0mat": d0}
        out.update({n: wall[i] for i, n in enumerate(names)})
        out.update({n: bc[i] for i, n in enumerate(bnames)})
        return out

    def buildrhs(self, ode, compute_cfl: bool):
        o = np.array(ode, dtype=np.float64)
        lib().orc_buildrhs(self.h, _dp(o), int(compute_cfl))

    def linsolve(self, lam: float):
        lib().orc_linsolve(self.h, lam)

    def convolve_plane(self, iy: int):
        out = np.empty((6, self.p.nx + 1, 2 * self.p.nz + 1), dtype=np.complex128)
        c = lib().orc_convolve_plane(self.h, iy, _dp(out.view(np.float64)))
        return out, c

    def set_body_force(self, F):
        if F is None:
            lib().orc_set_body_force(self.h, None)
            return
        a = np.ascontiguousarray(F, dtype=np.complex128)
        assert a.shape == self.shape
        lib().orc_set_body_force(self.h, _dp(a.view(np.float64)))

    def set_tau(self, tau):
        """tau (6, ny-1, nzd, 2nxd) added to the products, or None."""
        if tau is None:
            lib().orc_set_tau(self.h, None)
            return
        a = np.ascontiguousarray(tau, dtype=np.float64)
        assert a.shape == (6, self.p.ny - 1, self.nzd, 2 * self.nxd), a.shape
        lib().orc_set_tau(self.h, _dp(a))

    def deriv(self, f: np.ndarray) -> np.ndarray:
        """Compact first y-derivative of a complex y-line (iy=-1..ny+1)."""
        a = np.ascontiguousarray(f, dtype=np.complex128)
        out = np.empty_like(a)
        lib().orc_deriv(self.h, _dp(a.view(np.float64)), _dp(out.view(np.float64)))
        return out

    def deriv2(self, f: np.ndarray) -> np.ndarray:
        """Compact second y-derivative of a complex y-line (iy=-1..ny+1)."""
        a = np.ascontiguousarray(f, dtype=np.complex128)
        out = np.empty_like(a)
        lib().orc_deriv2(self.h, _dp(a.view(np.float64)), _dp(out.view(np.float64)))
        return out

    def yintegr(self, f: np.ndarray) -> float:
        a = np.ascontiguousarray(f, dtype=np.float64)
        return lib().orc_yintegr(self.h, _dp(a))

    def scalars(self) -> Scalars:
        s = Scalars()
        lib().orc_get_scalars(self.h, C.byref(s))
        return s

    def set_scalars(self, s: Scalars):
        lib().orc_set_scalars(self.h, C.byref(s))

    def start(self) -> np.ndarray:
        ln = Line()
        lib().orc_start(self.h, C.byref(ln))
        return np.array(ln.v)

    def step(self) -> np.ndarray:
        ln = Line()
        lib().orc_step(self.h, C.byref(ln))
        return np.array(ln.v)

    def outstats(self) -> np.ndarray:
        ln = Line()
        lib().orc_outstats(self.h, C.byref(ln))
        return np.array(ln.v)
