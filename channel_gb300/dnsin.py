"""dns.in reader/writer (the reference's twelve-line, list-directed input).

Follows ``read_dnsin`` (dnsdata.f90:98-125): line 1 ``nx ny nz``, line 2
``alfa0 beta0``, line 3 the Reynolds number (stored inverted as ``ni``),
line 4 ``a ymin ymax``, line 5 ``CPI CPI_type gamma``, line 6 ``meanpx
meanpz``, line 7 ``meanflowx meanflowz``, line 8 ``u0 uN``, line 9 ``deltat
cflmax time``, line 10 ``dt_field dt_save t_max time_from_restart``, line 11
``nstep``, line 12 ``npy``.  Values after the ones a line needs (the
``! comment`` text) are ignored, as a list-directed READ ignores them.
The padded FFT sizes follow dnsdata.f90:110-114 with ``fftFIT``
(ffts.f90:78-86).
"""
from __future__ import annotations

import dataclasses
import math
import re
from pathlib import Path

_COUNTS = [3, 2, 1, 3, 3, 2, 2, 2, 3, 4, 1, 1]


def fft_fit(n: int) -> bool:
    """True when n is a power of two or three times one (ffts.f90:78-86)."""
    j = n
    while j % 2 == 0:
        j >>= 1
    return j in (1, 3)


def padded_sizes(nx: int, nz: int) -> tuple[int, int]:
    """(nxd, nzd) as read_dnsin computes them (dnsdata.f90:110-114)."""
    nxd = 3 * (nx + 1) // 2
    nzd = 3 * nz
    while not fft_fit(nxd):
        nxd += 1
    while not fft_fit(nzd):
        nzd += 1
    return nxd, nzd


def _fortran_real(tok: str) -> float:
    return float(tok.replace("d", "e").replace("D", "E"))


def _fortran_logical(tok: str) -> bool:
    t = tok.strip().lstrip(".").upper()
    if t.startswith("T"):
        return True
    if t.startswith("F"):
        return False
    raise ValueError(f"not a Fortran logical: {tok!r}")


@dataclasses.dataclass
class DnsIn:
    nx: int
    ny: int
    nz: int
    alfa0: float
    beta0: float
    re: float  # line 3 as written; ni = 1/re
    a: float
    ymin: float
    ymax: float
    cpi: bool = False
    cpi_type: int = 0
    gamma: float = 0.0
    meanpx: float = 0.0
    meanpz: float = 0.0
    meanflowx: float = 0.0
    meanflowz: float = 0.0
    u0: float = 0.0
    uN: float = 0.0
    deltat: float = 0.0
    cflmax: float = 0.0
    time: float = 0.0
    dt_field: float = 1.0e9
    dt_save: float = -1.0
    t_max: float = 1.0e9
    time_from_restart: bool = False
    nstep: int = 1
    npy: int = 1

    @property
    def ni(self) -> float:
        """Kinematic viscosity as the solver stores it (ni=1/ni, dnsdata.f90:115)."""
        return 1 / self.re

    @property
    def nxd(self) -> int:
        return padded_sizes(self.nx, self.nz)[0]

    @property
    def nzd(self) -> int:
        return padded_sizes(self.nx, self.nz)[1]

    def grid_points(self) -> int:
        """Physical grid points (2nx+1)(ny+1)(2nz+1)."""
        return (2 * self.nx + 1) * (self.ny + 1) * (2 * self.nz + 1)

    def spectral_points(self) -> int:
        """Stored spectral unknowns per component (nx+1)(2nz+1)(ny+3)."""
        return (self.nx + 1) * (2 * self.nz + 1) * (self.ny + 3)

    def y(self):
        """Wall-normal grid y(iy), iy=-1..ny+1 (dnsdata.f90:153)."""
        import numpy as np

        iy = np.arange(-1, self.ny + 2, dtype=np.float64)
        return self.ymin + 0.5 * (self.ymax - self.ymin) * (
            np.tanh(self.a * (2.0 * iy / float(self.ny) - 1)) / math.tanh(self.a) + 1
        )


def parse(text: str) -> DnsIn:
    lines = [ln for ln in text.splitlines()]
    vals: list[list[str]] = []
    li = 0
    for need in _COUNTS:
        toks: list[str] = []
        while len(toks) < need:
            if li >= len(lines):
                raise ValueError("dns.in: unexpected end of file")
            raw = lines[li].split("!")[0]
            li += 1
            toks.extend(t for t in re.split(r"[,\s]+", raw.strip()) if t)
        vals.append(toks[:need])
    (nx, ny, nz), (al, be), (re_,), (a, ymin, ymax), (cpi, cpit, gam), (mpx, mpz), (mfx, mfz), (u0, un), \
        (dt, cfl, t0), (dtf, dts, tmax, tfr), (nstep,), (npy,) = vals
    return DnsIn(
        nx=int(nx), ny=int(ny), nz=int(nz), alfa0=_fortran_real(al), beta0=_fortran_real(be),
        re=_fortran_real(re_), a=_fortran_real(a), ymin=_fortran_real(ymin), ymax=_fortran_real(ymax),
        cpi=_fortran_logical(cpi), cpi_type=int(cpit), gamma=_fortran_real(gam),
        meanpx=_fortran_real(mpx), meanpz=_fortran_real(mpz), meanflowx=_fortran_real(mfx),
        meanflowz=_fortran_real(mfz), u0=_fortran_real(u0), uN=_fortran_real(un),
        deltat=_fortran_real(dt), cflmax=_fortran_real(cfl), time=_fortran_real(t0),
        dt_field=_fortran_real(dtf), dt_save=_fortran_real(dts), t_max=_fortran_real(tmax),
        time_from_restart=_fortran_logical(tfr), nstep=int(nstep), npy=int(npy),
    )


def read(path) -> DnsIn:
    return parse(Path(path).read_text())


def _r(x: float) -> str:
    return repr(float(x))


def _l(b: bool) -> str:
    return ".TRUE." if b else ".FALSE."


def format_dnsin(p: DnsIn) -> str:
    rows = [
        (f"{p.nx} {p.ny} {p.nz}", "nx, ny, nz"),
        (f"{_r(p.alfa0)} {_r(p.beta0)}", "alfa0 beta0"),
        (f"{_r(p.re)}", "ni"),
        (f"{_r(p.a)} {_r(p.ymin)} {_r(p.ymax)}", "a, ymin, ymax"),
        (f"{_l(p.cpi)} {p.cpi_type} {_r(p.gamma)}", "CPI, CPItype, gamma"),
        (f"{_r(p.meanpx)} {_r(p.meanpz)}", "meanpx, meanpz"),
        (f"{_r(p.meanflowx)} {_r(p.meanflowz)}", "meanflowx meanflowz"),
        (f"{_r(p.u0)} {_r(p.uN)}", "u0 uN"),
        (f"{_r(p.deltat)} {_r(p.cflmax)} {_r(p.time)}", "deltat, cflmax, time"),
        (f"{_r(p.dt_field)} {_r(p.dt_save)} {_r(p.t_max)} {_l(p.time_from_restart)}",
         "dt_field, dt_save, t_max, time_from_restart"),
        (f"{p.nstep}", "nstep"),
        (f"{p.npy}", "npy (no. processes y)"),
    ]
    return "".join(f"{v:<40} ! {c}\n" for v, c in rows)


def write(path, p: DnsIn) -> None:
    Path(path).write_text(format_dnsin(p))


# The channel workloads these tools are exercised on (sizes and physics).
def workload(name: str) -> DnsIn:
    """Named workloads: 'small' 32x64x32 fixed dt, 'retau180' 127x192x127,
    'retau550' 383x384x383, 'coarse' 47x96x47 on the Re_tau 550 domain; 'probe768' and
    'probe1536' are small profiling grids with that workload's x / z transform lengths."""
    if name == "small":
        return DnsIn(nx=32, ny=64, nz=32, alfa0=1.0, beta0=2.0, re=4000.0, a=1.6, ymin=0.0, ymax=2.0,
                     meanflowx=4.0 / 3.0, deltat=0.004, cflmax=0.0, nstep=200)
    if name == "retau180":
        return DnsIn(nx=127, ny=192, nz=127, alfa0=0.5, beta0=1.0, re=4200.0, a=1.6, ymin=0.0, ymax=2.0,
                     meanflowx=4.0 / 3.0, deltat=0.0, cflmax=1.0, nstep=2000)
    if name == "retau550":
        return DnsIn(nx=383, ny=384, nz=383, alfa0=0.5, beta0=1.0, re=14000.0, a=1.8, ymin=0.0, ymax=2.0,
                     meanflowx=4.0 / 3.0, deltat=0.0, cflmax=1.0, nstep=100)
    # profiling probes: the 383x384x383 domain with 64 planes, x rows of that
    # workload's length (768 complex points) or z columns of it (1536)
    if name == "probe768":
        return DnsIn(nx=511, ny=64, nz=64, alfa0=0.5, beta0=1.0, re=14000.0, a=1.8, ymin=0.0, ymax=2.0,
                     meanflowx=4.0 / 3.0, deltat=0.0, cflmax=1.0, nstep=10)
    if name == "probe1536":
        return DnsIn(nx=63, ny=64, nz=383, alfa0=0.5, beta0=1.0, re=14000.0, a=1.8, ymin=0.0, ymax=2.0,
                     meanflowx=4.0 / 3.0, deltat=0.0, cflmax=1.0, nstep=10)
    if name == "coarse":
        return DnsIn(nx=47, ny=96, nz=47, alfa0=0.5, beta0=1.0, re=14000.0, a=1.8, ymin=0.0, ymax=2.0,
                     meanflowx=4.0 / 3.0, deltat=0.0, cflmax=1.0, nstep=100)
    raise KeyError(name)


def ensemble_workloads(n: int = 64, seed: int = 0) -> list[DnsIn]:
    """The batched-ensemble workload: n independent minimal channels with
    nx, nz drawn from {16, 24, 32}, ny from {48, 64, 96}, Re uniform in
    [2000, 4000], alfa0 in [1, 2], beta0 in [2, 4] by numpy's default_rng(seed);
    fixed dt = 0.004 and constant flow rate 4/3 as in the 32x64x32 case.
    Member i starts from perturbed_laminar(p_i, 0.01, seed=i)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx, nz = (int(v) for v in rng.choice([16, 24, 32], size=2))
        ny = int(rng.choice([48, 64, 96]))
        re = float(rng.uniform(2000.0, 4000.0))
        alfa0, beta0 = float(rng.uniform(1.0, 2.0)), float(rng.uniform(2.0, 4.0))
        out.append(DnsIn(nx=nx, ny=ny, nz=nz, alfa0=alfa0, beta0=beta0, re=re, a=1.6, ymin=0.0, ymax=2.0,
                         meanflowx=4.0 / 3.0, deltat=0.004, cflmax=0.0, nstep=200))
    return out
