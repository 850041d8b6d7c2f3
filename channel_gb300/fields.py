"""Dati.cart.out restart/snapshot files and the Runtimedata log.

Restart file (dnsdata.f90:677-720 read, 821-848 write; README "Velocity
fields"): a 68-byte header of three int32 (nx, ny, nz) and seven float64
(alfa0, beta0, ni, a, ymin, ymax, time), then the complex128 field
V(iy,iz,ix,ic) in Fortran order, shape (ny+3, 2nz+1, nx+1, 3).  In numpy's
C order that is an array of shape (3, nx+1, 2nz+1, ny+3).

Runtimedata (dnsdata.f90:876-879): one line per step of eleven numbers,
``time dudy_bot -dudy_top dwdy_bot -dwdy_top fr_x dpdx fr_z dpdz CFL deltat``,
written list-directed, so readers split on whitespace.
"""
from __future__ import annotations

import dataclasses
import struct
from pathlib import Path

import numpy as np

from .dnsin import DnsIn

HEADER = struct.Struct("<3i7d")
assert HEADER.size == 68


@dataclasses.dataclass
class Header:
    nx: int
    ny: int
    nz: int
    alfa0: float
    beta0: float
    ni: float
    a: float
    ymin: float
    ymax: float
    time: float

    @classmethod
    def from_dnsin(cls, p: DnsIn, time: float) -> "Header":
        return cls(p.nx, p.ny, p.nz, p.alfa0, p.beta0, p.ni, p.a, p.ymin, p.ymax, time)

    def matches(self, p: DnsIn) -> bool:
        """Bit-equality check of read_restart_file (dnsdata.f90:696)."""
        return (self.nx, self.ny, self.nz, self.alfa0, self.beta0, self.ni, self.a, self.ymin, self.ymax) == (
            p.nx, p.ny, p.nz, p.alfa0, p.beta0, p.ni, p.a, p.ymin, p.ymax)


def field_shape(nx: int, ny: int, nz: int) -> tuple[int, int, int, int]:
    return (3, nx + 1, 2 * nz + 1, ny + 3)


def read_restart(path) -> tuple[Header, np.ndarray]:
    data = Path(path).read_bytes()
    if len(data) < HEADER.size:
        raise ValueError(f"{path}: truncated header ({len(data)} bytes)")
    h = Header(*HEADER.unpack_from(data, 0))
    shape = field_shape(h.nx, h.ny, h.nz)
    n = int(np.prod(shape))
    if len(data) != HEADER.size + 16 * n:
        raise ValueError(f"{path}: expected {HEADER.size + 16 * n} bytes for nx,ny,nz={h.nx},{h.ny},{h.nz}, "
                         f"found {len(data)}")
    V = np.frombuffer(data, dtype="<c16", count=n, offset=HEADER.size).reshape(shape).copy()
    return h, V


def write_restart(path, h: Header, V: np.ndarray) -> None:
    shape = field_shape(h.nx, h.ny, h.nz)
    if V.shape != shape:
        raise ValueError(f"field shape {V.shape} != {shape}")
    with open(path, "wb") as f:
        f.write(HEADER.pack(h.nx, h.ny, h.nz, h.alfa0, h.beta0, h.ni, h.a, h.ymin, h.ymax, h.time))
        f.write(np.ascontiguousarray(V, dtype="<c16").tobytes())


def runtimedata_line(vals) -> str:
    """One Runtimedata record: eleven numbers, 17 significant digits each,
    space separated (round-trips every float64)."""
    return "".join(f"{v: .16E}".rjust(26) for v in vals) + "\n"


def parse_runtimedata(path) -> np.ndarray:
    rows = []
    for ln in Path(path).read_text().splitlines():
        toks = ln.split()
        if len(toks) == 11:
            rows.append([float(t.replace("D", "E").replace("d", "e")) for t in toks])
    return np.array(rows, dtype=np.float64).reshape(-1, 11)


def stdout_line(vals) -> str:
    """Fixed-format echo (dnsdata.f90:876): F10.4,3X,4(F11.6,3X),4(F9.4,3X),2(F9.6,3X)."""
    t, a, b, c, d, e, f, g, h, i, j = vals
    return (f"{t:10.4f}   " + "".join(f"{x:11.6f}   " for x in (a, b, c, d)) +
            "".join(f"{x:9.4f}   " for x in (e, f, g, h)) + "".join(f"{x:9.6f}   " for x in (i, j)))
