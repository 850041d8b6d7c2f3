"""Seeded perturbed-laminar initial fields, written as Dati.cart.out.

The reference generates a laminar field with a zero-amplitude random part
when no restart file exists (dnsdata.f90:704-718); the channel workloads here
need a reproducible perturbation instead, so the field is produced here and
both this library and the oracle start from the same file.

Field: U(y) = s(2-s) with s = 2(y-ymin)/(ymax-ymin) on the mean mode
(ix=iz=0); for every mode with 0<=ix<=kmax, |iz|<=kmax, (ix,iz)!=(0,0):
  v   = A e^{i phi_v} (s(2-s))^2        (v = dv/dy = 0 at both walls)
  eta = A e^{i phi_e} s(2-s)            (eta = 0 at both walls)
and u, w from continuity i kx u + v' + i kz w = 0 and eta = i kz u - i kx w:
  u = (i kx v' - i kz eta)/k^2,  w = (i kz v' + i kx eta)/k^2
(the recovery of linsolve_blocking.inc:101-103).  The ix=0 modes with iz<0
are the complex conjugates of iz>0 (the field is real).  Phases come from
numpy.random.default_rng(seed), drawn in (ix, iz) loop order.  Ghost rows
iy=-1, ny+1 take the same analytic formulas.
"""
from __future__ import annotations

import numpy as np

from .dnsin import DnsIn
from .fields import Header, field_shape, write_restart


def perturbed_laminar(p: DnsIn, amplitude: float, seed: int, kmax: int = 4) -> np.ndarray:
    y = p.y()
    L = p.ymax - p.ymin
    s = 2.0 * (y - p.ymin) / L
    dsdy = 2.0 / L
    base = s * (2.0 - s)
    V = np.zeros(field_shape(p.nx, p.ny, p.nz), dtype=np.complex128)
    nz = p.nz
    V[0, 0, nz, :] = base
    rng = np.random.default_rng(seed)
    for ix in range(0, min(kmax, p.nx) + 1):
        for iz in range(-min(kmax, nz), min(kmax, nz) + 1):
            if ix == 0 and iz <= 0:
                continue
            phv, phe = rng.uniform(0.0, 2.0 * np.pi, size=2)
            v = amplitude * np.exp(1j * phv) * base**2
            dv = amplitude * np.exp(1j * phv) * 2.0 * base * (2.0 - 2.0 * s) * dsdy
            eta = amplitude * np.exp(1j * phe) * base
            kx, kz = p.alfa0 * ix, p.beta0 * iz
            k2 = kx * kx + kz * kz
            u = (1j * kx * dv - 1j * kz * eta) / k2
            w = (1j * kz * dv + 1j * kx * eta) / k2
            V[0, ix, iz + nz, :] = u
            V[1, ix, iz + nz, :] = v
            V[2, ix, iz + nz, :] = w
            if ix == 0:
                V[0, 0, -iz + nz, :] = np.conj(u)
                V[1, 0, -iz + nz, :] = np.conj(v)
                V[2, 0, -iz + nz, :] = np.conj(w)
    return V


def write_initial(path, p: DnsIn, amplitude: float, seed: int, kmax: int = 4) -> np.ndarray:
    V = perturbed_laminar(p, amplitude, seed, kmax)
    write_restart(path, Header.from_dnsin(p, p.time), V)
    return V
