"""Spanwise spectra of the Reynolds-stress budgets, restated from the
reference's post-processing program postpro/tke/uiuj_spectra.f90 in numpy
(test infrastructure: the checker of chgpu_tke_*; never used by the library).

Per snapshot (uiuj_spectra.f90:161-240), with the mean profiles removed from
the (0,0) mode (:172-174) and the velocity gradient g[i][k] = du_i/dx_k
(get_gradient_33, :469-486: i alfa0 kx, i beta0 kz, and the compact y
derivative COMPLEXderiv + LeftLU5divStep2), for every y plane and kz, summed
over kx with weight c = 1 (kx = 0) or 2 (kx > 0) and cprod(a, b) = Re(conj(a) b)
(:537-541):

  var(ij)      += c cprod(u_i, u_j)
  pstrain(ij)  += c cprod(p, g_ij + g_ji)
  prod(ij)     -= c sum_k [cprod(u_i, u_k) M_jk + cprod(u_j, u_k) M_ik],  M_12 = dU/dy, M_32 = dW/dy
  psdiss(ij)   -= 2 ni c sum_k cprod(g_ik, g_jk)
  PHIptrsp     -= c (cprod(p, v) + cprod(v, p)) for vv, c cprod(p, u) for uv, c cprod(p, w) for vw
  ttrsp(ij)    -= c sum_k [cprod(F(g_ik u_k), u_j) + cprod(F(g_jk u_k), u_i)]

where F(.) is the product formed on the 3/2-padded physical grid and brought
back to the kept modes with `factor` (:197-232).  After the snapshots
(:243-272): division by their number; PHIvdiff = ni REALderiv(var), vdiff =
ni REALderiv2(var), ptrsp = REALderiv(PHIptrsp); optionally var doubled
(-two); profiles = the sum of the spectra over kz.

Pair order irs = uu, vv, ww, uv, vw, uw (:7-9); term order var, prod, psdiss,
ttrsp, vdiff, pstrain, ptrsp, PHIttrsp, PHIvdiff, PHIptrsp (:13-14); PHIttrsp
is never assigned by the reference and stays zero.  The sum over k of the
ttrsp products is taken before the transforms here (the transforms and cprod
are linear), which changes only the rounding.
"""
from __future__ import annotations

import numpy as np

PAIRS = [(0, 0), (1, 1), (2, 2), (0, 1), (1, 2), (0, 2)]
VAR, PROD, PSDISS, TTRSP, VDIFF, PSTRAIN, PTRSP, PHITTRSP, PHIVDIFF, PHIPTRSP = range(10)


def cprod(a, b):
    return (np.conj(a) * b).real


class TkeOracle:
    """Accumulates the budget spectra of snapshots (restart-file layout
    V(3, nx+1, 2nz+1, ny+3)) with the oracle's y operators (an
    oracle/pyoracle.Oracle of the same dns.in)."""

    def __init__(self, p, orc, mean_u, mean_w, mean_p=None):
        self.p = p
        self.o = orc
        self.nxd, self.nzd = orc.nxd, orc.nzd
        ny = p.ny
        self.mean = np.zeros((7, ny + 3))
        self.mean[0] = mean_u
        self.mean[1] = mean_w
        if mean_p is not None:
            self.mean[6] = mean_p
        self.mean[2] = self.o.deriv(self.mean[0].astype(complex)).real  # uiuj_spectra.f90:152-155
        self.mean[4] = self.o.deriv2(self.mean[0].astype(complex)).real
        self.mean[3] = self.o.deriv(self.mean[1].astype(complex)).real
        self.mean[5] = self.o.deriv2(self.mean[1].astype(complex)).real
        self.acc = np.zeros((6, 10, 2 * p.nz + 1, ny + 3))
        self.n = 0

    def gradient(self, V):
        p = self.p
        kx = p.alfa0 * np.arange(p.nx + 1)
        kz = p.beta0 * np.arange(-p.nz, p.nz + 1)
        G = np.zeros((3, 3) + V.shape[1:], dtype=complex)
        for i in range(3):
            G[i, 0] = 1j * kx[:, None, None] * V[i]
            G[i, 2] = 1j * kz[None, :, None] * V[i]
            for ix in range(p.nx + 1):
                for iz in range(2 * p.nz + 1):
                    G[i, 1, ix, iz] = self.o.deriv(V[i, ix, iz])
        return G

    def to_physical(self, F):
        """(nx+1, 2nz+1, planes) spectral -> (planes, nzd, 2 nxd) physical on
        the padded grid (IFT, zTOx, RFT of uiuj_spectra.f90:202-211)."""
        p = self.p
        nz, nzd, nxd = p.nz, self.nzd, self.nxd
        Z = np.zeros((F.shape[2], p.nx + 1, nzd), dtype=complex)
        Fy = np.moveaxis(F, 2, 0)  # (planes, nx+1, 2nz+1)
        Z[:, :, : nz + 1] = Fy[:, :, nz:]
        Z[:, :, nzd - nz:] = Fy[:, :, :nz]
        Z = np.fft.ifft(Z, axis=2) * nzd  # unnormalised backward
        X = np.zeros((F.shape[2], nzd, nxd + 1), dtype=complex)
        X[:, :, : p.nx + 1] = np.moveaxis(Z, 1, 2)
        return np.fft.irfft(X, n=2 * nxd, axis=2) * (2 * nxd)  # c2r uses Re of kx = 0

    def to_spectral(self, R):
        """(planes, nzd, 2 nxd) physical -> kept modes (nx+1, 2nz+1, planes)
        times factor (HFT, xTOz, FFT, uiuj_spectra.f90:218-225)."""
        p = self.p
        nz, nzd, nxd = p.nz, self.nzd, self.nxd
        X = np.fft.rfft(R, axis=2)[:, :, : p.nx + 1]
        Z = np.fft.fft(np.moveaxis(X, 1, 2), axis=2)  # (planes, nx+1, nzd)
        out = np.concatenate([Z[:, :, nzd - nz:], Z[:, :, : nz + 1]], axis=2) / (2.0 * nxd * nzd)
        return np.moveaxis(out, 0, 2)

    def accumulate(self, V, P=None):
        p = self.p
        ni = p.ni
        nz = p.nz
        V = V.copy()
        V[0, 0, nz, :] -= self.mean[0]
        V[2, 0, nz, :] -= self.mean[1]
        if P is not None:
            P = P.copy()
            P[0, nz, :] -= self.mean[6]
        G = self.gradient(V)
        c = np.full(p.nx + 1, 2.0)
        c[0] = 1.0
        cw = c[:, None, None]
        Mg = np.zeros((3, 3, p.ny + 3))
        Mg[0, 1] = self.mean[2]
        Mg[2, 1] = self.mean[3]
        # convective term of each component, F(sum_k u_k g_ik)
        phys_u = [self.to_physical(V[k]) for k in range(3)]
        N = []
        for i in range(3):
            s = sum(self.to_physical(G[i, k]) * phys_u[k] for k in range(3))
            N.append(self.to_spectral(s))
        for irs, (i, j) in enumerate(PAIRS):
            a = self.acc[irs]
            a[VAR] += (cw * cprod(V[i], V[j])).sum(axis=0)
            prod = np.zeros_like(a[VAR])
            for k in range(3):
                prod -= (cw * (cprod(V[i], V[k]) * Mg[j, k] + cprod(V[j], V[k]) * Mg[i, k])).sum(axis=0)
                a[PSDISS] -= 2 * ni * (cw * cprod(G[i, k], G[j, k])).sum(axis=0)
            a[PROD] += prod
            a[TTRSP] -= (cw * (cprod(N[i], V[j]) + cprod(N[j], V[i]))).sum(axis=0)
            if P is not None:
                a[PSTRAIN] += (cw * cprod(P, G[i, j] + G[j, i])).sum(axis=0)
                if irs == 1:
                    a[PHIPTRSP] -= (cw * (cprod(P, V[1]) + cprod(V[1], P))).sum(axis=0)
                elif irs == 3:
                    a[PHIPTRSP] -= (cw * cprod(P, V[0])).sum(axis=0)
                elif irs == 4:
                    a[PHIPTRSP] -= (cw * cprod(P, V[2])).sum(axis=0)
        self.n += 1

    def result(self, timestwo=False):
        """(mean(7, ny+3), spectra(6, 10, 2nz+1, ny+3), profiles(6, 10, ny+3))."""
        sp = self.acc / max(self.n, 1)
        ni = self.p.ni
        for iz in range(sp.shape[2]):
            for irs in range(6):
                var = sp[irs, VAR, iz].astype(complex)
                sp[irs, PHIVDIFF, iz] = self.o.deriv(var).real * ni
                sp[irs, VDIFF, iz] = self.o.deriv2(var).real * ni
                sp[irs, PTRSP, iz] = self.o.deriv(sp[irs, PHIPTRSP, iz].astype(complex)).real
        if timestwo:
            sp[:, VAR] *= 2.0
        return self.mean.copy(), sp, sp.sum(axis=2)
