"""CPU oracle of the physical-space exporter (out_exporter/out2bin.f90).

TEST INFRASTRUCTURE ONLY: the tests and nothing else import this module, as
the checker of the CUDA exporter.  Parity unpinned: the reference exporter is
Fortran + MPI + FFTW and cannot be built in this image, so this restatement
follows the source line by line and the transforms are numpy's (pocketfft),
an implementation independent of the CUDA one.

Per y-plane 0..ny (out2bin.f90:157-199): the restart-file field V(iy,iz,ix,c)
optionally loses its mean mode (-f, :151-153) and the spanwise wavenumbers on
one side of z_threshold (filter_vfield, :338-347); the z transform is FFTW's
unnormalised backward complex DFT of length 2nz+1 over the modes placed in
FFT order (:169-172); the x transform is FFTW's c2r of odd logical length
2nx+1 (:184), which reads the imaginary part of no mode (the kx = 0 value
enters through its real part only).  The physical values are then sampled on
an nxtot x nztot grid by xz_interpolation (:236-275) with the index map of
undersampled_to_fullindex (:279-299), whose ratios are single precision
(Fortran `real`).  The output is vec(3, nxtot, 0:ny, nztot) in Fortran order,
i.e. a C array [nztot][ny+1][nxtot][3].
"""
from __future__ import annotations

import math

import numpy as np

ALL, LARGE, SMALL = 0, 1, 2
PI = 3.1415926535897932384626433832795028841971  # dnsdata.f90 PI


def nint(x: float) -> int:
    """Fortran NINT: nearest integer, halves away from zero."""
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


def export_dims(nx: int, ny: int, nz: int, undersample: float = 1.0) -> tuple[int, int, int]:
    """(nxtot, nytot, nztot) of out2bin.f90:76-78, the product in real*4."""
    u = np.float32(undersample)
    return (nint(float(u * np.float32(2 * nx + 1))), ny + 1, nint(float(u * np.float32(2 * nz + 1))))


def fullindex(n_full: int, n_tot: int, i: int) -> float:
    """undersampled_to_fullindex (out2bin.f90:296): 1-based i -> real index."""
    s = np.float32(n_full) / np.float32(n_tot)
    return float(s * (np.float32(i) - np.float32(1.0)) + np.float32(1.0))


def weights(prj: float) -> tuple[int, int, float, float]:
    """(c, f, w_c, w_f) of xz_interpolation (out2bin.f90:245-263)."""
    c, f = math.ceil(prj), math.floor(prj)
    if c == f:
        return c, f, 0.5, 0.5
    wc = abs(float(np.float32(f)) - prj) / abs(c - f)
    wf = abs(float(np.float32(c)) - prj) / abs(c - f)
    return c, f, wc, wf


def filtered_field(V: np.ndarray, beta0: float, fluct_only: bool, part: int, z_threshold: int) -> np.ndarray:
    """The field after -f (:151-153) and filter_vfield (:338-347)."""
    V = V.copy()
    nz = (V.shape[2] - 1) // 2
    if fluct_only:
        V[:, 0, nz, :] = 0.0
    if part != ALL:
        for iz in range(-nz, nz + 1):
            k = abs(beta0 * iz)
            if (k <= z_threshold and part == SMALL) or (k > z_threshold and part == LARGE):
                V[:, :, iz + nz, :] = 0.0
    return V


def physical_planes(V: np.ndarray) -> np.ndarray:
    """u[c][iy][l][j] on the full (2nx+1) x (2nz+1) grid for iy = 0..ny
    (out2bin.f90:169-184): z = l dz, x = j dx."""
    _, nx1, nzt, _ = V.shape
    nx, nz = nx1 - 1, (nzt - 1) // 2
    Nx = 2 * nx + 1
    W = V[:, :, :, 1:-1]  # planes 0..ny of the iy = -1..ny+1 axis
    # FFT order along z: kz = 0..nz then -nz..-1
    Wz = np.concatenate([W[:, :, nz:, :], W[:, :, :nz, :]], axis=2)
    Wz = np.fft.ifft(Wz, axis=2) * nzt  # unnormalised exp(+i) transform
    X = Wz.transpose(0, 3, 2, 1).copy()  # [c][ix][l][iy] -> [c][iy][l][kx]
    X[..., 0] = X[..., 0].real  # c2r ignores Im of the kx = 0 value
    return np.fft.irfft(X, n=Nx, axis=3) * Nx


def out2bin(V: np.ndarray, beta0: float, fluct_only: bool = False, part: int = ALL, z_threshold: int = 0,
            undersample: float = 1.0) -> np.ndarray:
    """vec as a C array [nztot][ny+1][nxtot][3] (out2bin.f90:141-203, 236-275)."""
    _, nx1, nzt, nyp3 = V.shape
    nx, nz, ny = nx1 - 1, (nzt - 1) // 2, nyp3 - 3
    Nx, Nz = 2 * nx + 1, nzt
    u = physical_planes(filtered_field(V, beta0, fluct_only, part, z_threshold))  # [c][iy][l][j]
    nxtot, nytot, nztot = export_dims(nx, ny, nz, undersample)
    out = np.empty((nztot, nytot, nxtot, 3))
    xs = [weights(fullindex(Nx, nxtot, xx)) for xx in range(1, nxtot + 1)]
    zs = [weights(fullindex(Nz, nztot, zz)) for zz in range(1, nztot + 1)]
    # indices past the last point wrap to the first (periodic domain)
    for zz, (zc, zf, wzc, wzf) in enumerate(zs):
        zc0, zf0 = (zc - 1) % Nz, (zf - 1) % Nz
        for xx, (xc, xf, wxc, wxf) in enumerate(xs):
            xc0, xf0 = (xc - 1) % Nx, (xf - 1) % Nx
            ucc, uff = u[:, :, zc0, xc0], u[:, :, zf0, xf0]
            ucf, ufc = u[:, :, zf0, xc0], u[:, :, zc0, xf0]
            val = ucc * (wxc * wzc) + uff * (wxf * wzf) + ufc * (wxf * wzc) + ucf * (wxc * wzf)
            out[zz, :, xx, :] = val.T
    return out


def grid_spacing(nx: int, nz: int, alfa0: float, beta0: float, undersample: float = 1.0) -> tuple[float, float]:
    """dx, dz of write_metadata (out2bin.f90:303-323)."""
    nxtot, _, nztot = export_dims(nx, 0, nz, undersample)
    dx = abs(fullindex(2 * nx + 1, nxtot, 2) - fullindex(2 * nx + 1, nxtot, 1))
    dz = abs(fullindex(2 * nz + 1, nztot, 2) - fullindex(2 * nz + 1, nztot, 1))
    return dx * 2 * PI / alfa0 / (2 * nx + 1), dz * 2 * PI / beta0 / (2 * nz + 1)


def bin_name(fname: str, part: int = ALL) -> str:
    """write_brutal_bin's output name (out2bin.f90:217-221): the text after
    the last '.' replaced by [large.|small.]bin."""
    mid = {ALL: "", LARGE: "large.", SMALL: "small."}[part]
    k = fname.rfind(".")
    return (fname[: k + 1] if k >= 0 else fname + ".") + mid + "bin"
