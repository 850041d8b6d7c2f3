"""The exporter's oracle (out_exporter/out2bin.f90 restated with numpy)
against direct sums and hand-computed cases."""
import numpy as np
import pytest

import out2bin as ob


def random_field(nx, ny, nz, seed):
    rng = np.random.default_rng(seed)
    V = rng.standard_normal((3, nx + 1, 2 * nz + 1, ny + 3)) + 1j * rng.standard_normal((3, nx + 1, 2 * nz + 1, ny + 3))
    return V


def direct(V):
    """u[c][iy][l][j] by the defining sums: z with exp(+i), x by the c2r rule."""
    _, nx1, nzt, nyt = V.shape
    nx, nz = nx1 - 1, (nzt - 1) // 2
    Nx, Nz = 2 * nx + 1, nzt
    kz = np.arange(-nz, nz + 1)
    l = np.arange(Nz)
    Ez = np.exp(2j * np.pi * np.outer(l, kz) / Nz)  # [l][kz]
    W = np.einsum("lz,cxzy->cylx", Ez, V[:, :, :, 1:-1])  # [c][iy][l][kx]
    j = np.arange(Nx)
    kx = np.arange(1, nx + 1)
    Ex = np.exp(2j * np.pi * np.outer(kx, j) / Nx)  # [kx][j]
    return W[..., 0].real[..., None] + 2 * np.einsum("cylk,kj->cylj", W[..., 1:], Ex).real


@pytest.mark.parametrize("nx,nz", [(3, 2), (6, 5), (8, 11)])
def test_transform_matches_direct_sums(nx, nz):
    V = random_field(nx, 4, nz, nx * 31 + nz)
    u = ob.physical_planes(V)
    ref = direct(V)
    assert np.abs(u - ref).max() <= 1e-12 * np.abs(ref).max()


def test_single_mode_is_a_cosine_wave():
    nx, ny, nz = 4, 8, 3
    V = np.zeros((3, nx + 1, 2 * nz + 1, ny + 3), complex)
    a = 0.3 - 0.7j
    V[2, 3, nz - 2, :] = a  # kx = 3, kz = -2
    V[0, 0, nz, :] = 1.25
    out = ob.out2bin(V, 2.0)
    Nx, Nz = 2 * nx + 1, 2 * nz + 1
    j, l = np.arange(Nx), np.arange(Nz)
    wave = 2 * np.real(a * np.exp(2j * np.pi * (3 * j[None, :] / Nx - 2 * l[:, None] / Nz)))
    for iy in range(ny + 1):
        assert np.allclose(out[:, iy, :, 2], wave, atol=1e-14)
        assert np.allclose(out[:, iy, :, 0], 1.25, atol=1e-15)
    assert np.abs(ob.out2bin(V, 2.0, fluct_only=True)[..., 0]).max() == 0.0


def test_large_and_small_parts_add_up():
    V = random_field(5, 6, 7, 3)
    beta0 = 2.0
    full = ob.out2bin(V, beta0)
    lg = ob.out2bin(V, beta0, part=ob.LARGE, z_threshold=6)
    sm = ob.out2bin(V, beta0, part=ob.SMALL, z_threshold=6)
    assert np.abs(lg + sm - full).max() <= 1e-12 * np.abs(full).max()
    # |beta0 kz| <= 6 is kz in -3..3: the large scales are exactly those
    # modes, the small scales the rest (filter_vfield zeroes the other side)
    W = V.copy()
    W[:, :, np.abs(np.arange(-7, 8)) > 3, :] = 0
    assert np.abs(lg - ob.out2bin(W, beta0)).max() <= 1e-12 * np.abs(full).max()


def test_sampling_grid_and_weights():
    # 2nx+1 = 7 points sampled on nint(0.5 * 7) = 4: ratio 1.75 (real*4)
    assert ob.export_dims(3, 10, 3, 0.5) == (4, 11, 4)
    assert ob.export_dims(3, 10, 3, 1.0) == (7, 11, 7)
    assert ob.fullindex(7, 4, 2) == 2.75
    c, f, wc, wf = ob.weights(2.75)
    assert (c, f, wc, wf) == (3, 2, 0.75, 0.25)
    assert ob.weights(3.0) == (3, 3, 0.5, 0.5)
    # a field linear in the sample weights: the output of a single mode at an
    # undersampled point is the bilinear mix of its four neighbours
    V = random_field(3, 2, 3, 9)
    u = ob.physical_planes(V)
    out = ob.out2bin(V, 1.0, undersample=0.5)
    zc, zf, wzc, wzf = ob.weights(ob.fullindex(7, 4, 3))
    xc, xf, wxc, wxf = ob.weights(ob.fullindex(7, 4, 2))
    ref = (u[:, 1, zc - 1, xc - 1] * wxc * wzc + u[:, 1, zf - 1, xf - 1] * wxf * wzf
           + u[:, 1, zc - 1, xf - 1] * wxf * wzc + u[:, 1, zf - 1, xc - 1] * wxc * wzf)
    assert np.allclose(out[2, 1, 1, :], ref, rtol=0, atol=1e-15)
    # full grid: the sample is the grid value itself
    assert np.abs(ob.out2bin(V, 1.0) - u.transpose(2, 1, 3, 0)).max() <= 1e-15 * np.abs(u).max() * 4


def test_names_and_spacing():
    assert ob.bin_name("Dati.cart.12.out") == "Dati.cart.12.bin"
    assert ob.bin_name("run/field.out", ob.LARGE) == "run/field.large.bin"
    assert ob.bin_name("field", ob.SMALL) == "field.small.bin"
    dx, dz = ob.grid_spacing(3, 3, 1.0, 2.0)
    assert dx == pytest.approx(2 * np.pi / 7) and dz == pytest.approx(np.pi / 7)
