"""Known-answer tests that pin the CPU oracle (no GPU).

The reference ships no golden vectors, so the oracle is pinned by answers
that follow from the mathematics of the scheme it restates:
  - FFTs against numpy (FFTW conventions: forward e^-i, backward e^+i,
    unnormalised; ffts.f90:70-75)
  - compact stencils exact on the monomials they are built for
    (dnsdata.f90:246-257); one-sided wall stencils exact to degree 4
  - the compact first derivative (COMPLEXderiv + D0 solve) exact on quartics
  - the non-uniform Simpson rule exact on quadratics (dnsdata.f90:312-324)
  - laminar Poiseuille flow: Runtimedata values and a steady field
  - the 3/2 rule: products of band-limited modes without aliasing
  - decay rate of a small Squire mode against the viscous eigenvalue
"""
import math

import numpy as np
import pytest

from channel_gb300 import DnsIn, dnsin, initial


def small(**over):
    p = dnsin.workload("small")
    for k, v in over.items():
        setattr(p, k, v)
    return p


@pytest.mark.parametrize("n", [48, 64, 96, 128, 192, 384, 768, 1536])
def test_fft_matches_numpy(oracle_mod, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))
    f = oracle_mod.fft(x, -1)
    b = oracle_mod.fft(x, +1)
    ref_f = np.fft.fft(x)
    ref_b = np.fft.ifft(x) * n
    assert np.abs(f - ref_f).max() <= 1e-14 * np.abs(ref_f).max()
    assert np.abs(b - ref_b).max() <= 1e-14 * np.abs(ref_b).max()
    rt = oracle_mod.fft(f, +1) / n
    assert np.abs(rt - x).max() <= 1e-14 * np.abs(x).max()


def test_grid_and_sizes(oracle_mod):
    p = small()
    o = oracle_mod.Oracle(p, 1)
    t = o.tables()
    y = t["y"]
    assert y[1] == 0.0 and abs(y[p.ny + 1] - 2.0) < 1e-15  # walls at iy=0, ny
    assert np.all(np.diff(y) > 0)
    assert abs(y[p.ny // 2 + 1] - 1.0) < 1e-15
    np.testing.assert_allclose(y, p.y(), rtol=0, atol=1e-15)
    for nx, nz, nxd, nzd in [(32, 32, 64, 96), (127, 127, 192, 384), (383, 383, 768, 1536), (47, 47, 96, 192),
                             (16, 16, 32, 48), (24, 24, 48, 96)]:
        assert dnsin.padded_sizes(nx, nz) == (nxd, nzd)


def test_compact_stencils_exact_on_monomials(oracle_mod):
    p = small()
    o = oracle_mod.Oracle(p, 1)
    t = o.tables()
    y = t["y"]
    der = t["der"]  # [iy-1][d0,d1,d2,d4][5]
    for iy in (1, 2, 7, p.ny // 2, p.ny - 2, p.ny - 1):
        d0, d1, d2, d4 = der[iy - 1]
        yy = y[iy - 1:iy + 4] - y[iy + 1]
        # compact 4th derivative exact up to degree 8 (dnsdata.f90:250-252)
        for m in range(9):
            f = yy ** m
            f4 = m * (m - 1) * (m - 2) * (m - 3) * yy ** (m - 4) if m >= 4 else 0 * yy
            lhs, rhs = np.dot(d0, f4), np.dot(d4, f)
            scale = np.abs(d4 * f).sum() + np.abs(d0 * f4).sum()
            assert abs(lhs - rhs) <= 1e-11 * scale, (iy, m, lhs, rhs, scale)
        # compact 2nd and 1st derivatives exact up to degree 4 (:253-257)
        for m in range(5):
            f = yy ** m
            f2 = m * (m - 1) * yy ** (m - 2) if m >= 2 else 0 * yy
            f1 = m * yy ** (m - 1) if m >= 1 else 0 * yy
            s2 = np.abs(d2).max() * np.abs(f).max()
            s1 = np.abs(d1).max() * np.abs(f).max()
            assert abs(np.dot(d0, f2) - np.dot(d2, f)) <= 1e-12 * max(s2, 1.0), (iy, m)
            assert abs(np.dot(d0, f1) - np.dot(d1, f)) <= 1e-12 * max(s1, 1.0), (iy, m)
        assert abs(d0.sum() - 1.0) < 1e-13  # normalisation of the compact operator
    # one-sided wall stencils: first and second derivative exact to degree 4
    for name, pts, at in (("d140", slice(0, 5), 1), ("d14m1", slice(0, 5), 0),
                          ("d14n", slice(p.ny - 2, p.ny + 3), p.ny + 1), ("d14np1", slice(p.ny - 2, p.ny + 3), p.ny + 2)):
        c = t[name]
        yy = y[pts] - y[at]
        for m in range(5):
            exact = 1.0 if m == 1 else 0.0
            assert abs(np.dot(c, yy ** m) - exact) <= 1e-10 * max(1.0, np.abs(c).max() * np.abs(yy ** m).max())


def test_compact_derivative_exact_on_quartics(oracle_mod):
    p = small()
    o = oracle_mod.Oracle(p, 1)
    y = o.tables()["y"]
    for coeffs in ([1.0, -2.0, 0.5, 0.25, -0.125], [0.0, 1.0, 0.0, 0.0, 0.0], [0.3, 0.0, 0.0, 0.0, 1.0]):
        f = np.polynomial.Polynomial(coeffs)
        val = (f(y) + 1j * 0.5 * f(y)).astype(np.complex128)
        d = o.deriv(val)
        ref = f.deriv()(y) * (1 + 0.5j)
        assert np.abs(d - ref).max() <= 1e-9 * max(1.0, np.abs(ref).max()), coeffs


def test_simpson_flow_rate_exact_on_quadratics(oracle_mod):
    p = small()
    o = oracle_mod.Oracle(p, 1)
    y = o.tables()["y"]
    assert abs(o.yintegr(y * (2 - y)) - 4.0 / 3.0) < 1e-14
    assert abs(o.yintegr(np.ones_like(y)) - 2.0) < 1e-14
    assert abs(o.yintegr(y) - 2.0) < 1e-14


def laminar(p, U=None):
    V = np.zeros((3, p.nx + 1, 2 * p.nz + 1, p.ny + 3), dtype=np.complex128)
    y = p.y()
    V[0, 0, p.nz, :] = y * (2 - y) if U is None else U(y)
    return V


def test_poiseuille_runtimedata(oracle_mod):
    """U = y(2-y), v = eta = 0: wall shear 2 at both walls, flow rate 4/3,
    pressure-gradient column 4*ni (the forcing that keeps the flow rate), a
    steady field, and v, w identically zero."""
    p = small()
    o = oracle_mod.Oracle(p, 2)
    V0 = laminar(p)
    o.set_field(V0)
    l0 = o.start()
    assert abs(l0[1] - 2.0) < 1e-11 and abs(l0[2] - 2.0) < 1e-11
    assert abs(l0[5] - 4.0 / 3.0) < 1e-14
    assert l0[3] == 0.0 and l0[4] == 0.0
    dx = math.pi / (p.alfa0 * p.nxd)
    assert abs(l0[9] - p.deltat / dx) < 1e-12  # CFL = max|U|/dx * dt, U=1 at the centreline
    for _ in range(5):
        line = o.step()
    assert abs(line[5] - 4.0 / 3.0) < 1e-13
    assert abs(line[6] - 4.0 * p.ni) < 1e-12
    assert abs(line[1] - 2.0) < 1e-10 and abs(line[2] - 2.0) < 1e-10
    V = o.field()
    assert np.abs(V[0, 0, p.nz, 1:-1] - V0[0, 0, p.nz, 1:-1]).max() < 1e-10
    assert np.abs(V[1]).max() == 0.0 and np.abs(V[2]).max() == 0.0
    mask = np.ones(V.shape[1:], bool)
    mask[0, p.nz, :] = False
    assert np.abs(V[0][mask]).max() == 0.0


def test_dealiased_products(oracle_mod):
    """Products of band-limited modes come out exact, including the highest
    kept modes whose squares fall outside the kept band (3/2 rule)."""
    p = small()
    o = oracle_mod.Oracle(p, 1)
    nz, nx = p.nz, p.nx
    V = np.zeros((3, nx + 1, 2 * nz + 1, p.ny + 3), dtype=np.complex128)
    iy = 5
    V[0, 1, nz, iy + 1] = 0.5            # u = cos(alfa0 x)
    V[1, 0, nz + 1, iy + 1] = 0.5        # v = cos(beta0 z)
    V[1, 0, nz - 1, iy + 1] = 0.5
    V[2, nx, nz + nz, iy + 1] = 0.25     # w = 0.5 cos(nx alfa0 x + nz beta0 z)
    o.set_field(V)
    out, _ = o.convolve_plane(iy)
    uu, vv, ww, uv, vw, uw = out
    exp_uu = np.zeros_like(uu)
    exp_uu[0, nz] = 0.5
    exp_uu[2, nz] = 0.25
    assert np.abs(uu - exp_uu).max() < 1e-15
    exp_uv = np.zeros_like(uv)
    exp_uv[1, nz + 1] = 0.25
    exp_uv[1, nz - 1] = 0.25
    assert np.abs(uv - exp_uv).max() < 1e-15
    exp_ww = np.zeros_like(ww)
    exp_ww[0, nz] = 0.125  # the doubled mode (2nx, 2nz) lies outside the kept band
    assert np.abs(ww - exp_ww).max() < 1e-15
    exp_vv = np.zeros_like(vv)
    exp_vv[0, nz] = 0.5
    exp_vv[0, nz + 2] = 0.25
    exp_vv[0, nz - 2] = 0.25
    assert np.abs(vv - exp_vv).max() < 1e-15


def test_squire_mode_decay(oracle_mod):
    """With no mean flow, a small eta = A sin(pi y / 2) mode at (kx, 0)
    decays at the viscous rate -ni (kx^2 + (pi/2)^2)."""
    p = small(meanflowx=0.0, deltat=0.01)
    o = oracle_mod.Oracle(p, 2)
    V = np.zeros((3, p.nx + 1, 2 * p.nz + 1, p.ny + 3), dtype=np.complex128)
    y = p.y()
    A = 1e-6
    eta = A * np.sin(np.pi * y / 2)
    V[2, 1, p.nz, :] = 1j * eta / p.alfa0  # w = i kx eta / k^2, u = 0 (v = 0)
    o.set_field(V)
    o.start()
    nsteps = 40
    for _ in range(nsteps):
        o.step()
    W = o.field()[2, 1, p.nz, :]
    amp0 = np.linalg.norm(V[2, 1, p.nz, 2:-2])
    amp1 = np.linalg.norm(W[2:-2])
    rate = math.log(amp1 / amp0) / (nsteps * p.deltat)
    sigma = -p.ni * (p.alfa0 ** 2 + (math.pi / 2) ** 2)
    assert abs(rate - sigma) <= 1e-5 * abs(sigma), (rate, sigma)


def test_oracle_body_force_ghost_rows_are_rebuilt(oracle_mod):
    """buildrhs overwrites the forcing's rows iy = -1, 0, ny, ny+1
    (dnsdata.f90:617-628): values planted there change nothing, a zero force
    changes nothing, and a force in the interior does."""
    from channel_gb300 import dnsin, initial

    p = dnsin.workload("small")
    p.nx, p.ny, p.nz = 8, 20, 8
    V0 = initial.perturbed_laminar(p, 0.01, 1)
    ny = p.ny
    G = np.zeros((3, p.nx + 1, 2 * p.nz + 1, ny + 3), dtype=np.complex128)
    rng = np.random.default_rng(4)
    for iy in (-1, 0, ny, ny + 1):
        G[..., iy + 1] = rng.standard_normal(G.shape[:3]) + 1j * rng.standard_normal(G.shape[:3])
    out = []
    for F in (None, np.zeros_like(G), G):
        o = oracle_mod.Oracle(p)
        o.set_field(V0)
        o.set_body_force(F)
        o.start()
        o.step()
        out.append(o.field())
        o.close()
    assert np.array_equal(out[0], out[1]) and np.array_equal(out[0], out[2])
    H = G.copy()
    H[0, 0, p.nz, 5] = 0.5
    o = oracle_mod.Oracle(p)
    o.set_field(V0)
    o.set_body_force(H)
    o.start()
    o.step()
    assert not np.array_equal(o.field(), out[0])
    o.close()


def test_oracle_stepped_field_is_divergence_free(oracle_mod):
    """i alfa u + v' + i beta w = 0 for every mode of a stepped field
    (linsolve_blocking.inc:99-103 builds u, w from v' and eta)."""
    p = dnsin.workload("small")
    p.nx, p.ny, p.nz = 8, 24, 8
    o = oracle_mod.Oracle(p)
    o.set_field(initial.perturbed_laminar(p, 0.05, 2))
    o.start()
    for _ in range(3):
        o.step()
    V = o.field()
    worst = 0.0
    for ix in range(p.nx + 1):
        for iz in range(-p.nz, p.nz + 1):
            if ix == 0 and iz == 0:
                continue
            u, v, w = V[0, ix, iz + p.nz], V[1, ix, iz + p.nz], V[2, ix, iz + p.nz]
            vp = o.deriv(v)
            res = 1j * p.alfa0 * ix * u + vp + 1j * p.beta0 * iz * w
            worst = max(worst, float(np.abs(res).max() / max(np.abs(vp).max(), 1e-30)))
    o.close()
    assert worst <= 1e-13, worst
