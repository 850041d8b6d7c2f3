"""The closure inside the channel solver, on the GPU against the oracle:
the product spectra, the transforms to the closure points, the gradient
features, a prescribed stress entering the step, and the network evaluated
in the step equal to the same stresses prescribed."""
import numpy as np
import pytest

from helpers import per_field_rel

pytestmark = pytest.mark.gpu


def physical(S, nxd, nzd):
    """numpy restatement of the z-backward + x c2r transforms (FFTW sign
    conventions, unnormalised, x zero band, Re of the kx=0 entry), at the
    points of the planes iy = 1..ny-1: (ncomp, ny-1, nzd, 2nxd)."""
    ncomp, nxp, nzt, nyp = S.shape
    nz = (nzt - 1) // 2
    Z = np.zeros((ncomp, nxp, nzd, nyp), complex)
    Z[:, :, :nz + 1] = S[:, :, nz:]
    Z[:, :, nzd - nz:] = S[:, :, :nz]
    Zt = np.fft.ifft(Z, axis=2) * nzd
    X = np.zeros((ncomp, nxd + 1, nzd, nyp), complex)
    X[:, :nxp] = Zt
    X[:, 0] = X[:, 0].real
    x = np.fft.irfft(X, n=2 * nxd, axis=1) * (2 * nxd)
    return np.transpose(x, (0, 3, 2, 1))[:, 2:nyp - 2]


def setup(prec="fp64", seed=0, amp=0.05):
    import pyoracle
    from channel_gb300 import Channel, dnsin, initial

    p = dnsin.workload("small")
    V0 = initial.perturbed_laminar(p, amp, seed)
    g = Channel(p, prec)
    g.upload(V0)
    return p, V0, g


def test_products_match_oracle(gpu_lib):
    import pyoracle

    p, V0, g = setup()
    o = pyoracle.Oracle(p)
    o.set_field(V0)
    P = g.products()
    for iy in (-1, 0, 1, 7, p.ny // 2, p.ny - 1, p.ny + 1):
        ref, _ = o.convolve_plane(iy)
        got = P[:, :, :, iy + 1]
        assert np.abs(got - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max()), iy


def test_physical_transform_matches_numpy(gpu_lib):
    from channel_gb300 import dnsin

    p, V0, g = setup()
    nxd, nzd = dnsin.padded_sizes(p.nx, p.nz)
    assert g.closure_dims() == (2 * nxd, nzd, p.ny - 1)
    rng = np.random.default_rng(3)
    S = (rng.normal(size=(6,) + V0.shape[1:]) + 1j * rng.normal(size=(6,) + V0.shape[1:])) * 0.1
    got = g.closure_physical(S).reshape(6, p.ny - 1, nzd, 2 * nxd)
    ref = physical(S, nxd, nzd)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 2e-6, err


def test_features_match_oracle_gradients(gpu_lib):
    import pyoracle
    from channel_gb300 import dnsin

    p, V0, g = setup(amp=0.1)
    nxd, nzd = dnsin.padded_sizes(p.nx, p.nz)
    o = pyoracle.Oracle(p)
    o.set_field(V0)
    ix = np.arange(p.nx + 1)[:, None, None]
    kz = (np.arange(2 * p.nz + 1) - p.nz)[None, :, None]
    G = np.zeros((9,) + V0.shape[1:], complex)
    for c in range(3):
        G[3 * c] = 1j * p.alfa0 * ix * V0[c]
        G[3 * c + 2] = 1j * p.beta0 * kz * V0[c]
        for a in range(p.nx + 1):
            for b in range(2 * p.nz + 1):
                G[3 * c + 1, a, b] = o.deriv(V0[c, a, b])
    ref = physical(G, nxd, nzd).reshape(9, -1)
    f = g.closure_features()
    assert f.shape == (10, g.closure_points())
    for k in range(9):
        err = np.abs(f[k] - ref[k]).max() / max(np.abs(ref[k]).max(), 1e-30)
        assert err < 5e-6, (k, err)
    # the wall distance: one value per plane, in (0, 1]
    wd = f[9].reshape(p.ny - 1, -1)
    assert np.all(wd.max(1) == wd.min(1)) and wd.min() > 0 and wd.max() <= 1.0


def test_prescribed_tau_steps_match_oracle(gpu_lib):
    import pyoracle
    from channel_gb300 import dnsin

    p, V0, g = setup()
    nxd, nzd = dnsin.padded_sizes(p.nx, p.nz)
    rng = np.random.default_rng(5)
    yy = np.linspace(0, 1, p.ny - 1)[None, :, None, None]
    tau = (1e-3 * rng.normal(size=(6, p.ny - 1, nzd, 2 * nxd)) * np.sin(np.pi * yy)).astype(np.float32)
    o = pyoracle.Oracle(p)
    o.set_field(V0)
    o.set_tau(tau.astype(np.float64))
    g.closure_set_tau(tau.reshape(6, -1))
    o.start()
    g.start()
    for _ in range(2):
        o.step()
        g.step()
    errs = per_field_rel(g.download(), o.field())
    assert max(errs) < 1e-12, errs
    # the stress changes the flow: against a run without it
    p2, V2, g2 = setup()
    g2.start()
    for _ in range(2):
        g2.step()
    assert max(per_field_rel(g2.download(), o.field())) > 1e-9


def test_network_in_the_step_equals_its_prescribed_stresses(gpu_lib):
    from channel_gb300 import lib
    from channel_gb300.closure import Mlp

    p, V0, g = setup(amp=0.1)
    m = Mlp(5)
    feat = g.closure_features()
    m.norm = {"mu_in": feat.mean(1), "sd_in": feat.std(1) + 1e-6, "mu_out": np.zeros(6), "sd_out": np.full(6, 1e-3)}
    tau = m.predict(feat)
    assert np.abs(tau).max() > 0
    ode = lib.RK[0]
    # buildrhs with the network attached ...
    g.start(deltat=1e-3)
    g.closure_attach(m, True)
    g.buildrhs(ode, False)
    a = g.download()
    # ... equals buildrhs with the network's stresses prescribed
    g2 = setup(amp=0.1)[2]
    g2.start(deltat=1e-3)
    g2.closure_set_tau(tau)
    g2.buildrhs(ode, False)
    b = g2.download()
    assert np.array_equal(a, b)
    # detached: the plain solver
    g3 = setup(amp=0.1)[2]
    g3.start(deltat=1e-3)
    g3.closure_attach(m, True)
    g3.closure_attach(m, False)
    g3.buildrhs(ode, False)
    g4 = setup(amp=0.1)[2]
    g4.start(deltat=1e-3)
    g4.buildrhs(ode, False)
    assert np.array_equal(g3.download(), g4.download())
    assert not np.array_equal(a, g4.download())


def test_network_steps_run_in_the_graph(gpu_lib):
    from channel_gb300.closure import Mlp

    p, V0, g = setup(amp=0.1)
    m = Mlp(6)
    feat = g.closure_features()
    m.norm = {"mu_in": feat.mean(1), "sd_in": feat.std(1) + 1e-6, "mu_out": np.zeros(6), "sd_out": np.full(6, 1e-4)}
    g.closure_attach(m, True)
    g.start()
    for _ in range(3):
        g.step()
    V = g.download()
    assert np.all(np.isfinite(V))
    g.closure_attach(m, False)
    g.step()
    assert np.all(np.isfinite(g.download()))


@pytest.mark.parametrize("prec,tol", [("fp64dd", 1e-12), ("mixed", 2e-5)])
def test_products_of_every_precision(gpu_lib, prec, tol):
    """chgpu_products converts the double-float and FP32 product spectra to
    complex128: against the oracle within the precision of each path."""
    import pyoracle

    p, V0, g = setup(prec)
    o = pyoracle.Oracle(p)
    o.set_field(V0)
    P = g.products()
    for iy in (0, 5, p.ny // 2, p.ny):
        ref, _ = o.convolve_plane(iy)
        assert np.abs(P[:, :, :, iy + 1] - ref).max() <= tol * np.abs(ref).max(), iy


@pytest.mark.parametrize("ncomp", [3, 9])
def test_physical_transform_component_counts(gpu_lib, ncomp):
    from channel_gb300 import dnsin

    p, V0, g = setup("mixed")
    nxd, nzd = dnsin.padded_sizes(p.nx, p.nz)
    rng = np.random.default_rng(ncomp)
    S = (rng.normal(size=(ncomp,) + V0.shape[1:]) + 1j * rng.normal(size=(ncomp,) + V0.shape[1:])) * 0.1
    got = g.closure_physical(S).reshape(ncomp, p.ny - 1, nzd, 2 * nxd)
    ref = physical(S, nxd, nzd)
    assert np.abs(got - ref).max() / np.abs(ref).max() < 2e-6
    with pytest.raises(Exception):
        g.closure_physical(S[:2])


def test_network_in_a_mixed_coarse_step(gpu_lib):
    """The closure in the FP32-transform path: the network's stresses enter
    as in the FP64 path (prescribed equivalence, bit for bit)."""
    from channel_gb300 import lib
    from channel_gb300.closure import Mlp

    p, V0, g = setup("mixed", amp=0.1)
    m = Mlp(8)
    feat = g.closure_features()
    m.norm = {"mu_in": feat.mean(1), "sd_in": feat.std(1) + 1e-6, "mu_out": np.zeros(6), "sd_out": np.full(6, 1e-3)}
    tau = m.predict(feat)
    g.start(deltat=1e-3)
    g.closure_attach(m, True)
    g.buildrhs(lib.RK[1], False)
    g2 = setup("mixed", amp=0.1)[2]
    g2.start(deltat=1e-3)
    g2.closure_set_tau(tau)
    g2.buildrhs(lib.RK[1], False)
    assert np.array_equal(g.download(), g2.download())
