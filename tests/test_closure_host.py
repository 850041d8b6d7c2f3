"""Host logic of the learned closure (no GPU): the coarse-mode restriction
that defines the Fourier-cutoff filter, the normalisation and the explained
variance, and the closure header's layout constants."""
import re
from pathlib import Path

import numpy as np
import pytest

from channel_gb300 import closure as cl

ROOT = Path(__file__).resolve().parent.parent


def test_restrict_keeps_the_coarse_modes():
    rng = np.random.default_rng(0)
    nxf, nzf, nyp = 7, 5, 6
    S = rng.normal(size=(3, nxf + 1, 2 * nzf + 1, nyp)) + 1j * rng.normal(size=(3, nxf + 1, 2 * nzf + 1, nyp))
    R = cl.restrict(S, 3, 2)
    assert R.shape == (3, 4, 5, nyp)
    for ix in range(4):
        for kz in range(-2, 3):
            assert np.array_equal(R[:, ix, kz + 2], S[:, ix, kz + nzf])
    assert np.array_equal(cl.restrict(S, nxf, nzf), S)
    with pytest.raises(ValueError):
        cl.restrict(S, nxf + 1, 1)
    with pytest.raises(ValueError):
        cl.restrict(S, 1, nzf + 1)


def test_restriction_of_a_product_spectrum_is_the_filtered_product():
    """The subgrid-stress target is filter(u u) - u~ u~: for a field of two
    x modes, the product's coarse modes minus the product of the truncated
    field is the part the truncation removed (numpy, one z-constant line)."""
    N = 64
    x = 2 * np.pi * np.arange(N) / N
    u = np.cos(x) + 0.5 * np.cos(6 * x)  # mode 6 is beyond a cutoff of 4
    uu_hat = np.fft.rfft(u * u) / N
    ut = np.cos(x)
    utut_hat = np.fft.rfft(ut * ut) / N
    tau_hat = uu_hat[:5] - utut_hat[:5]
    # u u = cos^2 + cos cos6 + 0.25 cos^2 6: within |k| <= 4 only cos^2's and
    # 0.25 cos^2(6x)'s mean survive, so tau is the constant 0.125
    assert abs(tau_hat[0] - 0.125) < 1e-14
    assert np.abs(tau_hat[1:]).max() < 1e-14


def test_norm_and_explained_variance():
    rng = np.random.default_rng(1)
    feat = rng.normal(2.0, 3.0, (10, 5000))
    feat[4] = 7.0  # a constant feature keeps unit scale
    targ = rng.normal(-1.0, 0.5, (6, 5000))
    nm = cl.norm_from(feat, targ)
    assert abs(nm["mu_in"][0] - 2.0) < 0.2 and abs(nm["sd_in"][0] - 3.0) < 0.2
    assert nm["sd_in"][4] == 1.0
    assert np.allclose(cl.explained(targ, targ), 1.0)
    mean_pred = np.broadcast_to(targ.mean(1, keepdims=True), targ.shape)
    assert np.allclose(cl.explained(mean_pred, targ), 0.0, atol=1e-12)
    assert np.all(cl.explained(np.zeros_like(targ), targ) < -1.0)  # tau = 0 is worse than the mean here


def test_header_constants_match_the_binding():
    text = (ROOT / "include" / "chgpu_closure.h").read_text()
    assert int(re.search(r"#define CHGPU_MLP_NPARAMS (\d+)", text).group(1)) == cl.NPARAMS
    assert int(re.search(r"#define CHGPU_MLP_IN (\d+)", text).group(1)) == cl.NIN
    assert int(re.search(r"#define CHGPU_MLP_OUT (\d+)", text).group(1)) == cl.NOUT
    # W1[64][16] + W2 + b2 + W3 + b3 + W4[6][64] + b4
    assert 64 * 16 + 64 * 64 + 64 + 64 * 64 + 64 + 6 * 64 + 6 == cl.NPARAMS
    import mlp_oracle as mo

    assert mo.NPARAMS == cl.NPARAMS and mo.OFF_B4 + 6 == cl.NPARAMS


def test_y_restriction_injects_and_extrapolates():
    """Coarse plane iy is fine plane 2 iy (the tanh grids coincide), and the
    ghost planes come from cubic extrapolation: exact for cubic profiles."""
    import dataclasses

    from channel_gb300 import closure as cl
    from channel_gb300 import dnsin

    pf = dnsin.workload("retau180")
    pc = dataclasses.replace(pf, nx=47, nz=47, ny=96)
    yf, yc = pf.y(), pc.y()
    assert np.allclose(yc[1:-1], yf[1:-1:2][: pc.ny + 1], rtol=0, atol=1e-15)
    rng = np.random.default_rng(0)
    coef = rng.normal(size=(2, 3, 4)) + 1j * rng.normal(size=(2, 3, 4))
    poly = np.polynomial.polynomial.polyval
    S = np.array([[poly(yf, coef[i, j]) for j in range(3)] for i in range(2)])
    R = cl.restrict_y(S, pf, pc)
    want = np.array([[poly(yc, coef[i, j]) for j in range(3)] for i in range(2)])
    assert R.shape == (2, 3, pc.ny + 3)
    np.testing.assert_allclose(R, want, rtol=1e-10, atol=1e-10)
    with pytest.raises(ValueError):
        cl.restrict_y(S, pf, dataclasses.replace(pc, ny=64))
