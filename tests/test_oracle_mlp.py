"""The CPU oracle of the subgrid-stress network: its gradient against
central finite differences of its own FP64 loss, and the BF16-rounded form
against the FP64 form."""
import numpy as np

import mlp_oracle as mo


def data(n, seed=1):
    rng = np.random.default_rng(seed)
    feat = rng.normal(0.0, 1.0, (mo.NIN, n))
    targ = np.stack([np.tanh(feat[0] * feat[1]), feat[2] ** 2 - 1, np.sin(feat[3]), feat[4] * feat[9],
                     np.cos(feat[5] + feat[6]), feat[7] - feat[8]])
    norm = {"mu_in": np.zeros(mo.NIN), "sd_in": np.ones(mo.NIN), "mu_out": np.zeros(mo.NOUT),
            "sd_out": np.ones(mo.NOUT)}
    return feat, targ, norm


def test_gradient_matches_finite_differences():
    feat, targ, norm = data(64)
    theta = mo.init(3)
    _, g = mo.loss_and_grad(theta, feat, targ, norm, bf16_=False)
    rng = np.random.default_rng(5)
    live = np.r_[np.arange(0, 64) * 16 + rng.integers(0, 11, 64), mo.OFF_W2 + rng.integers(0, 4096, 40),
                 mo.OFF_B2 + rng.integers(0, 64, 10), mo.OFF_W3 + rng.integers(0, 4096, 40),
                 mo.OFF_B3 + rng.integers(0, 64, 10), mo.OFF_W4 + rng.integers(0, 384, 20),
                 mo.OFF_B4 + np.arange(6)]
    h = 1e-6
    for j in live:
        tp, tm = theta.copy(), theta.copy()
        tp[j] += h
        tm[j] -= h
        fd = (mo.loss_and_grad(tp, feat, targ, norm, False)[0] - mo.loss_and_grad(tm, feat, targ, norm, False)[0]) / (2 * h)
        assert abs(fd - g[j]) <= 1e-7 + 1e-6 * abs(fd), (j, fd, g[j])
    # the unused input columns of W1 carry no gradient
    assert np.all(g[:1024].reshape(64, 16)[:, 11:] == 0)


def test_bf16_rounding_points_stay_close_to_fp64():
    feat, targ, norm = data(512)
    theta = mo.init(4)
    l64, g64 = mo.loss_and_grad(theta, feat, targ, norm, False)
    l16, g16 = mo.loss_and_grad(theta, feat, targ, norm, True)
    assert abs(l16 - l64) / l64 < 2e-2
    assert np.linalg.norm(g16 - g64) / np.linalg.norm(g64) < 5e-2
    y64 = mo.forward(theta, feat, norm, False)
    y16 = mo.forward(theta, feat, norm, True)
    assert np.linalg.norm(y16 - y64) / np.linalg.norm(y64) < 2e-2


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 0.0, 3.0e-39], np.float64)
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5 and r[4] == 0.0
    assert np.all(np.abs(r - x) <= np.abs(x) * 2 ** -8 + 1e-40)


def test_adam_oracle_first_step_is_signed_lr():
    a = mo.Adam(4)
    th = a.step(np.zeros(4), np.array([1e-3, -2.0, 0.0, 5.0]), 0.01)
    assert np.allclose(th, [-0.01, 0.01, 0.0, -0.01], atol=1e-7)
