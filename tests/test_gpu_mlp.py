"""The subgrid-stress network on the tensor cores against its CPU oracle:
inference, the loss gradient of the forward + backward kernel, the Adam
step, and training that learns a smooth map."""
import numpy as np
import pytest

import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def data(n, seed=1):
    rng = np.random.default_rng(seed)
    feat = rng.normal(0.0, 1.0, (mo.NIN, n))
    feat[9] = rng.uniform(0.0, 2.0, n)  # the wall distance
    targ = np.stack([np.tanh(feat[0] * feat[1]), feat[2] ** 2 - 1, np.sin(feat[3]), feat[4] * feat[9],
                     np.cos(feat[5] + feat[6]), feat[7] - feat[8]])
    return feat.astype(np.float32), targ.astype(np.float32)


NORM = {"mu_in": np.r_[np.zeros(9), 1.0], "sd_in": np.r_[np.ones(9), 0.6], "mu_out": np.full(6, 0.1),
        "sd_out": np.linspace(0.5, 1.5, 6)}


def make(seed=0):
    from channel_gb300.closure import Mlp

    m = Mlp(seed)
    m.norm = NORM
    return m


def test_params_roundtrip_and_init(gpu_lib):
    m = make(7)
    th = m.params
    W1 = th[:1024].reshape(64, 16)
    assert np.all(W1[:, 10:] == 0) and np.abs(W1[:, :10]).max() <= np.sqrt(6 / 10)
    assert np.all(th[mo.OFF_B2:mo.OFF_B2 + 64] == 0)
    t2 = mo.init(2).astype(np.float32)
    m.params = t2
    assert np.array_equal(m.params, t2)
    n = m.norm
    assert np.allclose(n["sd_out"], NORM["sd_out"])


@pytest.mark.parametrize("n", [128, 1000, 40000])
def test_inference_matches_oracle(gpu_lib, n):
    m = make()
    theta = mo.init(11).astype(np.float32)
    m.params = theta
    feat, _ = data(n, 3)
    y = m.predict(feat)
    ref = mo.forward(theta.astype(np.float64), feat, NORM, bf16_=True)
    assert y.shape == (6, n)
    # FP32 accumulation on the GPU against FP64 sums of the same BF16 operands
    err = np.linalg.norm(y - ref) / np.linalg.norm(ref)
    assert err < 2e-3, err
    ref64 = mo.forward(theta.astype(np.float64), feat, NORM, bf16_=False)
    assert np.linalg.norm(y - ref64) / np.linalg.norm(ref64) < 3e-2


@pytest.mark.parametrize("count,first", [(128, 0), (2048, 640), (152 * 128 * 3, 0)])
def test_gradient_matches_oracle(gpu_lib, count, first):
    m = make()
    theta = mo.init(12).astype(np.float32)
    m.params = theta
    n = max(count, 4096)
    feat, targ = data(n, 4)
    m.set_data(feat, targ)
    loss, g = m.gradient(first, count)
    idx = (first + np.arange(count)) % n
    lref, gref = mo.loss_and_grad(theta.astype(np.float64), feat[:, idx], targ[:, idx], NORM, bf16_=True)
    assert abs(loss - lref) / lref < 1e-3, (loss, lref)
    # per tensor: W1, W2, b2, W3, b3, W4, b4
    bounds = [0, 1024, 5120, 5184, 9280, 9344, 9728, 9734]
    for a, b in zip(bounds[:-1], bounds[1:]):
        e = np.linalg.norm(g[a:b] - gref[a:b]) / np.linalg.norm(gref[a:b])
        assert e < 1e-2, (a, b, e)
    assert np.all(g[:1024].reshape(64, 16)[:, 11:] == 0)


def test_adam_step_matches_oracle(gpu_lib):
    m = make()
    theta = mo.init(13).astype(np.float32)
    m.params = theta
    feat, targ = data(4096, 5)
    m.set_data(feat, targ)
    _, g = m.gradient(0, 1024)
    m.train(1, 1024, 1e-3)
    adam = mo.Adam(mo.NPARAMS)
    ref = adam.step(theta.astype(np.float64), g.astype(np.float64), 1e-3)
    assert np.allclose(m.params, ref, rtol=1e-5, atol=1e-7)


def test_training_learns_a_smooth_map(gpu_lib):
    m = make(3)
    feat, targ = data(1 << 17, 6)
    m.set_data(feat, targ)
    l0, _ = m.gradient(0, 8192)
    losses = m.train(600, 4096, 2e-3)
    l1, _ = m.gradient(0, 8192)
    assert np.all(np.isfinite(losses))
    assert l1 < 0.1 * l0, (l0, l1)
    # held-out points
    fv, tv = data(8192, 99)
    y = m.predict(fv)
    rv = np.mean((y - tv) ** 2) / np.mean((tv - tv.mean(1, keepdims=True)) ** 2)
    assert rv < 0.1, rv


def test_bad_arguments_are_rejected(gpu_lib):
    from channel_gb300 import ChannelError

    m = make()
    with pytest.raises(ChannelError):
        m.gradient(0, 128)  # no data yet
    feat, targ = data(512, 1)
    m.set_data(feat, targ)
    with pytest.raises(ChannelError):
        m.gradient(0, 100)
    with pytest.raises(ChannelError):
        m.train(1, 64, 1e-3)
    bad = dict(NORM)
    bad["sd_in"] = np.zeros(10)
    with pytest.raises(ChannelError):
        m.norm = bad


def test_save_and_load(gpu_lib, tmp_path):
    from channel_gb300.closure import Mlp

    m = make(9)
    m.params = mo.init(21).astype(np.float32)
    path = tmp_path / "net.npz"
    m.save(path)
    m2 = Mlp.load(path)
    assert np.array_equal(m2.params, m.params)
    for k, v in m.norm.items():
        assert np.array_equal(m2.norm[k], v)
    feat, _ = data(512, 2)
    assert np.array_equal(m2.predict(feat), m.predict(feat))
