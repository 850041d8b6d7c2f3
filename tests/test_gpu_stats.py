"""On-device statistics (mean and variance profiles of the reference's
post-processing, postpro/history/var_history.f90:37-84) and asynchronous
snapshots, against the field read back to the host."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def host_profiles(fields_):
    """var_history's definitions over a list of fields (restart layout)."""
    nz = fields_[0].shape[2] // 2
    mean = np.mean([F[:, 0, nz, :].real for F in fields_], axis=0)
    f = np.ones(fields_[0].shape[1])
    f[1:] = 2.0
    var = 0.0
    for F in fields_:
        D = F.copy()
        D[:, 0, nz, :] -= mean
        var = var + np.einsum("x,cxzy->cy", f, np.abs(D) ** 2)
    return mean, var / len(fields_)


def test_profiles_match_host(gpu_lib):
    from channel_gb300 import Channel, dnsin, initial

    p = dnsin.workload("small")
    g = Channel(p, "fp64")
    g.upload(initial.perturbed_laminar(p, 0.01, 0))
    g.start()
    g.stats_reset()
    seen = []
    for _ in range(4):
        g.step()
        g.stats_accumulate()
        seen.append(g.download())
    mean, var, n = g.profiles()
    assert n == 4
    hm, hv = host_profiles(seen)
    assert np.abs(mean - hm).max() <= 1e-14
    assert np.abs(var - hv).max() <= 1e-12 * np.abs(hv).max()
    g.close()


def test_snapshot_async_equals_download(gpu_lib):
    from channel_gb300 import Channel, dnsin, initial

    p = dnsin.workload("small")
    g = Channel(p, "mixed")
    g.upload(initial.perturbed_laminar(p, 0.01, 2))
    g.start()
    g.step()
    ref = g.download()
    g.snapshot_async()
    g.step()  # runs while the snapshot leaves the device
    snap = g.snapshot_wait()
    assert np.array_equal(snap, ref)
    assert not np.array_equal(g.download(), ref)
    g.close()
