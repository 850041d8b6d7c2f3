"""The time-out path of a device-side wait, exercised without a fault or a
hang: the first bulk-copy wait of the generic z-transform kernels is given
no polls (chgpu_set_wait_limit(0)), so it gives up at once, records the
cause in the handle's error word, waits with the full limit for the copy in
flight and returns; the next synchronising call reports CHGPU_E_CUDA with
the cause, and the GPU context stays usable (a new handle steps normally)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bulk_copy_wait_times_out_cleanly(gpu_lib):
    from channel_gb300 import Channel, ChannelError, dnsin, initial

    p = dnsin.workload("small")
    V0 = initial.perturbed_laminar(p, 0.01, 0)
    with Channel(p, "fp64") as g:
        t = g.tiles()
        g.set_tiles((1,) + t[1:])  # the generic z kernels, which wait on bulk copies
        g.upload(V0)
        g.set_wait_limit(0)
        with pytest.raises(ChannelError) as e:
            g.start()
        assert e.value.code == -2
        assert "did not complete in time" in str(e.value)
    with Channel(p, "fp64") as g:
        t = g.tiles()
        g.set_tiles((1,) + t[1:])
        g.upload(V0)
        g.set_wait_limit(-1)
        g.start()
        line = g.step()
        assert np.isfinite(line).all()
