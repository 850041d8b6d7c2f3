"""The learned closure end to end on a small channel: FP64 DNS snapshots,
subgrid-stress targets, training on the tensor cores, and what the trained
network gains over the plain coarse solver against the filtered DNS; a
network that makes the coarse run worse falls back to the plain solver."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def fine_params():
    from channel_gb300.dnsin import DnsIn

    return DnsIn(nx=63, ny=96, nz=63, alfa0=0.5, beta0=1.0, re=4200.0, a=1.6, ymin=0.0, ymax=2.0,
                 meanflowx=4.0 / 3.0, deltat=0.0, cflmax=1.0, nstep=200)


@pytest.fixture(scope="module")
def trained(gpu_lib):
    from channel_gb300 import closure as cl

    net, rep = cl.pipeline(fine_params(), 23, 23, amp=0.004, kmax=24, spinup=100, every=10, nsnap=8, nval=2,
                           points=100_000, steps=4000, horizons=(10, 30))
    yield net, rep
    if net is not None:
        net.close()


def test_training_reduces_the_loss(trained):
    net, rep = trained
    assert rep["train"]["loss_last"] < 0.97 * rep["train"]["loss_first"], rep["train"]
    ev = rep["explained_variance"]["held_out"]
    assert all(np.isfinite(v) for v in ev.values())
    assert np.mean(list(ev.values())) > 0.0, ev


def test_network_beats_the_plain_coarse_solver(trained):
    net, rep = trained
    for hz, a in rep["a_posteriori"].items():
        assert a["closure"] < a["plain"], (hz, a)
    assert rep["kept"] and net is not None


def test_harmful_network_falls_back_to_the_plain_solver(trained):
    import dataclasses

    from channel_gb300 import closure as cl
    from channel_gb300 import initial

    net, rep = trained
    pf = fine_params()
    pc = dataclasses.replace(pf, nx=23, nz=23)
    bad = cl.Mlp(1)
    bad.params = net.params
    nm = net.norm
    nm["sd_out"] = nm["sd_out"] * 200.0  # stresses two hundred times too large
    bad.norm = nm
    V0 = initial.perturbed_laminar(pf, 0.004, 0, kmax=24)
    a = cl.a_posteriori(pf, pc, V0, 10, 0.004, {"plain": None, "closure": bad})
    assert a["closure"] > a["plain"]
    bad.close()


def test_pipeline_with_y_restriction(gpu_lib):
    """The pipeline with a coarse y grid of half the planes (every other DNS
    plane; the closure grid of 47x96x47 against a 192-plane DNS has this
    ratio): snapshots by time, spin-up in another precision, a finite report."""
    from channel_gb300 import closure as cl

    net, rep = cl.pipeline(fine_params(), 23, 23, amp=0.004, kmax=24, nyc=48, spinup_time=0.3, every_time=0.04,
                           nsnap=4, nval=1, points=50_000, steps=600, horizons=(5,), precision="fp64dd",
                           coarse_precision="fp64", spinup_precision="mixed")
    assert rep["coarse"] == [23, 48, 23]
    assert rep["dns"]["spinup_steps"] > 0 and rep["snapshots"]["count"] == 4
    a = rep["a_posteriori"]["5"]
    assert np.isfinite(a["plain"]) and np.isfinite(a["closure"])
    if net is not None:
        net.close()
