"""The body-force hook (dnsdata.f90:617-659): the forcing terms of buildrhs on
the GPU against the oracle, switched on and off between steps."""
import numpy as np
import pytest

from helpers import per_field_rel, rel_l2

pytestmark = pytest.mark.gpu


def forcing(p, seed, amp=0.05):
    """A force with the structure of a field: modes up to |k| = 4, Hermitian
    at kx = 0, plus a uniform mean streamwise and spanwise part."""
    from channel_gb300 import initial

    F = amp * (initial.perturbed_laminar(p, 1.0, seed) - initial.perturbed_laminar(p, 0.0, seed))
    F[0, 0, p.nz, :] = 0.3
    F[2, 0, p.nz, :] = -0.1
    return F


def setup(prec):
    import pyoracle
    from channel_gb300 import Channel, dnsin, initial

    p = dnsin.workload("small")
    V0 = initial.perturbed_laminar(p, 0.01, 0)
    o = pyoracle.Oracle(p)
    o.set_field(V0)
    g = Channel(p, prec)
    g.upload(V0)
    return p, o, g


@pytest.mark.parametrize("prec", ["fp64", "fp64dd"])
def test_body_force_steps_match_oracle(gpu_lib, prec):
    p, o, g = setup(prec)
    F = forcing(p, 7)
    o.set_body_force(F)
    g.set_body_force(F)
    lo, lg = o.start(), g.start()
    for _ in range(3):
        lo, lg = o.step(), g.step()
    assert max(per_field_rel(g.download(), o.field())) <= 1e-11
    assert np.allclose(lg, lo, rtol=1e-9, atol=1e-12)
    g.close()


def test_body_force_switched_on_and_off(gpu_lib):
    """Setting and clearing the force between steps (the captured step is
    rebuilt each time the forcing switches) follows the oracle doing the same."""
    p, o, g = setup("fp64")
    o.start()
    g.start()
    o.step()
    g.step()
    F1, F2 = forcing(p, 3), forcing(p, 5, 0.02)
    for F in (F1, F2, None, F1):
        o.set_body_force(F)
        g.set_body_force(F)
        o.step()
        g.step()
    assert max(per_field_rel(g.download(), o.field())) <= 1e-11
    g.close()


def test_body_force_mixed_close_to_fp64(gpu_lib):
    p, _, g64 = setup("fp64")
    _, _, gm = setup("mixed")
    F = forcing(p, 11)
    for g in (g64, gm):
        g.set_body_force(F)
        g.start()
        for _ in range(10):
            g.step()
    A, B = g64.download(), gm.download()
    for c in range(3):
        assert rel_l2(B[c], A[c]) <= 1e-4, c
    g64.close()
    gm.close()
