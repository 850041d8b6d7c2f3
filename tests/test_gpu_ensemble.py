"""The ensemble of uneven runs: one graph launch per step for all members
gives, member by member, exactly the step of a lone handle, and the oracle's
numbers."""
import numpy as np
import pytest

from helpers import per_field_rel

pytestmark = pytest.mark.gpu


def members(n=4):
    from channel_gb300 import dnsin

    return dnsin.ensemble_workloads(n, seed=3)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_ensemble_matches_lone_handles(gpu_lib, prec):
    from channel_gb300 import Channel, Ensemble, initial

    ps = members()
    assert len({(p.nx, p.ny, p.nz) for p in ps}) > 1  # uneven sizes
    V0 = [initial.perturbed_laminar(p, 0.01, i) for i, p in enumerate(ps)]
    ens = Ensemble(ps, prec)
    lone = [Channel(p, prec) for p in ps]
    for m, g, V in zip(ens.members, lone, V0):
        m.upload(V)
        g.upload(V)
        m.start()
        g.start()
    for _ in range(4):
        lines = ens.step()
        ref = [g.step() for g in lone]
    for m, g, line, r in zip(ens.members, lone, lines, ref):
        assert np.array_equal(m.download(), g.download())
        assert np.array_equal(line, r)
    for g in lone:
        g.close()
    ens.close()


def test_ensemble_member_against_oracle_and_retuning(gpu_lib):
    """FP64 members follow the oracle; changing one member's tiles between
    steps re-captures the ensemble graph without changing the numbers."""
    import pyoracle
    from channel_gb300 import Ensemble, initial

    ps = members(3)
    V0 = [initial.perturbed_laminar(p, 0.01, i) for i, p in enumerate(ps)]
    ens = Ensemble(ps, "fp64")
    orc = []
    for p, m, V in zip(ps, ens.members, V0):
        m.upload(V)
        m.start()
        o = pyoracle.Oracle(p)
        o.set_field(V)
        o.start()
        orc.append(o)
    ens.step()
    ens.members[1].autotune()
    for _ in range(2):
        ens.step()
    for o in orc:
        for _ in range(3):
            o.step()
    for m, o in zip(ens.members, orc):
        assert max(per_field_rel(m.download(), o.field())) <= 1e-11
        o.close()
    ens.close()
