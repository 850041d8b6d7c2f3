"""The oracle and the CUDA step against the committed golden fixture
(tests/golden/small_seed0.npz, generated by tests/golden/make_golden.py)."""
from pathlib import Path

import numpy as np
import pytest

from helpers import line_close, rel_l2

GOLD = Path(__file__).resolve().parent / "golden" / "small_seed0.npz"


def load():
    return np.load(GOLD)


def lines_close(a, b, rtol):
    """Every Runtimedata line within rtol, each column group in its own norm
    (helpers.LINE_GROUPS: the pressure gradient at constant flow rate with
    its conditioning allowance, which also covers the same code compiled for
    another host architecture)."""
    return all(line_close(x, y, rtol)[0] for x, y in zip(np.asarray(a), np.asarray(b)))


def run(engine, nsteps):
    from channel_gb300 import dnsin, initial

    p = dnsin.workload("small")
    V0 = initial.perturbed_laminar(p, 0.01, 0)
    engine.upload(V0) if hasattr(engine, "upload") else engine.set_field(V0)
    lines = [engine.start()]
    fields = {}
    for s in range(1, nsteps + 1):
        lines.append(engine.step())
        if s in (1, 10):
            V = engine.download() if hasattr(engine, "download") else engine.field()
            fields[s] = V
    return p, np.array(lines), fields


def check(p, lines, fields, g, tol1, tol10, line_tol):
    assert lines_close(lines, g["lines"][: len(lines)], line_tol)
    nz = p.nz
    for s, tol in ((1, tol1), (10, tol10)):
        V = fields[s]
        samp = V[:, :3, nz - 2:nz + 3, :]
        for c in range(3):
            assert rel_l2(samp[c], g[f"modes_{s}"][c]) <= tol, (s, c)
            assert abs(np.linalg.norm(V[c]) - g[f"norms_{s}"][c]) <= tol * g[f"norms_{s}"][c], (s, c)


def test_oracle_reproduces_golden(oracle_mod):
    from channel_gb300 import dnsin

    o = oracle_mod.Oracle(dnsin.workload("small"))
    p, lines, fields = run(o, 20)
    check(p, lines, fields, load(), 1e-12, 1e-10, 1e-10)


@pytest.mark.gpu
def test_gpu_matches_golden(gpu_lib):
    from channel_gb300 import Channel, dnsin

    g = Channel(dnsin.workload("small"), "fp64")
    p, lines, fields = run(g, 20)
    g.close()
    check(p, lines, fields, load(), 1e-12, 1e-10, 1e-9)
