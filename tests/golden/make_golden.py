"""Generates tests/golden/small_seed0.npz from the CPU oracle.

Workload: the 32x64x32 channel (alfa0=1, beta0=2, Re=4000, a=1.6, fixed
dt=0.004, constant flow rate 4/3), seeded perturbed-laminar start
(amplitude 0.01, numpy default_rng(0)).  Stored: the start-up Runtimedata
line and those of steps 1..20, the field's low modes (ix<=2, |iz|<=2, every
y, u/v/w) and per-component L2 norms after 1 and 10 steps.

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import pyoracle  # noqa: E402
from channel_gb300 import dnsin, initial  # noqa: E402

NSTEPS = 20


def sample(V, nz):
    return V[:, :3, nz - 2:nz + 3, :].copy()


def main():
    p = dnsin.workload("small")
    V0 = initial.perturbed_laminar(p, 0.01, 0)
    o = pyoracle.Oracle(p)
    o.set_field(V0)
    lines = [o.start()]
    snaps = {}
    for s in range(1, NSTEPS + 1):
        lines.append(o.step())
        if s in (1, 10):
            V = o.field()
            snaps[f"modes_{s}"] = sample(V, p.nz)
            snaps[f"norms_{s}"] = np.array([np.linalg.norm(V[c]) for c in range(3)])
    np.savez_compressed(HERE / "small_seed0.npz", lines=np.array(lines), **snaps)
    print("wrote", HERE / "small_seed0.npz")


if __name__ == "__main__":
    main()
