"""Generates the golden fixtures of tests/golden/ from the CPU oracle.

small_seed0.npz -- the 32x64x32 channel (alfa0=1, beta0=2, Re=4000, a=1.6,
  fixed dt=0.004, constant flow rate 4/3), seeded perturbed-laminar start
  (amplitude 0.01, numpy default_rng(0)), 200 steps.  Stored: the start-up
  Runtimedata line and those of steps 1..200, the field's low modes (ix<=2,
  |iz|<=2, every y, u/v/w) and per-component L2 norms after 1 and 10 steps,
  and the mean and rms profiles after 200 steps.

retau180_seed0.npz -- the Re_tau~180 channel (127x192x127 modes, alfa0=0.5,
  beta0=1, Re=4200, a=1.6, constant flow rate 4/3, cflmax=1 so the time
  step adapts), perturbed-laminar start with amplitude 0.05 (seed 0), 2000
  steps.  Stored: the 2001 Runtimedata lines, the low modes and norms after
  2000 steps, the mean and rms profiles after 2000 steps.

    python tests/golden/make_golden.py [small|retau180 ...] [--threads N]

The long run checkpoints its field and scalars every 50 steps into
tests/golden/ckpt/ (not committed) and resumes from there when restarted:
at a step boundary the whole oracle state is the field and the scalars (the
first substep gives the RK history zero weight), so a resumed run is bit
for bit the uninterrupted one.
"""
import argparse
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import pyoracle  # noqa: E402
from channel_gb300 import dnsin, initial  # noqa: E402

RUNS = {"small": (0.01, 200, (1, 10)), "retau180": (0.05, 2000, ())}
CKPT = HERE / "ckpt"


def sample(V, nz):
    return V[:, :3, nz - 2:nz + 3, :].copy()


def profiles(V):
    """Mean profile U(y) and rms of u, v, w over the non-mean modes (weights
    1 for kx = 0 and 2 for kx > 0, postpro/history/var_history.f90:58-84)."""
    nz = V.shape[2] // 2
    U = V[0, 0, nz, :].real.copy()
    w = np.ones(V.shape[1])
    w[1:] = 2.0
    D = V.copy()
    D[:, 0, nz, :] = 0.0
    rms = np.sqrt(np.einsum("x,cxzy->cy", w, np.abs(D) ** 2))
    return U, rms


def save_ckpt(name, o, lines):
    CKPT.mkdir(exist_ok=True)
    s = o.scalars()
    sc = np.array([s.time, s.deltat, s.cfl, s.fr[0], s.fr[1], s.fr[2], s.corrpx, s.corrpz, s.meanpx, s.meanpz,
                   float(s.istep)])
    tmp = CKPT / f"{name}.tmp.npz"
    np.savez(tmp, V=o.field(), scalars=sc, lines=np.array(lines))
    os.replace(tmp, CKPT / f"{name}.npz")


def load_ckpt(name, o):
    f = CKPT / f"{name}.npz"
    if not f.exists():
        return None
    z = np.load(f)
    o.set_field(z["V"])
    sc = z["scalars"]
    s = pyoracle.Scalars()
    s.time, s.deltat, s.cfl = sc[0], sc[1], sc[2]
    s.fr[0], s.fr[1], s.fr[2] = sc[3], sc[4], sc[5]
    s.corrpx, s.corrpz, s.meanpx, s.meanpz = sc[6], sc[7], sc[8], sc[9]
    s.istep = int(sc[10])
    o.set_scalars(s)
    return [np.array(x) for x in z["lines"]]


def generate(name, threads=None, every=50):
    amp, nsteps, snap_at = RUNS[name]
    p = dnsin.workload(name)
    o = pyoracle.Oracle(p, nthreads=threads)
    lines = load_ckpt(name, o) if nsteps > every else None
    if lines is None:
        o.set_field(initial.perturbed_laminar(p, amp, 0))
        lines = [o.start()]
    snaps = {}
    t0 = time.time()
    for s in range(len(lines), nsteps + 1):
        lines.append(o.step())
        if s in snap_at:
            V = o.field()
            snaps[f"modes_{s}"] = sample(V, p.nz)
            snaps[f"norms_{s}"] = np.array([np.linalg.norm(V[c]) for c in range(3)])
        if nsteps > every and s % every == 0 and s < nsteps:
            save_ckpt(name, o, lines)
            print(f"{name}: step {s}/{nsteps}, {time.time() - t0:.0f} s", flush=True)
    V = o.field()
    U, rms = profiles(V)
    snaps[f"modes_{nsteps}"] = sample(V, p.nz)
    snaps[f"norms_{nsteps}"] = np.array([np.linalg.norm(V[c]) for c in range(3)])
    out = HERE / f"{name}_seed0.npz"
    np.savez_compressed(out, lines=np.array(lines), U=U, rms=rms, **snaps)
    o.close()
    print("wrote", out, flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("runs", nargs="*", default=["small"], choices=list(RUNS) + [[]])
    ap.add_argument("--threads", type=int, default=None)
    a = ap.parse_args()
    for name in a.runs or ["small"]:
        generate(name, a.threads)


if __name__ == "__main__":
    main()
