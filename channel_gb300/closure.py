"""The learned subgrid-stress closure (include/chgpu_closure.h).

``Mlp`` binds the pointwise network: parameters, normalisation, resident
training set, gradient, Adam training and inference, all on the tensor
cores of the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .lib import ChannelError, load_library

NIN, NOUT, NPARAMS = 10, 6, 9734
FEATURES = ("du/dx", "du/dy", "du/dz", "dv/dx", "dv/dy", "dv/dz", "dw/dx", "dw/dy", "dw/dz", "y")
STRESSES = ("uu", "vv", "ww", "uv", "vw", "uw")

_FP = C.POINTER(C.c_float)
_DP = C.POINTER(C.c_double)


class Norm(C.Structure):
    _fields_ = [("mu_in", C.c_float * NIN), ("sd_in", C.c_float * NIN),
                ("mu_out", C.c_float * NOUT), ("sd_out", C.c_float * NOUT)]


def _f32(a, shape=None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None and a.shape != shape:
        raise ValueError(f"shape {a.shape} != {shape}")
    return a


class Mlp:
    """The 10 -> 64 -> 64 -> 64 -> 6 SiLU network on the current CUDA device."""

    def __init__(self, seed: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        rc = self.lib.chgpu_mlp_create(C.c_ulonglong(seed), C.byref(h))
        if rc != 0:
            if h:
                self.lib.chgpu_mlp_destroy(h)
            raise ChannelError(rc, self.lib.chgpu_mlp_last_error(None).decode())
        self.h = h

    def _check(self, rc: int):
        if rc != 0:
            raise ChannelError(rc, self.lib.chgpu_mlp_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.chgpu_mlp_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self) -> np.ndarray:
        t = np.empty(NPARAMS, np.float32)
        self._check(self.lib.chgpu_mlp_get_params(self.h, t.ctypes.data_as(_FP)))
        return t

    @params.setter
    def params(self, theta):
        t = _f32(theta, (NPARAMS,))
        self._check(self.lib.chgpu_mlp_set_params(self.h, t.ctypes.data_as(_FP)))

    @property
    def norm(self) -> dict:
        n = Norm()
        self._check(self.lib.chgpu_mlp_get_norm(self.h, C.byref(n)))
        return {k: np.array(getattr(n, k)[:], np.float32) for k in ("mu_in", "sd_in", "mu_out", "sd_out")}

    @norm.setter
    def norm(self, d: dict):
        n = Norm()
        for k, size in (("mu_in", NIN), ("sd_in", NIN), ("mu_out", NOUT), ("sd_out", NOUT)):
            v = np.asarray(d[k], np.float32)
            if v.shape != (size,):
                raise ValueError(f"{k}: shape {v.shape} != ({size},)")
            getattr(n, k)[:] = list(map(float, v))
        self._check(self.lib.chgpu_mlp_set_norm(self.h, C.byref(n)))

    def set_data(self, feat, targ):
        """feat (10, n), targ (6, n) in physical units."""
        f = _f32(feat)
        t = _f32(targ)
        if f.ndim != 2 or f.shape[0] != NIN or t.shape != (NOUT, f.shape[1]):
            raise ValueError("need feat (10, n) and targ (6, n)")
        self._check(self.lib.chgpu_mlp_set_data(self.h, f.ctypes.data_as(_FP), t.ctypes.data_as(_FP), f.shape[1]))

    @property
    def data_size(self) -> int:
        return int(self.lib.chgpu_mlp_data_size(self.h))

    def gradient(self, first: int = 0, count: int | None = None):
        """(loss, gradient) on resident points first .. first+count-1."""
        count = self.data_size if count is None else count
        g = np.empty(NPARAMS, np.float32)
        loss = C.c_double()
        self._check(self.lib.chgpu_mlp_gradient(self.h, first, count, g.ctypes.data_as(_FP), C.byref(loss)))
        return loss.value, g

    def train(self, steps: int, batch: int, lr: float) -> np.ndarray:
        """Adam steps on consecutive windows of the resident set; per-step losses."""
        out = np.zeros(max(steps, 1), np.float64)
        self._check(self.lib.chgpu_mlp_train(self.h, steps, batch, C.c_float(lr), out.ctypes.data_as(_DP)))
        return out[:steps]

    def save(self, path):
        """Parameters and normalisation to an .npz file."""
        np.savez(path, theta=self.params, **self.norm)

    @classmethod
    def load(cls, path) -> "Mlp":
        with np.load(path) as z:
            m = cls()
            m.params = z["theta"]
            m.norm = {k: z[k] for k in ("mu_in", "sd_in", "mu_out", "sd_out")}
        return m

    def predict(self, feat) -> np.ndarray:
        f = _f32(feat)
        if f.ndim != 2 or f.shape[0] != NIN:
            raise ValueError("need feat (10, n)")
        out = np.empty((NOUT, f.shape[1]), np.float32)
        self._check(self.lib.chgpu_mlp_predict(self.h, f.ctypes.data_as(_FP), f.shape[1], out.ctypes.data_as(_FP)))
        return out


# ---------------------------------------------------------------------------
# training data and evaluation: a fine (DNS) handle and a coarse handle on the
# same domain and y grid; the filter is the Fourier cutoff at the coarse modes
# ---------------------------------------------------------------------------
def restrict(S: np.ndarray, nx: int, nz: int) -> np.ndarray:
    """The modes kx <= nx, |kz| <= nz of spectra shaped (..., nxf+1, 2nzf+1, ny+3)."""
    nzf = (S.shape[-2] - 1) // 2
    if nx > S.shape[-3] - 1 or nz > nzf:
        raise ValueError("the coarse modes must be a subset of the fine ones")
    return np.ascontiguousarray(S[..., :nx + 1, nzf - nz:nzf + nz + 1, :])


def sgs_sample(fine, coarse, V: np.ndarray | None = None):
    """(features, targets) at every closure point of the coarse handle for the
    fine field V (default: the fine handle's current field).  Targets are the
    subgrid stresses tau_ij = filter(u_i u_j) - u~_i u~_j: the fine handle's
    products at the coarse modes minus the coarse handle's products of the
    truncated field, transformed to the coarse closure points."""
    if V is None:
        V = fine.download()
    else:
        fine.upload(V)
    if fine.p.ny != coarse.p.ny or fine.p.a != coarse.p.a or fine.p.alfa0 != coarse.p.alfa0 \
            or fine.p.beta0 != coarse.p.beta0:
        raise ValueError("fine and coarse runs need the same domain and y grid")
    Pf = fine.products()
    nx, nz = coarse.p.nx, coarse.p.nz
    coarse.upload(restrict(V, nx, nz))
    Pc = coarse.products()
    targ = coarse.closure_physical(restrict(Pf, nx, nz) - Pc)
    feat = coarse.closure_features()
    return feat, targ


def norm_from(feat: np.ndarray, targ: np.ndarray) -> dict:
    sd_in = feat.std(1)
    sd_out = targ.std(1)
    return {"mu_in": feat.mean(1), "sd_in": np.where(sd_in > 0, sd_in, 1.0),
            "mu_out": targ.mean(1), "sd_out": np.where(sd_out > 0, sd_out, 1.0)}


def fit(feat: np.ndarray, targ: np.ndarray, steps: int, batch: int = 152 * 128, lr: float = 2e-3, seed: int = 0,
        lr_final: float | None = None) -> tuple[Mlp, np.ndarray]:
    """Train a network on (features, targets) in shuffled order; the learning
    rate falls geometrically from lr to lr_final over the steps."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(feat.shape[1])
    m = Mlp(seed)
    m.norm = norm_from(feat, targ)
    m.set_data(feat[:, perm], targ[:, perm])
    lr_final = lr if lr_final is None else lr_final
    losses = []
    chunks = 10
    for k in range(chunks):
        rate = lr * (lr_final / lr) ** (k / max(chunks - 1, 1))
        losses.append(m.train(steps // chunks, batch, rate))
    return m, np.concatenate(losses)


def explained(pred: np.ndarray, targ: np.ndarray) -> np.ndarray:
    """Per stress: 1 - mean (pred - t)^2 / var t (1 is perfect, 0 the mean, < 0 worse)."""
    return 1.0 - ((pred - targ) ** 2).mean(1) / targ.var(1)


def _rel(a: np.ndarray, b: np.ndarray) -> float:
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def a_posteriori(pf, pc, V0: np.ndarray, nsteps: int, dt: float, nets: dict, precision: str = "fp64") -> dict:
    """Coarse runs against the filtered DNS.  From the fine field V0, the fine
    run and coarse runs (one per entry of nets: None is the plain solver) take
    nsteps at the fixed step dt; returns, per coarse run, the L2 distance of
    its field from the truncated fine field, relative to the change of the
    truncated fine field over the interval."""
    import dataclasses

    from .lib import Channel

    pf = dataclasses.replace(pf, deltat=dt, cflmax=0.0)
    pc = dataclasses.replace(pc, deltat=dt, cflmax=0.0)
    with Channel(pf, precision) as f:
        f.upload(V0)
        f.start()
        for _ in range(nsteps):
            f.step(sync=False)
        ref = restrict(f.download(), pc.nx, pc.nz)
    V0c = restrict(V0, pc.nx, pc.nz)
    change = np.linalg.norm(ref - V0c)
    out = {}
    for name, net in nets.items():
        with Channel(pc, precision) as c:
            c.upload(V0c)
            if net is not None:
                c.closure_attach(net, True)
            c.start()
            for _ in range(nsteps):
                c.step(sync=False)
            V = c.download()
        out[name] = float(np.linalg.norm(V - ref) / change) if np.all(np.isfinite(V)) else float("inf")
    return out


def pipeline(pf, nxc: int, nzc: int, amp: float, kmax: int, seed: int = 0, spinup: int = 150, every: int = 15,
             nsnap: int = 12, nval: int = 3, points: int = 400_000, steps: int = 20_000, horizons=(10, 40),
             precision: str = "fp64", lr: float = 3e-3, lr_final: float = 2e-4) -> tuple[Mlp | None, dict]:
    """The closure end to end on one GPU.

    1. The fine DNS (precision, adaptive dt) from a seeded broadband field
       (initial.perturbed_laminar with modes up to kmax), spinup steps, then
       nsnap snapshots every `every` steps.
    2. Per snapshot, features and subgrid-stress targets at the closure
       points of the coarse grid (nxc, nzc; the fine y grid), a random subset
       of `points` of them.
    3. A network trained on the first nsnap - nval snapshots; the explained
       variance of each stress on the last nval (a priori).
    4. A posteriori: from the first held-out snapshot, the filtered DNS
       against the coarse solver with and without the network over each
       horizon, at 0.8 x the DNS step there.
    5. The fallback: the network is kept only when it lowers the coarse
       solver's error at every horizon; otherwise the plain solver is the
       result (None).
    Returns (network or None, report)."""
    import dataclasses
    import time

    from . import initial
    from .lib import Channel

    t0 = time.time()
    pc = dataclasses.replace(pf, nx=nxc, nz=nzc)
    V0 = initial.perturbed_laminar(pf, amp, seed, kmax=kmax)
    snaps, dts = [], []
    with Channel(pf, precision) as f:
        f.upload(V0)
        f.start()
        for k in range(spinup + every * nsnap):
            st = f.step()
            if k >= spinup and (k - spinup) % every == every - 1:
                snaps.append(f.download())
                dts.append(float(st[10]))
    t1 = time.time()
    rng = np.random.default_rng(seed)
    feats, targs = [], []
    with Channel(pf, precision) as fs, Channel(pc, precision) as c:
        npts = c.closure_points()
        for V in snaps:
            feat, targ = sgs_sample(fs, c, V)
            idx = np.sort(rng.choice(feat.shape[1], min(points, feat.shape[1]), replace=False))
            feats.append(feat[:, idx])
            targs.append(targ[:, idx])
    t2 = time.time()
    ntr = nsnap - nval
    Ftr, Ttr = np.concatenate(feats[:ntr], 1), np.concatenate(targs[:ntr], 1)
    Fva, Tva = np.concatenate(feats[ntr:], 1), np.concatenate(targs[ntr:], 1)
    net, losses = fit(Ftr, Ttr, steps, lr=lr, lr_final=lr_final, seed=seed)
    t3 = time.time()
    r2_val = explained(net.predict(Fva), Tva)
    r2_train = explained(net.predict(Ftr[:, :points]), Ttr[:, :points])
    apost = {}
    for hz in horizons:
        apost[hz] = a_posteriori(pf, pc, snaps[ntr], hz, 0.8 * dts[ntr], {"plain": None, "closure": net}, precision)
    t4 = time.time()
    keep = all(a["closure"] < a["plain"] for a in apost.values())
    report = {
        "fine": [pf.nx, pf.ny, pf.nz], "coarse": [pc.nx, pc.ny, pc.nz], "precision": precision,
        "initial_field": {"amplitude": amp, "kmax": kmax, "seed": seed},
        "snapshots": {"spinup": spinup, "every": every, "count": nsnap, "held_out": nval,
                      "closure_points_per_snapshot": npts, "sampled_per_snapshot": int(feats[0].shape[1])},
        "train": {"points": int(Ftr.shape[1]), "steps": steps, "batch": 152 * 128,
                  "loss_first": float(losses[:max(1, steps // 100)].mean()),
                  "loss_last": float(losses[-max(1, steps // 100):].mean())},
        "explained_variance": {"held_out": dict(zip(STRESSES, map(float, r2_val))),
                               "train": dict(zip(STRESSES, map(float, r2_train)))},
        "tau_rms": dict(zip(STRESSES, map(float, np.sqrt((Tva ** 2).mean(1))))),
        "a_posteriori": {str(hz): {**a, "gain": a["plain"] / a["closure"] if a["closure"] > 0 else None}
                         for hz, a in apost.items()},
        "kept": keep,
        "seconds": {"dns": t1 - t0, "samples": t2 - t1, "training": t3 - t2, "a_posteriori": t4 - t3},
    }
    if not keep:
        net.close()
        net = None
    return net, report
