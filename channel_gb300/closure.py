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


def restrict_y(S: np.ndarray, pf, pc) -> np.ndarray:
    """Spectra shaped (..., ny_f+3) on the fine y grid to the coarse one of
    ny_c = ny_f / 2 planes and the same stretching: coarse plane iy is fine
    plane 2 iy (the tanh grids coincide there, dnsdata.f90:153), so the
    interior and wall planes are injected; the two ghost planes iy = -1 and
    ny_c + 1, which the coarse solver rebuilds from its wall conditions in
    its first solve, are extrapolated from the four nearest coarse planes
    (cubic Lagrange in y).  Equal y grids: S unchanged."""
    if pf.ny == pc.ny:
        return S
    if pf.ny != 2 * pc.ny or pf.a != pc.a or pf.ymin != pc.ymin or pf.ymax != pc.ymax:
        raise ValueError("the coarse y grid must be every other point of the fine one")
    nyc = pc.ny
    out = np.empty(S.shape[:-1] + (nyc + 3,), dtype=S.dtype)
    out[..., 1:nyc + 2] = S[..., 1:2 * nyc + 2:2]  # iy_c = 0..nyc <- iy_f = 0, 2, .., 2 nyc
    yc = pc.y()

    def extrap(target, idx):
        x = yc[idx]
        acc = 0.0
        for a, ia in enumerate(idx):
            w = 1.0
            for b in range(len(idx)):
                if b != a:
                    w *= (yc[target] - x[b]) / (x[a] - x[b])
            acc = acc + w * out[..., ia]
        return acc

    out[..., 0] = extrap(0, [1, 2, 3, 4])
    out[..., nyc + 2] = extrap(nyc + 2, [nyc - 2, nyc - 1, nyc, nyc + 1])
    return out


def filtered(V: np.ndarray, pf, pc) -> np.ndarray:
    """The filtered DNS field on the coarse grid: Fourier cutoff at the coarse
    modes, then the y restriction."""
    return restrict_y(restrict(V, pc.nx, pc.nz), pf, pc)


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
    if fine.p.alfa0 != coarse.p.alfa0 or fine.p.beta0 != coarse.p.beta0:
        raise ValueError("fine and coarse runs need the same domain")
    Pf = fine.products()
    coarse.upload(filtered(V, fine.p, coarse.p))
    Pc = coarse.products()
    targ = coarse.closure_physical(filtered(Pf, fine.p, coarse.p) - Pc)
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
        ref = filtered(f.download(), pf, pc)
    V0c = filtered(V0, pf, pc)
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
             precision: str = "fp64", lr: float = 3e-3, lr_final: float = 2e-4, nyc: int | None = None,
             spinup_time: float | None = None, every_time: float | None = None,
             coarse_precision: str | None = None,
             spinup_precision: str | None = None) -> tuple[Mlp | None, dict]:
    """The closure end to end on one GPU.

    1. The fine DNS (precision, adaptive dt) from a seeded broadband field
       (initial.perturbed_laminar with modes up to kmax), spinup steps (or
       spinup_time time units), then nsnap snapshots every `every` steps (or
       every_time time units).  The wall shear is recorded along the way, so
       the report shows whether the flow had settled.  spinup_precision
       runs the spin-up in another precision (the field is handed over).
       The coarse grid is (nxc, nyc, nzc) on the same domain; nyc = ny/2
       restricts in y as well (restrict_y).
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
    cprec = coarse_precision or precision
    pc = dataclasses.replace(pf, nx=nxc, nz=nzc, ny=nyc or pf.ny)
    V0 = initial.perturbed_laminar(pf, amp, seed, kmax=kmax)
    snaps, dts, history = {}, [], []
    rng = np.random.default_rng(seed)
    feats, targs = [], []
    ntr = nsnap - nval
    t_sample = 0.0
    # each snapshot is sampled as it is taken (fs: the fine products, c: the
    # coarse run); only the first held-out field is kept, for the a posteriori test
    k = 0
    if spinup_precision is not None and spinup_precision != precision:
        with Channel(pf, spinup_precision) as s:
            s.upload(V0)
            st = s.start()
            t_start = float(st[0])
            while (float(st[0]) - t_start < spinup_time) if spinup_time is not None else (k < spinup):
                st = s.step()
                k += 1
                if k % 100 == 0:
                    history.append([float(st[0]), float(st[1]), float(st[2])])
            V0 = s.download()
            t_resume = float(st[0])
        spun = True
    else:
        spun = False
    with Channel(pf, precision) as f, Channel(pf, precision) as fs, Channel(pc, cprec) as c:
        npts = c.closure_points()
        f.upload(V0)
        st = f.start(time=t_resume) if spun else f.start()
        t_start = float(st[0])
        if not spun:
            if spinup_time is not None:
                while float(st[0]) - t_start < spinup_time:
                    st = f.step()
                    k += 1
                    if k % 100 == 0:
                        history.append([float(st[0]), float(st[1]), float(st[2])])
            else:
                for _ in range(spinup):
                    st = f.step()
                    k += 1
        spin_steps = k
        t_next = float(st[0])
        while len(feats) < nsnap:
            st = f.step()
            k += 1
            if k % 100 == 0:
                history.append([float(st[0]), float(st[1]), float(st[2])])
            due = (float(st[0]) >= t_next + every_time) if every_time is not None else ((k - spin_steps) % every == 0)
            if not due:
                continue
            t_next = float(st[0])
            ts = time.time()
            V = f.download()
            if len(feats) == ntr:
                snaps[ntr] = V
            dts.append(float(st[10]))
            feat, targ = sgs_sample(fs, c, V)
            idx = np.sort(rng.choice(feat.shape[1], min(points, feat.shape[1]), replace=False))
            feats.append(feat[:, idx])
            targs.append(targ[:, idx])
            t_sample += time.time() - ts
        dns_steps = k
    t1 = time.time()
    t2 = t1
    ntr = nsnap - nval
    Ftr, Ttr = np.concatenate(feats[:ntr], 1), np.concatenate(targs[:ntr], 1)
    Fva, Tva = np.concatenate(feats[ntr:], 1), np.concatenate(targs[ntr:], 1)
    net, losses = fit(Ftr, Ttr, steps, lr=lr, lr_final=lr_final, seed=seed)
    t3 = time.time()
    r2_val = explained(net.predict(Fva), Tva)
    r2_train = explained(net.predict(Ftr[:, :points]), Ttr[:, :points])
    apost = {}
    for hz in horizons:
        apost[hz] = a_posteriori(pf, pc, snaps[ntr], hz, 0.8 * dts[ntr], {"plain": None, "closure": net}, cprec)
    t4 = time.time()
    keep = all(a["closure"] < a["plain"] for a in apost.values())
    report = {
        "fine": [pf.nx, pf.ny, pf.nz], "coarse": [pc.nx, pc.ny, pc.nz], "precision": precision,
        "initial_field": {"amplitude": amp, "kmax": kmax, "seed": seed},
        "dns": {"steps": dns_steps, "spinup_steps": spin_steps, "time_units": history[-1][0] if history else None,
                "wall_shear_history": history[::max(1, len(history) // 60)]},
        "snapshots": {"spinup": spinup_time if spinup_time is not None else spinup,
                      "every": every_time if every_time is not None else every, "count": nsnap, "held_out": nval,
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
        "seconds": {"dns": t1 - t0 - t_sample, "samples": t_sample, "training": t3 - t2, "a_posteriori": t4 - t3},
    }
    if not keep:
        net.close()
        net = None
    return net, report
