"""Benchmark of the channel RK3/CN time step on GB300.

Headline: RK3 steps/s of the plain FP64 step on the Re_tau~550 channel
(383x384x383 modes, 1536x385x1536 physical grid after 3/2 padding), with the
double-float and mixed-precision steps measured side by side from the same
seeded field and their statistics error against FP64.  One JSON line on
stdout (rank 0).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload retau550|retau180|small|coarse]

--impl reference times the reference algorithm on the host cores.  The
reference itself (Fortran 2008 + MPI + FFTW3) cannot be built on these
machines (no gfortran, MPI or FFTW), so that arm runs the C restatement of
it (oracle/), with every host thread.

Multi-GPU: independent replicas, one per rank (the step does not shard on one
node without MPI; runs are independent), value = all ranks' steps / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "RK3 steps/s & ns/pt/step, FP64 vs mixed on 1 GB300 at ≤1e-4 stats error"
AMPLITUDE = {"small": 0.01, "retau180": 0.05, "retau550": 0.05, "coarse": 0.05, "probe768": 0.05,
             "probe1536": 0.05}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload_desc(p, prec: str) -> str:
    return (f"channel {p.nx}x{p.ny}x{p.nz} modes (physical {2 * p.nxd}x{p.ny + 1}x{p.nzd} with 3/2 padding), "
            f"alfa0={p.alfa0} beta0={p.beta0} Re={p.re} a={p.a}, "
            + (f"cflmax={p.cflmax} (adaptive dt)" if p.cflmax > 0 else f"fixed dt={p.deltat}") + f", {prec}")


def bench_config(p, ws: int) -> dict:
    """The `config` object of the JSON line, identical in both arms."""
    field_mb = 3 * (p.nx + 1) * (2 * p.nz + 1) * (p.ny + 3) * 16 / 1e6
    return {"workload": workload_desc(p, "FP64"), "grid_points": p.grid_points(),
            "spectral_points": p.spectral_points(),
            "l2": f"inputs larger than L2 (field {field_mb:.0f} MB + product spectra per step)",
            "parallelism": f"replicas x{ws}"}


def bench_data(seed: int, amp: float) -> str:
    return f"synthetic: seeded perturbed-laminar field (numpy default_rng({seed}), amplitude {amp})"


# ---------------------------------------------------------------------------
# algorithmic bytes / flops per kernel launch (one substep over all planes)
# ---------------------------------------------------------------------------
def fft_flops(n: int) -> float:
    """Real flops of the radix-4/2/3 Stockham transform of length n."""
    cost = {4: 34.0, 2: 10.0, 3: 28.0}
    f, m = 0.0, n
    rs = []
    while m % 4 == 0:
        rs.append(4)
        m //= 4
    if m % 2 == 0:
        rs.append(2)
        m //= 2
    if m % 3 == 0:
        rs.append(3)
    for r in rs:
        f += n / r * cost[r]
    return f


def kernel_model(p, mixed: bool) -> dict:
    """Per-launch algorithmic HBM bytes and FP flops of each kernel kind."""
    ts = 8 if mixed else 16
    nplanes, nxp, nzd, M = p.ny + 3, p.nx + 1, p.nzd, p.nxd
    nmodes = nxp * (2 * p.nz + 1)
    rows = (p.ny - 1) * nmodes
    zinv_b = 3 * nplanes * nmodes * 16 + 3 * nplanes * nxp * nzd * ts
    xrow_b = 9 * nplanes * nxp * nzd * ts
    zfwd_b = 6 * nplanes * nxp * nzd * ts + 6 * nplanes * nmodes * ts
    rhs_b = 6 * nplanes * nmodes * ts + 3 * nplanes * nmodes * 16 + 4 * rows * ts + 2 * rows * 16
    lin_b = 2 * rows * 16 + 3 * nplanes * nmodes * 16
    xrow_f = nplanes * nzd * (9 * fft_flops(M) + 3 * M * 12 + 2 * M * (6 * 2 + 8) + 6 * nxp * 16)
    return {
        "k_zinv": {"bytes": zinv_b, "flops": 3 * nplanes * nxp * fft_flops(nzd)},
        "k_xrow": {"bytes": xrow_b, "flops": xrow_f},
        "k_zfwd": {"bytes": zfwd_b, "flops": 6 * nplanes * nxp * fft_flops(nzd)},
        "k_rhs": {"bytes": rhs_b, "flops": rows * 330.0},
        "k_linsolve": {"bytes": lin_b, "flops": rows * 150.0},
    }


def measured_peaks() -> dict:
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return json.loads(f.read_text())
        except Exception:
            pass
    return {}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in (getattr(self, "out", "") or "").splitlines():
            t = [x.strip() for x in ln.split(",")]
            if len(t) < 9:
                continue
            try:
                sm.append(float(t[1]))
                mx.append(float(t[2]))
            except ValueError:
                continue
            for nm, v in zip(names, t[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# GPU arms
# ---------------------------------------------------------------------------
def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, ws: int) -> float:
    """Max of a per-rank time over the replicas (NCCL on GPUs, gloo on CPU)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_steps_per_s(max_ms: float, steps: int, ws: int) -> float:
    """Replicas: every rank advances its own run `steps` times; the job's
    throughput is all ranks' steps over the slowest rank's time."""
    return ws * steps / (max_ms * 1e-3)


TILES = {}


def tuned(g, prec):
    """Autotunes the first handle of a precision; later handles reuse its tiles."""
    if prec not in TILES:
        TILES[prec] = g.autotune()
    else:
        g.set_tiles(TILES[prec])
    return g


def timed_run(p, V0, prec, K, W, ws, clocks_gpu=None):
    import torch

    from channel_gb300 import Channel

    g = tuned(Channel(p, prec), prec)
    tiles = g.tiles()
    g.upload(V0)
    g.start()
    for _ in range(W):
        g.step(sync=False)
    g.synchronize()
    stream = torch.cuda.ExternalStream(g.stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier(ws)
    torch.cuda.synchronize()
    l0 = g.launches
    sampler = ClockSampler(clocks_gpu) if clocks_gpu is not None else None
    if sampler:
        sampler.__enter__()
    torch.cuda.nvtx.range_push("timed")  # the timed steps, for profiler range filters
    e0.record(stream)
    for _ in range(K):
        g.step(sync=False)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    if sampler:
        sampler.__exit__()
    barrier(ws)
    ms = e0.elapsed_time(e1)
    launches = g.launches - l0
    g.synchronize()
    st = g.stats()
    V = g.download()
    g.close()
    return {"ms": max_over_ranks(ms, ws), "launches": launches, "V": V, "line": np.array(st.line),
            "clocks": sampler.summary() if sampler else None, "tiles": tiles}


def kernel_attribution(p, V0, prec, nsteps):
    from channel_gb300 import Channel

    g = tuned(Channel(p, prec), prec)
    g.upload(V0)
    g.start()
    g.step()
    g.set_profiling(True)
    for _ in range(nsteps):
        g.step(sync=False)
    kt = g.kernel_times()
    g.close()
    return kt


def e2e_run(p, V0, prec, K, W):
    """Steps through the C ABI with the field in pinned host memory: every
    step uploads the field, advances one RK3 step and reads the field and the
    Runtimedata numbers back (the drop-in usage where the Fortran host owns V)."""
    import torch

    from channel_gb300 import Channel

    host = torch.empty(V0.shape, dtype=torch.complex128, pin_memory=True).numpy()
    host[...] = V0
    g = tuned(Channel(p, prec), prec)
    g.upload(host)
    g.start()
    for _ in range(W):
        g.upload(host)
        g.step()
        g.download(host)
    t0 = time.perf_counter()
    for _ in range(K):
        g.upload(host)
        g.step()
        g.download(host)
    t1 = time.perf_counter()
    g.close()
    nbytes = host.nbytes
    return {"s": t1 - t0, "h2d": nbytes, "d2h": nbytes + 8 * 24}


def ensemble_run(K=10, W=3, n=64):
    """The batched-ensemble workload (64 uneven minimal channels, mixed
    precision, one graph launch per step for all members)."""
    import torch

    from channel_gb300 import Ensemble, dnsin, initial

    ps = dnsin.ensemble_workloads(n, 0)
    ens = Ensemble(ps, "mixed")
    tiles = {}
    for p, m in zip(ps, ens.members):
        key = (p.nx, p.ny, p.nz)
        if key not in tiles:
            tiles[key] = m.autotune()
        else:
            m.set_tiles(tiles[key])

    def restart():
        for i, (p, m) in enumerate(zip(ps, ens.members)):
            m.upload(initial.perturbed_laminar(p, 0.01, i))
            m.start()

    s = torch.cuda.ExternalStream(ens.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # Each member's tiles are tuned on the member alone; the solve form that
    # is fastest alone (more threads per pair for these few pairs) is not the
    # fastest when 64 members share the GPU, so the members' solve form is
    # chosen by timing whole ensemble steps.
    best = None
    for form in (2, 3, 5):
        for p, m in zip(ps, ens.members):
            m.set_tiles(tiles[(p.nx, p.ny, p.nz)][:5] + (form, 1))
        restart()
        for _ in range(2):
            ens.step(sync=False)
        e0.record(s)
        for _ in range(3):
            ens.step(sync=False)
        e1.record(s)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        if best is None or ms < best[0]:
            best = (ms, form)
    for p, m in zip(ps, ens.members):
        m.set_tiles(tiles[(p.nx, p.ny, p.nz)][:5] + (best[1], 1))
    restart()
    for _ in range(W):
        ens.step(sync=False)
    ens.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed")
    e0.record(s)
    for _ in range(K):
        ens.step(sync=False)
    e1.record(s)
    e1.synchronize()
    torch.cuda.nvtx.range_pop()
    lines = ens.step()
    ms = e0.elapsed_time(e1) / K
    ens.close()
    pts = sum((p.nx + 1) * (2 * p.nz + 1) * (p.ny + 3) for p in ps)
    ok = all(np.isfinite(l).all() for l in lines)
    peak = measured_peaks().get("hbm_gbs") or 6800.0
    gbs = 912.0 * pts / (ms * 1e-3) / 1e9  # the mixed step's compulsory bytes per spectral point and step
    return {"members": n, "precision": "mixed", "ms_per_ensemble_step": ms, "member_steps_per_s": n * 1e3 / ms,
            "members_solve_form": best[1],
            "spectral_points": pts, "ns_per_spectral_pt_step": ms * 1e6 / pts, "steps": K, "warmup": W,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "bytes": "912 B per spectral point and step (the mixed step's compulsory traffic: "
                                  "field in, products out, products and field and history in, history and "
                                  "field out)"},
            "finite": ok, "workload": "dnsin.ensemble_workloads(64, seed 0): nx,nz in {16,24,32}, ny in {48,64,96}, "
                                      "Re 2000-4000, alfa0 1-2, beta0 2-4, dt 0.004; one graph launch per step"}


def profiles(V):
    nz = V.shape[2] // 2
    U = V[0, 0, nz, :].real
    w = np.ones(V.shape[1])
    w[1:] = 2.0
    D = V.copy()
    D[:, 0, nz, :] = 0.0
    rms = np.sqrt(np.einsum("x,cxzy->cy", w, np.abs(D) ** 2))
    return U, rms


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def cpu_baseline(p, V0, max_seconds=20.0):
    """The oracle (the reference's algorithm restated in C, OpenMP over planes
    and modes, every host thread) on a bounded sample of the same workload:
    whole RK3 substeps (buildrhs over every plane, linsolve over every mode,
    in the reference's order) after the start-up pass, until about
    max_seconds of work; steps/s = substeps / 3 / time."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    threads = os.cpu_count() or 1
    o = pyoracle.Oracle(p, nthreads=threads)
    o.set_field(V0)
    o.start()
    n, t = 0, 0.0
    while n == 0 or (t + t / n <= max_seconds and n < 150):
        k = n % 3
        t0 = time.perf_counter()
        s = o.scalars()
        s.time = s.time + 2.0 / pyoracle.RK[k][0] * s.deltat
        o.set_scalars(s)
        o.buildrhs(pyoracle.RK[k], k == 2)
        o.linsolve(pyoracle.RK[k][0] / s.deltat)
        if k == 2:
            o.outstats()
        t += time.perf_counter() - t0
        n += 1
    o.close()
    return {"value": n / 3.0 / t, "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": f"{n} RK3 substep(s) (buildrhs over all {p.ny + 3} planes + linsolve over all modes) of the "
                      f"same workload after start-up, {t:.1f} s; oracle C restatement (reference "
                      f"Fortran/MPI/FFTW not buildable here), OpenMP over planes and modes"}


def run_long(args):
    """FP64, FP64DD and mixed stepped side by side from the same field for
    --steps steps: the largest deviation from FP64 over the run of the wall
    shear, the pressure gradient and the time step, and the final mean and
    rms profiles (the statistics the correctness statement names)."""
    from channel_gb300 import Channel, dnsin, initial

    p = dnsin.workload(args.workload)
    V0 = initial.perturbed_laminar(p, AMPLITUDE[args.workload], seed=0)
    runs = {}
    for prec in ("fp64", "fp64dd", "mixed"):
        g = tuned(Channel(p, prec), prec)
        g.upload(V0)
        lines = [g.start()]
        t0 = time.perf_counter()
        for _ in range(args.steps):
            lines.append(g.step())
        wall = time.perf_counter() - t0
        runs[prec] = {"lines": np.array(lines), "V": g.download(), "s": wall}
        g.close()
    ref = runs["fp64"]
    U64, r64 = profiles(ref["V"])
    out = {"mode": "long", "workload": workload_desc(p, "FP64"), "steps": args.steps,
           "time_units": float(ref["lines"][-1][0] - ref["lines"][0][0])}
    for prec in ("fp64dd", "mixed"):
        L, R = runs[prec]["lines"], ref["lines"]

        def dev(cols):
            return float(np.max(np.abs(L[:, cols] - R[:, cols])) / np.max(np.abs(R[:, cols])))

        U, rr = profiles(runs[prec]["V"])
        out[prec] = {"wall_shear_max_rel": dev([1, 2]), "dpdx_max_rel": dev([6]), "dt_max_rel": dev([10]),
                     "mean_U_final": rel(U, U64), "rms_u_final": rel(rr[0], r64[0]), "rms_v_final": rel(rr[1], r64[1]),
                     "rms_w_final": rel(rr[2], r64[2]), "fields_final": [rel(runs[prec]["V"][c], ref["V"][c])
                                                                          for c in range(3)],
                     "wall_s": runs[prec]["s"]}
    out["fp64_wall_s"] = ref["s"]
    out["wall_shear_fp64_first_last"] = [float(ref["lines"][0][1]), float(ref["lines"][-1][1])]
    print(json.dumps(out), flush=True)


def run_ours(args):
    from channel_gb300 import dnsin, initial

    ws, rank, local = dist_env()
    if ws > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import torch

    torch.cuda.set_device(local)
    p = dnsin.workload(args.workload)
    amp = AMPLITUDE[args.workload]
    V0 = initial.perturbed_laminar(p, amp, seed=rank)
    K, W = args.steps, args.warmup
    gpts = p.grid_points()
    gpu_id = str(local)
    try:
        gpu_id = "GPU-" + str(torch.cuda.get_device_properties(local).uuid)
    except Exception:
        pass
    if args.mode == "timed" and args.only:  # one precision's timed steps alone (profiler captures)
        r = timed_run(p, V0, args.only, K, W, ws)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "precision": args.only, "ms_per_step": r["ms"] / K,
                              "tiles": r["tiles"], "mode": "timed"}), flush=True)
        return
    r64 = timed_run(p, V0, "fp64", K, W, ws, clocks_gpu=gpu_id)
    rdd = timed_run(p, V0, "fp64dd", K, W, ws)
    rmx = timed_run(p, V0, "mixed", K, W, ws)
    ms64 = r64["ms"] / K
    if args.mode == "timed":  # short form for profiler captures
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": ws * 1000.0 / ms64, "unit": "steps/s", "ms_per_step": ms64,
                              "fp64dd_ms_per_step": rdd["ms"] / K, "mixed_ms_per_step": rmx["ms"] / K,
                              "tiles": {"fp64": r64["tiles"], "fp64dd": rdd["tiles"], "mixed": rmx["tiles"]},
                              "mode": "timed"}), flush=True)
        return
    U64, rr64 = profiles(r64["V"])

    def stats_err(r):
        U, rr = profiles(r["V"])
        return {"mean_U": rel(U, U64), "rms_u": rel(rr[0], rr64[0]), "rms_v": rel(rr[1], rr64[1]),
                "rms_w": rel(rr[2], rr64[2]),
                "wall_shear": float(abs(r["line"][1] - r64["line"][1]) / abs(r64["line"][1])),
                "fields": [rel(r["V"][c], r64["V"][c]) for c in range(3)], "after_steps": W + K}

    from channel_gb300.lib import measure_peaks

    in_run_peaks = measure_peaks()
    peaks = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs")
    peak_src = "measured (MEASURED_PEAKS.json)" if hbm_peak else "fallback (6.8 TB/s, no MEASURED_PEAKS.json)"
    hbm_peak = hbm_peak or 6800.0
    fp64_peak_tflops = in_run_peaks["fp64_tflops"]
    nprof = max(2, min(K, 10))

    def attribution(prec, mixed):
        kt = kernel_attribution(p, V0, prec, nprof)
        model = kernel_model(p, mixed)
        dom = max((k for k in kt if k in model), key=lambda k: kt[k][0])
        ms_total, n = kt[dom]
        per = ms_total / max(n, 1) * 1e-3
        tot = max(sum(x[0] for x in kt.values()), 1e-30)
        kin = {k: {"ms_per_step": v[0] / nprof, "launches_per_step": v[1] / nprof, "share": v[0] / tot}
               for k, v in kt.items()}
        return dom, per, model[dom]["bytes"] / per / 1e9, model[dom]["flops"] / per / 1e12, kin

    dom, per, gbs, tfl, kin64 = attribution("fp64", False)
    domd, perd, gbsd, tfld, kindd = attribution("fp64dd", False)
    domm, perm, gbsm, tflm, kinmx = attribution("mixed", True)
    tf = ROOT / "profiles" / "traffic.json"
    try:
        traffic_tab = json.loads(tf.read_text()) if tf.exists() else {}
    except Exception:
        traffic_tab = {}

    def traffic_of(prec, kernel):
        return traffic_tab.get(f"{args.workload}:{prec}:{kernel}")
    e2e = e2e_run(p, V0, "fp64", min(K, 10), 2)
    ens = ensemble_run()
    cpu = cpu_baseline(p, V0) if rank == 0 else None

    def variant(r, dom_, per_, gbs_, tfl_, kin_, what, prec):
        msv = r["ms"] / K
        return {"value": whole_job_steps_per_s(r["ms"], K, ws), "unit": "steps/s", "ms_per_step": msv,
                "ns_per_pt_step": msv * 1e6 / gpts, "ns_per_spectral_pt_step": msv * 1e6 / p.spectral_points(),
                "speedup_vs_fp64": ms64 / msv, "arithmetic": what,
                "stats_err_vs_fp64": stats_err(r), "dominant_kernel": dom_, "kernels": kin_,
                "roofline": {"bound": "hbm", "kernel": dom_, "achieved": gbs_, "peak": hbm_peak, "unit": "GB/s",
                             "frac": gbs_ / hbm_peak, "traffic": traffic_of(prec, dom_), "launch_ms": per_ * 1e3,
                             "flops_tflops": tfl_}}

    line = {
        "metric": METRIC,
        "value": whole_job_steps_per_s(r64["ms"], K, ws),
        "unit": "steps/s",
        "n_gpus": ws,
        "steps": K,
        "warmup": W,
        "ms_per_step": ms64,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": bench_data(rank, amp),
        "config": bench_config(p, ws),
        "tiles": {k: {"z_cols": t[0], "x_rows": t[1], "x_variant": t[2], "z_threads": t[3],
                      "x_threads": t[4], "solve_form": t[5] if len(t) > 5 else None,
                      "step_halves": t[6] if len(t) > 6 else None} for k, t in TILES.items()},
        "tiles_from": "--tiles" if args.tiles else "chgpu_autotune on the first handle of each precision",
        "ns_per_pt_step": ms64 * 1e6 / gpts,
        "ns_per_spectral_pt_step": ms64 * 1e6 / p.spectral_points(),
        "fp64dd": variant(rdd, domd, perd, gbsd, tfld, kindd,
                          "transforms, products and nonlinear stencils in double-float (2 x FP32, ~48 bits) on the "
                          "FP32 pipes; linear terms, banded solves, walls and mean flow FP64; meets the FP64 parity bars",
                          "fp64dd"),
        "mixed": variant(rmx, domm, perm, gbsm, tflm, kinmx,
                         "transforms, products and nonlinear stencils FP32; linear terms double-float; banded "
                         "solves, walls and mean flow FP64", "mixed"),
        "ensemble": ens,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": gbs / hbm_peak, "traffic": traffic_of("fp64", dom), "peak_source": peak_src,
                     "launch_ms": per * 1e3,
                     "fp64": {"achieved": tfl, "peak": fp64_peak_tflops, "unit": "TFLOP/s", "frac": tfl / fp64_peak_tflops,
                              "peak_source": "measured in this run (chgpu_measure_peaks: FP64 FMA loop, CUDA events)",
                              "note": "the FP64 pipe binds this kernel; the HBM fraction is low by design"}},
        "peaks_in_run": in_run_peaks,
        "kernels": kin64,
        "e2e": {"value": min(K, 10) / e2e["s"] * ws, "unit": "steps/s", "h2d_bytes_per_step": e2e["h2d"],
                "d2h_bytes_per_step": e2e["d2h"]},
        "gpu_launches": r64["launches"],
        "clocks": r64["clocks"],
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def run_reference(args):
    """The reference arm: the oracle (the reference's algorithm restated in
    C; the reference's Fortran/MPI/FFTW build is impossible on these
    machines) on every host core, from the same seeded field as the GPU arm,
    whole RK3 steps after the start-up pass and one untimed step.  At sizes
    where a step takes tens of seconds it times as many of the requested
    steps as fit a ~2 minute budget and reports that count as `steps`."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from channel_gb300 import dnsin, initial

    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    p = dnsin.workload(args.workload)
    amp = AMPLITUDE[args.workload]
    V0 = initial.perturbed_laminar(p, amp, seed=0)
    threads = os.cpu_count() or 1
    o = pyoracle.Oracle(p, nthreads=threads)
    o.set_field(V0)
    o.start()
    t0 = time.perf_counter()
    o.step()
    t_one = time.perf_counter() - t0
    budget = 120.0
    W = max(0, min(args.warmup - 1, int(budget / 4 / max(t_one, 1e-9))))
    for _ in range(W):
        o.step()
    K = max(1, min(args.steps, int(budget / max(t_one, 1e-9))))
    t0 = time.perf_counter()
    for _ in range(K):
        o.step()
    t = time.perf_counter() - t0
    o.close()
    v = K / t
    line = {
        "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": ws, "steps": K, "steps_requested": args.steps,
        "warmup": W + 1, "ms_per_step": 1000.0 * t / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": bench_data(0, amp),
        "config": bench_config(p, ws),
        "ns_per_pt_step": 1e9 * t / K / p.grid_points(),
        "impl": "reference",
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": threads, "kind": "port",
                         "sample": f"{K} whole RK3 step(s) after start-up and {W + 1} untimed; the reference "
                                   f"Fortran/MPI/FFTW build is not possible here (no gfortran, MPI or FFTW), so "
                                   f"its C restatement runs, OpenMP over planes and modes"},
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_closure(args):
    """The learned closure on the 47x96x47 coarse grid: the 127x192x127
    (Re_tau~180) DNS from the seeded perturbed-laminar field, spun up to
    developed turbulence (200 time units, mixed precision), then FP64DD (FP64
    parity bars) snapshots 0.5 time units apart; per snapshot the subgrid
    stresses of the Fourier cutoff at 47x47 modes and the y restriction to 96
    planes (every other DNS plane); training on the tensor cores; explained
    variance on held-out snapshots and the FP64 coarse solver's error against
    the filtered DNS with and without the network; then the training kernel's
    throughput and the cost of the closure in the coarse step."""
    import dataclasses

    import torch
    from channel_gb300 import Channel, dnsin, initial
    from channel_gb300 import closure as cl

    pf = dnsin.workload("retau180")
    nsnap = args.steps if args.steps >= 10 else 200
    net, rep = cl.pipeline(pf, 47, 47, amp=0.05, kmax=4, nyc=96, spinup_time=200.0, every_time=0.5, nsnap=nsnap,
                           nval=max(2, nsnap // 10), points=200_000, steps=100_000, horizons=(10, 40, 100),
                           precision="fp64dd", coarse_precision="fp64", spinup_precision="mixed")
    if net is not None and args.save_net:
        net.save(args.save_net)
    # training throughput: Adam steps of 152 x 128 points on resident data
    m = cl.Mlp(1)
    rng = np.random.default_rng(0)
    n = 1 << 21
    m.set_data(rng.normal(size=(10, n)).astype(np.float32), rng.normal(size=(6, n)).astype(np.float32))
    batch = 152 * 128
    m.train(50, batch, 1e-3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    steps = 2000
    m.train(steps, batch, 1e-3)
    dt_train = (time.perf_counter() - t0) / steps
    feat = rng.normal(size=(10, n)).astype(np.float32)
    m.predict(feat)
    t0 = time.perf_counter()
    for _ in range(5):
        m.predict(feat)
    dt_pred = (time.perf_counter() - t0) / 5
    # MMA work issued per point (padded shapes): forward 11 264 and backward
    # 35 840 multiply-adds
    fl_train = 2.0 * (11264 + 35840) * batch / dt_train
    m.close()
    # the closure's share of the coarse step
    pc = dataclasses.replace(pf, nx=47, nz=47, ny=96)
    V0 = cl.filtered(initial.perturbed_laminar(pf, 0.05, 0), pf, pc)
    step_ms = {}
    probe = cl.Mlp(2) if net is None else net
    for name, on in (("plain", False), ("closure", True)):
        with Channel(pc, "fp64") as c:
            c.upload(V0)
            if on:
                c.closure_attach(probe, True)
            c.start()
            for _ in range(3):
                c.step(sync=False)
            c.synchronize()
            t0 = time.perf_counter()
            for _ in range(20):
                c.step(sync=False)
            c.synchronize()
            step_ms[name] = 1e3 * (time.perf_counter() - t0) / 20
    out = {"mode": "closure", **rep,
           "training_kernel": {"batch": batch, "ms_per_adam_step": 1e3 * dt_train,
                               "points_per_s": batch / dt_train, "mma_tflops_issued": fl_train / 1e12,
                               "arithmetic": "tcgen05.mma kind::f16, BF16 operands, FP32 accumulators in TMEM"},
           "inference_points_per_s": n / dt_pred,
           "coarse_step_ms": step_ms,
           "data": "synthetic: seeded perturbed-laminar field spun up to developed turbulence, FP64DD DNS"}
    print(json.dumps(out), flush=True)
    if net is not None:
        net.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="retau550", choices=list(AMPLITUDE))
    ap.add_argument("--save-net", default="", help="closure mode: write the kept network (parameters and "
                                                     "normalisation, .npz) to this path")
    ap.add_argument("--tiles", default="",
                    help="fixed tiles instead of autotuning, e.g. fp64:0,4,2,256,256,2,1/mixed:0,2,4,256,256,1,2 "
                         "(z columns, x rows, x-row variant, z threads, x threads; for reproducible profiler "
                         "captures)")
    ap.add_argument("--only", default="", choices=["", "fp64", "fp64dd", "mixed"],
                    help="timed mode: time this precision alone")
    ap.add_argument("--mode", default="full", choices=["full", "timed", "long", "closure", "ensemble"],
                    help="timed: only the three timed runs (for profiler captures); ensemble: only the batched "
                         "ensemble of uneven runs (--steps, --warmup); long: --steps steps of FP64, "
                         "FP64DD and mixed from one field, Runtimedata and profile errors against FP64 over the run; "
                         "closure: the learned closure trained and evaluated against the FP64 DNS")
    args = ap.parse_args()
    for item in filter(None, args.tiles.split("/")):
        prec, t = item.split(":")
        TILES[prec] = tuple(int(v) for v in t.split(","))
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    from channel_gb300 import build as b

    if args.impl == "ours":
        b.build()
        if args.mode == "ensemble":
            print(json.dumps(ensemble_run(K=args.steps, W=args.warmup)), flush=True)
        elif args.mode == "long":
            run_long(args)
        elif args.mode == "closure":
            run_closure(args)
        else:
            run_ours(args)
    else:
        run_reference(args)


if __name__ == "__main__":
    main()
