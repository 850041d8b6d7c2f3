"""The C++ driver (channel.f90's program flow over the C ABI) run in a scratch
directory with dns.in and Dati.cart.out, against the oracle; then a restart
with time_from_restart=.TRUE. that rewinds Runtimedata."""
import subprocess

import numpy as np
import pytest

from helpers import per_field_rel

pytestmark = pytest.mark.gpu


def test_driver_run_and_restart(gpu_lib, tmp_path):
    import pyoracle
    from channel_gb300 import build, dnsin, fields, initial

    p = dnsin.workload("small")
    p.nstep = 5
    p.dt_field = 0.01  # a snapshot every 2.5 steps of dt=0.004
    dnsin.write(tmp_path / "dns.in", p)
    V0 = initial.write_initial(tmp_path / "Dati.cart.out", p, 0.01, 0)
    r = subprocess.run([str(build.DRIVER), "--quiet"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = fields.parse_runtimedata(tmp_path / "Runtimedata")
    assert rows.shape == (6, 11)
    o = pyoracle.Oracle(p)
    o.set_field(V0)
    ref = [o.start()] + [o.step() for _ in range(5)]
    ref = np.array(ref)
    scale = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max(axis=1, keepdims=True))
    assert float((np.abs(rows - ref) / scale).max()) <= 1e-9
    h, V = fields.read_restart(tmp_path / "Dati.cart.out")
    assert h.matches(p) and abs(h.time - 5 * 0.004) < 1e-15
    assert max(per_field_rel(V, o.field())) <= 1e-11
    snaps = sorted(tmp_path.glob("Dati.cart.*.out"))
    assert len(snaps) >= 1  # Dati.cart.1.out, ... at t=0.012, ...
    # the first snapshot (written while later steps ran) holds the field of its step
    hs, Vs = fields.read_restart(tmp_path / "Dati.cart.1.out")
    k = int(round(hs.time / 0.004))
    o2 = pyoracle.Oracle(p)
    o2.set_field(V0)
    o2.start()
    for _ in range(k):
        o2.step()
    assert max(per_field_rel(Vs, o2.field())) <= 1e-11
    # restart: time from the file, Runtimedata rewound to that record
    p.time_from_restart = True
    p.nstep = 3
    dnsin.write(tmp_path / "dns.in", p)
    r = subprocess.run([str(build.DRIVER), "--quiet"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows2 = fields.parse_runtimedata(tmp_path / "Runtimedata")
    assert rows2.shape == (9, 11)  # start + 5 steps, then the restart record replaced and 3 more
    ref2 = [o.step() for _ in range(3)]
    assert float((np.abs(rows2[-3:] - ref2) / np.maximum(np.abs(ref2), 1e-12)).max()) <= 1e-8
    h, V = fields.read_restart(tmp_path / "Dati.cart.out")
    assert abs(h.time - 8 * 0.004) < 1e-14
    assert max(per_field_rel(V, o.field())) <= 1e-11


def test_driver_rejects_mismatched_restart(gpu_lib, tmp_path):
    from channel_gb300 import build, dnsin, initial

    p = dnsin.workload("small")
    p.nstep = 1
    initial.write_initial(tmp_path / "Dati.cart.out", p, 0.01, 0)
    p.re = 4001.0
    dnsin.write(tmp_path / "dns.in", p)
    r = subprocess.run([str(build.DRIVER), "--quiet"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 1
    assert "mismatch in metadata" in r.stderr


@pytest.mark.parametrize("flag,tol", [("--fp64dd", 1e-10), ("--mixed", 1e-4)])
def test_driver_precision_flags(gpu_lib, tmp_path, flag, tol):
    """The driver's --fp64dd and --mixed runs give the FP64 run's
    Runtimedata to their precision (wall shear, flow rate, CFL*dt)."""
    from channel_gb300 import build, dnsin, fields, initial

    p = dnsin.workload("small")
    p.nstep = 4
    runs = {}
    for f in ("", flag):
        d = tmp_path / (f.strip("-") or "fp64")
        d.mkdir()
        dnsin.write(d / "dns.in", p)
        initial.write_initial(d / "Dati.cart.out", p, 0.01, 0)
        r = subprocess.run([str(build.DRIVER), "--quiet"] + ([f] if f else []), cwd=d, capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        runs[f] = fields.parse_runtimedata(d / "Runtimedata")
    a, b = runs[flag], runs[""]
    assert a.shape == b.shape == (5, 11)
    for col in (1, 2, 5, 9):
        assert np.abs(a[:, col] - b[:, col]).max() <= tol * np.abs(b[:, col]).max(), col
