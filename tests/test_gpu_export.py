"""The physical-space exporter (out_exporter/out2bin.f90) on the GPU against
its numpy oracle: full field, mean removed, large/small scales, sampled
grids, odd transform lengths with large prime factors, several plane
chunks, and the out2bin program's files."""
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # max abs error relative to the field's largest value (FP64 transforms)


def stepped_field(p, steps=3):
    from channel_gb300 import Channel, initial

    V0 = initial.perturbed_laminar(p, 0.05, 2)
    g = Channel(p, "fp64")
    g.upload(V0)
    if steps:
        g.start()
        for _ in range(steps):
            g.step()
    return g, g.download()


def close(a, b):
    return float(np.abs(a - b).max()) <= TOL * float(np.abs(b).max())


@pytest.mark.parametrize("opts", [
    {},
    {"fluct_only": True},
    {"part": "large", "z_threshold": 6},
    {"part": "small", "z_threshold": 6, "fluct_only": True},
    {"undersample": 0.5},
    {"undersample": 0.37},
    {"undersample": 1.6},
])
def test_export_small_matches_oracle(gpu_lib, opts):
    import out2bin as ob
    from channel_gb300 import dnsin

    p = dnsin.workload("small")
    g, V = stepped_field(p)
    out = g.export_physical(**opts)
    part = {"all": ob.ALL, "large": ob.LARGE, "small": ob.SMALL}[opts.get("part", "all")]
    ref = ob.out2bin(V, p.beta0, opts.get("fluct_only", False), part, opts.get("z_threshold", 0),
                     opts.get("undersample", 1.0))
    assert out.shape == ref.shape
    assert close(out, ref)
    g.close()


def test_export_prime_lengths(gpu_lib):
    """2nx+1 = 97 and 2nz+1 = 23 are prime: each is one stage of that radix."""
    import out2bin as ob
    from channel_gb300 import dnsin

    p = dnsin.workload("small")
    p.nx, p.ny, p.nz = 48, 20, 11
    g, V = stepped_field(p, steps=0)
    assert close(g.export_physical(), ob.out2bin(V, p.beta0))
    g.close()


def test_export_retau180_in_chunks(gpu_lib):
    """127 x 192 x 127 (2n+1 = 255 = 3 5 17): the planes go through the
    transforms in several chunks."""
    import out2bin as ob
    from channel_gb300 import dnsin, initial

    p = dnsin.workload("retau180")
    from channel_gb300 import Channel

    V = initial.perturbed_laminar(p, 0.05, 4, kmax=20)
    g = Channel(p, "fp64")
    g.upload(V)
    out = g.export_physical(fluct_only=True)
    assert close(out, ob.out2bin(V, p.beta0, fluct_only=True))
    g.close()


def test_out2bin_program(gpu_lib, tmp_path):
    import out2bin as ob
    from channel_gb300 import build, dnsin, fields

    p = dnsin.workload("small")
    g, V = stepped_field(p)
    g.close()
    dnsin.write(tmp_path / "dns.in", p)
    fields.write_restart(tmp_path / "Dati.cart.3.out", fields.Header.from_dnsin(p, 0.012), V)
    (tmp_path / "largesmall_settings.in").write_text("10\n")
    r = subprocess.run([str(build.OUT2BIN), "-f", "-ls", "-u", "0.5", "Dati.cart.3.out"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Writing Dati.cart.3.bin" in r.stdout
    nxtot, nytot, nztot = ob.export_dims(p.nx, p.ny, p.nz, 0.5)
    for part, name in ((ob.ALL, "Dati.cart.3.bin"), (ob.LARGE, "Dati.cart.3.large.bin"),
                       (ob.SMALL, "Dati.cart.3.small.bin")):
        got = np.fromfile(tmp_path / name, dtype=np.float64).reshape(nztot, nytot, nxtot, 3)
        assert close(got, ob.out2bin(V, p.beta0, True, part, 10, 0.5)), name
    nfo = (tmp_path / "spatial_grid.nfo").read_text().split("\n")
    a = nfo[0].split()
    assert (int(a[0]), int(a[1])) == (nxtot, nztot)
    dx, dz = ob.grid_spacing(p.nx, p.nz, p.alfa0, p.beta0, 0.5)
    assert float(a[2]) == pytest.approx(dx, rel=1e-15) and float(a[3]) == pytest.approx(dz, rel=1e-15)
    b = nfo[1].split()
    assert (int(b[0]), int(b[1])) == (p.ny, p.ny + 1)
    # a restart file that does not match dns.in stops the program
    p2 = dnsin.workload("small")
    p2.a = 1.7
    fields.write_restart(tmp_path / "other.out", fields.Header.from_dnsin(p2, 0.0), V)
    r = subprocess.run([str(build.OUT2BIN), "other.out"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 1 and "mismatch in metadata" in r.stderr
