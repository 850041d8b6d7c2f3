"""Formats (dns.in, Dati.cart.out, Runtimedata), the initial-field generator,
and the C ABI's symbol table -- all without a GPU."""
import ctypes
import re
import struct
from pathlib import Path

import numpy as np
import pytest

from channel_gb300 import dnsin, fields, initial

ROOT = Path(__file__).resolve().parent.parent

REFERENCE_STYLE_DNSIN = """191       384    189                     ! nx, ny, nz
0.5d0       1.0                            ! alfa0 beta0
12431.d0                                    ! ni
1.5       0.0    2.0                     ! a, ymin, ymax
.TRUE.    1      0.161436                ! CPI, CPItype, gamma
0.0       0.0                            ! meanpx, meanpz
0.0       0.0                            ! meanflowx meanflowz
0.0       0.0                            ! u0 uN
0.0       1.0    0.0                     ! deltat, cflmax, time
30       -1      7000        .TRUE.      ! dt_field, dt_save, t_max, time_from_restart
999999                                  ! nstep
1                                       ! npy (no. processes y)
"""


def test_dnsin_parse_reference_style():
    p = dnsin.parse(REFERENCE_STYLE_DNSIN)
    assert (p.nx, p.ny, p.nz) == (191, 384, 189)
    assert p.alfa0 == 0.5 and p.re == 12431.0 and p.ni == 1 / 12431.0
    assert p.cpi is True and p.cpi_type == 1 and p.gamma == 0.161436
    assert p.cflmax == 1.0 and p.dt_save == -1.0 and p.time_from_restart is True
    assert p.nstep == 999999 and p.npy == 1
    assert (p.nxd, p.nzd) == (384, 768)  # 3*192/2=288 -> 384; 3*189=567 -> 768


def test_dnsin_roundtrip(tmp_path):
    for name in ("small", "retau180", "retau550", "coarse"):
        p = dnsin.workload(name)
        f = tmp_path / f"{name}.in"
        dnsin.write(f, p)
        q = dnsin.read(f)
        assert q == p


def test_fftfit_and_padding():
    assert [n for n in range(1, 50) if dnsin.fft_fit(n)] == [1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48]
    for nx in range(1, 400, 7):
        nxd, nzd = dnsin.padded_sizes(nx, nx)
        assert nxd >= 3 * (nx + 1) // 2 and dnsin.fft_fit(nxd)
        assert nzd >= 3 * nx and dnsin.fft_fit(nzd)


def test_restart_roundtrip_and_layout(tmp_path):
    p = dnsin.workload("small")
    V = initial.perturbed_laminar(p, 0.01, 7)
    f = tmp_path / "Dati.cart.out"
    fields.write_restart(f, fields.Header.from_dnsin(p, 1.25), V)
    raw = f.read_bytes()
    assert len(raw) == 68 + 16 * V.size
    nx, ny, nz = struct.unpack_from("<3i", raw, 0)
    assert (nx, ny, nz) == (p.nx, p.ny, p.nz)
    assert struct.unpack_from("<7d", raw, 12)[2] == p.ni and struct.unpack_from("<7d", raw, 12)[6] == 1.25
    # Fortran order: iy fastest -> element (iy=-1, iz=-nz, ix=0, ic=1) first, then iy=0
    first = np.frombuffer(raw, "<c16", count=2, offset=68)
    assert first[0] == V[0, 0, 0, 0] and first[1] == V[0, 0, 0, 1]
    h, W = fields.read_restart(f)
    assert h.matches(p) and h.time == 1.25
    assert np.array_equal(W, V)


def test_restart_rejects_truncated_and_mismatch(tmp_path):
    p = dnsin.workload("small")
    V = initial.perturbed_laminar(p, 0.01, 0)
    f = tmp_path / "x.out"
    fields.write_restart(f, fields.Header.from_dnsin(p, 0.0), V)
    f.write_bytes(f.read_bytes()[:-16])
    with pytest.raises(ValueError):
        fields.read_restart(f)
    h = fields.Header.from_dnsin(p, 0.0)
    q = dnsin.workload("small")
    q.re = 4000.0000001
    assert not h.matches(q)


def test_runtimedata_roundtrip(tmp_path):
    vals = [0.004, 2.0000000123, 2.0, -8.5e-09, 1.6e-08, 4.0 / 3.0, 9.9999964e-04, 6.7e-15, 0.0, 0.1065154, 0.004]
    f = tmp_path / "Runtimedata"
    f.write_text(fields.runtimedata_line(vals) * 3)
    rows = fields.parse_runtimedata(f)
    assert rows.shape == (3, 11)
    assert np.array_equal(rows[0], np.array(vals))
    assert fields.stdout_line(vals).startswith("    0.0040")


def test_initial_field_properties():
    p = dnsin.workload("small")
    V = initial.perturbed_laminar(p, 0.01, 0)
    y = p.y()
    nz = p.nz
    np.testing.assert_allclose(V[0, 0, nz].real, y * (2 - y), rtol=0, atol=1e-15)
    # walls: v = 0 and eta = 0 at y=0 and y=2 (iy=0 -> index 1, iy=ny -> index ny+1)
    for iw in (1, p.ny + 1):
        assert np.abs(V[1, :, :, iw]).max() < 1e-15
    # Hermitian symmetry of the kx=0 plane
    for c in range(3):
        np.testing.assert_array_equal(V[c, 0, nz + 1:], np.conj(V[c, 0, nz - 1::-1]))
    # continuity i kx u + dv/dy + i kz w = 0, with dv/dy analytic
    s = 2 * (y - p.ymin) / (p.ymax - p.ymin)
    for ix, iz in ((1, 2), (3, -4), (0, 1)):
        kx, kz = p.alfa0 * ix, p.beta0 * iz
        v = V[1, ix, iz + nz]
        shape = (s * (2 - s)) ** 2
        c = v[p.ny // 2 + 1] / shape[p.ny // 2 + 1]
        dv = c * 2 * s * (2 - s) * (2 - 2 * s) * (2 / (p.ymax - p.ymin))
        div = 1j * kx * V[0, ix, iz + nz] + dv + 1j * kz * V[2, ix, iz + nz]
        assert np.abs(div).max() < 1e-15
    # deterministic
    assert np.array_equal(V, initial.perturbed_laminar(p, 0.01, 0))
    assert not np.array_equal(V, initial.perturbed_laminar(p, 0.01, 1))


def header_functions():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(chgpu_\w+)\s*\(", text))
    return sorted(names)


def test_capi_library_exports_every_declared_symbol():
    """libchgpu.so builds (nvcc cross-compiles here), loads without a GPU and
    exports each function the headers in include/ declare; the ctypes binding
    binds each one."""
    from channel_gb300 import build, lib

    build.build()
    L = ctypes.CDLL(str(build.LIB))
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    assert set(names) <= set(lib.SIGNATURES), set(names) - set(lib.SIGNATURES)
    assert lib.load_library() is not None


def test_library_fails_loudly_without_build(tmp_path, monkeypatch):
    from channel_gb300 import lib

    monkeypatch.setattr(lib, "_lib", None)
    monkeypatch.setenv("CHGPU_LIB", str(tmp_path / "missing.so"))
    with pytest.raises(FileNotFoundError):
        lib.load_library()
    monkeypatch.setattr(lib, "_lib", None)


def test_create_without_gpu_reports_error():
    """On a machine without a GPU the library returns an error code with a
    message rather than exiting or falling back to the CPU."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from channel_gb300 import Channel, ChannelError

    with pytest.raises(ChannelError) as e:
        Channel(dnsin.workload("small"))
    assert e.value.code in (-2, -3)


def test_fortran_interface_binds_declared_symbols():
    """Every BIND(C, name=...) of the Fortran interface module names a
    function the headers declare (the module is not compiled here: no
    gfortran), and the mirrored struct types list the C fields in order."""
    f90 = (ROOT / "channel_gb300" / "fortran" / "chgpu_interface.f90").read_text()
    bound = set(re.findall(r'BIND\(C,\s*name="(chgpu_\w+)"\)', f90))
    assert len(bound) >= 20
    assert bound <= set(header_functions()), bound - set(header_functions())
    text = (ROOT / "include" / "chgpu.h").read_text()
    body = re.search(r"typedef struct chgpu_params \{(.*?)\} chgpu_params;", text, re.S).group(1)
    c_fields = re.findall(r"\b(\w+)\s*[;,]", re.sub(r"/\*.*?\*/", "", body, flags=re.S))
    ftype = re.search(r"TYPE, BIND\(C\) :: chgpu_params(.*?)END TYPE", f90, re.S).group(1)
    f_fields = re.findall(r"::\s*([\w, ]+)", ftype)
    f_fields = [x.strip() for grp in f_fields for x in grp.split(",")]
    assert [c.lower() for c in c_fields] == [f.lower() for f in f_fields], (c_fields, f_fields)
