"""Reynolds-stress budget spectra on the device (chgpu_tke_*) against the numpy
restatement of postpro/tke/uiuj_spectra.f90 (oracle/tke_oracle.py), through
the C ABI: two samples of a stepped field, with and without a pressure field,
at the 32x64x32 workload and at an uneven size (transform lengths 24 and 48,
a radix-3 stage)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TERMS = ["var", "prod", "psdiss", "ttrsp", "vdiff", "pstrain", "ptrsp", "PHIttrsp", "PHIvdiff", "PHIptrsp"]


def random_pressure(p, seed):
    rng = np.random.default_rng(seed)
    shape = (p.nx + 1, 2 * p.nz + 1, p.ny + 3)
    return 1e-3 * (rng.normal(size=shape) + 1j * rng.normal(size=shape))


def run_case(p, with_pressure, timestwo):
    import pyoracle
    import tke_oracle
    from channel_gb300 import Channel, initial

    V0 = initial.perturbed_laminar(p, 0.05, 2, kmax=min(p.nx, p.nz, 6))
    o = pyoracle.Oracle(p)
    with Channel(p, "fp64") as g:
        g.upload(V0)
        g.start()
        g.step()
        V1 = g.download()
        nz = p.nz
        U = V1[0, 0, nz].real * 0.97
        W = V1[2, 0, nz].real + 0.01
        Pm = np.linspace(0.0, 1e-3, p.ny + 3) if with_pressure else None
        g.tke_reset(U, W, Pm)
        T = tke_oracle.TkeOracle(p, o, U, W, Pm)
        for s in range(2):
            V = g.download()
            P = random_pressure(p, s) if with_pressure else None
            g.tke_accumulate(P)
            T.accumulate(V, P)
            g.step()
        mean, sp, pr, n = g.tke_result(timestwo)
    om, osp, opr = T.result(timestwo)
    assert n == 2
    np.testing.assert_allclose(mean, om, rtol=1e-12, atol=1e-12 * np.abs(om).max())
    for t, name in enumerate(TERMS):
        ref = osp[:, t]
        scale = max(float(np.abs(ref).max()), 1e-300)
        err = float(np.abs(sp[:, t] - ref).max()) / scale
        if not with_pressure and name in ("pstrain", "ptrsp", "PHIptrsp"):
            assert np.abs(sp[:, t]).max() == 0.0, name
            continue
        if name == "PHIttrsp":
            assert np.abs(sp[:, t]).max() == 0.0
            continue
        assert err <= 1e-10, (name, err)
        perr = float(np.abs(pr[:, t] - opr[:, t]).max()) / max(float(np.abs(opr[:, t]).max()), 1e-300)
        assert perr <= 1e-10, (name, perr)


@pytest.mark.parametrize("with_pressure,timestwo", [(True, False), (False, True)])
def test_tke_spectra_small(gpu_lib, with_pressure, timestwo):
    from channel_gb300 import dnsin

    run_case(dnsin.workload("small"), with_pressure, timestwo)


def test_tke_spectra_uneven(gpu_lib):
    from channel_gb300 import dnsin

    p = dnsin.DnsIn(nx=11, ny=20, nz=13, alfa0=1.3, beta0=2.1, re=3000.0, a=1.6, ymin=0.0, ymax=2.0,
                    meanflowx=4.0 / 3.0, deltat=0.003, cflmax=0.0, nstep=3)
    run_case(p, True, False)


def test_tke_profile_of_var_is_rms(gpu_lib):
    """The kz-sum of the var spectra of uu, vv, ww is the rms profile of the
    fluctuation (postpro/history/var_history.f90's weights), a check that
    needs no oracle."""
    from channel_gb300 import Channel, dnsin, initial

    p = dnsin.workload("small")
    with Channel(p, "fp64") as g:
        g.upload(initial.perturbed_laminar(p, 0.05, 3))
        g.start()
        g.step()
        V = g.download()
        U = V[0, 0, p.nz].real
        W = V[2, 0, p.nz].real
        g.tke_reset(U, W)
        g.tke_accumulate()
        _, _, pr, _ = g.tke_result()
    w = np.ones(p.nx + 1)
    w[1:] = 2.0
    D = V.copy()
    D[0, 0, p.nz] -= U
    D[2, 0, p.nz] -= W
    for c in range(3):
        rms2 = np.einsum("x,xzy->y", w, np.abs(D[c]) ** 2)
        np.testing.assert_allclose(pr[c, 0], rms2, rtol=1e-12, atol=1e-14 * rms2.max())
