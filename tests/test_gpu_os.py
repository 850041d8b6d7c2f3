"""The GPU step against linear stability theory: the Orr-Sommerfeld /
Squire eigenmodes of tests/test_oracle_os.py stepped through the C ABI in
the FP64 and double-float paths reproduce their eigenvalues as the oracle
does."""
import numpy as np
import pytest

from test_oracle_os import interpolate, least_stable_mode

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "fp64dd"])
@pytest.mark.parametrize("Re,a,b,steps,t1", [(10000.0, 1.0, 0.0, 1000, 200), (5000.0, 1.0, 1.0, 600, 100)])
def test_eigenmode_rates(gpu_lib, prec, Re, a, b, steps, t1):
    from channel_gb300 import Channel, dnsin, initial

    dt = 0.01
    lam, x, q, dq, e = least_stable_mode(Re, a, b)
    p = dnsin.DnsIn(nx=1, ny=128, nz=1, alfa0=a, beta0=1.0, re=Re, a=1.6, ymin=0.0, ymax=2.0,
                    meanflowx=4.0 / 3.0, deltat=dt, cflmax=0.0, nstep=steps)
    xx = p.y() - 1.0
    qv, dqv, ev = interpolate(x, q, xx), interpolate(x, dq, xx), interpolate(x, e, xx)
    v = (1.0 - xx ** 2) * qv
    dv = -2.0 * xx * qv + (1.0 - xx ** 2) * dqv
    s = 1e-6 / np.abs(v).max()
    v, dv, eta = s * v, s * dv, s * ev
    k2 = a * a + b * b
    iz = p.nz + (1 if b else 0)
    V0 = initial.perturbed_laminar(p, 0.0, 0)
    V0[0, 1, iz, :] = (1j * a * dv - 1j * b * eta) / k2
    V0[1, 1, iz, :] = v
    V0[2, 1, iz, :] = (1j * b * dv + 1j * a * eta) / k2
    g = Channel(p, prec)
    g.upload(V0)
    g.start()
    inner = slice(2, p.ny + 1)
    got = {}
    for k in range(1, steps + 1):
        g.step(sync=False)
        if k in (t1, steps):
            F = g.download()
            got[k] = np.vdot(V0[1, 1, iz, inner], F[1, 1, iz, inner])
    g.close()
    lam_v = np.log(got[steps] / got[t1]) / ((steps - t1) * dt)
    assert abs(lam_v - lam) / abs(lam) < 3e-5, (lam_v, lam)
