"""The oracle's linear dynamics pinned by hydrodynamic stability theory.

A small disturbance of laminar Poiseuille flow that is an eigenmode of the
Orr-Sommerfeld / Squire operators evolves as exp(lambda t).  The eigenvalue
and the eigenfunctions are computed here independently of the oracle, by
Chebyshev collocation (the clamped fourth-derivative construction with
v = (1 - x^2) q, and the Squire equation for the wall-normal vorticity
forced by the mode's v), and the oracle's time step -- the convective
products with the mean flow in `convolutions`/`buildrhs`
(dnsdata.f90:487-673), the implicit viscous solves of `linsolve`
(linsolve_blocking.inc:3-107) and the RK3/CN scheme (dnsdata.f90:70-72) --
must reproduce lambda from the disturbance's own evolution.  The first case
is the two-dimensional Tollmien-Schlichting wave of Re = 10^4, alpha = 1,
the classic unstable mode (growth rate 0.0037 per unit time); the second an
oblique damped mode (alpha = beta = 1, Re = 5000), which also exercises the
eta equation and the u, w recovery."""
import numpy as np
import pytest

scipy_linalg = pytest.importorskip("scipy.linalg")


def cheb(N):
    """Chebyshev points x_j = cos(pi j / N) and the differentiation matrix."""
    x = np.cos(np.pi * np.arange(N + 1) / N)
    c = np.r_[2.0, np.ones(N - 1), 2.0] * (-1.0) ** np.arange(N + 1)
    dX = x[:, None] - x[None, :]
    D = np.outer(c, 1.0 / c) / (dX + np.eye(N + 1))
    return D - np.diag(D.sum(1)), x


def least_stable_mode(Re, a, b, N=120):
    """Least stable eigenvalue of Orr-Sommerfeld for U = 1 - x^2 on [-1, 1]
    (lambda = -i omega, disturbances exp(i(a x + b z) + lambda t)) and the
    mode's v (as q = v / (1 - x^2) and dq/dx on the Chebyshev points) and
    eta."""
    D, x = cheb(N)
    D2 = D @ D
    S = np.diag(np.r_[0.0, 1.0 / (1.0 - x[1:N] ** 2), 0.0])
    D3 = D2 @ D
    D4 = (np.diag(1.0 - x ** 2) @ D3 @ D - 8.0 * np.diag(x) @ D3 - 12.0 * D2) @ S
    D2i, D4i = D2[1:N, 1:N], D4[1:N, 1:N]
    I = np.eye(N - 1)
    k2 = a * a + b * b
    B = D2i - k2 * I
    U = 1.0 - x[1:N] ** 2
    A = (D4i - 2.0 * k2 * D2i + k2 * k2 * I) / Re - 1j * a * np.diag(U) @ B - 2j * a * I  # U'' = -2
    lam, vec = scipy_linalg.eig(A, B)
    k = np.argmax(lam.real)
    lam, vi = lam[k], vec[:, k]
    # Squire: (lambda + i a U - (D^2 - k^2)/Re) eta = -i b U' v, eta = 0 at the walls
    M = lam * I + 1j * a * np.diag(U) - B / Re
    eta = np.linalg.solve(M, -1j * b * (-2.0 * x[1:N]) * vi)
    q = np.zeros(N + 1, complex)
    q[1:N] = vi / (1.0 - x[1:N] ** 2)
    e = np.zeros(N + 1, complex)
    e[1:N] = eta
    return lam, x, q, D @ q, e


def interpolate(xn, fn, xe):
    """Barycentric interpolation on Chebyshev points (also just outside [-1, 1])."""
    N = len(xn) - 1
    w = np.r_[0.5, np.ones(N - 1), 0.5] * (-1.0) ** np.arange(N + 1)
    out = np.empty(len(xe), complex)
    for i, xx in enumerate(xe):
        d = xx - xn
        j = np.argmin(np.abs(d))
        if abs(d[j]) < 1e-14:
            out[i] = fn[j]
        else:
            t = w / d
            out[i] = (t @ fn) / t.sum()
    return out


def run(Re, a, b, steps, t1, dt=0.01):
    import pyoracle
    from channel_gb300 import dnsin, initial

    lam, x, q, dq, e = least_stable_mode(Re, a, b)
    p = dnsin.DnsIn(nx=1, ny=128, nz=1, alfa0=a, beta0=max(b, 1.0), re=Re, a=1.6, ymin=0.0, ymax=2.0,
                    meanflowx=4.0 / 3.0, deltat=dt, cflmax=0.0, nstep=steps)
    xx = p.y() - 1.0  # the channel y in [0, 2] is x + 1; U = y(2 - y) = 1 - x^2
    qv, dqv, ev = interpolate(x, q, xx), interpolate(x, dq, xx), interpolate(x, e, xx)
    v = (1.0 - xx ** 2) * qv
    dv = -2.0 * xx * qv + (1.0 - xx ** 2) * dqv
    s = 1e-6 / np.abs(v).max()  # linear regime: products of the disturbance ~1e-12
    v, dv, eta = s * v, s * dv, s * ev
    kb = b  # the mode (kx, kz) = (1, 1 or 0) in units of alfa0, beta0
    k2 = a * a + kb * kb
    iz = p.nz + (1 if b else 0)
    V0 = initial.perturbed_laminar(p, 0.0, 0)  # laminar U = y(2 - y)
    V0[0, 1, iz, :] = (1j * a * dv - 1j * kb * eta) / k2  # u, w from continuity and eta
    V0[1, 1, iz, :] = v
    V0[2, 1, iz, :] = (1j * kb * dv + 1j * a * eta) / k2
    o = pyoracle.Oracle(p, 4)
    o.set_field(V0)
    o.start()
    inner = slice(2, p.ny + 1)

    def probe(F):
        et = 1j * kb * F[0, 1, iz] - 1j * a * F[2, 1, iz]
        return np.vdot(V0[1, 1, iz, inner], F[1, 1, iz, inner]), np.vdot(eta[inner], et[inner]) if b else 0.0

    got = {}
    for k in range(1, steps + 1):
        o.step()
        if k in (t1, steps):
            got[k] = probe(o.field())
    T = (steps - t1) * dt
    lam_v = np.log(got[steps][0] / got[t1][0]) / T
    lam_e = np.log(got[steps][1] / got[t1][1]) / T if b else None
    return lam, lam_v, lam_e


def test_tollmien_schlichting_wave():
    lam, lam_v, _ = run(10000.0, 1.0, 0.0, 1000, 200)
    # the independent solver reproduces the classic eigenvalue of this case
    assert abs(lam.real - 0.0037397) < 2e-7 and abs(lam.imag + 0.2375265) < 2e-7, lam
    assert abs(lam_v - lam) / abs(lam) < 3e-5, (lam_v, lam)
    assert abs(lam_v.real - lam.real) / abs(lam.real) < 2e-3, (lam_v, lam)


def test_oblique_orr_sommerfeld_squire_mode():
    lam, lam_v, lam_e = run(5000.0, 1.0, 1.0, 600, 100)
    assert lam.real < 0  # damped at this Reynolds number
    assert abs(lam_v - lam) / abs(lam) < 3e-5, (lam_v, lam)
    assert abs(lam_e - lam) / abs(lam) < 3e-5, (lam_e, lam)
