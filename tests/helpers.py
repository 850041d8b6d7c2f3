"""Shared helpers of the test suite."""
import numpy as np


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def per_field_rel(a, b):
    """Relative L2 error of each velocity component (u, v, w)."""
    return [rel_l2(a[c], b[c]) for c in range(a.shape[0])]


# Runtimedata columns (dnsdata.f90:878): time; dU/dy and dW/dy at both walls;
# flow rate x; dp/dx; flow rate z; dp/dz; CFL*dt; dt.  The vector quantities
# (wall shear, flow rate, pressure gradient) are compared in their own norm:
# a spanwise component that is round-off around zero (no spanwise forcing)
# is measured against the streamwise one, as FP64 itself would resolve it.
# The pressure gradient at constant flow rate is meanpx + (meanflowx - fr)/fc
# (linsolve_blocking.inc:86-92): a flow-rate difference ~1e-3 of its terms
# divided by the unit-forcing flow rate, which turns a 1e-16 rounding of the
# field into ~1e-10 of dp/dx in any FP64 evaluation order; its bar is ten
# times the others'.
LINE_GROUPS = [([0], 1.0), ([1, 2, 3, 4], 1.0), ([5, 7], 1.0), ([6, 8], 10.0), ([9], 1.0), ([10], 1.0)]


def line_close(a, b, tol):
    a, b = np.asarray(a), np.asarray(b)
    err = np.zeros_like(b)
    for g, widen in LINE_GROUPS:
        scale = max(float(np.abs(b[g]).max()), 1e-300)
        err[g] = np.abs(a[g] - b[g]) / scale / widen
    return float(err.max()) <= tol, float(err.max())


def profiles(V):
    """Mean U(y) and rms of u, v, w (postpro/history/var_history.f90:37-84)."""
    U = V[0, 0, V.shape[2] // 2, :].real
    w = np.ones(V.shape[1])
    w[1:] = 2.0
    D = V.copy()
    D[:, 0, V.shape[2] // 2, :] = 0.0
    rms = np.sqrt(np.einsum("x,cxzy->cy", w, np.abs(D) ** 2))
    return U, rms
