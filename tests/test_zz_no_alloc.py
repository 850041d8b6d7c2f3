"""chgpu_linsolve_noalloc -- the solve for callers that cannot allocate device
memory (hosts that own all device memory in their own arena) -- against the
handle-based chgpu_linsolve, through the C ABI, on two calls in a row.

Collected last (file name) so a run that stops at the first failure has run
every other test before this one."""
import ctypes as C

import numpy as np
import pytest

from helpers import per_field_rel

pytestmark = pytest.mark.gpu


def to_plane_major(V):
    """Restart-file layout (3, nx+1, 2nz+1, ny+3) -> device layout (3, ny+3, (nx+1)(2nz+1))."""
    return np.ascontiguousarray(V.transpose(0, 3, 1, 2).reshape(V.shape[0], V.shape[3], -1))


def from_plane_major(A, shape):
    return np.ascontiguousarray(A.reshape(shape[0], shape[3], shape[1], shape[2]).transpose(0, 2, 3, 1))


# the default constant flow rate in x; a constant spanwise flow rate (corrpz);
# the two CPI forms of the pressure gradient (meanpx updated in the call)
CASES = [{}, {"meanflowz": 0.2}, {"cpi": True, "cpi_type": 0, "gamma": 0.2, "meanflowx": 0.0},
         {"cpi": True, "cpi_type": 1, "gamma": 0.5, "meanflowx": 0.0}]


@pytest.mark.parametrize("over", CASES, ids=["flowrate_x", "flowrate_z", "cpi0", "cpi1"])
def test_linsolve_noalloc_matches_linsolve(gpu_lib, over):
    """Two calls in a row (different lambdas and fields) against the
    handle's solve: the field to 1e-12 and all seven in/out scalars."""
    import torch

    from channel_gb300 import RK, Channel, dnsin, initial
    from channel_gb300.lib import params_struct

    p = dnsin.workload("small")
    for k, v in over.items():
        setattr(p, k, v)
    V0 = initial.perturbed_laminar(p, 0.01, 0)
    g = Channel(p, "fp64")
    g.upload(V0)
    g.start()
    st = g.stats()
    params = params_struct(p)
    scalars = np.array([st.fr[0], st.fr[1], st.fr[2], st.corrpx, st.corrpz, st.meanpx, st.meanpz])
    err = C.create_string_buffer(256)
    for call, ode in enumerate(RK[:2]):
        g.buildrhs(ode, False)
        rhs_field = g.download()
        dev = torch.from_numpy(to_plane_major(rhs_field)).to("cuda")
        stream = torch.cuda.current_stream().cuda_stream
        lam = ode[0] / p.deltat
        rc = gpu_lib.chgpu_linsolve_noalloc(C.byref(params), lam, C.c_void_p(dev.data_ptr()),
                                           scalars.ctypes.data_as(C.POINTER(C.c_double)), C.c_void_p(stream),
                                           err, len(err))
        assert rc == 0, err.value
        g.linsolve(lam)
        ref = g.download()
        got = from_plane_major(dev.cpu().numpy(), ref.shape)
        assert max(per_field_rel(got, ref)) <= 1e-12, (call, per_field_rel(got, ref))
        st = g.stats()
        want = np.array([st.fr[0], st.fr[1], st.fr[2], st.corrpx, st.corrpz, st.meanpx, st.meanpz])
        scale = np.maximum(np.abs(want), 1e-3 * np.abs(want).max())
        assert float((np.abs(scalars - want) / scale).max()) <= 1e-11, (call, scalars, want)
    g.close()


def test_linsolve_noalloc_rejects_oversize(gpu_lib):
    import torch

    from channel_gb300 import dnsin
    from channel_gb300.lib import params_struct

    p = dnsin.workload("retau180")  # 4*191*128*128 doubles > 64 MiB of scratch
    field = torch.zeros((3, p.ny + 3, (p.nx + 1) * (2 * p.nz + 1)), dtype=torch.complex128, device="cuda")
    err = C.create_string_buffer(256)
    scalars = np.zeros(7)
    rc = gpu_lib.chgpu_linsolve_noalloc(C.byref(params_struct(p)), 1.0, C.c_void_p(field.data_ptr()),
                                       scalars.ctypes.data_as(C.POINTER(C.c_double)), None, err, len(err))
    assert rc == -1
    assert b"CHGPU_NOALLOC_SCRATCH_BYTES" in err.value
