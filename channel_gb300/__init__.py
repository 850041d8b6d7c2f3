"""channel_gb300: the channel-flow RK3/Crank-Nicolson step of davecats/channel
(v-eta formulation, Fourier in x and z, compact finite differences in y) as
hand-written CUDA for GB300 (sm_103a), behind a C ABI (include/chgpu.h).

Python here is plumbing: a ctypes binding of libchgpu.so (``Channel``), the
dns.in / Dati.cart.out / Runtimedata formats, and the seeded initial-field
generator.  There is no CPU fallback: if the library is missing, loading
fails loudly.
"""
from .dnsin import DnsIn, padded_sizes, fft_fit, workload  # noqa: F401
from .lib import Channel, ChannelError, Ensemble, load_library, library_path, RK  # noqa: F401
