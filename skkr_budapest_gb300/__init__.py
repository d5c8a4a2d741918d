"""GB300-native 2D Brillouin-zone integration of the screened-KKR scattering
path operator (the per-(E,k) tau / CPA loop of laszloffy/skkr_budapest).

Compute runs in libskkr_gpu.so (hand-written sm_103a CUDA behind the C ABI
of include/skkr_gpu.h); this package is the host-side mirror of the
reference's cpacoord interface plus seeded synthetic inputs.
"""
from .api import Context, cpacoord  # noqa: F401

__all__ = ["Context", "cpacoord"]
