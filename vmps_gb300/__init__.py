"""GB300-native effective-Hamiltonian engine for block-sparse MPS algorithms.

Drop-in for the HxV / contract_L / contract_R hot path of VMPS (TNWorkers):
hand-written sm_103a CUDA kernels behind a C ABI (include/vmps_gb300.h),
with a Python front-end mirroring the reference's PivotMatrix / PivotVector API.
"""
from .blocks import Blocks, MpoSite, Symmetry  # noqa: F401

__version__ = "0.1.0"


def native():
    """The loaded native library (raises ImportError if it is not built)."""
    from . import _native
    return _native.lib()
