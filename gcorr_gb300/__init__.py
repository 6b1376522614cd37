"""GB300-native FX correlator engine: FxKernel-compatible host API over libgxcorr.so.

The compute path is CUDA only (sm_103a kernels in csrc/, exposed through the C
ABI of include/gxc.h).  This package holds the host-side mirror of the
reference FxKernel interface, the synthetic workload generator and the
visibility text I/O.
"""
from .fxkernel import FxKernel, make_config  # noqa: F401
from ._lib import GxcError, lib, LIB_PATH  # noqa: F401


def build(verbose: bool = False, force: bool = False) -> str:
    from .buildlib import build as _b
    return _b(verbose=verbose, force=force)
