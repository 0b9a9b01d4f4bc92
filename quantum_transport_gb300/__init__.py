"""GB300-native batched recursive Green's function (RGF) for quantum transport.

The compute path is ``libqtgpu.so`` (hand-written sm_103a CUDA behind the
C-ABI in include/qt_rgf.h); this package holds its build, the ctypes binding
and the host-side mirror of the reference's Fortran interface.
"""
from .devices import ChainDevice, make_chain_device  # noqa: F401

__all__ = ["ChainDevice", "make_chain_device", "build", "rgf"]


def build(force=False):
    from .build import build as _b
    return _b(force=force)
