"""GB300-native (sm_103a) engine for the 2-D elastic P-SV FWI hot path.

The compute runs in ``_lib/libfwi_psv.so`` (hand-written CUDA kernels behind
the C ABI of ``include/fwi_psv.h``); this package is the host-side mirror of
the reference's interface: problem setup, the batched forward/backward
engine, and a torch.autograd wrapper.
"""
from . import _capi
from ._capi import FwiError, FwiLibraryMissing
from .problem import Problem

__all__ = ["Problem", "FwiError", "FwiLibraryMissing", "Engine", "_capi"]


def __getattr__(name):
    if name == "Engine":
        from .engine import Engine
        return Engine
    raise AttributeError(name)
