"""Device memory of the engines through a caller's allocator.

``set_device_allocator(alloc, free)`` routes every device allocation of the
library's engines (single-model, multi-model, the FWI loop) through two Python
callables, ``alloc(nbytes) -> int`` (a device pointer of the current device,
256-byte aligned, or 0 on failure) and ``free(ptr)``; ``None, None`` restores
cudaMalloc / cudaFree.  ``use_torch_allocator()`` routes it through PyTorch's
caching allocator, so the engines and the application share one memory pool.
A failing ``alloc`` makes the call that needed the memory raise FwiError
FWI_ERR_NOMEM and leaves the engine usable.
"""
from __future__ import annotations

from . import _capi
from ._capi import check

# Every ctypes callback pair ever installed, kept for the life of the process:
# a buffer is released through the allocator that made it, also after the
# allocator has been changed, so the library may call an old pair at any time.
_hooks = []


def set_device_allocator(alloc=None, free=None):
    if (alloc is None) != (free is None):
        raise ValueError("give both alloc and free, or neither")
    if alloc is None:
        check(_capi.lib().fwi_psv_set_device_allocator(_capi.ALLOC_FN(), _capi.FREE_FN(), None),
              "set_device_allocator")
        return

    def _alloc(nbytes, ctx):
        try:
            return int(alloc(int(nbytes)) or 0) or None
        except Exception:
            return None

    def _free(ptr, ctx):
        if ptr:
            free(int(ptr))

    hooks = (_capi.ALLOC_FN(_alloc), _capi.FREE_FN(_free))
    _hooks.append(hooks)
    check(_capi.lib().fwi_psv_set_device_allocator(hooks[0], hooks[1], None), "set_device_allocator")


def use_torch_allocator():
    """Device memory from torch.cuda's caching allocator (current device)."""
    import torch

    def alloc(nbytes):
        return torch.cuda.caching_allocator_alloc(nbytes)

    def free(ptr):
        torch.cuda.caching_allocator_delete(ptr)

    set_device_allocator(alloc, free)
