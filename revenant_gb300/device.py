"""A thin host mirror of the reference's core/gpu Context/Buffer surface.

``Device`` wraps rv_context (core/gpu/context.h Context) and hands out
``Buffer`` objects wrapping rv_buffer (core/gpu/buffer.h Buffer with its three
MemoryKinds). Launches go straight to the rv_* entry points with the
buffers' device addresses; this module adds no compute of its own.
"""
import ctypes as C

import numpy as np

from . import abi
from .library import LibraryError, check, lib


class Buffer:
    def __init__(self, device, nbytes, kind=abi.MEMORY_DEVICE_LOCAL):
        self.device = device
        self.nbytes = int(nbytes)
        self.kind = kind
        handle = C.c_void_p()
        check(lib().rv_buffer_create(device.handle, self.nbytes, kind, C.byref(handle)))
        self.handle = handle
        self.address = lib().rv_buffer_address(handle)

    @property
    def ptr(self):
        return C.c_void_p(self.address)

    def upload(self, array, offset=0):
        a = np.ascontiguousarray(array)
        check(lib().rv_buffer_upload(self.handle, offset, a.ctypes.data_as(C.c_void_p), a.nbytes))

    def download(self, dtype, shape, offset=0):
        out = np.empty(shape, dtype=dtype)
        check(lib().rv_buffer_download(self.handle, offset, out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def clear(self):
        check(lib().rv_buffer_clear(self.handle))

    def free(self):
        if self.handle:
            lib().rv_buffer_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Device:
    """One context on one GPU (device index, or REVENANT_GPU_INDEX when -1)."""

    def __init__(self, index=-1):
        handle = C.c_void_p()
        status = lib().rv_context_create(index, C.byref(handle))
        if status != abi.RV_OK:
            raise LibraryError("rv_context_create failed (%d): %s" % (status, lib().rv_last_error().decode()))
        self.handle = handle
        info = abi.DeviceInfo()
        check(lib().rv_context_device_info(handle, C.byref(info)))
        self.info = info
        self.stream = lib().rv_context_stream(handle)

    def buffer(self, nbytes, kind=abi.MEMORY_DEVICE_LOCAL):
        return Buffer(self, max(int(nbytes), 4), kind)

    def array(self, array):
        """Upload a numpy array into a new device-local buffer."""
        a = np.ascontiguousarray(array)
        b = self.buffer(a.nbytes)
        b.upload(a)
        return b

    def zeros(self, nbytes):
        b = self.buffer(nbytes)
        b.clear()
        return b

    def copy_to_host(self, out, device_address):
        """Copy out.nbytes from a device address into numpy array `out`."""
        check(lib().rv_copy(self.handle, out.ctypes.data_as(C.c_void_p), C.c_void_p(device_address), out.nbytes))
        return out

    def synchronize(self):
        check(lib().rv_context_synchronize(self.handle))

    def close(self):
        if self.handle:
            lib().rv_context_destroy(self.handle)
            self.handle = None
