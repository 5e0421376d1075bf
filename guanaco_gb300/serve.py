"""Serving many tilt series at once: the request server of the C ABI
(gnc_server_*), with continuous batching on one GPU.

    srv = Server(budget_bytes=64 << 30, slots=8)
    rid = srv.submit(desc, projections, volume)     # returns at once
    info = srv.wait(rid)                            # volume is filled

Requests of any shape and parameters are queued, admitted as slots and device
memory free up, and run concurrently; plans and their captured CUDA graphs are
cached by shape.  Inputs and outputs are host arrays that must stay alive until
``wait`` returns; page-locked arrays (``pinned_empty``) make the copies
asynchronous.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .fbp import FbpDesc


class _PinnedBlock:
    """Exactly the array's bytes of page-locked host memory (gnc_host_alloc; a
    caching host allocator would round a 34 GB volume up to 64 GB of locked
    pages), freed when the last array over it is gone."""

    def __init__(self, shape, dtype):
        self._lib = _lib.load()
        nbytes = max(1, int(np.prod(shape, dtype=np.int64)) * dtype.itemsize)
        ptr = ctypes.c_void_p()
        _lib.check(self._lib.gnc_host_alloc(nbytes, ctypes.byref(ptr)))
        self._ptr = ptr.value
        self.__array_interface__ = dict(shape=tuple(int(n) for n in shape), typestr=dtype.str,
                                        data=(self._ptr, False), version=3)

    def __del__(self):
        if getattr(self, "_ptr", None):
            self._lib.gnc_host_free(self._ptr)
            self._ptr = None


def pinned_empty(shape, dtype=np.float32):
    """A page-locked host array of exactly its own size."""
    return np.asarray(_PinnedBlock(tuple(shape), np.dtype(dtype)))


class Server:
    """Request server on the current CUDA device."""

    def __init__(self, budget_bytes, slots=8):
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(self._lib.gnc_server_create(int(budget_bytes), int(slots), ctypes.byref(h)))
        self._h = h
        self._live = {}  # request id -> (desc, input, output): kept alive until wait

    def submit(self, desc: FbpDesc, inp, out):
        """Queue one request; returns its id."""
        a = np.ascontiguousarray(inp, dtype=np.float32)
        if a.shape != desc.input_shape:
            raise ValueError(f"input shape {a.shape} != {desc.input_shape}")
        if out.shape != desc.volume_shape or out.dtype != np.float32 or not out.flags.c_contiguous:
            raise ValueError("volume must be a C-contiguous float32 array of volume_shape")
        rid = ctypes.c_uint64()
        _lib.check(self._lib.gnc_server_submit(self._h, ctypes.byref(desc.c), a.ctypes.data,
                                               out.ctypes.data, ctypes.byref(rid)))
        self._live[rid.value] = (desc, a, out)
        return rid.value

    def wait(self, rid, timeout=None):
        """Wait for a request; returns its info dict (raises GncError, with the
        same dict as its ``info``, if it failed).  Returns None if the timeout
        passes first."""
        info = _lib.GncRequestInfo()
        st = self._lib.gnc_server_wait(self._h, int(rid), -1.0 if timeout is None else timeout,
                                       ctypes.byref(info))
        if st == _lib.GNC_ERR_PENDING:
            return None
        return self._collected(int(rid), st, info)

    def wait_any(self, timeout=None):
        """Wait for whichever request finishes next (in the order requests
        finish); returns ``(id, info)``, or None if none finished within the
        timeout or none is outstanding.  A failed request raises GncError with
        ``info`` and ``rid`` attached."""
        info = _lib.GncRequestInfo()
        rid = ctypes.c_uint64()
        st = self._lib.gnc_server_wait_any(self._h, -1.0 if timeout is None else timeout,
                                           ctypes.byref(rid), ctypes.byref(info))
        if st == _lib.GNC_ERR_PENDING:
            return None
        try:
            return rid.value, self._collected(rid.value, st, info)
        except _lib.GncError as e:
            e.rid = rid.value
            raise

    def _collected(self, rid, st, info):
        self._live.pop(rid, None)
        out = {"status": info.status, "graph": bool(info.graph),
               "device_error": bool(info.device_error), "t_submit": info.t_submit,
               "t_start": info.t_start, "t_done": info.t_done}
        try:
            _lib.check(st)
        except _lib.GncError as e:
            e.info = out  # the failed request's outcome, e.g. device_error
            raise
        return out

    def now(self):
        """Seconds on the server clock (the clock of the request times)."""
        return self._lib.gnc_server_now(self._h)

    def stats(self):
        s = _lib.GncServerStats()
        _lib.check(self._lib.gnc_server_get_stats(self._h, ctypes.byref(s)))
        return {name: getattr(s, name) for name, _ in s._fields_}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gnc_server_destroy(self._h)
            self._h = None
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()
