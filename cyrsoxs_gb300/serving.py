"""Serving engine (continuous batching) over the C ABI: cyr_server_*.

    srv = Server(slots=8, graphs=True, groups=True)
    rid = srv.submit(opts, optical, voxels, out)          # host arrays (keep them alive)
    rid = srv.submit(opts, optical, d_vox_ptr, d_out_ptr, device=True)
    latency_s, queue_s = srv.wait(rid)
    srv.close()

Each request computes exactly what cuda_main computes for it; requests in
different slots overlap on the GPU.  There is no CPU fallback: without the
native library or a device this raises.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native

GRAPHS = 1
GROUPS = 2


def _bind(L):
    if getattr(L, "_serving_bound", False):
        return L
    vp = ctypes.c_void_p
    L.cyr_server_create.argtypes = [ctypes.c_uint32, ctypes.c_size_t, ctypes.c_uint32, ctypes.POINTER(vp)]
    L.cyr_server_submit.argtypes = [vp, ctypes.POINTER(_native.CyrOptions), ctypes.POINTER(ctypes.c_float), vp, vp,
                                    ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint64)]
    L.cyr_server_poll.argtypes = [vp, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int)]
    L.cyr_server_wait.argtypes = [vp, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(ctypes.c_double)]
    L.cyr_server_stats.argtypes = [vp] + [ctypes.POINTER(ctypes.c_uint64)] * 4
    L.cyr_server_group_stats.argtypes = [vp] + [ctypes.POINTER(ctypes.c_uint64)] * 2
    L.cyr_server_destroy.argtypes = [vp]
    L._serving_bound = True
    return L


class Server:
    """A serving engine on the current CUDA device."""

    def __init__(self, slots: int = 8, hbm_budget: int = 0, graphs: bool = False, groups: bool = False):
        self._L = _bind(_native.lib())
        h = ctypes.c_void_p()
        flags = (GRAPHS if graphs else 0) | (GROUPS if groups else 0)
        _native.check(self._L.cyr_server_create(int(slots), int(hbm_budget), flags, ctypes.byref(h)))
        self._h = h
        self._keep = {}  # id -> objects the request reads or writes until it is done

    def submit(self, opts: _native.Options, optical: np.ndarray, voxels, out, device: bool = False) -> int:
        opt_arr = _native.optical_array(opts, optical)
        if device:
            vptr, optr = ctypes.c_void_p(int(voxels)), ctypes.c_void_p(int(out))
            keep = (opts, opt_arr)
        else:
            # the engine reads and writes these in place until the request is done: no copies
            _native.expect_size(voxels, _native.voxel_count(opts), "voxels [M][Z][Y][X][4]")
            _native.expect_size(out, _native.pattern_count(opts), "out [E][K][Ny][Nx]")
            vptr, optr = ctypes.c_void_p(voxels.ctypes.data), ctypes.c_void_p(out.ctypes.data)
            keep = (opts, opt_arr, voxels, out)
        rid = ctypes.c_uint64()
        _native.check(self._L.cyr_server_submit(self._h, opts.ref, _native.fptr(opt_arr), vptr, optr,
                                                1 if device else 0, ctypes.byref(rid)))
        self._keep[rid.value] = keep
        return rid.value

    def done(self, rid: int) -> bool:
        d = ctypes.c_int()
        _native.check(self._L.cyr_server_poll(self._h, rid, ctypes.byref(d)))
        return bool(d.value)

    def wait(self, rid: int):
        """Blocks until the request is done; returns (latency_s, queue_s); raises CyrError on failure."""
        lat, q = ctypes.c_double(), ctypes.c_double()
        try:
            _native.check(self._L.cyr_server_wait(self._h, rid, ctypes.byref(lat), ctypes.byref(q)))
        finally:
            self._keep.pop(rid, None)
        return lat.value, q.value

    def stats(self) -> dict:
        v = [ctypes.c_uint64() for _ in range(4)]
        _native.check(self._L.cyr_server_stats(self._h, *[ctypes.byref(x) for x in v]))
        g = [ctypes.c_uint64() for _ in range(2)]
        _native.check(self._L.cyr_server_group_stats(self._h, *[ctypes.byref(x) for x in g]))
        return dict(zip(("completed", "failed", "graph_replays", "graph_captures", "group_runs", "grouped_requests"),
                        (x.value for x in v + g)))

    def close(self):
        if self._h:
            _native.check(self._L.cyr_server_destroy(self._h))
            self._h = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
