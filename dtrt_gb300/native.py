"""Python handle over the C ABI: build a device scene from a SceneSpec, render
forward-mode images, read counters, run BVH queries.

Everything here calls libdtrt_gb300.so; there is no CPU fallback. Importing works
on a machine without a GPU (the library loads), but scene creation then fails with
DTRT_ERR_NO_DEVICE.
"""
import ctypes

import numpy as np

from . import _abi


class NativeScene:
    """A device-resident scene (dtrt_scene_create / dtrt_scene_destroy)."""

    def __init__(self, spec):
        self.lib = _abi.load()
        self.spec = spec
        self.nder = spec.nder
        desc, keep = spec.to_desc()
        h = ctypes.c_void_p()
        _abi.check(self.lib.dtrt_scene_create(ctypes.byref(desc), ctypes.byref(h)))
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self.lib.dtrt_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---------------------------------------------------------------- controls
    def set_edge_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        _abi.check(self.lib.dtrt_scene_set_edge_weights(self.handle, w.ctypes.data_as(_abi.c_float_p), w.size))

    def enable_counters(self, on=True):
        _abi.check(self.lib.dtrt_scene_enable_counters(self.handle, int(bool(on))))

    def set_queue_capacity(self, n):
        _abi.check(self.lib.dtrt_scene_set_queue_capacity(self.handle, int(n)))

    def set_tracking_cap(self, n):
        _abi.check(self.lib.dtrt_scene_set_tracking_cap(self.handle, int(n)))

    def last_stats(self):
        st = _abi.RenderStats()
        _abi.check(self.lib.dtrt_scene_last_stats(self.handle, ctypes.byref(st)))
        return st.as_dict()

    # ---------------------------------------------------------------- render
    @staticmethod
    def options(seed=0, spp=1, max_bounces=1, sppe=0, sppse=0, quiet=True, mode=-1, ddist_coeff=0.0):
        return _abi.RenderOptions(int(seed), int(spp), int(max_bounces), int(sppe), int(sppse), int(bool(quiet)),
                                  int(mode), float(ddist_coeff))

    def render(self, out=None, stream=None, **kw):
        """Render into a host float32 array [(nder+1), H, W, 3] (allocated when
        `out` is None) or into a device pointer given as an int (`out`)."""
        o = kw.pop("options", None) or self.options(**kw)
        if isinstance(out, int):
            _abi.check(self.lib.dtrt_render_fwd(self.handle, ctypes.byref(o), ctypes.c_void_p(out), 1,
                                                 ctypes.c_void_p(stream or 0)))
            return out
        if out is None:
            out = np.zeros(self.spec.out_shape(), np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.shape == self.spec.out_shape()
        _abi.check(self.lib.dtrt_render_fwd(self.handle, ctypes.byref(o), out.ctypes.data_as(ctypes.c_void_p), 0,
                                             ctypes.c_void_p(stream or 0)))
        return out

    def trace_closest(self, rays):
        rays = np.ascontiguousarray(rays, np.float32)
        n = rays.shape[0]
        hits = np.zeros((n, 2), np.int32)
        t = np.zeros(n, np.float32)
        _abi.check(self.lib.dtrt_trace_closest(self.handle, rays.ctypes.data_as(_abi.c_float_p), n,
                                               hits.ctypes.data_as(_abi.c_int_p), t.ctypes.data_as(_abi.c_float_p)))
        return hits, t


def device_count():
    return _abi.load().dtrt_device_count()
