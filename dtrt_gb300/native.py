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

    def update(self, spec, rebuild_bvh=False):
        """Rebuild in place from a spec with the same triangles (dtrt_scene_update): the BVH
        is refit and unchanged-size device arrays are rewritten. Returns the update stats."""
        desc, keep = spec.to_desc()
        st = _abi.UpdateStats()
        _abi.check(self.lib.dtrt_scene_update(self.handle, ctypes.byref(desc),
                                              _abi.UPDATE_REBUILD_BVH if rebuild_bvh else 0, ctypes.byref(st)))
        self.spec = spec
        return st.as_dict()

    # ---------------------------------------------------------------- controls
    def set_edge_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        _abi.check(self.lib.dtrt_scene_set_edge_weights(self.handle, w.ctypes.data_as(_abi.c_float_p), w.size))

    def enable_counters(self, on=True):
        _abi.check(self.lib.dtrt_scene_enable_counters(self.handle, int(bool(on))))

    def set_queue_capacity(self, n):
        _abi.check(self.lib.dtrt_scene_set_queue_capacity(self.handle, int(n)))

    def set_camera_schedule(self, schedule):
        """'auto', 'megakernel' or 'wavefront' (dtrt_scene_set_camera_schedule)."""
        v = {"auto": _abi.CAMERA_AUTO, "megakernel": _abi.CAMERA_MEGAKERNEL, "wavefront": _abi.CAMERA_WAVEFRONT}
        _abi.check(self.lib.dtrt_scene_set_camera_schedule(self.handle, v[schedule] if isinstance(schedule, str)
                                                           else int(schedule)))

    def set_tracking_cap(self, n):
        _abi.check(self.lib.dtrt_scene_set_tracking_cap(self.handle, int(n)))

    def set_estimator_flags(self, flags):
        _abi.check(self.lib.dtrt_scene_set_estimator_flags(self.handle, int(flags)))

    def gradient_sizes(self):
        nv, nvert = ctypes.c_int64(), ctypes.c_int64()
        _abi.check(self.lib.dtrt_scene_gradient_sizes(self.handle, ctypes.byref(nv), ctypes.byref(nvert)))
        return nv.value, nvert.value

    def set_density(self, medium_id, density):
        d = np.ascontiguousarray(density, np.float32)
        _abi.check(self.lib.dtrt_scene_set_density(self.handle, int(medium_id), d.ctypes.data_as(_abi.c_float_p)))

    def set_density_derivatives(self, medium_id, grids):
        """grids: [nder, rz, ry, rx] per-voxel directions (None removes them)."""
        if grids is None:
            _abi.check(self.lib.dtrt_scene_set_density_derivatives(self.handle, int(medium_id), None))
            return
        g = np.ascontiguousarray(grids, np.float32)
        assert g.shape[0] == self.nder
        _abi.check(self.lib.dtrt_scene_set_density_derivatives(self.handle, int(medium_id),
                                                               g.ctypes.data_as(_abi.c_float_p)))

    def bvh_info(self):
        """How the scene's BVH was made (dtrt_scene_bvh_info): builder, nodes, depth, time."""
        bi = _abi.BvhInfo()
        _abi.check(self.lib.dtrt_scene_bvh_info(self.handle, ctypes.byref(bi)))
        return bi.as_dict()

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

    def render_primal(self, out=None, stream=None, **kw):
        """VolPathTracer image (dtrt_render_primal) into a host float32 [H, W, 3] array
        (allocated when None) or a device pointer given as an int."""
        o = kw.pop("options", None) or self.options(**kw)
        if isinstance(out, int) and not isinstance(out, bool):
            _abi.check(self.lib.dtrt_render_primal(self.handle, ctypes.byref(o), ctypes.c_void_p(out), 1,
                                                    ctypes.c_void_p(stream or 0)))
            return out
        if out is None:
            out = np.zeros(self.spec.out_shape()[1:], np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.shape == self.spec.out_shape()[1:]
        _abi.check(self.lib.dtrt_render_primal(self.handle, ctypes.byref(o), out.ctypes.data_as(ctypes.c_void_p), 0,
                                                ctypes.c_void_p(stream or 0)))
        return out

    def render_adjoint(self, d_image=None, image=True, density_grad=True, stream=None, device=False, **kw):
        """Reverse-mode density adjoint (dtrt_render_adjoint).

        Host mode (device=False): `d_image` is a float32 [H, W, 3] array; returns
        (image or None, d_density or None) as new host arrays.
        Device mode (device=True): `d_image`, `image` and `density_grad` are device
        pointers (ints, or None/0 to skip) on `stream`; returns None."""
        o = kw.pop("options", None) or self.options(**kw)
        vp = ctypes.c_void_p
        if device:
            def dptr(x):  # a device address given as a plain int; anything else (None, bool) means absent
                return vp(x) if type(x) is int and x != 0 else None
            _abi.check(self.lib.dtrt_render_adjoint(self.handle, ctypes.byref(o), dptr(d_image), dptr(image),
                                                     dptr(density_grad), None, 1, vp(stream or 0)))
            return None
        h, w = self.spec.out_shape()[1:3]
        img = np.zeros((h, w, 3), np.float32) if image else None
        grad = None
        if density_grad:
            grad = np.zeros(self.gradient_sizes()[0], np.float32)
        dimg = None
        if d_image is not None:
            dimg = np.ascontiguousarray(d_image, np.float32)
            assert dimg.shape == (h, w, 3)
        ptr = lambda a: a.ctypes.data_as(vp) if a is not None else None
        _abi.check(self.lib.dtrt_render_adjoint(self.handle, ctypes.byref(o), ptr(dimg), ptr(img), ptr(grad), None, 0,
                                                 vp(stream or 0)))
        return img, grad

    def render_vertex_adjoint(self, d_image, image=True, stream=None, device=False, vertex_grad=None, **kw):
        """Reverse-mode vertex-position adjoint (dtrt_render_adjoint with d_vertices).

        Host mode: `d_image` float32 [H, W, 3]; returns (image or None, grad [num_vertices, 3]).
        Device mode: `d_image`, `image`, `vertex_grad` are device pointers (ints); returns None."""
        o = kw.pop("options", None) or self.options(**kw)
        vp = ctypes.c_void_p
        if device:
            def dptr(x):
                return vp(x) if type(x) is int and x != 0 else None
            _abi.check(self.lib.dtrt_render_adjoint(self.handle, ctypes.byref(o), dptr(d_image), dptr(image), None,
                                                     dptr(vertex_grad), 1, vp(stream or 0)))
            return None
        h, w = self.spec.out_shape()[1:3]
        img = np.zeros((h, w, 3), np.float32) if image else None
        grad = np.zeros((self.gradient_sizes()[1], 3), np.float32)
        dimg = np.ascontiguousarray(d_image, np.float32)
        assert dimg.shape == (h, w, 3)
        ptr = lambda a: a.ctypes.data_as(vp) if a is not None else None
        _abi.check(self.lib.dtrt_render_adjoint(self.handle, ctypes.byref(o), ptr(dimg), ptr(img), None, ptr(grad), 0,
                                                 vp(stream or 0)))
        return img, grad

    def trace_closest(self, rays):
        rays = np.ascontiguousarray(rays, np.float32)
        if rays.ndim != 2 or rays.shape[1] != 8:
            raise ValueError("rays must be [n][8]: org.xyz, tmin, dir.xyz, tmax")
        n = rays.shape[0]
        hits = np.zeros((n, 2), np.int32)
        t = np.zeros(n, np.float32)
        _abi.check(self.lib.dtrt_trace_closest(self.handle, rays.ctypes.data_as(_abi.c_float_p), n,
                                               hits.ctypes.data_as(_abi.c_int_p), t.ctypes.data_as(_abi.c_float_p)))
        return hits, t


class Batch:
    """Many scenes rendered together (dtrt_batch_create / _launch / _destroy): a persistent
    launch, per-item launches over streams, or one replay wavefront over all items.

    items: list of (NativeScene, options, d_image_ptr, image_ptr, d_density_ptr[, d_vertices_ptr])
    with device pointers as ints (0 = none). The scenes and buffers must outlive the batch."""

    def __init__(self, items, autotune=True, graph=True, stream=None, tune_full=False, wavefront=False):
        self.lib = _abi.load()
        self.scenes = [it[0] for it in items]  # keep the scenes alive
        arr = (_abi.BatchItem * len(items))()
        for i, item in enumerate(items):
            sc, opts, dimg, img, dden = item[:5]
            arr[i].scene = sc.handle.value
            arr[i].opts = opts
            arr[i].d_image = dimg or None
            arr[i].image = img or None
            arr[i].d_density = dden or None
            arr[i].d_vertices = (item[5] if len(item) > 5 else 0) or None
        flags = (_abi.BATCH_AUTOTUNE if autotune else 0) | (_abi.BATCH_GRAPH if graph else 0) | \
            (_abi.BATCH_TUNE_FULL if tune_full else 0) | (_abi.BATCH_WAVEFRONT if wavefront else 0)
        h = ctypes.c_void_p()
        _abi.check(self.lib.dtrt_batch_create(arr, len(items), flags, ctypes.c_void_p(stream or 0), ctypes.byref(h)))
        self.handle = h

    def launch(self, stream=None):
        _abi.check(self.lib.dtrt_batch_launch(self.handle, ctypes.c_void_p(stream or 0)))

    def stats(self):
        st = _abi.BatchStats()
        _abi.check(self.lib.dtrt_batch_stats_get(self.handle, ctypes.byref(st)))
        return st.as_dict()

    def close(self):
        if getattr(self, "handle", None):
            self.lib.dtrt_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def device_count():
    return _abi.load().dtrt_device_count()


def rng_sequence(seed, idx, n):
    """n draws of the device PCG32 stream RndSampler(seed, idx) (dtrt_rng_sequence):
    raw uint32 outputs, FP32 uniforms and FP64 uniforms, each from a fresh stream."""
    lib = _abi.load()
    u = np.zeros(n, np.uint32)
    f = np.zeros(n, np.float32)
    d = np.zeros(n, np.float64)
    _abi.check(lib.dtrt_rng_sequence(int(seed), int(idx), int(n), u.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                     f.ctypes.data_as(_abi.c_float_p), d.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    return u, f, d


def set_bvh_builder(builder):
    """'auto', 'host' or 'device' (dtrt_set_bvh_builder): the BVH builder of scenes created
    or updated afterwards, process-wide."""
    v = {"auto": _abi.BVH_AUTO, "host": _abi.BVH_HOST, "device": _abi.BVH_DEVICE}
    _abi.check(_abi.load().dtrt_set_bvh_builder(v[builder] if isinstance(builder, str) else int(builder)))
