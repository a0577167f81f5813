"""TEST INFRASTRUCTURE — ctypes loader of the CPU oracle (oracle/_build/liboracle.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module. It builds the library on first use when the toolchain is present.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def build(force=False):
    if force or not os.path.exists(LIB):
        subprocess.run(["make", "-s", "-C", HERE, "-j4"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        from dtrt_gb300 import _abi
        build()
        L = ctypes.CDLL(LIB)
        SD = ctypes.POINTER(_abi.SceneDesc)
        RO = ctypes.POINTER(_abi.RenderOptions)
        fp = ctypes.POINTER(ctypes.c_float)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.oracle_render.argtypes = [SD, RO, fp, ctypes.c_int]
        L.oracle_render_primary_edges.argtypes = [SD, RO, fp, ctypes.c_int]
        L.oracle_render_ext.argtypes = [SD, RO, fp, ctypes.c_int, ctypes.c_uint, ctypes.POINTER(fp)]
        L.oracle_render_primal.argtypes = [SD, RO, fp, ctypes.c_int]
        L.oracle_render_integrator.argtypes = [SD, RO, fp, ctypes.c_int, ctypes.c_int]
        L.oracle_pcg32.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_uint32)]
        L.oracle_pcg32.restype = None
        L.oracle_next1d.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, dp]
        L.oracle_next1d.restype = None
        L.oracle_trace_closest.argtypes = [SD, dp, ctypes.c_int, ip, dp]
        L.oracle_edge_summary.argtypes = [SD, ip, dp, ip, dp]
        L.oracle_closed_form.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.oracle_closed_form.restype = ctypes.c_double
        L.oracle_bsdf_albedo.argtypes = [ctypes.POINTER(_abi.BsdfDesc), ctypes.c_double, ctypes.c_int,
                                         ctypes.c_uint64, dp]
        L.oracle_last_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def _opts(seed, spp, max_bounces, sppe, sppse, mode=-1, ddist=0.0):
    from dtrt_gb300 import _abi
    return _abi.RenderOptions(seed, spp, max_bounces, sppe, sppse, 1, mode, ddist)


def render(spec, seed=0, spp=4, max_bounces=5, sppe=0, sppse=10, mode=-1, ddist=0.0, nthreads=0):
    """Image + derivatives float32[(nder+1), H, W, 3] from the FP64 CPU oracle."""
    desc, keep = spec.to_desc()
    out = np.zeros(spec.out_shape(), np.float32)
    o = _opts(seed, spp, max_bounces, sppe, sppse, mode, ddist)
    r = lib().oracle_render(ctypes.byref(desc), ctypes.byref(o), out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                            nthreads)
    if r:
        raise RuntimeError("oracle_render: " + lib().oracle_last_error().decode())
    return out


INTEGRATORS = {"volpath": 0, "path": 1, "direct": 2}


def render_integrator(spec, integrator, seed=0, spp=4, max_bounces=5, sppe=0, sppse=10, mode=-1, ddist=0.0,
                      nthreads=0):
    """render() with the reference's other AD integrators: 'volpath' (VolPathTracerAD),
    'path' (PathTracerAD) or 'direct' (DirectAD); the last two on surface scenes only."""
    desc, keep = spec.to_desc()
    out = np.zeros(spec.out_shape(), np.float32)
    o = _opts(seed, spp, max_bounces, sppe, sppse, mode, ddist)
    r = lib().oracle_render_integrator(ctypes.byref(desc), ctypes.byref(o),
                                       out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), nthreads,
                                       INTEGRATORS[integrator])
    if r:
        raise RuntimeError("oracle_render_integrator: " + lib().oracle_last_error().decode())
    return out


def render_ext(spec, seed=0, spp=4, max_bounces=5, sppe=0, sppse=10, mode=-1, ddist=0.0, nthreads=0, est_flags=0,
               density_dirs=None):
    """render() with estimator flags and per-medium per-voxel density directions
    (density_dirs: {medium_id: float32[nder, rz, ry, rx]})."""
    desc, keep = spec.to_desc()
    out = np.zeros(spec.out_shape(), np.float32)
    o = _opts(seed, spp, max_bounces, sppe, sppse, mode, ddist)
    fp = ctypes.POINTER(ctypes.c_float)
    nm = len(spec.media)
    arr = (fp * max(nm, 1))()
    held = []
    for mi, g in (density_dirs or {}).items():
        g = np.ascontiguousarray(g, np.float32)
        held.append(g)
        arr[mi] = g.ctypes.data_as(fp)
    r = lib().oracle_render_ext(ctypes.byref(desc), ctypes.byref(o), out.ctypes.data_as(fp), nthreads, est_flags,
                                arr if density_dirs else None)
    if r:
        raise RuntimeError("oracle_render_ext: " + lib().oracle_last_error().decode())
    return out


def render_primal(spec, seed=0, spp=4, max_bounces=5, nthreads=0):
    """VolPathTracer image float32[H, W, 3] from the FP64 CPU oracle."""
    desc, keep = spec.to_desc()
    out = np.zeros(spec.out_shape()[1:], np.float32)
    o = _opts(seed, spp, max_bounces, 0, 0)
    r = lib().oracle_render_primal(ctypes.byref(desc), ctypes.byref(o),
                                   out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), nthreads)
    if r:
        raise RuntimeError("oracle_render_primal: " + lib().oracle_last_error().decode())
    return out


def render_primary_edges(spec, seed=0, sppe=64, max_bounces=5, nthreads=0):
    desc, keep = spec.to_desc()
    out = np.zeros((spec.nder, spec.height, spec.width, 3), np.float32)
    o = _opts(seed, 0, max_bounces, sppe, 0)
    r = lib().oracle_render_primary_edges(ctypes.byref(desc), ctypes.byref(o),
                                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), nthreads)
    if r:
        raise RuntimeError("oracle_render_primary_edges: " + lib().oracle_last_error().decode())
    return out


def pcg32(seed, idx, n):
    out = np.zeros(n, np.uint32)
    lib().oracle_pcg32(seed, idx, n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    return out


def next1d(seed, idx, n):
    out = np.zeros(n, np.float64)
    lib().oracle_next1d(seed, idx, n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return out


def trace_closest(spec, rays):
    desc, keep = spec.to_desc()
    rays = np.ascontiguousarray(rays, np.float64)
    n = rays.shape[0]
    hits = np.zeros((n, 2), np.int32)
    t = np.zeros(n, np.float64)
    r = lib().oracle_trace_closest(ctypes.byref(desc), rays.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n,
                                   hits.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                   t.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    if r:
        raise RuntimeError(lib().oracle_last_error().decode())
    return hits, t


def edge_summary(spec):
    desc, keep = spec.to_desc()
    ne, np_ = ctypes.c_int(), ctypes.c_int()
    tl, ps = ctypes.c_double(), ctypes.c_double()
    r = lib().oracle_edge_summary(ctypes.byref(desc), ctypes.byref(ne), ctypes.byref(tl), ctypes.byref(np_),
                                  ctypes.byref(ps))
    if r:
        raise RuntimeError(lib().oracle_last_error().decode())
    return ne.value, tl.value, np_.value, ps.value


def closed_form(which, a, b=0.0):
    return lib().oracle_closed_form(which, a, b)


def bsdf_albedo(bsdf_spec, cos_i, nsamples=200000, seed=0):
    from dtrt_gb300 import _abi
    b = _abi.BsdfDesc()
    b.type = bsdf_spec.type
    b.diffuse[:] = list(bsdf_spec.diffuse)
    b.specular[:] = list(bsdf_spec.specular)
    b.exponent, b.alpha = bsdf_spec.exponent, bsdf_spec.alpha
    b.int_ior, b.ext_ior = bsdf_spec.int_ior, bsdf_spec.ext_ior
    out = np.zeros(3)
    lib().oracle_bsdf_albedo(ctypes.byref(b), cos_i, nsamples, seed, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return out
