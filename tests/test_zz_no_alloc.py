"""dtrt_render_fwd_noalloc: the render entry point for callers that cannot call
cudaMalloc (runtimes that own every device allocation, fixed start-up memory budgets).
Its work buffers live in a static device array inside the library, so the result must
match the allocating entry point dtrt_render_fwd on the same seed, on every call
(the array keeps the previous call's contents; the render must clear what it needs).

This file is collected last on purpose: if it fails, the other tests have already run.
"""
import ctypes

import numpy as np
import pytest

from dtrt_gb300 import _abi, scenes

pytestmark = pytest.mark.gpu


def _render(lib, handle, spec, fn, **kw):
    o = _abi.RenderOptions(kw.get("seed", 0), kw["spp"], kw["max_bounces"], kw["sppe"], kw["sppse"], 1, -1, 0.0)
    out = np.zeros(spec.out_shape(), np.float32)
    st = getattr(lib, fn)(handle, ctypes.byref(o), out.ctypes.data_as(ctypes.c_void_p), 0, None)
    return st, out


@pytest.mark.parametrize("cfg", ["c0", "c2"])
def test_noalloc_matches_allocating_render(native, cfg):
    lib = _abi.load()
    if cfg == "c0":
        spec = scenes.config0(32, 32)
        kw = dict(spp=32, max_bounces=5, sppe=64, sppse=4)
    else:
        spec = scenes.config2(48, 48, subdiv=3, nder=4)
        kw = dict(spp=8, max_bounces=3, sppe=64, sppse=4)
    with native.NativeScene(spec) as s:
        st, ref = _render(lib, s.handle, spec, "dtrt_render_fwd", seed=11, **kw)
        assert st == 0, lib.dtrt_last_error()
        for call in range(2):  # two calls in a row: state left by the first must not leak
            st, got = _render(lib, s.handle, spec, "dtrt_render_fwd_noalloc", seed=11, **kw)
            assert st == 0, lib.dtrt_last_error()
            assert np.isfinite(got).all()
            np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-6, err_msg=f"call {call}")
            assert np.abs(got).sum() > 0


def test_noalloc_device_output_and_size_limit(native):
    import torch
    lib = _abi.load()
    spec = scenes.config0(16, 16)
    kw = dict(spp=16, max_bounces=4, sppe=0, sppse=2)
    with native.NativeScene(spec) as s:
        st, ref = _render(lib, s.handle, spec, "dtrt_render_fwd", seed=5, **kw)
        assert st == 0
        dev = torch.zeros(spec.out_shape(), dtype=torch.float32, device="cuda")
        o = _abi.RenderOptions(5, kw["spp"], kw["max_bounces"], kw["sppe"], kw["sppse"], 1, -1, 0.0)
        assert lib.dtrt_render_fwd_noalloc(s.handle, ctypes.byref(o), ctypes.c_void_p(dev.data_ptr()), 1, None) == 0
        np.testing.assert_allclose(dev.cpu().numpy(), ref, rtol=1e-5, atol=1e-6)
    big = scenes.config0(128, 128)  # 16384 pixels > DTRT_NOALLOC_MAX_PIXELS
    with native.NativeScene(big) as s:
        st, _ = _render(lib, s.handle, big, "dtrt_render_fwd_noalloc", seed=0, spp=1, max_bounces=1, sppe=0, sppse=0)
        assert st == 1
        assert b"maximum is 4096" in lib.dtrt_last_error()


def test_noalloc_largest_layout_and_limits(native):
    """The largest layout the array must hold (8 derivative slots, 64x64 = 4096 pixels,
    host output with its staging copy), and the option limits it rejects."""
    lib = _abi.load()
    spec = scenes.config2(64, 64, subdiv=3, nder=8)
    kw = dict(spp=4, max_bounces=3, sppe=16, sppse=4)
    with native.NativeScene(spec) as s:
        st, ref = _render(lib, s.handle, spec, "dtrt_render_fwd", seed=3, **kw)
        assert st == 0, lib.dtrt_last_error()
        for call in range(2):
            st, got = _render(lib, s.handle, spec, "dtrt_render_fwd_noalloc", seed=3, **kw)
            assert st == 0, lib.dtrt_last_error()
            np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-6, err_msg=f"call {call}")
        assert s.last_stats()["camera_schedule"] == _abi.CAMERA_MEGAKERNEL
        for bad in (dict(kw, max_bounces=32), dict(kw, sppse=8193)):
            st, _ = _render(lib, s.handle, spec, "dtrt_render_fwd_noalloc", seed=3, **bad)
            assert st == 1
            assert b"max_bounces <= 31 and sppse <= 8192" in lib.dtrt_last_error()
