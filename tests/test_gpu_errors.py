"""Error paths of the device code, provoked on the host: a work queue forced below one
camera path's worst case reports DTRT_ERR_OVERFLOW, a tracking iteration cap of 0 reports
DTRT_ERR_STEP_CAP, and in both cases the scene stays usable once the setting is restored.
No kernel faults or hangs for any of this: pushes past capacity are dropped and flagged,
tracking loops stop at the cap."""
import numpy as np
import pytest

from dtrt_gb300 import _abi, scenes

pytestmark = pytest.mark.gpu


def test_queue_overflow_is_reported_and_recoverable(native):
    spec = scenes.config0(16, 16)  # moving null-bounded sphere: Lins and edge records
    kw = dict(seed=1, spp=8, max_bounces=5, sppe=0, sppse=4)
    with native.NativeScene(spec) as ns:
        ref = ns.render(**kw)
        ns.set_queue_capacity(8)
        with pytest.raises(_abi.DtrtError) as ei:
            ns.render(**kw)
        assert ei.value.status == _abi.DTRT_ERR_OVERFLOW
        ns.set_queue_capacity(0)
        again = ns.render(**kw)
    assert np.allclose(again, ref, rtol=1e-5, atol=1e-7)


def test_tracking_cap_is_reported_and_recoverable(native):
    spec = scenes.config1(16, 16)  # heterogeneous medium: delta and ratio tracking
    kw = dict(seed=2, spp=4, max_bounces=6, sppe=0, sppse=0)
    with native.NativeScene(spec) as ns:
        ref = ns.render(**kw)
        ns.set_tracking_cap(0)
        with pytest.raises(_abi.DtrtError) as ei:
            ns.render(**kw)
        assert ei.value.status == _abi.DTRT_ERR_STEP_CAP
        with pytest.raises(_abi.DtrtError) as ei:
            ns.render_adjoint(np.ones((16, 16, 3), np.float32), **kw)
        assert ei.value.status == _abi.DTRT_ERR_STEP_CAP
        ns.set_tracking_cap(10000)
        again = ns.render(**kw)
    assert np.allclose(again, ref, rtol=1e-5, atol=1e-7)


def test_invalid_options_are_rejected(native):
    spec = scenes.config0(8, 8)
    with native.NativeScene(spec) as ns:
        for bad in (dict(spp=-1), dict(max_bounces=-1), dict(sppse=-2)):
            kw = dict(seed=0, spp=1, max_bounces=2, sppe=0, sppse=0)
            kw.update(bad)
            with pytest.raises(_abi.DtrtError) as ei:
                ns.render(**kw)
            assert ei.value.status == _abi.DTRT_ERR_INVALID
