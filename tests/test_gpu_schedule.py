"""Camera-path schedules of forward-mode renders (dtrt_scene_set_camera_schedule).

The wavefront schedule runs one launch per path vertex over the live paths only; the
megakernel carries each path to its end in one thread. Both execute the same vertex code
with the same random numbers per path, and both sum a pixel's paths in path order, so
the images, derivative images and work counters must agree exactly.
"""
import numpy as np
import pytest

from dtrt_gb300 import _abi, native, scenes

pytestmark = pytest.mark.gpu

CASES = {
    "c0": (lambda: scenes.config0(48, 48, nder=1), dict(spp=16, max_bounces=5, sppe=64, sppse=4)),
    "c1": (lambda: scenes.config1(48, 48, res=32, nder=3), dict(spp=32, max_bounces=10, sppe=0, sppse=4)),
    "c2": (lambda: scenes.config2(40, 40, subdiv=3, nder=8), dict(spp=16, max_bounces=4, sppe=64, sppse=4)),
    "c3": (lambda: scenes.config3(40, 40, res=32, nder=4, nblobs=8), dict(spp=16, max_bounces=16, sppe=0, sppse=4)),
}
KEYS = ("rays", "node_visits", "tri_tests", "grid_lookups", "edge_records", "lins_records", "li_tasks")


@pytest.mark.parametrize("name", sorted(CASES))
def test_wavefront_equals_megakernel(name):
    make, kw = CASES[name]
    with native.NativeScene(make()) as ns:
        ns.enable_counters(True)
        out = {}
        for sched in ("megakernel", "wavefront"):
            ns.set_camera_schedule(sched)
            img = ns.render(seed=21, **kw)
            out[sched] = (img, ns.last_stats())
    (a, sa), (b, sb) = out["megakernel"], out["wavefront"]
    assert np.abs(a[0]).sum() > 0
    assert np.array_equal(a, b)
    for k in KEYS:
        assert sa[k] == sb[k], k
    # the wavefront launches one kernel per vertex level plus start and accumulation
    assert sb["kernel_launches"] > sa["kernel_launches"]


def test_schedule_argument_checks():
    with native.NativeScene(scenes.config0(8, 8, nder=1)) as ns:
        assert ns.lib.dtrt_scene_set_camera_schedule(ns.handle, 3) == _abi.DTRT_ERR_INVALID
        assert ns.lib.dtrt_scene_set_camera_schedule(ns.handle, -1) == _abi.DTRT_ERR_INVALID
        ns.set_camera_schedule("auto")
        img = ns.render(seed=1, spp=4, max_bounces=3, sppe=0, sppse=0)
        assert np.isfinite(img).all()


def test_density_adjoint_wavefront_equals_megakernel():
    """The density replay under both schedules: the same image (pass A sums in path
    order) and the same gradient up to the order of its FP32 atomic sums."""
    spec = scenes.config3(40, 40, res=16, nder=1, param_slots=False, nblobs=6)
    dimg = np.random.default_rng(4).normal(size=(40, 40, 3)).astype(np.float32)
    kw = dict(seed=13, spp=16, max_bounces=8, sppe=0, sppse=0)
    out = {}
    with native.NativeScene(spec) as ns:
        for sched in ("megakernel", "wavefront"):
            ns.set_camera_schedule(sched)
            out[sched] = ns.render_adjoint(dimg, **kw)
            assert ns.last_stats()["camera_schedule"] == {"megakernel": 1, "wavefront": 2}[sched]
    (ia, ga), (ib, gb) = out["megakernel"], out["wavefront"]
    assert np.array_equal(ia, ib) and ia.sum() > 0
    assert np.abs(ga).max() > 0
    assert np.abs(ga - gb).max() <= 1e-4 * np.abs(ga).max()


@pytest.mark.parametrize("name", ["c0", "c1"])
def test_primal_wavefront_equals_megakernel(name):
    """dtrt_render_primal under both schedules: same li_step code and random numbers per
    path, pixel sums in path order."""
    make, kw = CASES[name]
    out = {}
    with native.NativeScene(make()) as ns:
        ns.enable_counters(True)
        for sched in ("megakernel", "wavefront"):
            ns.set_camera_schedule(sched)
            img = ns.render_primal(seed=17, spp=kw["spp"], max_bounces=kw["max_bounces"])
            out[sched] = (img, ns.last_stats())
    (a, sa), (b, sb) = out["megakernel"], out["wavefront"]
    assert sa["camera_schedule"] == 1 and sb["camera_schedule"] == 2
    assert a.sum() > 0 and np.array_equal(a, b)
    for k in ("rays", "node_visits", "tri_tests", "grid_lookups"):
        assert sa[k] == sb[k], k


def test_full_size_c1_schedules_equal():
    """The forward workload at its full size (512x512, 64 spp, depth 10, nder 3: 16.7 M paths
    in 11 batches of 1.5 M) renders the same image and derivative images under both
    schedules, and AUTO picks the wavefront."""
    spec = scenes.config1(512, 512, res=64, nder=3)
    kw = dict(spp=64, max_bounces=10, sppe=1024, sppse=10)
    with native.NativeScene(spec) as ns:
        auto = ns.render(seed=3, **kw)
        st = ns.last_stats()
        assert st["camera_schedule"] == 2 and st["batches"] > 1
        ns.set_camera_schedule("megakernel")
        mega = ns.render(seed=3, **kw)
    assert np.abs(auto[0]).sum() > 0 and np.array_equal(auto, mega)
