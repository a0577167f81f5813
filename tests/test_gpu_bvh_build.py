"""The BVH built on the device (dt_bvh_build.cu: Morton codes, radix sort, radix tree,
bottom-up boxes) against the host's binned-SAH tree: the same closest hits except at
exact ties, identical renders for the same seed, and the build time (the reference builds
an Embree BVH on the host for every scene, src/scene.cpp:17-43)."""
import time

import numpy as np
import pytest

from dtrt_gb300 import _abi, scenes

pytestmark = pytest.mark.gpu


def _rays(spec, n, seed=0):
    rng = np.random.default_rng(seed)
    org = rng.uniform(-2.5, 2.5, size=(n, 3))
    org[: n // 2] = np.array([0.0, 0.0, 4.0]) + rng.normal(scale=0.1, size=(n // 2, 3))
    d = rng.uniform(-1.0, 1.0, size=(n, 3)) - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, :3], r[:, 4:7], r[:, 7] = org, d, np.inf
    return r


def _scene(native, spec, builder):
    native.set_bvh_builder(builder)
    try:
        return native.NativeScene(spec)
    finally:
        native.set_bvh_builder("auto")


@pytest.mark.parametrize("cfg", ["c0", "c2", "c4"])
def test_device_tree_gives_the_host_trees_hits(native, cfg):
    if cfg == "c0":
        spec = scenes.config0(16, 16)
    elif cfg == "c2":
        spec = scenes.config2(16, 16, nder=1)
    else:
        spec = scenes.config4(5, side_scale=0.1, spp_scale=0.1)[0]
    rays = _rays(spec, 200000)
    with _scene(native, spec, "host") as a, _scene(native, spec, "device") as b:
        assert a.bvh_info()["builder"] == _abi.BVH_HOST and b.bvh_info()["builder"] == _abi.BVH_DEVICE
        ha, ta = a.trace_closest(rays)
        hb, tb = b.trace_closest(rays)
    hit = ha[:, 0] >= 0
    assert hit.sum() > 20000
    assert np.array_equal(hit, hb[:, 0] >= 0)
    same = ha[:, 0] == hb[:, 0]
    # a different triangle only at the same distance (a tie on a shared edge or vertex)
    assert np.all(ta[hit & ~same] == tb[hit & ~same]), "different hits at different distances"
    assert (~same[hit]).mean() < 1e-3
    assert np.array_equal(ta[hit], tb[hit]) or np.abs(ta[hit] - tb[hit]).max() == 0.0


def test_device_tree_renders_like_the_host_tree(native):
    spec = scenes.config2(48, 48, subdiv=4, nder=4)
    kw = dict(seed=9, spp=8, max_bounces=3, sppe=64, sppse=4)
    with _scene(native, spec, "host") as a, _scene(native, spec, "device") as b:
        ia, ib = a.render(**kw), b.render(**kw)
    # hits differ at most at exact ties, so the images agree but for those few paths
    assert np.abs(ia - ib).sum() <= 1e-3 * np.abs(ia).sum()


def test_device_tree_update_and_auto_choice(native):
    spec = scenes.config2(16, 16, subdiv=6, nder=1)  # 81924 triangles: AUTO builds on the device
    assert spec.num_triangles() >= _abi.BVH_DEVICE_MIN_TRIS
    with native.NativeScene(spec) as s:
        info = s.bvh_info()
        assert info["builder"] == _abi.BVH_DEVICE and info["num_nodes"] > 0
        img0 = s.render(seed=1, spp=4, max_bounces=2, sppe=0, sppse=0)
        v = spec.shapes[0].vertices
        spec.shapes[0].vertices = (v * 1.01).astype(np.float32)
        s.update(spec)  # same triangles: the device tree is built again
        assert s.bvh_info()["builder"] == _abi.BVH_DEVICE
        img1 = s.render(seed=1, spp=4, max_bounces=2, sppe=0, sppse=0)
    with native.NativeScene(spec) as fresh:
        img2 = fresh.render(seed=1, spp=4, max_bounces=2, sppe=0, sppse=0)
    assert not np.array_equal(img0, img1)
    assert np.abs(img1 - img2).sum() <= 1e-3 * np.abs(img2).sum()


def test_device_build_time(native):
    """Device against host build time from 1k to 328k triangles (printed; the device build
    must win at the larger sizes)."""
    rows = []
    for sub in (3, 4, 5, 6, 7):
        spec = scenes.config2(16, 16, subdiv=sub, nder=1)
        ms = {}
        for b in ("host", "device"):
            best = 1e9
            for _ in range(3):
                with _scene(native, spec, b) as s:
                    best = min(best, s.bvh_info()["ms_build"])
            ms[b] = best
        rows.append((spec.num_triangles(), ms["host"], ms["device"]))
        print(f"{spec.num_triangles():7d} triangles: host {ms['host']:.2f} ms, device {ms['device']:.2f} ms")
    assert rows[-1][2] < rows[-1][1]
