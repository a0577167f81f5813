"""In-place scene rebuild with cached topology (dtrt_scene_update).

* an update from the same description refits the BVH to itself: bit-identical renders,
  every device array reused;
* after moving vertices, the updated scene (refit BVH, cached edge adjacency) answers
  closest-hit queries and renders (image and derivative images) like a scene created
  from scratch on the moved vertices, for the same seed;
* a deformation that wrecks the refit tree's surface-area cost (more than 2x its cost at
  build time) triggers a full rebuild, and the flag forces one;
* topology changes are rejected and leave the scene as it was;
* estimator flags and per-voxel density directions survive an update.
"""
import ctypes

import numpy as np
import pytest

from dtrt_gb300 import _abi, native, scenes

pytestmark = pytest.mark.gpu


def sphere(displaced, sigma=0.01, size=64, nder=4):
    return scenes.config2(width=size, height=size, subdiv=4, nder=nder, seed=2, displaced=displaced, sigma=sigma)


def random_rays(n, seed):
    rng = np.random.default_rng(seed)
    o = rng.normal(size=(n, 3)) * 2.5
    target = rng.uniform(-0.8, 0.8, size=(n, 3))
    d = target - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tmin, tmax = np.zeros((n, 1)), np.full((n, 1), 1e30)
    return np.concatenate([o, tmin, d, tmax], axis=1).astype(np.float32)  # org, tmin, dir, tmax


KW = dict(spp=8, max_bounces=3, sppe=2, sppse=2)


def test_update_with_same_description_is_bit_exact():
    spec = sphere(False)
    with native.NativeScene(spec) as ns:
        before = ns.render(seed=5, **KW)
        st = ns.update(spec)
        after = ns.render(seed=5, **KW)
    print(st)
    assert st["bvh_refit"] == 1 and st["sah_ratio"] == 1.0
    assert st["buffers_allocated"] == 0 and st["buffers_reused"] > 10
    assert np.array_equal(before, after)


@pytest.mark.parametrize("sigma", [0.01, 0.05])
def test_moved_vertices_match_a_fresh_scene(sigma):
    base, moved = sphere(False), sphere(True, sigma=sigma)
    rays = random_rays(1 << 16, 7)
    with native.NativeScene(base) as ns, native.NativeScene(moved) as fresh:
        st = ns.update(moved)
        hu, tu = ns.trace_closest(rays)
        hf, tf = fresh.trace_closest(rays)
        iu = ns.render(seed=11, **KW)
        ifr = fresh.render(seed=11, **KW)
    print(st)
    assert st["sah_ratio"] >= 1.0 and st["bvh_refit"] == 1
    same = np.all(hu == hf, axis=1)
    print("rays", rays.shape[0], "hit mismatches", int((~same).sum()), "hits", int((hf[:, 0] >= 0).sum()))
    assert (hf[:, 0] >= 0).sum() > rays.shape[0] // 4  # the rays do hit the sphere and the stage
    assert (~same).sum() <= 2  # only exact ties between triangles may resolve differently
    assert np.array_equal(tu[same], tf[same])
    # same hits, same edge lists, same sampling: the renders agree except where a tie flips
    diff = np.any(iu != ifr, axis=-1)
    print("pixels differing per image", diff.reshape(diff.shape[0], -1).sum(1))
    assert diff.mean() <= 1e-3
    assert np.abs(iu - ifr).sum() <= 1e-3 * np.abs(ifr).sum()


def test_wrecked_tree_is_rebuilt_and_flag_forces_rebuild():
    base = sphere(False)
    folded = sphere(False)
    v = folded.shapes[0].vertices.astype(np.float64)
    v[:, 1] += 1.5 * np.sign(np.sin(6 * np.pi * v[:, 0]))  # stripes of the sphere pushed up and down
    folded.shapes[0].vertices = v.astype(np.float32)
    rays = random_rays(1 << 14, 9)
    with native.NativeScene(base) as ns:
        st = ns.update(folded)
        with native.NativeScene(folded) as fresh:
            hu, tu = ns.trace_closest(rays)
            hf, tf = fresh.trace_closest(rays)
        print(st)
        assert st["bvh_refit"] == 0 and st["sah_ratio"] > 2.0
        same = np.all(hu == hf, axis=1)
        assert (~same).sum() <= 2 and np.array_equal(tu[same], tf[same])
        st2 = ns.update(base, rebuild_bvh=True)
        assert st2["bvh_refit"] == 0
        st3 = ns.update(base)
        assert st3["bvh_refit"] == 1 and st3["sah_ratio"] == 1.0


def test_topology_changes_are_rejected_and_leave_the_scene_unchanged():
    spec = sphere(False)
    with native.NativeScene(spec) as ns:
        before = ns.render(seed=3, **KW)
        lib, h = ns.lib, ns.handle
        # flipped winding of one triangle: same counts, different index list
        bad = sphere(False)
        f = bad.shapes[0].indices.copy()
        f[0] = f[0][::-1]
        bad.shapes[0].indices = f
        # another derivative width
        other_nder = sphere(False, nder=1)
        # fewer shapes
        fewer = sphere(False)
        fewer.shapes = fewer.shapes[:1]
        fewer.emitters = []
        for s in (bad, other_nder, fewer):
            desc, keep = s.to_desc()
            assert lib.dtrt_scene_update(h, ctypes.byref(desc), 0, None) == _abi.DTRT_ERR_INVALID
            print(lib.dtrt_last_error())
        desc, keep = spec.to_desc()
        assert lib.dtrt_scene_update(h, ctypes.byref(desc), 0x10, None) == _abi.DTRT_ERR_INVALID
        # a description that passes the topology check but fails the build (negative edge weight)
        w = np.full(len(spec.shapes), -1.0, np.float32)
        desc.edge_weights = w.ctypes.data_as(_abi.c_float_p)
        assert lib.dtrt_scene_update(h, ctypes.byref(desc), 0, None) == _abi.DTRT_ERR_INVALID
        after = ns.render(seed=3, **KW)
    assert np.array_equal(before, after)


def test_update_keeps_density_directions_and_flags():
    res, size = 16, 32
    spec = scenes.config3(width=size, height=size, res=res, nder=1, seed=3, param_slots=False, nblobs=4)
    dirs = np.random.default_rng(1).normal(size=(1, res, res, res)).astype(np.float32)
    kw = dict(spp=8, max_bounces=4, sppe=0, sppse=4)
    with native.NativeScene(spec) as ns:
        ns.set_estimator_flags(_abi.EST_SCATTER_SEGMENT_FROM_ORIGIN)
        ns.set_density_derivatives(0, dirs)
        before = ns.render(seed=9, **kw)
        st = ns.update(spec)
        after = ns.render(seed=9, **kw)
        assert st["bvh_refit"] == 1
        assert np.array_equal(before, after)
        assert np.abs(after[1]).sum() > 0
        # a different density resolution is a topology change
        other = scenes.config3(width=size, height=size, res=res + 2, nder=1, seed=3, param_slots=False, nblobs=4)
        with pytest.raises(_abi.DtrtError):
            ns.update(other)
        assert np.array_equal(ns.render(seed=9, **kw), before)


def test_render_scene_reuse_matches_fresh_builds(monkeypatch):
    """The pydtrt flat-argument path with reuse_scene on: the second render (vertices
    scaled) updates the kept scene and renders the same image as a scene built anew."""
    torch = pytest.importorskip("torch")
    from test_pydtrt_host import _pydtrt_c2
    from dtrt_gb300 import dtrt
    from dtrt_gb300.pydtrt import scene_renderer as sr
    _, scene = _pydtrt_c2(32, 32)
    args = sr.serialize_scene(scene)
    integ = dtrt.VolPathTracerAD()
    opts = dtrt.RenderOptions(4, 8, 3, 2, 2, True)
    monkeypatch.setattr(sr, "reuse_scene", True)
    monkeypatch.setattr(sr, "_kept", None)
    img1 = sr.render_scene(integ, opts, *args)
    kept = sr._kept
    args[12] = (args[12] * 1.05).contiguous()
    img2 = sr.render_scene(integ, opts, *args)
    assert sr._kept is kept
    monkeypatch.setattr(sr, "reuse_scene", False)
    fresh = sr.render_scene(integ, opts, *args)
    assert sr._kept is None
    assert torch.equal(img2, fresh)
    assert not torch.equal(img1[0], img2[0])


def test_render_buffers_pass_to_the_next_scene():
    """A destroyed scene's render work buffers go to the next scene created on the device:
    renders are unchanged by the reuse and by releasing the cached buffers."""
    spec = sphere(False)
    lib = _abi.load()
    with native.NativeScene(spec) as a:
        ref = a.render(seed=2, **KW)
        ref_adj = a.render_adjoint(np.ones((64, 64, 3), np.float32), seed=2, spp=4, max_bounces=3, sppe=0)[0]
    with native.NativeScene(spec) as b:  # takes a's buffers
        assert np.array_equal(b.render(seed=2, **KW), ref)
        assert np.array_equal(b.render_adjoint(np.ones((64, 64, 3), np.float32), seed=2, spp=4, max_bounces=3,
                                               sppe=0)[0], ref_adj)
    assert lib.dtrt_release_cached_memory() == _abi.DTRT_OK
    assert lib.dtrt_release_cached_memory() == _abi.DTRT_OK  # nothing cached: still fine
    with native.NativeScene(spec) as c:  # fresh buffers
        assert np.array_equal(c.render(seed=2, **KW), ref)
