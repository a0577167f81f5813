"""Host logic of the reference-facing Python layer, on the CPU (no device calls): a scene
written with the pydtrt classes goes through serialize_scene and build_native_scene (the
reference's flat-argument path, scene_renderer.py) to the same description as the scene
generator, which the FP64 oracle renders identically; SceneManager offsets and parameter
updates follow the flat layout (scene_manager.py:146-224)."""
import math

import numpy as np
import pytest
import torch

from dtrt_gb300 import native, scenes


class _Capture:
    """Stands in for the device scene: records the description it is built from."""
    last = None

    def __init__(self, spec):
        _Capture.last = spec
        self.handle = None

    def close(self):
        pass


def _pydtrt_c2(width=24, height=24):
    from dtrt_gb300.pydtrt import scene_objects as so
    ref = scenes.config2(width, height, subdiv=2, nder=1)
    cam = so.Camera(torch.tensor([0.0, 0.0, 4.0]), torch.tensor([0.0, 0.0, 0.0]), torch.tensor([0.0, 1.0, 0.0]),
                    torch.tensor([45.0]), 1e-2, (width, height))
    shapes = [so.Shape(torch.tensor(np.ascontiguousarray(s.vertices)), torch.tensor(np.ascontiguousarray(s.indices)),
                       None, None, bsdf_id=s.bsdf_id)
              for s in ref.shapes]
    bsdfs = [so.BSDF_diffuse(torch.tensor(b.diffuse, dtype=torch.float32)) for b in ref.bsdfs]
    lights = [so.AreaLight(ref.emitters[0].shape_id, torch.tensor([10.0, 10.0, 10.0]))]
    return ref, so.Scene(cam, shapes, bsdfs, [], [], lights)


def test_flat_arguments_build_the_generator_scene(monkeypatch, oracle):
    from dtrt_gb300.pydtrt import scene_renderer as sr
    monkeypatch.setattr(native, "NativeScene", _Capture)
    ref, scene = _pydtrt_c2()
    args = sr.serialize_scene(scene)
    assert args[0:5] == [3, 3, 1, 0, 0]
    sr.build_native_scene(*args)
    spec = _Capture.last
    assert len(spec.shapes) == 3 and spec.shapes[ref.emitters[0].shape_id].light_id == 0
    for a, b in zip(spec.shapes, ref.shapes):
        assert np.array_equal(np.asarray(a.vertices), b.vertices) and np.array_equal(np.asarray(a.indices), b.indices)
    assert np.allclose(np.asarray(spec.camera.cam_to_world).reshape(4, 4), ref.camera.cam_to_world, atol=1e-6)
    assert np.allclose(np.asarray(spec.camera.cam_to_ndc).reshape(3, 3), ref.camera.cam_to_ndc, atol=1e-6)
    kw = dict(seed=3, spp=4, max_bounces=3, sppe=0, sppse=0)
    a, b = oracle.render(spec, **kw), oracle.render(ref, **kw)
    assert np.allclose(a[0], b[0], rtol=1e-5, atol=1e-6) and a[0].sum() > 0


def test_scene_manager_offsets_and_translation(monkeypatch):
    from dtrt_gb300.pydtrt import scene_manager as sm, scene_renderer as sr
    from dtrt_gb300 import dtrt
    monkeypatch.setattr(dtrt, "nder", 2)
    _, scene = _pydtrt_c2()
    args = sr.serialize_scene(scene)
    T = [[sm.SceneTransform("SHAPE_TRANSLATE", torch.tensor([1.0, 0.0, 0.0]), 0)],
         [sm.SceneTransform("BSDF_VARY", "diffuse", 0, torch.tensor([0.1, 0.1, 0.1]))]]
    m = sm.SceneManager(args, T)
    assert m.offsets["shape"] == [12, 21, 30]
    assert m.offsets["bsdf"] == [39, 42, 45] and m.offsets["emitter"] == [48] and m.offsets["weight"] == 52
    v0 = args[12].clone()
    m.set_arguments(torch.tensor([0.25, 0.5]))
    assert torch.allclose(m.args[12], v0 + torch.tensor([0.25, 0.0, 0.0]))
    assert torch.allclose(torch.as_tensor(m.args[40]), torch.as_tensor(args[40]) + 0.05)
    vel = m.args[20].reshape(2, -1, 3)  # velocity seeds: slot 0 moves the sphere along +x
    assert torch.allclose(vel[0], torch.tensor([1.0, 0.0, 0.0]).expand_as(vel[0]))
    assert float(vel[1].abs().sum()) == 0.0
    m.reset()
    assert torch.allclose(m.args[12], v0)


def test_obj_and_vol_roundtrip(tmp_path):
    from dtrt_gb300.pydtrt import loaders
    v, f = scenes.icosphere(1, 0.5)
    p = tmp_path / "m.obj"
    with open(p, "w") as fh:
        for x in v:
            fh.write(f"v {x[0]} {x[1]} {x[2]}\n")
        for t in f + 1:
            fh.write(f"f {t[0]} {t[1]} {t[2]}\n")
    (mesh,) = loaders.load_obj(str(p))  # vertices are renumbered in order of first use
    tri = np.asarray(mesh.vertices)[np.asarray(mesh.indices)]
    assert np.allclose(tri, v[f], atol=1e-6) and mesh.uvs is None and mesh.normals is None
    g, _ = scenes.blob_grid(6, 2, 1)
    scenes.write_vol(str(tmp_path / "g.vol"), g, (0, 0, 0), (1, 1, 1))
    back, vmin, vmax = scenes.read_vol(str(tmp_path / "g.vol"))
    assert np.array_equal(back, g) and vmax == (1.0, 1.0, 1.0)


def test_render_scene_reuses_the_device_scene(monkeypatch):
    """reuse_scene: the second render_scene call with the same triangles updates the kept
    scene in place; changed triangles build a new scene and close the kept one."""
    from dtrt_gb300 import _abi
    from dtrt_gb300.pydtrt import scene_renderer as sr

    class FakeNative:
        made = []

        def __init__(self, spec):
            FakeNative.made.append(self)
            self.spec, self.updates, self.closed = spec, 0, False

        def update(self, spec, rebuild_bvh=False):
            same = len(spec.shapes) == len(self.spec.shapes) and all(
                np.array_equal(np.asarray(a.indices), np.asarray(b.indices)) for a, b in zip(spec.shapes, self.spec.shapes))
            if not same:
                raise _abi.DtrtError(_abi.DTRT_ERR_INVALID, "scene update: triangles differ")
            self.spec, self.updates = spec, self.updates + 1
            return {}

        def set_edge_weights(self, w):
            pass

        def close(self):
            self.closed = True

    class Integrator:
        def render(self, scene, options, image):
            self.scene = scene

    monkeypatch.setattr(native, "NativeScene", FakeNative)
    monkeypatch.setattr(sr, "reuse_scene", True)
    monkeypatch.setattr(sr, "_kept", None)
    _, scene = _pydtrt_c2()
    args = sr.serialize_scene(scene)
    it = Integrator()
    sr.render_scene(it, None, *args)
    first = it.scene
    args[12] = args[12] + 0.01  # vertices of shape 0 move
    sr.render_scene(it, None, *args)
    assert it.scene is first and first.native.updates == 1 and len(FakeNative.made) == 1
    assert np.allclose(np.asarray(first.spec.shapes[0].vertices), np.asarray(args[12]))
    f = args[13].clone()
    f[0] = f[0].flip(0)  # one triangle's winding: other triangles
    args[13] = f
    sr.render_scene(it, None, *args)
    assert it.scene is not first and first.native.closed and len(FakeNative.made) == 2
    monkeypatch.setattr(sr, "reuse_scene", False)
    sr.render_scene(it, None, *args)  # reuse off: the kept scene is released, the new one closed after use
    assert FakeNative.made[1].closed and FakeNative.made[2].closed and sr._kept is None
