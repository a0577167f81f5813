"""The reference's example scene examples/glass_1 (Phong apple, rough-dielectric tank
around a homogeneous medium, area light, floor) as a committed fixture of its flat
render_scene arguments (tests/golden/make_examples.py). On the CPU: the Mitsuba loader
reproduces the fixture from the reference's own files when they are present, and the
fixture parses into the scene description the renderer consumes."""
import os

import numpy as np
import pytest
import torch

from dtrt_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "glass_1_args.pt")
REF_ROOT = "/root/reference"


def load_fixture():
    return torch.load(FIXTURE, weights_only=False)


def _same(a, b):
    if torch.is_tensor(a) or torch.is_tensor(b):
        return torch.is_tensor(a) and torch.is_tensor(b) and a.shape == b.shape and torch.equal(a, b)
    if isinstance(a, (list, tuple)):
        return isinstance(b, (list, tuple)) and len(a) == len(b) and all(_same(x, y) for x, y in zip(a, b))
    return a == b


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_ROOT, "examples", "glass_1", "scene.xml")),
                    reason="reference checkout not present")
def test_loader_reproduces_fixture_from_reference_files():
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_examples
    args, integ = make_examples.glass_1_args(REF_ROOT)
    fx = load_fixture()
    assert integ == fx["integrator"]
    assert len(args) == len(fx["args"])
    for i, (a, b) in enumerate(zip(args, fx["args"])):
        assert _same(a, b), f"argument {i} differs"


def test_fixture_scene_description():
    from dtrt_gb300 import dtrt
    from dtrt_gb300.pydtrt import scene_renderer
    fx = load_fixture()
    dtrt.set_nder(fx["nder"])
    spec = scene_renderer.scene_spec(*fx["args"])
    assert spec.nder == 4 and (spec.camera.width, spec.camera.height) == (256, 256)
    assert sorted(b.type for b in spec.bsdfs) == sorted([_abi.BSDF_ROUGHDIELECTRIC, _abi.BSDF_PHONG,
                                                         _abi.BSDF_DIFFUSE, _abi.BSDF_DIFFUSE])
    assert [m.type for m in spec.media] == [_abi.MEDIUM_HOMOGENEOUS]
    assert len(spec.emitters) == 1 and spec.emitters[0].type == _abi.EMITTER_AREA
    apple = spec.shapes[0]
    nv = apple.vertices.shape[0]
    vel = np.asarray(apple.velocities).reshape(-1, nv, 3)
    assert np.allclose(vel[0], [1, 0, 0]) and np.allclose(vel[1], [0, 1, 0]) and np.allclose(vel[2], [0, 0, 1])
    rd = [b for b in spec.bsdfs if b.type == _abi.BSDF_ROUGHDIELECTRIC][0]
    assert np.allclose(np.asarray(rd.d_alpha), [0, 0, 0, 0.1])


def test_fixture_renders_on_the_oracle(oracle):
    from dtrt_gb300 import dtrt
    from dtrt_gb300.pydtrt import scene_renderer
    fx = load_fixture()
    dtrt.set_nder(fx["nder"])
    spec = scene_renderer.scene_spec(*fx["args"])
    img = oracle.render(spec, seed=1, spp=1, max_bounces=4, sppe=8, sppse=2)
    assert img.shape == (5, 256, 256, 3) and np.isfinite(img).all()
    assert (np.abs(img).sum(axis=(1, 2, 3)) > 0).all()  # image and all four derivative images
