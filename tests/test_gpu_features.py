"""Every scene feature of the drop-in API rendered on the GPU against the FP64 oracle:
Phong (src/bsdf/phong.cpp:19-95), rough dielectric above the alpha floor
(src/bsdf/roughdielectric.cpp:9-206), AreaLightEx (src/emitter/area2.cpp:5-44),
two-sided area lights (src/emitter/area.cpp:5-7), camera translation and rotation
velocities (src/camera.cpp:92-127), the crop window (Camera.set_rect, src/dtrt.cpp:35-37),
albedo grids (src/medium/heterogeneous.h:20-25) and the volume edge term
EVolumeBoundary2 (src/integrator/differential/volpathAD.cpp:207-305); and the device
PCG32 generator bit for bit against the committed fixture (src/sampler.cpp:3-41)."""
import json
import os

import numpy as np
import pytest

import statcheck
from dtrt_gb300 import _abi, scenes
from dtrt_gb300.scenes import BsdfSpec, EmitterSpec, MediumSpec, PhaseSpec, SceneSpec, ShapeSpec

pytestmark = pytest.mark.gpu

RUNS = 16
# runs per side, reduced to 16 batch means by statcheck (edge-term estimates are heavy-tailed)
GPU_RUNS, CPU_RUNS = 256, 64


def _pair(native, oracle, spec, kw, gruns=GPU_RUNS, cruns=CPU_RUNS):
    with native.NativeScene(spec) as s:
        g = np.stack([s.render(seed=100 + k, **kw) for k in range(gruns)])
    c = np.stack([oracle.render(spec, seed=900 + k, **kw) for k in range(cruns)])
    return g, c


def _translate(nv, nder, slot, axis=0):
    v = np.zeros((nder * nv, 3), np.float32)
    v[slot * nv:(slot + 1) * nv, axis] = 1.0
    return v


def _sphere_scene(bsdf, nder, slot_translate, w=32, h=32, subdiv=2, radius=0.7, center=(0.0, 0.0, 0.0),
                  med_int=-1):
    """A sphere of the given BSDF over the ground, under the 1x1 light (config-0 stage)."""
    shapes, bsdfs, emitters = [], [bsdf], []
    sv, sf = scenes.icosphere(subdiv, radius, center)
    vel = _translate(sv.shape[0], nder, slot_translate) if slot_translate is not None else None
    shapes.append(ShapeSpec(sv, sf, bsdf_id=0, velocities=vel, med_int_id=med_int))
    scenes._stage(shapes, bsdfs, emitters)
    return SceneSpec(nder, scenes._camera(w, h, nder=nder), shapes, bsdfs, emitters, [], [], name="feature")


def _live_slots(g):
    return np.abs(g[:, 1:]).sum(axis=(0, 2, 3, 4))


def test_phong_parity(native, oracle):
    nder = 4
    d_kd = np.zeros((nder, 3), np.float32)
    d_ks = np.zeros((nder, 3), np.float32)
    d_e = np.zeros(nder, np.float32)
    d_kd[0], d_ks[1], d_e[2] = 1.0, 1.0, 1.0
    b = BsdfSpec(_abi.BSDF_PHONG, diffuse=(0.4, 0.3, 0.2), specular=(0.3, 0.3, 0.3), exponent=20.0,
                 d_diffuse=d_kd, d_specular=d_ks, d_exponent=d_e)
    spec = _sphere_scene(b, nder, slot_translate=3)
    g, c = _pair(native, oracle, spec, dict(spp=16, max_bounces=3, sppe=64, sppse=4))
    print(statcheck.assert_parity(g, c, label="phong"))
    assert (_live_slots(g) > 0).all()


def test_rough_dielectric_parity(native, oracle):
    nder = 3
    d_a = np.zeros(nder, np.float32)
    d_eta = np.zeros(nder, np.float32)
    d_a[0], d_eta[1] = 1.0, 1.0
    b = BsdfSpec(_abi.BSDF_ROUGHDIELECTRIC, alpha=0.2, int_ior=1.5, ext_ior=1.0, d_alpha=d_a, d_eta=d_eta)
    spec = _sphere_scene(b, nder, slot_translate=2)
    g, c = _pair(native, oracle, spec, dict(spp=16, max_bounces=4, sppe=64, sppse=4))
    print(statcheck.assert_parity(g, c, label="rough dielectric alpha 0.2"))
    assert (_live_slots(g) > 0).all()


def test_area_light_ex_parity(native, oracle):
    nder = 3
    spec = _sphere_scene(BsdfSpec(_abi.BSDF_DIFFUSE, diffuse=(0.6, 0.6, 0.6)), nder, slot_translate=2)
    d_i = np.zeros((nder, 3), np.float32)
    d_k = np.zeros(nder, np.float32)
    d_i[0], d_k[1] = 1.0, 1.0
    e = spec.emitters[0]
    spec.emitters[0] = EmitterSpec(shape_id=e.shape_id, intensity=(10.0, 10.0, 10.0), type=_abi.EMITTER_AREA_EX,
                                   kappa=3.0, d_intensity=d_i, d_kappa=d_k)
    g, c = _pair(native, oracle, spec, dict(spp=16, max_bounces=3, sppe=64, sppse=4))
    print(statcheck.assert_parity(g, c, label="AreaLightEx"))
    assert (_live_slots(g) > 0).all()


def _two_sided_scene(two_sided):
    """A 0.6x0.6 light at y=-0.4 facing down: the camera (at eye height 0) sees its back
    side, the ground its front side; a diffuse sphere above it is lit by the back side."""
    nder = 1
    shapes, bsdfs, emitters = [], [], []
    gv, gf = scenes.quad((0.0, -1.0, 0.0), 2.0, 2.0, +1.0)
    bsdfs.append(BsdfSpec(_abi.BSDF_DIFFUSE, diffuse=(0.5, 0.5, 0.5)))
    shapes.append(ShapeSpec(gv, gf, bsdf_id=0))
    lv, lf = scenes.quad((0.0, -0.4, 0.0), 0.3, 0.3, -1.0)
    bsdfs.append(BsdfSpec(_abi.BSDF_DIFFUSE, diffuse=(0.0, 0.0, 0.0)))
    shapes.append(ShapeSpec(lv, lf, bsdf_id=1, light_id=0))
    emitters.append(EmitterSpec(shape_id=1, intensity=(5.0, 5.0, 5.0), two_sided=two_sided))
    sv, sf = scenes.icosphere(2, 0.35, (0.0, 0.3, 0.0))
    bsdfs.append(BsdfSpec(_abi.BSDF_DIFFUSE, diffuse=(0.7, 0.7, 0.7)))
    shapes.append(ShapeSpec(sv, sf, bsdf_id=2, velocities=_translate(sv.shape[0], nder, 0)))
    cam = scenes._camera(32, 32, nder=nder)
    return SceneSpec(nder, cam, shapes, bsdfs, emitters, [], [], name="two-sided light")


def test_two_sided_light_parity(native, oracle):
    kw = dict(spp=16, max_bounces=3, sppe=64, sppse=4)
    g, c = _pair(native, oracle, _two_sided_scene(True), kw)
    print(statcheck.assert_parity(g, c, label="two-sided light"))
    with native.NativeScene(_two_sided_scene(False)) as s:
        one = np.stack([s.render(seed=100 + k, **kw) for k in range(4)])
    # the back side's emission and the light it throws on the sphere are there only when two-sided
    assert g[:, 0].mean() > 1.2 * one[:, 0].mean()


def test_camera_velocity_parity(native, oracle):
    """Static geometry, moving camera: slot 0 translates along x, slot 1 along y, slot 2
    rotates about the y axis (interior, secondary-edge and primary-edge terms)."""
    nder = 3
    spec = scenes.config2(32, 32, subdiv=3, nder=nder)
    spec.shapes[0].velocities = None
    vel = np.zeros((2 * nder, 3), np.float32)
    vel[0] = (1.0, 0.0, 0.0)
    vel[1] = (0.0, 1.0, 0.0)
    vel[nder + 2] = (0.0, 1.0, 0.0)
    spec.camera.velocities = vel
    g, c = _pair(native, oracle, spec, dict(spp=16, max_bounces=3, sppe=64, sppse=4))
    print(statcheck.assert_parity(g, c, label="camera velocities"))
    assert (_live_slots(g) > 0).all()


def test_crop_window_parity(native, oracle):
    """An off-centre, non-square window across the silhouette of a translating diffuse
    sphere, with the primary edges clipped to the window."""
    spec = scenes.config2(64, 64, subdiv=3, nder=1)
    spec.shapes[0].velocities = _translate(spec.shapes[0].vertices.shape[0], 1, 0)
    spec = scenes.with_crop(spec, 24, 16, x=30, y=12)
    kw = dict(spp=16, max_bounces=3, sppe=64, sppse=4)
    g, c = _pair(native, oracle, spec, kw)
    assert g.shape == (GPU_RUNS, 2, 16, 24, 3)
    print(statcheck.assert_parity(g, c, label="crop window"))
    with native.NativeScene(spec) as s:
        s.render(seed=1, **kw)
        ns = s.last_stats()["primary_edge_samples"]
    assert ns > 0


def test_albedo_grid_parity(native, oracle):
    """A heterogeneous medium with a 3-channel albedo grid (and the reference's sigma_s,
    which uses the constant albedo, heterogeneous.h:88-90)."""
    spec = scenes.config1(32, 32, res=16)
    rng = np.random.default_rng(5)
    alb = rng.uniform(0.5, 0.95, size=(8, 8, 8, 3)).astype(np.float32)
    m = spec.media[0]
    m.albedo_grid = alb
    m.albedo_min, m.albedo_max = (-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)
    g, c = _pair(native, oracle, spec, dict(spp=16, max_bounces=6, sppe=0, sppse=4))
    print(statcheck.assert_parity(g, c, label="albedo grid"))
    with native.NativeScene(scenes.config1(32, 32, res=16)) as s:
        plain = np.stack([s.render(seed=100 + k, spp=16, max_bounces=6, sppe=0, sppse=4) for k in range(4)])
    assert abs(g[:, 0].mean() - plain[:, 0].mean()) > 1e-3  # the grid does change the image


def _fog_scene(nder=1):
    """A translating diffuse sphere inside a null-bounded homogeneous fog box: volume
    vertices see its silhouette edges, so the volume edge term is non-zero."""
    shapes, bsdfs, emitters = [], [], []
    scenes._stage(shapes, bsdfs, emitters)
    bv, bf = scenes.box((-1.0, -0.95, -1.0), (1.0, 1.0, 1.0))
    bsdfs.append(BsdfSpec(_abi.BSDF_NULL))
    shapes.append(ShapeSpec(bv, bf, bsdf_id=len(bsdfs) - 1, med_int_id=0))
    sv, sf = scenes.icosphere(2, 0.4)
    bsdfs.append(BsdfSpec(_abi.BSDF_DIFFUSE, diffuse=(0.7, 0.7, 0.7)))
    shapes.append(ShapeSpec(sv, sf, bsdf_id=len(bsdfs) - 1, velocities=_translate(sv.shape[0], nder, 0)))
    media = [MediumSpec(_abi.MEDIUM_HOMOGENEOUS, phase_id=0, sigma_t=0.8, albedo=(0.9, 0.9, 0.9))]
    return SceneSpec(nder, scenes._camera(32, 32, nder=nder), shapes, bsdfs, emitters,
                     [PhaseSpec(_abi.PHASE_ISOTROPIC)], media, name="fog")


@pytest.mark.parametrize("mode", [0x20, -1])
def test_volume_edge_term_parity(native, oracle, mode):
    spec = _fog_scene()
    kw = dict(spp=16, max_bounces=4, sppe=0, sppse=4, mode=mode)
    with native.NativeScene(spec) as s:
        g = np.stack([s.render(seed=100 + k, **kw) for k in range(GPU_RUNS)])
        st = s.last_stats()
    c = np.stack([oracle.render(spec, seed=900 + k, **kw) for k in range(CPU_RUNS)])
    print(statcheck.assert_parity(g, c, label=f"volume edge term mode={mode:#x}"))
    assert st["edge_records"] > 0
    if mode == 0x20:
        assert np.abs(g[:, 0]).max() == 0.0  # only the boundary term is on
        # the term is non-zero: the block means of the derivative image are far from zero
        # (sum of squared block z against zero well above its null expectation, the count)
        z, _, _, _, _ = statcheck.zscores(g[:, 1:], np.zeros_like(g[:, 1:]))
        z = z[np.isfinite(z)]
        assert (z ** 2).sum() > z.size + 10 * np.sqrt(2 * z.size), ((z ** 2).sum(), z.size)


def test_device_pcg32_bit_exact(native):
    data = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "pcg32.json")))
    for case in data["cases"]:
        n = len(case["u32"])
        u, f, d = native.rng_sequence(case["seed"], case["idx"], n)
        want = np.array(case["u32"], np.uint64)
        assert [int(x) for x in u] == case["u32"]
        assert np.array_equal(f, ((want >> 8).astype(np.float64) / 2.0 ** 24).astype(np.float32))
        assert np.array_equal(d, want.astype(np.float64) / 2.0 ** 32)


def test_reference_example_glass_1(native, oracle):
    """The reference's example scene examples/glass_1 (committed as its flat argument
    list, tests/golden/make_examples.py) rendered through the reference-facing API
    (`import dtrt, pydtrt` names, pydtrt.render_scene with dtrt.VolPathTracerAD) against
    the oracle: Phong, rough dielectric alpha 0.3 around a homogeneous medium, four
    derivative slots (apple translation x/y/z, tank roughness)."""
    import dtrt_gb300
    import test_examples
    from dtrt_gb300.pydtrt import scene_renderer
    fx = test_examples.load_fixture()
    dtrt, pydtrt = dtrt_gb300.install_reference_names()
    dtrt.set_nder(fx["nder"])
    integ = dtrt.VolPathTracerAD()
    kw = dict(spp=2, max_bounces=4, sppe=16, sppse=2)
    g = np.stack([pydtrt.render_scene(integ, dtrt.RenderOptions(100 + k, kw["spp"], kw["max_bounces"], kw["sppe"],
                                                                 kw["sppse"], True), *fx["args"]).numpy()
                  for k in range(RUNS)])
    spec = scene_renderer.scene_spec(*fx["args"])
    c = np.stack([oracle.render(spec, seed=900 + k, **kw) for k in range(RUNS)])
    assert g.shape == c.shape == (RUNS, 5, 256, 256, 3)
    print(statcheck.assert_parity(g, c, block=8, label="glass_1"))
    assert (_live_slots(g) > 0).all()
