"""The reference's other forward-mode integrators, PathTracerAD (pathAD.cpp:10-228) and
DirectAD (directAD.cpp:1-163), as rendered here: the volumetric estimator on surface
scenes (all bounces, or one bounce for DirectAD). The oracle restates both reference
integrators with their own random-number order, MIS heuristics (power / balance),
occlusion test and edge parametrisation; the GPU images must agree with them in
expectation (block z-test), which pins the mapping."""
import numpy as np
import pytest

import statcheck
from dtrt_gb300 import _abi, dtrt, scenes
from dtrt_gb300.scenes import BsdfSpec

pytestmark = pytest.mark.gpu

GPU_RUNS, CPU_RUNS = 256, 64


def _moving_sphere(bsdf=None):
    spec = scenes.config2(32, 32, subdiv=3, nder=3)
    nv = spec.shapes[0].vertices.shape[0]
    vel = np.zeros((3 * nv, 3), np.float32)
    vel[2 * nv:, 0] = 1.0  # slot 2: translation along x
    spec.shapes[0].velocities = vel
    if bsdf is not None:
        spec.bsdfs[0] = bsdf
    return spec


def _phong():
    d_kd = np.zeros((3, 3), np.float32)
    d_e = np.zeros(3, np.float32)
    d_kd[0], d_e[1] = 1.0, 1.0
    return BsdfSpec(_abi.BSDF_PHONG, diffuse=(0.5, 0.4, 0.3), specular=(0.3, 0.3, 0.3), exponent=15.0,
                    d_diffuse=d_kd, d_exponent=d_e)


def _gpu(integrator, spec, kw, runs=GPU_RUNS):
    scene = dtrt.Scene.from_spec(spec)
    try:
        out = []
        for k in range(runs):
            img = np.zeros(spec.out_shape(), np.float32)
            o = dtrt.RenderOptions(100 + k, kw["spp"], kw["max_bounces"], kw["sppe"], kw["sppse"], True)
            integrator.render(scene, o, dtrt.float_ptr(img.ctypes.data))
            out.append(img)
        return np.stack(out)
    finally:
        scene.close()


@pytest.mark.parametrize("bsdf", ["diffuse", "phong"])
def test_path_tracer_ad_matches_reference_estimator(native, oracle, bsdf):
    spec = _moving_sphere(_phong() if bsdf == "phong" else None)
    kw = dict(spp=16, max_bounces=3, sppe=64, sppse=4)
    g = _gpu(dtrt.PathTracerAD(), spec, kw)
    c = np.stack([oracle.render_integrator(spec, "path", seed=900 + k, **kw) for k in range(CPU_RUNS)])
    print(statcheck.assert_parity(g, c, label=f"PathTracerAD {bsdf}"))
    live = np.abs(g[:, 1:]).sum(axis=(0, 2, 3, 4))
    assert (live > 0).all() if bsdf == "phong" else live[2] > 0  # the diffuse BSDF has no parameter slots


@pytest.mark.parametrize("bsdf", ["diffuse", "phong"])
def test_direct_ad_matches_reference_estimator(native, oracle, bsdf):
    spec = _moving_sphere(_phong() if bsdf == "phong" else None)
    kw = dict(spp=16, max_bounces=3, sppe=64, sppse=4)  # DirectAD renders one bounce whatever max_bounces
    g = _gpu(dtrt.DirectAD(), spec, kw)
    c = np.stack([oracle.render_integrator(spec, "direct", seed=900 + k, **kw) for k in range(CPU_RUNS)])
    print(statcheck.assert_parity(g, c, label=f"DirectAD {bsdf}"))
    live = np.abs(g[:, 1:]).sum(axis=(0, 2, 3, 4))
    assert (live > 0).all() if bsdf == "phong" else live[2] > 0


def test_surface_integrators_refuse_scenes_outside_the_mapping(native):
    img = np.zeros((2, 16, 16, 3), np.float32)
    o = dtrt.RenderOptions(1, 1, 2, 0, 0, True)
    for spec in (scenes.config0(16, 16), scenes.config1(16, 16, res=8, nder=1)):  # media, null / dielectric BSDFs
        scene = dtrt.Scene.from_spec(spec)
        try:
            for integ in (dtrt.PathTracerAD(), dtrt.DirectAD()):
                with pytest.raises(NotImplementedError):
                    integ.render(scene, o, dtrt.float_ptr(img.ctypes.data))
        finally:
            scene.close()
