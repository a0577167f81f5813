"""GPU parity: the CUDA renderer against the FP64 CPU oracle on identical seeded
scenes. Image and derivative images must agree per 4x4 pixel block within 3 sigma
of the combined Monte Carlo standard error (see statcheck.py), and the BVH must
return the same closest hits."""
import numpy as np
import pytest

from dtrt_gb300 import scenes
from statcheck import assert_parity

pytestmark = pytest.mark.gpu


# 256 GPU and 64 oracle renders per comparison, reduced to 16 batch means per side by
# statcheck.assert_parity (edge-term estimates are heavy-tailed)
def gpu_runs(native, spec, seeds, **kw):
    with native.NativeScene(spec) as s:
        return np.stack([s.render(seed=sd, **kw).copy() for sd in seeds])


def cpu_runs(oracle, spec, seeds, **kw):
    return np.stack([oracle.render(spec, seed=sd, **kw) for sd in seeds])


def _random_rays(rng, n, spec):
    org = rng.uniform(-2.5, 2.5, size=(n, 3))
    org[: n // 2] = np.array([0.0, 0.0, 4.0]) + rng.normal(scale=0.1, size=(n // 2, 3))
    tgt = rng.uniform(-1.0, 1.0, size=(n, 3))
    d = tgt - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8))
    rays[:, :3], rays[:, 3], rays[:, 4:7], rays[:, 7] = org, 0.0, d, np.inf
    return rays


@pytest.mark.parametrize("cfg", ["c0", "c2"])
def test_bvh_closest_hit_matches_oracle(native, oracle, cfg):
    spec = scenes.config0(16, 16) if cfg == "c0" else scenes.config2(16, 16, subdiv=4, nder=1)
    rays = _random_rays(np.random.default_rng(0), 20000, spec)
    with native.NativeScene(spec) as s:
        hg, tg = s.trace_closest(rays.astype(np.float32))
    ho, to = oracle.trace_closest(spec, rays)
    same = hg[:, 0] == ho[:, 0]
    # disagreements are allowed only at near-ties (shared edges / grazing)
    both = (hg[:, 0] >= 0) & (ho[:, 0] >= 0)
    assert (hg[:, 0] >= 0).sum() > 5000
    close_t = np.abs(tg - to) <= 1e-4 * np.maximum(1.0, np.abs(to))
    bad = ~same & ~(both & close_t)
    assert bad.mean() < 1e-3, f"{bad.sum()} mismatching hits"
    assert np.all(close_t[same & both])


def test_c0_homogeneous_sphere_parity(native, oracle):
    spec = scenes.config0(32, 32)
    kw = dict(spp=16, max_bounces=5, sppe=0, sppse=10)
    g = gpu_runs(native, spec, range(1000, 1256), **kw)
    c = cpu_runs(oracle, spec, range(2000, 2064), **kw)
    print(assert_parity(g, c, label="C0"))


def test_c0_primary_edge_parity(native, oracle):
    spec = scenes.config0(32, 32)
    with native.NativeScene(spec) as s:
        g = np.stack([s.render(seed=sd, spp=0, max_bounces=5, sppe=64, sppse=0)[1:].copy() for sd in range(256)])
    c = np.stack([oracle.render_primary_edges(spec, seed=sd, sppe=64, max_bounces=5) for sd in range(1000, 1064)])
    print(assert_parity(g, c, label="C0 primary"))


def test_c1_heterogeneous_parity(native, oracle):
    spec = scenes.config1(32, 32, res=32)
    kw = dict(spp=16, max_bounces=6, sppe=0, sppse=10)
    g = gpu_runs(native, spec, range(3000, 3256), **kw)
    c = cpu_runs(oracle, spec, range(4000, 4064), **kw)
    print(assert_parity(g, c, label="C1"))


def test_c2_mesh_derivative_parity(native, oracle):
    spec = scenes.config2(32, 32, subdiv=3, nder=4)
    kw = dict(spp=8, max_bounces=3, sppe=0, sppse=4)
    g = gpu_runs(native, spec, range(5000, 5256), **kw)
    c = cpu_runs(oracle, spec, range(6000, 6064), **kw)
    print(assert_parity(g, c, label="C2"))


def _translating_diffuse_sphere(w, h, subdiv=3):
    spec = scenes.config2(w, h, subdiv=subdiv, nder=1)
    nv = spec.shapes[0].vertices.shape[0]
    spec.shapes[0].velocities = np.tile(np.array([[1.0, 0.0, 0.0]], np.float32), (nv, 1))
    return spec


def test_primary_edge_parity_moving_diffuse_sphere(native, oracle):
    spec = _translating_diffuse_sphere(32, 32)
    sppe = 256
    ne, tl, npe, psum = oracle.edge_summary(spec)
    with native.NativeScene(spec) as s:
        g = []
        for sd in range(48):
            g.append(s.render(seed=sd, spp=0, max_bounces=3, sppe=sppe, sppse=0)[1:].copy())
            if sd == 0:  # same projected-edge table: same sample count ceil(PDFsum*sppe/128)*128
                assert s.last_stats()["primary_edge_samples"] == int(np.ceil(psum * sppe / 128.0)) * 128
        g = np.stack(g)
    c = np.stack([oracle.render_primary_edges(spec, seed=sd, sppe=sppe, max_bounces=3) for sd in range(100, 148)])
    assert np.abs(c).sum() > 0 and np.abs(g).sum() > 0
    print(assert_parity(g, c, label="primary edges (moving sphere)"))


def test_full_forward_render_moving_diffuse_sphere(native, oracle):
    spec = _translating_diffuse_sphere(32, 32)
    kw = dict(spp=16, max_bounces=3, sppe=64, sppse=4)
    g = gpu_runs(native, spec, range(7000, 7256), **kw)
    c = cpu_runs(oracle, spec, range(8000, 8064), **kw)
    print(assert_parity(g, c, label="moving sphere all terms"))
