"""Reverse-mode vertex-position adjoint (dtrt_render_adjoint with d_vertices) on the
mesh configuration (diffuse icosphere over the ground quad under the area light):

* for the same seed, <grad, V_k> equals sum(dL/dI * forward derivative image) along the
  shape velocities V_k, for each term alone (interior BSDF frames, secondary edges, primary
  edges) and for all together;
* central finite differences of the loss along random vertex displacements agree with the
  adjoint (common random numbers, statistical);
* scenes outside the covered class are rejected.
"""
import numpy as np
import pytest

from dtrt_gb300 import _abi, scenes

pytestmark = pytest.mark.gpu


def c2_small(nder=4, size=48, subdiv=2, seed=2):
    return scenes.config2(width=size, height=size, subdiv=subdiv, nder=nder, seed=seed)


def directions(spec):
    """[nder, total vertices, 3] velocity fields of the spec's shapes (global vertex order)."""
    tot = sum(s.vertices.shape[0] for s in spec.shapes)
    V = np.zeros((spec.nder, tot, 3))
    off = 0
    for s in spec.shapes:
        nv = s.vertices.shape[0]
        if s.velocities is not None:
            V[:, off:off + nv] = np.asarray(s.velocities, np.float64)[:spec.nder * nv].reshape(spec.nder, nv, 3)
        off += nv
    return V


TERMS = {
    "interior": dict(mode=_abi.MODE_EMISSION | _abi.MODE_SURFACE_MAIN, sppse=0, sppe=0),
    "secondary": dict(mode=_abi.MODE_SURFACE_BOUNDARY, sppse=10, sppe=0),
    "primary": dict(mode=0, sppse=0, sppe=256),
    "all": dict(mode=-1, sppse=10, sppe=64),
}


@pytest.mark.parametrize("term", list(TERMS))
def test_vertex_adjoint_is_transpose_of_forward(native, term):
    spec = c2_small()
    V = directions(spec)
    size = spec.width
    dimg = np.random.default_rng(5).normal(size=(size, size, 3)).astype(np.float32)
    kw = dict(seed=7, spp=16, max_bounces=4, **TERMS[term])
    with native.NativeScene(spec) as ns:
        fwd = ns.render(**kw)
        img, grad = ns.render_vertex_adjoint(dimg, **kw)
        nv = ns.gradient_sizes()[1]
    assert grad.shape == (nv, 3) == V.shape[1:]
    if term != "primary":
        assert np.abs(img - fwd[0]).max() <= 1e-4 * max(1e-3, np.abs(fwd[0]).max())
    worst = 0.0
    for k in range(spec.nder):
        pf = float((dimg.astype(np.float64) * fwd[k + 1]).sum())
        pa = float((grad.astype(np.float64) * V[k]).sum())
        scale = float(np.abs(dimg.astype(np.float64) * fwd[k + 1]).sum())
        assert scale > 0, term
        worst = max(worst, abs(pa - pf) / scale)
        print(term, k, pf, pa, scale)
    assert worst <= 5e-3, worst


def test_vertex_adjoint_matches_finite_differences(native):
    """Central differences of L = sum(w * I) along 3 random displacement fields of the sphere
    vertices, common random numbers, 16 seeds; all terms (interior + both edge terms)."""
    size, h = 32, 2e-3
    base = c2_small(nder=1, size=size)
    sv = base.shapes[0].vertices.astype(np.float64)
    rng = np.random.default_rng(11)
    w = rng.uniform(0.5, 1.5, size=(size, size, 3)).astype(np.float32)
    seeds = [2000 + i for i in range(16)]
    kw = dict(spp=64, max_bounces=4, sppse=10, sppe=256)
    with native.NativeScene(base) as ns:
        G = np.stack([ns.render_vertex_adjoint(w, image=False, seed=s, **kw)[1] for s in seeds])[:, :sv.shape[0]]
    resolved = 0
    for trial in range(3):
        D = rng.normal(size=sv.shape)
        D /= np.sqrt((D ** 2).mean())  # rms vertex displacement h
        loss = {}
        for sgn in (+1, -1):
            spec = c2_small(nder=1, size=size)
            spec.shapes[0].vertices = (sv + sgn * h * D).astype(np.float32)
            with native.NativeScene(spec) as ns:
                loss[sgn] = np.array([float((w * ns.render_adjoint(None, image=True, density_grad=False, seed=s,
                                                                     spp=kw["spp"], max_bounces=4)[0]).sum())
                                      for s in seeds])
        fd = (loss[+1] - loss[-1]) / (2 * h)
        adj = (G.astype(np.float64) * D[None]).sum(axis=(1, 2))
        se = np.sqrt(fd.var(ddof=1) / len(seeds) + adj.var(ddof=1) / len(seeds))
        z = (adj.mean() - fd.mean()) / se
        print("trial", trial, "adjoint", adj.mean(), "fd", fd.mean(), "se", se, "z", z)
        assert abs(z) < 4.0, (trial, adj.mean(), fd.mean(), se)
        resolved += abs(adj.mean()) > 3.0 * np.sqrt(adj.var(ddof=1) / len(seeds))
    assert resolved >= 2  # the comparison is not vacuous: most directions have a resolved derivative


def test_vertex_adjoint_rejects_uncovered_scenes(native):
    c0 = scenes.config0(width=16, height=16)  # has a medium
    with native.NativeScene(c0) as ns:
        with pytest.raises(_abi.DtrtError) as ei:
            ns.render_vertex_adjoint(np.ones((16, 16, 3), np.float32), seed=1, spp=1, max_bounces=2)
        assert ei.value.status == _abi.DTRT_ERR_UNSUPPORTED


def test_vertex_render_func_autograd(native):
    torch = pytest.importorskip("torch")
    from dtrt_gb300.pydtrt import VertexRenderFunc
    spec = c2_small(nder=1, size=24)
    verts = torch.tensor(np.concatenate([s.vertices for s in spec.shapes]), requires_grad=True)
    with native.NativeScene(spec) as ns:
        o = ns.options(seed=5, spp=8, max_bounces=3, sppse=4, sppe=32)
        img = VertexRenderFunc.apply(verts, spec, o, 5)  # backward replays the forward seed
        target = torch.zeros_like(img)
        ((img - target) ** 2).sum().backward()
        _, g = ns.render_vertex_adjoint(2.0 * (img.detach().numpy() - target.numpy()), image=False, options=o)
    assert verts.grad.shape == verts.shape
    assert np.abs(verts.grad.numpy() - g).max() <= 1e-4 * np.abs(g).max()
    assert np.abs(g).max() > 0
