"""Reverse-mode density adjoint (dtrt_render_adjoint) and per-voxel density directions.

* forward-mode per-voxel directions on the GPU against the FP64 oracle (statistical);
* the adjoint against the forward-mode directional derivatives of the same paths: for
  the same seed, <dL/drho, D_k> must equal sum(dL/dI * dI/dtheta_k) up to rounding;
* the adjoint against central finite differences on 16 voxels (common random numbers,
  statistical), with the estimator variant that integrates the travelled segment;
* argument checks, parameter updates in place, and device-pointer mode.
"""
import numpy as np
import pytest

import statcheck
from dtrt_gb300 import _abi, scenes

pytestmark = pytest.mark.gpu

FLAG = _abi.EST_SCATTER_SEGMENT_FROM_ORIGIN


def small_c3(nder, res, size, seed=3, nblobs=8):
    return scenes.config3(width=size, height=size, res=res, nder=nder, seed=seed, param_slots=False, nblobs=nblobs)


def rand_dirs(nder, res, seed):
    return np.random.default_rng(seed).normal(size=(nder, res, res, res)).astype(np.float32)


def smooth_dirs(grid, nder, seed):
    """Low-variance directions: the grid itself, then smooth random blob fields, then
    white noise (nder >= 3)."""
    res = grid.shape[0]
    out = [grid.astype(np.float32)]
    for k in range(1, nder - 1):
        g, _ = scenes.blob_grid(res, 6, seed + k, amp_range=(-1.0, 1.0))
        out.append(g)
    out.append(rand_dirs(1, res, seed)[0])
    return np.stack(out[:nder]).astype(np.float32)


@pytest.mark.parametrize("flags", [0, FLAG])
def test_density_directions_match_oracle(native, oracle, flags):
    spec = small_c3(nder=3, res=16, size=32)
    dirs = smooth_dirs(spec.media[0].density, 3, 11)
    kw = dict(spp=32, max_bounces=6, sppe=0, sppse=10)
    ns = native.NativeScene(spec)
    ns.set_estimator_flags(flags)
    ns.set_density_derivatives(0, dirs)
    gpu = np.stack([ns.render(seed=100 + k, **kw) for k in range(64)])
    ns.close()
    orc = np.stack([oracle.render_ext(spec, seed=500 + k, est_flags=flags, density_dirs={0: dirs}, **kw)
                    for k in range(48)])
    msg = statcheck.assert_parity(gpu, orc, block=4, label=f"flags={flags}")
    print(msg)
    assert np.abs(gpu[:, 1:]).sum() > 0  # the directions do reach the derivative images


@pytest.mark.parametrize("flags", [0, FLAG])
def test_adjoint_is_transpose_of_forward(native, flags):
    res, size, nd = 24, 48, 4
    spec = small_c3(nder=nd, res=res, size=size)
    dirs = rand_dirs(nd, res, 21)
    dimg = np.random.default_rng(5).normal(size=(size, size, 3)).astype(np.float32)
    kw = dict(seed=7, spp=16, max_bounces=8, sppe=0, sppse=10)
    ns = native.NativeScene(spec)
    ns.set_estimator_flags(flags)
    ns.set_density_derivatives(0, dirs)
    fwd = ns.render(**kw)
    img, grad = ns.render_adjoint(dimg, **kw)
    nvox, _ = ns.gradient_sizes()
    ns.close()
    assert nvox == res ** 3 and grad.shape == (nvox,)
    # the replayed paths are the forward paths: same image
    assert np.abs(img - fwd[0]).max() <= 1e-4 * max(1e-3, np.abs(fwd[0]).max())
    for k in range(nd):
        pf = float((dimg.astype(np.float64) * fwd[k + 1]).sum())
        pa = float(grad.astype(np.float64) @ dirs[k].reshape(-1).astype(np.float64))
        scale = float(np.abs(dimg.astype(np.float64) * fwd[k + 1]).sum())
        assert scale > 0
        assert abs(pa - pf) <= 2e-3 * scale, (k, pa, pf, scale)


def test_adjoint_matches_finite_differences(native):
    """Central differences with common random numbers on 16 voxels inside the blobs,
    for the estimator that integrates the travelled free-flight segment (the reference's
    aliased segment is a biased derivative, so finite differences do not apply to it)."""
    res, size = 10, 32
    spec = small_c3(nder=1, res=res, size=size, nblobs=4)
    grid = spec.media[0].density.copy()
    rng = np.random.default_rng(9)
    dimg = rng.uniform(0.5, 1.5, size=(size, size, 3)).astype(np.float32)
    inner = np.zeros_like(grid, bool)
    inner[1:-1, 1:-1, 1:-1] = True
    h = 0.2 * float(grid.max())
    # voxels inside the blobs whose +-h step leaves the majorant (the grid maximum) unchanged,
    # so that common random numbers keep every free-flight distance of the two renders equal
    cand = np.flatnonzero((grid > 0.3 * grid.max()) & (grid + h < grid.max()) & inner)
    vox = rng.choice(cand, size=16, replace=False)
    seeds = [1000 + i for i in range(24)]
    kw = dict(spp=1024, max_bounces=6, sppe=0, sppse=10)
    ns = native.NativeScene(spec)
    ns.set_estimator_flags(FLAG)
    adj = np.stack([ns.render_adjoint(dimg, image=False, seed=s, **kw)[1] for s in seeds])[:, vox]
    fd = np.zeros((len(seeds), len(vox)))
    for i, v in enumerate(vox):
        loss = {}
        for sgn in (+1, -1):
            g = grid.copy().reshape(-1)
            g[v] += sgn * h
            ns.set_density(0, g.reshape(grid.shape))
            loss[sgn] = [float((dimg * ns.render(seed=s, **kw)[0]).sum()) for s in seeds]
        fd[:, i] = (np.array(loss[+1]) - np.array(loss[-1])) / (2 * h)
    ns.set_density(0, grid)
    ns.close()
    ma, mf = adj.mean(0), fd.mean(0)
    se = np.sqrt(adj.var(0, ddof=1) / len(seeds) + fd.var(0, ddof=1) / len(seeds))
    z = (ma - mf) / np.maximum(se, 1e-12)
    print("adjoint", np.round(ma, 5), "\nfd     ", np.round(mf, 5), "\nz", np.round(z, 2))
    print("snr adjoint", np.round(np.abs(ma) / (adj.std(0, ddof=1) / np.sqrt(len(seeds))), 1),
          "\nsnr fd     ", np.round(np.abs(mf) / (fd.std(0, ddof=1) / np.sqrt(len(seeds))), 1))
    assert np.sum(np.abs(z) > 3.0) <= 1, z
    assert np.abs(z).max() < 5.0, z
    # the comparison is not vacuous: the gradient is resolved above its noise
    assert np.median(np.abs(ma) / np.maximum(se, 1e-12)) > 2.0


def test_adjoint_arguments_and_updates(native):
    res, size = 16, 24
    spec = small_c3(nder=1, res=res, size=size)
    grid = spec.media[0].density
    kw = dict(seed=3, spp=8, max_bounces=4, sppe=0, sppse=0)
    ns = native.NativeScene(spec)
    zero = np.zeros((size, size, 3), np.float32)
    img, grad = ns.render_adjoint(zero, **kw)
    assert np.all(grad == 0) and img.sum() > 0
    lib, h = ns.lib, ns.handle
    o = ns.options(**kw)
    g = np.zeros(res ** 3, np.float32)
    vp = _abi.ctypes.c_void_p
    # a grid-medium scene has no vertex adjoint; d_density needs d_image; homogeneous medium ids are rejected
    assert lib.dtrt_render_adjoint(h, _abi.ctypes.byref(o), zero.ctypes.data_as(vp), None, g.ctypes.data_as(vp),
                                   g.ctypes.data_as(vp), 0, None) == _abi.DTRT_ERR_UNSUPPORTED
    assert lib.dtrt_render_adjoint(h, _abi.ctypes.byref(o), None, None, g.ctypes.data_as(vp), None, 0,
                                   None) == _abi.DTRT_ERR_INVALID
    assert lib.dtrt_scene_set_density(h, 5, g.ctypes.data_as(_abi.c_float_p)) == _abi.DTRT_ERR_INVALID
    assert lib.dtrt_scene_set_estimator_flags(h, 0x80) == _abi.DTRT_ERR_INVALID
    # an all-zero density is rejected (zero majorant) and leaves the scene unchanged
    assert lib.dtrt_scene_set_density(h, 0, g.ctypes.data_as(_abi.c_float_p)) == _abi.DTRT_ERR_INVALID
    a = ns.render(**kw)
    ns.set_density(0, grid)  # same values: same render
    b = ns.render(**kw)
    assert np.array_equal(a, b)
    ns.set_density(0, grid * 2.0)
    c = ns.render(**kw)
    assert not np.array_equal(a[0], c[0])
    ns.close()
    # a scene without a grid medium: empty gradient, image still rendered
    c0 = scenes.config0(width=16, height=16)
    with native.NativeScene(c0) as n0:
        assert n0.gradient_sizes()[0] == 0
        img0, g0 = n0.render_adjoint(np.ones((16, 16, 3), np.float32), seed=1, spp=4, max_bounces=3, sppe=0)
        f0 = n0.render(seed=1, spp=4, max_bounces=3, sppe=0, sppse=0)
        assert g0.size == 0
        assert np.abs(img0 - f0[0]).max() <= 1e-4 * max(1e-3, np.abs(f0[0]).max())


def test_adjoint_device_pointers(native):
    torch = pytest.importorskip("torch")
    res, size = 16, 32
    spec = small_c3(nder=1, res=res, size=size)
    kw = dict(seed=4, spp=8, max_bounces=5, sppe=0, sppse=0)
    dimg = np.random.default_rng(2).normal(size=(size, size, 3)).astype(np.float32)
    with native.NativeScene(spec) as ns:
        img_h, grad_h = ns.render_adjoint(dimg, **kw)
        d = torch.from_numpy(dimg).cuda()
        img_d = torch.zeros((size, size, 3), device="cuda")
        grad_d = torch.zeros(res ** 3, device="cuda")
        s = torch.cuda.current_stream().cuda_stream
        ns.render_adjoint(d.data_ptr(), image=img_d.data_ptr(), density_grad=grad_d.data_ptr(), stream=s, device=True,
                          **kw)
        torch.cuda.synchronize()
        assert np.allclose(img_d.cpu().numpy(), img_h, rtol=1e-5, atol=1e-7)
        gd = grad_d.cpu().numpy()
        assert np.abs(gd - grad_h).max() <= 1e-4 * np.abs(grad_h).max()


def test_density_render_func_autograd(native):
    torch = pytest.importorskip("torch")
    from dtrt_gb300.pydtrt import DensityRenderFunc
    res, size = 16, 24
    spec = small_c3(nder=1, res=res, size=size)
    with native.NativeScene(spec) as ns:
        o = ns.options(seed=5, spp=16, max_bounces=5, sppe=0)
        dens = torch.tensor(spec.media[0].density, requires_grad=True)
        target = torch.zeros((size, size, 3))
        img = DensityRenderFunc.apply(dens, ns, 0, o, 5)  # backward replays the forward seed
        loss = ((img - target) ** 2).sum()
        loss.backward()
        _, g = ns.render_adjoint(2.0 * (img.detach().numpy() - target.numpy()), image=False, options=o)
        gt = dens.grad.numpy().reshape(-1)
        assert dens.grad.shape == dens.shape
        assert np.abs(gt - g).max() <= 1e-4 * np.abs(g).max()
        assert np.abs(g).max() > 0
