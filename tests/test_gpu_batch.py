"""Batches of uneven scenes (dtrt_batch_*): every item's image and density gradient equal the
single-scene adjoint render of the same options (up to the order of floating-point atomic
adds), with and without autotuning and graph capture, under the batch wavefront (one replay
wavefront over the paths of all items), and across repeated launches."""
import numpy as np
import pytest

from dtrt_gb300 import _abi, scenes

pytestmark = pytest.mark.gpu


def _items(native, torch, n=6):
    out = []
    for i in range(n):
        spec, kw = scenes.config4(i, side_scale=0.125, spp_scale=0.125)
        sc = native.NativeScene(spec)
        h, w = spec.height, spec.width
        opts = sc.options(seed=40 + i, spp=kw["spp"], max_bounces=kw["max_bounces"], sppe=0)
        nvox = sc.gradient_sizes()[0]
        dimg = torch.randn((h, w, 3), device="cuda", generator=torch.Generator("cuda").manual_seed(i))
        img = torch.zeros((h, w, 3), device="cuda")
        grad = torch.zeros(max(nvox, 1), device="cuda")
        out.append(dict(scene=sc, opts=opts, dimg=dimg, img=img, grad=grad, nvox=nvox))
    return out


def _single(it, torch):
    img = torch.zeros_like(it["img"])
    grad = torch.zeros_like(it["grad"])
    s = torch.cuda.current_stream().cuda_stream
    it["scene"].render_adjoint(it["dimg"].data_ptr(), image=img.data_ptr(),
                               density_grad=grad.data_ptr() if it["nvox"] else None, stream=s, device=True,
                               options=it["opts"])
    torch.cuda.synchronize()
    return img.cpu().numpy(), grad.cpu().numpy()


@pytest.mark.parametrize("autotune,graph,wavefront", [(True, True, False), (False, False, False),
                                                     (False, True, False), (False, False, True),
                                                     (False, True, True)])
def test_batch_matches_single_renders(native, autotune, graph, wavefront):
    torch = pytest.importorskip("torch")
    items = _items(native, torch)
    assert any(it["nvox"] for it in items) and any(not it["nvox"] for it in items)
    ref = [_single(it, torch) for it in items]
    batch = native.Batch([(it["scene"], it["opts"], it["dimg"].data_ptr(), it["img"].data_ptr(),
                           it["grad"].data_ptr() if it["nvox"] else 0) for it in items], autotune=autotune,
                         graph=graph, stream=torch.cuda.current_stream().cuda_stream, wavefront=wavefront)
    st = batch.stats()
    assert st["num_items"] == len(items) and st["graph"] == graph
    if wavefront:
        assert st["schedule"] == "wavefront" and st["wave_capacity"] > 0
    if autotune:
        assert len(st["trials"]) >= 2
        assert sorted(st["order"]) == list(range(len(items)))
    for rep in range(2):  # a second launch rewrites the same results
        batch.launch(torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        for it, (img_r, grad_r) in zip(items, ref):
            img = it["img"].cpu().numpy()
            assert np.abs(img - img_r).max() <= 1e-5 * max(1e-3, np.abs(img_r).max())
            assert img.sum() > 0
            if it["nvox"]:
                g = it["grad"].cpu().numpy()
                assert np.abs(g - grad_r).max() <= 1e-4 * max(1e-12, np.abs(grad_r).max())
                assert np.abs(g).max() > 0
    batch.close()
    for it in items:
        it["scene"].close()


def test_batch_wavefront_single_item(native):
    """A batch wavefront over one item is that item's replay wavefront."""
    torch = pytest.importorskip("torch")
    items = _items(native, torch)
    it = next(x for x in items if x["nvox"])
    for x in items:
        if x is not it:
            x["scene"].close()
    img_r, grad_r = _single(it, torch)
    batch = native.Batch([(it["scene"], it["opts"], it["dimg"].data_ptr(), it["img"].data_ptr(),
                           it["grad"].data_ptr())], autotune=False, graph=False,
                         stream=torch.cuda.current_stream().cuda_stream, wavefront=True)
    assert batch.stats()["schedule"] == "wavefront"
    batch.launch(stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    img = it["img"].cpu().numpy()
    g = it["grad"].cpu().numpy()
    assert np.abs(img - img_r).max() <= 1e-5 * max(1e-3, np.abs(img_r).max())
    assert np.abs(g - grad_r).max() <= 1e-4 * max(1e-12, np.abs(grad_r).max()) and np.abs(g).max() > 0
    batch.close()
    it["scene"].close()


def test_batch_vertex_items_match_single_renders(native):
    """Items with d_vertices (surface scenes) run the vertex-position replay after the
    batch's launch: their image and vertex gradient equal dtrt_render_adjoint's, next to
    density items in the same batch."""
    torch = pytest.importorskip("torch")
    s = torch.cuda.current_stream().cuda_stream
    dens = _items(native, torch, n=3)
    verts = []
    for i in range(2):
        spec = scenes.config2(32, 32, subdiv=2, nder=1, seed=5 + i)
        sc = native.NativeScene(spec)
        opts = sc.options(seed=70 + i, spp=8, max_bounces=3, sppe=4, sppse=2)
        nv = sc.gradient_sizes()[1]
        dimg = torch.randn((32, 32, 3), device="cuda", generator=torch.Generator("cuda").manual_seed(50 + i))
        verts.append(dict(scene=sc, opts=opts, dimg=dimg, img=torch.zeros((32, 32, 3), device="cuda"),
                          vg=torch.zeros((nv, 3), device="cuda"), nv=nv))
    refs = []
    for it in verts:
        img = torch.zeros_like(it["img"])
        vg = torch.zeros_like(it["vg"])
        it["scene"].render_vertex_adjoint(it["dimg"].data_ptr(), image=img.data_ptr(), vertex_grad=vg.data_ptr(),
                                          stream=s, device=True, options=it["opts"])
        torch.cuda.synchronize()
        refs.append((img.cpu().numpy(), vg.cpu().numpy()))
    lib = _abi.load()
    arr = (_abi.BatchItem * (len(dens) + len(verts)))()
    for k, it in enumerate(dens):
        arr[k].scene = it["scene"].handle.value
        arr[k].opts = it["opts"]
        arr[k].d_image = it["dimg"].data_ptr()
        arr[k].image = it["img"].data_ptr()
        arr[k].d_density = it["grad"].data_ptr() if it["nvox"] else None
    for k, it in enumerate(verts):
        a = arr[len(dens) + k]
        a.scene = it["scene"].handle.value
        a.opts = it["opts"]
        a.d_image = it["dimg"].data_ptr()
        a.image = it["img"].data_ptr()
        a.d_vertices = it["vg"].data_ptr()
    h = _abi.ctypes.c_void_p()
    _abi.check(lib.dtrt_batch_create(arr, len(arr), _abi.BATCH_AUTOTUNE | _abi.BATCH_GRAPH, _abi.ctypes.c_void_p(s),
                                     _abi.ctypes.byref(h)))
    st = _abi.BatchStats()
    _abi.check(lib.dtrt_batch_stats_get(h, _abi.ctypes.byref(st)))
    assert st.as_dict()["vertex_items"] == 2
    _abi.check(lib.dtrt_batch_launch(h, _abi.ctypes.c_void_p(s)))
    torch.cuda.synchronize()
    for it, (img_r, vg_r) in zip(verts, refs):
        img, vg = it["img"].cpu().numpy(), it["vg"].cpu().numpy()
        assert np.abs(img - img_r).max() <= 1e-5 * max(1e-3, np.abs(img_r).max()) and img.sum() > 0
        assert np.abs(vg - vg_r).max() <= 1e-4 * max(1e-12, np.abs(vg_r).max()) and np.abs(vg).max() > 0
    for it in dens:  # the density items still render
        assert it["img"].cpu().numpy().sum() > 0
    lib.dtrt_batch_destroy(h)
    for it in dens + verts:
        it["scene"].close()


def test_batch_rejects_bad_items(native):
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    h = _abi.ctypes.c_void_p()
    arr = (_abi.BatchItem * 1)()
    assert lib.dtrt_batch_create(arr, 0, 0, None, _abi.ctypes.byref(h)) == _abi.DTRT_ERR_INVALID
    spec, kw = scenes.config4(1, side_scale=0.125, spp_scale=0.125)
    with native.NativeScene(spec) as sc:
        arr[0].scene = sc.handle.value
        arr[0].opts = sc.options(spp=1, max_bounces=2)
        # no output buffer
        assert lib.dtrt_batch_create(arr, 1, 0, None, _abi.ctypes.byref(h)) == _abi.DTRT_ERR_INVALID
        g = torch.zeros(16, device="cuda")
        arr[0].d_density = g.data_ptr()  # d_density without d_image
        assert lib.dtrt_batch_create(arr, 1, 0, None, _abi.ctypes.byref(h)) == _abi.DTRT_ERR_INVALID
        arr[0].d_density = None
        arr[0].d_vertices = g.data_ptr()  # d_vertices without d_image
        assert lib.dtrt_batch_create(arr, 1, 0, None, _abi.ctypes.byref(h)) == _abi.DTRT_ERR_INVALID
        arr[0].d_image = g.data_ptr()
        arr[0].d_density = g.data_ptr()  # d_vertices with d_density
        assert lib.dtrt_batch_create(arr, 1, 0, None, _abi.ctypes.byref(h)) == _abi.DTRT_ERR_INVALID
