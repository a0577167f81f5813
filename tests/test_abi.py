"""C-ABI checks that need no GPU: the library builds and loads, exports every symbol
include/dtrt_gb300.h declares, the ctypes structs match the C layout, and calls
that need a device fail with a status instead of crashing."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

from dtrt_gb300 import _abi, build_ext, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build_ext.build()
    return _abi.load()


def test_exports_every_declared_symbol(lib):
    names = _abi.declared_symbols()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(_abi._SIGNATURES), "ctypes signatures out of sync with the header"


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "dtrt_gb300.h"\nint main(void){'
                   'printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(dtrt_camera_desc), '
                   'sizeof(dtrt_shape_desc), sizeof(dtrt_bsdf_desc), sizeof(dtrt_emitter_desc), '
                   'sizeof(dtrt_phase_desc), sizeof(dtrt_medium_desc), sizeof(dtrt_scene_desc), '
                   'sizeof(dtrt_render_options), sizeof(dtrt_render_stats), sizeof(dtrt_batch_item), '
                   'sizeof(dtrt_batch_stats), offsetof(dtrt_medium_desc, to_world), '
                   'offsetof(dtrt_scene_desc, edge_weights), offsetof(dtrt_batch_item, d_image), '
                   'offsetof(dtrt_batch_stats, item_ms_estimate), sizeof(dtrt_update_stats), '
                   'offsetof(dtrt_update_stats, ms_device)); return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [ctypes.sizeof(t) for t in (_abi.CameraDesc, _abi.ShapeDesc, _abi.BsdfDesc, _abi.EmitterDesc,
                                       _abi.PhaseDesc, _abi.MediumDesc, _abi.SceneDesc, _abi.RenderOptions,
                                       _abi.RenderStats, _abi.BatchItem, _abi.BatchStats)]
    want += [_abi.MediumDesc.to_world.offset, _abi.SceneDesc.edge_weights.offset, _abi.BatchItem.d_image.offset,
             _abi.BatchStats.item_ms_estimate.offset, ctypes.sizeof(_abi.UpdateStats), _abi.UpdateStats.ms_device.offset]
    assert got == want


def test_abi_version_and_nder(lib):
    assert lib.dtrt_abi_version() == 1
    assert [lib.dtrt_nder_supported(n) for n in (0, 1, 2, 3, 4, 5, 8, 9)] == [0, 1, 0, 1, 1, 0, 1, 0]


def test_scene_create_reports_status_without_gpu(lib):
    if lib.dtrt_device_count() > 0:
        pytest.skip("a GPU is visible")
    spec = scenes.config0(8, 8)
    desc, keep = spec.to_desc()
    h = ctypes.c_void_p()
    st = lib.dtrt_scene_create(ctypes.byref(desc), ctypes.byref(h))
    assert st == 7 and not h.value
    assert b"no CUDA device" in lib.dtrt_last_error()


def test_invalid_arguments_are_statuses(lib):
    spec = scenes.config0(8, 8, nder=1)
    desc, keep = spec.to_desc()
    desc.nder = 2
    h = ctypes.c_void_p()
    assert lib.dtrt_scene_create(ctypes.byref(desc), ctypes.byref(h)) == 4
    assert lib.dtrt_scene_create(None, ctypes.byref(h)) == 1
    assert lib.dtrt_render_fwd(None, None, None, 0, None) == 1
    assert lib.dtrt_scene_destroy(None) == 0
    assert lib.dtrt_scene_update(None, ctypes.byref(desc), 0, None) == 1


def test_vol_reader_roundtrip(lib, tmp_path):
    g = np.random.default_rng(3).random((5, 6, 7)).astype(np.float32)
    p = str(tmp_path / "g.vol")
    scenes.write_vol(p, g, (-1, -2, -3), (1, 2, 3))
    res = (ctypes.c_int * 3)()
    ch = ctypes.c_int()
    vmin, vmax = (ctypes.c_float * 3)(), (ctypes.c_float * 3)()
    assert lib.dtrt_vol_read(p.encode(), res, ctypes.byref(ch), vmin, vmax, None) == 0
    assert list(res) == [7, 6, 5] and ch.value == 1
    assert list(vmin) == [-1, -2, -3] and list(vmax) == [1, 2, 3]
    data = np.zeros(g.size, np.float32)
    assert lib.dtrt_vol_read(p.encode(), res, ctypes.byref(ch), vmin, vmax, data.ctypes.data_as(_abi.c_float_p)) == 0
    assert np.array_equal(data.reshape(g.shape), g)
    back, lo, hi = scenes.read_vol(p)
    assert np.array_equal(back, g)
    assert lib.dtrt_vol_read(b"/nonexistent.vol", res, ctypes.byref(ch), vmin, vmax, None) == 5
