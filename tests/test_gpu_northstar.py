"""Forward-mode parity at the benchmark configurations' own scene sizes and derivative
widths, against the FP64 oracle, plus the 4096-spp image gate.

The scenes are the full-size C1 (64^3 grid, 512x512), C2 (20480-triangle sphere, nder 8)
and C3 (128^3 grid, nder 8 with the grid's translation and rotation slots,
gridvolume.h:282-312 / heterogeneous.h:46-75 of the reference); only a window of each
image is rendered (Camera.set_rect), so that the oracle finishes in seconds. Parity is
the block z-test of statcheck.assert_parity with 256 GPU and 64 oracle renders (16 batch
means per side)."""
import numpy as np
import pytest

import statcheck
from dtrt_gb300 import scenes

pytestmark = pytest.mark.gpu

RUNS = 16
# Edge-sampled derivative estimates are heavy-tailed: statcheck reduces each side's runs to
# 16 batch means before the test. GPU runs are cheap, so the GPU side takes more of them.
GPU_RUNS, CPU_RUNS = 256, 64


def _pair(native, oracle, spec, kw, gseed=1000, cseed=5000, gruns=GPU_RUNS, cruns=CPU_RUNS):
    with native.NativeScene(spec) as s:
        g = np.stack([s.render(seed=gseed + k, **kw) for k in range(gruns)])
    c = np.stack([oracle.render(spec, seed=cseed + k, **kw) for k in range(cruns)])
    return g, c


def test_c1_full_grid_window_parity(native, oracle):
    spec = scenes.with_crop(scenes.config1(512, 512), 32, 32)
    kw = dict(spp=16, max_bounces=10, sppe=0, sppse=10)
    g, c = _pair(native, oracle, spec, kw)
    print(statcheck.assert_parity(g, c, label="C1 64^3 window"))
    assert np.abs(g[:, 1:]).sum(axis=(0, 2, 3, 4)).min() > 0  # all three derivative slots live


def test_c3_forward_nder8_parity(native, oracle):
    """C3 forward mode at nder 8: density scale, albedo, g, grid translation x/y/z,
    grid rotation about y and x."""
    spec = scenes.with_crop(scenes.config3(512, 512), 32, 32)
    kw = dict(spp=16, max_bounces=16, sppe=0, sppse=10)
    g, c = _pair(native, oracle, spec, kw)
    print(statcheck.assert_parity(g, c, label="C3 nder 8 window"))
    live = np.abs(g[:, 1:]).sum(axis=(0, 2, 3, 4))
    assert (live > 0).all(), live  # every slot, translation and rotation included, carries derivatives


def test_c2_nder8_parity(native, oracle):
    """C2 at nder 8 on the full 20480-triangle sphere: a window across the silhouette,
    interior, secondary-edge and primary-edge terms."""
    spec = scenes.with_crop(scenes.config2(256, 256), 32, 32, x=112, y=56)
    kw = dict(spp=8, max_bounces=4, sppe=64, sppse=4)
    g, c = _pair(native, oracle, spec, kw)
    print(statcheck.assert_parity(g, c, label="C2 nder 8 window"))
    assert (np.abs(g[:, 1:]).sum(axis=(0, 2, 3, 4)) > 0).all()


@pytest.mark.parametrize("name", ["c0", "c1"])
def test_4096spp_image_mean_error(native, oracle, name):
    """A 4096-spp image: relative error of its mean against the oracle's 4096-spp image
    <= 1%, and per-block agreement at 3 sigma (16 runs of 256 spp per side).

    C0: 32x32 window of the 256x256 image. C1: the whole frame at 64x64 (a window of the
    caustic-heavy cube alone has an oracle-vs-oracle spread of the mean near 1% at 4096
    spp, which would make the gate a noise test)."""
    if name == "c0":
        spec = scenes.with_crop(scenes.config0(256, 256), 32, 32)
        kw = dict(spp=256, max_bounces=5, sppe=0, sppse=10)
    else:
        spec = scenes.config1(64, 64)
        kw = dict(spp=256, max_bounces=10, sppe=0, sppse=10)
    g, c = _pair(native, oracle, spec, kw, gseed=7000, cseed=9000, gruns=RUNS, cruns=RUNS)
    gi, ci = g[:, 0].mean(0), c[:, 0].mean(0)  # 16 x 256 = 4096 spp images
    mre = statcheck.image_mean_rel_error(gi, ci)
    # standard error of that difference from the run-to-run spread of the image means
    sg, sc = g[:, 0].mean(axis=(1, 2, 3)), c[:, 0].mean(axis=(1, 2, 3))
    se = np.sqrt(sg.var(ddof=1) / RUNS + sc.var(ddof=1) / RUNS) / abs(ci.mean())
    print(f"{name}: 4096-spp image mean relative error {mre:.5f} (standard error {se:.5f}), "
          f"relative L1 {statcheck.rel_l1(gi, ci):.4f}")
    assert mre <= 0.01, (mre, se)
    print(statcheck.assert_parity(g[:, :1], c[:, :1], label=f"{name} 4096 spp"))
