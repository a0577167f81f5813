"""Host BVH build and refit (dtrt_gb300/csrc/dt_bvh.cpp), compiled into a small driver with
g++ (no GPU): the refit that dtrt_scene_update uses reproduces a build bit for bit when the
positions are unchanged, keeps every box around its triangles after a deformation, and the
surface-area cost ratio separates a small displacement from a fold."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from dtrt_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = "/usr/local/cuda/include"

DRIVER = r"""
#include "dt_bvh.h"
#include <cstdio>
#include <cstring>
#include <vector>
using namespace dt;
static bool read(const char *path, std::vector<float> &a, std::vector<float> &b, int &n) {
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    bool ok = fread(&n, 4, 1, f) == 1;
    a.resize(9 * (size_t)n); b.resize(9 * (size_t)n);
    ok = ok && fread(a.data(), 4, a.size(), f) == a.size() && fread(b.data(), 4, b.size(), f) == b.size();
    fclose(f);
    return ok;
}
static bool inside(const float *lo, const float *hi, const float *p) {
    for (int a = 0; a < 3; ++a) if (p[a] < lo[a] || p[a] > hi[a]) return false;
    return true;
}
// every leaf triangle of child `code` lies in the box (lo, hi)
static bool check(const BvhBuildOut &t, const std::vector<float> &tv, int code, const float *lo, const float *hi) {
    if (code >= 0) {
        const BvhNode &nd = t.nodes[code];
        const float l0[3] = {nd.x.x, nd.y.x, nd.z.x}, h0[3] = {nd.x.y, nd.y.y, nd.z.y};
        const float l1[3] = {nd.x.z, nd.y.z, nd.z.z}, h1[3] = {nd.x.w, nd.y.w, nd.z.w};
        for (int a = 0; a < 3; ++a)
            if (l0[a] < lo[a] || h0[a] > hi[a] || l1[a] < lo[a] || h1[a] > hi[a]) return false;
        return check(t, tv, nd.child.x, l0, h0) && check(t, tv, nd.child.y, l1, h1);
    }
    const int v = ~code, base = v >> 3, count = (v & 7) + 1;
    for (int k = base; k < base + count; ++k) {
        int id;
        memcpy(&id, &t.leaf_tris[3 * (size_t)k].w, 4);
        for (int q = 0; q < 3; ++q) if (!inside(lo, hi, &tv[9 * (size_t)id + 3 * q])) return false;
    }
    return true;
}
int main(int argc, char **argv) {
    std::vector<float> a, b;
    int n;
    if (!read(argv[1], a, b, n)) return 2;
    BvhBuildOut built, refit;
    build_bvh(a, n, built);
    refit = built;
    refit_bvh(a, refit);
    const bool same = refit.nodes.size() == built.nodes.size() &&
                      memcmp(refit.nodes.data(), built.nodes.data(), built.nodes.size() * sizeof(BvhNode)) == 0 &&
                      memcmp(refit.leaf_tris.data(), built.leaf_tris.data(), built.leaf_tris.size() * 16) == 0;
    const double c0 = bvh_sah_cost(built);
    refit_bvh(b, refit);
    const BvhNode &r = refit.nodes[0];
    const float rl[3] = {-1e30f, -1e30f, -1e30f}, rh[3] = {1e30f, 1e30f, 1e30f};
    const bool bounds = check(refit, b, 0, rl, rh) && r.child.x != 0;
    printf("%d %d %.6f\n", same ? 1 : 0, bounds ? 1 : 0, bvh_sah_cost(refit) / c0);
    return 0;
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if not shutil.which("g++") or not os.path.isdir(CUDA_INC):
        pytest.skip("g++ or the CUDA headers are missing")
    d = tmp_path_factory.mktemp("bvh")
    src = d / "drv.cpp"
    src.write_text(DRIVER)
    exe = d / "drv"
    csrc = os.path.join(ROOT, "dtrt_gb300", "csrc")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", csrc, "-I", CUDA_INC, str(src), os.path.join(csrc, "dt_bvh.cpp"),
                    "-o", str(exe)], check=True)
    return d, exe


def tris(spec):
    return np.concatenate([s.vertices[s.indices].reshape(-1, 9) for s in spec.shapes]).astype(np.float32)


def run(driver, a, b):
    d, exe = driver
    path = d / "tv.bin"
    path.write_bytes(np.int32(a.shape[0]).tobytes() + a.tobytes() + b.tobytes())
    out = subprocess.run([str(exe), str(path)], capture_output=True, text=True, check=True).stdout.split()
    return int(out[0]), int(out[1]), float(out[2])


def deformed(fn):
    s = scenes.config2(16, 16, subdiv=4, nder=1, seed=2)
    s.shapes[0].vertices = fn(s.shapes[0].vertices.astype(np.float64)).astype(np.float32)
    return tris(s)


def test_refit_reproduces_build_and_bounds(driver):
    base = tris(scenes.config2(16, 16, subdiv=4, nder=1, seed=2))
    small = tris(scenes.config2(16, 16, subdiv=4, nder=1, seed=2, displaced=True, sigma=0.01))
    same, bounds, ratio = run(driver, base, small)
    assert same == 1 and bounds == 1
    assert 1.0 <= ratio < 1.2


def test_cost_ratio_flags_folds_not_stretches(driver):
    base = tris(scenes.config2(16, 16, subdiv=4, nder=1, seed=2))
    fold = deformed(lambda v: v + np.stack([0 * v[:, 0], 1.5 * np.sign(np.sin(6 * np.pi * v[:, 0])), 0 * v[:, 0]], 1))
    _, bounds, r_fold = run(driver, base, fold)
    assert bounds == 1 and r_fold > 2.0  # dtrt_scene_update builds this tree again
    stretch = deformed(lambda v: v * np.array([3.0, 1.0, 1.0]))
    _, bounds, r_stretch = run(driver, base, stretch)
    assert bounds == 1 and r_stretch < 2.0  # refit kept: a new tree is no better here
