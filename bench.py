#!/usr/bin/env python
"""Benchmark of the forward-mode differentiable volumetric path tracer on GB300.

One step = one forward-mode render (image + nder derivative images) of the workload
scene. Default workload: C1 (512x512, 64 spp, max depth 10, nder 3: a 64^3 seeded
Gaussian-blob density grid inside a smooth-dielectric cube; derivatives w.r.t. the
density scale, the albedo and the HG g). Scenes are seeded synthetic scenes (no
dataset). Prints one JSON line (rank 0).

  python bench.py [--gpus N --steps K --warmup W --config c0|c1|c2|c3]
  python bench.py --impl reference ...   # the reference's CPU algorithm (FP64 oracle port)

N > 1 (torchrun): independent replicas, one per GPU (the path tracer does not shard
in this build), value = paths of all ranks / slowest rank's time.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "paths/s + time to 1% grad RMSE: adjoint vs fwd-mode on 1 GB300; CPU ref beside"

WORKLOADS = {
    "c0": dict(desc="C0 null-bounded homogeneous icosphere (1280 tris), diffuse ground, 1x1 area light; "
                    "derivative = sphere x-translation", w=256, h=256, spp=32, depth=5, nder=1, sppse=10, sppe=1024),
    "c1": dict(desc="C1 64^3 Gaussian-blob grid (8 blobs, scale 5, albedo 0.9, HG g=0.3) in a smooth-dielectric "
                    "cube; derivatives = scale, albedo, g", w=512, h=512, spp=64, depth=10, nder=3, sppse=10, sppe=1024),
    "c2": dict(desc="C2 diffuse icosphere 20480 tris, 8 seeded vertex directions", w=256, h=256, spp=64, depth=4,
               nder=8, sppse=10, sppe=1024),
    "c3": dict(desc="C3 128^3 grid of 32 blobs in a null-bounded cube (scale 8, albedo 0.95, HG 0.5), nder 8 "
                    "(scale, albedo, g, translation, rotation)", w=512, h=512, spp=128, depth=16, nder=8, sppse=10,
               sppe=1024),
}


def workload_config(name, world, spec=None):
    """The `config` of both arms' lines: the workload, its sizes and the run's layout."""
    wl = WORKLOADS[name]
    return {"workload": wl["desc"], "width": spec.width if spec else wl["w"],
            "height": spec.height if spec else wl["h"], "spp": wl["spp"], "max_bounces": wl["depth"],
            "nder": wl["nder"], "sppse": wl["sppse"], "sppe": wl["sppe"], "parallelism": f"replicas x{world}",
            "l2": "flushed between timed steps (256 MiB write)", "accumulation": "f64"}


def build_spec(name, size=None):
    """The workload scene; `size` overrides the image side (small ncu captures only)."""
    from dtrt_gb300 import scenes
    wl = WORKLOADS[name]
    w = h = size if size else None
    w, h = w or wl["w"], h or wl["h"]
    if name == "c0":
        return scenes.config0(w, h, nder=wl["nder"])
    if name == "c1":
        return scenes.config1(w, h, nder=wl["nder"])
    if name == "c2":
        return scenes.config2(w, h, nder=wl["nder"])
    return scenes.config3(w, h, nder=wl["nder"])


def render_kw(name, seed):
    wl = WORKLOADS[name]
    return dict(seed=seed, spp=wl["spp"], max_bounces=wl["depth"], sppe=wl["sppe"], sppse=wl["sppse"])


def spec_h2d_bytes(spec):
    n = 0
    for s in spec.shapes:
        for a in (s.vertices, s.indices, s.normals, s.uvs, s.velocities):
            if a is not None:
                n += np.asarray(a).nbytes
    for m in spec.media:
        for a in (m.density, m.albedo_grid):
            if a is not None:
                n += np.asarray(a).nbytes
    return int(n)


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi sampling every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = tempfile.mktemp(suffix=".csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = max(float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


# --------------------------------------------------------------------------- replicas
def max_over_ranks(ms, world, device="cuda"):
    """The slowest rank's time (ms): replicas run in parallel, the job ends with the last."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([ms], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank_step, steps, world, ms_local, device="cuda"):
    """Whole-job throughput: the units every rank processed over the slowest rank's time."""
    t_max = max_over_ranks(ms_local, world, device)
    return units_per_rank_step * steps * world / (t_max / 1e3), t_max


# --------------------------------------------------------------------------- reference arm
def run_reference(args, wl_name, rank):
    """The reference's CPU algorithm (IntegratorAD::render + VolPathTracerAD restated in
    FP64 C++/OpenMP; the reference itself needs Eigen + Embree, absent here) on all host
    cores, one bounded crop of the workload per step."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    wl = WORKLOADS[wl_name]
    spec = build_spec(wl_name)
    cores = os.cpu_count() or 1
    spp, _ = choose_cpu_spp(oracle_py, spec, wl_name, target_s=args.cpu_seconds_per_step, nthreads=cores)
    kw = lambda seed: dict(render_kw(wl_name, seed), spp=spp)
    for k in range(min(args.warmup, 1)):
        oracle_py.render(spec, **kw(1000 + k), nthreads=cores)
    t0 = time.perf_counter()
    for k in range(args.steps):
        oracle_py.render(spec, **kw(k), nthreads=cores)
    dt = (time.perf_counter() - t0) / args.steps
    paths = spec.width * spec.height * spp
    v = paths / dt
    sample = f"full {spec.width}x{spec.height} image at {spp} spp per step (workload: {wl['spp']} spp), all other settings equal"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "paths/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded scene generator)",
            "config": workload_config(wl_name, args.gpus),
            "cpu_baseline": {"value": v, "unit": "paths/s", "cores": cores, "kind": "port",
                             "sample": sample, "cpu": cpu_model()},
            "e2e": {"value": v, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "derivative_samples_per_s": v * wl["nder"]}
    print(json.dumps(line), flush=True)


def choose_cpu_spp(oracle_py, spec, wl_name, target_s=4.0, nthreads=0):
    """Samples per pixel of a full-image oracle render taking about target_s seconds
    (every camera path has the distribution of the full workload's paths)."""
    wl = WORKLOADS[wl_name]
    kw = render_kw(wl_name, 99)
    kw["spp"] = 1
    t0 = time.perf_counter()
    oracle_py.render(spec, **kw, nthreads=nthreads)
    dt = max(time.perf_counter() - t0, 1e-3)
    return int(max(1, min(wl["spp"], round(target_s / dt)))), dt


# --------------------------------------------------------------------------- GPU arm
def roofline_of(wl_name, spec, cstats, kms, steps, paths_per_step, full_size=True):
    """Roofline of the dominant kernel stage: algorithmic bytes per step (device counters of
    one instrumented render: 64 B per BVH node visit, 48 B per triangle test, 32 B per
    trilinear lookup, 8 B per light-CDF probe, and for the wavefront camera stage the path
    state read and written per vertex launch) over the stage's CUDA-event time per step
    (kms: stage -> ms summed over `steps` renders); traffic = DRAM bytes per path of an ncu
    capture of that stage over one full render (profiles/traffic.json), scaled to the step."""
    kernels = ["camera", "edge", "li", "lins", "primary"]
    dom = max(kms, key=kms.get)
    ki = kernels.index(dom)
    node_b, tri_b, grid_b = 64, 48, 32
    probe_b = 8 * light_cdf_probes(spec)  # one FP32/FP64 CDF entry per binary-search step
    state_b = cstats["camera_state_bytes"] if dom == "camera" else 0
    alg_terms = {"bvh_nodes": node_b * cstats["k_node_visits"][ki], "triangles": tri_b * cstats["k_tri_tests"][ki],
                 "grid_lookups": grid_b * cstats["k_grid_lookups"][ki],
                 "light_cdf_probes": probe_b * cstats["k_light_samples"][ki], "path_state": state_b}
    alg_bytes = sum(alg_terms.values())
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg_bytes / (kms[dom] / steps / 1e3) / 1e9 if kms[dom] > 0 else 0.0
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tfile) and full_size:
        t = json.load(open(tfile)).get(f"{wl_name}:{dom}")
        if t:
            traffic = t["dram_bytes_per_path"] * paths_per_step
    kname = f"k_{dom}"
    if dom == "camera" and cstats.get("camera_schedule") == 2:
        kname = ("k_cam_vertex (camera stage: k_cam_start, then per vertex level k_cam_vertex for the "
                 "volume and the interface vertices, k_cam_accum)")
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if peak else None, "traffic": traffic, "kernel": kname,
            "peak_source": "measured" if peaks else "fallback",
            "bytes_per_step": alg_bytes, "bytes_per_step_terms": alg_terms,
            "traffic_over_algorithmic": traffic / alg_bytes if traffic and alg_bytes else None,
            "bytes_model": "64 B per BVH node visit + 48 B per triangle test + 32 B per trilinear lookup + "
                           "8 B per light-CDF probe (binary-search steps per emitter sample) + the wavefront "
                           "path-state bytes read and written per vertex launch (CamState + VertexIn; device "
                           "counters of one instrumented render)",
            "traffic_note": "DRAM read+write per path of the stage's launches over one full render (ncu, "
                            "profiles/traffic.json), scaled to the step's paths"}


def run_gpu(args, wl_name, rank, world, local_rank):
    import torch
    from dtrt_gb300 import native
    torch.cuda.set_device(local_rank)
    wl = WORKLOADS[wl_name]
    spec = build_spec(wl_name, args.size)
    paths_per_step = spec.width * spec.height * wl["spp"]
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    out = torch.empty(spec.out_shape(), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    scene = native.NativeScene(spec)
    # instrumented render (device counters) for the roofline bytes
    scene.enable_counters(True)
    scene.render(out.data_ptr(), stream=sptr, **render_kw(wl_name, 12345))
    cstats = scene.last_stats()
    scene.enable_counters(False)
    for k in range(args.warmup):
        scene.render(out.data_ptr(), stream=sptr, **render_kw(wl_name, 1000 + k))
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stage = {"ms_camera": 0.0, "ms_edge": 0.0, "ms_li": 0.0, "ms_primary": 0.0}
    launches = 0
    runs = []  # the timed renders' images, kept (after the step's end event) for the FP64 comparison
    for k in range(args.steps):
        flush.zero_()  # L2 flushed between timed steps (not timed)
        ev[k][0].record(stream)
        scene.render(out.data_ptr(), stream=sptr, **render_kw(wl_name, k))
        ev[k][1].record(stream)
        runs.append(out.clone())
        st = scene.last_stats()
        for key in stage:
            stage[key] += st[key]
        launches += st["kernel_launches"]
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    value, t_max = job_throughput(paths_per_step, args.steps, world, ms, "cuda")
    # end to end through the public API with host buffers: scene upload + BVH build + render + D2H
    e2e_steps = max(1, min(args.steps, 3))
    host_t = torch.zeros(spec.out_shape(), dtype=torch.float32).pin_memory()  # pinned result buffer
    host_out = host_t.numpy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        with native.NativeScene(spec) as s2:
            s2.render(host_out, **render_kw(wl_name, 500 + k))
    e2e_dt = (time.perf_counter() - t0) / e2e_steps
    e2e = {"value": paths_per_step * world / e2e_dt, "unit": "paths/s", "h2d_bytes_per_step": spec_h2d_bytes(spec),
           "d2h_bytes_per_step": int(host_out.nbytes), "ms_per_step": e2e_dt * 1e3}
    kms = {"camera": stage["ms_camera"], "edge": stage["ms_edge"], "li": stage["ms_li"],
           "primary": stage["ms_primary"]}
    roofline = roofline_of(wl_name, spec, cstats, kms, args.steps, paths_per_step, args.size is None)
    line = {"metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
            "config": workload_config(wl_name, world, spec),
            "roofline": roofline, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
            "derivative_samples_per_s": value * wl["nder"],
            "stages_ms_per_step": {k: v / args.steps for k, v in stage.items()},
            "counters_per_path": {"rays": cstats["rays"] / paths_per_step,
                                  "node_visits": cstats["node_visits"] / paths_per_step,
                                  "tri_tests": cstats["tri_tests"] / paths_per_step,
                                  "grid_lookups": cstats["grid_lookups"] / paths_per_step,
                                  "edge_records": cstats["edge_records"] / paths_per_step,
                                  "li_tasks": cstats["li_tasks"] / paths_per_step,
                                  "light_samples": cstats["light_samples"] / paths_per_step,
                                  "camera_state_bytes": cstats["camera_state_bytes"] / paths_per_step}}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"], cpu_imgs = cpu_baseline(wl_name, args.cpu_seconds_per_step, args.size, keep_images=True)
        line["error_vs_fp64"] = error_vs_fp64(torch.stack(runs).cpu().numpy(), cpu_imgs, wl["spp"],
                                              line["cpu_baseline"]["spp_per_run"])
    runs.clear()
    if rank == 0 and not args.no_c3:
        line["c3_forward"] = c3_forward(args.no_cpu_baseline)
    if rank == 0 and not args.no_grad_rmse:
        line["adjoint"] = adjoint_throughput_c3()
        line["grad_rmse"] = grad_rmse_c3(size=args.grad_size)
        line["grad_rmse_c2"] = grad_rmse_c2()
    if rank == 0 and not args.no_batch:
        line["batch_c4"] = batch_c4()
    if rank == 0 and not args.no_update:
        line["scene_update_c2"] = scene_update_c2()
    scene.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- gradient accuracy vs time
def rmse_summary(G, run_spp, g_ref, ref_spp):
    """Gradient error against a high-spp forward-mode reference g_ref (ref_spp samples per
    pixel; same estimator): the bias of the run mean and its standard error, and the spp at
    which the RMSE sqrt(|bias|^2 + tr Cov(run) * run_spp / spp) falls to 1% of |g_ref|
    (variance term measured from the runs). |g_hat - g_ref|^2 holds the Monte Carlo noise
    of both sides, tr Cov / runs + tr Cov run_spp / ref_spp in expectation; the bias term
    of the spp estimate is the excess over that noise (0 when the difference is all noise)."""
    runs = G.shape[0]
    g_hat = G.mean(0)
    tr = float(G.var(0, ddof=1).sum())
    ref2 = float(g_ref @ g_ref)
    b = g_hat - g_ref
    bias2 = float(b @ b)
    noise2 = tr / runs + tr * run_spp / ref_spp  # expected |g_hat - g_ref|^2 of an unbiased estimator
    bias2_excess = max(0.0, bias2 - noise2)
    target2 = 1e-4 * ref2
    spp_var_only = run_spp * tr / target2
    spp_with_bias = run_spp * tr / (target2 - bias2_excess) if bias2_excess < target2 else float("inf")
    return {"reference": f"forward mode at {ref_spp} spp", "rel_diff": float(np.sqrt(bias2 / ref2)),
            "rel_noise_expected": float(np.sqrt(noise2 / ref2)),
            "rel_bias_excess": float(np.sqrt(bias2_excess / ref2)),
            "diff_over_noise": float(bias2 / noise2) if noise2 > 0 else None,
            "spp_to_1pct_variance_only": spp_var_only, "spp_to_1pct_with_bias": spp_with_bias}


def grad_rmse_c3(size=None, runs=16, run_spp=64, ladder_max=64, seed=31, ref_spp=2048, full_passes=4):
    """Time to 1% gradient RMSE on the 128^3-grid volume-density workload (C3: 512x512,
    depth 16, scale 8, albedo 0.95, HG 0.5): the reverse-mode adjoint (dtrt_render_adjoint,
    one replay pass gives all 2,097,152 voxel derivatives) against the forward-mode path
    (dtrt_render_fwd with per-voxel density directions, 8 per pass).

    Quantities: the gradient of an L2 image loss (target: the same grid with +-20% blob
    amplitudes) along the shapes of 8 of the 32 blobs (the derivatives with respect to
    those amplitudes) and at 16 random voxels inside the blobs: 24 numbers = 3 forward
    passes of nder 8, or 1 adjoint pass.

    Both methods trace the same paths for the same seed (the adjoint is the transpose of
    the forward-mode estimator), so their per-seed estimates coincide (checked on a ladder
    of runs) and so does the spp at which the relative RMSE sqrt(E||g_s - g||^2) / ||g||
    reaches 1%. That spp is estimated from `runs` independent adjoint runs at run_spp:
    E||g_s - g||^2 = tr Cov(g_run) * run_spp / s, with a bootstrap interval. The time of
    each method is that spp times its measured CUDA-event time per spp."""
    import torch
    from dtrt_gb300 import native, scenes
    W = H = size or 512
    res, depth = 128, 16
    spec = scenes.config3(W, H, res=res, nder=8, param_slots=False)
    tgt = scenes.config3(W, H, res=res, nder=8, param_slots=False, amp_jitter=0.2)
    grid = spec.media[0].density
    rng = np.random.default_rng(seed)
    _, (centres, sigmas, _amps) = scenes.blob_grid(res, 32, 3)  # the generator of config3's grid
    blobs = np.stack([scenes.blob_field(res, centres[k], sigmas[k]) for k in range(8)])
    inner = np.zeros_like(grid, bool)
    inner[1:-1, 1:-1, 1:-1] = True
    vox = rng.choice(np.flatnonzero((grid > 0.2 * grid.max()) & inner), size=16, replace=False)
    unit = np.zeros((16,) + grid.shape, np.float32)
    for i, v in enumerate(vox):
        unit[i].flat[v] = 1.0
    sets = [blobs.astype(np.float32), unit[:8], unit[8:]]
    kw = dict(max_bounces=depth, sppe=0, sppse=10)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    fwd_scenes = []
    for d in sets:
        sc = native.NativeScene(spec)
        sc.set_density_derivatives(0, d)
        fwd_scenes.append(sc)
    adj_scene = fwd_scenes[0]
    with native.NativeScene(tgt) as nt:
        T = nt.render_adjoint(None, image=True, density_grad=False, seed=2, spp=512, **kw)[0]
    I = adj_scene.render_adjoint(None, image=True, density_grad=False, seed=1, spp=512, **kw)[0]
    dimg = torch.from_numpy(2.0 * (I - T) / I.size).cuda()
    dirs_dev = torch.from_numpy(blobs.reshape(8, -1)).cuda()
    vox_dev = torch.from_numpy(vox).cuda()
    out = torch.empty(spec.out_shape(), dtype=torch.float32, device="cuda")
    grad = torch.empty(res ** 3, dtype=torch.float32, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def forward_mode(spp, sd):
        vals, ms = [], 0.0
        for sc in fwd_scenes:
            e0.record(stream)
            sc.render(out.data_ptr(), stream=sptr, seed=sd, spp=spp, **kw)
            e1.record(stream)
            torch.cuda.synchronize()
            ms += e0.elapsed_time(e1)
            vals.append((dimg[None] * out[1:]).double().sum(dim=(1, 2, 3)))
        return torch.cat(vals).cpu().numpy(), ms

    def adjoint(spp, sd):
        e0.record(stream)
        adj_scene.render_adjoint(dimg.data_ptr(), image=None, density_grad=grad.data_ptr(), stream=sptr, device=True,
                                 seed=sd, spp=spp, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
        g = grad.double()
        v = torch.cat([dirs_dev.double() @ g, g[vox_dev]])
        return v.cpu().numpy(), e0.elapsed_time(e1)

    t0 = time.perf_counter()
    G = np.stack([adjoint(run_spp, 30000 + r)[0] for r in range(runs)])
    g_hat = G.mean(0)
    gn2 = float(g_hat @ g_hat)

    def spp_1pct(Gs):
        m = Gs.mean(0)
        return run_spp * float(Gs.var(0, ddof=1).sum()) / (1e-4 * float(m @ m))

    s1 = spp_1pct(G)
    brng = np.random.default_rng(0)
    boots = sorted(spp_1pct(G[brng.integers(0, runs, runs)]) for _ in range(200))
    t_var = time.perf_counter() - t0
    # high-spp forward-mode reference for the gradient (the run mean's bias is measured against it)
    g_ref = forward_mode(ref_spp, 777)[0]
    result = {"workload": f"C3 {W}x{H}, {res}^3 grid, depth {depth}, L2 loss vs +-20% amplitude target",
              "against_reference": rmse_summary(G, run_spp, g_ref, ref_spp),
              "quantities": "derivatives along 8 blob-amplitude directions + at 16 random voxels (24)",
              "variance_runs": {"runs": runs, "spp": run_spp, "seconds": t_var,
                                "rel_se_of_mean": float(np.sqrt(G.var(0, ddof=1).sum() / runs / gn2))},
              "spp_to_1pct": s1, "spp_to_1pct_bootstrap_90": [boots[10], boots[189]], "threshold": 0.01}
    ladders = {}
    for name, fn in (("adjoint", adjoint), ("forward_mode", forward_mode)):
        ladder, spp = [], 1
        while spp <= ladder_max:
            v, ms = fn(spp, 20000 + spp)
            ladders.setdefault(spp, []).append(v)
            ladder.append({"spp": spp, "ms": ms, "rel_err_vs_mean": float(np.linalg.norm(v - g_hat) / np.sqrt(gn2))})
            spp *= 2
        ms_per_spp = ladder[-1]["ms"] / ladder[-1]["spp"]
        result[name] = {"ladder": ladder, "ms_per_spp": ms_per_spp, "ms_to_1pct": s1 * ms_per_spp}
    # same seed, same paths: the two methods' estimates agree run by run
    result["max_rel_diff_adjoint_vs_forward"] = max(float(np.linalg.norm(a - b) / np.sqrt(gn2))
                                                    for a, b in ladders.values())
    a, f = result["adjoint"], result["forward_mode"]
    result["speedup_time_to_1pct"] = f["ms_to_1pct"] / a["ms_to_1pct"]
    # all 2,097,152 voxel derivatives by forward mode: one nder-8 pass per 8 voxels. The time
    # per pass is measured on `full_passes` real passes, each over 8 other random voxels;
    # the full gradient is that time times the pass count (not run: 262,144 passes).
    pass_ms = []
    for k in range(full_passes):
        u = np.zeros((8,) + grid.shape, np.float32)
        for i, v in enumerate(rng.choice(grid.size, size=8, replace=False)):
            u[i].flat[v] = 1.0
        fwd_scenes[1].set_density_derivatives(0, u)
        e0.record(stream)
        fwd_scenes[1].render(out.data_ptr(), stream=sptr, seed=4000 + k, spp=16, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
        pass_ms.append(e0.elapsed_time(e1) / 16)
    per_pass = float(np.mean(pass_ms)) * s1
    npass = res ** 3 // 8
    result["forward_mode_full_gradient"] = {"passes": npass, "measured_passes": full_passes,
                                            "ms_per_spp_measured": pass_ms, "s_estimate": per_pass * npass / 1e3}
    result["forward_mode_full_gradient_s_estimate"] = per_pass * npass / 1e3
    result["speedup_full_gradient_estimate"] = per_pass * npass / a["ms_to_1pct"]
    for sc in fwd_scenes:
        sc.close()
    return result


def grad_rmse_c2(size=None, runs=16, run_spp=16, ladder_max=16, ref_spp=1024, full_passes=4):
    """Time to 1% gradient RMSE on the mesh workload (C2: 20480-triangle diffuse icosphere,
    256x256, depth 4, sppse 10, primary-edge samples 16 per spp): the vertex-position adjoint
    (one replay gives all 30,726 vertex coordinates) against forward mode (8 seeded unit
    vertex directions per nder-8 pass). L2 image loss against the target with every vertex
    displaced along its normal by N(0, 0.01^2). Quantities: the gradient along the 8
    directions (1 forward pass or 1 adjoint pass). As for C3, both methods give the same
    estimate for the same seed, the spp to 1% relative RMSE comes from `runs` independent
    adjoint runs, and each method's time is that spp times its measured time per spp."""
    import torch
    from dtrt_gb300 import native, scenes
    W = H = size or 256
    spec = scenes.config2(W, H, nder=8)
    tgt = scenes.config2(W, H, nder=8, displaced=True)
    nv = spec.shapes[0].vertices.shape[0]
    V = torch.from_numpy(np.asarray(spec.shapes[0].velocities, np.float64).reshape(8, nv, 3)).cuda()
    kw = lambda spp: dict(max_bounces=4, sppse=10, sppe=16 * spp)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    with native.NativeScene(tgt) as nt:
        T = nt.render_adjoint(None, image=True, density_grad=False, seed=2, spp=256, max_bounces=4)[0]
    sc = native.NativeScene(spec)
    I = sc.render_adjoint(None, image=True, density_grad=False, seed=1, spp=256, max_bounces=4)[0]
    dimg = torch.from_numpy(2.0 * (I - T) / I.size).cuda()
    nvt = sc.gradient_sizes()[1]
    out = torch.empty(spec.out_shape(), dtype=torch.float32, device="cuda")
    grad = torch.empty((nvt, 3), dtype=torch.float32, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def forward_mode(spp, sd):
        e0.record(stream)
        sc.render(out.data_ptr(), stream=sptr, seed=sd, spp=spp, **kw(spp))
        e1.record(stream)
        torch.cuda.synchronize()
        return (dimg[None] * out[1:]).double().sum(dim=(1, 2, 3)).cpu().numpy(), e0.elapsed_time(e1)

    def adjoint(spp, sd):
        e0.record(stream)
        sc.render_vertex_adjoint(dimg.data_ptr(), image=None, vertex_grad=grad.data_ptr(), stream=sptr, device=True,
                                 seed=sd, spp=spp, **kw(spp))
        e1.record(stream)
        torch.cuda.synchronize()
        return (V * grad[:nv].double()[None]).sum(dim=(1, 2)).cpu().numpy(), e0.elapsed_time(e1)

    t0 = time.perf_counter()
    G = np.stack([adjoint(run_spp, 30000 + r)[0] for r in range(runs)])
    g_hat = G.mean(0)
    gn2 = float(g_hat @ g_hat)

    def spp_1pct(Gs):
        m = Gs.mean(0)
        return run_spp * float(Gs.var(0, ddof=1).sum()) / (1e-4 * float(m @ m))

    s1 = spp_1pct(G)
    brng = np.random.default_rng(0)
    boots = sorted(spp_1pct(G[brng.integers(0, runs, runs)]) for _ in range(200))
    g_ref = forward_mode(ref_spp, 777)[0]
    result = {"workload": f"C2 {W}x{H}, 20480-triangle diffuse icosphere, depth 4, L2 loss vs normal-displaced "
                          "target (N(0, 0.01^2))",
              "against_reference": rmse_summary(G, run_spp, g_ref, ref_spp),
              "quantities": "derivatives along 8 seeded unit vertex directions",
              "variance_runs": {"runs": runs, "spp": run_spp, "seconds": time.perf_counter() - t0,
                                "rel_se_of_mean": float(np.sqrt(G.var(0, ddof=1).sum() / runs / gn2))},
              "spp_to_1pct": s1, "spp_to_1pct_bootstrap_90": [boots[10], boots[189]], "threshold": 0.01}
    ladders = {}
    for name, fn in (("adjoint", adjoint), ("forward_mode", forward_mode)):
        ladder, spp = [], 1
        while spp <= ladder_max:
            v, ms = fn(spp, 20000 + spp)
            ladders.setdefault(spp, []).append(v)
            ladder.append({"spp": spp, "ms": ms, "rel_err_vs_mean": float(np.linalg.norm(v - g_hat) / np.sqrt(gn2))})
            spp *= 2
        ms_per_spp = ladder[-1]["ms"] / ladder[-1]["spp"]
        result[name] = {"ladder": ladder, "ms_per_spp": ms_per_spp, "ms_to_1pct": s1 * ms_per_spp}
    result["max_rel_diff_adjoint_vs_forward"] = max(float(np.linalg.norm(a - b) / np.sqrt(gn2))
                                                    for a, b in ladders.values())
    a, f = result["adjoint"], result["forward_mode"]
    result["speedup_time_to_1pct"] = f["ms_to_1pct"] / a["ms_to_1pct"]
    # all 30,726 vertex coordinates by forward mode: one nder-8 pass per 8 directions; the
    # time per pass measured on `full_passes` real passes with other random unit directions
    pass_ms = []
    prng = np.random.default_rng(11)
    for k in range(full_passes):
        dirs = prng.normal(size=(8, nv * 3))
        dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
        spec_k = scenes.config2(W, H, nder=8)
        spec_k.shapes[0].velocities = dirs.reshape(8 * nv, 3).astype(np.float32)
        with native.NativeScene(spec_k) as sk:
            sk.render(out.data_ptr(), stream=sptr, seed=4100 + k, spp=4, **kw(4))
            e0.record(stream)
            sk.render(out.data_ptr(), stream=sptr, seed=4000 + k, spp=16, **kw(16))
            e1.record(stream)
            torch.cuda.synchronize()
        pass_ms.append(e0.elapsed_time(e1) / 16)
    per_pass = float(np.mean(pass_ms)) * s1
    npass = -(-3 * nv // 8)
    result["forward_mode_full_gradient"] = {"passes": npass, "measured_passes": full_passes,
                                            "ms_per_spp_measured": pass_ms, "s_estimate": per_pass * npass / 1e3}
    result["forward_mode_full_gradient_s_estimate"] = per_pass * npass / 1e3
    result["speedup_full_gradient_estimate"] = per_pass * npass / a["ms_to_1pct"]
    sc.close()
    return result


def adjoint_throughput_c3(steps=3, warmup=1, size=512, spp=128):
    """Paths/s of the density adjoint (both replay passes) on the C3 workload (512x512,
    128 spp, depth 16, 128^3 grid), device-resident dL/dI and gradient."""
    import torch
    from dtrt_gb300 import native, scenes
    spec = scenes.config3(size, size, res=128, nder=8, param_slots=False)
    stream = torch.cuda.current_stream()
    dimg = torch.randn((size, size, 3), device="cuda") * 1e-3
    grad = torch.empty(128 ** 3, device="cuda")
    kw = dict(spp=spp, max_bounces=16, sppe=0, sppse=10)
    with native.NativeScene(spec) as sc:
        for k in range(warmup):
            sc.render_adjoint(dimg.data_ptr(), image=None, density_grad=grad.data_ptr(), stream=stream.cuda_stream,
                              device=True, seed=900 + k, **kw)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for k in range(steps):
            sc.render_adjoint(dimg.data_ptr(), image=None, density_grad=grad.data_ptr(), stream=stream.cuda_stream,
                              device=True, seed=k, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
    return {"workload": f"C3 {size}x{size}, {spp} spp, depth 16, 128^3 grid: full density gradient",
            "paths_per_s": size * size * spp / (ms / 1e3), "ms_per_pass": ms}


def batch_c4(n=64, side_scale=1.0, spp_scale=1.0, reps=2, tune_full=True):
    """C4: n seeded scenes of uneven size (1k-50k triangles, half with a 32^3-128^3 grid,
    128^2-512^2, 16-256 spp, depth 4-16), image + density gradient per scene, as one
    autotuned persistent launch replayed from a CUDA graph, against the same renders issued
    one scene at a time (dtrt_render_adjoint per scene) on the same stream."""
    import torch
    from dtrt_gb300 import native, scenes
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    items, total_paths = [], 0
    for i in range(n):
        spec, kw = scenes.config4(i, side_scale=side_scale, spp_scale=spp_scale)
        sc = native.NativeScene(spec)
        opts = sc.options(seed=100 + i, spp=kw["spp"], max_bounces=kw["max_bounces"], sppe=0)
        nvox = sc.gradient_sizes()[0]
        h, w = spec.height, spec.width
        dimg = torch.randn((h, w, 3), device="cuda") * 1e-3
        img = torch.zeros((h, w, 3), device="cuda")
        grad = torch.zeros(max(nvox, 1), device="cuda")
        items.append((sc, opts, dimg, img, grad, nvox))
        total_paths += h * w * kw["spp"]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def one_at_a_time():
        for sc, opts, dimg, img, grad, nvox in items:
            sc.render_adjoint(dimg.data_ptr(), image=img.data_ptr(), density_grad=grad.data_ptr() if nvox else None,
                              stream=sptr, device=True, options=opts)

    t0 = time.perf_counter()
    batch = native.Batch([(sc, opts, dimg.data_ptr(), img.data_ptr(), grad.data_ptr() if nvox else 0)
                          for sc, opts, dimg, img, grad, nvox in items], autotune=True, graph=True, stream=sptr,
                         tune_full=tune_full)
    tune_s = time.perf_counter() - t0
    one_at_a_time()  # warm-up
    batch.launch(sptr)  # warm-up
    torch.cuda.synchronize()
    # interleaved repetitions: both schedules run under the same clocks and power state
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    t_seq, t_batch = [], []
    for _ in range(reps):
        for fn, acc in ((one_at_a_time, t_seq), (lambda: batch.launch(sptr), t_batch)):
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            acc.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    ms_seq, ms_batch = float(np.median(t_seq)), float(np.median(t_batch))
    st = batch.stats()
    batch.close()
    for it in items:
        it[0].close()
    return {"workload": f"C4 {n} scenes (side x{side_scale}, spp x{spp_scale}): image + density gradient",
            "paths": total_paths, "ms_one_at_a_time": ms_seq, "ms_batch": ms_batch,
            "paths_per_s_batch": total_paths / (ms_batch / 1e3), "speedup": ms_seq / ms_batch,
            "tune_and_capture_s": tune_s, "schedule": st["schedule"], "streams": st["streams"],
            "chunk_paths": st["chunk_paths"],
            "order_longest_first": st["order_longest_first"], "grid_blocks": st["grid_blocks"],
            "confirm_trials_ms_quarter_of_items": st["full_size_ms"], "reps_ms": {"one_at_a_time": t_seq, "batch": t_batch},
            "clocks": clk, "trials": st["trials"]}


# --------------------------------------------------------------------------- scene rebuild per optimisation step
def scene_update_c2(iters=6, step=0.002, seed=5):
    """Host cost of the scene rebuild an optimisation step needs on C2 (20,480-triangle
    sphere, 256x256, nder 8), the vertices moved along their normals by a small random step
    each iteration: a new scene (BVH build, edge search, allocations and copies) against an
    in-place update (refit BVH, cached edge adjacency, arrays rewritten in place) and an
    in-place update with the BVH built again. Wall time, description conversion included."""
    import time
    from dtrt_gb300 import native, scenes
    spec = scenes.config2(256, 256, subdiv=5, nder=8)
    v = spec.shapes[0].vertices.copy()
    nrm = scenes.vertex_normals(v, spec.shapes[0].indices)
    rng = np.random.default_rng(seed)
    steps = []
    for _ in range(iters):
        v = (v + nrm * rng.normal(0.0, step, size=(v.shape[0], 1))).astype(np.float32)
        steps.append(v)

    def timed(fn):
        t = time.perf_counter()
        r = fn()
        return (time.perf_counter() - t) * 1e3, r

    ns = native.NativeScene(spec)
    native.NativeScene(spec).close()  # first-use costs out of the timings
    create, refit, rebuild, stats = [], [], [], []
    for vk in steps:
        spec.shapes[0].vertices = vk
        ms, sc = timed(lambda: native.NativeScene(spec))
        sc.close()
        create.append(ms)
    spec.shapes[0].vertices = v.copy()
    for vk in steps:
        spec.shapes[0].vertices = vk
        ms, st = timed(lambda: ns.update(spec))
        refit.append(ms)
        stats.append(st)
    for vk in steps:
        spec.shapes[0].vertices = vk
        ms, _ = timed(lambda: ns.update(spec, rebuild_bvh=True))
        rebuild.append(ms)
    ns.close()
    med = lambda a: float(np.median(a))
    return {"workload": f"C2 sphere, {sum(sh.indices.shape[0] for sh in spec.shapes)} triangles, 256x256, nder 8: "
                        f"{iters} steps of normal displacement (sigma {step})",
            "create_ms": med(create), "update_refit_ms": med(refit), "update_rebuild_bvh_ms": med(rebuild),
            "speedup_refit_vs_create": med(create) / med(refit),
            "bvh_refit": [s["bvh_refit"] for s in stats], "sah_ratio_last": stats[-1]["sah_ratio"],
            "buffers_reused": stats[-1]["buffers_reused"], "buffers_allocated": stats[-1]["buffers_allocated"],
            "host_ms_inside_update": med([s["host_ms"] for s in stats]),
            "update_phases_ms": {k: med([s[k] for s in stats]) for k in ("ms_bvh", "ms_arrays", "ms_device")}}


def cpu_baseline(wl_name, target_s, size=None, keep_images=False, runs=8):
    """The oracle port on all host cores over a bounded sample of the workload: the full
    image, `runs` independent renders of equal spp taking about target_s seconds in all."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    wl = WORKLOADS[wl_name]
    spec = build_spec(wl_name, size)
    cores = os.cpu_count() or 1
    spp, _ = choose_cpu_spp(oracle_py, spec, wl_name, target_s=target_s, nthreads=cores)
    per_run = max(1, spp // runs)
    imgs = []
    t0 = time.perf_counter()
    for r in range(runs):
        imgs.append(oracle_py.render(spec, **dict(render_kw(wl_name, 7 + r), spp=per_run), nthreads=cores))
    dt = time.perf_counter() - t0
    res = {"value": spec.width * spec.height * per_run * runs / dt, "unit": "paths/s", "cores": cores, "kind": "port",
           "sample": f"full {spec.width}x{spec.height} image, {runs} renders at {per_run} spp ({dt:.1f} s)",
           "spp_per_run": per_run, "cpu": cpu_model()}
    return (res, np.stack(imgs)) if keep_images else res


def error_vs_fp64(gpu_runs, cpu_runs, gpu_spp, cpu_spp, block=16):
    """Error of the timed GPU renders (FP32 paths, FP64 accumulation) against the FP64
    oracle's renders of the same workload (the CPU baseline's). Per slot (image, then each
    derivative image): the relative error of the whole-image mean with its standard error
    from the run-to-run spread, and the block z-test (block x block pixels): the fraction
    of blocks beyond 3 sigma next to the fraction a correct renderer gives by chance
    (Student t with the Welch degrees of freedom)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import statcheck
    out = {"gpu_renders": int(gpu_runs.shape[0]), "gpu_spp_per_render": gpu_spp,
           "oracle_renders": int(cpu_runs.shape[0]), "oracle_spp_per_render": cpu_spp, "block_pixels": block,
           "slots": []}
    z, ma, mb, se, df = statcheck.zscores(gpu_runs, cpu_runs, block)
    for sl in range(gpu_runs.shape[1]):
        g = gpu_runs[:, sl].astype(np.float64).mean(axis=(1, 2, 3))
        c = cpu_runs[:, sl].astype(np.float64).mean(axis=(1, 2, 3))
        ref = abs(c.mean()) if abs(c.mean()) > 0 else 1.0
        sem = float(np.sqrt(g.var(ddof=1) / len(g) + c.var(ddof=1) / len(c)) / ref)
        live = se[sl] > 0
        zs = z[sl][live]
        out["slots"].append({"slot": sl, "mean_rel_error": float(abs(g.mean() - c.mean()) / ref),
                             "mean_rel_error_se": sem, "blocks": int(zs.size),
                             "frac_blocks_beyond_3sigma": float((np.abs(zs) > 3).mean()) if zs.size else 0.0,
                             "null_frac": statcheck.null_exceedance_prob(df[sl][live]) if zs.size else 0.0})
    return out


def light_cdf_probes(spec):
    """Binary-search steps of one emitter sample: the light CDF, then the light shape's
    triangle-area CDF (scene.cpp:45-98, upper_bound over each)."""
    nl = max(1, len(spec.emitters))
    nt = max([spec.shapes[e.shape_id].indices.shape[0] for e in spec.emitters] or [1])
    return int(math.ceil(math.log2(nl + 1)) + math.ceil(math.log2(nt + 1)))


def c3_forward(no_cpu=False, steps=3, warmup=1, cpu_target_s=4.0):
    """Forward mode on the largest single-GPU configuration, C3 (512x512, 128 spp, depth 16,
    nder 8: density scale, albedo, g, grid translation x/y/z, rotation about y and x; 128^3
    grid), device-resident output, CUDA events; and the oracle port on the host cores over
    a bounded sample (the full image at a reduced spp)."""
    import torch
    from dtrt_gb300 import native
    spec = build_spec("c3")
    kw = lambda seed: render_kw("c3", seed)
    stream = torch.cuda.current_stream()
    out = torch.empty(spec.out_shape(), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    paths = spec.width * spec.height * WORKLOADS["c3"]["spp"]
    kms = {"camera": 0.0, "edge": 0.0, "li": 0.0, "primary": 0.0}
    with native.NativeScene(spec) as sc:
        sc.enable_counters(True)  # instrumented render: the roofline's algorithmic bytes
        sc.render(out.data_ptr(), stream=stream.cuda_stream, **kw(12345))
        cstats = sc.last_stats()
        sc.enable_counters(False)
        for k in range(warmup):
            sc.render(out.data_ptr(), stream=stream.cuda_stream, **kw(600 + k))
        ms = []
        for k in range(steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sc.render(out.data_ptr(), stream=stream.cuda_stream, **kw(k))
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
            st = sc.last_stats()
            for key in kms:
                kms[key] += st["ms_" + key]
    t = float(np.median(ms))
    res = {"workload": WORKLOADS["c3"]["desc"], "width": 512, "height": 512, "spp": WORKLOADS["c3"]["spp"],
           "max_bounces": 16, "nder": 8, "paths_per_s": paths / (t / 1e3), "ms_per_render": t,
           "derivative_samples_per_s": paths * 8 / (t / 1e3),
           "roofline": roofline_of("c3", spec, cstats, kms, steps, paths)}
    if not no_cpu:
        cb = cpu_baseline("c3", cpu_target_s, runs=1)
        res["cpu_baseline"] = cb
        res["speedup_vs_cpu"] = res["paths_per_s"] / cb["value"]
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--config", default="c1", choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds-per-step", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--size", type=int, default=None, help="image side override for small profiling runs")
    ap.add_argument("--no-grad-rmse", action="store_true", help="skip the adjoint vs forward-mode gradient leg")
    ap.add_argument("--grad-size", type=int, default=None, help="image side of the gradient leg (default 512)")
    ap.add_argument("--adjoint-only", action="store_true", help="time only the C3 density adjoint replay")
    ap.add_argument("--no-batch", action="store_true", help="skip the C4 batch leg")
    ap.add_argument("--no-update", action="store_true", help="skip the C2 scene rebuild leg")
    ap.add_argument("--no-c3", action="store_true", help="skip the C3 forward-mode leg")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.adjoint_only:  # the adjoint replay alone (small profiling runs with --size)
        print(json.dumps(adjoint_throughput_c3(steps=args.steps, warmup=args.warmup, size=args.size or 512)),
              flush=True)
        return
    if args.impl == "reference":
        if rank == 0:
            run_reference(args, args.config, rank)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    run_gpu(args, args.config, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
