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
            "config": {"workload": wl["desc"], "width": wl["w"], "height": wl["h"], "spp": wl["spp"],
                       "max_bounces": wl["depth"], "nder": wl["nder"], "sppse": wl["sppse"], "sppe": wl["sppe"]},
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
    for k in range(args.steps):
        flush.zero_()  # L2 flushed between timed steps (not timed)
        ev[k][0].record(stream)
        scene.render(out.data_ptr(), stream=sptr, **render_kw(wl_name, k))
        ev[k][1].record(stream)
        st = scene.last_stats()
        for key in stage:
            stage[key] += st[key]
        launches += st["kernel_launches"]
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    t_max = ms
    if world > 1:
        t = torch.tensor([ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_max = float(t.item())
    value = paths_per_step * args.steps * world / (t_max / 1e3)
    # end to end through the public API with host buffers: scene upload + BVH build + render + D2H
    e2e_steps = max(1, min(args.steps, 3))
    host_out = np.zeros(spec.out_shape(), np.float32)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        with native.NativeScene(spec) as s2:
            s2.render(host_out, **render_kw(wl_name, 500 + k))
    e2e_dt = (time.perf_counter() - t0) / e2e_steps
    e2e = {"value": paths_per_step * world / e2e_dt, "unit": "paths/s", "h2d_bytes_per_step": spec_h2d_bytes(spec),
           "d2h_bytes_per_step": int(host_out.nbytes), "ms_per_step": e2e_dt * 1e3}
    # roofline of the dominant kernel (per-launch algorithmic bytes / its event time)
    kernels = ["camera", "edge", "li", "lins", "primary"]
    kms = {"camera": stage["ms_camera"], "edge": stage["ms_edge"], "li": stage["ms_li"],
           "primary": stage["ms_primary"]}
    dom = max(kms, key=kms.get)
    ki = kernels.index(dom)
    node_b, tri_b, grid_b = 64, 48, 32
    alg_bytes = (node_b * cstats["k_node_visits"][ki] + tri_b * cstats["k_tri_tests"][ki] +
                 grid_b * cstats["k_grid_lookups"][ki])
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg_bytes / (kms[dom] / args.steps / 1e3) / 1e9 if kms[dom] > 0 else 0.0
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tfile):
        traffic = json.load(open(tfile)).get(f"{wl_name}:{dom}")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak if peak else None, "traffic": traffic, "kernel": f"k_{dom}",
                "peak_source": "measured" if peaks else "fallback",
                "bytes_per_step": alg_bytes,
                "bytes_model": "64 B per BVH node visit + 48 B per triangle test + 32 B per trilinear lookup "
                               "(device counters of one instrumented render)"}
    line = {"metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
            "config": {"workload": wl["desc"], "width": spec.width, "height": spec.height, "spp": wl["spp"],
                       "max_bounces": wl["depth"], "nder": wl["nder"], "sppse": wl["sppse"], "sppe": wl["sppe"],
                       "parallelism": f"replicas x{world}", "l2": "flushed between timed steps (256 MiB write)",
                       "accumulation": "f64"},
            "roofline": roofline, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
            "derivative_samples_per_s": value * wl["nder"],
            "stages_ms_per_step": {k: v / args.steps for k, v in stage.items()},
            "counters_per_path": {"rays": cstats["rays"] / paths_per_step,
                                  "node_visits": cstats["node_visits"] / paths_per_step,
                                  "tri_tests": cstats["tri_tests"] / paths_per_step,
                                  "grid_lookups": cstats["grid_lookups"] / paths_per_step,
                                  "edge_records": cstats["edge_records"] / paths_per_step,
                                  "li_tasks": cstats["li_tasks"] / paths_per_step}}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(wl_name, args.cpu_seconds_per_step, args.size)
    scene.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


def cpu_baseline(wl_name, target_s, size=None):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    wl = WORKLOADS[wl_name]
    spec = build_spec(wl_name, size)
    cores = os.cpu_count() or 1
    spp, _ = choose_cpu_spp(oracle_py, spec, wl_name, target_s=target_s, nthreads=cores)
    t0 = time.perf_counter()
    oracle_py.render(spec, **dict(render_kw(wl_name, 7), spp=spp), nthreads=cores)
    dt = time.perf_counter() - t0
    return {"value": spec.width * spec.height * spp / dt, "unit": "paths/s", "cores": cores, "kind": "port",
            "sample": f"full {spec.width}x{spec.height} image at {spp} spp ({dt:.1f} s)", "cpu": cpu_model()}


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
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
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
