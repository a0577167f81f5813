"""Build libdtrt_gb300.so: nvcc for sm_103a, one translation unit per derivative
width compiled in parallel, linked into dtrt_gb300/_build/. No cmake, no torch."""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libdtrt_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
           "--expt-relaxed-constexpr", "-Xptxas", "-O3"]
UNITS = ["dt_api.cu", "dt_noalloc.cu", "dt_adjoint.cu", "dt_batch.cu", "dt_primal.cu", "dt_vadjoint.cu", "dt_render_n1.cu", "dt_render_n3.cu", "dt_render_n4.cu", "dt_render_n8.cu", "dt_bvh.cpp", "dt_bvh_build.cu"]


def _nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _needs(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [os.path.join(HERE, "..", "include", "dtrt_gb300.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, ptxas_info=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    objs, jobs = [], []
    for u in UNITS:
        src = os.path.join(SRC, u)
        obj = os.path.join(OUT, os.path.splitext(u)[0] + ".o")
        objs.append(obj)
        if force or _needs(obj, src):
            cmd = [nvcc] + ARCH + NVFLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + ["-c", src, "-o", obj]
            if u.endswith(".cpp"):
                cmd = [nvcc, "-x", "cu"] + ARCH + NVFLAGS + ["-c", src, "-o", obj]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or r.returncode != 0 or ptxas_info:
                sys.stderr.write(" ".join(cmd[-3:]) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    if jobs or not os.path.exists(LIB):
        link = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv, force="--force" in sys.argv)
    print(LIB)
