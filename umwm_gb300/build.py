"""Build the GB300 UMWM library in-tree: umwm_gb300/_lib/libumwm_gb300.so.

Device code is compiled for sm_103a only.  Translation units compile in
parallel; the host set-up is compiled without FMA contraction so that its
fp32 tables are reproducible on x86-64 and aarch64 hosts alike.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libumwm_gb300.so")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["k_source.cu", "k_advect.cu", "k_misc.cu", "k_persist.cu", "umwm_gpu.cu", "k_mlp.cu", "k_sur.cu",
              "surrogate.cu"]
CXX_SOURCES = ["host_model.cpp", "ncfile.cpp"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-ftz=true", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, extra_nvcc=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    # extra nvcc definitions for tuning experiments (e.g. "-DUMWM_INTEG_MINB=4");
    # a change of flags rebuilds everything
    extra_nvcc = list(extra_nvcc) + os.environ.get("UMWM_NVCC_DEFS", "").split()
    stamp = os.path.join(BUILD_DIR, "flags.txt")
    flags = " ".join(NVCC_FLAGS + extra_nvcc)
    if not os.path.exists(stamp) or open(stamp).read() != flags:
        for f in os.listdir(BUILD_DIR):
            if f.endswith(".o"):
                os.remove(os.path.join(BUILD_DIR, f))
        with open(stamp, "w") as fh:
            fh.write(flags)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "umwm_gpu.h"))
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append([NVCC] + NVCC_FLAGS + list(extra_nvcc) + ["-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", s, "-o", o])
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
            logs = list(ex.map(_run, jobs))
    if jobs or _stale(LIB, objs):
        logs.append(_run([NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs + ["-lpthread"]))
    if verbose:
        for l in logs:
            if l.strip():
                sys.stdout.write(l)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
