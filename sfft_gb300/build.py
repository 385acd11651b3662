"""Builds sfft_gb300/libsfft.so in place (sm_103a only).

    python -m sfft_gb300.build          # or sfft_gb300.build.build()

Host C++ is compiled by g++ with -ffp-contract=off (plan-time math must not
fuse multiply-adds); CUDA sources by nvcc for sm_103a.  Translation units
compile in parallel; the link is skipped when the library is newer than
every source.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsfft.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["v12.cu", "v3.cu", "noalloc.cu"]
# v3 reproduces the reference's phase arguments (up to ~1e12 rad), whose
# last-ulp rounding matters: no multiply-add contraction in that file.
CU_EXTRA = {"v3.cu": ["--fmad=false"]}
CC_SOURCES = ["api.cc", "host_plan.cc", "serve.cc", "mixed.cc", "tune.cc"]
HEADERS = ["common.cuh", "engine.h", "host_plan.h", "tuned_table.inc"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, ptxas_info=False):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    inc = ["-I" + os.path.join(cuda, "include"), "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "sfft.h")]
    jobs = []
    for s in CU_SOURCES:
        src, obj = os.path.join(CSRC, s), os.path.join(OBJ, s + ".o")
        if _stale(obj, [src] + hdrs):
            cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "--expt-relaxed-constexpr", "-c", src, "-o", obj] + inc + CU_EXTRA.get(s, [])
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for s in CC_SOURCES:
        src, obj = os.path.join(CSRC, s), os.path.join(OBJ, s + ".o")
        if _stale(obj, [src] + hdrs):
            jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-Wall",
                         "-Wno-unused-function", "-c", src, "-o", obj] + inc)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose or ptxas_info:
        for o in outs:
            if o.strip():
                print(o)
    objs = [os.path.join(OBJ, s + ".o") for s in CU_SOURCES + CC_SOURCES]
    if _stale(LIB, objs):
        _run([nvcc, ARCH, "-shared", "-o", LIB] + objs + ["-lpthread", "-lgomp"])
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
