"""In-tree build of the native library: host C++ (group model, .oso reader,
lowering, C ABI) with g++ and the sm_103a interpreter with nvcc, linked
into openshadinglanguage_gb300/liboslg_gb300.so.

Translation units compile in parallel; the whole build takes well under a
minute. Nothing here depends on torch.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liboslg_gb300.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HOST_SOURCES = ["oslg_oso.cpp", "oslg_lower.cpp", "oslg_capi.cpp", "oslg_spec.cpp"]
# (source, object name, extra flags): the interpreter is compiled once per
# feature tier (oslg_tier.cu with -DOSLG_TIER=N), in parallel
CUDA_SOURCES = [("oslg_kernels.cu", "oslg_kernels", []), ("oslg_batch_host.cu", "oslg_batch_host", []),
                ("oslg_serve.cu", "oslg_serve", []), ("oslg_wavefront.cu", "oslg_wavefront", [])] + [
    ("oslg_tier.cu", "oslg_tier%d" % t, ["-DOSLG_TIER=%d" % t]) for t in range(8)] + [
    ("oslg_batch.cu", "oslg_batch%d_%d" % (m, q), ["-DOSLG_BATCH_MAXT=%d" % m, "-DOSLG_BATCH_PPT=%d" % q])
    for m in (256, 512) for q in (1, 2, 4)]


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
    return p.stdout + p.stderr


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


LUTS = os.path.join(CSRC, "oslg_bsdl_luts.inc")


def bsdl_luts():
    """Bake the BSDL energy-compensation tables (csrc/gen_bsdl_luts.cpp) into
    csrc/oslg_bsdl_luts.inc unless it is newer than the baker."""
    gen = os.path.join(CSRC, "gen_bsdl_luts.cpp")
    if _newer(LUTS, [gen]):
        return LUTS
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, "gen_bsdl_luts")
    _run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-pthread", gen, "-o", exe])
    _run([exe, LUTS + ".tmp"])
    os.replace(LUTS + ".tmp", LUTS)
    return LUTS


def build(verbose=False, ptxas_verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    bsdl_luts()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh", ".inc"))]
    headers.append(os.path.join(HERE, "..", "include", "oslg.h"))
    jobs, objs = [], []
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if not _newer(o, [s] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-Wall", "-Wno-unused-function",
                         "-I", os.path.join(CUDA_HOME, "include"), "-c", s, "-o", o])
    for src, name, extra in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, name + ".o")
        objs.append(o)
        if not _newer(o, [s] + headers) or ptxas_verbose:
            cmd = [NVCC] + ARCH + ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC"] + extra + [
                "-c", s, "-o", o]
            if ptxas_verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    outs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
            outs = list(ex.map(_run, jobs))
    if verbose or ptxas_verbose:
        for o in outs:
            if o.strip():
                print(o)
    if jobs or not os.path.exists(LIB):
        _run([NVCC] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + objs
             + ["-ldl", "-Xlinker", "-rpath=" + os.path.join(CUDA_HOME, "lib64")])
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_verbose="-v" in sys.argv)
    print(LIB)
