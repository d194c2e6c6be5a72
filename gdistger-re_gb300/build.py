"""Builds libsgns.so (the CUDA kernels + C ABI) and the sgns_train CLI for sm_103a.

Each translation unit compiles in its own process (in parallel), then nvcc links the
shared library.  Outputs go to gdistger-re_gb300/build/.  Usage:
    python gdistger-re_gb300/build.py [--verbose-ptxas]
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "build")
ROOT = os.path.dirname(HERE)
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["dsgl_window.cu", "dsgl_plain.cu", "dsgl_aux.cu", "dsgl_adjoint.cu", "dsgl_noalloc.cu",
              "dsgl_ingest.cu", "dsgl_eval.cu", "dsgl_walk.cu"]
CPP_SOURCES = ["sgns_host.cpp"]
LIB = os.path.join(OUT, "libsgns.so")
CLI = os.path.join(OUT, "sgns_train")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose_ptxas=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "sgns.h"))
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                   "-I", os.path.join(ROOT, "include"), "-c", s, "-o", o]
            if verbose_ptxas:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            # -ffp-contract=off: host float expressions (vocabulary tables, the walker's
            # entropy table) evaluate as written, with no fused multiply-add, on every host
            jobs.append([NVCC, "-O2", "-std=c++17", "-Xcompiler", "-fPIC,-Wall,-ffp-contract=off",
                         "-I", os.path.join(ROOT, "include"),
                         "-c", s, "-o", o])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    if force or jobs or not os.path.exists(LIB):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    cli_src = os.path.join(CSRC, "sgns_train_main.cpp")
    if os.path.exists(cli_src) and (force or _stale(CLI, [cli_src, LIB] + headers)):
        _run(["g++", "-O2", "-std=c++17", cli_src, "-I", os.path.join(ROOT, "include"), "-o", CLI,
              "-L", OUT, "-lsgns", "-Wl,-rpath,$ORIGIN"])
    return "\n".join(l for l in logs if l.strip())


if __name__ == "__main__":
    print(build(verbose_ptxas="--verbose-ptxas" in sys.argv, force="--force" in sys.argv))
    print("built", LIB)
