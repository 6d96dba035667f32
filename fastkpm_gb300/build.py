"""Build recipe for libfastkpm_gb300.so (sm_103a only).

Compiles the CUDA translation units (one per precision, compiled in parallel)
with nvcc -gencode arch=compute_103a,code=sm_103a, the host C++ layer with
g++, and links everything into fastkpm_gb300/_build/libfastkpm_gb300.so
(in-tree, git-ignored). Rebuilds only what changed.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libfastkpm_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_UNITS = ["fk_inst_f64.cu", "fk_inst_f32.cu", "fk_inst_f32a.cu", "fk_inst_ds.cu", "fk_engine.cu", "fk_batch.cu",
              "fk_noalloc.cu"]
CXX_UNITS = ["fk_host.cpp"]
HEADERS = ["fk_sys.cuh", "fk_kernels.cuh", "fk_dispatch.h", "fk_inst.cuh", "fk_prep.h", "fk_staged.cuh", "fk_post.cuh",
           "fk_gram.cuh"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fastkpm_gb300")
    return cand


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.exists(d) and os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, h) for h in HEADERS]
    hs += [os.path.join(INCLUDE, "fastkpm_gb300.h"), os.path.join(INCLUDE, "fastkpm.h")]
    return hs


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(force=False, verbose=False, ptxas_verbose=False):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs, objs = [], []
    for u in CUDA_UNITS:
        src = os.path.join(CSRC, u)
        if not os.path.exists(src):
            continue
        obj = os.path.join(OUT, u + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + hdrs):
            cmd = [nvcc] + GENCODE + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                                      "-I" + INCLUDE, "-c", src, "-o", obj]
            if ptxas_verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for u in CXX_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(OUT, u + ".o")
        objs.append(obj)
        if force or _newer(obj, [src] + hdrs):
            cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
            jobs.append([os.environ.get("CXX", "g++"), "-O3", "-std=c++17", "-fPIC", "-I" + INCLUDE,
                         "-I" + cuda_inc, "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, log in zip(jobs, ex.map(_compile, jobs)):
                if verbose or ptxas_verbose:
                    print(" ".join(cmd))
                    if log:
                        print(log)
    if force or jobs or _newer(LIB, objs):
        tmp = LIB + ".tmp"
        _compile([nvcc] + GENCODE + ["-shared", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, ptxas_verbose="--ptxas" in sys.argv))
