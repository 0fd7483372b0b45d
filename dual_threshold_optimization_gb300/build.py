"""Build libdto.so in-tree: nvcc for sm_103a, translation units compiled in parallel.

The library is written to ``dual_threshold_optimization_gb300/libdto.so`` (git-ignored)
and loaded from there by ``dual_threshold_optimization_gb300._lib``.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libdto.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libdto.so")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return sorted(hs + [os.path.join(INCLUDE, "dto.h")])


def _digest(paths, extra):
    h = hashlib.sha256()
    for p in paths:
        h.update(p.encode())
        with open(p, "rb") as fh:
            h.update(fh.read())
    h.update(" ".join(extra).encode())
    return h.hexdigest()


def _compile(nvcc, src, obj, flags):
    cmd = [nvcc] + flags + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stderr


def build(force=False, verbose=False, jobs=None):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                    "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fvisibility=hidden",
                    "-I", INCLUDE, "-I", CSRC]
    if verbose:
        flags += ["-Xptxas", "-v"]
    srcs = _sources()
    key = _digest(srcs + _headers(), flags)
    stamp = os.path.join(BUILD, "stamp")
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == key:
                return LIB
    objs = [os.path.join(BUILD, os.path.basename(s) + ".o") for s in srcs]
    jobs = jobs or min(len(srcs), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        logs = list(ex.map(lambda so: _compile(nvcc, so[0], so[1], flags), zip(srcs, objs)))
    if verbose:
        for s, lg in zip(srcs, logs):
            sys.stderr.write("== %s\n%s" % (os.path.basename(s), lg))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(key)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
