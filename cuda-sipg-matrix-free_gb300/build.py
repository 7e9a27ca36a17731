#!/usr/bin/env python3
"""Build the GB300 SIPG-SEM library: lib/libsipg_gb300.so (sm_103a only).

Every .cu/.cpp under csrc/ is compiled by nvcc in parallel (one -gencode,
compute_103a -> sm_103a, -lineinfo) and linked into one shared library with
the shared CUDA runtime.  Objects go to _build/ (git-ignored); the library is
rebuilt only when a source or header is newer than it.
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib", "libsipg_gb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))


def _mtime(p):
    return os.path.getmtime(p) if os.path.exists(p) else -1.0


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    newest_dep = max([_mtime(src)] + [_mtime(h) for h in headers()])
    if _mtime(obj) >= newest_dep:
        return obj, None
    cmd = [NVCC] + ARCH + FLAGS + extra + ["-c", src, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, "%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr)
    os.replace(obj + ".tmp", obj)
    return obj, None


def build(verbose=False, jobs=None, extra=None):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    objs, errors = [], []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for obj, err in ex.map(lambda s: _compile(s, extra or []), srcs):
            objs.append(obj)
            if err:
                errors.append(err)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    if _mtime(LIB) < max(_mtime(o) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB + ".tmp"] + objs
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
