#!/usr/bin/env python3
"""Build oracle/_ref/libref_emul.so: the reference's own code, run on a CPU.

TEST INFRASTRUCTURE ONLY.  The reference (paogor/CUDA-SIPG-matrix-free) is
header-only CUDA C++.  Its kernels use no shared memory, barriers or atomics,
so calling each kernel once per (block, thread) on one CPU thread reproduces
what the GPU computes.  This recipe:

1. reads the reference headers from the reference checkout (default
   /root/reference, or $SIPG_REFERENCE_DIR) -- they are never copied into the
   repository;
2. rewrites each ``kernel<<<grid, block>>>(args)`` launch into
   ``::emu::launch([&](auto&&... a) { kernel(a...); }, grid, block)(args)``
   (the only change; written to a temporary directory under oracle/_ref/
   that is deleted after the compile);
3. compiles oracle/ref_emul.cpp with oracle/cuda_emul.h against them with
   g++ -O2 -ffp-contract=off into oracle/_ref/libref_emul.so, and again with
   -DUSE_PRECONDITIONER (the block-Jacobi path; LAPACK, absent here, replaced
   by oracle/lapacke_emul/lapacke.h) into oracle/_ref/libref_emul_pcg.so;
4. compiles the reference's FP64 kernels, unchanged, for sm_103a into
   oracle/_ref/ref_kernels.cubin (oracle/ref_gpu_kernels.cu holds only their
   explicit instantiations).  The cubin is device code and travels with the
   repository to the GPU machine, where oracle/ref_gpu.cpp runs it as the
   "reference kernels on the same GPU" baseline.

The outputs are test infrastructure: libref_emul.so generates and checks the
golden fixtures under tests/golden/; nothing in the product links either.
Exit status 0 on success, 2 if the reference checkout is absent (skipped).
"""
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
OUT_LIB = os.path.join(OUT_DIR, "libref_emul.so")

LAUNCH = re.compile(r"([A-Za-z_]\w*(?:\s*<[^<>;(){}]*>)?)\s*<<<(.*?)>>>", re.S)


def rewrite(text):
    def sub(m):
        return "::emu::launch([&](auto&&... emu_a) { %s(emu_a...); }, %s)" % (m.group(1), m.group(2))

    return LAUNCH.sub(sub, text)


def build(ref_dir=None, verbose=False):
    ref_dir = ref_dir or os.environ.get("SIPG_REFERENCE_DIR", "/root/reference")
    inc = os.path.join(ref_dir, "include")
    if not os.path.isdir(inc):
        if verbose:
            print("reference checkout not found at %s: skipping oracle/_ref" % ref_dir)
        return 2
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = os.path.join(OUT_DIR, "tmp_headers")
    shutil.rmtree(tmp, ignore_errors=True)
    try:
        for sub in ("include", "performance_tests", "validation_tests"):
            src = os.path.join(ref_dir, sub)
            dst = os.path.join(tmp, sub)
            os.makedirs(dst, exist_ok=True)
            for name in os.listdir(src):
                if name.endswith(".hpp") or (sub == "include" and name.endswith(".cpp")):
                    with open(os.path.join(src, name)) as f:
                        text = f.read()
                    with open(os.path.join(dst, name), "w") as f:
                        f.write(rewrite(text))
        cmd = [
            "g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w",
            "-I", HERE, "-I", os.path.join(tmp, "include"), "-I", os.path.join(tmp, "validation_tests"),
            os.path.join(HERE, "ref_emul.cpp"), "-o", OUT_LIB,
        ]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        # the same with the block-Jacobi preconditioner (USE_PRECONDITIONER),
        # LAPACK replaced by oracle/lapacke_emul/lapacke.h
        cmd_pcg = cmd[:-2] + ["-DUSE_PRECONDITIONER", "-I", os.path.join(HERE, "lapacke_emul"), "-o",
                              os.path.join(OUT_DIR, "libref_emul_pcg.so")]
        if verbose:
            print(" ".join(cmd_pcg))
        subprocess.check_call(cmd_pcg)
        cubin = os.path.join(OUT_DIR, "ref_kernels.cubin")
        cmd = [os.environ.get("NVCC", "nvcc"), "-std=c++14", "-O3", "-cubin", "-gencode",
               "arch=compute_103a,code=sm_103a", "-w", "-I", inc, os.path.join(HERE, "ref_gpu_kernels.cu"),
               "-o", cubin + ".tmp"]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        os.replace(cubin + ".tmp", cubin)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return 0


if __name__ == "__main__":
    sys.exit(build(sys.argv[1] if len(sys.argv) > 1 else None, verbose=True))
