#!/usr/bin/env python3
"""Generate tests/golden/reference_golden.npz from the reference's own code.

Runs oracle/_ref/libref_emul.so -- paogor/CUDA-SIPG-matrix-free's headers
(LGL_quadrature_table, sem_function, volume, flux_term6a/6b, volume_mvm,
sipg_sem_2d, conjugate_gradient) compiled for a CPU by oracle/build_ref.py --
on small seeded inputs and stores inputs and outputs; and
oracle/_ref/libref_emul_pcg.so, the same built with USE_PRECONDITIONER, for
the block-Jacobi preconditioner and the preconditioned CG.  Run it where the
reference checkout exists:

    python3 oracle/build_ref.py && python3 tests/golden/make_golden.py

The fixture is what the CPU tests check the oracle against, bit for bit, and
what the GPU tests check the CUDA path against, to tolerance, on machines where
the reference is absent.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(ROOT, "oracle", "_ref", "libref_emul.so")
LIB_PCG = os.path.join(ROOT, "oracle", "_ref", "libref_emul_pcg.so")
OUT = os.path.join(HERE, "reference_golden.npz")

dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
fp = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")


def load():
    ref = C.CDLL(LIB)
    ref.ref_lgl.argtypes = [C.c_int, dp, dp]
    ref.ref_lgl_f32.argtypes = [C.c_int, fp, fp]
    ref.ref_dphi.argtypes = [C.c_int, dp]
    ref.ref_laplace2d.argtypes = [C.c_int, dp]
    ref.ref_mesh_coords.argtypes = [C.c_int, dp, dp]
    ref.ref_apply.argtypes = [C.c_int, C.c_int, C.c_double, dp, dp]
    ref.ref_apply_f32.argtypes = [C.c_int, C.c_int, C.c_float, fp, fp]
    ref.ref_volume_mvm.argtypes = [C.c_int, C.c_int, dp, dp]
    ref.ref_solve.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, dp, dp]
    ref.ref_rhs.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, dp]
    return ref


def load_pcg():
    ref = C.CDLL(LIB_PCG)
    ref.ref_prec_block.argtypes = [C.c_int, C.c_double, dp, dp]
    ref.ref_prec_rows.argtypes = [C.c_int, C.c_double, dp]
    ref.ref_solve.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, dp, dp]
    ref.ref_rhs.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, dp]
    return ref


# (p, dim) cases for the matvec: every supported degree on tiny meshes (1x1 is
# all boundary; 2x2 has every face kind), plus odd, non-tile-multiple sizes.
APPLY_CASES = [(p, d) for p in range(1, 9) for d in (1, 2, 3, 5)] + [(4, 16), (4, 33), (8, 12), (6, 7)]
# full solves through the reference driver: (solution, p, dim, pen, absolute tol)
SOLVE_CASES = [
    (5, 2, 4, 4.0, 1e-12), (5, 4, 4, 16.0, 1e-12), (5, 3, 8, 9.0, 1e-12), (1, 2, 4, 4.0, 1e-13),
    (2, 3, 4, 9.0, 1e-12), (3, 2, 2, 4.0, 1e-13), (4, 1, 3, 1.0, 1e-13), (5, 2, 8, 400.0, 1e-15),
]


# the block-Jacobi preconditioner: every degree, the drivers' penalties (p^2,
# 100 p^2) and one that the reference's int parameter truncates (37.9 -> 37)
PREC_PENS = lambda p: (float(p * p), 100.0 * p * p, 37.9)
# preconditioned solves (USE_PRECONDITIONER): (solution, p, dim, pen, absolute tol)
PCG_CASES = [
    (5, 2, 4, 400.0, 1e-15), (5, 3, 8, 900.0, 1e-15), (6, 4, 16, 16.0, 1e-12), (5, 4, 8, 1600.0, 1e-14),
    (1, 6, 6, 36.0, 1e-13),
]


def main():
    if not os.path.exists(LIB):
        print("missing %s: run oracle/build_ref.py first" % LIB)
        return 2
    ref = load()
    g = {}
    for n in range(2, 34):
        a, b = np.zeros(n), np.zeros(n)
        ref.ref_lgl(n, a, b)
        g["lgl_nodes_%d" % n], g["lgl_weights_%d" % n] = a, b
        af, bf = np.zeros(n, np.float32), np.zeros(n, np.float32)
        ref.ref_lgl_f32(n, af, bf)
        g["lgl_nodes_f32_%d" % n], g["lgl_weights_f32_%d" % n] = af, bf
    for p in range(1, 17):
        n = p + 1
        D = np.zeros(n * n)
        ref.ref_dphi(p, D)
        g["dphi_%d" % p] = D
    for p in range(1, 9):
        L = np.zeros((p + 1) ** 4)
        ref.ref_laplace2d(p, L)
        g["laplace2d_%d" % p] = L
    for d in (1, 2, 3, 16):
        x, y = np.zeros(4 * d * d), np.zeros(4 * d * d)
        ref.ref_mesh_coords(d, x, y)
        g["mesh_x_%d" % d], g["mesh_y_%d" % d] = x, y
    for (p, d) in APPLY_CASES:
        rng = np.random.default_rng(1000 * p + d)
        n = d * d * (p + 1) ** 2
        x = rng.uniform(-1.0, 1.0, n)
        g["apply_in_%d_%d" % (p, d)] = x
        pens = (("ref", float(p * p)), ("thesis", 100.0 * p * p)) if d <= 5 else (("ref", float(p * p)),)
        for pen_name, pen in pens:
            y = np.zeros(n)
            ref.ref_apply(p, d, pen, x, y)
            g["apply_out_%s_%d_%d" % (pen_name, p, d)] = y
        if d <= 5:
            xf = x.astype(np.float32)
            yf = np.zeros(n, np.float32)
            ref.ref_apply_f32(p, d, np.float32(p * p), xf, yf)
            g["apply_out_f32_%d_%d" % (p, d)] = yf
        if d <= 3:
            yv = np.zeros(n)
            ref.ref_volume_mvm(p, d, x, yv)
            g["volume_mvm_out_%d_%d" % (p, d)] = yv
    solves = []
    for i, (sol, p, d, pen, tol) in enumerate(SOLVE_CASES):
        n = d * d * (p + 1) ** 2
        u, st = np.zeros(n), np.zeros(4)
        ref.ref_solve(p, d, pen, tol, sol, u, st)
        b = np.zeros(n)
        ref.ref_rhs(p, d, pen, sol, b)
        g["solve_u_%d" % i], g["solve_rhs_%d" % i] = u, b
        solves.append([sol, p, d, pen, tol] + list(st))
    g["solve_table"] = np.array(solves)
    # the 16x16, p=4 sin-sin Poisson case: pen = p^2 (the reference drivers'
    # choice), CG to ||r|| <= 1e-12 ||b|| (absolute tolerance handed to the
    # reference's absolute-stop CG)
    p, d, pen = 4, 16, 16.0
    n = d * d * (p + 1) ** 2
    b = np.zeros(n)
    ref.ref_rhs(p, d, pen, 6, b)
    tol = 1e-12 * float(np.sqrt(np.dot(b, b)))
    u, st = np.zeros(n), np.zeros(4)
    ref.ref_solve(p, d, pen, tol, 6, u, st)
    g["poisson16_rhs"], g["poisson16_u"] = b, u
    g["poisson16_stats"] = np.array([p, d, pen, tol] + list(st))
    pref = load_pcg()
    for p in range(1, 9):
        nn = (p + 1) ** 2
        for k, pen in enumerate(PREC_PENS(p)):
            rows = np.zeros(nn * (2 * p + 1))
            pref.ref_prec_rows(p, pen, rows)
            g["prec_rows_%d_%d" % (p, k)] = rows
            if k == 0 and p in (3, 8):
                blk, inv = np.zeros(nn * nn), np.zeros(nn * nn)
                pref.ref_prec_block(p, pen, blk, inv)
                g["prec_block_%d" % p], g["prec_inverse_%d" % p] = blk, inv
    pcg = []
    for i, (sol, p, d, pen, tol) in enumerate(PCG_CASES):
        n = d * d * (p + 1) ** 2
        u, st = np.zeros(n), np.zeros(4)
        pref.ref_solve(p, d, pen, tol, sol, u, st)
        b = np.zeros(n)
        pref.ref_rhs(p, d, pen, sol, b)
        g["pcg_u_%d" % i], g["pcg_rhs_%d" % i] = u, b
        pcg.append([sol, p, d, pen, tol] + list(st))
    g["pcg_table"] = np.array(pcg)
    np.savez_compressed(OUT, **g)
    print("wrote %s (%d arrays, %.1f KB)" % (OUT, len(g), os.path.getsize(OUT) / 1024))
    return 0


if __name__ == "__main__":
    sys.exit(main())
