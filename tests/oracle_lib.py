"""ctypes binding of oracle/liboracle.so -- the CPU checker (tests only)."""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB = os.path.join(ORACLE_DIR, "liboracle.so")

dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
fp = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")


class OrModes(C.Structure):
    _fields_ = [("nmodes", C.c_int), ("amp", C.c_double * 8), ("k", C.c_int * 8), ("l", C.c_int * 8)]


class Oracle:
    def __init__(self, L):
        self.L = L
        L.sipg_oracle_lgl.argtypes = [C.c_int, dp, dp]
        L.sipg_oracle_dphi.argtypes = [C.c_int, dp]
        L.sipg_oracle_laplace2d.argtypes = [C.c_int, dp]
        L.sipg_oracle_mesh_coords.argtypes = [C.c_int, dp, dp]
        L.sipg_oracle_apply.argtypes = [C.c_int, C.c_int, C.c_double, dp, dp, C.c_int]
        L.sipg_oracle_apply_f32.argtypes = [C.c_int, C.c_int, C.c_float, fp, fp, C.c_int]
        L.sipg_oracle_volume.argtypes = [C.c_int, C.c_int, dp, dp]
        L.sipg_oracle_cg.argtypes = [C.c_int, C.c_int, C.c_double, dp, dp, C.c_double, C.c_int, C.c_int,
                                     C.POINTER(C.c_double), C.c_int]
        L.sipg_oracle_rhs.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p, dp]
        L.sipg_oracle_err_norms.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, dp, dp]
        L.sipg_oracle_u_exact.argtypes = [C.c_int, C.c_void_p, C.c_double, C.c_double]
        L.sipg_oracle_u_exact.restype = C.c_double
        L.sipg_oracle_prec_block.argtypes = [C.c_int, C.c_double, dp]
        L.sipg_oracle_invert.argtypes = [C.c_int, dp]
        L.sipg_oracle_prec_rows.argtypes = [C.c_int, C.c_double, dp]
        L.sipg_oracle_prec_apply.argtypes = [C.c_int, C.c_int, dp, dp, dp]
        L.sipg_oracle_pcg.argtypes = [C.c_int, C.c_int, C.c_double, dp, dp, C.c_double, C.c_int, C.c_int,
                                      C.POINTER(C.c_double), C.c_int]
        self.nthreads = max(1, min(16, os.cpu_count() or 1))

    def lgl(self, n):
        x, w = np.zeros(n), np.zeros(n)
        assert self.L.sipg_oracle_lgl(n, x, w) == 0
        return x, w

    def dphi(self, p):
        D = np.zeros((p + 1) ** 2)
        assert self.L.sipg_oracle_dphi(p, D) == 0
        return D

    def laplace2d(self, p):
        Lm = np.zeros((p + 1) ** 4)
        assert self.L.sipg_oracle_laplace2d(p, Lm) == 0
        return Lm

    def mesh_coords(self, dim):
        x, y = np.zeros(4 * dim * dim), np.zeros(4 * dim * dim)
        assert self.L.sipg_oracle_mesh_coords(dim, x, y) == 0
        return x, y

    def apply(self, p, dim, pen, x, nthreads=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        assert self.L.sipg_oracle_apply(p, dim, pen, x, y, nthreads or self.nthreads) == 0
        return y

    def apply_f32(self, p, dim, pen, x, nthreads=None):
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.zeros_like(x)
        assert self.L.sipg_oracle_apply_f32(p, dim, pen, x, y, nthreads or self.nthreads) == 0
        return y

    def volume(self, p, dim, x):
        y = np.zeros_like(x)
        assert self.L.sipg_oracle_volume(p, dim, np.ascontiguousarray(x), y) == 0
        return y

    def cg(self, p, dim, pen, b, tol, rel=False, max_it=0, x0=None, nthreads=1):
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        rr = C.c_double()
        it = self.L.sipg_oracle_cg(p, dim, pen, x, np.ascontiguousarray(b), tol, int(rel), max_it, C.byref(rr),
                                   nthreads)
        return it, x, rr.value

    def prec_block(self, p, pen):
        nn = (p + 1) ** 2
        a = np.zeros(nn * nn)
        assert self.L.sipg_oracle_prec_block(p, pen, a) == 0
        return a

    def invert(self, a):
        n = int(round(np.sqrt(a.size)))
        b = np.array(a, dtype=np.float64)
        assert self.L.sipg_oracle_invert(n, b) == 0
        return b

    def prec_rows(self, p, pen):
        rows = np.zeros((p + 1) ** 2 * (2 * p + 1))
        assert self.L.sipg_oracle_prec_rows(p, pen, rows) == 0
        return rows

    def prec_apply(self, p, dim, rows, x):
        y = np.zeros_like(x)
        assert self.L.sipg_oracle_prec_apply(p, dim, np.ascontiguousarray(rows), np.ascontiguousarray(x), y) == 0
        return y

    def pcg(self, p, dim, pen, b, tol, rel=False, max_it=0, x0=None, nthreads=1):
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        rr = C.c_double()
        it = self.L.sipg_oracle_pcg(p, dim, pen, x, np.ascontiguousarray(b), tol, int(rel), max_it, C.byref(rr),
                                    nthreads)
        assert it >= 0
        return it, x, rr.value

    @staticmethod
    def modes(amps, ks, ls):
        m = OrModes()
        m.nmodes = len(amps)
        for i, (a, k, l) in enumerate(zip(amps, ks, ls)):
            m.amp[i], m.k[i], m.l[i] = a, k, l
        return m

    def rhs(self, p, dim, pen, sol, modes=None):
        b = np.zeros(dim * dim * (p + 1) ** 2)
        assert self.L.sipg_oracle_rhs(p, dim, pen, sol, C.byref(modes) if modes else None, b) == 0
        return b

    def err_norms(self, p, dim, sol, u, modes=None):
        e = np.zeros(3)
        assert self.L.sipg_oracle_err_norms(p, dim, sol, C.byref(modes) if modes else None,
                                            np.ascontiguousarray(u), e) == 0
        return e


_cached = None


def load():
    """Build (if needed) and load the oracle library."""
    global _cached
    if _cached is None:
        src = [os.path.join(ORACLE_DIR, f) for f in ("sipg_oracle.c", "sipg_oracle_real.inc", "sipg_oracle.h")]
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(s) for s in src):
            subprocess.check_call(["make", "-s", "-C", ORACLE_DIR, "liboracle.so"])
        _cached = Oracle(C.CDLL(LIB))
    return _cached


REF_GPU_LIB = os.path.join(ORACLE_DIR, "_ref", "libref_gpu.so")
REF_CUBIN = os.path.join(ORACLE_DIR, "_ref", "ref_kernels.cubin")


class RefGpu:
    """The reference's own CUDA kernels (oracle/ref_gpu.cpp over the cubin built
    from the reference headers): same-GPU parity and baseline timing."""

    def __init__(self):
        L = C.CDLL(REF_GPU_LIB)
        L.refgpu_init.argtypes = [C.c_char_p]
        L.refgpu_apply.argtypes = [C.c_int, C.c_int, C.c_double, C.c_void_p, C.c_void_p, C.c_int,
                                   C.POINTER(C.c_float)]
        L.refgpu_cg.argtypes = [C.c_int, C.c_int, C.c_double, C.c_void_p, C.c_void_p, C.c_double,
                                C.POINTER(C.c_int), C.POINTER(C.c_float)]
        L.refgpu_last_error.restype = C.c_char_p
        self.L = L
        rc = L.refgpu_init(REF_CUBIN.encode())
        if rc:
            raise RuntimeError("refgpu_init: " + L.refgpu_last_error().decode())

    def apply(self, p, dim, pen, d_in, d_out, reps=1):
        ms = C.c_float()
        rc = self.L.refgpu_apply(p, dim, pen, C.c_void_p(d_in), C.c_void_p(d_out), reps, C.byref(ms))
        if rc:
            raise RuntimeError("refgpu_apply: " + self.L.refgpu_last_error().decode())
        return ms.value

    def cg(self, p, dim, pen, d_x, d_b, tol):
        it, ms = C.c_int(), C.c_float()
        rc = self.L.refgpu_cg(p, dim, pen, C.c_void_p(d_x), C.c_void_p(d_b), tol, C.byref(it), C.byref(ms))
        if rc:
            raise RuntimeError("refgpu_cg: " + self.L.refgpu_last_error().decode())
        return it.value, ms.value


def ref_gpu_available():
    return os.path.exists(REF_GPU_LIB) and os.path.exists(REF_CUBIN)


_ref_gpu = None


def ref_gpu():
    global _ref_gpu
    if _ref_gpu is None:
        _ref_gpu = RefGpu()
    return _ref_gpu
