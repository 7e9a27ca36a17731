"""Python binding of the GB300 SIPG-SEM library (libsipg_gb300.so) via ctypes.

The C ABI in include/sipg_gb300.h is the product boundary; this module only
marshals torch tensors (device memory and streams) and numpy arrays onto it.
There is no fallback: if the CUDA library is missing or the device is not
sm_103a, every call raises SipgError.

Vectors are node-major: entry (i1, i2) of element e at ((i1*(p+1)+i2)*noe + e),
the layout of the reference's mode_vector (mode_vector.hpp:108-120).
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libsipg_gb300.so")

SIPG_OK = 0
STATUS_NAMES = {
    0: "SIPG_OK", 1: "SIPG_ERR_INVALID", 2: "SIPG_ERR_CUDA", 3: "SIPG_ERR_NOT_CONVERGED",
    4: "SIPG_ERR_BREAKDOWN", 5: "SIPG_ERR_UNSUPPORTED", 6: "SIPG_ERR_NOMEM", 7: "SIPG_ERR_REJECTED",
    8: "SIPG_ERR_TIMEOUT",
}
SOL = {"A": 1, "B": 2, "C": 3, "D": 4, "E": 5, "sinsin": 6, "modes": 7}
MAX_DEGREE = 8


class SipgError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), msg))


class CgResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("rr", C.c_double), ("stop", C.c_double), ("time_ms", C.c_double),
                ("converged", C.c_int)]


class MixedOpts(C.Structure):
    _fields_ = [("inner_tol", C.c_double), ("outer_tol", C.c_double), ("max_outer", C.c_int), ("max_inner", C.c_int),
                ("inner", C.c_int), ("outer", C.c_int)]


INNER = {"auto": 0, "f32": 1, "pairs": 2, "f64": 3, "twolevel": 4}
OUTER = {"auto": 0, "reliable": 1, "flexible": 2}


class MixedResult(C.Structure):
    _fields_ = [("outer_iterations", C.c_int), ("inner_iterations", C.c_int), ("rel_residual", C.c_double),
                ("time_ms", C.c_double), ("converged", C.c_int), ("inner_kind", C.c_int), ("outer_kind", C.c_int),
                ("fp64_applies", C.c_int)]


class Problem(C.Structure):
    _fields_ = [("dim", C.c_int), ("degree", C.c_int), ("pen", C.c_double)]


class ServerOpts(C.Structure):
    _fields_ = [("budget_bytes", C.c_size_t), ("max_active", C.c_int), ("iters_per_step", C.c_int),
                ("inner_tol", C.c_double)]


class RequestResult(C.Structure):
    _fields_ = [("done", C.c_int), ("status", C.c_int), ("iterations", C.c_int), ("corrections", C.c_int),
                ("rel_residual", C.c_double), ("queue_ms", C.c_double), ("latency_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("queued", C.c_int), ("active", C.c_int), ("completed", C.c_ulonglong), ("rejected", C.c_ulonglong),
                ("bytes_in_use", C.c_size_t), ("setup_ms", C.c_double), ("prep_ms", C.c_double)]


class Modes(C.Structure):
    _fields_ = [("nmodes", C.c_int), ("amp", C.c_double * 8), ("k", C.c_int * 8), ("l", C.c_int * 8)]

    @staticmethod
    def make(amps, ks, ls):
        m = Modes()
        m.nmodes = len(amps)
        for i, (a, k, l) in enumerate(zip(amps, ks, ls)):
            m.amp[i], m.k[i], m.l[i] = float(a), int(k), int(l)
        return m


class TileChoice(C.Structure):
    _fields_ = [("elements_per_row", C.c_int * 3), ("rows", C.c_int * 3), ("threads_per_element", C.c_int * 3),
                ("ms_per_apply", C.c_float * 3)]


TILE_KINDS = {"f64": 0, "f32": 1, "pairs": 2}

_lib = None

_VP = C.c_void_p
_SIGS = {
    "sipg_lgl_table": (C.c_int, [C.c_int, _VP, _VP]),
    "sipg_dphi_table": (C.c_int, [C.c_int, _VP]),
    "sipg_laplacian_rows_f64": (C.c_int, [C.c_int, _VP]),
    "sipg_selftest_barrier_timeout": (C.c_int, [C.POINTER(C.c_int)]),
    "sipg_square_mesh_coords": (C.c_int, [C.c_int, _VP, _VP]),
    "sipg_op_create": (C.c_int, [C.c_int, C.c_int, C.c_double, C.POINTER(_VP)]),
    "sipg_op_destroy": (C.c_int, [_VP]),
    "sipg_op_solve_footprint": (C.c_size_t, [C.c_int, C.c_int, C.c_int]),
    "sipg_op_autotune": (C.c_int, [_VP, _VP, C.POINTER(TileChoice)]),
    "sipg_op_set_tile": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_int]),
    "sipg_op_get_tile": (C.c_int, [_VP, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "sipg_apply_f64": (C.c_int, [_VP, _VP, _VP, _VP]),
    "sipg_apply_f32": (C.c_int, [_VP, _VP, _VP, _VP]),
    "sipg_apply_pairs": (C.c_int, [_VP, _VP, _VP, _VP]),
    "sipg_apply_host_f64": (C.c_int, [_VP, _VP, _VP, _VP]),
    "sipg_cg_f64": (C.c_int, [_VP, _VP, _VP, C.c_double, C.c_int, C.c_int, C.POINTER(CgResult), _VP]),
    "sipg_cg_f32": (C.c_int, [_VP, _VP, _VP, C.c_float, C.c_int, C.c_int, C.POINTER(CgResult), _VP]),
    "sipg_pcg_f64": (C.c_int, [_VP, _VP, _VP, C.c_double, C.c_int, C.c_int, C.POINTER(CgResult), _VP]),
    "sipg_apply_prec_f64": (C.c_int, [_VP, _VP, _VP, _VP]),
    "sipg_volume_mvm_f64": (C.c_int, [C.c_int, C.c_int, _VP, C.c_int, _VP, _VP, _VP]),
    "sipg_solve_mixed": (C.c_int, [_VP, _VP, _VP, C.POINTER(MixedOpts), C.POINTER(MixedResult), _VP]),
    "sipg_apply_twolevel_f32": (C.c_int, [_VP, _VP, _VP, _VP]),
    "sipg_residual_f64": (C.c_int, [_VP, _VP, _VP, _VP, C.POINTER(C.c_double), _VP]),
    "sipg_rhs_f64": (C.c_int, [_VP, C.c_int, C.POINTER(Modes), _VP, _VP]),
    "sipg_err_norms_f64": (C.c_int, [_VP, C.c_int, C.POINTER(Modes), _VP, _VP, _VP]),
    "sipg_last_error": (C.c_char_p, []),
    "sipg_version": (C.c_char_p, []),
    "sipg_launch_count": (C.c_ulonglong, []),
    "sipg_probe_fma_peak": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "sipg_batch_create": (C.c_int, [C.c_int, _VP, C.POINTER(_VP)]),
    "sipg_batch_destroy": (C.c_int, [_VP]),
    "sipg_batch_op": (C.c_int, [_VP, C.c_int, C.POINTER(_VP)]),
    "sipg_batch_footprint": (C.c_size_t, [_VP]),
    "sipg_batch_solve_mixed": (C.c_int, [_VP, _VP, _VP, C.POINTER(MixedOpts), _VP, _VP]),
    "sipg_server_create": (C.c_int, [_VP, C.POINTER(_VP)]),
    "sipg_server_destroy": (C.c_int, [_VP]),
    "sipg_server_submit": (C.c_int, [_VP, _VP, C.POINTER(C.c_ulonglong)]),
    "sipg_server_step": (C.c_int, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "sipg_server_poll": (C.c_int, [_VP, C.c_ulonglong, C.POINTER(RequestResult)]),
    "sipg_server_release": (C.c_int, [_VP, C.c_ulonglong]),
    "sipg_server_solution": (C.c_int, [_VP, C.c_ulonglong, _VP, C.c_size_t]),
    "sipg_server_stats": (C.c_int, [_VP, C.POINTER(ServerStats)]),
    "sipg_dot_f64": (C.c_int, [C.c_size_t, _VP, _VP, C.POINTER(C.c_double), _VP]),
    "sipg_dot_f64_noalloc": (C.c_int, [C.c_size_t, _VP, _VP, C.POINTER(C.c_double), _VP]),
}


def lib():
    """Load libsipg_gb300.so (raises SipgError if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SipgError(5, "CUDA library not built: %s (run __graft_entry__.build())" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(status, what=""):
    if status != SIPG_OK:
        raise SipgError(status, "%s %s" % (what, lib().sipg_last_error().decode()))


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _stream(stream=None):
    if stream is not None:
        return C.c_void_p(stream)
    import torch

    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def selftest_barrier_timeout():
    """True when the persistent CG's grid barrier gives up on a wait that
    cannot complete (the abort path) and the device stays usable."""
    g = C.c_int(0)
    _check(lib().sipg_selftest_barrier_timeout(C.byref(g)), "selftest_barrier_timeout")
    return bool(g.value)


def laplacian_rows(degree):
    """The element Laplacian's stored rows (numpy, (p+1)^2 * (2p+1) values):
    the mode_matrix of the reference's host_laplacian_matrix(1, p), for
    volume_mvm."""
    n, R = degree + 1, 2 * degree + 1
    rows = np.zeros(n * n * R)
    _check(lib().sipg_laplacian_rows_f64(int(degree), rows.ctypes.data), "laplacian_rows")
    return rows


def volume_mvm(dim, degree, mat, x, out=None, stream=None):
    """out = M x for a stored operator in the reference's mode_matrix layout
    (float64 CUDA tensors; mat holds one operator, or one per element)."""
    import torch

    n1 = degree + 1
    per = n1 * n1 * (2 * degree + 1)
    mat_noe = mat.numel() // per
    if out is None:
        out = torch.empty_like(x)
    _check(lib().sipg_volume_mvm_f64(int(dim), int(degree), _ptr(mat), int(mat_noe), _ptr(x), _ptr(out),
                                     _stream(stream)), "volume_mvm")
    return out


def to_pairs(x64):
    """float64 tensor -> float32 pair vector (hi plane, lo plane)."""
    import torch

    hi = x64.float()
    lo = (x64 - hi.double()).float()
    return torch.cat([hi, lo])


def from_pairs(v):
    """float32 pair vector -> float64 tensor hi + lo."""
    n = v.numel() // 2
    return v[:n].double() + v[n:].double()


def launch_count():
    return int(lib().sipg_launch_count())


def probe_fma_peak():
    """(FP64, FP32) FMA throughput of the current device in TFLOP/s."""
    a, b = C.c_double(), C.c_double()
    _check(lib().sipg_probe_fma_peak(C.byref(a), C.byref(b)), "probe")
    return a.value, b.value


def version():
    return lib().sipg_version().decode()


def lgl_table(npts):
    x, w = np.zeros(npts), np.zeros(npts)
    _check(lib().sipg_lgl_table(npts, x.ctypes.data, w.ctypes.data), "sipg_lgl_table")
    return x, w


def dphi_table(p):
    D = np.zeros((p + 1) * (p + 1))
    _check(lib().sipg_dphi_table(p, D.ctypes.data), "sipg_dphi_table")
    return D


def square_mesh_coords(dim):
    x, y = np.zeros(4 * dim * dim), np.zeros(4 * dim * dim)
    _check(lib().sipg_square_mesh_coords(dim, x.ctypes.data, y.ctypes.data), "sipg_square_mesh_coords")
    return x, y


def pernode_tile(p, shape=0):
    """(elements per row, rows, threads per element) of the per-node FP64 tile
    of degree p: shape 0 holds the fewest elements per CTA, shape 1 twice as
    many along the row; (p+1)^2 threads per element."""
    return (4 if p <= 2 else 2) * (2 if shape else 1), 4 if p == 1 else 2, (p + 1) ** 2


PERNODE_DEFAULT_DIM = 128  # FP64 operators up to this size start with the per-node tile,
PERNODE_WIDE_DIM = 32  # shape 1 above this size


class Operator:
    """The SIPG operator of a dim x dim mesh of degree p with kernel penalty pen."""

    def __init__(self, dim, degree, pen, _handle=None):
        if _handle is None:
            h = C.c_void_p()
            _check(lib().sipg_op_create(int(dim), int(degree), float(pen), C.byref(h)), "sipg_op_create")
            self._owned = True
        else:  # an operator owned by a Batch
            h = _handle
            self._owned = False
        self._h = h
        self.dim, self.degree, self.pen = int(dim), int(degree), float(pen)
        self.noe = self.dim * self.dim
        self.ndof = self.noe * (self.degree + 1) ** 2

    def close(self):
        if self._h and self._owned:
            lib().sipg_op_destroy(self._h)
        self._h = None

    def autotune(self, stream=None):
        """Times the tile shapes on this operator and keeps the fastest per apply
        kind; returns {kind: (elements_per_row, rows, threads_per_element, ms_per_apply)}."""
        tc = TileChoice()
        _check(lib().sipg_op_autotune(self._h, _stream(stream), C.byref(tc)), "autotune")
        return {k: (tc.elements_per_row[i], tc.rows[i], tc.threads_per_element[i], tc.ms_per_apply[i])
                for k, i in TILE_KINDS.items()}

    def set_pernode(self, shape=0):
        """Switches the FP64 apply to the per-node tile (one thread per output
        node; shape 0 or 1, see pernode_tile)."""
        ex, ey, tpe = pernode_tile(self.degree, shape)
        self.set_tile("f64", ey, tpe, ex)

    def set_tile(self, kind, rows, threads_per_element=1, elements_per_row=32):
        _check(lib().sipg_op_set_tile(self._h, TILE_KINDS[kind], int(elements_per_row), int(rows),
                                      int(threads_per_element)), "set_tile")

    def get_tile(self, kind):
        """(rows, threads per element) of the apply kind's tile."""
        return self.get_shape(kind)[1:]

    def get_shape(self, kind):
        """(elements per row, rows, threads per element) of the apply kind's tile."""
        x, r, t = C.c_int(), C.c_int(), C.c_int()
        _check(lib().sipg_op_get_tile(self._h, TILE_KINDS[kind], C.byref(x), C.byref(r), C.byref(t)), "get_tile")
        return x.value, r.value, t.value

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _vec(self, t, dtype=None):
        import torch

        assert t.is_cuda and t.is_contiguous() and t.numel() == self.ndof, "expected a contiguous CUDA vector"
        if dtype is not None:
            assert t.dtype == dtype
        return t

    def empty(self, dtype=None):
        import torch

        return torch.empty(self.ndof, dtype=dtype or torch.float64, device="cuda")

    def apply(self, x, out=None, stream=None):
        """out = A x (float64 or float32 CUDA tensors)."""
        import torch

        self._vec(x)
        if out is None:
            out = torch.empty_like(x)
        self._vec(out, x.dtype)
        f = lib().sipg_apply_f64 if x.dtype == torch.float64 else lib().sipg_apply_f32
        _check(f(self._h, _ptr(x), _ptr(out), _stream(stream)), "apply")
        return out

    def apply_pairs(self, x, out=None, stream=None):
        """A x on double-float pair vectors: float32 CUDA tensors of 2 ndof
        values (hi plane, then lo plane), compensated arithmetic."""
        import torch

        assert x.dtype == torch.float32 and x.is_cuda and x.is_contiguous() and x.numel() == 2 * self.ndof
        if out is None:
            out = torch.empty_like(x)
        assert out.dtype == torch.float32 and out.numel() == 2 * self.ndof and out.data_ptr() != x.data_ptr()
        _check(lib().sipg_apply_pairs(self._h, _ptr(x), _ptr(out), _stream(stream)), "apply_pairs")
        return out

    def apply_host(self, x, out=None, stream=0):
        """Host numpy float64 in and out (copies inside)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        if out is None:
            out = np.empty_like(x)
        _check(lib().sipg_apply_host_f64(self._h, x.ctypes.data, out.ctypes.data, C.c_void_p(stream)),
               "apply_host")
        return out

    def cg(self, x, b, tol, relative=False, max_it=0, stream=None, raise_on=("breakdown",)):
        """Conjugate gradient from x (in place).  Returns (status, CgResult)."""
        import torch

        self._vec(x)
        self._vec(b, x.dtype)
        res = CgResult()
        if x.dtype == torch.float64:
            st = lib().sipg_cg_f64(self._h, _ptr(x), _ptr(b), float(tol), int(bool(relative)), int(max_it),
                                   C.byref(res), _stream(stream))
        else:
            st = lib().sipg_cg_f32(self._h, _ptr(x), _ptr(b), float(tol), int(bool(relative)), int(max_it),
                                   C.byref(res), _stream(stream))
        if st not in (0, 3, 4):
            _check(st, "cg")
        return st, res

    def pcg(self, x, b, tol, relative=False, max_it=0, stream=None):
        """Block-Jacobi preconditioned CG (FP64) from x (in place): the
        reference's USE_PRECONDITIONER solve.  Returns (status, CgResult)."""
        import torch

        self._vec(x, torch.float64)
        self._vec(b, torch.float64)
        res = CgResult()
        st = lib().sipg_pcg_f64(self._h, _ptr(x), _ptr(b), float(tol), int(bool(relative)), int(max_it),
                                C.byref(res), _stream(stream))
        if st not in (0, 3, 4):
            _check(st, "pcg")
        return st, res

    def apply_prec(self, x, out=None, stream=None):
        """out = M x, the block-Jacobi preconditioner (FP64)."""
        import torch

        self._vec(x, torch.float64)
        if out is None:
            out = torch.empty_like(x)
        _check(lib().sipg_apply_prec_f64(self._h, _ptr(x), _ptr(out), _stream(stream)), "apply_prec")
        return out

    def solve_mixed(self, x, b, inner_tol=0.1, outer_tol=1e-10, max_outer=200, max_inner=0, inner="auto",
                    outer="auto", stream=None):
        """Inner CG on the FP32 pipes inside an FP64 outer iteration; stops at
        ||b - Ax|| <= outer_tol ||b|| (FP64).  outer = "flexible": flexible CG
        in FP64 preconditioned by an FP32 inner CG that runs until its residual
        fell by inner_tol -- inner = "twolevel" (the default: the inner CG
        preconditioned by the two-level preconditioner) or "f32" (plain);
        "reliable": defect correction with reliable updates (an FP64 correction
        whenever the inner residual fell by inner_tol), inner = "f32" (FP32
        vectors), "pairs" (double-float pairs), "f64" or "auto" (by the
        condition-number estimate); outer = "auto": flexible unless inner names
        pairs or f64.  Returns (status, MixedResult)."""
        import torch

        self._vec(x, torch.float64)
        self._vec(b, torch.float64)
        o = MixedOpts(float(inner_tol), float(outer_tol), int(max_outer), int(max_inner), INNER[inner], OUTER[outer])
        res = MixedResult()
        st = lib().sipg_solve_mixed(self._h, _ptr(x), _ptr(b), C.byref(o), C.byref(res), _stream(stream))
        if st not in (0, 3, 4):
            _check(st, "solve_mixed")
        return st, res

    def true_residual(self, x, b, stream=None):
        """||b - A x|| / ||b|| evaluated in FP64 with the operator's zero-sum
        contractions over differences (sipg_residual_f64)."""
        import torch

        self._vec(x, torch.float64)
        self._vec(b, torch.float64)
        rel = C.c_double()
        _check(lib().sipg_residual_f64(self._h, _ptr(x), _ptr(b), None, C.byref(rel), _stream(stream)),
               "true_residual")
        return rel.value

    def apply_twolevel(self, r, out=None, stream=None):
        """out = M r, the two-level preconditioner of the flexible mixed solve
        (float32 CUDA tensors)."""
        import torch

        self._vec(r, torch.float32)
        if out is None:
            out = torch.empty_like(r)
        _check(lib().sipg_apply_twolevel_f32(self._h, _ptr(r), _ptr(out), _stream(stream)), "apply_twolevel")
        return out

    def rhs(self, sol, modes=None, out=None, stream=None):
        """Right-hand side of a test problem (SOL name or id) as a float64 CUDA vector."""
        sid = SOL[sol] if isinstance(sol, str) else int(sol)
        if out is None:
            out = self.empty()
        m = C.byref(modes) if modes is not None else None
        _check(lib().sipg_rhs_f64(self._h, sid, m, _ptr(out), _stream(stream)), "rhs")
        return out

    def err_norms(self, sol, u, modes=None, stream=None):
        """(L2, H1, max) nodal errors of u against test problem sol."""
        sid = SOL[sol] if isinstance(sol, str) else int(sol)
        e = np.zeros(3)
        m = C.byref(modes) if modes is not None else None
        _check(lib().sipg_err_norms_f64(self._h, sid, m, _ptr(u), e.ctypes.data, _stream(stream)), "err_norms")
        return float(e[0]), float(e[1]), float(e[2])


class Batch:
    """Many SIPG problems solved together (sipg_batch_*): problems is a list of
    (dim, degree, pen)."""

    def __init__(self, problems):
        arr = (Problem * len(problems))(*[Problem(int(d), int(p), float(pen)) for d, p, pen in problems])
        h = C.c_void_p()
        _check(lib().sipg_batch_create(len(problems), C.cast(arr, C.c_void_p), C.byref(h)), "sipg_batch_create")
        self._h = h
        self.problems = [(int(d), int(p), float(pen)) for d, p, pen in problems]

    def __len__(self):
        return len(self.problems)

    def op(self, i):
        h = C.c_void_p()
        _check(lib().sipg_batch_op(self._h, int(i), C.byref(h)), "sipg_batch_op")
        d, p, pen = self.problems[i]
        return Operator(d, p, pen, _handle=h)

    def footprint(self):
        return int(lib().sipg_batch_footprint(self._h))

    def solve_mixed(self, xs, bs, inner_tol=1e-2, outer_tol=1e-10, max_outer=200, max_inner=0, stream=None):
        """Solves every problem with flexible CG in FP64 around an FP32 inner
        CG (to relative inner_tol), all problems together; stops each at a
        true ||b - Ax|| <= outer_tol ||b||.  Returns (status, [MixedResult])."""
        n = len(self.problems)
        assert len(xs) == n and len(bs) == n
        px = (C.c_void_p * n)(*[x.data_ptr() for x in xs])
        pb = (C.c_void_p * n)(*[b.data_ptr() for b in bs])
        res = (MixedResult * n)()
        o = MixedOpts(float(inner_tol), float(outer_tol), int(max_outer), int(max_inner), INNER["auto"],
                      OUTER["auto"])
        st = lib().sipg_batch_solve_mixed(self._h, C.cast(px, C.c_void_p), C.cast(pb, C.c_void_p), C.byref(o),
                                          C.cast(res, C.c_void_p), _stream(stream))
        if st not in (0, 3, 4):
            _check(st, "batch_solve_mixed")
        return st, list(res)

    def close(self):
        if self._h:
            lib().sipg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Request(C.Structure):
    _fields_ = [("dim", C.c_int), ("degree", C.c_int), ("pen", C.c_double), ("sol", C.c_int), ("modes", Modes),
                ("tol", C.c_double), ("precision", C.c_int)]


F64, F32 = 0, 1


class Server:
    """Continuous-batching solve server (sipg_server_*).  submit() queues a
    request, step() runs one scheduling step, poll() reads a result."""

    def __init__(self, budget_bytes=150 << 30, max_active=256, iters_per_step=8, inner_tol=1e-2):
        o = ServerOpts(int(budget_bytes), int(max_active), int(iters_per_step), float(inner_tol))
        h = C.c_void_p()
        _check(lib().sipg_server_create(C.byref(o), C.byref(h)), "sipg_server_create")
        self._h = h

    def submit(self, dim, degree, pen, tol, sol="modes", modes=None, precision=F32):
        r = Request()
        r.dim, r.degree, r.pen, r.tol, r.precision = int(dim), int(degree), float(pen), float(tol), int(precision)
        r.sol = SOL[sol] if isinstance(sol, str) else int(sol)
        if modes is not None:
            r.modes = modes
        rid = C.c_ulonglong()
        st = lib().sipg_server_submit(self._h, C.byref(r), C.byref(rid))
        if st not in (0, 7):
            _check(st, "sipg_server_submit")
        return rid.value, st

    def step(self):
        a, c = C.c_int(), C.c_int()
        _check(lib().sipg_server_step(self._h, C.byref(a), C.byref(c)), "sipg_server_step")
        return a.value, c.value

    def poll(self, rid):
        res = RequestResult()
        _check(lib().sipg_server_poll(self._h, C.c_ulonglong(rid), C.byref(res)), "sipg_server_poll")
        return res

    def solution(self, rid, ndof):
        x = np.empty(int(ndof))
        _check(lib().sipg_server_solution(self._h, C.c_ulonglong(rid), x.ctypes.data, C.c_size_t(int(ndof))),
               "sipg_server_solution")
        return x

    def release(self, rid):
        _check(lib().sipg_server_release(self._h, C.c_ulonglong(rid)), "sipg_server_release")

    def stats(self):
        s = ServerStats()
        _check(lib().sipg_server_stats(self._h, C.byref(s)), "sipg_server_stats")
        return s

    def close(self):
        if self._h:
            lib().sipg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
