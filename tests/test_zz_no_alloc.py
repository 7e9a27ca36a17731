"""sipg_dot_f64_noalloc: the dot product for callers that cannot allocate device
memory (their device memory belongs to another allocator, or an allocation's
implicit synchronisation or failure is not acceptable where they call it).

It must give the same result as the allocating sipg_dot_f64, within the FP64
tolerance the other tests use (1e-12 relative to sum |x_i y_i|), on two calls
in a row (the shared scratch keeps the previous call's contents), and must
reject vectors longer than its fixed scratch allows.  Called through the C ABI.
This file is collected last on purpose."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu

MAX_N = 2048 * 8192
RTOL = 1e-12


@pytest.fixture(scope="module")
def torch():
    import torch as t

    return t


def _dot(fn, n, x, y, stream):
    r = C.c_double()
    st = fn(C.c_size_t(n), C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.byref(r), C.c_void_p(stream))
    return st, r.value


@pytest.mark.parametrize("n", [1, 777, 2048 * 37 + 5, 3_000_001, MAX_N])
def test_noalloc_dot_matches_allocating_dot_twice(sipg, torch, n):
    L = sipg.lib()
    g = torch.Generator(device="cuda").manual_seed(n)
    x = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    y = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    stream = torch.cuda.current_stream().cuda_stream
    st, ref = _dot(L.sipg_dot_f64, n, x, y, stream)
    assert st == 0
    scale = (x * y).abs().sum().item()
    st1, r1 = _dot(L.sipg_dot_f64_noalloc, n, x, y, stream)
    st2, r2 = _dot(L.sipg_dot_f64_noalloc, n, x, y, stream)
    assert st1 == 0 and st2 == 0, L.sipg_last_error()
    assert abs(r1 - ref) <= RTOL * scale
    assert abs(r2 - ref) <= RTOL * scale
    assert r1 == r2  # deterministic, and the second call starts from a clean counter


def test_noalloc_dot_rejects_sizes_beyond_its_scratch(sipg, torch):
    L = sipg.lib()
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    st, _ = _dot(L.sipg_dot_f64_noalloc, MAX_N + 1, x, x, torch.cuda.current_stream().cuda_stream)
    assert st == 1  # SIPG_ERR_INVALID, before any launch
    assert b"maximum" in L.sipg_last_error()
